// Device-side bodies shared by the per-molecule kernels and the batched engine.
#pragma once
#include <cmath>
#include "gfn2_kernels.h"

namespace xg {


__device__ __forceinline__ double sqi(double x) { return x * x; }


// ================================================================== multipole integrals
// build_SDQH0 (src/xtb/hamiltonian.F90:146-371) with get_multiints / multipole_3d / olapp
// (src/intgrad.f90:95-111, 509-555, 879-955) and dtrf2 (src/intgrad.f90:144-231).
template <int L> struct Cart;

template <> struct Cart<0> { static constexpr int n = 1; };

template <> struct Cart<1> { static constexpr int n = 3; };

template <> struct Cart<2> { static constexpr int n = 6; };

template <int L> struct Sph { static constexpr int n = 2 * L + 1; };


__device__ __forceinline__ void cart_pow(int l, int c, int& x, int& y, int& z) {
    if (l == 0) { x = y = z = 0; return; }
    if (l == 1) { x = (c == 0); y = (c == 1); z = (c == 2); return; }
    // xx yy zz xy xz yz
    const int px[6] = {2, 0, 0, 1, 1, 0}, py[6] = {0, 2, 0, 1, 0, 1}, pz[6] = {0, 0, 2, 0, 1, 1};
    x = px[c]; y = py[c]; z = pz[c];
}


// moment exponents: S, x, y, z, xx, yy, zz, xy, xz, yz
static __constant__ int c_mom[10][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 0},
                                 {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}};


__device__ __forceinline__ double dscale(int l, int c) { return (l == 2 && c >= 3) ? 1.7320508075688772935 : 1.0; }


// d Cartesian -> spherical rows (dx2-y2, dz2, dxy, dxz, dyz)
__device__ __forceinline__ double dtr(int s, int c) {
    const double h3 = 0.86602540378443864676;
    switch (s) {
        case 0: return c == 0 ? h3 : (c == 1 ? -h3 : 0.0);
        case 1: return c == 0 ? 0.5 : (c == 1 ? 0.5 : (c == 2 ? -1.0 : 0.0));
        case 2: return c == 3 ? 1.0 : 0.0;
        case 3: return c == 4 ? 1.0 : 0.0;
        default: return c == 5 ? 1.0 : 0.0;
    }
}

// effective transform: sph[s] = sum_c T(l)[s][c] * cart[c] (includes the d contraction scale)
__device__ __forceinline__ double tr(int l, int s, int c) {
    if (l < 2) return s == c ? 1.0 : 0.0;
    return dtr(s, c) * dscale(l, c);
}


// 1D integrals v[e][i][j] = int (x-A)^i (x-B)^j (x-C)^e exp(-g (x-P)^2) dx / sqrt(pi/g)
template <int MI, int MJ>
__device__ __forceinline__ void mom1d(double PA, double PB, double PC, double g, double (&v)[3][MI + 1][MJ + 1]) {
    constexpr int MT = MI + MJ + 3;
    double t[MT];
    const double h = 0.5 / g;
    t[0] = 1.0;
    t[1] = 0.0;
#pragma unroll
    for (int k = 2; k < MT; ++k) t[k] = (k - 1) * h * t[k - 2];
    const int binom[4][4] = {{1, 0, 0, 0}, {1, 1, 0, 0}, {1, 2, 1, 0}, {1, 3, 3, 1}};
    double pa[MI + 1], pb[MJ + 1];
    pa[0] = 1.0;
#pragma unroll
    for (int k = 1; k <= MI; ++k) pa[k] = pa[k - 1] * PA;
    pb[0] = 1.0;
#pragma unroll
    for (int k = 1; k <= MJ; ++k) pb[k] = pb[k - 1] * PB;
#pragma unroll
    for (int i = 0; i <= MI; ++i)
#pragma unroll
        for (int j = 0; j <= MJ; ++j) {
            double s0 = 0.0, s1 = 0.0, s2 = 0.0;
#pragma unroll
            for (int a = 0; a <= i; ++a)
#pragma unroll
                for (int b = 0; b <= j; ++b) {
                    const double c = binom[i][a] * binom[j][b] * pa[i - a] * pb[j - b];
                    const int mm = a + b;
                    s0 += c * t[mm];
                    s1 += c * (t[mm + 1] + PC * t[mm]);
                    s2 += c * (t[mm + 2] + 2.0 * PC * t[mm + 1] + PC * PC * t[mm]);
                }
            v[0][i][j] = s0;
            v[1][i][j] = s1;
            v[2][i][j] = s2;
        }
}


__device__ __forceinline__ void tri_index(long t, int& a, int& b) {
    long aa = (long)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (aa * (aa + 1) / 2 > t) --aa;
    while ((aa + 1) * (aa + 2) / 2 <= t) ++aa;
    a = (int)aa;
    b = (int)(t - aa * (aa + 1) / 2);
}


// shell pairs of class (LI, LJ), LI >= LJ: all pairs of an LI shell with an LJ shell, for LI == LJ
// the pairs with ish >= jsh (diagonal included)
template <int LI, int LJ>
__host__ __device__ __forceinline__ long class_pairs(const DevMol& m) {
    const long ni = m.l_off[LI + 1] - m.l_off[LI], nj = m.l_off[LJ + 1] - m.l_off[LJ];
    return LI == LJ ? ni * (ni + 1) / 2 : ni * nj;
}

// pair t (< class_pairs) of class (LI, LJ) in canonical order (the LI shell first)
template <int LI, int LJ>
__device__ __forceinline__ bool canonical_pair(const DevMol& m, long t, int& ish, int& jsh) {
    if (LI == LJ) {
        int a, b;
        tri_index(t, a, b);
        ish = m.sh_byl[m.l_off[LI] + a];
        jsh = m.sh_byl[m.l_off[LI] + b];
    } else {
        const long nj = m.l_off[LJ + 1] - m.l_off[LJ];
        ish = m.sh_byl[m.l_off[LI] + (int)(t / nj)];
        jsh = m.sh_byl[m.l_off[LJ] + (int)(t % nj)];
    }
    return true;
}


// H0 off-diagonal prefactor hav * shpoly (eV), h0scal + shellPoly (src/scc_core.f90:644-680, 728-754)
__device__ __forceinline__ double h0_factor(const DevMol& m, const double* se, int ish, int jsh, double r) {
    const int li = m.sh_l[ish], lj = m.sh_l[jsh];
    const int iat = m.sh_atom[ish], jat = m.sh_atom[jsh];
    const double kshell[4] = {1.85, 2.23, 2.23, 2.23};
    double ks = 0.5 * (kshell[li] + kshell[lj]);
    if ((li == 0 && lj == 2) || (li == 2 && lj == 0)) ks = 2.0;   // ksd
    if ((li == 1 && lj == 2) || (li == 2 && lj == 1)) ks = 2.0;   // kpd
    const double den = sqi(m.en[iat] - m.en[jat]);
    const double enpoly = 1.0 + 0.02 * den * (1.0 + 0.0 * den);
    const double km = ks * enpoly;
    const double zi = m.sh_zeta[ish], zj = m.sh_zeta[jsh];
    const double zetaij = pow(2.0 * sqrt(zi * zj) / (zi + zj), 0.5);
    const double hav = 0.5 * km * (se[ish] + se[jsh]) * zetaij;
    const double rr = m.arad[jat] + m.arad[iat];
    const double rs = sqrt(r / rr);
    const double rf1 = 1.0 + 0.01 * m.sh_poly[ish] * rs;
    const double rf2 = 1.0 + 0.01 * m.sh_poly[jsh] * rs;
    return hav * rf1 * rf2;
}


template <int LI, int LJ>
__device__ inline void d_sdqh0(DevMol m, const double* __restrict__ se, double intcut, long npairs,
                                               double* __restrict__ S, double* __restrict__ D, double* __restrict__ Q,
                                               double* __restrict__ H0, long t) {
    int ish, jsh;
    if (!canonical_pair<LI, LJ>(m, t, ish, jsh)) return;
    constexpr int NCI = Cart<LI>::n, NCJ = Cart<LJ>::n, NSI = Sph<LI>::n, NSJ = Sph<LJ>::n;
    const int iat = m.sh_atom[ish], jat = m.sh_atom[jsh];
    const bool same = iat == jat;
    const double A[3] = {m.xyz[3 * iat], m.xyz[3 * iat + 1], m.xyz[3 * iat + 2]};
    const double B[3] = {m.xyz[3 * jat], m.xyz[3 * jat + 1], m.xyz[3 * jat + 2]};
    const double r2 = sqi(A[0] - B[0]) + sqi(A[1] - B[1]) + sqi(A[2] - B[2]);
    const size_t nao = m.nao, nn = nao * nao;
    const int ai0 = m.sh_ao[ish], aj0 = m.sh_ao[jsh];
    if (same && ish == jsh) {
        for (int s = 0; s < NSI; ++s) {
            S[(ai0 + s) * nao + ai0 + s] = 1.0;
            H0[(ai0 + s) * nao + ai0 + s] = se[ish];
        }
    }
    if (r2 > 2000.0) return;
    double res[NCI][NCJ][10];
#pragma unroll
    for (int a = 0; a < NCI; ++a)
#pragma unroll
        for (int b = 0; b < NCJ; ++b)
#pragma unroll
            for (int k = 0; k < 10; ++k) res[a][b][k] = 0.0;
    const double sqrtpi = 1.7724538509055160273;
    const int npi = m.sh_nprim[ish], npj = m.sh_nprim[jsh];
    for (int p = 0; p < npi; ++p) {
        const double ai = m.sh_alpha[ish * MAXPRIM + p], ci = m.sh_coef[ish * MAXPRIM + p];
        for (int q = 0; q < npj; ++q) {
            const double aj = m.sh_alpha[jsh * MAXPRIM + q], cj = m.sh_coef[jsh * MAXPRIM + q];
            double est = r2 * ai * aj;
            if (est > intcut * (ai + aj)) continue;
            const double g = ai + aj, ab = 1.0 / g;
            est *= ab;
            const double sab = sqrtpi * sqrt(ab);
            const double kab = exp(-est) * (sab * sab * sab);
            const double cc = kab * ci * cj;
            double v[3][3][LI + 1][LJ + 1];
#pragma unroll
            for (int x = 0; x < 3; ++x) {
                const double P = (ai * A[x] + aj * B[x]) * ab;
                mom1d<LI, LJ>(P - A[x], P - B[x], P, g, v[x]);
            }
#pragma unroll
            for (int a = 0; a < NCI; ++a) {
                int ix, iy, iz;
                cart_pow(LI, a, ix, iy, iz);
#pragma unroll
                for (int b = 0; b < NCJ; ++b) {
                    int jx, jy, jz;
                    cart_pow(LJ, b, jx, jy, jz);
#pragma unroll
                    for (int k = 0; k < 10; ++k)
                        res[a][b][k] += cc * v[0][c_mom[k][0]][ix][jx] * v[1][c_mom[k][1]][iy][jy] *
                                        v[2][c_mom[k][2]][iz][jz];
                }
            }
        }
    }
    const double hfac = same ? 0.0 : h0_factor(m, se, ish, jsh, sqrt(r2));
#pragma unroll
    for (int s = 0; s < NSI; ++s)
#pragma unroll
        for (int u = 0; u < NSJ; ++u) {
            double val[10];
#pragma unroll
            for (int k = 0; k < 10; ++k) {
                double acc = 0.0;
#pragma unroll
                for (int a = 0; a < NCI; ++a)
#pragma unroll
                    for (int b = 0; b < NCJ; ++b) {
                        const double w = tr(LI, s, a) * tr(LJ, u, b);
                        if (w != 0.0) acc += w * res[a][b][k];
                    }
                val[k] = acc;
            }
            const size_t ia = ai0 + s, ja = aj0 + u;
            if (!same) {
                S[ia * nao + ja] = val[0];
                S[ja * nao + ia] = val[0];
                H0[ia * nao + ja] = hfac * val[0];
                H0[ja * nao + ia] = hfac * val[0];
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                D[k * nn + ia * nao + ja] = val[1 + k];
                D[k * nn + ja * nao + ia] = val[1 + k];
            }
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                Q[k * nn + ia * nao + ja] = val[4 + k];
                Q[k * nn + ja * nao + ia] = val[4 + k];
            }
        }
}


// ================================================================== gradient of the S/D/Q/H0 terms
// build_dSDQH0_noreset (src/xtb/hamiltonian.F90:575-792) with get_grad_multiint / multipole_grad_3d /
// shiftintg (src/intgrad.f90:607-728, 958-1035) and dshellPoly (src/grad_core.f90:40-72).  The derivative
// integrals are contracted with their energy weights inside the primitive loop (fused kernel).
template <int LI, int LJ>
__device__ inline void d_grad_sdqh0(DevMol m, const double* __restrict__ se, double intcut, long npairs,
                                                    const double* __restrict__ P, const double* __restrict__ Pew,
                                                    const double* __restrict__ shift, const double* __restrict__ vs,
                                                    const double* __restrict__ vd, const double* __restrict__ vq,
                                                    double* __restrict__ grad, double* __restrict__ dhdcn, long t) {
    int ish, jsh;
    if (!canonical_pair<LI, LJ>(m, t, ish, jsh)) return;
    const int iat = m.sh_atom[ish], jat = m.sh_atom[jsh];
    if (iat == jat) return;
    constexpr int NCI = Cart<LI>::n, NCJ = Cart<LJ>::n, NSI = Sph<LI>::n, NSJ = Sph<LJ>::n;
    const double A[3] = {m.xyz[3 * iat], m.xyz[3 * iat + 1], m.xyz[3 * iat + 2]};
    const double B[3] = {m.xyz[3 * jat], m.xyz[3 * jat + 1], m.xyz[3 * jat + 2]};
    const double rij[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
    const double rab2 = sqi(rij[0]) + sqi(rij[1]) + sqi(rij[2]);
    if (rab2 > 1600.0) return;
    const size_t nao = m.nao;
    const int ai0 = m.sh_ao[ish], aj0 = m.sh_ao[jsh];
    // shell polynomial and its derivative w.r.t. A
    const double rab = sqrt(rab2);
    const double rr = m.arad[iat] + m.arad[jat];
    const double t14 = sqrt(rab / rr);
    const double k1 = m.sh_poly[ish] * 0.01, k2 = m.sh_poly[jsh] * 0.01;
    const double t15 = k1 * t14, t23 = k2 * t14;
    const double shpoly = (1.0 + t15) * (1.0 + k2 * t14);
    const double dsp = (t15 * (1.0 + t23) + (1.0 + t15) * k2 * t14) * 0.5 / rab2;
    const double hnov = h0_factor(m, se, ish, jsh, rab) * EVTOAU;   // H0 without overlap (Eh)
    const double hav0 = 0.5 * (se[ish] + se[jsh]);
    const double vsum = vs[iat] + vs[jat];
    const double esum = shift[ish] + shift[jsh];
    // Cartesian contraction weights: [0] S term, [1..3] D about A, [4..6] D about B,
    // [7..12] Q about A, [13..18] Q about B, [19] H*P (for the shell-polynomial and CN terms)
    double w[NCI][NCJ][20];
#pragma unroll
    for (int a = 0; a < NCI; ++a)
#pragma unroll
        for (int b = 0; b < NCJ; ++b)
#pragma unroll
            for (int k = 0; k < 20; ++k) w[a][b][k] = 0.0;
    for (int s = 0; s < NSI; ++s)
        for (int u = 0; u < NSJ; ++u) {
            const size_t ia = ai0 + s, ja = aj0 + u;
            const double p = P[ja * nao + ia];
            const double hp = hnov * p;
            double ws[20];
            ws[0] = 2.0 * hp - 2.0 * Pew[ja * nao + ia] - p * esum + p * vsum;
            for (int k = 0; k < 3; ++k) { ws[1 + k] = p * vd[3 * iat + k]; ws[4 + k] = p * vd[3 * jat + k]; }
            for (int k = 0; k < 6; ++k) { ws[7 + k] = p * vq[6 * iat + k]; ws[13 + k] = p * vq[6 * jat + k]; }
            ws[19] = hp;
#pragma unroll
            for (int a = 0; a < NCI; ++a)
#pragma unroll
                for (int b = 0; b < NCJ; ++b) {
                    const double f = tr(LI, s, a) * tr(LJ, u, b);
                    if (f == 0.0) continue;
#pragma unroll
                    for (int k = 0; k < 20; ++k) w[a][b][k] += f * ws[k];
                }
        }
    double gx[3] = {0.0, 0.0, 0.0};
    double sHPS = 0.0;
    const double sqrtpi = 1.7724538509055160273;
    const int npi = m.sh_nprim[ish], npj = m.sh_nprim[jsh];
    for (int p = 0; p < npi; ++p) {
        const double ai = m.sh_alpha[ish * MAXPRIM + p], ci = m.sh_coef[ish * MAXPRIM + p];
        for (int q = 0; q < npj; ++q) {
            const double aj = m.sh_alpha[jsh * MAXPRIM + q], cj = m.sh_coef[jsh * MAXPRIM + q];
            double est = ai * aj * rab2;
            if (est > intcut * (ai + aj)) continue;
            const double g = ai + aj, ab = 1.0 / g;
            est *= ab;
            const double sab = sqrtpi * sqrt(ab);
            const double cc = exp(-est) * (sab * sab * sab) * ci * cj;
            double vB[3][3][LI + 2][LJ + 1], vA[3][3][LI + 2][LJ + 1];
#pragma unroll
            for (int x = 0; x < 3; ++x) {
                const double Pp = (ai * A[x] + aj * B[x]) * ab;
                mom1d<LI + 1, LJ>(Pp - A[x], Pp - B[x], Pp - B[x], g, vB[x]);
                mom1d<LI + 1, LJ>(Pp - A[x], Pp - B[x], Pp - A[x], g, vA[x]);
            }
#pragma unroll
            for (int a = 0; a < NCI; ++a) {
                int pi[3];
                cart_pow(LI, a, pi[0], pi[1], pi[2]);
#pragma unroll
                for (int b = 0; b < NCJ; ++b) {
                    int pj[3];
                    cart_pow(LJ, b, pj[0], pj[1], pj[2]);
                    const double* wt = w[a][b];
                    // overlap (no derivative) for the H*P*S sums
                    sHPS += cc * wt[19] * vB[0][0][pi[0]][pj[0]] * vB[1][0][pi[1]][pj[1]] * vB[2][0][pi[2]][pj[2]];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        // derivative factor on axis c for moment order e: 2 ai I(i+1) - i I(i-1)
                        auto dB = [&](int e) {
                            double r = 2.0 * ai * vB[c][e][pi[c] + 1][pj[c]];
                            if (pi[c] > 0) r -= pi[c] * vB[c][e][pi[c] - 1][pj[c]];
                            return r;
                        };
                        auto dA = [&](int e) {
                            double r = 2.0 * ai * vA[c][e][pi[c] + 1][pj[c]];
                            if (pi[c] > 0) r -= pi[c] * vA[c][e][pi[c] - 1][pj[c]];
                            return r;
                        };
                        double acc = 0.0;
#pragma unroll
                        for (int k = 0; k < 10; ++k) {
                            // moment k about B, derivative on axis c
                            double fb = 1.0, fa = 1.0;
#pragma unroll
                            for (int x = 0; x < 3; ++x) {
                                const int e = c_mom[k][x];
                                if (x == c) { fb *= dB(e); fa *= dA(e); }
                                else { fb *= vB[x][e][pi[x]][pj[x]]; fa *= vA[x][e][pi[x]][pj[x]]; }
                            }
                            // origin moves with A: subtract e_c * M_{e - 1_c}(A)
                            const int ec = c_mom[k][c];
                            if (ec > 0) {
                                double lo = 1.0;
#pragma unroll
                                for (int x = 0; x < 3; ++x) {
                                    const int e = c_mom[k][x] - (x == c ? 1 : 0);
                                    lo *= vA[x][e][pi[x]][pj[x]];
                                }
                                fa -= ec * lo;
                            }
                            if (k == 0) acc += wt[0] * fb;
                            else if (k < 4) acc += wt[k] * fa + wt[3 + k] * fb;
                            else acc += wt[3 + k] * fa + wt[9 + k] * fb;
                        }
                        gx[c] += cc * acc;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) gx[c] += 2.0 * sHPS * dsp * rij[c] / shpoly;
    const double dcn = sHPS / hav0;
    atomicAdd(&grad[3 * iat + 0], gx[0]);
    atomicAdd(&grad[3 * iat + 1], gx[1]);
    atomicAdd(&grad[3 * iat + 2], gx[2]);
    atomicAdd(&grad[3 * jat + 0], -gx[0]);
    atomicAdd(&grad[3 * jat + 1], -gx[1]);
    atomicAdd(&grad[3 * jat + 2], -gx[2]);
    atomicAdd(&dhdcn[iat], dcn * (-m.sh_kcn[ish]));
    atomicAdd(&dhdcn[jat], dcn * (-m.sh_kcn[jsh]));
}


// ================================================================== one warp per shell pair
// The same integrals and gradient contraction with a warp per shell pair, for the classes whose
// per-thread form would hold hundreds of doubles (p-p, d-s, d-p, d-d).  Per primitive pair the
// lanes share the 1D moment integrals through the warp's shared-memory slice, and each lane owns
// one or two Cartesian component pairs (a, b) with their contraction weights in registers.

// shared-memory doubles one warp needs for class (LI, LJ): the gradient's 1D integrals about
// two centres (powers up to LI + 1), or the integrals' 1D table plus the Cartesian results
template <int LI, int LJ>
struct WarpInt {
    static constexpr int NV = 3 * 3 * (LI + 1) * (LJ + 1);       // [x][e][i][j]
    static constexpr int NRES = Cart<LI>::n * Cart<LJ>::n * 10;  // [a*NCJ + b][k]
    static constexpr int NG = 2 * 3 * 3 * (LI + 2) * (LJ + 1);   // [o][x][e][i][j]
    static constexpr int SMEM = (NV + NRES > NG ? NV + NRES : NG);
};

// one entry (i, j) of mom1d: s_e = int (x-A)^i (x-B)^j (x-C)^e exp(-g (x-P)^2) dx / sqrt(pi/g)
template <int MT>
__device__ __forceinline__ void mom1d_entry(double PA, double PB, double PC, double g, int i, int j, double& s0,
                                            double& s1, double& s2) {
    double t[MT];
    const double h = 0.5 / g;
    t[0] = 1.0;
    t[1] = 0.0;
#pragma unroll
    for (int k = 2; k < MT; ++k) t[k] = (k - 1) * h * t[k - 2];
    const int binom[4][4] = {{1, 0, 0, 0}, {1, 1, 0, 0}, {1, 2, 1, 0}, {1, 3, 3, 1}};
    double pa[4], pb[4];
    pa[0] = pb[0] = 1.0;
#pragma unroll
    for (int k = 1; k < 4; ++k) {
        pa[k] = pa[k - 1] * PA;
        pb[k] = pb[k - 1] * PB;
    }
    s0 = s1 = s2 = 0.0;
    for (int a = 0; a <= i; ++a)
        for (int b = 0; b <= j; ++b) {
            const double c = binom[i][a] * binom[j][b] * pa[i - a] * pb[j - b];
            const int mm = a + b;
            s0 += c * t[mm];
            s1 += c * (t[mm + 1] + PC * t[mm]);
            s2 += c * (t[mm + 2] + 2.0 * PC * t[mm + 1] + PC * PC * t[mm]);
        }
}

template <int LI, int LJ>
__device__ inline void d_sdqh0_warp(const DevMol& m, const double* __restrict__ se, double intcut, double* __restrict__ S,
                                    double* __restrict__ D, double* __restrict__ Q, double* __restrict__ H0, long t,
                                    int lane, double* __restrict__ sm) {
    int ish, jsh;
    if (!canonical_pair<LI, LJ>(m, t, ish, jsh)) return;
    constexpr int NCI = Cart<LI>::n, NCJ = Cart<LJ>::n, NSI = Sph<LI>::n, NSJ = Sph<LJ>::n;
    constexpr int NAB = NCI * NCJ, LJ1 = LJ + 1, SZ = (LI + 1) * (LJ + 1);
    static_assert(NAB <= 64, "at most two component pairs per lane");
    const int iat = m.sh_atom[ish], jat = m.sh_atom[jsh];
    const bool same = iat == jat;
    const double A[3] = {m.xyz[3 * iat], m.xyz[3 * iat + 1], m.xyz[3 * iat + 2]};
    const double B[3] = {m.xyz[3 * jat], m.xyz[3 * jat + 1], m.xyz[3 * jat + 2]};
    const double r2 = sqi(A[0] - B[0]) + sqi(A[1] - B[1]) + sqi(A[2] - B[2]);
    const size_t nao = m.nao, nn = nao * nao;
    const int ai0 = m.sh_ao[ish], aj0 = m.sh_ao[jsh];
    if (same && ish == jsh && lane < NSI) {
        S[(ai0 + lane) * nao + ai0 + lane] = 1.0;
        H0[(ai0 + lane) * nao + ai0 + lane] = se[ish];
    }
    if (r2 > 2000.0) return;
    double* v = sm;                              // [x][e][i][j]
    double* res = sm + WarpInt<LI, LJ>::NV;      // [ab][k]
    double acc[2][10];
    int ab_x[2][3], ab_y[2][3];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int ab = lane + 32 * h;
#pragma unroll
        for (int k = 0; k < 10; ++k) acc[h][k] = 0.0;
        int ix = 0, iy = 0, iz = 0, jx = 0, jy = 0, jz = 0;
        if (ab < NAB) {
            cart_pow(LI, ab / NCJ, ix, iy, iz);
            cart_pow(LJ, ab % NCJ, jx, jy, jz);
        }
        ab_x[h][0] = ix; ab_x[h][1] = iy; ab_x[h][2] = iz;
        ab_y[h][0] = jx; ab_y[h][1] = jy; ab_y[h][2] = jz;
    }
    const double sqrtpi = 1.7724538509055160273;
    const int npi = m.sh_nprim[ish], npj = m.sh_nprim[jsh];
    for (int p = 0; p < npi; ++p) {
        const double ai = m.sh_alpha[ish * MAXPRIM + p], ci = m.sh_coef[ish * MAXPRIM + p];
        for (int q = 0; q < npj; ++q) {
            const double aj = m.sh_alpha[jsh * MAXPRIM + q], cj = m.sh_coef[jsh * MAXPRIM + q];
            double est = r2 * ai * aj;
            if (est > intcut * (ai + aj)) continue;
            const double g = ai + aj, ab = 1.0 / g;
            est *= ab;
            const double sab = sqrtpi * sqrt(ab);
            const double cc = exp(-est) * (sab * sab * sab) * ci * cj;
            __syncwarp();
            for (int u = lane; u < 3 * SZ; u += 32) {
                const int x = u / SZ, i = (u % SZ) / LJ1, j = u % LJ1;
                const double P = (ai * A[x] + aj * B[x]) * ab;
                double s0, s1, s2;
                mom1d_entry<LI + LJ + 3>(P - A[x], P - B[x], P, g, i, j, s0, s1, s2);
                v[(x * 3 + 0) * SZ + i * LJ1 + j] = s0;
                v[(x * 3 + 1) * SZ + i * LJ1 + j] = s1;
                v[(x * 3 + 2) * SZ + i * LJ1 + j] = s2;
            }
            __syncwarp();
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (lane + 32 * h >= NAB) continue;
                const int* pi = ab_x[h];
                const int* pj = ab_y[h];
#pragma unroll
                for (int k = 0; k < 10; ++k)
                    acc[h][k] += cc * v[(0 * 3 + c_mom[k][0]) * SZ + pi[0] * LJ1 + pj[0]] *
                                 v[(1 * 3 + c_mom[k][1]) * SZ + pi[1] * LJ1 + pj[1]] *
                                 v[(2 * 3 + c_mom[k][2]) * SZ + pi[2] * LJ1 + pj[2]];
            }
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
        if (lane + 32 * h < NAB)
#pragma unroll
            for (int k = 0; k < 10; ++k) res[(lane + 32 * h) * 10 + k] = acc[h][k];
    __syncwarp();
    const double hfac = same ? 0.0 : h0_factor(m, se, ish, jsh, sqrt(r2));
    for (int su = lane; su < NSI * NSJ; su += 32) {
        const int s = su / NSJ, u = su % NSJ;
        double val[10];
#pragma unroll
        for (int k = 0; k < 10; ++k) val[k] = 0.0;
        for (int a = 0; a < NCI; ++a) {
            const double ta = tr(LI, s, a);
            if (ta == 0.0) continue;
            for (int b = 0; b < NCJ; ++b) {
                const double w = ta * tr(LJ, u, b);
                if (w == 0.0) continue;
#pragma unroll
                for (int k = 0; k < 10; ++k) val[k] += w * res[(a * NCJ + b) * 10 + k];
            }
        }
        const size_t ia = ai0 + s, ja = aj0 + u;
        if (!same) {
            S[ia * nao + ja] = val[0];
            S[ja * nao + ia] = val[0];
            H0[ia * nao + ja] = hfac * val[0];
            H0[ja * nao + ia] = hfac * val[0];
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            D[k * nn + ia * nao + ja] = val[1 + k];
            D[k * nn + ja * nao + ia] = val[1 + k];
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            Q[k * nn + ia * nao + ja] = val[4 + k];
            Q[k * nn + ja * nao + ia] = val[4 + k];
        }
    }
    __syncwarp();
}

template <int LI, int LJ>
__device__ inline void d_grad_sdqh0_warp(const DevMol& m, const double* __restrict__ se, double intcut,
                                         const double* __restrict__ P, const double* __restrict__ Pew,
                                         const double* __restrict__ shift, const double* __restrict__ vs,
                                         const double* __restrict__ vd, const double* __restrict__ vq,
                                         double* __restrict__ grad, double* __restrict__ dhdcn, long t, int lane,
                                         double* __restrict__ sm) {
    int ish, jsh;
    if (!canonical_pair<LI, LJ>(m, t, ish, jsh)) return;
    const int iat = m.sh_atom[ish], jat = m.sh_atom[jsh];
    if (iat == jat) return;
    constexpr int NCI = Cart<LI>::n, NCJ = Cart<LJ>::n, NSI = Sph<LI>::n, NSJ = Sph<LJ>::n;
    constexpr int NAB = NCI * NCJ, MI1 = LI + 2, LJ1 = LJ + 1, SZ = MI1 * LJ1;
    const double A[3] = {m.xyz[3 * iat], m.xyz[3 * iat + 1], m.xyz[3 * iat + 2]};
    const double B[3] = {m.xyz[3 * jat], m.xyz[3 * jat + 1], m.xyz[3 * jat + 2]};
    const double rij[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
    const double rab2 = sqi(rij[0]) + sqi(rij[1]) + sqi(rij[2]);
    if (rab2 > 1600.0) return;
    const size_t nao = m.nao;
    const int ai0 = m.sh_ao[ish], aj0 = m.sh_ao[jsh];
    const double rab = sqrt(rab2);
    const double rr = m.arad[iat] + m.arad[jat];
    const double t14 = sqrt(rab / rr);
    const double k1 = m.sh_poly[ish] * 0.01, k2 = m.sh_poly[jsh] * 0.01;
    const double t15 = k1 * t14, t23 = k2 * t14;
    const double shpoly = (1.0 + t15) * (1.0 + k2 * t14);
    const double dsp = (t15 * (1.0 + t23) + (1.0 + t15) * k2 * t14) * 0.5 / rab2;
    const double hnov = h0_factor(m, se, ish, jsh, rab) * EVTOAU;
    const double hav0 = 0.5 * (se[ish] + se[jsh]);
    const double vsum = vs[iat] + vs[jat];
    const double esum = shift[ish] + shift[jsh];
    // contraction weights of this lane's component pairs (same meaning as in d_grad_sdqh0)
    double w[2][20];
    int pi_[2][3], pj_[2][3];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int ab = lane + 32 * h;
#pragma unroll
        for (int k = 0; k < 20; ++k) w[h][k] = 0.0;
        int a = 0, b = 0;
        if (ab < NAB) {
            a = ab / NCJ;
            b = ab % NCJ;
        }
        cart_pow(LI, a, pi_[h][0], pi_[h][1], pi_[h][2]);
        cart_pow(LJ, b, pj_[h][0], pj_[h][1], pj_[h][2]);
        if (ab >= NAB) continue;
        for (int s = 0; s < NSI; ++s) {
            const double fa = tr(LI, s, a);
            if (fa == 0.0) continue;
            for (int u = 0; u < NSJ; ++u) {
                const double f = fa * tr(LJ, u, b);
                if (f == 0.0) continue;
                const size_t ia = ai0 + s, ja = aj0 + u;
                const double p = P[ja * nao + ia];
                const double hp = hnov * p;
                w[h][0] += f * (2.0 * hp - 2.0 * Pew[ja * nao + ia] - p * esum + p * vsum);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    w[h][1 + k] += f * p * vd[3 * iat + k];
                    w[h][4 + k] += f * p * vd[3 * jat + k];
                }
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    w[h][7 + k] += f * p * vq[6 * iat + k];
                    w[h][13 + k] += f * p * vq[6 * jat + k];
                }
                w[h][19] += f * hp;
            }
        }
    }
    double gx[3] = {0.0, 0.0, 0.0};
    double sHPS = 0.0;
    const double sqrtpi = 1.7724538509055160273;
    const int npi = m.sh_nprim[ish], npj = m.sh_nprim[jsh];
    for (int p = 0; p < npi; ++p) {
        const double ai = m.sh_alpha[ish * MAXPRIM + p], ci = m.sh_coef[ish * MAXPRIM + p];
        for (int q = 0; q < npj; ++q) {
            const double aj = m.sh_alpha[jsh * MAXPRIM + q], cj = m.sh_coef[jsh * MAXPRIM + q];
            double est = ai * aj * rab2;
            if (est > intcut * (ai + aj)) continue;
            const double g = ai + aj, ab = 1.0 / g;
            est *= ab;
            const double sab = sqrtpi * sqrt(ab);
            const double cc = exp(-est) * (sab * sab * sab) * ci * cj;
            __syncwarp();
            // 1D integrals about B (o = 0) and about A (o = 1): sm[((o*3 + x)*3 + e)*SZ + i*LJ1 + j]
            for (int u = lane; u < 6 * SZ; u += 32) {
                const int o = u / (3 * SZ), x = (u / SZ) % 3, i = (u % SZ) / LJ1, j = u % LJ1;
                const double Pp = (ai * A[x] + aj * B[x]) * ab;
                double s0, s1, s2;
                mom1d_entry<LI + LJ + 4>(Pp - A[x], Pp - B[x], o == 0 ? Pp - B[x] : Pp - A[x], g, i, j, s0, s1, s2);
                double* dst = sm + ((o * 3 + x) * 3) * SZ + i * LJ1 + j;
                dst[0] = s0;
                dst[SZ] = s1;
                dst[2 * SZ] = s2;
            }
            __syncwarp();
            auto vB = [&](int x, int e, int i, int j) { return sm[((0 * 3 + x) * 3 + e) * SZ + i * LJ1 + j]; };
            auto vA = [&](int x, int e, int i, int j) { return sm[((1 * 3 + x) * 3 + e) * SZ + i * LJ1 + j]; };
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (lane + 32 * h >= NAB) continue;
                const int* pi = pi_[h];
                const int* pj = pj_[h];
                const double* wt = w[h];
                sHPS += cc * wt[19] * vB(0, 0, pi[0], pj[0]) * vB(1, 0, pi[1], pj[1]) * vB(2, 0, pi[2], pj[2]);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    auto dB = [&](int e) {
                        double r = 2.0 * ai * vB(c, e, pi[c] + 1, pj[c]);
                        if (pi[c] > 0) r -= pi[c] * vB(c, e, pi[c] - 1, pj[c]);
                        return r;
                    };
                    auto dA = [&](int e) {
                        double r = 2.0 * ai * vA(c, e, pi[c] + 1, pj[c]);
                        if (pi[c] > 0) r -= pi[c] * vA(c, e, pi[c] - 1, pj[c]);
                        return r;
                    };
                    double acc = 0.0;
#pragma unroll
                    for (int k = 0; k < 10; ++k) {
                        double fb = 1.0, fa = 1.0;
#pragma unroll
                        for (int x = 0; x < 3; ++x) {
                            const int e = c_mom[k][x];
                            if (x == c) {
                                fb *= dB(e);
                                fa *= dA(e);
                            } else {
                                fb *= vB(x, e, pi[x], pj[x]);
                                fa *= vA(x, e, pi[x], pj[x]);
                            }
                        }
                        const int ec = c_mom[k][c];
                        if (ec > 0) {
                            double lo = 1.0;
#pragma unroll
                            for (int x = 0; x < 3; ++x) lo *= vA(x, c_mom[k][x] - (x == c ? 1 : 0), pi[x], pj[x]);
                            fa -= ec * lo;
                        }
                        if (k == 0) acc += wt[0] * fb;
                        else if (k < 4) acc += wt[k] * fa + wt[3 + k] * fb;
                        else acc += wt[3 + k] * fa + wt[9 + k] * fb;
                    }
                    gx[c] += cc * acc;
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) gx[c] = warp_sum(gx[c]);
    sHPS = warp_sum(sHPS);
    __syncwarp();
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) gx[c] += 2.0 * sHPS * dsp * rij[c] / shpoly;
        const double dcn = sHPS / hav0;
        atomicAdd(&grad[3 * iat + 0], gx[0]);
        atomicAdd(&grad[3 * iat + 1], gx[1]);
        atomicAdd(&grad[3 * iat + 2], gx[2]);
        atomicAdd(&grad[3 * jat + 0], -gx[0]);
        atomicAdd(&grad[3 * jat + 1], -gx[1]);
        atomicAdd(&grad[3 * jat + 2], -gx[2]);
        atomicAdd(&dhdcn[iat], dcn * (-m.sh_kcn[ish]));
        atomicAdd(&dhdcn[jat], dcn * (-m.sh_kcn[jsh]));
    }
}

}  // namespace xg
