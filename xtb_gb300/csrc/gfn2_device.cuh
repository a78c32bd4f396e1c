// Device-side bodies shared by the per-molecule kernels and the batched engine.
#pragma once
#include <cmath>
#include "gfn2_kernels.h"

namespace xg {


__device__ __forceinline__ double sq(double x) { return x * x; }
// x^N for the small integer exponents of the pair terms, by multiplication (the reference's
// Fortran x**n with an integer n is evaluated the same way), instead of the general pow
template <int N>
__device__ __forceinline__ double powi(double x) {
    static_assert(N >= 1 && N <= 8, "small integer powers only");
    const double x2 = x * x;
    if constexpr (N == 1) return x;
    else if constexpr (N == 2) return x2;
    else if constexpr (N == 3) return x2 * x;
    else if constexpr (N == 4) return x2 * x2;
    else if constexpr (N == 5) return x2 * x2 * x;
    else if constexpr (N == 6) return x2 * x2 * x2;
    else if constexpr (N == 7) return x2 * x2 * x2 * x;
    else return (x2 * x2) * (x2 * x2);
}


// linear index t -> (a, b) with a >= b of a packed lower triangle
__device__ __forceinline__ void tri_pair(long t, int& a, int& b) {
    long aa = (long)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (aa * (aa + 1) / 2 > t) --aa;
    while ((aa + 1) * (aa + 2) / 2 <= t) ++aa;
    a = (int)aa;
    b = (int)(t - aa * (aa + 1) / 2);
}


// ================================================================== coordination numbers
// getCoordinationNumberLP (src/disp/coordinationnumber.F90:304-479), ncoord_erf / ncoord_d4
// (src/disp/ncoord.f90:469-506, 575-615).
struct CNTerm { double cf, df; };


__device__ __forceinline__ double expc(double k, double r, double r0) { return 1.0 / (1.0 + exp(-k * (r0 / r - 1.0))); }

__device__ __forceinline__ double dexpc(double k, double r, double r0) {
    const double e = exp(-k * (r0 / r - 1.0));
    return (-k * r0 * e) / (r * r * ((e + 1.0) * (e + 1.0)));
}


__device__ __forceinline__ bool cn_term(const DevMol& m, int mode, int i, int j, double r2, CNTerm& t) {
    constexpr double k4 = 4.10451, k5 = 19.08857, k6 = 2 * 11.28174 * 11.28174;
    const double sqrtpi = 1.7724538509055160273;
    if (mode == 0 || mode == 1) {
        if (r2 > 1600.0 || r2 < 1e-12) return false;
    } else {
        if (r2 > 1600.0) return false;
    }
    const double r = sqrt(r2);
    if (mode == 0) {
        const double rc = m.rcov[i] + m.rcov[j];
        t.cf = expc(10.0, r, rc) * expc(20.0, r, rc + 2.0);
        t.df = dexpc(10.0, r, rc) * expc(20.0, r, rc + 2.0) + expc(10.0, r, rc) * dexpc(20.0, r, rc + 2.0);
    } else if (mode == 1) {
        const double rc = m.rcov[i] + m.rcov[j];
        const double den = k4 * exp(-sq(fabs(m.en[i] - m.en[j]) + k5) / k6);
        t.cf = den * 0.5 * (1.0 + erf(-7.5 * (r - rc) / rc));
        t.df = den * (-7.5 / sqrtpi / rc * exp(-56.25 * sq(r - rc) / (rc * rc)));
    } else if (mode == 2) {
        const double rc = m.rcov4[j] + m.rcov4[i];
        t.cf = 0.5 * (1.0 + erf(-7.5 * (r - rc) / rc));
        t.df = 0.0;
    } else {
        const double rc = m.rcov4[j] + m.rcov4[i];
        const double den = k4 * exp(-sq(fabs(m.en4[i] - m.en4[j]) + k5) / k6);
        t.cf = den * 0.5 * (1.0 + erf(-7.5 * (r - rc) / rc));
        t.df = 0.0;
    }
    return true;
}


__device__ inline void d_cn(DevMol m, int mode, double* __restrict__ cn, int i) {
    const double xi = m.xyz[3 * i], yi = m.xyz[3 * i + 1], zi = m.xyz[3 * i + 2];
    double s = 0.0;
    for (int j = 0; j < m.nat; ++j) {
        if (j == i) continue;
        const double r2 = sq(m.xyz[3 * j] - xi) + sq(m.xyz[3 * j + 1] - yi) + sq(m.xyz[3 * j + 2] - zi);
        CNTerm t;
        if (cn_term(m, mode, i, j, r2, t)) s += t.cf;
    }
    cn[i] = s;
}


// Warp-cooperative form of d_cn (one warp per atom, lanes over the partner atoms): the plain
// engine's molecules have hundreds to thousands of atoms, and one thread per atom would leave
// most SMs idle.
__device__ inline void d_cn_warp(DevMol m, int mode, double* __restrict__ cn, int i, int lane) {
    const double xi = m.xyz[3 * i], yi = m.xyz[3 * i + 1], zi = m.xyz[3 * i + 2];
    double s = 0.0;
    for (int j = lane; j < m.nat; j += 32) {
        if (j == i) continue;
        const double r2 = sq(m.xyz[3 * j] - xi) + sq(m.xyz[3 * j + 1] - yi) + sq(m.xyz[3 * j + 2] - zi);
        CNTerm t;
        if (cn_term(m, mode, i, j, r2, t)) s += t.cf;
    }
    s = warp_sum(s);
    if (lane == 0) cn[i] = s;
}

// g[a] += sum_b den*dcount(r_ab)*(R_a - R_b)/r_ab * (v_a + v_b)  ==  sum_b dCN_b/dR_a v_b
__device__ inline void d_cn_chain(DevMol m, int mode, const double* __restrict__ v, double* __restrict__ g, int a) {
    const double xa = m.xyz[3 * a], ya = m.xyz[3 * a + 1], za = m.xyz[3 * a + 2];
    double gx = 0, gy = 0, gz = 0;
    for (int b = 0; b < m.nat; ++b) {
        if (b == a) continue;
        const double dx = xa - m.xyz[3 * b], dy = ya - m.xyz[3 * b + 1], dz = za - m.xyz[3 * b + 2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        CNTerm t;
        if (!cn_term(m, mode, a, b, r2, t)) continue;
        const double f = t.df / sqrt(r2) * (v[a] + v[b]);
        gx += f * dx; gy += f * dy; gz += f * dz;
    }
    g[3 * a] += gx; g[3 * a + 1] += gy; g[3 * a + 2] += gz;
}


// Warp-cooperative form of d_cn_chain (one warp per atom, lanes over the partner atoms).
__device__ inline void d_cn_chain_warp(DevMol m, int mode, const double* __restrict__ v, double* __restrict__ g, int a,
                                       int lane) {
    const double xa = m.xyz[3 * a], ya = m.xyz[3 * a + 1], za = m.xyz[3 * a + 2];
    double gx = 0, gy = 0, gz = 0;
    for (int b = lane; b < m.nat; b += 32) {
        if (b == a) continue;
        const double dx = xa - m.xyz[3 * b], dy = ya - m.xyz[3 * b + 1], dz = za - m.xyz[3 * b + 2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        CNTerm t;
        if (!cn_term(m, mode, a, b, r2, t)) continue;
        const double f = t.df / sqrt(r2) * (v[a] + v[b]);
        gx += f * dx; gy += f * dy; gz += f * dz;
    }
    gx = warp_sum(gx); gy = warp_sum(gy); gz = warp_sum(gz);
    if (lane == 0) { g[3 * a] += gx; g[3 * a + 1] += gy; g[3 * a + 2] += gz; }
}


// ================================================================== EEQ guess
// get_coulomb_matrix_0d and eeq_chrgeq_core (src/eeq_model.f90:60-80, 678-880), 2019 model.
__device__ inline void d_eeq_matrix(DevMol m, const double* __restrict__ cn, double* __restrict__ A, double* __restrict__ X, long t) {
    const int n = m.nat;
    const int i = (int)(t / n), j = (int)(t % n);
    if (i == j) {
        A[t] = m.eeq_gam[i] + sqrt(2.0 / PI) / m.eeq_alpha[i];
        const double tmp = m.eeq_kappa[i] / (sqrt(cn[i]) + 1e-14);
        X[i] = -m.eeq_en[i] + tmp * cn[i];
        X[n + i] = 1.0;
    } else {
        const double r = sqrt(sq(m.xyz[3 * j] - m.xyz[3 * i]) + sq(m.xyz[3 * j + 1] - m.xyz[3 * i + 1]) +
                              sq(m.xyz[3 * j + 2] - m.xyz[3 * i + 2]));
        const double gij = 1.0 / sqrt(sq(m.eeq_alpha[i]) + sq(m.eeq_alpha[j]));
        A[t] = erf(gij * r) / r;
    }
}


// Solve U^T U x = b for two right-hand sides in X[0:n], X[n:2n]; then the charge constraint.
__device__ inline void d_eeq_solve(int n, const double* __restrict__ U, double* __restrict__ X, double charge,
                            double* __restrict__ q) {
    __shared__ double red[32];
    __shared__ double y0, y1;
    double* b0 = X;
    double* b1 = X + n;
    // forward: U^T y = b (row i of U holds column i of U^T)
    for (int i = 0; i < n; ++i) {
        if (threadIdx.x == 0) {
            y0 = b0[i] / U[(size_t)i * n + i];
            y1 = b1[i] / U[(size_t)i * n + i];
            b0[i] = y0;
            b1[i] = y1;
        }
        __syncthreads();
        const double* ur = U + (size_t)i * n;
        for (int k = i + 1 + threadIdx.x; k < n; k += blockDim.x) {
            b0[k] -= ur[k] * y0;
            b1[k] -= ur[k] * y1;
        }
        __syncthreads();
    }
    // backward: U x = y
    for (int i = n - 1; i >= 0; --i) {
        const double* ur = U + (size_t)i * n;
        double s0 = 0.0, s1 = 0.0;
        for (int k = i + 1 + threadIdx.x; k < n; k += blockDim.x) {
            s0 += ur[k] * b0[k];
            s1 += ur[k] * b1[k];
        }
        s0 = block_sum(s0, red);
        s1 = block_sum(s1, red);
        if (threadIdx.x == 0) {
            b0[i] = (b0[i] - s0) / ur[i];
            b1[i] = (b1[i] - s1) / ur[i];
        }
        __syncthreads();
    }
    double sx0 = 0.0, sx1 = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) { sx0 += b0[k]; sx1 += b1[k]; }
    sx0 = block_sum(sx0, red);
    sx1 = block_sum(sx1, red);
    const double lam = (sx0 - charge) / sx1;
    for (int k = threadIdx.x; k < n; k += blockDim.x) q[k] = b0[k] - lam * b1[k];
}


// dE/dCN from the diagonal self energies (src/xtb/hamiltonian.F90:778-786)
__device__ inline void d_dhdcn_diag(DevMol m, const double* __restrict__ P, double* __restrict__ dhdcn, int a) {
    double s = 0.0;
    for (int mu = m.at_ao0[a]; mu < m.at_ao0[a] + m.at_nao[a]; ++mu)
        s += P[(size_t)mu * m.nao + mu] * (-m.sh_kcn[m.ao_sh[mu]]) * EVTOAU;
    dhdcn[a] += s;
}


// ================================================================== isotropic electrostatics
// getCoulombMatrixCluster with arithmetic hardness average (src/coulomb/klopmanohno.F90:257-312, 742-755)
__device__ inline void d_jmat(DevMol m, double* __restrict__ J, long t) {
    const int ns = m.nsh;
    const int s = (int)(t / ns), u = (int)(t % ns);
    const int a = m.sh_atom[s], b = m.sh_atom[u];
    const double gij = 0.5 * (m.sh_eta[s] + m.sh_eta[u]);
    if (a == b) {
        J[t] = (s == u) ? m.sh_eta[s] : gij;
    } else {
        const double r = sqrt(sq(m.xyz[3 * a] - m.xyz[3 * b]) + sq(m.xyz[3 * a + 1] - m.xyz[3 * b + 1]) +
                              sq(m.xyz[3 * a + 2] - m.xyz[3 * b + 2]));
        J[t] = 1.0 / sqrt(r * r + 1.0 / (gij * gij));
    }
}


// shift_s = (J qsh)_s + Gamma_s qsh_s^2 + v_D4[atom(s)]  (TxTBCoulomb%addShift, src/xtb/coulomb.f90:89-114,
// src/xtb/thirdorder.f90:100-131); one warp per shell row
__device__ inline void d_shell_shift(DevMol m, const double* __restrict__ J, const double* __restrict__ qsh,
                              const double* __restrict__ vat, double* __restrict__ shift, double* __restrict__ Jq, int s, int lane) {
    const double* row = J + (size_t)s * m.nsh;
    double acc = 0.0;
    for (int u = lane; u < m.nsh; u += 32) acc = fma(row[u], qsh[u], acc);
    acc = warp_sum(acc);
    if (lane == 0) {
        Jq[s] = acc;
        shift[s] = acc + m.sh_gam3[s] * qsh[s] * qsh[s] + (vat ? vat[m.sh_atom[s]] : 0.0);
    }
}


// ================================================================== anisotropic electrostatics
// get_radcn + mmomgabzero (src/aespot.F90:1219-1281, 1309-1329)
__device__ inline void d_radcn(DevMol m, const double* __restrict__ cn, double* __restrict__ radcn, int i) {
    const double rco = m.mrad[i];
    const double t1 = cn[i] - m.valcn[i] - 1.2;
    radcn[i] = rco + (5.0 - rco) / (1.0 + exp(-4.0 * t1));
}


__device__ inline void d_gab(DevMol m, const double* __restrict__ radcn, double* __restrict__ gab3, double* __restrict__ gab5, long t) {
    const int n = m.nat;
    const int i = (int)(t / n), j = (int)(t % n);
    if (i == j) { gab3[t] = 0.0; gab5[t] = 0.0; return; }
    const double r = sqrt(sq(m.xyz[3 * j] - m.xyz[3 * i]) + sq(m.xyz[3 * j + 1] - m.xyz[3 * i + 1]) +
                          sq(m.xyz[3 * j + 2] - m.xyz[3 * i + 2]));
    const double ri = 1.0 / r;
    const double rco = 0.5 * (radcn[i] + radcn[j]);
    const double d3 = 1.0 / (1.0 + 6.0 * powi<3>(rco * ri));
    const double d5 = 1.0 / (1.0 + 6.0 * powi<4>(rco * ri));
    gab3[t] = d3 * powi<3>(ri);
    gab5[t] = d5 * powi<5>(ri);
}


__device__ __forceinline__ int lin3(int a, int b) {  // packed index of (a,b): xx xy yy xz yz zz
    const int hi = a > b ? a : b, lo = a > b ? b : a;
    return hi * (hi + 1) / 2 + lo;
}


// setvsdq (shifted = true, src/aespot.F90:727-848) / setdvsdq (src/aespot.F90:861-952); one warp per atom
__device__ inline void d_aes_pot(DevMol m, const double* __restrict__ q, const double* __restrict__ dipm,
                          const double* __restrict__ qp, const double* __restrict__ gab3, const double* __restrict__ gab5,
                          int shifted, double* __restrict__ vs, double* __restrict__ vd, double* __restrict__ vq, int i, int lane) {
    const int n = m.nat;
    const double ra[3] = {m.xyz[3 * i], m.xyz[3 * i + 1], m.xyz[3 * i + 2]};
    const double r2a = ra[0] * ra[0] + ra[1] * ra[1] + ra[2] * ra[2];
    double stmp = 0.0, dt[3] = {0, 0, 0}, qt[6] = {0, 0, 0, 0, 0, 0};
    for (int j = lane; j < n; j += 32) {
        const double g3 = gab3[(size_t)j * n + i], g5 = gab5[(size_t)j * n + i];
        if (g3 == 0.0 && g5 == 0.0) continue;
        const double dra[3] = {ra[0] - m.xyz[3 * j], ra[1] - m.xyz[3 * j + 1], ra[2] - m.xyz[3 * j + 2]};
        const double qj = q[j];
        const double* dj = dipm + 3 * j;
        const double* qpj = qp + 6 * j;
        double r2ab = 0, t1a = 0, t2a = 0, t3a = 0, qdd = 0;
        for (int l1 = 0; l1 < 3; ++l1) {
            r2ab += dra[l1] * dra[l1];
            t1a += ra[l1] * dra[l1];
            t2a += dj[l1] * dra[l1];
            t3a += ra[l1] * dj[l1];
            for (int l2 = 0; l2 < 3; ++l2) qdd += qpj[lin3(l1, l2)] * dra[l1] * dra[l2];
        }
        double dum3a, dum5a;
        if (shifted) {
            dum5a = -qdd - 1.5 * qj * t1a * t1a;
            dum3a = -t1a * qj - t2a;
            dum5a += t3a * r2ab - 3.0 * t1a * t2a + 0.5 * qj * r2a * r2ab;
        } else {
            dum3a = -t2a;
            dum5a = -qdd;
        }
        stmp += dum5a * g5 + dum3a * g3;
        for (int l1 = 0; l1 < 3; ++l1) {
            double d5 = 3.0 * dra[l1] * t2a - r2ab * dj[l1];
            if (shifted) d5 += -qj * r2ab * ra[l1] + 3.0 * qj * dra[l1] * t1a;
            dt[l1] += dra[l1] * qj * g3 + d5 * g5;
            qt[l1] += -1.5 * qj * g5 * dra[l1] * dra[l1] + 0.5 * r2ab * qj * g5;
        }
        qt[3] += -3.0 * qj * g5 * dra[0] * dra[1];
        qt[4] += -3.0 * qj * g5 * dra[0] * dra[2];
        qt[5] += -3.0 * qj * g5 * dra[1] * dra[2];
    }
    stmp = warp_sum(stmp);
    for (int k = 0; k < 3; ++k) dt[k] = warp_sum(dt[k]);
    for (int k = 0; k < 6; ++k) qt[k] = warp_sum(qt[k]);
    if (lane != 0) return;
    const double qs1 = m.dkern[i] * 2.0, qs2 = m.qkern[i] * 6.0;
    const double* di = dipm + 3 * i;
    const double* qpi = qp + 6 * i;
    double t3 = 0.0;
    for (int l1 = 0; l1 < 3; ++l1) {
        if (shifted) t3 += ra[l1] * di[l1] * qs1;
        dt[l1] -= qs1 * di[l1];
        for (int l2 = 0; l2 < l1; ++l2) {
            const int ll = lin3(l1, l2), ki = l1 + l2 + 2;
            qt[ki] -= qpi[ll] * qs2;
            if (shifted) {
                t3 -= ra[l1] * ra[l2] * qpi[ll] * qs2;
                dt[l1] += ra[l2] * qpi[ll] * qs2;
                dt[l2] += ra[l1] * qpi[ll] * qs2;
            }
        }
        const int ll = lin3(l1, l1);
        qt[l1] -= qpi[ll] * qs2 * 0.5;
        if (shifted) {
            t3 -= ra[l1] * ra[l1] * qpi[ll] * qs2 * 0.5;
            dt[l1] += ra[l1] * qpi[ll] * qs2;
        }
    }
    if (shifted) stmp += t3;
    const double tr = (qpi[0] + qpi[2] + qpi[5]) * m.qkern[i];
    for (int l1 = 0; l1 < 3; ++l1) {
        qt[l1] += tr;
        if (shifted) {
            dt[l1] -= 2.0 * ra[l1] * tr;
            stmp += tr * ra[l1] * ra[l1];
        }
    }
    vs[i] = stmp;
    for (int k = 0; k < 3; ++k) vd[3 * i + k] = dt[k];
    for (int k = 0; k < 6; ++k) vq[6 * i + k] = qt[k];
}


// aniso_electro_cpu (src/aespot.F90:566-664): e_part[i] = pair terms with j < i, e_part[n+i] = kernel term
__device__ inline void d_aes_energy(DevMol m, const double* __restrict__ q, const double* __restrict__ dipm,
                             const double* __restrict__ qp, const double* __restrict__ gab3,
                             const double* __restrict__ gab5, double* __restrict__ e_part, int i, int lane) {
    const int n = m.nat;
    const double* di = dipm + 3 * i;
    const double* qi = qp + 6 * i;
    double e = 0.0;
    for (int j = lane; j < i; j += 32) {
        const double rij[3] = {m.xyz[3 * j] - m.xyz[3 * i], m.xyz[3 * j + 1] - m.xyz[3 * i + 1],
                               m.xyz[3 * j + 2] - m.xyz[3 * i + 2]};
        const double r2 = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
        const double* dj = dipm + 3 * j;
        const double* qj = qp + 6 * j;
        double ed = 0, eq = 0, edd = 0;
        for (int k = 0; k < 3; ++k) {
            ed += q[j] * di[k] * rij[k] - dj[k] * q[i] * rij[k];
            for (int l = 0; l < 3; ++l) {
                const int kl = lin3(l, k);
                const double tt = rij[l] * rij[k];
                eq += q[j] * qi[kl] * tt + qj[kl] * q[i] * tt;
                edd -= dj[k] * di[l] * 3.0 * tt;
            }
            edd += dj[k] * di[k] * r2;
        }
        e += ed * gab3[(size_t)j * n + i] + (eq + edd) * gab5[(size_t)j * n + i];
    }
    e = warp_sum(e);
    if (lane == 0) {
        double tt = di[0] * di[0] + di[1] * di[1] + di[2] * di[2];
        double tt3 = 0.0;
        for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l) tt3 += qi[lin3(l, k)] * qi[lin3(l, k)];
        e_part[i] = e;
        e_part[n + i] = m.dkern[i] * tt + tt3 * m.qkern[i];
    }
}


// aniso_grad (src/aespot.F90:1060-1165); tmp2[i] collects the radius-derivative prefactor
__device__ inline void d_aes_grad(DevMol m, const double* __restrict__ q, const double* __restrict__ dipm,
                           const double* __restrict__ qp, const double* __restrict__ radcn,
                           const double* __restrict__ gab3, const double* __restrict__ gab5, double* __restrict__ grad,
                           double* __restrict__ tmp2, int i, int lane) {
    const int n = m.nat;
    const double* di = dipm + 3 * i;
    const double* Qi = qp + 6 * i;
    double g[3] = {0, 0, 0}, t2 = 0.0;
    for (int j = lane; j < n; j += 32) {
        if (j == i) continue;
        const double rij[3] = {m.xyz[3 * j] - m.xyz[3 * i], m.xyz[3 * j + 1] - m.xyz[3 * i + 1],
                               m.xyz[3 * j + 2] - m.xyz[3 * i + 2]};
        const double r2 = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
        const double rabi = 1.0 / sqrt(r2);
        const double rco = 0.5 * (radcn[i] + radcn[j]);
        const double damp1 = 1.0 / (1.0 + 6.0 * powi<3>(rco * rabi));
        const double dd1 = -3.0 * rabi * (damp1 * damp1 - damp1);
        const double r3 = powi<3>(rabi), r5 = powi<5>(rabi);
        const double dgab3 = (-3.0 * rabi * r3) * damp1 + dd1 * r3;
        const double damp2 = 1.0 / (1.0 + 6.0 * powi<4>(rco * rabi));
        const double dd2 = -4.0 * rabi * (damp2 * damp2 - damp2);
        const double dgab5 = (-5.0 * rabi * r5) * damp2 + dd2 * r5;
        const double G3 = gab3[(size_t)j * n + i], G5 = gab5[(size_t)j * n + i];
        const double* dj = dipm + 3 * j;
        const double* Qj = qp + 6 * j;
        double ed = 0, eq = 0, edd = 0;
        for (int k = 0; k < 3; ++k) {
            ed += q[j] * di[k] * rij[k] - dj[k] * q[i] * rij[k];
            g[k] += G3 * (q[i] * dj[k] - q[j] * di[k]);
            double ddm2 = 0, ddm3a = 0, ddm3b = 0, qqa = 0, qqb = 0;
            for (int l = 0; l < 3; ++l) {
                const int kl = lin3(l, k);
                const double tt = rij[l] * rij[k];
                eq += q[j] * Qi[kl] * tt + Qj[kl] * q[i] * tt;
                edd -= dj[k] * di[l] * 3.0 * tt;
                ddm2 += dj[l] * di[l];
                ddm3a += di[l] * rij[l];
                ddm3b += dj[l] * rij[l];
                qqa += rij[l] * Qj[kl];
                qqb += rij[l] * Qi[kl];
            }
            edd += dj[k] * di[k] * r2;
            g[k] += -2.0 * G5 * ddm2 * rij[k] + 3.0 * G5 * ddm3a * dj[k] + 3.0 * G5 * ddm3b * di[k] -
                    2.0 * G5 * qqa * q[i] - 2.0 * G5 * qqb * q[j];
        }
        for (int k = 0; k < 3; ++k) {
            const double dxi = rij[k] * rabi;
            g[k] -= ed * dgab3 * dxi + (eq + edd) * dgab5 * dxi;
        }
        const double rab = 0.5 * (radcn[i] + radcn[j]);
        t2 += ed * 3.0 * G3 * (damp1 / rab) * powi<3>(rab * rabi) + (eq + edd) * 4.0 * G5 * (damp2 / rab) * powi<4>(rab * rabi);
    }
    for (int k = 0; k < 3; ++k) g[k] = warp_sum(g[k]);
    t2 = warp_sum(t2);
    if (lane == 0) {
        grad[3 * i] += g[0];
        grad[3 * i + 1] += g[1];
        grad[3 * i + 2] += g[2];
        tmp2[i] = 3.0 * t2;
    }
}


// dradcn (src/aespot.F90:1292-1307): dhdcn[i] -= tmp2[i] * dR0_i/dCN_i (chain through the gfn CN)
__device__ inline void d_aes_dradcn(DevMol m, const double* __restrict__ cn, const double* __restrict__ tmp2,
                             double* __restrict__ dhdcn, int i) {
    const double rco = m.mrad[i];
    const double t1 = exp(-4.0 * (cn[i] - m.valcn[i] - 1.2));
    double t2 = (5.0 - rco) / (1.0 + 2.0 * t1 + t1 * t1);
    t2 = t2 * 4.0 * t1;
    dhdcn[i] -= tmp2[i] * t2;
}


// ================================================================== Hamiltonian build
// buildIsoAnisotropicH1 (src/scc_core.f90:154-251) with the setdqlist screening (src/aespot.F90:34-85)
__device__ inline void d_build_h(DevMol m, double neglect, const double* __restrict__ H0, const double* __restrict__ S,
                          const double* __restrict__ D, const double* __restrict__ Q, const double* __restrict__ shift,
                          const double* __restrict__ vs, const double* __restrict__ vd, const double* __restrict__ vq,
                          double* __restrict__ H, size_t t) {
    const size_t nao = m.nao, nn = nao * nao;
    const int i = (int)(t / nao), j = (int)(t % nao);
    const int si = m.ao_sh[i], sj = m.ao_sh[j], ai = m.ao_at[i], aj = m.ao_at[j];
    const double dum = S[t] * AUTOEV * 0.5;
    double h = H0[t] - dum * (shift[si] + shift[sj]) + dum * (vs[ai] + vs[aj]);
    const double thr2 = neglect * 1.0e-2;
    double d[3], tmp1 = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) { d[k] = D[k * nn + t]; tmp1 += d[k] * d[k]; }
    if (tmp1 > thr2) {
        double e = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) e += d[k] * (vd[3 * ai + k] + vd[3 * aj + k]);
        h += 0.5 * e * AUTOEV;
    }
    double qq[6], tmp2 = 0.0;
#pragma unroll
    for (int k = 0; k < 6; ++k) { qq[k] = Q[k * nn + t]; tmp2 += (k < 3 ? 1.0 : 2.0) * qq[k] * qq[k]; }
    if (tmp2 > thr2) {
        double e = 0.0;
#pragma unroll
        for (int k = 0; k < 6; ++k) e += qq[k] * (vq[6 * ai + k] + vq[6 * aj + k]);
        h += 0.5 * e * AUTOEV;
    }
    H[t] = h;
}


// ================================================================== Fermi smearing
// fermismear (src/scc_core.f90:983-1064) for one spin channel; one block.
__device__ inline void fermi_channel(int n, const double* emo, int nel, double etemp, double* occ, double* red,
                              double& s_out, double& ef_out) {
    const double bkt = KB_AU * AUTOEV * etemp;
    const double thr = 1e-9;
    double ef;
    if (nel + 1 > n) {
        // no LUMO: the integer occupations of occu are kept (src/scc_core.f90:1001-1004)
        ef = emo[nel - 1];
        for (int i = threadIdx.x; i < n; i += blockDim.x) occ[i] = (i < nel) ? 1.0 : 0.0;
    } else if (nel == 0) {
        ef = emo[0];
        for (int i = threadIdx.x; i < n; i += blockDim.x) occ[i] = 0.0;
    } else {
        ef = 0.5 * (emo[nel - 1] + emo[nel]);
        const double occt = (double)nel;
        for (int cyc = 0; cyc < 200; ++cyc) {
            double tot = 0.0, totd = 0.0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const double x = (emo[i] - ef) / bkt;
                double f = 0.0, df = 0.0;
                if (x < 50.0) {
                    const double ex = exp(x);
                    f = 1.0 / (ex + 1.0);
                    df = ex / (bkt * (ex + 1.0) * (ex + 1.0));
                }
                occ[i] = f;
                tot += f;
                totd += df;
            }
            tot = block_sum(tot, red);
            totd = block_sum(totd, red);
            ef += (occt - tot) / totd;
            if (fabs(occt - tot) <= thr) break;
        }
    }
    __syncthreads();
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double o = occ[i];
        if (o > thr && 1.0 - o > thr) s += o * log(o) + (1.0 - o) * log(1.0 - o);
    }
    s = block_sum(s, red);
    s_out = s * KB_AU * etemp;
    ef_out = ef;
}


__device__ inline void d_fermi(int n, const double* __restrict__ emo, int nel_a, int nel_b, double etemp,
                        double* __restrict__ focc, double* __restrict__ fa, double* __restrict__ fb,
                        double* __restrict__ scal, int* __restrict__ kocc) {
    __shared__ double red[32];
    __shared__ int kmax;
    double sa, efa, sb, efb;
    fermi_channel(n, emo, nel_a, etemp, fa, red, sa, efa);
    if (nel_b == nel_a) {
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) fb[i] = fa[i];
        sb = sa;
        efb = efa;
    } else {
        fermi_channel(n, emo, nel_b, etemp, fb, red, sb, efb);
    }
    if (threadIdx.x == 0) kmax = max(nel_a, nel_b);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double f = fa[i] + fb[i];
        focc[i] = f;
        if (f > 0.0) atomicMax(&kmax, i + 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        kocc[0] = min(kmax, n);
        scal[0] = sa + sb;
        scal[1] = efa;
        scal[2] = efb;
    }
}


__device__ inline void d_scale_cols(int n, const double* __restrict__ C, const double* __restrict__ f, double* __restrict__ Cf, size_t t) {
    const double fj = f[t % n];
    Cf[t] = (fj == 0.0) ? 0.0 : C[t] * fj;     // exact zeros for unoccupied columns
}


// ================================================================== populations
// mpopsh + qsh2qat + mmompop_cpu + the H0 energy sum (src/scc_core.f90:1408-1444, src/aespot.F90:288-428,
// src/scc_core.f90:686-722).  Pass 1: one warp per AO row computes 11 row sums.
__device__ inline void d_rowsums(DevMol m, const double* __restrict__ P, const double* __restrict__ S,
                          const double* __restrict__ D, const double* __restrict__ Q, const double* __restrict__ H0,
                          double* __restrict__ rows, int mu, int lane) {
    const size_t nao = m.nao, nn = nao * nao, off = (size_t)mu * nao;
    double acc[11];
#pragma unroll
    for (int k = 0; k < 11; ++k) acc[k] = 0.0;
    for (int nu = lane; nu < m.nao; nu += 32) {
        const double p = P[off + nu];
        acc[0] += p * S[off + nu];
#pragma unroll
        for (int k = 0; k < 3; ++k) acc[1 + k] += p * D[k * nn + off + nu];
#pragma unroll
        for (int k = 0; k < 6; ++k) acc[4 + k] += p * Q[k * nn + off + nu];
        acc[10] += p * H0[off + nu];
    }
#pragma unroll
    for (int k = 0; k < 11; ++k) acc[k] = warp_sum(acc[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < 11; ++k) rows[(size_t)mu * 12 + k] = acc[k];
}


// The same row sums by one thread per row, for the small matrices of the batched engine: a warp
// FP64 instruction costs the same with any number of lanes active, and at n ~ 100 the eleven
// five-level shuffle sums of the warp form outweigh the products.
__device__ inline void d_rowsums_thread(DevMol m, const double* __restrict__ P, const double* __restrict__ S,
                                       const double* __restrict__ D, const double* __restrict__ Q,
                                       const double* __restrict__ H0, double* __restrict__ rows, int mu) {
    const size_t nao = m.nao, nn = nao * nao, off = (size_t)mu * nao;
    double acc[11];
#pragma unroll
    for (int k = 0; k < 11; ++k) acc[k] = 0.0;
    for (int nu = 0; nu < m.nao; ++nu) {
        const double p = P[off + nu];
        acc[0] = fma(p, S[off + nu], acc[0]);
#pragma unroll
        for (int k = 0; k < 3; ++k) acc[1 + k] = fma(p, D[k * nn + off + nu], acc[1 + k]);
#pragma unroll
        for (int k = 0; k < 6; ++k) acc[4 + k] = fma(p, Q[k * nn + off + nu], acc[4 + k]);
        acc[10] = fma(p, H0[off + nu], acc[10]);
    }
#pragma unroll
    for (int k = 0; k < 11; ++k) rows[(size_t)mu * 12 + k] = acc[k];
}


// Pass 2: one thread per atom.
__device__ inline void d_atom_pop(DevMol m, const double* __restrict__ rows, double* __restrict__ qsh, double* __restrict__ q,
                           double* __restrict__ dipm, double* __restrict__ qp, double* __restrict__ eh0, int a) {
    const double R[3] = {m.xyz[3 * a], m.xyz[3 * a + 1], m.xyz[3 * a + 2]};
    double qa = 0.0, e = 0.0;
    double dp[3] = {0, 0, 0}, qq[6] = {0, 0, 0, 0, 0, 0};
    for (int s = m.at_sh0[a]; s < m.at_sh0[a] + m.at_nsh[a]; ++s) {
        double pop = 0.0;
        const int nfun = 2 * m.sh_l[s] + 1;
        for (int mu = m.sh_ao[s]; mu < m.sh_ao[s] + nfun; ++mu) {
            const double* r = rows + (size_t)mu * 12;
            pop += r[0];
            e += r[10];
            for (int k = 0; k < 3; ++k) dp[k] += R[k] * r[0] - r[1 + k];
            // packed (xx, xy, yy, xz, yz, zz); qpint order xx yy zz xy xz yz
            const int qidx[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l <= k; ++l) {
                    const int kl = k * (k + 1) / 2 + l;
                    double t;
                    if (k == l) t = 2.0 * r[1 + k] * R[k] - R[k] * R[k] * r[0] - r[4 + qidx[k][k]];
                    else t = r[1 + k] * R[l] + r[1 + l] * R[k] - R[l] * R[k] * r[0] - r[4 + qidx[k][l]];
                    qq[kl] += t;
                }
        }
        const double v = m.sh_zsh[s] - pop;
        qsh[s] = v;
        qa += v;
    }
    q[a] = qa;
    const double tr = 0.5 * (qq[0] + qq[2] + qq[5]);
    for (int k = 0; k < 6; ++k) qq[k] *= 1.5;
    qq[0] -= tr; qq[2] -= tr; qq[5] -= tr;
    for (int k = 0; k < 3; ++k) dipm[3 * a + k] = dp[k];
    for (int k = 0; k < 6; ++k) qp[6 * a + k] = qq[k];
    eh0[a] = e;
}


__device__ inline void d_reduce(const double* __restrict__ x, int n, double* __restrict__ out) {
    __shared__ double red[32];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += x[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) *out = s;
}


// One block: dq = qout - qin, rms, Broyden update of qin in place.
__device__ inline void d_broyden(int nbr, int it, int maxit, double alpha, double* __restrict__ qin,
                          const double* __restrict__ qout, double* __restrict__ dq, double* __restrict__ df,
                          double* __restrict__ u, double* __restrict__ amat, double* __restrict__ omega,
                          double* __restrict__ qlast, double* __restrict__ dqlast, double* __restrict__ work,
                          double* __restrict__ rms_out, int nat) {
    __shared__ double red[32];
    __shared__ double s_inv;
    double ss = 0.0;
    for (int i = threadIdx.x; i < nbr; i += blockDim.x) {
        const double d = qout[i] - qin[i];
        dq[i] = d;
        ss += d * d;
    }
    ss = block_sum(ss, red);
    if (threadIdx.x == 0) { rms_out[0] = sqrt(ss / (double)nat); rms_out[1] = ss; }
    if (it == 1) {
        for (int i = threadIdx.x; i < nbr; i += blockDim.x) {
            dqlast[i] = dq[i];
            qlast[i] = qin[i];
            qin[i] += alpha * dq[i];
        }
        return;
    }
    const int it1 = it - 1, r = it1 - 1;   // new history row r (0-based)
    const double omega0 = 0.01, minw = 1.0, maxw = 100000.0, wfac = 0.01;
    double om = sqrt(ss);
    om = (om > wfac / maxw) ? wfac / om : maxw;
    if (om < minw) om = minw;
    double* dfr = df + (size_t)r * nbr;
    double n2 = 0.0;
    for (int i = threadIdx.x; i < nbr; i += blockDim.x) {
        const double d = dq[i] - dqlast[i];
        dfr[i] = d;
        n2 += d * d;
    }
    n2 = block_sum(n2, red);
    if (threadIdx.x == 0) { omega[r] = om; s_inv = 1.0 / sqrt(n2); }
    __syncthreads();
    const double inv = s_inv;
    for (int i = threadIdx.x; i < nbr; i += blockDim.x) dfr[i] *= inv;
    __syncthreads();
    // a(i, r) for i <= r, c(i) = omega_i df_i . dq: one warp per history row, warp sums only
    double* c = work;                      // [maxit]
    double* beta = work + maxit;           // [it1 x it1]
    double* binv = beta + (size_t)maxit * maxit;
    {
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int i = wid; i < it1; i += nw) {
            const double* dfi = df + (size_t)i * nbr;
            double s1 = 0.0, s2 = 0.0;
            for (int k = lane; k < nbr; k += 32) {
                s1 += dfi[k] * dfr[k];
                s2 += dfi[k] * dq[k];
            }
            s1 = warp_sum(s1);
            s2 = warp_sum(s2);
            if (lane == 0) {
                amat[(size_t)i * maxit + r] = s1;
                amat[(size_t)r * maxit + i] = s1;
                c[i] = omega[i] * s2;
            }
        }
    }
    __syncthreads();
    // beta = omega_i omega_j a_ij + omega0^2 delta_ij, inverted by Gauss-Jordan with partial
    // pivoting; the history is short, so one warp does it with warp barriers only
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        for (int t = lane; t < it1 * it1; t += 32) {
            const int i = t / it1, j = t % it1;
            beta[t] = omega[i] * omega[j] * amat[(size_t)i * maxit + j] + (i == j ? omega0 * omega0 : 0.0);
            binv[t] = (i == j) ? 1.0 : 0.0;
        }
        __syncwarp();
        for (int k = 0; k < it1; ++k) {
            // pivot: the row of largest magnitude in column k (first one on ties)
            int p = k;
            double best = -1.0;
            for (int i = k + lane; i < it1; i += 32) {
                const double v = fabs(beta[i * it1 + k]);
                if (v > best) { best = v; p = i; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int op = __shfl_xor_sync(0xffffffffu, p, o);
                if (ob > best || (ob == best && op < p)) { best = ob; p = op; }
            }
            if (p != k)
                for (int j = lane; j < it1; j += 32) {
                    double t1 = beta[k * it1 + j]; beta[k * it1 + j] = beta[p * it1 + j]; beta[p * it1 + j] = t1;
                    double t2 = binv[k * it1 + j]; binv[k * it1 + j] = binv[p * it1 + j]; binv[p * it1 + j] = t2;
                }
            __syncwarp();
            const double pk = beta[k * it1 + k];
            __syncwarp();
            for (int j = lane; j < it1; j += 32) { beta[k * it1 + j] /= pk; binv[k * it1 + j] /= pk; }
            __syncwarp();
            for (int t = lane; t < it1 * it1; t += 32) {
                const int i = t / it1, j = t % it1;
                if (i == k) continue;
                const double f = beta[i * it1 + k];
                if (j != k) beta[t] -= f * beta[k * it1 + j];
                binv[t] -= f * binv[k * it1 + j];
            }
            __syncwarp();
            for (int i = lane; i < it1; i += 32)
                if (i != k) beta[i * it1 + k] = 0.0;
            __syncwarp();
        }
    }
    __syncthreads();
    // gamma_j = sum_i c_i binv_ij ; store omega_j * gamma_j in work tail
    double* og = binv + (size_t)maxit * maxit;
    for (int j = threadIdx.x; j < it1; j += blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < it1; ++i) s += c[i] * binv[i * it1 + j];
        og[j] = omega[j] * s;
    }
    __syncthreads();
    double* ur = u + (size_t)r * nbr;
    for (int k = threadIdx.x; k < nbr; k += blockDim.x) {
        const double qi = qin[k];
        ur[k] = alpha * dfr[k] + inv * (qi - qlast[k]);
        dqlast[k] = dq[k];
        qlast[k] = qi;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nbr; k += blockDim.x) {
        double v = qin[k] + alpha * dq[k];
        for (int i = 0; i < it1; ++i) v -= og[i] * u[(size_t)i * nbr + k];
        qin[k] = v;
    }
}


// ================================================================== repulsion
// repulsionEnGrad_latp, molecular case (src/xtb/repulsion.F90:41-158)
__device__ inline void d_repulsion(DevMol m, double* __restrict__ e_atom, double* __restrict__ grad, int a) {
    double e = 0.0, g[3] = {0, 0, 0};
    for (int b = 0; b < m.nat; ++b) {
        if (b == a) continue;
        const double rij[3] = {m.xyz[3 * a] - m.xyz[3 * b], m.xyz[3 * a + 1] - m.xyz[3 * b + 1],
                               m.xyz[3 * a + 2] - m.xyz[3 * b + 2]};
        const double r2 = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
        if (r2 > 1600.0 || r2 < 1e-8) continue;
        const double r1 = sqrt(r2);
        const double alpha = sqrt(m.rep_alpha[a] * m.rep_alpha[b]);
        const double zeff = m.rep_zeff[a] * m.rep_zeff[b];
        const double kexp = (m.Z[a] > 2 || m.Z[b] > 2) ? 1.5 : 1.0;
        const double t16 = pow(r1, kexp);
        const double t26 = exp(-alpha * t16);
        const double dE = zeff * t26 / r1;
        const double f = -(alpha * t16 * kexp + 1.0) * dE / r2;
        e += 0.5 * dE;
        for (int k = 0; k < 3; ++k) g[k] += f * rij[k];
    }
    e_atom[a] = e;
    for (int k = 0; k < 3; ++k) grad[3 * a + k] += g[k];
}


// Warp-cooperative form of d_repulsion for the plain engine (one warp per atom).
__device__ inline void d_repulsion_warp(DevMol m, double* __restrict__ e_atom, double* __restrict__ grad, int a,
                                        int lane) {
    double e = 0.0, g[3] = {0, 0, 0};
    for (int b = lane; b < m.nat; b += 32) {
        if (b == a) continue;
        const double rij[3] = {m.xyz[3 * a] - m.xyz[3 * b], m.xyz[3 * a + 1] - m.xyz[3 * b + 1],
                               m.xyz[3 * a + 2] - m.xyz[3 * b + 2]};
        const double r2 = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
        if (r2 > 1600.0 || r2 < 1e-8) continue;
        const double r1 = sqrt(r2);
        const double alpha = sqrt(m.rep_alpha[a] * m.rep_alpha[b]);
        const double zeff = m.rep_zeff[a] * m.rep_zeff[b];
        const double kexp = (m.Z[a] > 2 || m.Z[b] > 2) ? 1.5 : 1.0;
        const double t16 = (m.Z[a] > 2 || m.Z[b] > 2) ? r1 * sqrt(r1) : r1;   // r^kexp
        const double t26 = exp(-alpha * t16);
        const double dE = zeff * t26 / r1;
        const double f = -(alpha * t16 * kexp + 1.0) * dE / r2;
        e += 0.5 * dE;
        for (int k = 0; k < 3; ++k) g[k] += f * rij[k];
    }
    e = warp_sum(e);
    for (int k = 0; k < 3; ++k) g[k] = warp_sum(g[k]);
    if (lane == 0) {
        e_atom[a] = e;
        for (int k = 0; k < 3; ++k) grad[3 * a + k] += g[k];
    }
}


// ================================================================== Coulomb gradient
// getCoulombDerivsCluster contracted with qsh (src/coulomb/klopmanohno.F90:471-573); warp per atom
__device__ inline void d_coulomb_grad(DevMol m, const double* __restrict__ qsh, double* __restrict__ grad, int a, int lane) {
    double g[3] = {0, 0, 0};
    for (int b = lane; b < m.nat; b += 32) {
        if (b == a) continue;
        const double vec[3] = {m.xyz[3 * b] - m.xyz[3 * a], m.xyz[3 * b + 1] - m.xyz[3 * a + 1],
                               m.xyz[3 * b + 2] - m.xyz[3 * a + 2]};
        const double r2 = vec[0] * vec[0] + vec[1] * vec[1] + vec[2] * vec[2];
        double f = 0.0;
        for (int s = m.at_sh0[a]; s < m.at_sh0[a] + m.at_nsh[a]; ++s)
            for (int u = m.at_sh0[b]; u < m.at_sh0[b] + m.at_nsh[b]; ++u) {
                const double gij = 0.5 * (m.sh_eta[s] + m.sh_eta[u]);
                const double g1 = 1.0 / (r2 + 1.0 / (gij * gij));
                f += g1 * sqrt(g1) * qsh[s] * qsh[u];
            }
        for (int k = 0; k < 3; ++k) g[k] += f * vec[k];
    }
    for (int k = 0; k < 3; ++k) g[k] = warp_sum(g[k]);
    if (lane == 0)
        for (int k = 0; k < 3; ++k) grad[3 * a + k] += g[k];
}


// ================================================================== D4 dispersion
__device__ __forceinline__ double zeta_fn(double a, double c, double qref, double qmod) {
    if (qmod < 0.0) return exp(a);
    return exp(a * (1.0 - exp(c * (1.0 - qref / qmod))));
}

__device__ __forceinline__ double dzeta_fn(double a, double c, double qref, double qmod) {
    if (qmod < 0.0) return 0.0;
    return -a * c * exp(c * (1.0 - qref / qmod)) * zeta_fn(a, c, qref, qmod) * qref / (qmod * qmod);
}


// Gaussian CN weights of the reference systems: d4 (src/disp/dftd4.F90:588-657) and
// weight_references (:948-1065); gw[a*MAXREF + r], dgw = d gw / d CN
__device__ inline void d_d4_weights(DevMol m, const double* __restrict__ cnv, double* __restrict__ gw, double* __restrict__ dgw, int a) {
    const int e = m.eid[a];
    const int nref = m.d4_nref[e];
    const double wf = 6.0;
    double expw[MAXREF], expd[MAXREF], norm = 0.0, dnorm = 0.0, rmax = -1e300;
    for (int r = 0; r < nref; ++r) {
        const double rcn = m.d4_refcn[e * MAXREF + r];
        rmax = fmax(rmax, rcn);
        expw[r] = 0.0;
        expd[r] = 0.0;
        for (int c = 1; c <= m.d4_ncount[e * MAXREF + r]; ++c) {
            const double twf = c * wf;
            const double val = -twf * sq(cnv[a] - rcn);
            const double g = (val < -200.0) ? 0.0 : exp(val);
            expw[r] += g;
            expd[r] += 2.0 * twf * (rcn - cnv[a]) * g;
        }
        norm += expw[r];
        dnorm += expd[r];
    }
    norm = (norm > 1e-80) ? 1.0 / norm : 0.0;
    for (int r = 0; r < MAXREF; ++r) {
        double g = 0.0, dg = 0.0;
        if (r < nref) {
            g = expw[r] * norm;
            dg = expd[r] * norm - expw[r] * dnorm * norm * norm;
            if (norm == 0.0) g = (fabs(rmax - m.d4_refcn[e * MAXREF + r]) < 1e-12) ? 1.0 : 0.0;
        }
        gw[a * MAXREF + r] = g;
        if (dgw) dgw[a * MAXREF + r] = dg;
    }
}


// zeta / dzeta of the SCC dispersion (disppot, src/disp/dftd4.F90:735-818)
__device__ inline void d_d4_zeta(DevMol m, const double* __restrict__ gw, const double* __restrict__ q,
                          double* __restrict__ zeta, double* __restrict__ dzeta, int a) {
    const int e = m.eid[a];
    const double iz = m.d4_zeff[e], gi = m.d4_gam[e] * 2.0;
    for (int r = 0; r < MAXREF; ++r) {
        double z = 0.0, dz = 0.0;
        if (r < m.d4_nref[e] && gw[a * MAXREF + r] >= 1e-7) {
            const double qref = m.d4_refq[e * MAXREF + r] + iz;
            z = zeta_fn(3.0, gi, qref, q[a] + iz);
            dz = dzeta_fn(3.0, gi, qref, q[a] + iz);
        }
        zeta[a * MAXREF + r] = z;
        dzeta[a * MAXREF + r] = dz;
    }
}


// (W zeta) for atom a, W = build_wdispmat (src/disp/dftd4.F90:660-732) evaluated on the fly; warp per atom
__device__ inline void d_d4_wz(DevMol m, const double* __restrict__ gw, const double* __restrict__ zeta,
                        const double* __restrict__ dzeta, double* __restrict__ Wz, double* __restrict__ vat,
                        double* __restrict__ e_atom, int a, int lane) {
    const int ea = m.eid[a], na = m.d4_nref[ea];
    double acc[MAXREF];
    for (int r = 0; r < MAXREF; ++r) acc[r] = 0.0;
    for (int b = lane; b < m.nat; b += 32) {
        if (b == a) continue;
        const double r2 = sq(m.xyz[3 * a] - m.xyz[3 * b]) + sq(m.xyz[3 * a + 1] - m.xyz[3 * b + 1]) +
                          sq(m.xyz[3 * a + 2] - m.xyz[3 * b + 2]);
        if (r2 > 72.0 * 72.0) continue;
        const double r4r2 = 3.0 * m.r4r2[a] * m.r4r2[b];
        const double cut = 0.52 * sqrt(r4r2) + 5.0;
        const double cut2 = cut * cut, cut6 = cut2 * cut2 * cut2, r6 = r2 * r2 * r2;
        const double oor6 = rcp_fast(r6 + cut6);
        const double oor8 = rcp_fast(r6 * r2 + cut6 * cut2);
        const double h = oor6 + 2.7 * r4r2 * oor8;   // -(C6 oor6 + 2.7 r4r2 C6 oor8) = -C6 h
        const int eb = m.eid[b], nb = m.d4_nref[eb];
        const double* c6 = m.d4_c6 + ((size_t)(ea * m.nelem + eb) * MAXREF) * MAXREF;
        for (int r = 0; r < na; ++r) {
            const double gr = gw[a * MAXREF + r];
            double s = 0.0;
            for (int u = 0; u < nb; ++u) {
                const double gg = gr * gw[b * MAXREF + u];
                if (gg < 1e-7) continue;
                s = fma(gg * c6[r * MAXREF + u], zeta[b * MAXREF + u], s);
            }
            acc[r] -= h * s;
        }
    }
    double v = 0.0, e = 0.0;
    for (int r = 0; r < MAXREF; ++r) {
        const double t = warp_sum(acc[r]);
        if (lane == 0 && r < na) {
            Wz[a * MAXREF + r] = t;
            v += t * dzeta[a * MAXREF + r];
            e += 0.5 * t * zeta[a * MAXREF + r];
        }
    }
    if (lane == 0) {
        vat[a] = v;
        e_atom[a] = e;
    }
}


// weight_references: zeta-weighted vectors for q and for q = 0 (src/disp/dftd4.F90:948-1065)
__device__ inline void d_d4_refvec(DevMol m, const double* __restrict__ gw, const double* __restrict__ dgw,
                            const double* __restrict__ q, double* __restrict__ zv, double* __restrict__ zr,
                            double* __restrict__ zdcn, double* __restrict__ zrdcn, int a) {
    const int e = m.eid[a];
    const double zi = m.d4_zeff[e], gi = 2.0 * m.d4_gam[e];
    for (int r = 0; r < MAXREF; ++r) {
        double v0 = 0, v1 = 0, v2 = 0, v3 = 0;
        if (r < m.d4_nref[e]) {
            const double qref = m.d4_refq[e * MAXREF + r] + zi;
            const double zq = zeta_fn(3.0, gi, qref, q[a] + zi);
            const double z0 = zeta_fn(3.0, gi, qref, zi);
            const double g = gw[a * MAXREF + r], dg = dgw[a * MAXREF + r];
            v0 = zq * g; v1 = z0 * g; v2 = zq * dg; v3 = z0 * dg;
        }
        zv[a * MAXREF + r] = v0; zr[a * MAXREF + r] = v1; zdcn[a * MAXREF + r] = v2; zrdcn[a * MAXREF + r] = v3;
    }
}


// get_atomic_c6 (src/disp/dftd4.F90:1069-1147): c6[a][b], dc6[a][b] = d c6_ab / d CN_a
__device__ inline void d_d4_c6(DevMol m, const double* __restrict__ zv, const double* __restrict__ zdcn,
                        double* __restrict__ c6o, double* __restrict__ dc6o, long t) {
    const int n = m.nat;
    const int a = (int)(t / n), b = (int)(t % n);
    const int ea = m.eid[a], eb = m.eid[b];
    const double* c6 = m.d4_c6 + ((size_t)(ea * m.nelem + eb) * MAXREF) * MAXREF;
    double c = 0.0, d = 0.0;
    for (int r = 0; r < m.d4_nref[ea]; ++r)
        for (int u = 0; u < m.d4_nref[eb]; ++u) {
            const double ref = c6[r * MAXREF + u];
            c += zv[a * MAXREF + r] * zv[b * MAXREF + u] * ref;
            d += zdcn[a * MAXREF + r] * zv[b * MAXREF + u] * ref;
        }
    c6o[t] = c;
    dc6o[t] = d;
}


// two-body dispersion energy / gradient (disp_gradient_latp, src/disp/dftd4.F90:1832-1933); thread per atom
__device__ inline void d_d4_2body(DevMol m, const double* __restrict__ c6, const double* __restrict__ dc6,
                           double* __restrict__ e_atom, double* __restrict__ dEdcn, double* __restrict__ grad, int a) {
    const int n = m.nat;
    double e = 0.0, dcn = 0.0, g[3] = {0, 0, 0};
    for (int b = 0; b < n; ++b) {
        if (b == a) continue;
        const double rij[3] = {m.xyz[3 * a] - m.xyz[3 * b], m.xyz[3 * a + 1] - m.xyz[3 * b + 1],
                               m.xyz[3 * a + 2] - m.xyz[3 * b + 2]};
        const double r2 = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
        if (r2 > 3600.0 || r2 < 1e-10) continue;
        const double r4r2 = 3.0 * m.r4r2[a] * m.r4r2[b];
        const double r0 = 0.52 * sqrt(r4r2) + 5.0;
        const double t6 = 1.0 / (r2 * r2 * r2 + powi<6>(r0));
        const double t8 = 1.0 / (r2 * r2 * r2 * r2 + powi<8>(r0));
        const double d6 = -6.0 * r2 * r2 * t6 * t6;
        const double d8 = -8.0 * r2 * r2 * r2 * t8 * t8;
        const double disp = 1.0 * t6 + 2.7 * r4r2 * t8;
        const double ddisp = 1.0 * d6 + 2.7 * r4r2 * d8;
        const double cab = c6[(size_t)a * n + b];
        e += -cab * disp * 0.5;
        dcn += -dc6[(size_t)a * n + b] * disp;
        for (int k = 0; k < 3; ++k) g[k] += -cab * ddisp * rij[k];
    }
    e_atom[a] = e;
    dEdcn[a] += dcn;
    for (int k = 0; k < 3; ++k) grad[3 * a + k] += g[k];
}

// Warp-cooperative form of d_d4_2body for the plain engine (one warp per atom).
__device__ inline void d_d4_2body_warp(DevMol m, const double* __restrict__ c6, const double* __restrict__ dc6,
                                       double* __restrict__ e_atom, double* __restrict__ dEdcn,
                                       double* __restrict__ grad, int a, int lane) {
    const int n = m.nat;
    double e = 0.0, dcn = 0.0, g[3] = {0, 0, 0};
    for (int b = lane; b < n; b += 32) {
        if (b == a) continue;
        const double rij[3] = {m.xyz[3 * a] - m.xyz[3 * b], m.xyz[3 * a + 1] - m.xyz[3 * b + 1],
                               m.xyz[3 * a + 2] - m.xyz[3 * b + 2]};
        const double r2 = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
        if (r2 > 3600.0 || r2 < 1e-10) continue;
        const double r4r2 = 3.0 * m.r4r2[a] * m.r4r2[b];
        const double r0 = 0.52 * sqrt(r4r2) + 5.0;
        const double t6 = 1.0 / (r2 * r2 * r2 + powi<6>(r0));
        const double t8 = 1.0 / (r2 * r2 * r2 * r2 + powi<8>(r0));
        const double d6 = -6.0 * r2 * r2 * t6 * t6;
        const double d8 = -8.0 * r2 * r2 * r2 * t8 * t8;
        const double disp = 1.0 * t6 + 2.7 * r4r2 * t8;
        const double ddisp = 1.0 * d6 + 2.7 * r4r2 * d8;
        const double cab = c6[(size_t)a * n + b];
        e += -cab * disp * 0.5;
        dcn += -dc6[(size_t)a * n + b] * disp;
        for (int k = 0; k < 3; ++k) g[k] += -cab * ddisp * rij[k];
    }
    e = warp_sum(e);
    dcn = warp_sum(dcn);
    for (int k = 0; k < 3; ++k) g[k] = warp_sum(g[k]);
    if (lane == 0) {
        e_atom[a] = e;
        dEdcn[a] += dcn;
        for (int k = 0; k < 3; ++k) grad[3 * a + k] += g[k];
    }
}

// Broyden vector [qsh; per atom (dipm 3, qp 6)] (gfn2broyden_*, src/aespot.F90:1360-1425)
__device__ inline void d_broyden_pack(DevMol m, const double* __restrict__ qsh, const double* __restrict__ dipm,
                               const double* __restrict__ qp, double* __restrict__ v, int t) {
    if (t < m.nsh) v[t] = qsh[t];
    if (t < m.nat) {
        double* o = v + m.nsh + 9 * t;
        for (int k = 0; k < 3; ++k) o[k] = dipm[3 * t + k];
        for (int k = 0; k < 6; ++k) o[3 + k] = qp[6 * t + k];
    }
}

__device__ inline void d_broyden_unpack(DevMol m, const double* __restrict__ v, double* __restrict__ qsh,
                                 double* __restrict__ dipm, double* __restrict__ qp, double* __restrict__ q, int t) {
    if (t < m.nsh) qsh[t] = v[t];
    if (t < m.nat) {
        const double* o = v + m.nsh + 9 * t;
        for (int k = 0; k < 3; ++k) dipm[3 * t + k] = o[k];
        for (int k = 0; k < 6; ++k) qp[6 * t + k] = o[3 + k];
        double s = 0.0;
        for (int sh = m.at_sh0[t]; sh < m.at_sh0[t] + m.at_nsh[t]; ++sh) s += v[sh];
        q[t] = s;
    }
}

// three-body (ATM) dispersion, atm_gradient_latp / deriv_atm_triple (src/disp/dftd4.F90:2023-2177, 2354-2433)
// The derivative polynomial of the ATM angular factor for the pair whose squared distance is x
// (y, z: the other two): x^3 + x^2 (y + z) + x (3 y^2 + 2 y z + 3 z^2) - 5 (y - z)^2 (y + z), with
// u = y + z, v = y - z and 3 y^2 + 2 y z + 3 z^2 = 2 u^2 + v^2 (ten FP64 operations).
__device__ __forceinline__ double atm_dpoly(double x, double y, double z) {
    const double u = y + z, v = y - z, v2 = v * v;
    const double w = fma(2.0 * u, u, v2);
    return fma(x, fma(x, x + u, w), -5.0 * u * v2);
}

__device__ inline void d_d4_atm(DevMol m, const double* __restrict__ c6, const double* __restrict__ dc6, long npair,
                         double* __restrict__ e_pair, double* __restrict__ dEdcn, double* __restrict__ grad, long t) {
    int ia, ja;
    tri_pair(t, ia, ja);
    if (ja >= ia) { e_pair[t] = 0.0; return; }
    const int n = m.nat;
    const double cut2 = 1600.0;
    const double rij[3] = {m.xyz[3 * ja] - m.xyz[3 * ia], m.xyz[3 * ja + 1] - m.xyz[3 * ia + 1],
                           m.xyz[3 * ja + 2] - m.xyz[3 * ia + 2]};
    const double r2ij = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
    double esum = 0.0;
    if (r2ij <= cut2) {
        double gi[3] = {0, 0, 0}, gj[3] = {0, 0, 0}, dci = 0.0, dcj = 0.0;
        const double c6ij = c6[(size_t)ja * n + ia];
        const double cij = 0.52 * sqrt(3.0 * m.r4r2[ia] * m.r4r2[ja]) + 5.0;
        for (int ka = 0; ka < ja; ++ka) {
            const double rik[3] = {m.xyz[3 * ka] - m.xyz[3 * ia], m.xyz[3 * ka + 1] - m.xyz[3 * ia + 1],
                                   m.xyz[3 * ka + 2] - m.xyz[3 * ia + 2]};
            const double r2ik = rik[0] * rik[0] + rik[1] * rik[1] + rik[2] * rik[2];
            if (r2ik > cut2) continue;
            const double rjk[3] = {m.xyz[3 * ka] - m.xyz[3 * ja], m.xyz[3 * ka + 1] - m.xyz[3 * ja + 1],
                                   m.xyz[3 * ka + 2] - m.xyz[3 * ja + 2]};
            const double r2jk = rjk[0] * rjk[0] + rjk[1] * rjk[1] + rjk[2] * rjk[2];
            if (r2jk > cut2) continue;
            const double c6ik = c6[(size_t)ka * n + ia], c6jk = c6[(size_t)ka * n + ja];
            const double cik = 0.52 * sqrt(3.0 * m.r4r2[ia] * m.r4r2[ka]) + 5.0;
            const double cjk = 0.52 * sqrt(3.0 * m.r4r2[ja] * m.r4r2[ka]) + 5.0;
            const double c9 = -sqrt(c6ij * c6ik * c6jk);
            const double ccc1 = cij * cjk * cik;
            const double rrr2 = r2ij * r2jk * r2ik;
            const double rrr1 = sqrt(rrr2);
            const double rrr3 = rrr1 * rrr2;
            const double ang_fact = 0.375 / (rrr2 * rrr3);
            const double ang = ang_fact * (r2ij + r2jk - r2ik) * (r2ij - r2jk + r2ik) * (-r2ij + r2jk + r2ik) + 1.0 / rrr3;
            // (C_ijk / R_ijk)^(16/3) = x^5 cbrt(x): one cube root instead of a general power
            const double xr = ccc1 / rrr1, xr2 = xr * xr;
            const double cralp = xr2 * xr2 * xr * cbrt(xr);
            const double fdmp = 1.0 / (1.0 + 6.0 * cralp);
            const double dfdmp = -(2.0 * 16.0 * cralp) * fdmp * fdmp;
            const double dE = -fdmp * ang * c9;
            const double dang1 = -ang_fact * atm_dpoly(r2ij, r2jk, r2ik);
            const double dGr1 = (-dang1 * c9 * fdmp + dfdmp * c9 * ang) / r2ij;
            const double dang2 = -ang_fact * atm_dpoly(r2ik, r2jk, r2ij);
            const double dGr2 = (-dang2 * c9 * fdmp + dfdmp * c9 * ang) / r2ik;
            const double dang3 = -ang_fact * atm_dpoly(r2jk, r2ik, r2ij);
            const double dGr3 = (-dang3 * c9 * fdmp + dfdmp * c9 * ang) / r2jk;
            const double s9 = 5.0;
            esum += dE * s9;
            for (int x = 0; x < 3; ++x) {
                gi[x] += s9 * (-dGr1 * rij[x] - dGr2 * rik[x]);
                gj[x] += s9 * (dGr1 * rij[x] - dGr3 * rjk[x]);
                atomicAdd(&grad[3 * ka + x], s9 * (dGr2 * rik[x] + dGr3 * rjk[x]));
            }
            const double dc9i = 0.5 * c9 * (dc6[(size_t)ia * n + ja] / c6ij + dc6[(size_t)ia * n + ka] / c6ik);
            const double dc9j = 0.5 * c9 * (dc6[(size_t)ja * n + ia] / c6ij + dc6[(size_t)ja * n + ka] / c6jk);
            const double dc9k = 0.5 * c9 * (dc6[(size_t)ka * n + ia] / c6ik + dc6[(size_t)ka * n + ja] / c6jk);
            dci += s9 * (-ang * fdmp * dc9i);
            dcj += s9 * (-ang * fdmp * dc9j);
            atomicAdd(&dEdcn[ka], s9 * (-ang * fdmp * dc9k));
        }
        for (int x = 0; x < 3; ++x) {
            atomicAdd(&grad[3 * ia + x], gi[x]);
            atomicAdd(&grad[3 * ja + x], gj[x]);
        }
        atomicAdd(&dEdcn[ia], dci);
        atomicAdd(&dEdcn[ja], dcj);
    }
    e_pair[t] = esum;
}

}  // namespace xg
