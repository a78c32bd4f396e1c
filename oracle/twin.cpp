// GFN2-xTB single point: C++/OpenMP + LAPACK restatement of the CPU oracle (test and
// baseline infrastructure only; never linked into the engine).
//
// It restates oracle/gfn2.py and oracle/integrals.py equation by equation (the same
// screening rules, the same LAPACK sequence dpotrf once, then dsygst + dsyevd + dtrsm per SCC
// iteration, src/mctc/lapack/eigensolve.F90:218-246) with the O(N^2) and O(N^3) loops in
// OpenMP, so the reference's CPU algorithm can be timed on every molecule of a workload,
// including those of a few thousand orbitals.  Per-function sources in the reference are
// cited at each function.  The LAPACK/BLAS routines come in as function pointers (the
// Fortran-ABI entry points SciPy exports), so this file links against no BLAS itself.
//
// Layout: every n x n matrix is one contiguous array; LAPACK sees it column-major.  S, H, P,
// W and the moment matrices are symmetric, so the row-major and column-major views agree;
// the eigenvector matrix C holds orbital j in C[j*nao .. j*nao+nao).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include <omp.h>

namespace {

constexpr double PI = 3.1415926535897932384626433832795029;
constexpr double AUTOEV = 27.21138505;
constexpr double EVTOAU = 1.0 / AUTOEV;
constexpr double KB = 3.166808578545117e-06;
constexpr double AES_SHIFT = 1.2, AES_EXP = 4.0, AES_RMAX = 5.0, AES_DMP3 = 3.0, AES_DMP5 = 4.0;
constexpr double D4_S6 = 1.0, D4_S8 = 2.7, D4_S10 = 0.0, D4_A1 = 0.52, D4_A2 = 5.0, D4_S9 = 5.0, D4_ALP = 16.0;
constexpr double D4_GA = 3.0, D4_GC = 2.0, D4_WF = 6.0;
constexpr double REP_KEXP = 1.5, REP_KEXP_LIGHT = 1.0, REP_REXP = 1.0;
constexpr double MAX_R2 = 2000.0;
constexpr int MAXREF = 7;

using dpotrf_t = void (*)(char*, int*, double*, int*, int*);
using dsygst_t = void (*)(int*, char*, int*, double*, int*, double*, int*, int*);
using dsyevd_t = void (*)(char*, char*, int*, double*, int*, double*, double*, int*, int*, int*, int*);
using dsysv_t = void (*)(char*, int*, int*, double*, int*, int*, double*, int*, double*, int*, int*);
using dtrsm_t = void (*)(char*, char*, char*, char*, int*, int*, double*, double*, int*, double*, int*);
using dgemm_t = void (*)(char*, char*, int*, int*, int*, double*, double*, int*, double*, int*, double*, double*,
                         int*);

}  // namespace

extern "C" {

// LAPACK / BLAS entry points (Fortran calling convention, 32-bit integers).
struct TwinLapack {
    void* dpotrf;
    void* dsygst;
    void* dsyevd;
    void* dsysv;
    void* dtrsm;
    void* dgemm;
};

// One molecule with its parameters gathered per atom and per shell by the caller.
struct TwinInput {
    int nat, nsh, nao, maxprim, nelem, maxiter, ihomoa, ihomob;
    double charge, etemp, accuracy;
    const double* xyz;       // [nat][3] Bohr
    const int* Z;            // [nat]
    // per atom
    const double *zval, *en, *covd3, *rcovd4, *end4, *eeq_en, *eeq_gam, *eeq_kappa, *eeq_alpha;
    const double *multirad, *valcn, *dipk, *quadk, *sqrtzr4r2, *atomicrad, *rep_alpha, *rep_zeff;
    const int *d4_nref, *d4_off, *eidx;  // refs of atom i at d4_off[i] .. d4_off[i] + d4_nref[i]
    const double *d4_zeff, *d4_gam;
    const double *d4_refcn, *d4_refq;    // [ndim]
    const int* d4_ncount;                // [ndim]
    const double* c6ref;                 // [nelem][nelem][7][7]
    // per shell
    const int *sh_atom, *sh_l, *sh_nprim, *sh_ao;
    const double *alpha, *coef;          // [nsh][maxprim]
    const double *zeta, *se0, *kcn, *shpoly, *gam3, *eta, *zsh;
    const double* kscale;                // [4][4], [lj][li]
    const double* enscale;               // [4][4]
    int guess_eeq;                       // 1: EEQ start charges; 0: q = charge / nat
};

struct TwinOutput {
    double energy, e_elec, e_rep, e_es, e_aes, e_axc, e_disp;
    int iterations, converged;
    double* q;          // [nat]
    double* qsh;        // [nsh]
    double* gradient;   // [nat][3]
    double* dipole;     // [3]
    double* wbo;        // [nat][nat] or null
    double* emo;        // [nao] eV
    double* focc;       // [nao]
    double seconds[4];  // set-up, SCC, gradient, properties
};

}  // extern "C"

namespace {

struct Ctx {
    const TwinInput& in;
    int nat, nsh, nao;
    dpotrf_t dpotrf;
    dsygst_t dsygst;
    dsyevd_t dsyevd;
    dsysv_t dsysv;
    dtrsm_t dtrsm;
    dgemm_t dgemm;
    explicit Ctx(const TwinInput& i) : in(i), nat(i.nat), nsh(i.nsh), nao(i.nao) {}
    const double* R(int a) const { return in.xyz + 3 * a; }
};

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// per-thread accumulation of [nat][3] (and [nat]) arrays, summed in thread order
struct ThreadAcc {
    int width;
    std::vector<double> buf;
    ThreadAcc(int nthreads, int w) : width(w), buf((size_t)nthreads * w, 0.0) {}
    double* mine() { return buf.data() + (size_t)omp_get_thread_num() * width; }
    void reduce_into(double* out, double sign = 1.0) const {
        int nt = (int)(buf.size() / width);
        for (int t = 0; t < nt; ++t)
            for (int k = 0; k < width; ++k) out[k] += sign * buf[(size_t)t * width + k];
    }
};

// ------------------------------------------------------------------ coordination numbers
// getCoordinationNumberLP, src/disp/coordinationnumber.F90:304-479 ('gfn': gfnCount with D3
// covalent radii; 'cov': erfCount with the EN covalency factor).  Pair term and its radial
// derivative factor (dCN/dr / r).
inline void cn_pair(const Ctx& c, bool cov, int i, int j, double r2, double& cf, double& dfr) {
    const TwinInput& in = c.in;
    double r = std::sqrt(r2);
    double rc = in.covd3[i] + in.covd3[j];
    if (!cov) {
        auto ec = [](double kk, double rr, double r0) { return 1.0 / (1.0 + std::exp(-kk * (r0 / rr - 1.0))); };
        auto dec = [](double kk, double rr, double r0) {
            double e = std::exp(-kk * (r0 / rr - 1.0));
            return (-kk * r0 * e) / (rr * rr * ((e + 1.0) * (e + 1.0)));
        };
        const double k = 10.0;
        cf = ec(k, r, rc) * ec(2 * k, r, rc + 2);
        double df = dec(k, r, rc) * ec(2 * k, r, rc + 2) + ec(k, r, rc) * dec(2 * k, r, rc + 2);
        dfr = df / r;
    } else {
        const double k = 7.5, k4 = 4.10451, k5 = 19.08857, k6 = 2 * 11.28174 * 11.28174;
        double cfe = 0.5 * (1.0 + std::erf(-k * (r - rc) / rc));
        double df = -k / std::sqrt(PI) / rc * std::exp(-k * k * (r - rc) * (r - rc) / (rc * rc));
        double t = std::fabs(in.en[i] - in.en[j]) + k5;
        double den = k4 * std::exp(-t * t / k6);
        cf = den * cfe;
        dfr = den * df / r;
    }
}

std::vector<double> cn_lp(const Ctx& c, bool cov) {
    int n = c.nat;
    std::vector<double> cn(n, 0.0);
    int nt = omp_get_max_threads();
    ThreadAcc acc(nt, n);
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; ++i) {
        double* a = acc.mine();
        for (int j = 0; j < i; ++j) {
            double d[3] = {c.R(i)[0] - c.R(j)[0], c.R(i)[1] - c.R(j)[1], c.R(i)[2] - c.R(j)[2]};
            double r2 = dot3(d, d);
            if (r2 > 1600.0 || r2 < 1e-12) continue;
            double cf, dfr;
            cn_pair(c, cov, i, j, r2, cf, dfr);
            a[i] += cf;
            a[j] += cf;
        }
    }
    acc.reduce_into(cn.data());
    return cn;
}

// g[a] += sign * sum_b dCN_b/dR_a x[b]; with countd = dfr * (R_i - R_j) per pair i > j:
// g_i += countd (x_i + x_j), g_j -= countd (x_i + x_j).
void cn_chain(const Ctx& c, bool cov, const std::vector<double>& x, double* g, double sign) {
    int n = c.nat;
    ThreadAcc acc(omp_get_max_threads(), 3 * n);
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; ++i) {
        double* a = acc.mine();
        for (int j = 0; j < i; ++j) {
            double d[3] = {c.R(i)[0] - c.R(j)[0], c.R(i)[1] - c.R(j)[1], c.R(i)[2] - c.R(j)[2]};
            double r2 = dot3(d, d);
            if (r2 > 1600.0 || r2 < 1e-12) continue;
            double cf, dfr;
            cn_pair(c, cov, i, j, r2, cf, dfr);
            double s = dfr * (x[i] + x[j]);
            for (int k = 0; k < 3; ++k) {
                a[3 * i + k] += s * d[k];
                a[3 * j + k] -= s * d[k];
            }
        }
    }
    acc.reduce_into(g, sign);
}

// ncoord_erf (src/disp/ncoord.f90:469-506) and ncoord_d4 (:575-615)
std::vector<double> cn_erf(const Ctx& c, bool d4) {
    const TwinInput& in = c.in;
    int n = c.nat;
    std::vector<double> cn(n, 0.0);
    ThreadAcc acc(omp_get_max_threads(), n);
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; ++i) {
        double* a = acc.mine();
        for (int j = 0; j < i; ++j) {
            double d[3] = {c.R(j)[0] - c.R(i)[0], c.R(j)[1] - c.R(i)[1], c.R(j)[2] - c.R(i)[2]};
            double r2 = dot3(d, d);
            if (r2 > 1600.0) continue;
            double r = std::sqrt(r2);
            double rco = in.rcovd4[j] + in.rcovd4[i];
            double tmp = 0.5 * (1.0 + std::erf(-7.5 * (r - rco) / rco));
            if (d4) {
                double t = std::fabs(in.end4[i] - in.end4[j]) + 19.08857;
                tmp *= 4.10451 * std::exp(-t * t / (2 * 11.28174 * 11.28174));
            }
            a[i] += tmp;
            a[j] += tmp;
        }
    }
    acc.reduce_into(cn.data());
    return cn;
}

// ------------------------------------------------------------------ EEQ guess
// eeq_chrgeq_core (0D) with the 2019 model, src/eeq_model.f90:678-880 (dsysv :857-862)
bool eeq_guess(const Ctx& c, std::vector<double>& q) {
    const TwinInput& in = c.in;
    int n = c.nat, m = n + 1;
    std::vector<double> cn = cn_erf(c, false);
    std::vector<double> A((size_t)m * m, 0.0), X(m, 0.0);
    for (int i = 0; i < n; ++i) {
        double tmp = in.eeq_kappa[i] / (std::sqrt(cn[i]) + 1e-14);
        X[i] = -in.eeq_en[i] + tmp * cn[i];
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            if (i == j) {
                A[(size_t)i * m + i] = in.eeq_gam[i] + std::sqrt(2.0 / PI) / in.eeq_alpha[i];
                continue;
            }
            double d[3] = {c.R(i)[0] - c.R(j)[0], c.R(i)[1] - c.R(j)[1], c.R(i)[2] - c.R(j)[2]};
            double r = std::sqrt(dot3(d, d));
            double g = 1.0 / std::sqrt(in.eeq_alpha[i] * in.eeq_alpha[i] + in.eeq_alpha[j] * in.eeq_alpha[j]);
            A[(size_t)i * m + j] = std::erf(g * r) / r;
        }
        A[(size_t)i * m + n] = 1.0;
        A[(size_t)n * m + i] = 1.0;
    }
    A[(size_t)n * m + n] = 0.0;
    X[n] = in.charge;
    char uplo = 'U';
    int nrhs = 1, info = 0, lwork = -1;
    std::vector<int> ipiv(m);
    double wq = 0;
    c.dsysv(&uplo, &m, &nrhs, A.data(), &m, ipiv.data(), X.data(), &m, &wq, &lwork, &info);
    lwork = std::max(1, (int)wq);
    std::vector<double> work(lwork);
    c.dsysv(&uplo, &m, &nrhs, A.data(), &m, ipiv.data(), X.data(), &m, work.data(), &lwork, &info);
    if (info != 0) return false;
    q.assign(X.begin(), X.begin() + n);
    return true;
}

// ------------------------------------------------------------------ multipole integrals
// get_multiints / multipole_3d / olapp, src/intgrad.f90:95-111,509-555,879-955; the gradient
// get_grad_multiint / multipole_grad_3d / shiftintg :607-728,958-1035; dtrf2 :144-231.
// Each Cartesian factor is expanded about the Gaussian-product centre P.
const int CART[3][6][3] = {{{0, 0, 0}},
                           {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
                           {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}}};
const int NCART[3] = {1, 3, 6};
const int NSPH[3] = {1, 3, 5};
const int MOM[10][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 0},
                        {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}};
const double DFACT[8] = {1.0, 1.0, 3.0, 15.0, 105.0, 945.0, 10395.0, 135135.0};
const double BINOM[4][4] = {{1, 0, 0, 0}, {1, 1, 0, 0}, {1, 2, 1, 0}, {1, 3, 3, 1}};

// 1D moments I[i][j][e] = int (x-A)^i (x-B)^j (x-C)^e exp(-gam (x-P)^2) dx / sqrt(pi/gam),
// i <= imax (<= 3), j <= jmax (<= 2), e <= 2.
inline void mom1d(int imax, int jmax, double PA, double PB, double PC, double gam, double I[4][3][3]) {
    double t[8];
    double h = 0.5 / gam, hp = 1.0;
    for (int m = 0; m < 8; ++m) {
        if (m & 1) {
            t[m] = 0.0;
        } else {
            t[m] = hp * DFACT[m / 2];
            hp *= h;
        }
    }
    double pa[4] = {1.0, PA, PA * PA, PA * PA * PA};
    double pb[3] = {1.0, PB, PB * PB};
    for (int i = 0; i <= imax; ++i)
        for (int j = 0; j <= jmax; ++j) {
            double v0 = 0, v1 = 0, v2 = 0;
            for (int a = 0; a <= i; ++a) {
                double ca = BINOM[i][a] * pa[i - a];
                for (int b = 0; b <= j; ++b) {
                    double cab = ca * BINOM[j][b] * pb[j - b];
                    int m = a + b;
                    v0 += cab * t[m];
                    v1 += cab * (t[m + 1] + PC * t[m]);
                    v2 += cab * (t[m + 2] + 2 * PC * t[m + 1] + PC * PC * t[m]);
                }
            }
            I[i][j][0] = v0;
            I[i][j][1] = v1;
            I[i][j][2] = v2;
        }
}

struct ShellRef {
    int l, nprim;
    const double *alpha, *coef;
};

// Moment integrals of one shell pair about origin C, spherical on output:
// ints[k][a][b] (k = 0..9, a < nsph_i, b < nsph_j, stride 5x5); with grad also the
// derivative with respect to centre A, dints[c][k][a][b]; with shift the moment origin
// moves with A (C must equal A).
void pair_moments(const ShellRef& si, const ShellRef& sj, const double* A, const double* B, const double* C,
                  double intcut, bool grad, bool shift, double ints[10][6][6], double dints[3][10][6][6]) {
    int li = si.l, lj = sj.l, nci = NCART[li], ncj = NCART[lj];
    double ic[10][6][6];
    double dc[3][10][6][6];
    std::memset(ic, 0, sizeof(ic));
    if (grad) std::memset(dc, 0, sizeof(dc));
    double rab[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
    double r2 = dot3(rab, rab);
    if (r2 <= MAX_R2) {
        for (int p = 0; p < si.nprim; ++p) {
            double ai = si.alpha[p], ci = si.coef[p];
            if (ci == 0.0) continue;
            for (int qq = 0; qq < sj.nprim; ++qq) {
                double aj = sj.alpha[qq], cj = sj.coef[qq];
                if (cj == 0.0) continue;
                double gam = ai + aj;
                double est = r2 * ai * aj;
                if (!(est <= intcut * gam)) continue;
                double ab = 1.0 / gam;
                double s = std::sqrt(PI) * std::sqrt(ab);
                double cc = std::exp(-est * ab) * s * s * s * ci * cj;
                double I[3][4][3][3];
                for (int x = 0; x < 3; ++x) {
                    double P = (ai * A[x] + aj * B[x]) * ab;
                    mom1d(li + (grad ? 1 : 0), lj, P - A[x], P - B[x], P - C[x], gam, I[x]);
                }
                for (int a = 0; a < nci; ++a) {
                    const int* pi = CART[li][a];
                    for (int b = 0; b < ncj; ++b) {
                        const int* pj = CART[lj][b];
                        for (int k = 0; k < 10; ++k) {
                            const int* e = MOM[k];
                            double v0 = I[0][pi[0]][pj[0]][e[0]], v1 = I[1][pi[1]][pj[1]][e[1]],
                                   v2 = I[2][pi[2]][pj[2]][e[2]];
                            ic[k][a][b] += cc * v0 * v1 * v2;
                            if (grad) {
                                double v[3] = {v0, v1, v2};
                                for (int cx = 0; cx < 3; ++cx) {
                                    double g = 2 * ai * I[cx][pi[cx] + 1][pj[cx]][e[cx]];
                                    if (pi[cx] > 0) g -= pi[cx] * I[cx][pi[cx] - 1][pj[cx]][e[cx]];
                                    double f = cc * g;
                                    for (int y = 0; y < 3; ++y)
                                        if (y != cx) f *= v[y];
                                    dc[cx][k][a][b] += f;
                                }
                            }
                        }
                    }
                }
            }
        }
    }
    // contraction coefficients of the d Cartesian components (set_d_function trafo(5:10))
    const double s3 = std::sqrt(3.0);
    if (li == 2)
        for (int a = 3; a < 6; ++a)
            for (int k = 0; k < 10; ++k)
                for (int b = 0; b < ncj; ++b) {
                    ic[k][a][b] *= s3;
                    if (grad)
                        for (int cx = 0; cx < 3; ++cx) dc[cx][k][a][b] *= s3;
                }
    if (lj == 2)
        for (int b = 3; b < 6; ++b)
            for (int k = 0; k < 10; ++k)
                for (int a = 0; a < nci; ++a) {
                    ic[k][a][b] *= s3;
                    if (grad)
                        for (int cx = 0; cx < 3; ++cx) dc[cx][k][a][b] *= s3;
                }
    if (grad && shift) {
        // d/dA_c M_e gains -e_c M_{e - 1_c}
        for (int k = 0; k < 10; ++k)
            for (int cx = 0; cx < 3; ++cx) {
                int ec = MOM[k][cx];
                if (!ec) continue;
                int low[3] = {MOM[k][0], MOM[k][1], MOM[k][2]};
                low[cx] -= 1;
                int kl = 0;
                for (int kk = 0; kk < 10; ++kk)
                    if (MOM[kk][0] == low[0] && MOM[kk][1] == low[1] && MOM[kk][2] == low[2]) kl = kk;
                for (int a = 0; a < nci; ++a)
                    for (int b = 0; b < ncj; ++b) dc[cx][k][a][b] -= ec * ic[kl][a][b];
            }
    }
    // Cartesian -> spherical d (dx2-y2, dz2, dxy, dxz, dyz), src/intgrad.f90:150-164
    const double T[5][6] = {{0.5 * s3, -0.5 * s3, 0, 0, 0, 0},
                            {0.5, 0.5, -1.0, 0, 0, 0},
                            {0, 0, 0, 1, 0, 0},
                            {0, 0, 0, 0, 1, 0},
                            {0, 0, 0, 0, 0, 1}};
    auto sph = [&](double (*m)[6][6], int nk, double (*o)[6][6]) {
        for (int k = 0; k < nk; ++k) {
            double t1[6][6];
            int ni = NSPH[li], nj = NSPH[lj];
            for (int a = 0; a < ni; ++a)
                for (int b = 0; b < ncj; ++b) {
                    if (li == 2) {
                        double v = 0;
                        for (int x = 0; x < 6; ++x) v += T[a][x] * m[k][x][b];
                        t1[a][b] = v;
                    } else {
                        t1[a][b] = m[k][a][b];
                    }
                }
            for (int a = 0; a < ni; ++a)
                for (int b = 0; b < nj; ++b) {
                    if (lj == 2) {
                        double v = 0;
                        for (int x = 0; x < 6; ++x) v += T[b][x] * t1[a][x];
                        o[k][a][b] = v;
                    } else {
                        o[k][a][b] = t1[a][b];
                    }
                }
        }
    };
    sph(ic, 10, ints);
    if (grad)
        for (int cx = 0; cx < 3; ++cx) sph(dc[cx], 10, dints[cx]);
}

ShellRef shell_ref(const Ctx& c, int s) {
    return {c.in.sh_l[s], c.in.sh_nprim[s], c.in.alpha + (size_t)s * c.in.maxprim,
            c.in.coef + (size_t)s * c.in.maxprim};
}

// build_SDQH0, src/xtb/hamiltonian.F90:146-371 (h0scal/shellPoly src/scc_core.f90:644-680,728-754).
// S, D[3], Q[6] (origin 0), H0 and H0 without overlap (eV), full square matrices.
void build_sdqh0(const Ctx& c, const std::vector<double>& se, double intcut, std::vector<double>& S,
                 std::vector<double>& D, std::vector<double>& Q, std::vector<double>& H0,
                 std::vector<double>& H0n) {
    const TwinInput& in = c.in;
    size_t nn = (size_t)c.nao * c.nao;
    int n = c.nao;
    S.assign(nn, 0.0);
    D.assign(3 * nn, 0.0);
    Q.assign(6 * nn, 0.0);
    H0.assign(nn, 0.0);
    H0n.assign(nn, 0.0);
    const double origin[3] = {0, 0, 0};
#pragma omp parallel for schedule(dynamic, 8)
    for (int ish = 0; ish < c.nsh; ++ish) {
        int iat = in.sh_atom[ish];
        ShellRef si = shell_ref(c, ish);
        double ints[10][6][6];
        for (int jsh = 0; jsh <= ish; ++jsh) {
            int jat = in.sh_atom[jsh];
            if (jat > iat) continue;
            ShellRef sj = shell_ref(c, jsh);
            pair_moments(si, sj, c.R(iat), c.R(jat), origin, intcut, false, false, ints, nullptr);
            int ni = NSPH[si.l], nj = NSPH[sj.l];
            double fac = 0.0;
            if (jat != iat) {
                int li = si.l, lj = sj.l;
                double zi = in.zeta[ish], zj = in.zeta[jsh];
                double zetaij = std::sqrt(2 * std::sqrt(zi * zj) / (zi + zj));
                double den = (in.en[iat] - in.en[jat]) * (in.en[iat] - in.en[jat]);
                double enpoly = 1.0 + in.enscale[lj * 4 + li] * den;
                double km = in.kscale[lj * 4 + li] * enpoly;
                double hav = 0.5 * km * (se[ish] + se[jsh]) * zetaij;
                double d[3] = {c.R(iat)[0] - c.R(jat)[0], c.R(iat)[1] - c.R(jat)[1], c.R(iat)[2] - c.R(jat)[2]};
                double r = std::sqrt(dot3(d, d)) / (in.atomicrad[jat] + in.atomicrad[iat]);
                double rf1 = 1.0 + 0.01 * in.shpoly[ish] * std::sqrt(r);
                double rf2 = 1.0 + 0.01 * in.shpoly[jsh] * std::sqrt(r);
                fac = hav * rf1 * rf2;
            }
            for (int a = 0; a < ni; ++a)
                for (int b = 0; b < nj; ++b) {
                    size_t ia = in.sh_ao[ish] + a, jb = in.sh_ao[jsh] + b;
                    size_t u = ia * n + jb, l = jb * n + ia;
                    for (int k = 0; k < 3; ++k) D[k * nn + u] = D[k * nn + l] = ints[1 + k][a][b];
                    for (int k = 0; k < 6; ++k) Q[k * nn + u] = Q[k * nn + l] = ints[4 + k][a][b];
                    if (jat != iat) {
                        double s = ints[0][a][b];
                        S[u] = S[l] = s;
                        H0[u] = H0[l] = fac * s;
                        H0n[u] = H0n[l] = fac;
                    }
                }
        }
    }
    for (int k = 0; k < c.nsh; ++k)
        for (int a = 0; a < NSPH[in.sh_l[k]]; ++a) {
            size_t i = in.sh_ao[k] + a;
            S[i * n + i] = 1.0;
            H0[i * n + i] = se[k];
            H0n[i * n + i] = se[k];
        }
}

// ------------------------------------------------------------------ anisotropic electrostatics
// get_radcn src/aespot.F90:1267-1281, dradcn :1292-1307, mmomgabzero :1219-1255
void aes_setup(const Ctx& c, const std::vector<double>& cn, std::vector<double>& rad, std::vector<double>& dr,
               std::vector<double>& gab3, std::vector<double>& gab5) {
    const TwinInput& in = c.in;
    int n = c.nat;
    rad.resize(n);
    dr.resize(n);
    for (int i = 0; i < n; ++i) {
        double rco = in.multirad[i];
        double t1 = cn[i] - in.valcn[i] - AES_SHIFT;
        rad[i] = rco + (AES_RMAX - rco) / (1.0 + std::exp(-AES_EXP * t1));
        double e = std::exp(-AES_EXP * t1);
        dr[i] = (AES_RMAX - rco) / (1.0 + 2.0 * e + e * e) * AES_EXP * e;
    }
    gab3.assign((size_t)n * n, 0.0);
    gab5.assign((size_t)n * n, 0.0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            if (i == j) continue;
            double d[3] = {c.R(j)[0] - c.R(i)[0], c.R(j)[1] - c.R(i)[1], c.R(j)[2] - c.R(i)[2]};
            double rinv = 1.0 / std::sqrt(dot3(d, d));
            double rco = 0.5 * (rad[i] + rad[j]);
            double x = rco * rinv;
            double damp3 = 1.0 / (1.0 + 6.0 * x * x * x);
            double damp5 = 1.0 / (1.0 + 6.0 * x * x * x * x);
            double r3 = rinv * rinv * rinv;
            gab3[(size_t)i * n + j] = damp3 * r3;
            gab5[(size_t)i * n + j] = damp5 * r3 * rinv * rinv;
        }
}

const int QIDX[3][3] = {{0, 1, 3}, {1, 2, 4}, {3, 4, 5}};  // packed (xx, xy, yy, xz, yz, zz)

// mmompop, src/aespot.F90:288-428: cumulative atomic dipoles and traceless quadrupoles
void mmompop(const Ctx& c, const std::vector<double>& P, const std::vector<double>& S,
             const std::vector<double>& D, const std::vector<double>& Q, const std::vector<int>& ao_atom,
             std::vector<double>& dipm, std::vector<double>& qp) {
    int n = c.nao, N = c.nat;
    size_t nn = (size_t)n * n;
    std::vector<double> rs(n), rd(3 * n), rq(6 * n);
#pragma omp parallel for schedule(static)
    for (int mu = 0; mu < n; ++mu) {
        double s = 0, d[3] = {0, 0, 0}, q[6] = {0, 0, 0, 0, 0, 0};
        const double* p = P.data() + (size_t)mu * n;
        for (int nu = 0; nu < n; ++nu) {
            double pv = p[nu];
            size_t o = (size_t)mu * n + nu;
            s += pv * S[o];
            for (int k = 0; k < 3; ++k) d[k] += pv * D[k * nn + o];
            for (int k = 0; k < 6; ++k) q[k] += pv * Q[k * nn + o];
        }
        rs[mu] = s;
        for (int k = 0; k < 3; ++k) rd[3 * mu + k] = d[k];
        for (int k = 0; k < 6; ++k) rq[6 * mu + k] = q[k];
    }
    dipm.assign(3 * N, 0.0);
    qp.assign(6 * N, 0.0);
    // qpint order (xx, yy, zz, xy, xz, yz) of the moment arrays
    const int qi[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
    for (int mu = 0; mu < n; ++mu) {
        int a = ao_atom[mu];
        const double* R = c.R(a);
        for (int k = 0; k < 3; ++k) dipm[3 * a + k] += R[k] * rs[mu] - rd[3 * mu + k];
        for (int k = 0; k < 3; ++k)
            for (int l = 0; l <= k; ++l) {
                int kl = k * (k + 1) / 2 + l;
                double t;
                if (k == l)
                    t = 2.0 * rd[3 * mu + k] * R[k] - R[k] * R[k] * rs[mu] - rq[6 * mu + qi[k][k]];
                else
                    t = rd[3 * mu + k] * R[l] + rd[3 * mu + l] * R[k] - R[l] * R[k] * rs[mu] - rq[6 * mu + qi[k][l]];
                qp[6 * a + kl] += t;
            }
    }
    for (int a = 0; a < N; ++a) {
        double* p = qp.data() + 6 * a;
        double tr = 0.5 * (p[0] + p[2] + p[5]);
        for (int k = 0; k < 6; ++k) p[k] *= 1.5;
        p[0] -= tr;
        p[2] -= tr;
        p[5] -= tr;
    }
}

// aniso_electro_cpu, src/aespot.F90:566-664: (e_aes, e_axc)
void aniso_electro(const Ctx& c, const std::vector<double>& q, const std::vector<double>& dipm,
                   const std::vector<double>& qp, const std::vector<double>& gab3, const std::vector<double>& gab5,
                   double& eaes, double& epol) {
    const TwinInput& in = c.in;
    int n = c.nat;
    double ep = 0.0;
    for (int i = 0; i < n; ++i) {
        const double* d = dipm.data() + 3 * i;
        double tt3 = 0;
        for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l) tt3 += qp[6 * i + QIDX[k][l]] * qp[6 * i + QIDX[k][l]];
        ep += in.dipk[i] * dot3(d, d) + tt3 * in.quadk[i];
    }
    double e = 0.0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : e)
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) {
            double r[3] = {c.R(i)[0] - c.R(j)[0], c.R(i)[1] - c.R(j)[1], c.R(i)[2] - c.R(j)[2]};
            // the oracle's pair (i, j) with i > j and rij = R_j - R_i is (b, a) here
            int a = j, b = i;
            double rr[3] = {-r[0], -r[1], -r[2]};
            double r2 = dot3(rr, rr);
            const double *da = dipm.data() + 3 * a, *db = dipm.data() + 3 * b;
            const double *qa = qp.data() + 6 * a, *qb = qp.data() + 6 * b;
            double ed = q[a] * dot3(db, rr) - q[b] * dot3(da, rr);
            double qrb = 0, qra = 0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) {
                    qrb += qb[QIDX[k][l]] * rr[k] * rr[l];
                    qra += qa[QIDX[k][l]] * rr[k] * rr[l];
                }
            double eq = q[a] * qrb + q[b] * qra;
            double edd = -3.0 * dot3(da, rr) * dot3(db, rr) + dot3(da, db) * r2;
            size_t ab = (size_t)a * n + b;
            e += ed * gab3[ab] + eq * gab5[ab] + edd * gab5[ab];
        }
    eaes = e;
    epol = ep;
}

// setvsdq (shifted: origin-0 moments, src/aespot.F90:727-848) and setdvsdq (atom-centred,
// :861-952): vs[N], vd[N][3], vq[N][6] (qpint order xx, yy, zz, xy, xz, yz)
void setvsdq(const Ctx& c, const std::vector<double>& q, const std::vector<double>& dipm,
             const std::vector<double>& qp, const std::vector<double>& gab3, const std::vector<double>& gab5,
             bool shifted, std::vector<double>& vs, std::vector<double>& vd, std::vector<double>& vq) {
    const TwinInput& in = c.in;
    int n = c.nat;
    vs.assign(n, 0.0);
    vd.assign(3 * n, 0.0);
    vq.assign(6 * n, 0.0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const double* Ri = c.R(i);
        double r2a = dot3(Ri, Ri);
        double s = 0, d[3] = {0, 0, 0}, qv[6] = {0, 0, 0, 0, 0, 0};
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            double dra[3] = {Ri[0] - c.R(j)[0], Ri[1] - c.R(j)[1], Ri[2] - c.R(j)[2]};
            double g3 = gab3[(size_t)j * n + i], g5 = gab5[(size_t)j * n + i];
            double qj = q[j];
            const double* dj = dipm.data() + 3 * j;
            const double* Qj = qp.data() + 6 * j;
            double r2ab = dot3(dra, dra);
            double t2a = dot3(dj, dra);
            double qdd = 0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) qdd += Qj[QIDX[k][l]] * dra[k] * dra[l];
            double dum3a, dum5a, t1a = 0;
            if (shifted) {
                t1a = dot3(Ri, dra);
                double t3a = dot3(Ri, dj);
                dum5a = -qdd - 1.5 * qj * t1a * t1a;
                dum3a = -t1a * qj - t2a;
                dum5a = dum5a + t3a * r2ab - 3.0 * t1a * t2a + 0.5 * qj * r2a * r2ab;
            } else {
                dum3a = -t2a;
                dum5a = -qdd;
            }
            s += dum5a * g5 + dum3a * g3;
            for (int k = 0; k < 3; ++k) {
                double dd5 = 3.0 * dra[k] * t2a - r2ab * dj[k];
                if (shifted) dd5 = dd5 - qj * r2ab * Ri[k] + 3.0 * qj * t1a * dra[k];
                d[k] += dra[k] * qj * g3 + dd5 * g5;
            }
            double w = qj * g5;
            for (int l = 0; l < 3; ++l) qv[l] += -1.5 * w * dra[l] * dra[l] + 0.5 * r2ab * w;
            qv[3] += -3.0 * w * dra[0] * dra[1];
            qv[4] += -3.0 * w * dra[0] * dra[2];
            qv[5] += -3.0 * w * dra[1] * dra[2];
        }
        // on-site kernel terms
        const double* dm = dipm.data() + 3 * i;
        const double* qpi = qp.data() + 6 * i;
        double qs1 = in.dipk[i] * 2.0, qs2 = in.quadk[i] * 6.0;
        double t3 = 0;
        if (shifted) t3 = dot3(Ri, dm) * qs1;
        for (int k = 0; k < 3; ++k) d[k] -= qs1 * dm[k];
        for (int l1 = 0; l1 < 3; ++l1) {
            for (int l2 = 0; l2 < l1; ++l2) {
                int ll = l1 * (l1 + 1) / 2 + l2;
                int ki = l1 + l2 + 2;
                qv[ki] -= qpi[ll] * qs2;
                if (shifted) {
                    t3 -= Ri[l1] * Ri[l2] * qpi[ll] * qs2;
                    d[l1] += Ri[l2] * qpi[ll] * qs2;
                    d[l2] += Ri[l1] * qpi[ll] * qs2;
                }
            }
            int ll = l1 * (l1 + 1) / 2 + l1;
            qv[l1] -= qpi[ll] * qs2 * 0.5;
            if (shifted) {
                t3 -= Ri[l1] * Ri[l1] * qpi[ll] * qs2 * 0.5;
                d[l1] += Ri[l1] * qpi[ll] * qs2;
            }
        }
        double tr = (qpi[0] + qpi[2] + qpi[5]) * in.quadk[i];
        if (shifted) s += t3;
        for (int l1 = 0; l1 < 3; ++l1) {
            qv[l1] += tr;
            if (shifted) {
                d[l1] -= 2.0 * Ri[l1] * tr;
                s += tr * Ri[l1] * Ri[l1];
            }
        }
        vs[i] = s;
        for (int k = 0; k < 3; ++k) vd[3 * i + k] = d[k];
        for (int k = 0; k < 6; ++k) vq[6 * i + k] = qv[k];
    }
}

// aniso_grad, src/aespot.F90:1060-1165 (without the dR0/dR chain, which the caller adds)
void aniso_grad(const Ctx& c, const std::vector<double>& q, const std::vector<double>& dipm,
                const std::vector<double>& qp, const std::vector<double>& rad, const std::vector<double>& gab3,
                const std::vector<double>& gab5, double* g, std::vector<double>& tmp2) {
    int n = c.nat;
    tmp2.assign(n, 0.0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double gi[3] = {0, 0, 0}, t2 = 0;
        const double* di = dipm.data() + 3 * i;
        double Qi[3][3];
        for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l) Qi[k][l] = qp[6 * i + QIDX[k][l]];
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            double rij[3] = {c.R(j)[0] - c.R(i)[0], c.R(j)[1] - c.R(i)[1], c.R(j)[2] - c.R(i)[2]};
            double r2 = dot3(rij, rij);
            double rabi = 1.0 / std::sqrt(r2);
            double rco = 0.5 * (rad[i] + rad[j]);
            double x = rco * rabi;
            double damp1 = 1.0 / (1.0 + 6.0 * x * x * x);
            double dd1 = -AES_DMP3 * rabi * (damp1 * damp1 - damp1);
            double damp2 = 1.0 / (1.0 + 6.0 * x * x * x * x);
            double dd2 = -AES_DMP5 * rabi * (damp2 * damp2 - damp2);
            double r3 = rabi * rabi * rabi, r5 = r3 * rabi * rabi;
            double dgab3 = (-3.0 * rabi * r3) * damp1 + dd1 * r3;
            double dgab5 = (-5.0 * rabi * r5) * damp2 + dd2 * r5;
            double G3 = gab3[(size_t)j * n + i], G5 = gab5[(size_t)j * n + i];
            const double* dj = dipm.data() + 3 * j;
            double Qj[3][3];
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) Qj[k][l] = qp[6 * j + QIDX[k][l]];
            double qi = q[i], qj = q[j];
            double ed = qj * dot3(di, rij) - qi * dot3(dj, rij);
            double qri = 0, qrj = 0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) {
                    qri += Qi[k][l] * rij[k] * rij[l];
                    qrj += Qj[k][l] * rij[k] * rij[l];
                }
            double eq = qj * qri + qi * qrj;
            double edd = -3.0 * dot3(dj, rij) * dot3(di, rij) + dot3(dj, di) * r2;
            double ddm2 = dot3(dj, di), ddm3a = dot3(di, rij), ddm3b = dot3(dj, rij);
            for (int k = 0; k < 3; ++k) {
                double qqa = 0, qqb = 0;
                for (int l = 0; l < 3; ++l) {
                    qqa += rij[l] * Qj[l][k];
                    qqb += rij[l] * Qi[l][k];
                }
                double tt = qi * dj[k] - qj * di[k];
                double gk = G3 * tt - 2.0 * G5 * ddm2 * rij[k] + 3.0 * G5 * ddm3a * dj[k] + 3.0 * G5 * ddm3b * di[k] -
                            2.0 * G5 * qi * qqa - 2.0 * G5 * qj * qqb;
                double dxi = rij[k] * rabi;
                gk += -(ed * dgab3) * dxi - ((eq + edd) * dgab5) * dxi;
                gi[k] += gk;
            }
            double rab = rco;
            double y = rab * rabi;
            double tmp = ed * AES_DMP3 * G3 * (damp1 / rab) * y * y * y +
                         (eq + edd) * AES_DMP5 * G5 * (damp2 / rab) * y * y * y * y;
            t2 += tmp;
        }
        for (int k = 0; k < 3; ++k) g[3 * i + k] += gi[k];
        tmp2[i] = 3.0 * t2;
    }
}

// ------------------------------------------------------------------ D4 dispersion
// newD4Model / weight_references / zeta, src/disp/dftd4.F90:106-203, 588-657, 948-1065
inline double zeta_f(double a, double c, double qref, double qmod) {
    if (qmod < 0.0) return std::exp(a);
    return std::exp(a * (1.0 - std::exp(c * (1.0 - qref / qmod))));
}
inline double dzeta_f(double a, double c, double qref, double qmod) {
    if (qmod < 0.0) return 0.0;
    return -a * c * std::exp(c * (1.0 - qref / qmod)) * zeta_f(a, c, qref, qmod) * qref / (qmod * qmod);
}

void gweights(const Ctx& c, const std::vector<double>& cn, std::vector<double>& gw, std::vector<double>& dgw) {
    const TwinInput& in = c.in;
    int n = c.nat;
    int nd = in.d4_off[n - 1] + in.d4_nref[n - 1];
    gw.assign(nd, 0.0);
    dgw.assign(nd, 0.0);
    for (int i = 0; i < n; ++i) {
        int o = in.d4_off[i], nr = in.d4_nref[i];
        double expw[MAXREF] = {0}, expd[MAXREF] = {0};
        for (int r = 0; r < nr; ++r) {
            double rcn = in.d4_refcn[o + r];
            for (int cc = 1; cc <= in.d4_ncount[o + r]; ++cc) {
                double twf = cc * D4_WF;
                double val = -twf * (cn[i] - rcn) * (cn[i] - rcn);
                double g = val < -200.0 ? 0.0 : std::exp(val);
                expw[r] += g;
                expd[r] += 2 * twf * (rcn - cn[i]) * g;
            }
        }
        double norm = 0, dnorm = 0;
        for (int r = 0; r < nr; ++r) {
            norm += expw[r];
            dnorm += expd[r];
        }
        norm = norm > 1e-80 ? 1.0 / norm : 0.0;
        if (norm == 0.0) {
            double mx = -1e300;
            for (int r = 0; r < nr; ++r) mx = std::max(mx, in.d4_refcn[o + r]);
            for (int r = 0; r < nr; ++r) {
                gw[o + r] = std::fabs(mx - in.d4_refcn[o + r]) < 1e-12 ? 1.0 : 0.0;
                dgw[o + r] = expd[r] * norm - expw[r] * dnorm * norm * norm;
            }
        } else {
            for (int r = 0; r < nr; ++r) {
                gw[o + r] = expw[r] * norm;
                dgw[o + r] = expd[r] * norm - expw[r] * dnorm * norm * norm;
            }
        }
    }
}

inline const double* c6blk(const TwinInput& in, int i, int j) {
    return in.c6ref + ((size_t)in.eidx[i] * in.nelem + in.eidx[j]) * MAXREF * MAXREF;
}

// TxTBDispersion, src/xtb/dispersion.f90:69-138: dispersion matrix W[ndim][ndim] of the
// self-consistent D4 (build_wdispmat src/disp/dftd4.F90:660-732)
struct SCD4 {
    std::vector<double> gw, W;
    int nd = 0;
};

void scd4_setup(const Ctx& c, SCD4& d) {
    const TwinInput& in = c.in;
    int n = c.nat;
    std::vector<double> cn = cn_erf(c, true), dgw;
    gweights(c, cn, d.gw, dgw);
    d.nd = (int)d.gw.size();
    size_t nd = d.nd;
    d.W.assign(nd * nd, 0.0);
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) {
            double r4r2 = 3.0 * in.sqrtzr4r2[i] * in.sqrtzr4r2[j];
            double cut = D4_A1 * std::sqrt(r4r2) + D4_A2;
            double dd[3] = {c.R(j)[0] - c.R(i)[0], c.R(j)[1] - c.R(i)[1], c.R(j)[2] - c.R(i)[2]};
            double r2 = dot3(dd, dd);
            if (r2 > 72.0 * 72.0) continue;
            double c2 = cut * cut, c6 = c2 * c2 * c2;
            double oor6 = 1.0 / (r2 * r2 * r2 + c6);
            double oor8 = 1.0 / (r2 * r2 * r2 * r2 + c6 * c2);
            double oor10 = 1.0 / (r2 * r2 * r2 * r2 * r2 + c6 * c2 * c2);
            const double* blk = c6blk(in, i, j);
            int oi = in.d4_off[i], oj = in.d4_off[j];
            for (int k = 0; k < in.d4_nref[i]; ++k)
                for (int l = 0; l < in.d4_nref[j]; ++l) {
                    double gg = d.gw[oi + k] * d.gw[oj + l];
                    double cc = blk[k * MAXREF + l];
                    double v = gg * (-D4_S6 * cc * oor6 - D4_S8 * (r4r2 * cc) * oor8 -
                                     D4_S10 * (49.0 / 40.0 * r4r2 * r4r2 * cc) * oor10);
                    if (gg < 1e-7) v = 0.0;
                    d.W[(size_t)(oi + k) * nd + oj + l] = v;
                    d.W[(size_t)(oj + l) * nd + oi + k] = v;
                }
        }
}

void scd4_zeta(const Ctx& c, const SCD4& d, const std::vector<double>& q, std::vector<double>& zv,
               std::vector<double>& dz) {
    const TwinInput& in = c.in;
    zv.assign(d.nd, 0.0);
    dz.assign(d.nd, 0.0);
    for (int i = 0; i < c.nat; ++i) {
        double iz = in.d4_zeff[i], gi = in.d4_gam[i] * D4_GC;
        for (int r = 0; r < in.d4_nref[i]; ++r) {
            int o = in.d4_off[i] + r;
            if (d.gw[o] < 1e-7) continue;
            zv[o] = zeta_f(D4_GA, gi, in.d4_refq[o] + iz, q[i] + iz);
            dz[o] = dzeta_f(D4_GA, gi, in.d4_refq[o] + iz, q[i] + iz);
        }
    }
}

std::vector<double> matvec(const std::vector<double>& M, const std::vector<double>& x, int n) {
    std::vector<double> y(n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const double* m = M.data() + (size_t)i * n;
        double s = 0;
        for (int j = 0; j < n; ++j) s += m[j] * x[j];
        y[i] = s;
    }
    return y;
}

// disppot, src/disp/dftd4.F90:735-818 and edisp_scc :821-864
void scd4_potential(const Ctx& c, const SCD4& d, const std::vector<double>& q, std::vector<double>& v) {
    std::vector<double> zv, dz;
    scd4_zeta(c, d, q, zv, dz);
    std::vector<double> dum = matvec(d.W, zv, d.nd);
    v.assign(c.nat, 0.0);
    for (int i = 0; i < c.nat; ++i)
        for (int r = 0; r < c.in.d4_nref[i]; ++r) {
            int o = c.in.d4_off[i] + r;
            v[i] += dum[o] * dz[o];
        }
}

double scd4_energy(const Ctx& c, const SCD4& d, const std::vector<double>& q) {
    std::vector<double> zv, dz;
    scd4_zeta(c, d, q, zv, dz);
    std::vector<double> dum = matvec(d.W, zv, d.nd);
    double e = 0;
    for (int o = 0; o < d.nd; ++o) e += zv[o] * 0.5 * dum[o];
    return e;
}

// d4_full_gradient_latp for a molecule, src/disp/dftd4.F90:1624-1734 (2-body :1832-1933,
// ATM :2023-2177, deriv_atm_triple :2354-2433): returns embd, adds the gradient
double d4_gradient(const Ctx& c, const std::vector<double>& q, double* g) {
    const TwinInput& in = c.in;
    int n = c.nat;
    std::vector<double> cn = cn_lp(c, true), gw, dgw;
    gweights(c, cn, gw, dgw);
    int nd = (int)gw.size();
    std::vector<double> zv(nd), zr(nd), zdcn(nd), zrdcn(nd);
    for (int i = 0; i < n; ++i) {
        double zi = in.d4_zeff[i], gi = D4_GC * in.d4_gam[i];
        for (int r = 0; r < in.d4_nref[i]; ++r) {
            int o = in.d4_off[i] + r;
            double zq = zeta_f(D4_GA, gi, in.d4_refq[o] + zi, q[i] + zi);
            double z0 = zeta_f(D4_GA, gi, in.d4_refq[o] + zi, zi);
            zv[o] = zq * gw[o];
            zr[o] = z0 * gw[o];
            zdcn[o] = zq * dgw[o];
            zrdcn[o] = z0 * dgw[o];
        }
    }
    // c6[i][j] = v_i^T C6ref v_j, dc6[i][j] = dv_i^T C6ref v_j
    auto atomic_c6 = [&](const std::vector<double>& v, const std::vector<double>& dv, std::vector<double>& c6,
                         std::vector<double>& dc6) {
        c6.assign((size_t)n * n, 0.0);
        dc6.assign((size_t)n * n, 0.0);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                const double* blk = c6blk(in, i, j);
                int oi = in.d4_off[i], oj = in.d4_off[j];
                double s = 0, ds = 0;
                for (int k = 0; k < in.d4_nref[i]; ++k) {
                    double t = 0;
                    for (int l = 0; l < in.d4_nref[j]; ++l) t += blk[k * MAXREF + l] * v[oj + l];
                    s += v[oi + k] * t;
                    ds += dv[oi + k] * t;
                }
                c6[(size_t)i * n + j] = s;
                dc6[(size_t)i * n + j] = ds;
            }
    };
    std::vector<double> c6, dc6;
    atomic_c6(zv, zdcn, c6, dc6);
    std::vector<double> dEdcn(n, 0.0);
    int nt = omp_get_max_threads();
    ThreadAcc ga(nt, 3 * n), ca(nt, n);
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; ++i) {
        double* gg = ga.mine();
        double* cc = ca.mine();
        for (int j = 0; j < i; ++j) {
            double rij[3] = {c.R(i)[0] - c.R(j)[0], c.R(i)[1] - c.R(j)[1], c.R(i)[2] - c.R(j)[2]};
            double r2 = dot3(rij, rij);
            if (r2 > 3600.0 || r2 < 1e-10) continue;
            double r4r2 = 3 * in.sqrtzr4r2[i] * in.sqrtzr4r2[j];
            double r0 = D4_A1 * std::sqrt(r4r2) + D4_A2;
            double r02 = r0 * r0, r06 = r02 * r02 * r02;
            double t6 = 1.0 / (r2 * r2 * r2 + r06);
            double t8 = 1.0 / (r2 * r2 * r2 * r2 + r06 * r02);
            double t10 = 1.0 / (r2 * r2 * r2 * r2 * r2 + r06 * r02 * r02);
            double d6 = -6 * r2 * r2 * t6 * t6;
            double d8 = -8 * r2 * r2 * r2 * t8 * t8;
            double d10 = -10 * r2 * r2 * r2 * r2 * t10 * t10;
            double disp = D4_S6 * t6 + D4_S8 * r4r2 * t8 + D4_S10 * 49.0 / 40.0 * r4r2 * r4r2 * t10;
            double ddisp = D4_S6 * d6 + D4_S8 * r4r2 * d8 + D4_S10 * 49.0 / 40.0 * r4r2 * r4r2 * d10;
            double cij = c6[(size_t)i * n + j];
            for (int k = 0; k < 3; ++k) {
                double dG = -cij * ddisp * rij[k];
                gg[3 * i + k] += dG;
                gg[3 * j + k] -= dG;
            }
            cc[i] += -dc6[(size_t)i * n + j] * disp;
            cc[j] += -dc6[(size_t)j * n + i] * disp;
        }
    }
    // ATM three-body term with q = 0 reference charges
    std::vector<double> c6z, dc6z;
    atomic_c6(zr, zrdcn, c6z, dc6z);
    const double cut2 = 1600.0;
    double e3 = 0.0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : e3)
    for (int ia = 0; ia < n; ++ia) {
        double* gg = ga.mine();
        double* cc = ca.mine();
        for (int ja = 0; ja < ia; ++ja) {
            double rij[3] = {c.R(ja)[0] - c.R(ia)[0], c.R(ja)[1] - c.R(ia)[1], c.R(ja)[2] - c.R(ia)[2]};
            double r2ij = dot3(rij, rij);
            if (r2ij > cut2) continue;
            double c6ij = c6z[(size_t)ja * n + ia];
            double cij = D4_A1 * std::sqrt(3.0 * in.sqrtzr4r2[ia] * in.sqrtzr4r2[ja]) + D4_A2;
            for (int k = 0; k < ja; ++k) {
                double rik[3] = {c.R(k)[0] - c.R(ia)[0], c.R(k)[1] - c.R(ia)[1], c.R(k)[2] - c.R(ia)[2]};
                double r2ik = dot3(rik, rik);
                if (r2ik > cut2) continue;
                double rjk[3] = {c.R(k)[0] - c.R(ja)[0], c.R(k)[1] - c.R(ja)[1], c.R(k)[2] - c.R(ja)[2]};
                double r2jk = dot3(rjk, rjk);
                if (r2jk > cut2) continue;
                double c6ik = c6z[(size_t)k * n + ia], c6jk = c6z[(size_t)k * n + ja];
                double cik = D4_A1 * std::sqrt(3.0 * in.sqrtzr4r2[ia] * in.sqrtzr4r2[k]) + D4_A2;
                double cjk = D4_A1 * std::sqrt(3.0 * in.sqrtzr4r2[ja] * in.sqrtzr4r2[k]) + D4_A2;
                double c9 = -std::sqrt(c6ij * c6ik * c6jk);
                double ccc1 = cij * cjk * cik;
                double rrr2 = r2ij * r2jk * r2ik;
                double rrr1 = std::sqrt(rrr2);
                double rrr3 = rrr1 * rrr2;
                double ang_fact = 0.375 / (rrr2 * rrr3);
                double ang = ang_fact * (r2ij + r2jk - r2ik) * (r2ij - r2jk + r2ik) * (-r2ij + r2jk + r2ik) + 1.0 / rrr3;
                double cralp = std::pow(ccc1 / rrr1, D4_ALP / 3.0);
                double fdmp = 1.0 / (1.0 + 6.0 * cralp);
                double dfdmp = -(2.0 * D4_ALP * cralp) * fdmp * fdmp;
                double dE = -fdmp * ang * c9;
                double dang1 = -ang_fact * (r2ij * r2ij * r2ij + r2ij * r2ij * (r2jk + r2ik) +
                                            r2ij * (3.0 * r2jk * r2jk + 2.0 * r2jk * r2ik + 3.0 * r2ik * r2ik) -
                                            5.0 * (r2jk - r2ik) * (r2jk - r2ik) * (r2jk + r2ik));
                double dGr1 = (-dang1 * c9 * fdmp + dfdmp * c9 * ang) / r2ij;
                double dang2 = -ang_fact * (r2ik * r2ik * r2ik + r2ik * r2ik * (r2jk + r2ij) +
                                            r2ik * (3.0 * r2jk * r2jk + 2.0 * r2jk * r2ij + 3.0 * r2ij * r2ij) -
                                            5.0 * (r2jk - r2ij) * (r2jk - r2ij) * (r2jk + r2ij));
                double dGr2 = (-dang2 * c9 * fdmp + dfdmp * c9 * ang) / r2ik;
                double dang3 = -ang_fact * (r2jk * r2jk * r2jk + r2jk * r2jk * (r2ik + r2ij) +
                                            r2jk * (3.0 * r2ik * r2ik + 2.0 * r2ik * r2ij + 3.0 * r2ij * r2ij) -
                                            5.0 * (r2ik - r2ij) * (r2ik - r2ij) * (r2ik + r2ij));
                double dGr3 = (-dang3 * c9 * fdmp + dfdmp * c9 * ang) / r2jk;
                const double s = D4_S9;
                e3 += dE * s;
                for (int x = 0; x < 3; ++x) {
                    gg[3 * ia + x] += s * (-dGr1 * rij[x] - dGr2 * rik[x]);
                    gg[3 * ja + x] += s * (dGr1 * rij[x] - dGr3 * rjk[x]);
                    gg[3 * k + x] += s * (dGr2 * rik[x] + dGr3 * rjk[x]);
                }
                double dc9 = 0.5 * c9 * (dc6z[(size_t)ia * n + ja] / c6ij + dc6z[(size_t)ia * n + k] / c6ik);
                cc[ia] += s * (-ang * fdmp * dc9);
                dc9 = 0.5 * c9 * (dc6z[(size_t)ja * n + ia] / c6ij + dc6z[(size_t)ja * n + k] / c6jk);
                cc[ja] += s * (-ang * fdmp * dc9);
                dc9 = 0.5 * c9 * (dc6z[(size_t)k * n + ia] / c6ik + dc6z[(size_t)k * n + ja] / c6jk);
                cc[k] += s * (-ang * fdmp * dc9);
            }
        }
    }
    ga.reduce_into(g);
    ca.reduce_into(dEdcn.data());
    cn_chain(c, true, dEdcn, g, 1.0);
    return e3;
}

// ------------------------------------------------------------------ repulsion
// repulsionEnGrad_latp (molecular case), src/xtb/repulsion.F90:41-158
double repulsion(const Ctx& c, double* g) {
    const TwinInput& in = c.in;
    int n = c.nat;
    ThreadAcc ga(omp_get_max_threads(), 3 * n);
    double e = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : e)
    for (int i = 0; i < n; ++i) {
        double* gg = ga.mine();
        for (int j = 0; j < i; ++j) {
            double rij[3] = {c.R(i)[0] - c.R(j)[0], c.R(i)[1] - c.R(j)[1], c.R(i)[2] - c.R(j)[2]};
            double r2 = dot3(rij, rij);
            if (r2 > 1600.0 || r2 < 1e-8) continue;
            double r1 = std::sqrt(r2);
            double alpha = std::sqrt(in.rep_alpha[i] * in.rep_alpha[j]);
            double zeff = in.rep_zeff[i] * in.rep_zeff[j];
            double kexp = (in.Z[i] > 2 || in.Z[j] > 2) ? REP_KEXP : REP_KEXP_LIGHT;
            double t16 = std::pow(r1, kexp);
            double t26 = std::exp(-alpha * t16);
            double t27 = std::pow(r1, REP_REXP);
            double dE = zeff * t26 / t27;
            double f = -(alpha * t16 * kexp + REP_REXP) * dE / r2;
            e += dE;
            for (int k = 0; k < 3; ++k) {
                gg[3 * i + k] += f * rij[k];
                gg[3 * j + k] -= f * rij[k];
            }
        }
    }
    ga.reduce_into(g);
    return e;
}

// ------------------------------------------------------------------ SCC helpers
// fermismear, src/scc_core.f90:983-1064: occupations, returns -TS
double fermismear(const std::vector<double>& eig, int nel, double etemp, std::vector<double>& occ) {
    int norbs = (int)eig.size();
    double bkt = KB * AUTOEV * etemp;
    const double thr = 1e-9;
    occ.assign(norbs, 0.0);
    if (nel + 1 > norbs) {
        for (int i = 0; i < nel; ++i) occ[i] = 1.0;
    } else if (nel > 0) {
        double ef = 0.5 * (eig[nel - 1] + eig[nel]);
        double occt = nel;
        for (int it = 0; it < 200; ++it) {
            double tot = 0, totd = 0;
            for (int i = 0; i < norbs; ++i) {
                double x = (eig[i] - ef) / bkt;
                if (x < 50) {
                    double ex = std::exp(x);
                    occ[i] = 1.0 / (ex + 1.0);
                    totd += ex / (bkt * (ex + 1.0) * (ex + 1.0));
                } else {
                    occ[i] = 0.0;
                }
                tot += occ[i];
            }
            ef = ef + (occt - tot) / totd;
            if (std::fabs(occt - tot) <= thr) break;
        }
    }
    double s = 0;
    for (double o : occ)
        if (o > thr && 1.0 - o > thr) s += o * std::log(o) + (1.0 - o) * std::log(1.0 - o);
    return s * KB * etemp;
}

// small dense inverse by Gauss-Jordan with partial pivoting (the reference calls dgetrf/dgetri)
void invert(std::vector<double>& a, int m) {
    std::vector<double> inv((size_t)m * m, 0.0);
    for (int i = 0; i < m; ++i) inv[(size_t)i * m + i] = 1.0;
    for (int col = 0; col < m; ++col) {
        int piv = col;
        for (int r = col + 1; r < m; ++r)
            if (std::fabs(a[(size_t)r * m + col]) > std::fabs(a[(size_t)piv * m + col])) piv = r;
        if (piv != col)
            for (int k = 0; k < m; ++k) {
                std::swap(a[(size_t)piv * m + k], a[(size_t)col * m + k]);
                std::swap(inv[(size_t)piv * m + k], inv[(size_t)col * m + k]);
            }
        double d = 1.0 / a[(size_t)col * m + col];
        for (int k = 0; k < m; ++k) {
            a[(size_t)col * m + k] *= d;
            inv[(size_t)col * m + k] *= d;
        }
        for (int r = 0; r < m; ++r) {
            if (r == col) continue;
            double f = a[(size_t)r * m + col];
            if (f == 0.0) continue;
            for (int k = 0; k < m; ++k) {
                a[(size_t)r * m + k] -= f * a[(size_t)col * m + k];
                inv[(size_t)r * m + k] -= f * inv[(size_t)col * m + k];
            }
        }
    }
    a.swap(inv);
}

// Modified Broyden mixing (Johnson 1988), src/broyden.f90:37-153
struct Broyden {
    std::vector<double> omega;
    std::vector<std::vector<double>> df, u;
    std::vector<double> qlast, dqlast;
};

std::vector<double> broyden(const std::vector<double>& q, const std::vector<double>& dq, int it, double alpha,
                            Broyden& st) {
    const double omega0 = 0.01, minw = 1.0, maxw = 100000.0, wfac = 0.01;
    size_t nb = q.size();
    std::vector<double> qn(nb);
    if (it == 1) {
        st.dqlast = dq;
        st.qlast = q;
        for (size_t k = 0; k < nb; ++k) qn[k] = q[k] + alpha * dq[k];
        return qn;
    }
    int it1 = it - 1;
    double om = 0;
    for (double v : dq) om += v * v;
    om = std::sqrt(om);
    om = om > wfac / maxw ? wfac / om : maxw;
    om = std::max(om, minw);
    st.omega.push_back(om);
    std::vector<double> dfv(nb);
    double nrm = 0;
    for (size_t k = 0; k < nb; ++k) {
        dfv[k] = dq[k] - st.dqlast[k];
        nrm += dfv[k] * dfv[k];
    }
    double inv = 1.0 / std::sqrt(nrm);
    for (double& v : dfv) v *= inv;
    st.df.push_back(dfv);
    std::vector<double> beta((size_t)it1 * it1), cvec(it1);
    for (int i = 0; i < it1; ++i) {
        double cd = 0;
        for (size_t k = 0; k < nb; ++k) cd += st.df[i][k] * dq[k];
        cvec[i] = st.omega[i] * cd;
        for (int j = 0; j <= i; ++j) {
            double a = 0;
            for (size_t k = 0; k < nb; ++k) a += st.df[i][k] * st.df[j][k];
            beta[(size_t)i * it1 + j] = beta[(size_t)j * it1 + i] = st.omega[i] * st.omega[j] * a;
        }
        beta[(size_t)i * it1 + i] += omega0 * omega0;
    }
    invert(beta, it1);
    std::vector<double> gamma(it1, 0.0);
    for (int j = 0; j < it1; ++j)
        for (int i = 0; i < it1; ++i) gamma[j] += cvec[i] * beta[(size_t)i * it1 + j];
    std::vector<double> un(nb);
    for (size_t k = 0; k < nb; ++k) un[k] = alpha * dfv[k] + inv * (q[k] - st.qlast[k]);
    st.u.push_back(un);
    st.dqlast = dq;
    st.qlast = q;
    for (size_t k = 0; k < nb; ++k) qn[k] = q[k] + alpha * dq[k];
    for (int i = 0; i < it1; ++i) {
        double w = st.omega[i] * gamma[i];
        for (size_t k = 0; k < nb; ++k) qn[k] -= w * st.u[i][k];
    }
    return qn;
}

// dmat, src/scc_core.f90:1177-1205: P = C diag(f) C^T as one full GEMM (C column-major)
void density(const Ctx& c, const std::vector<double>& C, const std::vector<double>& f, std::vector<double>& P) {
    int n = c.nao;
    std::vector<double> Cf((size_t)n * n);
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) Cf[(size_t)j * n + i] = C[(size_t)j * n + i] * f[j];
    P.assign((size_t)n * n, 0.0);
    char tn = 'N', tt = 'T';
    double one = 1.0, zero = 0.0;
    c.dgemm(&tn, &tt, &n, &n, &n, &one, const_cast<double*>(C.data()), &n, Cf.data(), &n, &zero, P.data(), &n);
}

// build_dSDQH0_noreset, src/xtb/hamiltonian.F90:575-792: gradient of the overlap-, dipole- and
// quadrupole-dependent terms; accumulates g and dhdcn
void grad_sdqh0(const Ctx& c, const std::vector<double>& se, double intcut, const std::vector<double>& P,
                const std::vector<double>& Pew, const std::vector<double>& ves, const std::vector<double>& vs,
                const std::vector<double>& vd, const std::vector<double>& vq, const std::vector<double>& H0n,
                double* g, std::vector<double>& dhdcn) {
    const TwinInput& in = c.in;
    int n = c.nao, N = c.nat;
    int nt = omp_get_max_threads();
    ThreadAcc ga(nt, 3 * N), ca(nt, N);
#pragma omp parallel for schedule(dynamic, 4)
    for (int ish = 0; ish < c.nsh; ++ish) {
        double* gg = ga.mine();
        double* cc = ca.mine();
        int iat = in.sh_atom[ish];
        ShellRef si = shell_ref(c, ish);
        double ib[10][6][6], db[3][10][6][6], iaa[10][6][6], da[3][10][6][6];
        for (int jsh = 0; jsh < c.nsh; ++jsh) {
            int jat = in.sh_atom[jsh];
            if (!(iat > jat)) continue;
            const double *RA = c.R(iat), *RB = c.R(jat);
            double rij[3] = {RA[0] - RB[0], RA[1] - RB[1], RA[2] - RB[2]};
            double rab2 = dot3(rij, rij);
            if (rab2 > 1600.0) continue;
            ShellRef sj = shell_ref(c, jsh);
            pair_moments(si, sj, RA, RB, RB, intcut, true, false, ib, db);
            pair_moments(si, sj, RA, RB, RA, intcut, true, true, iaa, da);
            double rab = std::sqrt(rab2);
            double rr = in.atomicrad[iat] + in.atomicrad[jat];
            double t14 = std::sqrt(rab / rr);
            double k1 = in.shpoly[ish] * 0.01, k2 = in.shpoly[jsh] * 0.01;
            double t15 = k1 * t14, t23 = k2 * t14;
            double shp = (1.0 + t15) * (1.0 + k2 * t14);
            double dsf = (t15 * (1.0 + t23) + (1.0 + t15) * k2 * t14) * 0.5 / rab2;
            double hav = 0.5 * (se[ish] + se[jsh]);
            int ni = NSPH[si.l], nj = NSPH[sj.l];
            double gx[3] = {0, 0, 0}, dcn = 0;
            for (int a = 0; a < ni; ++a)
                for (int b = 0; b < nj; ++b) {
                    size_t ia = in.sh_ao[ish] + a, jb = in.sh_ao[jsh] + b;
                    size_t o = jb * n + ia;
                    double Pij = P[o];
                    double HP = H0n[o] * EVTOAU * Pij;
                    double Sij = ib[0][a][b];
                    double term = 2 * HP - 2 * Pew[o] - Pij * (ves[ish] + ves[jsh]) + Pij * (vs[iat] + vs[jat]);
                    for (int x = 0; x < 3; ++x) {
                        double v = 2 * HP * Sij / shp * dsf * rij[x] + db[x][0][a][b] * term;
                        double dt = 0, qt = 0;
                        for (int k = 0; k < 3; ++k)
                            dt += da[x][1 + k][a][b] * vd[3 * iat + k] + db[x][1 + k][a][b] * vd[3 * jat + k];
                        for (int k = 0; k < 6; ++k)
                            qt += da[x][4 + k][a][b] * vq[6 * iat + k] + db[x][4 + k][a][b] * vq[6 * jat + k];
                        gx[x] += v + Pij * (dt + qt);
                    }
                    dcn += HP / hav * Sij;
                }
            double dsei = -in.kcn[ish], dsej = -in.kcn[jsh];
            cc[iat] += dcn * dsei;
            cc[jat] += dcn * dsej;
            for (int x = 0; x < 3; ++x) {
                gg[3 * iat + x] += gx[x];
                gg[3 * jat + x] -= gx[x];
            }
        }
    }
    ga.reduce_into(g);
    ca.reduce_into(dhdcn.data());
}

}  // namespace

extern "C" {

// One GFN2-xTB single point (energy, charges, gradient, dipole, bond orders) following scf,
// src/scf_module.F90:74-920, and scc, src/scc_core.f90:255-640.  Returns 0 on success,
// 1 when the EEQ matrix is singular, 2 when a LAPACK step fails.
int twin_singlepoint(const TwinInput* inp, const TwinLapack* lap, TwinOutput* out);
}

namespace {
int singlepoint_impl(const TwinInput& in, const TwinLapack* lap, TwinOutput* out);
}

extern "C" {

int twin_singlepoint(const TwinInput* inp, const TwinLapack* lap, TwinOutput* out) {
    const TwinInput& in = *inp;
    // OpenMP threads scaled to the molecule: a few dozen orbitals per thread at least
    int saved_threads = omp_get_max_threads();
    omp_set_num_threads(std::max(1, std::min(omp_get_num_procs(), in.nao / 32)));
    int rc = singlepoint_impl(in, lap, out);
    omp_set_num_threads(saved_threads);
    return rc;
}

}  // extern "C"

namespace {

int singlepoint_impl(const TwinInput& in, const TwinLapack* lap, TwinOutput* out) {
    Ctx c(in);
    c.dpotrf = (dpotrf_t)lap->dpotrf;
    c.dsygst = (dsygst_t)lap->dsygst;
    c.dsyevd = (dsyevd_t)lap->dsyevd;
    c.dsysv = (dsysv_t)lap->dsysv;
    c.dtrsm = (dtrsm_t)lap->dtrsm;
    c.dgemm = (dgemm_t)lap->dgemm;
    int N = c.nat, nsh = c.nsh, n = c.nao;
    size_t nn = (size_t)n * n;
    double t0 = now();
    // thresholds, src/scf_module.F90:266-277
    double intcut = std::max(20.0, 25.0 - 10.0 * std::log10(in.accuracy));
    double neglect = 10.0e-9 * in.accuracy;
    double scfconv = 1.0e-6 * in.accuracy;
    double qconv = 1.0e-4 * in.accuracy;
    std::vector<int> ao_shell(n), ao_atom(n);
    for (int s = 0; s < nsh; ++s)
        for (int a = 0; a < NSPH[in.sh_l[s]]; ++a) {
            ao_shell[in.sh_ao[s] + a] = s;
            ao_atom[in.sh_ao[s] + a] = in.sh_atom[s];
        }
    // initial guess: EEQ charges, iniqshell src/scc_core.f90:1475-1506
    std::vector<double> q0(N, in.charge / N);
    if (in.guess_eeq && !eeq_guess(c, q0)) return 1;
    std::vector<double> qsh(nsh), q(N, 0.0), dipm(3 * N, 0.0), qp(6 * N, 0.0);
    for (int s = 0; s < nsh; ++s) {
        int a = in.sh_atom[s];
        qsh[s] = in.zsh[s] / in.zval[a] * q0[a];
    }
    for (int s = 0; s < nsh; ++s) q[in.sh_atom[s]] += qsh[s];
    std::vector<double> grad(3 * N, 0.0);
    double erep = repulsion(c, grad.data());
    std::vector<double> cn = cn_lp(c, false);
    SCD4 scd4;
    scd4_setup(c, scd4);
    std::vector<double> se(nsh);
    for (int s = 0; s < nsh; ++s) se[s] = in.se0[s] - in.kcn[s] * cn[in.sh_atom[s]];
    std::vector<double> S, D, Q, H0, H0n;
    build_sdqh0(c, se, intcut, S, D, Q, H0, H0n);
    // setdqlist screening, src/aespot.F90:34-85: masked copies of D and Q
    std::vector<double> Dm(D), Qm(Q);
    {
        double thr2 = neglect * 1.0e-2;
#pragma omp parallel for schedule(static)
        for (long long o = 0; o < (long long)nn; ++o) {
            double t1 = 0, t2 = 0;
            for (int k = 0; k < 3; ++k) t1 += D[k * nn + o] * D[k * nn + o];
            for (int k = 0; k < 3; ++k) t2 += Q[k * nn + o] * Q[k * nn + o];
            for (int k = 3; k < 6; ++k) t2 += 2.0 * Q[k * nn + o] * Q[k * nn + o];
            if (!(t1 > thr2))
                for (int k = 0; k < 3; ++k) Dm[k * nn + o] = 0.0;
            if (!(t2 > thr2))
                for (int k = 0; k < 6; ++k) Qm[k * nn + o] = 0.0;
        }
    }
    std::vector<double> rad, dr, gab3, gab5;
    aes_setup(c, cn, rad, dr, gab3, gab5);
    // Coulomb matrix, src/coulomb/klopmanohno.F90:257-312 (Klopman-Ohno, exponent 2)
    std::vector<double> J((size_t)nsh * nsh);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nsh; ++i)
        for (int j = 0; j < nsh; ++j) {
            int a = in.sh_atom[i], b = in.sh_atom[j];
            double gij = 0.5 * (in.eta[i] + in.eta[j]);
            if (a == b) {
                J[(size_t)i * nsh + j] = gij;
            } else {
                double d[3] = {c.R(a)[0] - c.R(b)[0], c.R(a)[1] - c.R(b)[1], c.R(a)[2] - c.R(b)[2]};
                J[(size_t)i * nsh + j] = 1.0 / std::sqrt(dot3(d, d) + 1.0 / (gij * gij));
            }
        }
    // Cholesky of S once, src/scc_core.f90:411-413
    std::vector<double> U(S);
    {
        char up = 'U';
        int info = 0;
        c.dpotrf(&up, &n, U.data(), &n, &info);
        if (info != 0) return 2;
    }
    double t1 = now();
    out->seconds[0] = t1 - t0;
    // SCC, src/scc_core.f90:406-640
    int nbr = nsh + 9 * N;
    Broyden st;
    double eel = 0, ees = 0, eaes = 0, epol = 0, ed = 0, ga = 0, gb = 0;
    bool lastdiag = false, converged = false;
    int iters = 0;
    std::vector<double> shift(nsh), vs, vd, vq, atshift, H(nn), A, emo(n), C, P, fa, fb, focc(n);
    int lwork = -1, liwork = -1;
    std::vector<double> work;
    std::vector<int> iwork;
    for (int it = 1; it <= in.maxiter; ++it) {
        iters = it;
        std::vector<double> Jq = matvec(J, qsh, nsh);
        for (int s = 0; s < nsh; ++s) shift[s] = Jq[s] + in.gam3[s] * qsh[s] * qsh[s];
        setvsdq(c, q, dipm, qp, gab3, gab5, true, vs, vd, vq);
        scd4_potential(c, scd4, q, atshift);
        for (int s = 0; s < nsh; ++s) shift[s] += atshift[in.sh_atom[s]];
        // buildIsoAnisotropicH1, src/scc_core.f90:154-251 (eV)
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            int ai = ao_atom[i], si = ao_shell[i];
            for (int j = 0; j < n; ++j) {
                size_t o = (size_t)i * n + j;
                int aj = ao_atom[j], sj = ao_shell[j];
                double dum = S[o] * AUTOEV * 0.5;
                double h = H0[o] - dum * (shift[si] + shift[sj]) + dum * (vs[ai] + vs[aj]);
                double t = 0;
                for (int k = 0; k < 3; ++k) t += Dm[k * nn + o] * (vd[3 * ai + k] + vd[3 * aj + k]);
                for (int k = 0; k < 6; ++k) t += Qm[k * nn + o] * (vq[6 * ai + k] + vq[6 * aj + k]);
                H[o] = h + 0.5 * AUTOEV * t;
            }
        }
        // generalised eigenproblem: dsygst + dsyevd + dtrsm
        A = H;
        {
            int itype = 1, info = 0;
            char up = 'U', jv = 'V';
            c.dsygst(&itype, &up, &n, A.data(), &n, U.data(), &n, &info);
            if (info != 0) return 2;
            if (lwork < 0) {
                double wq;
                int iwq, lw = -1, liw = -1;
                c.dsyevd(&jv, &up, &n, A.data(), &n, emo.data(), &wq, &lw, &iwq, &liw, &info);
                lwork = std::max(1, (int)wq);
                liwork = std::max(1, iwq);
                work.resize(lwork);
                iwork.resize(liwork);
            }
            c.dsyevd(&jv, &up, &n, A.data(), &n, emo.data(), work.data(), &lwork, iwork.data(), &liwork, &info);
            if (info != 0) return 2;
            char l = 'L', nt = 'N';
            double one = 1.0;
            c.dtrsm(&l, &up, &nt, &nt, &n, &n, &one, U.data(), &n, A.data(), &n);
            C.swap(A);
        }
        ga = fermismear(emo, in.ihomoa, in.etemp, fa);
        gb = fermismear(emo, in.ihomob, in.etemp, fb);
        for (int i = 0; i < n; ++i) focc[i] = fa[i] + fb[i];
        std::vector<double> q_in(nbr);
        std::copy(qsh.begin(), qsh.end(), q_in.begin());
        std::copy(dipm.begin(), dipm.end(), q_in.begin() + nsh);
        std::copy(qp.begin(), qp.end(), q_in.begin() + nsh + 3 * N);
        density(c, C, focc, P);
        // Mulliken shell populations, mpopsh src/scc_core.f90:1408-1444
        std::vector<double> rowps(n);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            double s = 0;
            for (int j = 0; j < n; ++j) s += P[(size_t)i * n + j] * S[(size_t)i * n + j];
            rowps[i] = s;
        }
        std::vector<double> pop(nsh, 0.0);
        for (int i = 0; i < n; ++i) pop[ao_shell[i]] += rowps[i];
        for (int s = 0; s < nsh; ++s) qsh[s] = in.zsh[s] - pop[s];
        std::fill(q.begin(), q.end(), 0.0);
        for (int s = 0; s < nsh; ++s) q[in.sh_atom[s]] += qsh[s];
        double eold = eel;
        // electro, src/scc_core.f90:686-722
        std::vector<double> Jq2 = matvec(J, qsh, nsh);
        double es = 0;
        for (int s = 0; s < nsh; ++s) es += 0.5 * qsh[s] * Jq2[s] + in.gam3[s] * qsh[s] * qsh[s] * qsh[s] / 3.0;
        double h = 0;
#pragma omp parallel for schedule(static) reduction(+ : h)
        for (int i = 0; i < n; ++i) {
            for (int j = 0; j < i; ++j) h += P[(size_t)i * n + j] * H0[(size_t)i * n + j];
            h += 0.5 * P[(size_t)i * n + i] * H0[(size_t)i * n + i];
        }
        eel = es + 2.0 * h * EVTOAU;
        ees = es;
        mmompop(c, P, S, D, Q, ao_atom, dipm, qp);
        aniso_electro(c, q, dipm, qp, gab3, gab5, eaes, epol);
        eel += eaes + epol;
        ed = scd4_energy(c, scd4, q);
        eel += ed;
        eel += ga + gb;
        bool econv = std::fabs(eel - eold) < scfconv;
        std::vector<double> dq(nbr);
        double rms = 0;
        for (int s = 0; s < nsh; ++s) dq[s] = qsh[s] - q_in[s];
        for (int k = 0; k < 3 * N; ++k) dq[nsh + k] = dipm[k] - q_in[nsh + k];
        for (int k = 0; k < 6 * N; ++k) dq[nsh + 3 * N + k] = qp[k] - q_in[nsh + 3 * N + k];
        for (double v : dq) rms += v * v;
        rms = std::sqrt(rms / N);
        bool qconvd = rms < qconv;
        std::vector<double> qn;
        if (N > 1) {
            qn = broyden(q_in, dq, it, 0.4, st);
        } else {
            qn.resize(nbr);
            for (int k = 0; k < nbr; ++k) qn[k] = q_in[k] + dq[k];
        }
        std::copy(qn.begin(), qn.begin() + nsh, qsh.begin());
        std::copy(qn.begin() + nsh, qn.begin() + nsh + 3 * N, dipm.begin());
        std::copy(qn.begin() + nsh + 3 * N, qn.end(), qp.begin());
        std::fill(q.begin(), q.end(), 0.0);
        for (int s = 0; s < nsh; ++s) q[in.sh_atom[s]] += qsh[s];
        if (econv && qconvd) {
            converged = true;
            if (lastdiag) break;
            lastdiag = true;
        }
    }
    double t2 = now();
    out->seconds[1] = t2 - t1;
    // gradient block, src/scf_module.F90:665-798
    std::vector<double> fw(n), Pew;
    for (int i = 0; i < n; ++i) fw[i] = focc[i] * emo[i] * EVTOAU;
    density(c, C, fw, Pew);
    std::vector<double> vs2, vd2, vq2;
    setvsdq(c, q, dipm, qp, gab3, gab5, false, vs2, vd2, vq2);
    std::vector<double> dhdcn(N, 0.0);
    grad_sdqh0(c, se, intcut, P, Pew, shift, vs2, vd2, vq2, H0n, grad.data(), dhdcn);
    for (int i = 0; i < n; ++i) dhdcn[ao_atom[i]] += P[(size_t)i * n + i] * (-in.kcn[ao_shell[i]]) * EVTOAU;
    cn_chain(c, false, dhdcn, grad.data(), 1.0);
    std::vector<double> tmp2;
    aniso_grad(c, q, dipm, qp, rad, gab3, gab5, grad.data(), tmp2);
    for (int i = 0; i < N; ++i) tmp2[i] *= dr[i];
    cn_chain(c, false, tmp2, grad.data(), -1.0);
    double embd = d4_gradient(c, q, grad.data());
    // getCoulombDerivsCluster contracted with qsh, src/coulomb/klopmanohno.F90:471-573
    {
        ThreadAcc gacc(omp_get_max_threads(), 3 * N);
#pragma omp parallel for schedule(dynamic, 16)
        for (int i = 0; i < nsh; ++i) {
            double* gg = gacc.mine();
            int a = in.sh_atom[i];
            for (int j = 0; j < nsh; ++j) {
                int b = in.sh_atom[j];
                if (!(a > b)) continue;
                double d[3] = {c.R(b)[0] - c.R(a)[0], c.R(b)[1] - c.R(a)[1], c.R(b)[2] - c.R(a)[2]};
                double gij = 0.5 * (in.eta[i] + in.eta[j]);
                double g1 = 1.0 / (dot3(d, d) + 1.0 / (gij * gij));
                double fac = -g1 * std::sqrt(g1) * qsh[i] * qsh[j];
                for (int k = 0; k < 3; ++k) {
                    gg[3 * a + k] -= fac * d[k];
                    gg[3 * b + k] += fac * d[k];
                }
            }
        }
        gacc.reduce_into(grad.data());
    }
    double t3 = now();
    out->seconds[2] = t3 - t2;
    // dipole moment (calc_dipole, src/dipole.f90:94-128) and Wiberg-Mayer bond orders
    // (get_wiberg src/scc_core.f90:1208-1245, get_unrestricted_wiberg :1248-1295)
    for (int k = 0; k < 3; ++k) {
        double s = 0;
        for (int a = 0; a < N; ++a) s += c.R(a)[k] * in.zval[a];
        double t = 0;
#pragma omp parallel for schedule(static) reduction(+ : t)
        for (long long o = 0; o < (long long)nn; ++o) t += D[k * nn + o] * P[o];
        out->dipole[k] = s - t;
    }
    {
        std::vector<std::vector<double>> PSs;
        double fac = 1.0;
        char tn = 'N';
        double one = 1.0, zero = 0.0;
        auto ps_of = [&](const std::vector<double>& Pm) {
            std::vector<double> PS(nn);
            // column-major: (P S)^T = S P for symmetric factors; PS[i][j] row-major = (P S)_ij
            c.dgemm(&tn, &tn, &n, &n, &n, &one, const_cast<double*>(S.data()), &n, const_cast<double*>(Pm.data()),
                    &n, &zero, PS.data(), &n);
            return PS;
        };
        if (in.ihomoa == in.ihomob) {
            PSs.push_back(ps_of(P));
        } else {
            std::vector<double> Pa, Pb;
            density(c, C, fa, Pa);
            density(c, C, fb, Pb);
            PSs.push_back(ps_of(Pa));
            PSs.push_back(ps_of(Pb));
            fac = 2.0;
        }
        std::vector<int> ao0(N, n), ao1(N, 0);
        for (int i = 0; i < n; ++i) {
            ao0[ao_atom[i]] = std::min(ao0[ao_atom[i]], i);
            ao1[ao_atom[i]] = std::max(ao1[ao_atom[i]], i + 1);
        }
        if (out->wbo) std::fill(out->wbo, out->wbo + (size_t)N * N, 0.0);
#pragma omp parallel for schedule(dynamic, 16)
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < i; ++j) {
                double d[3] = {c.R(i)[0] - c.R(j)[0], c.R(i)[1] - c.R(j)[1], c.R(i)[2] - c.R(j)[2]};
                if (dot3(d, d) >= 100.0) continue;
                double tot = 0;
                for (auto& PS : PSs)
                    for (int a = ao0[i]; a < ao1[i]; ++a)
                        for (int b = ao0[j]; b < ao1[j]; ++b)
                            tot += PS[(size_t)a * n + b] * PS[(size_t)b * n + a];
                if (out->wbo) out->wbo[(size_t)i * N + j] = out->wbo[(size_t)j * N + i] = fac * tot;
            }
    }
    out->seconds[3] = now() - t3;
    out->energy = eel + erep + embd;
    out->e_elec = eel + embd;
    out->e_rep = erep;
    out->e_es = ees;
    out->e_aes = eaes;
    out->e_axc = epol;
    out->e_disp = ed + embd;
    out->iterations = iters;
    out->converged = converged ? 1 : 0;
    std::copy(q.begin(), q.end(), out->q);
    std::copy(qsh.begin(), qsh.end(), out->qsh);
    std::copy(grad.begin(), grad.end(), out->gradient);
    std::copy(emo.begin(), emo.end(), out->emo);
    std::copy(focc.begin(), focc.end(), out->focc);
    return 0;
}

}  // namespace
