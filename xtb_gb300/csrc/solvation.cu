// GBSA / ALPB implicit solvation: host set-up and device kernels (see solvation.h).
//
// Reference algorithm (restated, not translated):
//   parameters        src/solv/model.f90:510-545 (paramToModel), src/solv/state.f90
//   model set-up      src/solv/gbsa.f90:217-389 (initBorn)
//   Born radii        src/solv/born.f90 (compute_psi, compute_bornr; GBOBC-II)
//   SASA              src/solv/sasa.f90 (compute_numsa, compute_w_sp), src/solv/lebedev.f90
//   Born matrix       src/solv/kernel.f90:586-760, src/solv/gbsa.f90:445-491
//   shift, energy     src/solv/gbsa.f90:495-548
//   gradient          src/solv/kernel.f90:171-378 (+ the salt variant), src/solv/gbsa.f90:600-777
//
// Device layout: every per-atom quantity is a plain array over atoms; the SASA switching
// products of every grid point are kept ([nat][npt]) so that the gradient can revisit a
// neighbour's surface points without recomputing their products; B is a full nat x nat matrix.
// Each kernel gives one owner (a warp or a block) per atom and sums in a fixed order, so the
// results are bitwise reproducible.
#include "solvation.h"

#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <map>
#include <set>

#include "common.cuh"
#include "solvation_params.inc"

namespace xg {

namespace {

constexpr double AATOAU = 1.0 / AUTOAA;
constexpr double KCALTOAU = 1.0 / 627.50947428;          // src/mctc/convert.f90:31-32
constexpr double MOLCM3TOAU = 8.92388e-2;                 // src/solv/model.f90:153
constexpr double SURFACE_TENSION = 1.0e-5;                // src/solv/model.f90:156
constexpr double LRCUT = 35.0 * AATOAU;                   // Born-radius pair cutoff
constexpr double ROFFSET = 2.0 * AATOAU;                  // SASA neighbour margin
constexpr double SW_W = 0.3 * AATOAU;                     // SASA switching half-width
constexpr double AH0 = 0.5;
constexpr double AH1 = 3.0 / (4.0 * SW_W);
constexpr double AH3 = -1.0 / (4.0 * SW_W * SW_W * SW_W);
constexpr double TOLSESP = 1.0e-6;
constexpr double OBC_A = 1.0, OBC_B = 0.8, OBC_G = 4.85;  // GBOBC-II
constexpr double ZETA_P16 = 1.028;
constexpr double ALPB_ALPHA = 0.571412;
constexpr double KAPPA_CONST = 0.7897e-3;

std::string lower(std::string s) {
    for (auto& c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}

// solvent aliases (normalizeSolventName, src/solv/model.f90:215-249)
std::string normalise(const std::string& in) {
    static const std::map<std::string, std::string> alias = {
        {"methylcyanide", "acetonitrile"}, {"methylenechloride", "ch2cl2"}, {"dichloromethane", "ch2cl2"},
        {"dcm", "ch2cl2"}, {"dichlormethane", "ch2cl2"}, {"chloroform", "chcl3"}, {"trichloromethane", "chcl3"},
        {"tcm", "chcl3"}, {"carbondisulfide", "cs2"}, {"diethylether", "ether"}, {"dimethylformamide", "dmf"},
        {"dimethylsulfoxide", "dmso"}, {"furan", "furane"}, {"nhexan", "hexane"}, {"n-hexan", "hexane"},
        {"nhexane", "hexane"}, {"n-hexane", "hexane"}, {"tetrahydrofuran", "thf"}, {"h2o", "water"}};
    const std::string s = lower(in);
    auto it = alias.find(s);
    return it == alias.end() ? s : it->second;
}

// the Lebedev-Laikov grid the reference selects for `nang` (bisection of src/mctc/search.f90:37-79:
// the largest size <= nang, except nang equal to the largest size selects the one below)
int grid_index(int nang) {
    using namespace solvdata;
    if (nang < GRID_SIZE[0]) return -1;
    if (nang == GRID_SIZE[NGRIDS - 1]) return NGRIDS - 2;
    int k = 0;
    for (int i = 0; i < NGRIDS; ++i)
        if (GRID_SIZE[i] <= nang) k = i;
    return k;
}

// points and weights of grid k: each generator expands to the orbit of its point under the
// octahedral group (all coordinate permutations and sign changes)
void expand_grid(int k, std::vector<double>& out) {
    using namespace solvdata;
    out.clear();
    for (int g = GRID_GEN_OFFSET[k]; g < GRID_GEN_OFFSET[k + 1]; ++g) {
        const int kind = (int)GRID_GEN[g][0];
        const double a = GRID_GEN[g][1], b = GRID_GEN[g][2], v = GRID_GEN[g][3];
        std::array<double, 3> base;
        switch (kind) {
            case 1: base = {1.0, 0.0, 0.0}; break;
            case 2: base = {0.0, std::sqrt(0.5), std::sqrt(0.5)}; break;
            case 3: {
                const double s = std::sqrt(1.0 / 3.0);
                base = {s, s, s};
                break;
            }
            case 4: base = {a, a, std::sqrt(1.0 - 2.0 * a * a)}; break;
            case 5: base = {a, std::sqrt(1.0 - a * a), 0.0}; break;
            default: base = {a, b, std::sqrt(1.0 - a * a - b * b)}; break;
        }
        std::set<std::array<double, 3>> orbit;
        std::array<int, 3> perm = {0, 1, 2};
        do {
            for (int sg = 0; sg < 8; ++sg) {
                std::array<double, 3> p;
                for (int c = 0; c < 3; ++c) p[c] = ((sg >> c) & 1 ? -1.0 : 1.0) * base[perm[c]];
                for (auto& x : p)
                    if (x == 0.0) x = 0.0;   // one zero, not +0 and -0
                orbit.insert(p);
            }
        } while (std::next_permutation(perm.begin(), perm.end()));
        for (const auto& p : orbit) out.insert(out.end(), {p[0], p[1], p[2], v});
    }
    if ((int)out.size() != 4 * GRID_SIZE[k]) throw std::runtime_error("Lebedev grid expansion failed");
}

}  // namespace

std::string make_solvent_spec(const std::string& solvent, const std::string& model, int state, double temperature,
                              int nang, SolventSpec& out, int kernel) {
    using namespace solvdata;
    SolventSpec s;
    const std::string raw = lower(solvent);
    if (raw == "none" || raw == "gas" || raw == "vac") {   // addSolvationModel, src/main/setup.f90:223-228
        out = s;
        return "";
    }
    const std::string m = lower(model);
    if (m == "gbsa") {
        s.kernel = 0;
        s.alpb = false;
    } else if (m == "alpb") {
        s.kernel = 1;
        s.alpb = true;
    } else if (m == "cosmo" || m == "tmcosmo" || m == "cpcmx") {
        return "Solvation model '" + m + "' is not supported by this engine (GBSA and ALPB are)";
    } else {
        return "Unknown solvation model";
    }
    if (kernel == 0 || kernel == 1) s.kernel = kernel;
    std::string name = normalise(solvent);
    // the GBSA tables name two solvents differently (loadInternalParam, src/solv/model.f90:280-300)
    std::string key = name;
    if (s.kernel == 0 && name == "water") key = "h2o";
    if (s.kernel == 0 && name == "hexane") key = "nhexan";
    for (int i = 0; i < NSETS; ++i)
        if (SETS[i].alpb == s.kernel && key == SETS[i].solvent) s.set = i;
    if (s.set < 0) return "solvent: '" + name + "' is not parametrized";
    if (grid_index(nang) < 0) return "Invalid angular grid size " + std::to_string(nang);
    if (!(temperature > 0.0) || !std::isfinite(temperature)) return "Invalid solvent temperature";
    s.on = true;
    s.solvent = name;
    s.state = state;
    s.temperature = temperature;
    s.nang = nang;
    out = s;
    return "";
}

void build_solv_host(const SolventSpec& spec, int nat, const int* Z, const double* xyz, SolvHost& h) {
    using namespace solvdata;
    const ParamSet& p = SETS[spec.set];
    h = SolvHost();
    h.nat = nat;
    h.kernel = spec.kernel;
    h.alpb = spec.alpb;
    h.eps = p.epsv;
    h.alpbet = spec.alpb ? ALPB_ALPHA / p.epsv : 0.0;
    h.keps = (1.0 / p.epsv - 1.0) / (1.0 + h.alpbet);
    h.c1 = p.c1;
    // free-energy shift of the parameter set plus that of the solution state (src/solv/state.f90)
    const double density = p.rhos / p.smass * MOLCM3TOAU;
    double sshift = 0.0;
    if (spec.state == 2)
        sshift = spec.temperature * KB_AU *
                 (std::log(24.79 * spec.temperature / 298.15) + std::log(density / 1.0e-3 * 1.0 / p.smass));
    else if (spec.state == 3)
        sshift = spec.temperature * KB_AU * std::log(24.79 * spec.temperature / 298.15);
    h.gshift = p.gshift * KCALTOAU + sshift;
    bool any_hb = false;
    for (int e = 0; e < 94; ++e) any_hb = any_hb || std::fabs(p.tmp[e]) > 1.0e-3;
    const double offset = p.soset * 0.1 * AATOAU, probe = p.rprobe * AATOAU;
    double maxsa = 0.0;
    for (int i = 0; i < nat; ++i) {
        const int e = Z[i] - 1;
        const double vdw = VDW_RAD_D3[e];
        const double sa = vdw + probe;
        h.vdwr.push_back(vdw);
        h.rho.push_back(vdw * p.sx[e]);
        h.svdw.push_back(vdw - offset);
        h.vdwsa.push_back(sa);
        auto part = [&](double r) {
            return (0.25 / SW_W + 3.0 * AH3 * (0.2 * r * r - 0.5 * r * sa + sa * sa / 3.0)) * r * r * r;
        };
        h.wrp.push_back(part(sa + SW_W) - part(sa - SW_W));
        h.gamsasa.push_back(p.gamscale[e] * 4.0 * PI * SURFACE_TENSION);
        const double hb = any_hb ? -(p.tmp[e] * p.tmp[e]) * KCALTOAU : 0.0;
        h.hbmag.push_back(hb);
        h.lhb = h.lhb || hb < 0.0;
        maxsa = std::max(maxsa, sa);
    }
    h.srcut = 2.0 * (SW_W + maxsa) + ROFFSET;
    expand_grid(grid_index(spec.nang), h.grid);
    h.npt = (int)h.grid.size() / 4;
    h.lsalt = spec.ion_strength > 0.0;
    if (h.lsalt) {
        h.kappa = 1.0 / (std::sqrt(p.epsv * spec.temperature * KAPPA_CONST / spec.ion_strength) * AATOAU);
        h.ion_rad = spec.ion_rad;
    }
    // SASA neighbour lists: pairs closer than srcut (update_nnlist_gbsa, src/solv/gbsa.f90:933-987)
    const double sr2 = h.srcut * h.srcut;
    h.nb_off.assign(nat + 1, 0);
    std::vector<std::vector<int>> nbl(nat);
    for (int i = 0; i < nat; ++i)
        for (int j = 0; j < i; ++j) {
            const double dx = xyz[3 * i] - xyz[3 * j], dy = xyz[3 * i + 1] - xyz[3 * j + 1],
                         dz = xyz[3 * i + 2] - xyz[3 * j + 2];
            if (dx * dx + dy * dy + dz * dz < sr2) {
                nbl[i].push_back(j);
                nbl[j].push_back(i);
            }
        }
    for (int i = 0; i < nat; ++i) {
        std::sort(nbl[i].begin(), nbl[i].end());
        h.nb_off[i + 1] = h.nb_off[i] + (int)nbl[i].size();
        h.nb.insert(h.nb.end(), nbl[i].begin(), nbl[i].end());
    }
}

// ------------------------------------------------------------------ device part
namespace {

// contribution of atom j's descreening sphere (radius rhoj) to psi of atom i (van der Waals
// radius rvdwi) at distance r, and dg = (dg/dr) / r (compute_psi, src/solv/born.f90)
__device__ __forceinline__ double gb_pair_g(double r, double rhoj, double rvdwi, double& dg) {
    const double ap = r + rhoj, am = r - rhoj;
    if (r >= rvdwi + rhoj) {               // separated spheres
        const double r1 = 1.0 / r;
        const double ab = ap * am;
        const double rhab = rhoj / ab;
        const double lnab = 0.5 * log(am / ap) * r1;
        dg = -2.0 * rhab / ab + (rhab - lnab) * r1 * r1;
        return rhab + lnab;
    }
    if (ap > rvdwi) {                      // j's sphere cuts i's van der Waals sphere
        const double r1 = 1.0 / r, r12 = 0.5 * r1, r24 = r12 * r12;
        const double rh1 = 1.0 / rvdwi, rhr1 = 1.0 / ap, aprh1 = ap * rh1;
        const double lnab = log(aprh1);
        dg = (rhr1 * rhr1 * (1.0 - 0.25 * am * r1 * (1.0 + aprh1 * aprh1)) + rhoj * r24 * (rhr1 - rh1 * aprh1) +
              r12 * (r1 * lnab - rhr1)) * r1;
        return rh1 - rhr1 + r12 * (0.5 * am * (rhr1 - rh1 * aprh1) - lnab);
    }
    dg = 0.0;
    return 0.0;
}

__device__ __forceinline__ double dist3(const double* __restrict__ xyz, int i, int j, double& dx, double& dy,
                                        double& dz) {
    dx = xyz[3 * i] - xyz[3 * j];
    dy = xyz[3 * i + 1] - xyz[3 * j + 1];
    dz = xyz[3 * i + 2] - xyz[3 * j + 2];
    return sqrt(dx * dx + dy * dy + dz * dz);
}

// Born radii: one warp per atom sums psi over all partners within LRCUT
__global__ void k_gb_born(SolvDev s, const double* __restrict__ xyz) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= s.nat) return;
    const double rvdwi = s.vdwr[i];
    double psi = 0.0;
    for (int j = lane; j < s.nat; j += 32) {
        if (j == i) continue;
        double dx, dy, dz;
        const double r = dist3(xyz, i, j, dx, dy, dz);
        if (r >= LRCUT) continue;
        double dg;
        psi += gb_pair_g(r, s.rho[j], rvdwi, dg);
    }
    psi = warp_sum(psi);
    if (lane == 0) {
        const double sv = s.svdw[i], s2 = 0.5 * sv;
        const double br = psi * s2;
        const double arg2 = br * (OBC_G * br - OBC_B);
        const double arg = br * (OBC_A + arg2);
        const double darg = 2.0 * arg2 + OBC_A + OBC_G * br * br;
        const double th = tanh(arg), ch = cosh(arg);
        const double den = 1.0 / sv - th / rvdwi;
        s.brad[i] = s.c1 / den;
        const double t = ch * den;
        s.dbrad[i] = s.c1 * s2 / rvdwi * darg / (t * t);
    }
}

// switching function of one neighbour (radius sa) at squared distance tj2 from a surface point:
// 0 buried, 1 outside the switching shell, 2 inside it with value f and log-derivative factor
// g = f' / (f |t|) (compute_w_sp, src/solv/sasa.f90)
__device__ __forceinline__ int gb_switch(double tj2, double sa, double& f, double& g) {
    const double lo = (sa - SW_W) * (sa - SW_W), hi = (sa + SW_W) * (sa + SW_W);
    if (!(tj2 < hi)) return 1;
    if (tj2 <= lo) return 0;
    const double sq = sqrt(tj2);
    const double u = sq - sa;
    const double a3u2 = AH3 * u * u;
    f = fmin(fmax(AH0 + (AH1 + a3u2) * u, 0.0), 1.0);
    g = (AH1 + 3.0 * a3u2) / (f * sq);
    return 2;
}

// SASA: one block per atom, one thread per surface point (strided); the product of the
// neighbours' switching functions of every point is kept for the gradient
__global__ void k_gb_sasa(SolvDev s, const double* __restrict__ xyz) {
    __shared__ double red[32];
    const int i = blockIdx.x;
    const double xi = xyz[3 * i], yi = xyz[3 * i + 1], zi = xyz[3 * i + 2], sai = s.vdwsa[i], wri = s.wrp[i];
    const int k0 = s.nb_off[i], k1 = s.nb_off[i + 1];
    double acc = 0.0;
    for (int p = threadIdx.x; p < s.npt; p += blockDim.x) {
        const double px = xi + sai * s.grid[4 * p], py = yi + sai * s.grid[4 * p + 1], pz = zi + sai * s.grid[4 * p + 2];
        double prod = 1.0;
        for (int k = k0; k < k1; ++k) {
            const int j = s.nb[k];
            const double tx = px - xyz[3 * j], ty = py - xyz[3 * j + 1], tz = pz - xyz[3 * j + 2];
            double f, g;
            const int c = gb_switch(tx * tx + ty * ty + tz * tz, s.vdwsa[j], f, g);
            if (c == 0 || (c == 2 && f < 2.2250738585072014e-308)) {
                prod = 0.0;
                break;
            }
            if (c == 2) prod *= f;
        }
        s.sasap[(size_t)i * s.npt + p] = prod;
        if (prod > TOLSESP) acc += s.grid[4 * p + 3] * wri * prod;
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) {
        s.sasa[i] = acc;
        if (s.lhb) s.hbw[i] = s.hbmag[i] * acc / (sai * sai);
    }
}

// inertia-like tensor of the van der Waals spheres and the ALPB shape descriptor aDet
// (getADet, src/solv/gbsa.f90:661-705); aux: [0] aDet, [1..9] tensor, [10..12] centre, [13] sum r^3
__global__ void k_gb_adet(SolvDev s, const double* __restrict__ xyz) {
    __shared__ double red[32];
    double t = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
    for (int a = threadIdx.x; a < s.nat; a += blockDim.x) {
        const double r3 = s.vdwr[a] * s.vdwr[a] * s.vdwr[a];
        t += r3;
        cx += xyz[3 * a] * r3;
        cy += xyz[3 * a + 1] * r3;
        cz += xyz[3 * a + 2] * r3;
    }
    t = block_sum(t, red);
    cx = block_sum(cx, red) / t;
    cy = block_sum(cy, red) / t;
    cz = block_sum(cz, red) / t;
    double I[6] = {0, 0, 0, 0, 0, 0};   // xx yy zz xy xz yz
    for (int a = threadIdx.x; a < s.nat; a += blockDim.x) {
        const double r2 = s.vdwr[a] * s.vdwr[a], r3 = r2 * s.vdwr[a];
        const double vx = xyz[3 * a] - cx, vy = xyz[3 * a + 1] - cy, vz = xyz[3 * a + 2] - cz;
        const double d = r3 * (vx * vx + vy * vy + vz * vz + 0.4 * r2);
        I[0] += d - r3 * vx * vx;
        I[1] += d - r3 * vy * vy;
        I[2] += d - r3 * vz * vz;
        I[3] -= r3 * vx * vy;
        I[4] -= r3 * vx * vz;
        I[5] -= r3 * vy * vz;
    }
    for (int k = 0; k < 6; ++k) I[k] = block_sum(I[k], red);
    if (threadIdx.x == 0) {
        const double det = I[0] * (I[1] * I[2] - I[5] * I[5]) - I[3] * (I[3] * I[2] - I[5] * I[4]) +
                           I[4] * (I[3] * I[5] - I[1] * I[4]);
        s.aux[0] = sqrt(cbrt(det) / (0.4 * t));
        const double full[9] = {I[0], I[3], I[4], I[3], I[1], I[5], I[4], I[5], I[2]};
        for (int k = 0; k < 9; ++k) s.aux[1 + k] = full[k];
        s.aux[10] = cx;
        s.aux[11] = cy;
        s.aux[12] = cz;
        s.aux[13] = t;
    }
}

// Debye-Hueckel screening factors of the salt kernel (getDebyeHueckel, src/solv/gbsa.f90:781-802)
__global__ void k_gb_salt(SolvDev s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.nat) return;
    const double aa = 0.5 / s.eps, gg = s.kappa * (s.brad[i] + s.ion_rad);
    s.ionscr[i] = aa * exp(gg) / (1.0 + gg);
    s.discr[i] = s.ionscr[i] * s.kappa * gg / (1.0 + gg);
}

// Born matrix, full n x n (addBornMatrix and the kernels of src/solv/kernel.f90)
__global__ void k_gb_bornmat(SolvDev s, const double* __restrict__ xyz) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= s.nat || j >= s.nat) return;
    const double ai = s.brad[i], aj = s.brad[j];
    double v;
    if (i == j) {
        if (s.lsalt)
            v = (exp(-s.kappa * ai) * 2.0 * s.ionscr[i] - 1.0) / ai;
        else
            v = s.keps / ai;
        if (s.lhb) v += 2.0 * s.hbw[i];
    } else {
        double dx, dy, dz;
        const double r = dist3(xyz, i, j, dx, dy, dz), r2 = r * r;
        const double aa = ai * aj;
        if (s.lsalt) {
            const double fgb = sqrt(r2 + aa * exp(-0.25 * r2 / aa));
            v = (exp(-s.kappa * fgb) * (s.ionscr[i] + s.ionscr[j]) - 1.0) / fgb;
        } else if (s.kernel == 0) {
            v = s.keps / sqrt(r2 + aa * exp(-0.25 * r2 / aa));
        } else {
            const double ab = sqrt(aa);
            double arg = ab / (ab + ZETA_P16 / 16.0 * r);
            arg *= arg;
            arg *= arg;
            arg *= arg;
            arg *= arg;
            v = s.keps / (r + ab * arg);
        }
    }
    if (s.alpbet > 0.0) v += s.keps * s.alpbet / s.aux[0];
    s.B[(size_t)i * s.nat + j] = v;
}

// out[i] (+)= sum_j B[i][j] q[j], one warp per row
__global__ void k_gb_bq(int n, const double* __restrict__ B, const double* __restrict__ q, double* __restrict__ out,
                        int accumulate) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= n) return;
    double a = 0.0;
    for (int j = lane; j < n; j += 32) a += B[(size_t)i * n + j] * q[j];
    a = warp_sum(a);
    if (lane == 0) out[i] = accumulate ? out[i] + a : a;
}

// energy from q and bq = B q: esolv = [total, G_hb, G_sasa, G_shift]
__global__ void k_gb_energy(SolvDev s, const double* __restrict__ q) {
    __shared__ double red[32];
    double e = 0.0, ghb = 0.0, gs = 0.0;
    for (int i = threadIdx.x; i < s.nat; i += blockDim.x) {
        e += 0.5 * q[i] * s.bq[i];
        if (s.lhb) ghb += s.hbw[i] * q[i] * q[i];
        gs += s.sasa[i] * s.gamsasa[i];
    }
    e = block_sum(e, red);
    ghb = block_sum(ghb, red);
    gs = block_sum(gs, red);
    if (threadIdx.x == 0) {
        s.esolv[0] = e + gs + s.gshift;
        s.esolv[1] = ghb;
        s.esolv[2] = gs;
        s.esolv[3] = s.gshift;
    }
}

// pair part of the Born-energy gradient and dE/d(Born radius) of every atom; one warp per atom
// over all partners (addGradientStill / addGradientP16 / addGradientSaltStill)
__global__ void k_gb_grad_pairs(SolvDev s, const double* __restrict__ xyz, const double* __restrict__ q,
                                double* __restrict__ grad) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= s.nat) return;
    const double ai = s.brad[i], qi = q[i];
    double gx = 0.0, gy = 0.0, gz = 0.0, gb = 0.0;
    for (int j = lane; j < s.nat; j += 32) {
        if (j == i) continue;
        double dx, dy, dz;
        const double r = dist3(xyz, i, j, dx, dy, dz), r2 = r * r;
        const double aj = s.brad[j], qq = qi * q[j], aa = ai * aj;
        double ap, bterm;
        if (s.lsalt) {
            const double dd = 0.25 * r2 / aa, expd = exp(-dd);
            const double fgb2 = r2 + aa * expd, fgb = sqrt(fgb2);
            const double ka = s.kappa * fgb, expa = exp(-ka);
            const double gg = (s.ionscr[i] + s.ionscr[j]) * expa;
            const double qfg = qq / fgb;
            const double dfgb3 = qfg * (gg * (1.0 + ka) - 1.0) / fgb2;
            ap = (1.0 - 0.25 * expd) * dfgb3;
            bterm = aj * (-0.5 * expd * (1.0 + dd) * dfgb3) + qfg * expa * s.discr[i];
        } else if (s.kernel == 0) {
            const double dd = 0.25 * r2 / aa, expd = exp(-dd);
            const double dfgb = 1.0 / sqrt(r2 + aa * expd);
            const double dfgb3 = dfgb * dfgb * dfgb * s.keps;
            ap = (1.0 - 0.25 * expd) * dfgb3 * qq;
            bterm = aj * (-0.5 * expd * (1.0 + dd) * dfgb3) * qq;
        } else {
            const double ab = sqrt(aa);
            const double arg1 = ab / (ab + ZETA_P16 / 16.0 * r);
            double a16 = arg1 * arg1;
            a16 *= a16;
            a16 *= a16;
            a16 *= a16;
            const double dfgb = 1.0 / (r + ab * a16), dfgb2 = dfgb * dfgb;
            ap = (1.0 - ZETA_P16 * arg1 * a16) * dfgb2 * s.keps / r * qq;
            bterm = aj * (-0.5 * (r * ZETA_P16 / ab * arg1 + 1.0) / ab * a16 * dfgb2) * s.keps * qq;
        }
        gx -= ap * dx;
        gy -= ap * dy;
        gz -= ap * dz;
        gb += bterm;
    }
    gx = warp_sum(gx);
    gy = warp_sum(gy);
    gz = warp_sum(gz);
    gb = warp_sum(gb);
    if (lane == 0) {
        if (s.lsalt) {
            const double ga = exp(-s.kappa * ai), sa = 2.0 * s.ionscr[i] * ga - 1.0;
            const double apd = sa - ai * 2.0 * (s.discr[i] + s.ionscr[i] * s.kappa) * ga;
            gb += -0.5 * (qi / ai) * (qi / ai) * apd;
        } else {
            gb += -0.5 * s.keps * qi * qi / (ai * ai);
        }
        s.grddb[i] = gb;
        grad[3 * i] += gx;
        grad[3 * i + 1] += gy;
        grad[3 * i + 2] += gz;
        // weight of the surface gradient: surface tension plus the H-bond term at these charges
        s.wsur[i] = s.gamsasa[i] + (s.lhb ? s.hbmag[i] / (s.vdwsa[i] * s.vdwsa[i]) * qi * qi : 0.0);
    }
}

// Born-radius chain rule: grad_k += sum_j (x_k - x_j) (w_k dg_k(j) + w_j dg_j(k)),
// w = dE/d(brad) * d(brad)/d(psi); one warp per atom
__global__ void k_gb_grad_born(SolvDev s, const double* __restrict__ xyz, double* __restrict__ grad) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (k >= s.nat) return;
    const double wk = s.grddb[k] * s.dbrad[k], rvk = s.vdwr[k], rhok = s.rho[k];
    double gx = 0.0, gy = 0.0, gz = 0.0;
    for (int j = lane; j < s.nat; j += 32) {
        if (j == k) continue;
        double dx, dy, dz;
        const double r = dist3(xyz, k, j, dx, dy, dz);
        if (r >= LRCUT) continue;
        double dkj, djk;
        gb_pair_g(r, s.rho[j], rvk, dkj);
        gb_pair_g(r, rhok, s.vdwr[j], djk);
        const double c = wk * dkj + s.grddb[j] * s.dbrad[j] * djk;
        gx += c * dx;
        gy += c * dy;
        gz += c * dz;
    }
    gx = warp_sum(gx);
    gy = warp_sum(gy);
    gz = warp_sum(gz);
    if (lane == 0) {
        grad[3 * k] += gx;
        grad[3 * k + 1] += gy;
        grad[3 * k + 2] += gz;
    }
}

// surface gradient: grad_k += sum_i wsur_i d sasa_i / d x_k, one block per atom k.  The own
// surface moves with k against every neighbour in its switching shell; each neighbour i's
// surface moves against k where k's switching shell covers i's points.
__global__ void k_gb_grad_sasa(SolvDev s, const double* __restrict__ xyz, double* __restrict__ grad) {
    __shared__ double red[32];
    const int k = blockIdx.x;
    const double xk = xyz[3 * k], yk = xyz[3 * k + 1], zk = xyz[3 * k + 2], sak = s.vdwsa[k];
    const int k0 = s.nb_off[k], k1 = s.nb_off[k + 1];
    double ax = 0.0, ay = 0.0, az = 0.0;
    // own points
    for (int p = threadIdx.x; p < s.npt; p += blockDim.x) {
        const double sp = s.sasap[(size_t)k * s.npt + p];
        if (!(sp > TOLSESP)) continue;
        const double wsa = s.grid[4 * p + 3] * s.wrp[k] * sp * s.wsur[k];
        const double px = xk + sak * s.grid[4 * p], py = yk + sak * s.grid[4 * p + 1], pz = zk + sak * s.grid[4 * p + 2];
        for (int kk = k0; kk < k1; ++kk) {
            const int j = s.nb[kk];
            const double tx = px - xyz[3 * j], ty = py - xyz[3 * j + 1], tz = pz - xyz[3 * j + 2];
            double f, g;
            if (gb_switch(tx * tx + ty * ty + tz * tz, s.vdwsa[j], f, g) != 2) continue;
            ax += wsa * g * tx;
            ay += wsa * g * ty;
            az += wsa * g * tz;
        }
    }
    // the neighbours' points
    for (int kk = k0; kk < k1; ++kk) {
        const int i = s.nb[kk];
        const double xi = xyz[3 * i], yi = xyz[3 * i + 1], zi = xyz[3 * i + 2], sai = s.vdwsa[i];
        const double wi = s.wrp[i] * s.wsur[i];
        for (int p = threadIdx.x; p < s.npt; p += blockDim.x) {
            const double sp = s.sasap[(size_t)i * s.npt + p];
            if (!(sp > TOLSESP)) continue;
            const double px = xi + sai * s.grid[4 * p], py = yi + sai * s.grid[4 * p + 1],
                         pz = zi + sai * s.grid[4 * p + 2];
            const double tx = px - xk, ty = py - yk, tz = pz - zk;
            double f, g;
            if (gb_switch(tx * tx + ty * ty + tz * tz, sak, f, g) != 2) continue;
            const double c = s.grid[4 * p + 3] * wi * sp * g;
            ax -= c * tx;
            ay -= c * ty;
            az -= c * tz;
        }
    }
    ax = block_sum(ax, red);
    ay = block_sum(ay, red);
    az = block_sum(az, red);
    if (threadIdx.x == 0) {
        grad[3 * k] += ax;
        grad[3 * k + 1] += ay;
        grad[3 * k + 2] += az;
    }
}

// ALPB shape-term gradient (addADetDeriv, src/solv/gbsa.f90:708-777); zero for neutral molecules
__global__ void k_gb_grad_adet(SolvDev s, const double* __restrict__ xyz, const double* __restrict__ q,
                               double* __restrict__ grad) {
    __shared__ double red[32];
    double qt = 0.0;
    for (int a = threadIdx.x; a < s.nat; a += blockDim.x) qt += q[a];
    qt = block_sum(qt, red);
    const double* I = s.aux + 1;   // row-major 3 x 3
    const double adet = s.aux[0], tot = s.aux[13];
    const double M[9] = {I[0] * (I[4] + I[8]) - I[1] * I[1] - I[2] * I[2], I[1] * I[8] - I[2] * I[5],
                         I[2] * I[4] - I[1] * I[7],
                         I[1] * I[8] - I[2] * I[5], I[4] * (I[0] + I[8]) - I[1] * I[1] - I[5] * I[5],
                         I[0] * I[5] - I[1] * I[2],
                         I[2] * I[4] - I[1] * I[7], I[0] * I[5] - I[1] * I[2],
                         I[8] * (I[0] + I[4]) - I[2] * I[2] - I[5] * I[5]};
    const double a2 = adet * adet;
    const double fac = (250.0 / (48.0 * tot * tot * tot * a2 * a2 * adet)) * (-0.5 * s.keps * s.alpbet * qt * qt / a2);
    for (int a = threadIdx.x; a < s.nat; a += blockDim.x) {
        const double r3 = s.vdwr[a] * s.vdwr[a] * s.vdwr[a];
        const double v[3] = {xyz[3 * a] - s.aux[10], xyz[3 * a + 1] - s.aux[11], xyz[3 * a + 2] - s.aux[12]};
        for (int c = 0; c < 3; ++c)
            grad[3 * a + c] += r3 * fac * (M[3 * c] * v[0] + M[3 * c + 1] * v[1] + M[3 * c + 2] * v[2]);
    }
}

}  // namespace

void solv_update(cudaStream_t st, const SolvDev& s, const double* xyz) {
    k_gb_born<<<ceil_div((long)s.nat * 32, 128), 128, 0, st>>>(s, xyz);
    XG_LAUNCH_CHECK();
    k_gb_sasa<<<s.nat, 256, 0, st>>>(s, xyz);
    XG_LAUNCH_CHECK();
    if (s.lsalt) {
        k_gb_salt<<<ceil_div(s.nat, 128), 128, 0, st>>>(s);
        XG_LAUNCH_CHECK();
    }
    if (s.alpbet > 0.0) {
        k_gb_adet<<<1, 256, 0, st>>>(s, xyz);
        XG_LAUNCH_CHECK();
    }
    dim3 b(16, 16), g(ceil_div(s.nat, 16), ceil_div(s.nat, 16));
    k_gb_bornmat<<<g, b, 0, st>>>(s, xyz);
    XG_LAUNCH_CHECK();
}

void solv_shift(cudaStream_t st, const SolvDev& s, const double* q, double* vat) {
    k_gb_bq<<<ceil_div((long)s.nat * 32, 128), 128, 0, st>>>(s.nat, s.B, q, vat, 1);
    XG_LAUNCH_CHECK();
}

void solv_energy(cudaStream_t st, const SolvDev& s, const double* q) {
    k_gb_bq<<<ceil_div((long)s.nat * 32, 128), 128, 0, st>>>(s.nat, s.B, q, s.bq, 0);
    XG_LAUNCH_CHECK();
    k_gb_energy<<<1, 512, 0, st>>>(s, q);
    XG_LAUNCH_CHECK();
}

void solv_gradient(cudaStream_t st, const SolvDev& s, const double* xyz, const double* q, double* grad) {
    k_gb_grad_pairs<<<ceil_div((long)s.nat * 32, 128), 128, 0, st>>>(s, xyz, q, grad);
    XG_LAUNCH_CHECK();
    k_gb_grad_born<<<ceil_div((long)s.nat * 32, 128), 128, 0, st>>>(s, xyz, grad);
    XG_LAUNCH_CHECK();
    k_gb_grad_sasa<<<s.nat, 256, 0, st>>>(s, xyz, grad);
    XG_LAUNCH_CHECK();
    if (s.alpbet > 0.0) {
        k_gb_grad_adet<<<1, 256, 0, st>>>(s, xyz, q, grad);
        XG_LAUNCH_CHECK();
    }
}

}  // namespace xg
