// Plain per-molecule FP64 GFN2-xTB single point: host orchestration of the device kernels.
//
// Follows scf (src/scf_module.F90:74-920) and scc (src/scc_core.f90:255-640):
// set-up (CN, EEQ guess, integrals, Coulomb/AES/D4 kernels) -> SCC iterations
// (potentials, H, generalised eigenproblem, Fermi smearing, density, Mulliken,
// energies, Broyden) -> analytic gradient.  All O(N^2) and O(N^3) work runs on
// the device; per iteration the host reads back four scalars for the
// convergence test.
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "engine.h"
#include "gfn2_kernels.h"
#include "linalg.h"
#include "splitgemm.h"

namespace xg {

long long& launch_counter() {
    thread_local long long n = 0;
    return n;
}

const char* const kPhaseNames[PH_COUNT] = {"setup", "integrals", "cholesky", "hbuild", "stdform", "sytrd",
                                           "trieig", "backtransform", "density", "popmix", "gradient", "total"};

int device_count() {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

namespace {

// --------------------------------------------------------------- small kernels
__global__ void k_self_energy(int nsh, const int* __restrict__ sh_atom, const double* __restrict__ se0,
                              const double* __restrict__ kcn, const double* __restrict__ cn, double* __restrict__ se) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nsh) se[s] = se0[s] - kcn[s] * cn[sh_atom[s]];
}

__global__ void k_ini_qsh(int nsh, const int* __restrict__ sh_atom, const double* __restrict__ zsh,
                          const double* __restrict__ zval, const double* __restrict__ q, double* __restrict__ qsh) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nsh) qsh[s] = zsh[s] / zval[sh_atom[s]] * q[sh_atom[s]];
}

__global__ void k_scale_energy_weights(int n, const double* __restrict__ focc, const double* __restrict__ emo,
                                       double* __restrict__ fe) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) fe[i] = focc[i] * emo[i] * EVTOAU;
}

// ---- external point charges (GFN2 forms of src/embedding.f90)
// shell potential of the charges, jpot_pcem_gfn2 (:225-256): V_s = sum_k q_k / sqrt(r^2 + 1/x^2),
// x = (eta_s + gam_k) / 2; one warp per shell
__global__ void k_pc_potential(DevMol m, int npc, const double* __restrict__ pcq, const double* __restrict__ pcx,
                               const double* __restrict__ pcg, double* __restrict__ vpc) {
    const int s = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (s >= m.nsh) return;
    const int a = m.sh_atom[s];
    const double eta = m.sh_eta[s];
    double acc = 0.0;
    for (int k = lane; k < npc; k += 32) {
        const double dx = pcx[3 * k] - m.xyz[3 * a], dy = pcx[3 * k + 1] - m.xyz[3 * a + 1],
                     dz = pcx[3 * k + 2] - m.xyz[3 * a + 2];
        const double x = 0.5 * (eta + pcg[k]);
        acc += pcq[k] / sqrt(dx * dx + dy * dy + dz * dz + 1.0 / (x * x));
    }
    acc = warp_sum(acc);
    if (lane == 0) vpc[s] = acc;
}

__global__ void k_add_vec(int n, const double* __restrict__ a, double* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] += a[i];
}

// gradient of sum_s qsh_s V_s, pcem_grad_gfn2 (:329-365): with dr = R_atom - R_k and
// y = qsh_s q_k (r^2 + 1/x^2)^(-3/2), the atom gains -dr y and the charge +dr y.  One warp per
// atom (its shells against all charges) and one warp per charge (against all shells): no atomics.
__global__ void k_pc_grad_atoms(DevMol m, int npc, const double* __restrict__ pcq, const double* __restrict__ pcx,
                                const double* __restrict__ pcg, const double* __restrict__ qsh,
                                double* __restrict__ grad) {
    const int a = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (a >= m.nat) return;
    double g[3] = {0.0, 0.0, 0.0};
    for (int s = m.at_sh0[a]; s < m.at_sh0[a] + m.at_nsh[a]; ++s)
        for (int k = lane; k < npc; k += 32) {
            const double dr[3] = {m.xyz[3 * a] - pcx[3 * k], m.xyz[3 * a + 1] - pcx[3 * k + 1],
                                  m.xyz[3 * a + 2] - pcx[3 * k + 2]};
            const double x = 0.5 * (m.sh_eta[s] + pcg[k]);
            const double t = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2] + 1.0 / (x * x);
            const double y = qsh[s] * pcq[k] / (t * sqrt(t));
            for (int c = 0; c < 3; ++c) g[c] -= dr[c] * y;
        }
    for (int c = 0; c < 3; ++c) {
        const double v = warp_sum(g[c]);
        if (lane == 0) grad[3 * a + c] += v;
    }
}

__global__ void k_pc_grad_charges(DevMol m, int npc, const double* __restrict__ pcq, const double* __restrict__ pcx,
                                  const double* __restrict__ pcg, const double* __restrict__ qsh,
                                  double* __restrict__ gpc) {
    const int k = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (k >= npc) return;
    double g[3] = {0.0, 0.0, 0.0};
    for (int s = lane; s < m.nsh; s += 32) {
        const int a = m.sh_atom[s];
        const double dr[3] = {m.xyz[3 * a] - pcx[3 * k], m.xyz[3 * a + 1] - pcx[3 * k + 1],
                              m.xyz[3 * a + 2] - pcx[3 * k + 2]};
        const double x = 0.5 * (m.sh_eta[s] + pcg[k]);
        const double t = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2] + 1.0 / (x * x);
        const double y = qsh[s] * pcq[k] / (t * sqrt(t));
        for (int c = 0; c < 3; ++c) g[c] += dr[c] * y;
    }
    for (int c = 0; c < 3; ++c) {
        const double v = warp_sum(g[c]);
        if (lane == 0) gpc[3 * k + c] = v;
    }
}

// SCC energy from the current populations (electro + aniso_electro + edisp_scc + entropy;
// src/scc_core.f90:686-722, src/aespot.F90:566-664, src/disp/dftd4.F90:821-864), and the shells'
// energy in the field of external charges (electro_pcem, src/embedding.f90:261-280; vpc may be null)
// and the implicit solvent's energy (esolv[0] from solv_energy; null without a solvent)
// out: [0] eel, [1] es, [2] eaes, [3] epol, [4] ed, [5] entropy term, [6] external charges, [7] solvent
__global__ void k_scc_energy(int nsh, int nat, const double* __restrict__ qsh, const double* __restrict__ Jq,
                             const double* __restrict__ gam3, const double* __restrict__ eh0,
                             const double* __restrict__ eaes, const double* __restrict__ ed4,
                             const double* __restrict__ fermi_scal, const double* __restrict__ vpc,
                             const double* __restrict__ esolv, double* __restrict__ out) {
    __shared__ double red[32];
    double es = 0.0, h = 0.0, ea = 0.0, ep = 0.0, ed = 0.0, epc = 0.0;
    for (int s = threadIdx.x; s < nsh; s += blockDim.x) {
        es += 0.5 * qsh[s] * Jq[s] + gam3[s] * qsh[s] * qsh[s] * qsh[s] / 3.0;
        if (vpc) epc += qsh[s] * vpc[s];
    }
    for (int a = threadIdx.x; a < nat; a += blockDim.x) {
        h += eh0[a];
        ea += eaes[a];
        ep += eaes[nat + a];
        ed += ed4[a];
    }
    es = block_sum(es, red);
    h = block_sum(h, red);
    ea = block_sum(ea, red);
    ep = block_sum(ep, red);
    ed = block_sum(ed, red);
    epc = block_sum(epc, red);
    if (threadIdx.x == 0) {
        const double ts = fermi_scal[0];
        const double gsolv = esolv ? esolv[0] : 0.0;
        out[0] = es + h * EVTOAU + ea + ep + ed + epc + gsolv + ts;
        out[7] = gsolv;
        out[1] = es;
        out[2] = ea;
        out[3] = ep;
        out[4] = ed;
        out[5] = ts;
        out[6] = epc;
    }
}

// dipole moment (calc_dipole, src/dipole.f90:94-128) from the population row sums
__global__ void k_dipole(int nat, int nao, const double* __restrict__ xyz, const double* __restrict__ zval,
                         const double* __restrict__ rows, double* __restrict__ out) {
    __shared__ double red[32];
    for (int k = 0; k < 3; ++k) {
        double s = 0.0;
        for (int a = threadIdx.x; a < nat; a += blockDim.x) s += xyz[3 * a + k] * zval[a];
        for (int mu = threadIdx.x; mu < nao; mu += blockDim.x) s -= rows[(size_t)mu * 12 + 1 + k];
        s = block_sum(s, red);
        if (threadIdx.x == 0) out[k] = s;
    }
}

// Wiberg-Mayer bond orders from PS (get_wiberg, src/scc_core.f90:1208-1245); one warp per atom pair
// closed shell: PS = P S, factor 1; open shell (get_unrestricted_wiberg, :1248-1295): PS = Pa S, PS2 = Pb S, factor 2
__global__ void k_wiberg(int nat, int nao, const double* __restrict__ xyz, const int* __restrict__ ao0,
                         const int* __restrict__ nao_at, const double* __restrict__ PS, const double* __restrict__ PS2,
                         double factor, double* __restrict__ wbo) {
    const long w = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (long)nat * nat) return;
    const int i = (int)(w / nat), j = (int)(w % nat);
    double s = 0.0;
    if (i != j) {
        const double r2 = (xyz[3 * i] - xyz[3 * j]) * (xyz[3 * i] - xyz[3 * j]) +
                          (xyz[3 * i + 1] - xyz[3 * j + 1]) * (xyz[3 * i + 1] - xyz[3 * j + 1]) +
                          (xyz[3 * i + 2] - xyz[3 * j + 2]) * (xyz[3 * i + 2] - xyz[3 * j + 2]);
        if (r2 < 100.0) {
            const int ni = nao_at[i], nj = nao_at[j];
            for (int t = lane; t < ni * nj; t += 32) {
                const int k = ao0[i] + t / nj, mm = ao0[j] + t % nj;
                s += PS[(size_t)k * nao + mm] * PS[(size_t)mm * nao + k];
                if (PS2) s += PS2[(size_t)k * nao + mm] * PS2[(size_t)mm * nao + k];
            }
        }
    }
    s = warp_sum(s);
    if (lane == 0) wbo[w] = factor * s;
}

// --------------------------------------------------------------- device workspace
struct Arena {
    char* base = nullptr;
    size_t cap = 0, used = 0;
    bool counting = false;
    // Stream-ordered (re)allocation on the engine stream: no device-wide synchronisation, so
    // single points on other threads' streams keep running while this one grows its workspace.
    void reset(size_t need, cudaStream_t st) {
        counting = false;
        need += 4096;
        if (need > cap) {
            if (base) XG_CUDA(cudaFreeAsync(base, st));
            base = nullptr;
            cap = 0;
            XG_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&base), need, st));
            cap = need;
        }
        used = 0;
    }
    template <typename T>
    T* take(size_t count) {
        const size_t bytes = ((count * sizeof(T) + 255) / 256) * 256;
        if (counting) {
            used += bytes;
            return nullptr;
        }
        if (used + bytes > cap) throw CudaError("workspace overflow");
        T* p = reinterpret_cast<T*>(base + used);
        used += bytes;
        return p;
    }
};

struct Sizer {
    size_t bytes = 0;
    template <typename T>
    void add(size_t count) { bytes += ((count * sizeof(T) + 255) / 256) * 256; }
};

thread_local Arena g_arena;
// engine streams of this thread, one per stream priority (slot = least priority - priority)
constexpr int kPrioritySlots = 16;
thread_local cudaStream_t g_streams[kPrioritySlots] = {};

cudaStream_t engine_stream(int priority) {
    int least = 0, greatest = 0;
    XG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    const int p = std::max(greatest, std::min(least, priority));
    const int slot = std::min(kPrioritySlots - 1, least - p);
    if (!g_streams[slot]) XG_CUDA(cudaStreamCreateWithPriority(&g_streams[slot], cudaStreamNonBlocking, p));
    return g_streams[slot];
}

// CUDA-event phase timer on the engine stream; elapsed times are read after the final sync.
struct PhaseTimer {
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<int, std::pair<int, int>>> spans;   // phase, (start event, stop event)
    size_t next = 0;
    cudaStream_t st = nullptr;
    int open_phase = -1, open_ev = -1;
    cudaEvent_t get() {
        if (next == pool.size()) {
            cudaEvent_t e;
            XG_CUDA(cudaEventCreate(&e));
            pool.push_back(e);
        }
        return pool[next++];
    }
    void begin(cudaStream_t s) { st = s; next = 0; spans.clear(); open_phase = -1; }
    void start(int ph) {
        const int idx = (int)next;
        XG_CUDA(cudaEventRecord(get(), st));
        open_phase = ph;
        open_ev = idx;
    }
    void stop() {
        const int idx = (int)next;
        XG_CUDA(cudaEventRecord(get(), st));
        spans.push_back({open_phase, {open_ev, idx}});
    }
    void mark(int ph) {   // stop the open phase and start the next one
        if (open_phase >= 0) stop();
        start(ph);
    }
    std::vector<double> collect() {
        std::vector<double> ms(PH_COUNT, 0.0);
        for (auto& sp : spans) {
            float t = 0.0f;
            XG_CUDA(cudaEventElapsedTime(&t, pool[sp.second.first], pool[sp.second.second]));
            ms[sp.first] += t;
        }
        return ms;
    }
};
thread_local PhaseTimer g_timer;

thread_local long long g_h2d = 0;

template <typename T>
T* upload(Arena& ar, cudaStream_t st, const std::vector<T>& v) {
    T* d = ar.take<T>(std::max<size_t>(v.size(), 1));
    if (!ar.counting && !v.empty()) {
        XG_CUDA(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        g_h2d += (long long)(v.size() * sizeof(T));
    }
    return d;
}

}  // namespace

void run_singlepoint(const HostMol& hm, const SPSettings& set, Wavefunction& wfn, SPResult& res, bool keep_orbitals,
                     bool& scc_failed, bool guess_only) {
    if (device_count() == 0) throw CudaError("no CUDA device available for the GFN2 engine");
    // every earlier single point of this thread has been synchronised, so the workspace may
    // move to a stream of another priority
    cudaStream_t st = engine_stream(set.stream_priority);
    const int nat = hm.nat, nsh = hm.nsh, nao = hm.nao, ne = hm.nelem;
    const size_t nn = (size_t)nao * nao;
    const size_t aa = (size_t)nat * nat;
    const int maxit = std::max(1, set.maxiter);
    const int nbr = nsh + 9 * nat;
    const bool split = set.precision == 1;
    if (split && (set.slices < 4 || set.slices > 7)) throw CudaError("split precision needs 4..7 slices");

    // ---- thresholds (src/scf_module.F90:266-277)
    const double acc = set.accuracy;
    Thresholds th;
    th.intcut = std::max(20.0, 25.0 - 10.0 * std::log10(acc));
    th.neglect = 10.0e-9 * acc;
    const double scfconv = 1.0e-6 * acc;
    const double qconv = 1.0e-4 * acc;

    g_h2d = 0;
    long long d2h = 0;
    const long long launches0 = launch_counter();
    PhaseTimer& tm = g_timer;
    tm.begin(st);
    const int total_ev = (int)tm.next;
    XG_CUDA(cudaEventRecord(tm.get(), st));
    tm.start(PH_SETUP);
    // ---- workspace: exact two-pass layout (count, allocate, carve)
    Arena& ar = g_arena;
    DevMol m;
    const double* d_zval = nullptr;
    double *S, *D, *Q, *H0, *X, *H, *A, *T1, *C, *Pm, *Wm, *V, *Y, *iscr, *J, *gab3, *gab5, *c6, *dc6, *c6z,
        *dc6z, *eeqA, *eeqX, *cn_gfn, *cn_tmp, *se, *q, *qsh, *dipm, *qp, *shift, *Jq, *vs, *vd, *vq, *radcn, *gw, *dgw,
        *zeta, *dzeta, *Wz, *zv, *zr, *zdcn, *zrdcn, *vat, *ed4, *eh0, *eaes, *erep, *e2, *e3, *grad, *dhdcn, *tmp2,
        *rows, *emo, *focc, *focca, *foccb, *fe, *tri_d, *tri_e, *tri_e2, *tri_tau, *tri_p, *bounds, *fscal, *escal, *rms, *dip, *qin,
        *qout, *dq;
    double *pcq = nullptr, *pcx = nullptr, *pcg = nullptr, *vpc = nullptr, *pcgrad = nullptr;
    const int npc = (int)set.pc_q.size();
    // implicit solvent: host model of this molecule, device state carved below
    const bool solv = set.solv.on;
    SolvHost sh;
    SolvDev sd;
    if (solv) build_solv_host(set.solv, nat, hm.Z.data(), hm.xyz.data(), sh);
    double* ormw;
    char* sgw = nullptr;
    unsigned char* piv;
    int* info;
    BroydenState bs;
    auto layout = [&]() {
    // ---- upload molecule
    m.nat = nat; m.nsh = nsh; m.nao = nao; m.nelem = ne;
    m.Z = upload(ar, st, hm.Z);
    m.eid = upload(ar, st, hm.eid);
    m.xyz = upload(ar, st, hm.xyz);
    m.at_sh0 = upload(ar, st, hm.at_sh0);
    m.at_nsh = upload(ar, st, hm.at_nsh);
    m.at_ao0 = upload(ar, st, hm.at_ao0);
    m.at_nao = upload(ar, st, hm.at_nao);
    m.rcov = upload(ar, st, hm.rcov);
    m.en = upload(ar, st, hm.en);
    m.rcov4 = upload(ar, st, hm.rcov4);
    m.en4 = upload(ar, st, hm.en4);
    m.eeq_en = upload(ar, st, hm.eeq_en);
    m.eeq_gam = upload(ar, st, hm.eeq_gam);
    m.eeq_kappa = upload(ar, st, hm.eeq_kappa);
    m.eeq_alpha = upload(ar, st, hm.eeq_alpha);
    m.mrad = upload(ar, st, hm.mrad);
    m.valcn = upload(ar, st, hm.valcn);
    m.dkern = upload(ar, st, hm.dkern);
    m.qkern = upload(ar, st, hm.qkern);
    m.rep_alpha = upload(ar, st, hm.rep_alpha);
    m.rep_zeff = upload(ar, st, hm.rep_zeff);
    m.r4r2 = upload(ar, st, hm.r4r2);
    m.arad = upload(ar, st, hm.arad);
    m.d4_nref = upload(ar, st, hm.d4_nref);
    m.d4_zeff = upload(ar, st, hm.d4_zeff);
    m.d4_gam = upload(ar, st, hm.d4_gam);
    m.d4_refq = upload(ar, st, hm.d4_refq);
    m.d4_refcn = upload(ar, st, hm.d4_refcn);
    m.d4_ncount = upload(ar, st, hm.d4_ncount);
    m.d4_c6 = upload(ar, st, hm.d4_c6);
    m.sh_atom = upload(ar, st, hm.sh_atom);
    m.sh_l = upload(ar, st, hm.sh_l);
    m.sh_ao = upload(ar, st, hm.sh_ao);
    m.sh_nprim = upload(ar, st, hm.sh_nprim);
    m.sh_alpha = upload(ar, st, hm.sh_alpha);
    m.sh_coef = upload(ar, st, hm.sh_coef);
    m.sh_zeta = upload(ar, st, hm.sh_zeta);
    m.sh_se0 = upload(ar, st, hm.sh_se0);
    m.sh_kcn = upload(ar, st, hm.sh_kcn);
    m.sh_poly = upload(ar, st, hm.sh_poly);
    m.sh_eta = upload(ar, st, hm.sh_eta);
    m.sh_gam3 = upload(ar, st, hm.sh_gam3);
    m.sh_zsh = upload(ar, st, hm.sh_zsh);
    m.sh_byl = upload(ar, st, hm.sh_byl);
    for (int l = 0; l < 4; ++l) m.l_off[l] = hm.l_off[l];
    m.ao_sh = upload(ar, st, hm.ao_sh);
    m.ao_at = upload(ar, st, hm.ao_at);
    d_zval = upload(ar, st, hm.zval);
    if (npc > 0) {
        pcq = upload(ar, st, set.pc_q);
        pcx = upload(ar, st, set.pc_xyz);
        pcg = upload(ar, st, set.pc_gam);
    }
    if (solv) {
        sd.nat = nat; sd.npt = sh.npt; sd.kernel = sh.kernel;
        sd.alpb = sh.alpb; sd.lhb = sh.lhb; sd.lsalt = sh.lsalt;
        sd.keps = sh.keps; sd.alpbet = sh.alpbet; sd.c1 = sh.c1; sd.gshift = sh.gshift; sd.eps = sh.eps;
        sd.kappa = sh.kappa; sd.ion_rad = sh.ion_rad;
        sd.vdwr = upload(ar, st, sh.vdwr);
        sd.rho = upload(ar, st, sh.rho);
        sd.svdw = upload(ar, st, sh.svdw);
        sd.vdwsa = upload(ar, st, sh.vdwsa);
        sd.wrp = upload(ar, st, sh.wrp);
        sd.gamsasa = upload(ar, st, sh.gamsasa);
        sd.hbmag = upload(ar, st, sh.hbmag);
        sd.grid = upload(ar, st, sh.grid);
        sd.nb_off = upload(ar, st, sh.nb_off);
        sd.nb = upload(ar, st, sh.nb);
        sd.brad = ar.take<double>(nat);
        sd.dbrad = ar.take<double>(nat);
        sd.sasa = ar.take<double>(nat);
        sd.hbw = ar.take<double>(nat);
        sd.ionscr = ar.take<double>(nat);
        sd.discr = ar.take<double>(nat);
        sd.bq = ar.take<double>(nat);
        sd.grddb = ar.take<double>(nat);
        sd.wsur = ar.take<double>(nat);
        sd.sasap = ar.take<double>((size_t)nat * sh.npt);
        sd.B = ar.take<double>(aa);
        sd.aux = ar.take<double>(16);
        sd.esolv = ar.take<double>(8);
    }

    // ---- device buffers
    S = ar.take<double>(nn);
    D = ar.take<double>(3 * nn);
    Q = ar.take<double>(6 * nn);
    H0 = ar.take<double>(nn);
    X = ar.take<double>(nn);
    H = ar.take<double>(nn);
    A = ar.take<double>(nn);
    T1 = ar.take<double>(nn);
    C = ar.take<double>(nn);
    Pm = ar.take<double>(nn);
    Wm = ar.take<double>(nn);
    V = ar.take<double>(nn);
    Y = ar.take<double>(nn);
    iscr = ar.take<double>(4 * nn);
    ormw = ar.take<double>(ormtr_workspace(nao));
    if (set.precision == 1) sgw = ar.take<char>(split_gemm_workspace(nao, nao, nao, set.slices));
    piv = ar.take<unsigned char>(nn);
    J = ar.take<double>((size_t)nsh * nsh);
    gab3 = ar.take<double>(aa);
    gab5 = ar.take<double>(aa);
    c6 = ar.take<double>(aa);
    dc6 = ar.take<double>(aa);
    c6z = ar.take<double>(aa);
    dc6z = ar.take<double>(aa);
    eeqA = ar.take<double>(std::max(aa, (size_t)1));
    eeqX = ar.take<double>(2 * (size_t)nat);
    cn_gfn = ar.take<double>(nat);
    cn_tmp = ar.take<double>(nat);
    se = ar.take<double>(nsh);
    q = ar.take<double>(nat);
    qsh = ar.take<double>(nsh);
    dipm = ar.take<double>(3 * (size_t)nat);
    qp = ar.take<double>(6 * (size_t)nat);
    shift = ar.take<double>(nsh);
    Jq = ar.take<double>(nsh);
    vs = ar.take<double>(nat);
    vd = ar.take<double>(3 * (size_t)nat);
    vq = ar.take<double>(6 * (size_t)nat);
    radcn = ar.take<double>(nat);
    gw = ar.take<double>((size_t)nat * MAXREF);
    dgw = ar.take<double>((size_t)nat * MAXREF);
    zeta = ar.take<double>((size_t)nat * MAXREF);
    dzeta = ar.take<double>((size_t)nat * MAXREF);
    Wz = ar.take<double>((size_t)nat * MAXREF);
    zv = ar.take<double>((size_t)nat * MAXREF);
    zr = ar.take<double>((size_t)nat * MAXREF);
    zdcn = ar.take<double>((size_t)nat * MAXREF);
    zrdcn = ar.take<double>((size_t)nat * MAXREF);
    vat = ar.take<double>(nat);
    ed4 = ar.take<double>(nat);
    eh0 = ar.take<double>(nat);
    eaes = ar.take<double>(2 * (size_t)nat);
    erep = ar.take<double>(nat);
    e2 = ar.take<double>(nat);
    e3 = ar.take<double>(((size_t)nat * (nat + 1)) / 2 + 1);
    grad = ar.take<double>(3 * (size_t)nat);
    dhdcn = ar.take<double>(nat);
    tmp2 = ar.take<double>(nat);
    rows = ar.take<double>((size_t)nao * 12);
    emo = ar.take<double>(nao);
    focc = ar.take<double>(nao);
    focca = ar.take<double>(nao);
    foccb = ar.take<double>(nao);
    fe = ar.take<double>(nao);
    tri_d = ar.take<double>(nao);
    tri_e = ar.take<double>(nao);
    tri_e2 = ar.take<double>(nao);
    tri_tau = ar.take<double>(nao);
    tri_p = ar.take<double>(sytrd_workspace(nao));
    bounds = ar.take<double>(8);
    fscal = ar.take<double>(8 + (size_t)nao);
    escal = ar.take<double>(16);
    rms = ar.take<double>(4);
    dip = ar.take<double>(4);
    qin = ar.take<double>(nbr);
    qout = ar.take<double>(nbr);
    dq = ar.take<double>(nbr);
    info = ar.take<int>(8);
    if (npc > 0) {
        vpc = ar.take<double>(nsh);
        pcgrad = ar.take<double>(3 * (size_t)npc);
    }
    bs.nbr = nbr;
    bs.maxit = maxit;
    bs.df = ar.take<double>((size_t)maxit * nbr);
    bs.u = ar.take<double>((size_t)maxit * nbr);
    bs.a = ar.take<double>((size_t)maxit * maxit);
    bs.omega = ar.take<double>(maxit);
    bs.qlast = ar.take<double>(nbr);
    bs.dqlast = ar.take<double>(nbr);
    bs.scratch = ar.take<double>(2 * (size_t)maxit * maxit + 2 * (size_t)maxit + 64);

    };
    ar.counting = true;
    ar.used = 0;
    layout();
    const size_t need = ar.used;
    ar.reset(need, st);
    layout();

    XG_CUDA(cudaMemsetAsync(grad, 0, 3 * (size_t)nat * sizeof(double), st));
    XG_CUDA(cudaMemsetAsync(dhdcn, 0, nat * sizeof(double), st));

    // ---- coordination number, self energies
    cn(st, m, 0, cn_gfn);
    k_self_energy<<<ceil_div(nsh, 128), 128, 0, st>>>(nsh, m.sh_atom, m.sh_se0, m.sh_kcn, cn_gfn, se);
    XG_LAUNCH_CHECK();

    // ---- initial charges: warm start or EEQ guess (newWavefunction, src/xtb/calculator.f90:432-496)
    const bool warm = wfn.valid() && wfn.nat == nat && wfn.nao == nao && wfn.nsh == nsh;
    if (warm) {
        XG_CUDA(cudaMemcpyAsync(qsh, wfn.qsh.data(), nsh * sizeof(double), cudaMemcpyHostToDevice, st));
        XG_CUDA(cudaMemcpyAsync(dipm, wfn.dipm.data(), 3 * nat * sizeof(double), cudaMemcpyHostToDevice, st));
        XG_CUDA(cudaMemcpyAsync(qp, wfn.qp.data(), 6 * nat * sizeof(double), cudaMemcpyHostToDevice, st));
    } else {
        cn(st, m, 2, cn_tmp);
        eeq_setup(st, m, cn_tmp, eeqA, eeqX);
        potrf_upper(st, nat, eeqA, nat, info);
        eeq_finish(st, nat, eeqA, eeqX, hm.charge, q, iscr);   // iscr: free until the first eigenvectors
        int hinfo = 0;
        XG_CUDA(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st));
        XG_CUDA(cudaStreamSynchronize(st));
        if (hinfo != 0) {
            // EEQ guess failed: uniform charges (the reference's rescue path)
            std::vector<double> qq(nat, hm.charge / nat);
            XG_CUDA(cudaMemcpyAsync(q, qq.data(), nat * sizeof(double), cudaMemcpyHostToDevice, st));
        }
        k_ini_qsh<<<ceil_div(nsh, 128), 128, 0, st>>>(nsh, m.sh_atom, m.sh_zsh, d_zval, q, qsh);
        XG_LAUNCH_CHECK();
        XG_CUDA(cudaMemsetAsync(dipm, 0, 3 * (size_t)nat * sizeof(double), st));
        XG_CUDA(cudaMemsetAsync(qp, 0, 6 * (size_t)nat * sizeof(double), st));
    }
    broyden_pack(st, m, qsh, dipm, qp, qin);
    broyden_unpack(st, m, qin, qsh, dipm, qp, q);   // q = sum of qsh (qsh2qat)
    if (guess_only) {
        // the initial-guess wavefunction only (newWavefunction, src/xtb/calculator.f90:432-496)
        wfn = Wavefunction();
        wfn.nat = nat; wfn.nao = nao; wfn.nsh = nsh;
        wfn.q.resize(nat); wfn.qsh.resize(nsh); wfn.dipm.resize(3 * nat); wfn.qp.resize(6 * nat);
        XG_CUDA(cudaMemcpyAsync(wfn.q.data(), q, nat * sizeof(double), cudaMemcpyDeviceToHost, st));
        XG_CUDA(cudaMemcpyAsync(wfn.qsh.data(), qsh, nsh * sizeof(double), cudaMemcpyDeviceToHost, st));
        XG_CUDA(cudaMemcpyAsync(wfn.dipm.data(), dipm, 3 * nat * sizeof(double), cudaMemcpyDeviceToHost, st));
        XG_CUDA(cudaMemcpyAsync(wfn.qp.data(), qp, 6 * nat * sizeof(double), cudaMemcpyDeviceToHost, st));
        tm.stop();
        XG_CUDA(cudaStreamSynchronize(st));
        scc_failed = false;
        return;
    }

    // ---- classical terms and integrals
    repulsion(st, m, erep, grad);
    tm.mark(PH_INTEGRALS);
    build_sdqh0(st, m, se, th, S, D, Q, H0);
    aes_setup(st, m, cn_gfn, radcn, gab3, gab5);
    coulomb_matrix(st, m, J);
    cn(st, m, 3, cn_tmp);
    d4_weights(st, m, cn_tmp, gw, nullptr);
    // S = U^T U, X = U^-1
    tm.mark(PH_CHOLESKY);
    XG_CUDA(cudaMemcpyAsync(T1, S, nn * sizeof(double), cudaMemcpyDeviceToDevice, st));
    potrf_upper(st, nao, T1, nao, info);
    trinv_upper(st, nao, T1, nao, X, nao);
    {
        int hinfo = 0;
        XG_CUDA(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st));
        XG_CUDA(cudaStreamSynchronize(st));
        if (hinfo != 0) throw std::runtime_error("overlap matrix is not positive definite (Cholesky failed)");
    }

    if (solv) solv_update(st, sd, m.xyz);   // Born radii, surface, Born matrix (src/scf_module.F90:298-321)
    if (npc > 0) {   // shell potential of the external charges, fixed for the single point
        k_pc_potential<<<ceil_div((long)nsh * 32, 128), 128, 0, st>>>(m, npc, pcq, pcx, pcg, vpc);
        XG_LAUNCH_CHECK();
    }
    // ---- SCC iterations
    double eel = 0.0, eold = 0.0;
    bool lastdiag = false, converged = false;
    int iter = 0;
    double hsc[8] = {0};
    for (int it = 1; it <= maxit; ++it) {
        iter = it;
        tm.mark(PH_HBUILD);
        d4_scc(st, m, gw, q, zeta, dzeta, Wz, vat, ed4);
        if (solv) solv_shift(st, sd, q, vat);          // atomic potential B q (src/scc_core.f90:444-448)
        shell_shift(st, m, J, qsh, vat, shift, Jq);
        if (npc > 0) {   // the external charges' field enters every iteration's shift
            k_add_vec<<<ceil_div(nsh, 256), 256, 0, st>>>(nsh, vpc, shift);
            XG_LAUNCH_CHECK();
        }
        aes_potential(st, m, q, dipm, qp, gab3, gab5, true, vs, vd, vq);
        build_hu(st, m, th, H0, S, D, Q, shift, vs, vd, vq, H);
        // standard form A = X^T H X (X = U^-1 upper triangular) as B + B^T with B = X^T (Hu X):
        // Hu X is a product of two upper triangular matrices (n^3/3 flops) and X^T (Hu X) needs
        // only k < min(i, j) (2 n^3/3), so n^3 flops in all against 5/3 n^3 for X^T (H X) --
        // the count of LAPACK's dsygst
        tm.mark(PH_STDFORM);
        dgemm(st, false, false, nao, nao, nao, 1.0, H, nao, X, nao, 0.0, T1, nao, GF_A_UPPER | GF_B_UPPER);
        dgemm(st, true, false, nao, nao, nao, 1.0, X, nao, T1, nao, 0.0, A, nao, GF_A_LOWER | GF_B_UPPER);
        sym_add(st, nao, A, nao);
        tm.mark(PH_SYTRD);
        sytrd_form(st, nao, A, nao, V, tri_tau, tri_d, tri_e, tri_p, -1, set.max_coop_blocks);
        // eigenvalues, occupations, then eigenvectors of the occupied orbitals only
        tm.mark(PH_TRIEIG);
        // inside the SCC only the levels that can carry occupation are needed: the lowest
        // nocc + max(32, n / 16), unless the smearing reaches further (then the rest follow, still
        // on the device); the last diagonalisation computes all of them for the results
        const bool all_levels = lastdiag || it == maxit;
        const int klev = all_levels ? nao : std::min(nao, std::max(hm.nel_a, hm.nel_b) + std::max(32, nao / 16));
        tridiag_eigvals(st, nao, tri_d, tri_e, tri_e2, bounds, emo, klev);
        fermi(st, nao, emo, hm.nel_a, hm.nel_b, set.etemp, focc, focca, foccb, fscal, info + 1);
        if (klev < nao) {
            tridiag_eigvals_rest(st, nao, tri_d, tri_e2, bounds, emo, klev, fscal, KB_AU * AUTOEV * set.etemp, info + 2);
            fermi(st, nao, emo, hm.nel_a, hm.nel_b, set.etemp, focc, focca, foccb, fscal, info + 1, info + 2);
        }
        tridiag_eigvecs(st, nao, tri_d, tri_e, bounds, emo, Y, iscr, piv, info + 1);
        tm.mark(PH_BACKTR);
        // Y[:, :kocc] = Q Y: compact-WY form (FP64 strips or split GEMMs) for large n, one warp per
        // vector below
        const int bform = set.backtransform_form(nao, split);
        if (bform > 0)
            ormtr_blocked(st, nao, V, tri_tau, Y, info + 1, ormw, bform == 2 ? set.slices : 0, sgw);
        else
            ormtr_inplace(st, nao, V, tri_tau, Y, info + 1);
        if (split)
            split_gemm(st, false, false, nao, nao, nao, 1.0, X, nao, Y, nao, 0.0, C, nao, set.slices, sgw, nullptr,
                       info + 1);
        else
            dgemm(st, false, false, nao, nao, nao, 1.0, X, nao, Y, nao, 0.0, C, nao, GF_A_UPPER, nullptr, info + 1);
        tm.mark(PH_DENSITY);
        scale_cols(st, nao, C, focc, T1);
        if (split) {
            split_gemm(st, false, true, nao, nao, nao, 1.0, T1, nao, C, nao, 0.0, Pm, nao, set.slices, sgw, info + 1);
        } else {
            dgemm(st, false, true, nao, nao, nao, 1.0, T1, nao, C, nao, 0.0, Pm, nao, GF_SYM, info + 1);
            mirror_lower(st, nao, Pm, nao);
        }
        tm.mark(PH_POPMIX);
        populations(st, m, Pm, S, D, Q, H0, rows, qsh, q, dipm, qp, eh0);
        shell_shift(st, m, J, qsh, nullptr, T1, Jq);    // Jq for the electrostatic energy
        aes_energy(st, m, q, dipm, qp, gab3, gab5, eaes);
        d4_scc(st, m, gw, q, zeta, dzeta, Wz, vat, ed4);
        if (solv) solv_energy(st, sd, q);               // src/scc_core.f90:544-548
        k_scc_energy<<<1, 512, 0, st>>>(nsh, nat, qsh, Jq, m.sh_gam3, eh0, eaes, ed4, fscal, vpc,
                                        solv ? sd.esolv : nullptr, escal);
        XG_LAUNCH_CHECK();
        broyden_pack(st, m, qsh, dipm, qp, qout);
        broyden_step(st, bs, it, 0.4, qin, qout, dq, rms, nat);
        broyden_unpack(st, m, qin, qsh, dipm, qp, q);
        XG_CUDA(cudaMemcpyAsync(hsc, escal, 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
        double hrms[2];
        XG_CUDA(cudaMemcpyAsync(hrms, rms, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
        XG_CUDA(cudaStreamSynchronize(st));
        d2h += 8 * sizeof(double);
        eold = eel;
        eel = hsc[0];
        const bool econv = std::fabs(eel - eold) < scfconv;
        const bool qconvd = hrms[0] < qconv;
        if (!std::isfinite(eel)) throw std::runtime_error("SCC energy is not finite");
        if (econv && qconvd) {
            converged = true;
            if (lastdiag) break;
            lastdiag = true;
        }
    }
    scc_failed = !converged;

    if (keep_orbitals) {
        // all MO coefficients of the last iteration (only occupied ones were needed inside the SCC)
        tridiag_eigvecs(st, nao, tri_d, tri_e, bounds, emo, Y, iscr, piv, nullptr);
        if (set.backtransform_form(nao, false) > 0) ormtr_blocked(st, nao, V, tri_tau, Y, nullptr, ormw);
        else ormtr_inplace(st, nao, V, tri_tau, Y, nullptr);
        dgemm(st, false, false, nao, nao, nao, 1.0, X, nao, Y, nao, 0.0, C, nao, GF_A_UPPER);
    }
    // ---- gradient (src/scf_module.F90:665-798)
    tm.mark(PH_GRADIENT);
    k_scale_energy_weights<<<ceil_div(nao, 128), 128, 0, st>>>(nao, focc, emo, fe);
    XG_LAUNCH_CHECK();
    scale_cols(st, nao, C, fe, T1);
    if (split) {
        split_gemm(st, false, true, nao, nao, nao, 1.0, T1, nao, C, nao, 0.0, Wm, nao, set.slices, sgw, info + 1);
    } else {
        dgemm(st, false, true, nao, nao, nao, 1.0, T1, nao, C, nao, 0.0, Wm, nao, GF_SYM, info + 1);
        mirror_lower(st, nao, Wm, nao);
    }
    aes_potential(st, m, q, dipm, qp, gab3, gab5, false, vs, vd, vq);
    grad_sdqh0(st, m, th, se, Pm, Wm, shift, vs, vd, vq, grad, dhdcn);
    dhdcn_diag(st, m, Pm, dhdcn);
    aes_grad(st, m, q, dipm, qp, radcn, gab3, gab5, grad, tmp2);
    aes_dradcn(st, m, cn_gfn, tmp2, dhdcn);
    cn_chain(st, m, 0, dhdcn, grad);
    // D4 two-body and ATM at the final charges, covalent CN
    cn(st, m, 1, cn_tmp);
    XG_CUDA(cudaMemsetAsync(tmp2, 0, nat * sizeof(double), st));
    d4_grad(st, m, cn_tmp, q, gw, dgw, zv, zr, zdcn, zrdcn, c6, dc6, c6z, dc6z, e2, e3, tmp2, grad, iscr);
    cn_chain(st, m, 1, tmp2, grad);
    coulomb_grad(st, m, qsh, grad);
    if (npc > 0) {
        k_pc_grad_atoms<<<ceil_div((long)nat * 32, 128), 128, 0, st>>>(m, npc, pcq, pcx, pcg, qsh, grad);
        k_pc_grad_charges<<<ceil_div((long)npc * 32, 128), 128, 0, st>>>(m, npc, pcq, pcx, pcg, qsh, pcgrad);
        XG_LAUNCH_CHECK();
    }
    double hsolv[4] = {0, 0, 0, 0};
    if (solv) {   // gradient and energy parts at the final charges (src/scf_module.F90:761-776)
        solv_gradient(st, sd, m.xyz, q, grad);
        solv_energy(st, sd, q);
        XG_CUDA(cudaMemcpyAsync(hsolv, sd.esolv, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
        d2h += 4 * sizeof(double);
    }
    k_dipole<<<1, 256, 0, st>>>(nat, nao, m.xyz, d_zval, rows, dip);
    XG_LAUNCH_CHECK();
    const bool closed = hm.nel_a == hm.nel_b;
    if (closed) {
        dgemm(st, false, false, nao, nao, nao, 1.0, Pm, nao, S, nao, 0.0, T1, nao);
        k_wiberg<<<ceil_div((long)aa * 32, 256), 256, 0, st>>>(nat, nao, m.xyz, m.at_ao0, m.at_nao, T1, nullptr,
                                                                1.0, c6);
        XG_LAUNCH_CHECK();
    } else {
        // spin densities Pa, Pb from the smeared alpha / beta occupations, then (Pa S), (Pb S)
        scale_cols(st, nao, C, focca, T1);
        dgemm(st, false, true, nao, nao, nao, 1.0, T1, nao, C, nao, 0.0, A, nao);
        dgemm(st, false, false, nao, nao, nao, 1.0, A, nao, S, nao, 0.0, H, nao);
        scale_cols(st, nao, C, foccb, T1);
        dgemm(st, false, true, nao, nao, nao, 1.0, T1, nao, C, nao, 0.0, A, nao);
        dgemm(st, false, false, nao, nao, nao, 1.0, A, nao, S, nao, 0.0, Y, nao);
        k_wiberg<<<ceil_div((long)aa * 32, 256), 256, 0, st>>>(nat, nao, m.xyz, m.at_ao0, m.at_nao, H, Y, 2.0, c6);
        XG_LAUNCH_CHECK();
    }
    reduce_sum(st, erep, nat, escal + 8);
    reduce_sum(st, e3, (int)(((size_t)nat * (nat + 1)) / 2), escal + 9);

    tm.stop();
    const int total_end = (int)tm.next;
    XG_CUDA(cudaEventRecord(tm.get(), st));
    // ---- results
    double hs2[2];
    res.gradient.assign(3 * (size_t)nat, 0.0);
    res.dipole.assign(3, 0.0);
    res.wbo.assign(aa, 0.0);
    XG_CUDA(cudaMemcpyAsync(res.wbo.data(), c6, aa * sizeof(double), cudaMemcpyDeviceToHost, st));
    wfn.nat = nat; wfn.nao = nao; wfn.nsh = nsh;
    wfn.q.resize(nat); wfn.qsh.resize(nsh); wfn.dipm.resize(3 * nat); wfn.qp.resize(6 * nat);
    wfn.emo.resize(nao); wfn.focc.resize(nao);
    XG_CUDA(cudaMemcpyAsync(hs2, escal + 8, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    res.pcgrad.assign(3 * (size_t)npc, 0.0);
    if (npc > 0)
        XG_CUDA(cudaMemcpyAsync(res.pcgrad.data(), pcgrad, 3 * (size_t)npc * sizeof(double), cudaMemcpyDeviceToHost,
                                st));
    XG_CUDA(cudaMemcpyAsync(res.gradient.data(), grad, 3 * nat * sizeof(double), cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaMemcpyAsync(res.dipole.data(), dip, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaMemcpyAsync(wfn.q.data(), q, nat * sizeof(double), cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaMemcpyAsync(wfn.qsh.data(), qsh, nsh * sizeof(double), cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaMemcpyAsync(wfn.dipm.data(), dipm, 3 * nat * sizeof(double), cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaMemcpyAsync(wfn.qp.data(), qp, 6 * nat * sizeof(double), cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaMemcpyAsync(wfn.emo.data(), emo, nao * sizeof(double), cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaMemcpyAsync(wfn.focc.data(), focc, nao * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (keep_orbitals) {
        wfn.C.resize(nn); wfn.P.resize(nn); wfn.S.resize(nn);
        XG_CUDA(cudaMemcpyAsync(wfn.C.data(), C, nn * sizeof(double), cudaMemcpyDeviceToHost, st));
        XG_CUDA(cudaMemcpyAsync(wfn.P.data(), Pm, nn * sizeof(double), cudaMemcpyDeviceToHost, st));
        XG_CUDA(cudaMemcpyAsync(wfn.S.data(), S, nn * sizeof(double), cudaMemcpyDeviceToHost, st));
    } else {
        wfn.C.clear(); wfn.P.clear(); wfn.S.clear();
    }
    XG_CUDA(cudaStreamSynchronize(st));
    d2h += (long long)sizeof(double) * (2 + 3 * nat + 3 + nat + nsh + 9 * nat + 2 * nao + aa +
                                        (keep_orbitals ? 3 * nn : 0));
    res.h2d_bytes = g_h2d;
    res.launches = launch_counter() - launches0;
    res.d2h_bytes = d2h;
    for (auto& e : wfn.emo) e *= EVTOAU;   // orbital energies are reported in Hartree
    res.phase_ms = tm.collect();
    {
        float t = 0.0f;
        XG_CUDA(cudaEventElapsedTime(&t, tm.pool[total_ev], tm.pool[total_end]));
        res.phase_ms[PH_TOTAL] = t;
    }
    res.e_pc = hsc[6];
    res.solvated = solv;
    res.g_solv = hsolv[0];
    res.g_hb = hsolv[1];
    res.g_sasa = hsolv[2];
    res.g_shift = hsolv[3];
    res.g_born = hsolv[0] - hsolv[1] - hsolv[2] - hsolv[3];
    res.e_rep = hs2[0];
    res.e_atm = hs2[1];
    res.energy = eel + hs2[0] + hs2[1];
    res.e_elec = eel + hs2[1];
    res.e_es = hsc[1];
    res.e_aes = hsc[2];
    res.e_axc = hsc[3];
    res.e_disp = hsc[4] + hs2[1];
    res.iterations = iter;
    res.converged = converged;
    const int ih = hm.nel_a;
    res.hl_gap = (ih >= 1 && ih < nao) ? (wfn.emo[ih] - wfn.emo[ih - 1]) * AUTOEV : 0.0;
    double g2 = 0.0;
    for (double g : res.gradient) g2 += g * g;
    res.gnorm = std::sqrt(g2);
}

}  // namespace xg
