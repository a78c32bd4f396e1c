// Batched GFN2-xTB single points: many molecules of uneven size, one thread block per
// molecule, every molecule's state resident on the device until it is done.
//
// A molecule moves through three stages -- set-up (CN, EEQ guess, integrals,
// Coulomb/AES/D4 kernels, S = U^T U, X = U^-1), SCC iterations, gradient -- and
// each launch of the step kernel advances every unfinished molecule by at most a
// given number of SCC iterations, so a batch can run to completion in one launch
// or be advanced step by step while a request loop admits new molecules into
// freed slots.  The arithmetic per molecule is the plain engine's (same device
// bodies), with the dense linear algebra done by one thread block.
#pragma once
#include <string>
#include <vector>

#include "engine.h"
#include "gfn2_kernels.h"
#include "host_model.h"

namespace xg {

// molecules with more AOs than this go to the plain per-molecule engine
constexpr int BATCH_MAX_NAO = 512;
// Broyden history rows kept per molecule; an SCC that needs more iterations is
// handed to the plain engine
constexpr int BATCH_HIST = 48;

enum BatchStage { BS_SETUP = 0, BS_SCC = 1, BS_GRAD = 2, BS_DONE = 3 };
enum BatchStatus { BST_OK = 0, BST_NOT_CONVERGED = 1, BST_CHOLESKY = 2, BST_NONFINITE = 3, BST_HISTORY = 4 };

// output slots per molecule
enum BatchOut {
    BO_ENERGY = 0, BO_ELEC, BO_REP, BO_ES, BO_AES, BO_AXC, BO_DISP, BO_ATM, BO_GAP, BO_DIPX, BO_DIPY, BO_DIPZ,
    BO_COUNT = 16
};

struct BatchMol {
    DevMol m;
    // set-up / SCC / gradient work arrays (device)
    double *S, *D, *Q, *H0, *X, *H, *A, *T1, *C, *P, *W, *V, *Y, *Zt, *iscr;
    unsigned char* piv;
    double *J, *gab3, *gab5, *c6, *dc6, *c6z, *dc6z, *eeqA, *eeqX, *cn_gfn, *cn_tmp, *se, *q, *qsh, *dipm, *qp,
        *shift, *Jq, *vs, *vd, *vq, *radcn, *gw, *dgw, *zeta, *dzeta, *Wz, *zv, *zr, *zdcn, *zrdcn, *vat, *ed4, *eh0,
        *eaes, *erep, *e2, *e3, *grad, *dhdcn, *tmp2, *rows, *emo, *focc, *focca, *foccb, *fe, *tri_d, *tri_e,
        *tri_e2, *tri_tau, *tri_p, *bounds, *fscal, *escal, *rms, *qin, *qout, *dq;
    int* kocc;
    BroydenState bs;
    const double* zval;
    const double* guess;   // optional initial wavefunction [qsh; per atom (dipm 3, qp 6)], else EEQ
    int nel_a, nel_b;
    double charge;
    int want_grad;
    // state, written by the device
    int stage, iter, lastdiag, converged, status;
    double eel, eold;
    double out[BO_COUNT];
};

struct BatchSettings {
    double accuracy = 1.0;
    double etemp = 300.0;
    int maxiter = 250;
};

// Integral (S, D, Q, H0) and integral-derivative kernels over a batch: molecules in the set-up
// (respectively gradient) stage, one grid row per molecule (batch_integrals.cu).
void batch_integrals(cudaStream_t st, BatchMol* mols, int nmol, int max_nsh, double intcut);
void batch_integral_gradient(cudaStream_t st, BatchMol* mols, int nmol, int max_nsh, double intcut);

// Device-resident batch: parameters and work arrays of every molecule in one allocation.
class DeviceBatch {
public:
    DeviceBatch() = default;
    DeviceBatch(const DeviceBatch&) = delete;
    DeviceBatch& operator=(const DeviceBatch&) = delete;
    ~DeviceBatch();
    // Lay out and upload the molecules (HostMol from build_host_mol); nao <= BATCH_MAX_NAO each.
    // guesses (optional, per molecule, may hold nullptr): initial wavefunction instead of the EEQ guess.
    void load(const std::vector<const HostMol*>& mols, const std::vector<int>& want_grad, cudaStream_t st,
              const std::vector<const Wavefunction*>* guesses = nullptr);
    // Advance every unfinished molecule by at most `max_iter` SCC iterations (set-up and
    // gradient included); returns the number of molecules still unfinished.
    int step(const BatchSettings& set, int max_iter, cudaStream_t st);
    // Copy the states back (after step); `mols` receives stage/status/out of every molecule.
    void fetch_states(std::vector<BatchMol>& mols, cudaStream_t st) const;
    // Pack every molecule's gradient [nat][3] and charges [nat] at atom offset d_off[i] into
    // d_grad [sum nat][3] and d_q [sum nat] (device arrays).
    void gather(const long* d_off, double* d_grad, double* d_q, cudaStream_t st) const;
    int count() const { return nmol_; }
    long long h2d_bytes() const { return h2d_; }
    size_t bytes() const { return bytes_; }
    static size_t bytes_for(const HostMol& hm);

private:
    char* base_ = nullptr;
    size_t bytes_ = 0;
    int nmol_ = 0;
    int max_nao_ = 0;
    int max_nsh_ = 0;
    BatchMol* d_mols_ = nullptr;
    std::vector<BatchMol> h_mols_;
    long long h2d_ = 0;
};

// Resident molecule pool for continuous batching.  One device allocation of a fixed
// budget holds a descriptor table of `max_slots` molecules followed by the molecules'
// regions (parameters + work arrays), handed out first-fit as molecules are admitted and
// returned when they finish.  Every step advances all resident molecules at once; a
// molecule's state stays on the device from admission to completion.
class SlotPool {
public:
    SlotPool(size_t budget_bytes, int max_slots);
    SlotPool(const SlotPool&) = delete;
    SlotPool& operator=(const SlotPool&) = delete;
    ~SlotPool();
    // Admit a molecule (nao <= BATCH_MAX_NAO): returns its slot, or -1 when no slot or no
    // region of the needed size is free.  Uploads on `st` (the caller keeps hm alive until
    // the next synchronisation of `st`).
    int admit(const HostMol& hm, int want_grad, cudaStream_t st);
    // Advance every resident molecule by at most max_iter SCC iterations.
    void step(const BatchSettings& set, int max_iter, cudaStream_t st);
    // Synchronise `st` and list the resident slots whose molecule is done, with their state.
    void finished(std::vector<int>& slots, std::vector<BatchMol>& states, cudaStream_t st);
    // Copy gradient [nat][3] and charges [nat] of a finished slot (asynchronous on `st`).
    void copy_results(const BatchMol& state, double* grad, double* q, cudaStream_t st) const;
    // Return the slot and its region to the pool.
    void release(int slot);
    int resident() const { return resident_; }
    // figures of the last step (valid after finished()): device ms of the SCC kernel (CUDA
    // events on the pool's stream), algorithmic FP64 flops of the SCC iterations it ran
    // (per molecule and iteration n^3 + 4/3 n^3 + 2 n^3 + n^3 + 2 n^2 k, the reference's
    // LAPACK sequence), and the state bytes copied back
    double last_scc_ms() const { return last_ms_; }
    double last_scc_flops() const { return last_flops_; }
    size_t last_state_bytes() const { return last_state_bytes_; }
    size_t free_bytes() const;
    size_t capacity() const { return cap_; }
    long long h2d_bytes() const { return h2d_; }
    // Host-side fault injection for tests: the next n admissions throw as if the device had run
    // out of memory, after the slot search and before any upload (the region is handed back).
    void fail_next_admissions(int n) { fail_admissions_ = n; }

private:
    char* base_ = nullptr;
    size_t cap_ = 0, desc_ = 0;
    int max_slots_ = 0, resident_ = 0, hi_ = 0;
    BatchMol* d_slots_ = nullptr;
    std::vector<size_t> slot_off_, slot_size_;
    std::vector<int> slot_nao_, slot_nsh_, slot_iter_, slot_nocc_;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    double last_ms_ = 0.0, last_flops_ = 0.0;
    size_t last_state_bytes_ = 0;
    std::vector<std::pair<size_t, size_t>> free_;   // (offset, size), sorted by offset
    int fail_admissions_ = 0;
    long long h2d_ = 0;
};

// Results of run_batch, in input order.
struct BatchResults {
    std::vector<double> energy;      // [nmol] Hartree
    std::vector<double> gradient;    // [sum nat][3] Hartree/Bohr
    std::vector<double> charges;     // [sum nat] Mulliken (Broyden-mixed, as the plain engine)
    std::vector<double> dipole;      // [nmol][3]
    std::vector<double> parts;       // [nmol][8] as xtbgb_getEnergyParts
    std::vector<int> iterations, converged, status, engine;   // engine: 0 batched, 1 plain
    double device_ms = 0.0, wall_ms = 0.0;
    long long h2d = 0, d2h = 0, launches = 0;
    int plain_count = 0;
};

// Single points of all molecules (batched engine, plain engine for the ones it cannot take).
// want_grad[i] (empty: all) selects the gradient.  Throws on device errors.
// guesses (optional): per molecule an initial wavefunction (qsh, dipm, qp of matching size) that
// replaces the EEQ guess, as a warm start does.
std::string run_batch(const std::vector<HostMol>& mols, const BatchSettings& set, const std::vector<int>& want_grad,
                      BatchResults& out, const std::vector<const Wavefunction*>* guesses = nullptr);

}  // namespace xg
