// Host driver of the batched engine: partition, launch, gather, hand-over.
//
// Molecules up to BATCH_MAX_NAO AOs run in one DeviceBatch (one thread block per
// molecule, ordered by decreasing AO count so that the large ones start first);
// larger molecules, and any molecule whose SCC outgrows the batched Broyden
// history, run on the plain per-molecule GPU engine.  Both paths compute on the
// device; there is no CPU fallback.
#include <algorithm>
#include <chrono>
#include <numeric>

#include "batch.h"

namespace xg {

namespace {
thread_local cudaStream_t g_bstream = nullptr;
thread_local DeviceBatch* g_batch = nullptr;
}  // namespace

std::string run_batch(const std::vector<HostMol>& mols, const BatchSettings& set, const std::vector<int>& want_grad,
                      BatchResults& out, const std::vector<const Wavefunction*>* guesses) {
    const auto t0 = std::chrono::steady_clock::now();
    if (device_count() == 0) throw CudaError("no CUDA device available for the GFN2 engine");
    if (!g_bstream) XG_CUDA(cudaStreamCreateWithFlags(&g_bstream, cudaStreamNonBlocking));
    if (!g_batch) g_batch = new DeviceBatch();
    cudaStream_t st = g_bstream;
    const int nmol = (int)mols.size();
    std::vector<long> atom_off(nmol + 1, 0);
    for (int i = 0; i < nmol; ++i) atom_off[i + 1] = atom_off[i] + mols[i].nat;
    const long natot = atom_off[nmol];
    out = BatchResults();
    out.energy.assign(nmol, 0.0);
    out.gradient.assign(3 * natot, 0.0);
    out.charges.assign(natot, 0.0);
    out.dipole.assign(3 * (size_t)nmol, 0.0);
    out.parts.assign(8 * (size_t)nmol, 0.0);
    out.iterations.assign(nmol, 0);
    out.converged.assign(nmol, 0);
    out.status.assign(nmol, BST_OK);
    out.engine.assign(nmol, 0);

    std::vector<int> batched, plain;
    for (int i = 0; i < nmol; ++i) (mols[i].nao <= BATCH_MAX_NAO ? batched : plain).push_back(i);
    std::stable_sort(batched.begin(), batched.end(), [&](int a, int b) { return mols[a].nao > mols[b].nao; });

    const long long launches0 = launch_counter();
    if (!batched.empty()) {
        std::vector<const HostMol*> hm;
        std::vector<const Wavefunction*> gs;
        std::vector<int> wg;
        std::vector<long> off(batched.size());
        long o = 0;
        for (size_t k = 0; k < batched.size(); ++k) {
            hm.push_back(&mols[batched[k]]);
            gs.push_back(guesses ? (*guesses)[batched[k]] : nullptr);
            wg.push_back(want_grad.empty() ? 1 : want_grad[batched[k]]);
            off[k] = o;
            o += mols[batched[k]].nat;
        }
        DeviceBatch& db = *g_batch;
        db.load(hm, wg, st, guesses ? &gs : nullptr);
        out.h2d += db.h2d_bytes() + (long long)(sizeof(long) * off.size());
        // outputs packed in batch order
        long* d_off = nullptr;
        double *d_grad = nullptr, *d_q = nullptr;
        XG_CUDA(cudaMallocAsync(&d_off, sizeof(long) * off.size(), st));
        XG_CUDA(cudaMallocAsync(&d_grad, sizeof(double) * 3 * std::max<long>(o, 1), st));
        XG_CUDA(cudaMallocAsync(&d_q, sizeof(double) * std::max<long>(o, 1), st));
        XG_CUDA(cudaMemcpyAsync(d_off, off.data(), sizeof(long) * off.size(), cudaMemcpyHostToDevice, st));
        cudaEvent_t e0, e1;
        XG_CUDA(cudaEventCreate(&e0));
        XG_CUDA(cudaEventCreate(&e1));
        XG_CUDA(cudaEventRecord(e0, st));
        db.step(set, std::max(1, set.maxiter), st);
        XG_CUDA(cudaEventRecord(e1, st));
        db.gather(d_off, d_grad, d_q, st);
        std::vector<double> g(3 * o), q(o);
        XG_CUDA(cudaMemcpyAsync(g.data(), d_grad, sizeof(double) * 3 * o, cudaMemcpyDeviceToHost, st));
        XG_CUDA(cudaMemcpyAsync(q.data(), d_q, sizeof(double) * o, cudaMemcpyDeviceToHost, st));
        std::vector<BatchMol> state;
        db.fetch_states(state, st);   // synchronises the stream
        float ms = 0.0f;
        XG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        out.device_ms += ms;
        XG_CUDA(cudaEventDestroy(e0));
        XG_CUDA(cudaEventDestroy(e1));
        XG_CUDA(cudaFreeAsync(d_off, st));
        XG_CUDA(cudaFreeAsync(d_grad, st));
        XG_CUDA(cudaFreeAsync(d_q, st));
        out.d2h += (long long)sizeof(double) * 4 * o + (long long)(sizeof(BatchMol) * state.size());
        for (size_t k = 0; k < batched.size(); ++k) {
            const int i = batched[k];
            const BatchMol& b = state[k];
            if (b.status == BST_HISTORY) {
                plain.push_back(i);
                continue;
            }
            out.status[i] = b.status;
            out.iterations[i] = b.iter;
            out.converged[i] = b.converged;
            out.energy[i] = b.out[BO_ENERGY];
            const double parts[8] = {b.out[BO_ELEC], b.out[BO_REP], b.out[BO_ES], b.out[BO_AES],
                                     b.out[BO_AXC], b.out[BO_DISP], b.out[BO_ATM], b.out[BO_GAP]};
            std::copy(parts, parts + 8, out.parts.begin() + 8 * (size_t)i);
            for (int x = 0; x < 3; ++x) out.dipole[3 * (size_t)i + x] = b.out[BO_DIPX + x];
            const int nat = mols[i].nat;
            std::copy(g.begin() + 3 * off[k], g.begin() + 3 * (off[k] + nat), out.gradient.begin() + 3 * atom_off[i]);
            std::copy(q.begin() + off[k], q.begin() + off[k] + nat, out.charges.begin() + atom_off[i]);
        }
    }
    // plain engine for the rest (large molecules, long SCCs)
    std::sort(plain.begin(), plain.end());
    for (int i : plain) {
        SPSettings ps;
        ps.accuracy = set.accuracy;
        ps.etemp = set.etemp;
        ps.maxiter = set.maxiter;
        Wavefunction wfn;
        if (guesses && (*guesses)[i]) wfn = *(*guesses)[i];   // warm start from the given guess
        SPResult r;
        bool failed = false;
        run_singlepoint(mols[i], ps, wfn, r, false, failed);
        out.engine[i] = 1;
        out.status[i] = failed ? BST_NOT_CONVERGED : BST_OK;
        out.iterations[i] = r.iterations;
        out.converged[i] = r.converged;
        out.energy[i] = r.energy;
        const double parts[8] = {r.e_elec, r.e_rep, r.e_es, r.e_aes, r.e_axc, r.e_disp, r.e_atm, r.hl_gap};
        std::copy(parts, parts + 8, out.parts.begin() + 8 * (size_t)i);
        std::copy(r.dipole.begin(), r.dipole.end(), out.dipole.begin() + 3 * (size_t)i);
        std::copy(r.gradient.begin(), r.gradient.end(), out.gradient.begin() + 3 * atom_off[i]);
        std::copy(wfn.q.begin(), wfn.q.end(), out.charges.begin() + atom_off[i]);
        out.device_ms += r.phase_ms[PH_TOTAL];
        out.h2d += r.h2d_bytes;
        out.d2h += r.d2h_bytes;
        ++out.plain_count;
    }
    out.launches = launch_counter() - launches0;
    out.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return std::string();
}

}  // namespace xg
