// Request loop of the GFN2-xTB engine: resident pool with continuous batching plus
// plain-engine workers (see serve.h).
#include "serve.h"

#include <algorithm>
#include <chrono>

namespace xg {

Server::Server(const ServeConfig& cfg) : cfg_(cfg), t0_(std::chrono::steady_clock::now()) {
    if (device_count() == 0) throw CudaError("no CUDA device available for the GFN2 engine");
    pool_thread_ = std::thread([this] { pool_loop(); });
    for (int i = 0; i < std::max(1, cfg_.plain_workers); ++i) plain_threads_.emplace_back([this] { plain_loop(); });
}

Server::~Server() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        stop_ = true;
    }
    cv_work_.notify_all();
    if (pool_thread_.joinable()) pool_thread_.join();
    {
        std::lock_guard<std::mutex> lk(mu_);
        pool_done_ = true;
    }
    cv_work_.notify_all();
    for (auto& t : plain_threads_)
        if (t.joinable()) t.join();
}

double Server::now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
}

long long Server::submit(int nat, const int* Z, const double* xyz, double charge, int uhf, int want_grad,
                         std::string& err) {
    auto r = std::make_unique<Req>();
    err = build_host_mol(nat, Z, xyz, charge, uhf, r->hm);
    if (!err.empty()) return -1;
    r->want_grad = want_grad;
    r->t_start = 0.0;
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (stop_) {
            err = "server is stopping";
            return -1;
        }
        r->id = next_id_++;
        r->t_submit = now();
        const long long id = r->id;
        if (r->hm.nao <= cfg_.pool_max_nao) small_q_.push_back(std::move(r));
        else large_q_.push_back(std::move(r));
        ++inflight_;
        cv_work_.notify_all();
        return id;
    }
}

bool Server::wait(long long id, Completed& out, double timeout) {
    std::unique_lock<std::mutex> lk(mu_);
    auto ready = [&] { return done_.count(id) > 0; };
    if (timeout < 0) cv_done_.wait(lk, ready);
    else if (!cv_done_.wait_for(lk, std::chrono::duration<double>(timeout), ready)) return false;
    out = std::move(done_[id]);
    done_.erase(id);
    return true;
}

std::vector<double> Server::stats() const {
    std::lock_guard<std::mutex> lk(mu_);
    return {n_done_, n_plain_, n_steps_, busy_, peak_, n_rerun_, h2d_, d2h_, launches_, scc_ms_, scc_flops_};
}

void Server::inject_admission_failures(int n) {
    std::lock_guard<std::mutex> lk(mu_);
    inject_admissions_ = std::max(0, n);
}

void Server::complete(Completed&& c) {
    std::lock_guard<std::mutex> lk(mu_);
    c.t_done = now();
    n_done_ += 1;
    if (c.engine == 1) n_plain_ += 1;
    --inflight_;
    done_[c.id] = std::move(c);
    cv_done_.notify_all();
}

void Server::pool_loop() {
    try {
        pool_body();
    } catch (const std::exception& e) {
        // a device error ends the pool: fail every request still waiting for it
        std::vector<std::unique_ptr<Req>> lost;
        {
            std::lock_guard<std::mutex> lk(mu_);
            pool_error_ = e.what();
            while (!small_q_.empty()) {
                lost.push_back(std::move(small_q_.front()));
                small_q_.pop_front();
            }
        }
        for (auto& r : lost) {
            Completed c;
            c.id = r->id;
            c.status = BST_NONFINITE;
            c.error = pool_error_;
            c.t_submit = r->t_submit;
            complete(std::move(c));
        }
        for (auto& c : failed_resident_) complete(std::move(c));
    }
}

void Server::pool_body() {
    cudaStream_t st = nullptr;
    XG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    SlotPool pool(cfg_.pool_bytes, cfg_.max_slots);
    std::vector<std::unique_ptr<Req>> resident(cfg_.max_slots);
    struct FailResident {   // on an exception, the resident requests complete with the error
        std::vector<std::unique_ptr<Req>>& res;
        std::vector<Completed>& out;
        ~FailResident() {
            for (auto& r : res)
                if (r) {
                    Completed c;
                    c.id = r->id;
                    c.status = BST_NONFINITE;
                    c.error = "device error in the resident pool";
                    c.t_submit = r->t_submit;
                    out.push_back(std::move(c));
                }
        }
    } guard{resident, failed_resident_};
    std::vector<int> slots;
    std::vector<BatchMol> states;
    for (;;) {
        std::vector<std::unique_ptr<Req>> incoming;
        {
            std::unique_lock<std::mutex> lk(mu_);
            if (pool.resident() == 0) cv_work_.wait(lk, [&] { return stop_ || !small_q_.empty(); });
            if (small_q_.empty() && pool.resident() == 0 && stop_) break;
            while (!small_q_.empty()) {
                incoming.push_back(std::move(small_q_.front()));
                small_q_.pop_front();
            }
            if (inject_admissions_ > 0) {
                pool.fail_next_admissions(inject_admissions_);
                inject_admissions_ = 0;
            }
        }
        // admission: in arrival order while slots and HBM budget last; a request whose
        // admission fails (its upload threw) completes with the error, the others go on
        std::vector<std::unique_ptr<Req>> back, to_plain;
        std::vector<Completed> rejected;
        bool full = false;
        for (auto& r : incoming) {
            int slot = -1;
            try {
                slot = full ? -1 : pool.admit(r->hm, r->want_grad, st);
            } catch (const std::exception& e) {
                Completed c;
                c.id = r->id;
                c.status = BST_NONFINITE;
                c.error = e.what();
                c.t_submit = r->t_submit;
                c.nao = r->hm.nao;
                rejected.push_back(std::move(c));
                continue;
            }
            if (slot >= 0) {
                r->t_start = now();
                resident[slot] = std::move(r);
            } else if (pool.resident() == 0 && DeviceBatch::bytes_for(r->hm) + 4096 > pool.capacity()) {
                to_plain.push_back(std::move(r));   // never fits the pool
            } else {
                full = true;
                back.push_back(std::move(r));
            }
        }
        if (!back.empty() || !to_plain.empty()) {
            std::lock_guard<std::mutex> lk(mu_);
            for (auto it = back.rbegin(); it != back.rend(); ++it) small_q_.push_front(std::move(*it));
            for (auto& r : to_plain) large_q_.push_back(std::move(r));
            cv_work_.notify_all();
        }
        for (auto& c : rejected) complete(std::move(c));
        {
            std::lock_guard<std::mutex> lk(mu_);
            h2d_ += (double)(pool.h2d_bytes() - pool_h2d_seen_);
            pool_h2d_seen_ = pool.h2d_bytes();
        }
        if (pool.resident() == 0) continue;
        {
            std::lock_guard<std::mutex> lk(mu_);
            peak_ = std::max(peak_, (double)pool.resident());
        }
        const double t1 = now();
        const long long l0 = launch_counter();
        pool.step(cfg_.set, std::max(1, cfg_.iters_per_step), st);
        pool.finished(slots, states, st);
        double step_d2h = (double)pool.last_state_bytes();
        std::vector<Completed> out;
        std::vector<int> rel;
        for (size_t k = 0; k < slots.size(); ++k) {
            const int slot = slots[k];
            const BatchMol& b = states[k];
            std::unique_ptr<Req> req = std::move(resident[slot]);
            rel.push_back(slot);
            if (b.status == BST_HISTORY) {
                std::lock_guard<std::mutex> lk(mu_);
                n_rerun_ += 1;
                large_q_.push_front(std::move(req));
                cv_work_.notify_all();
                continue;
            }
            Completed c;
            c.id = req->id;
            c.engine = 0;
            c.energy = b.out[BO_ENERGY];
            const double parts[8] = {b.out[BO_ELEC], b.out[BO_REP], b.out[BO_ES], b.out[BO_AES],
                                     b.out[BO_AXC], b.out[BO_DISP], b.out[BO_ATM], b.out[BO_GAP]};
            std::copy(parts, parts + 8, c.parts);
            for (int x = 0; x < 3; ++x) c.dipole[x] = b.out[BO_DIPX + x];
            c.iterations = b.iter;
            c.converged = b.converged;
            c.status = b.status;
            c.t_submit = req->t_submit;
            c.t_start = req->t_start;
            c.gradient.assign(3 * (size_t)b.m.nat, 0.0);
            c.charges.assign(b.m.nat, 0.0);
            c.nao = b.m.nao;
            out.push_back(std::move(c));
            pool.copy_results(b, out.back().gradient.data(), out.back().charges.data(), st);
            step_d2h += 4.0 * sizeof(double) * b.m.nat;
        }
        XG_CUDA(cudaStreamSynchronize(st));
        for (int slot : rel) pool.release(slot);
        {
            std::lock_guard<std::mutex> lk(mu_);
            n_steps_ += 1;
            busy_ += now() - t1;
            launches_ += (double)(launch_counter() - l0);
            d2h_ += step_d2h;
            scc_ms_ += pool.last_scc_ms();
            scc_flops_ += pool.last_scc_flops();
        }
        for (auto& c : out) complete(std::move(c));
    }
    cudaStreamDestroy(st);
}

void Server::plain_loop() {
    for (;;) {
        std::unique_ptr<Req> r;
        int rank = 0;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_work_.wait(lk, [&] { return (stop_ && pool_done_) || !large_q_.empty(); });
            if (large_q_.empty()) break;
            // largest first: the large requests dominate the makespan of a saturated stream
            auto it = std::max_element(large_q_.begin(), large_q_.end(),
                                       [](const std::unique_ptr<Req>& a, const std::unique_ptr<Req>& b) {
                                           return a->hm.nao < b->hm.nao;
                                       });
            r = std::move(*it);
            large_q_.erase(it);
            // the critical path of a saturated stream runs through the largest requests: the
            // k-th largest of those in flight gets the k-th most urgent stream priority, so its
            // blocks are dispatched before those of smaller requests and of the pool
            rank = (int)std::distance(running_nao_.upper_bound(r->hm.nao), running_nao_.end());
            running_nao_.insert(r->hm.nao);
        }
        r->t_start = now();
        Completed c;
        c.id = r->id;
        c.engine = 1;
        c.t_submit = r->t_submit;
        c.t_start = r->t_start;
        try {
            SPSettings ps;
            ps.accuracy = cfg_.set.accuracy;
            ps.etemp = cfg_.set.etemp;
            ps.maxiter = cfg_.set.maxiter;
            ps.precision = cfg_.precision;
            ps.slices = cfg_.slices;
            // a cap proportional to the request's size: the per-column chain bounds a medium
            // tridiagonalisation, so a few dozen blocks do it nearly as fast as every SM and leave
            // the rest to the other requests
            ps.max_coop_blocks = cfg_.coop_blocks >= 0 ? cfg_.coop_blocks
                                                        : std::max(8, r->hm.nao / (-cfg_.coop_blocks));
            int least = 0, greatest = 0;
            XG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
            ps.stream_priority = std::min(least, greatest + rank);
            Wavefunction wfn;
            SPResult res;
            bool failed = false;
            run_singlepoint(r->hm, ps, wfn, res, false, failed);
            {
                std::lock_guard<std::mutex> lk(mu_);
                h2d_ += (double)res.h2d_bytes;
                d2h_ += (double)res.d2h_bytes;
                launches_ += (double)res.launches;
            }
            c.nao = r->hm.nao;
            c.sytrd_ms = res.phase_ms[PH_SYTRD];
            c.energy = res.energy;
            const double parts[8] = {res.e_elec, res.e_rep, res.e_es, res.e_aes, res.e_axc, res.e_disp, res.e_atm,
                                     res.hl_gap};
            std::copy(parts, parts + 8, c.parts);
            std::copy(res.dipole.begin(), res.dipole.end(), c.dipole);
            c.gradient = res.gradient;
            c.charges = wfn.q;
            c.iterations = res.iterations;
            c.converged = res.converged;
            c.status = failed ? BST_NOT_CONVERGED : BST_OK;
        } catch (const std::exception& e) {
            c.error = e.what();
            c.status = BST_NONFINITE;
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            running_nao_.erase(running_nao_.find(r->hm.nao));
        }
        complete(std::move(c));
    }
}

}  // namespace xg
