// Request loop: continuous batching of GFN2-xTB single points on one GPU.
//
// Requests arrive at any time (submit is thread-safe).  Molecules up to
// BATCH_MAX_NAO AOs are admitted into a SlotPool as soon as a slot and a region of
// the HBM budget are free, and every step of the pool advances all resident
// molecules by a few SCC iterations, so requests that arrive while others are on
// the GPU join the next step.  Larger molecules (and any batched SCC that outgrows
// its mixing history) go to a set of plain-engine workers, each on its own CUDA
// stream, whose work overlaps with the pool's on the device.
#pragma once
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "batch.h"

namespace xg {

struct ServeConfig {
    size_t pool_bytes = size_t(16) << 30;   // HBM budget of the resident pool
    int max_slots = 1024;                     // resident molecules at most
    int plain_workers = 6;                    // concurrent plain-engine single points
    int iters_per_step = 1;                   // SCC iterations per pool step (a pool launch holds
                                              // its SMs for that long; one measured best)
    int precision = 0, slices = 5;            // plain-engine workers: 1 = split-precision products
    int coop_blocks = 0;                      // plain-engine workers: most blocks of a cooperative
                                              // tridiagonalisation (0: one per SM; -D: one per D
                                              // AOs of the request, at least 8)
    int pool_max_nao = BATCH_MAX_NAO;         // largest molecule (AOs) admitted to the pool; larger
                                              // ones go to the plain-engine workers.  A pool step
                                              // holds its SMs for one SCC iteration of its largest
                                              // molecule, and the workers' cooperative launches
                                              // wait behind it
    BatchSettings set;
};

struct Completed {
    long long id = -1;
    double energy = 0.0;
    double parts[8] = {0};
    double dipole[3] = {0};
    std::vector<double> gradient, charges;
    int iterations = 0, converged = 0, status = 0, engine = 0;   // engine: 0 pool, 1 plain
    double t_submit = 0.0, t_start = 0.0, t_done = 0.0;           // seconds since server start
    int nao = 0;
    double sytrd_ms = 0.0;   // plain engine: device time of the tridiagonalisations
    std::string error;
};

class Server {
public:
    explicit Server(const ServeConfig& cfg);
    ~Server();   // finishes the work in flight, then stops
    // Queue one single point; returns its id.  The molecule is set up on the host here.
    long long submit(int nat, const int* Z, const double* xyz, double charge, int uhf, int want_grad,
                     std::string& err);
    // Wait for a result (timeout in seconds, < 0: forever); false on timeout.
    bool wait(long long id, Completed& out, double timeout);
    double now() const;
    // [0] completed, [1] on the plain engine, [2] pool steps, [3] pool busy seconds,
    // [4] peak resident molecules, [5] requests re-run on the plain engine, [6] host->device
    // bytes, [7] device->host bytes, [8] kernel launches, [9] pool SCC-kernel device ms,
    // [10] FP64 flops of the pool's SCC iterations (algorithmic count)
    std::vector<double> stats() const;
    // Test hook, host side only: the next n admissions to the resident pool fail as if the
    // device had run out of memory; each such request completes with an error and the pool
    // keeps serving the others.
    void inject_admission_failures(int n);

private:
    struct Req {
        long long id;
        HostMol hm;
        int want_grad;
        double t_submit, t_start;
    };
    void pool_loop();
    void pool_body();
    void plain_loop();
    void complete(Completed&& c);

    ServeConfig cfg_;
    std::chrono::steady_clock::time_point t0_;
    mutable std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<std::unique_ptr<Req>> small_q_, large_q_;
    std::multiset<int> running_nao_;   // AO counts of the requests on the plain workers
    std::map<long long, Completed> done_;
    long long next_id_ = 0;
    bool stop_ = false, pool_done_ = false;
    int inflight_ = 0;
    int inject_admissions_ = 0;
    double n_done_ = 0, n_plain_ = 0, n_steps_ = 0, busy_ = 0, peak_ = 0, n_rerun_ = 0;
    double h2d_ = 0, d2h_ = 0, launches_ = 0, scc_ms_ = 0, scc_flops_ = 0;
    long long pool_h2d_seen_ = 0;
    std::string pool_error_;
    std::vector<Completed> failed_resident_;
    std::thread pool_thread_;
    std::vector<std::thread> plain_threads_;
};

}  // namespace xg
