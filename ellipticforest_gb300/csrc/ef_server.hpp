// Serving loop over several factored trees resident in HBM (no counterpart in the reference).
//
// Requests (tree, load f, root data a u = r) are queued per tree.  Every tree has one or more
// lanes: a mixed-precision block solver of up to bmax requests with its own CUDA stream.  A
// scheduler thread keeps every lane busy: when a lane is free it takes every request of its tree
// that has arrived so far (up to bmax), stages their inputs, launches one block solve and the copies
// of the results back, and records an event; completions are detected by polling the events.  So
// requests that arrive while a block is on the GPU join the next block of a free lane (continuous
// batching), blocks of different trees and lanes overlap on the device, and lanes are only created
// while their device memory fits the HBM budget given at creation (admission by memory).  A
// request's result does not depend on the other requests of its block (the block kernels work on
// each request's data independently in a fixed order).
#pragma once

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ef_hps.hpp"

namespace efgb {

class Server {
public:
    struct TreeSpec {
        Hps* hps;
        int bmax;
    };
    struct Stats {
        long long submitted = 0, completed = 0, batches = 0, max_batch = 0;
    };

    // lanes_per_tree lanes are created per tree while the total device memory of all lanes stays
    // within hbm_budget bytes (<= 0: no limit); every tree gets at least one lane.
    Server(const std::vector<TreeSpec>& trees, int lanes_per_tree, long long hbm_budget, int sweeps);
    ~Server();
    Server(const Server&) = delete;
    Server& operator=(const Server&) = delete;

    // Queues one request; f (leaves*n*n), a and r (4M) and u (leaves*n*n) are host arrays that must
    // stay valid until the request completes (page-locked memory lets the copies run async).
    long long submit(int tree, const double* f, const double* a, const double* r, double* u);
    // 1 when done (latency: seconds from submit to the result in u), 0 while pending;
    // throws on an unknown id or when the scheduler failed.
    int poll(long long id, double* latency);
    // waits up to timeout seconds; returns 1 when done, 0 on time-out
    int wait(long long id, double timeout, double* latency);
    Stats stats();
    // refinement sweeps of the tree's later blocks (the creation value until set)
    void set_sweeps(int tree, int sweeps);
    // Root operator a u + b du/dn = r (a, b: 4M host arrays) of every lane of the tree, for the
    // requests submitted from now on (their own `a` is then not read while b != 0); b == 0 returns to
    // per-request Dirichlet data.  The tree must have no request in flight; applied by the
    // scheduler thread between blocks, and this call returns once it is in place.
    void set_root_operator(int tree, const double* a, const double* b);
    int lanes(int tree) const { return int(trees_.at(tree).lanes.size()); }
    long long device_bytes() const { return bytes_; }

private:
    using Clock = std::chrono::steady_clock;
    struct Req {
        long long id;
        const double *f, *a, *r;
        double* u;
        Clock::time_point t0;
    };
    struct Lane {
        std::unique_ptr<MixedSolver> ms;
        cudaStream_t st = nullptr;
        cudaEvent_t done = nullptr;
        std::vector<Req> batch;
        bool busy = false;
    };
    struct Tree {
        Hps* hps = nullptr;
        int bmax = 1;
        std::atomic<int> sweeps{1};
        std::vector<Lane> lanes;
        std::deque<Req> queue;
        std::vector<double> root_a, root_b;  // a root operator waiting for the scheduler
        bool root_pending = false;
    };

    void loop();
    void launch(Tree& t, Lane& l);

    std::vector<Tree> trees_;
    long long bytes_ = 0;
    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::unordered_map<long long, double> done_;  // id -> latency (s); erased when read
    std::unordered_map<long long, int> pending_;  // id -> tree
    Stats stats_;
    long long next_id_ = 1;
    bool stop_ = false;
    std::string error_;
    std::thread worker_;
};

}  // namespace efgb
