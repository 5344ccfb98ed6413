// Serving loop: see ef_server.hpp.
#include "ef_server.hpp"

#include <stdexcept>

namespace efgb {

namespace {
void sck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}
}  // namespace

Server::Server(const std::vector<TreeSpec>& trees, int lanes_per_tree, long long hbm_budget, int sweeps) {
    if (trees.empty()) throw std::invalid_argument("server: no trees");
    if (lanes_per_tree < 1 || lanes_per_tree > 8) throw std::invalid_argument("server: lanes per tree must be in [1, 8]");
    if (sweeps < 0 || sweeps + 1 > MixedSolver::kMaxPasses) throw std::invalid_argument("server: sweeps out of range");
    trees_ = std::vector<Tree>(trees.size());  // built in place: Tree is not nothrow-movable
    try {
        // first lane of every tree (holds the tree's FP32 operators), then further lanes round-robin
        // while the budget allows
        for (size_t t = 0; t < trees.size(); ++t) {
            if (!trees[t].hps || (!trees[t].hps->built() && !trees[t].hps->built32()))
                throw std::invalid_argument("server: tree not built");
            trees_[t].hps = trees[t].hps;
            trees_[t].bmax = trees[t].bmax;
            trees_[t].sweeps.store(sweeps);
            Lane l;
            l.ms = std::make_unique<MixedSolver>(*trees[t].hps, trees[t].bmax);
            bytes_ += (long long)l.ms->device_bytes();
            trees_[t].lanes.push_back(std::move(l));
        }
        for (int k = 1; k < lanes_per_tree; ++k)
            for (size_t t = 0; t < trees.size(); ++t) {
                auto ms = std::make_unique<MixedSolver>(*trees[t].hps, trees[t].bmax, trees_[t].lanes[0].ms.get());
                if (hbm_budget > 0 && bytes_ + (long long)ms->device_bytes() > hbm_budget) continue;
                bytes_ += (long long)ms->device_bytes();
                Lane l;
                l.ms = std::move(ms);
                trees_[t].lanes.push_back(std::move(l));
            }
        for (auto& t : trees_)
            for (auto& l : t.lanes) {
                sck(cudaStreamCreateWithFlags(&l.st, cudaStreamNonBlocking), "server stream");
                sck(cudaEventCreateWithFlags(&l.done, cudaEventDisableTiming), "server event");
                l.ms->set_stream(l.st);
            }
    } catch (...) {
        for (auto& t : trees_)
            for (auto& l : t.lanes) {
                if (l.done) cudaEventDestroy(l.done);
                if (l.st) cudaStreamDestroy(l.st);
            }
        throw;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    worker_ = std::thread([this, dev] {
        cudaSetDevice(dev);
        loop();
    });
}

Server::~Server() {
    {
        std::lock_guard<std::mutex> g(mu_);
        stop_ = true;
    }
    cv_work_.notify_all();
    if (worker_.joinable()) worker_.join();
    for (auto& t : trees_)
        for (auto& l : t.lanes) {
            if (l.st) cudaStreamSynchronize(l.st);
            if (l.done) cudaEventDestroy(l.done);
            if (l.st) cudaStreamDestroy(l.st);
        }
    // lanes that share operators go before the lane that owns them
    for (auto& t : trees_)
        while (!t.lanes.empty()) t.lanes.pop_back();
}

long long Server::submit(int tree, const double* f, const double* a, const double* r, double* u) {
    if (tree < 0 || tree >= int(trees_.size())) throw std::invalid_argument("server: tree index out of range");
    if (!f || !a || !r || !u) throw std::invalid_argument("server: null request array");
    long long id;
    {
        std::lock_guard<std::mutex> g(mu_);
        if (!error_.empty()) throw std::runtime_error(error_);
        id = next_id_++;
        trees_[tree].queue.push_back(Req{id, f, a, r, u, Clock::now()});
        pending_[id] = tree;
        ++stats_.submitted;
    }
    cv_work_.notify_one();
    return id;
}

int Server::poll(long long id, double* latency) {
    std::lock_guard<std::mutex> g(mu_);
    auto it = done_.find(id);
    if (it != done_.end()) {
        if (latency) *latency = it->second;
        done_.erase(it);
        return 1;
    }
    if (!error_.empty()) throw std::runtime_error(error_);
    if (!pending_.count(id)) throw std::invalid_argument("server: unknown request id");
    return 0;
}

int Server::wait(long long id, double timeout, double* latency) {
    std::unique_lock<std::mutex> g(mu_);
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout));
    for (;;) {
        auto it = done_.find(id);
        if (it != done_.end()) {
            if (latency) *latency = it->second;
            done_.erase(it);
            return 1;
        }
        if (!error_.empty()) throw std::runtime_error(error_);
        if (!pending_.count(id)) throw std::invalid_argument("server: unknown request id");
        if (cv_done_.wait_until(g, until) == std::cv_status::timeout && !done_.count(id)) return 0;
    }
}

void Server::set_sweeps(int tree, int sweeps) {
    if (tree < 0 || tree >= int(trees_.size())) throw std::invalid_argument("server: tree index out of range");
    if (sweeps < 0 || sweeps + 1 > MixedSolver::kMaxPasses) throw std::invalid_argument("server: sweeps out of range");
    trees_[tree].sweeps.store(sweeps);
}

void Server::set_root_operator(int tree, const double* a, const double* b) {
    if (tree < 0 || tree >= int(trees_.size())) throw std::invalid_argument("server: tree index out of range");
    if (!a || !b) throw std::invalid_argument("server: null root operator");
    Tree& t = trees_[tree];
    const size_t m = 4 * size_t(t.hps->root_M());
    std::unique_lock<std::mutex> g(mu_);
    for (const auto& kv : pending_)
        if (kv.second == tree) throw std::invalid_argument("server: the tree has requests in flight");
    t.root_a.assign(a, a + m);
    t.root_b.assign(b, b + m);
    t.root_pending = true;
    cv_work_.notify_all();
    cv_done_.wait(g, [&] { return !t.root_pending || !error_.empty(); });
    if (!error_.empty()) throw std::runtime_error(error_);
}

Server::Stats Server::stats() {
    std::lock_guard<std::mutex> g(mu_);
    return stats_;
}

void Server::launch(Tree& t, Lane& l) {
    MixedSolver& X = *l.ms;
    const size_t cells = size_t(t.hps->num_leaves()) * t.hps->leaf_n() * t.hps->leaf_n();
    const size_t m = 4 * size_t(t.hps->root_M());
    const int B = int(l.batch.size());
    for (int b = 0; b < B; ++b) {
        const Req& q = l.batch[b];
        sck(cudaMemcpyAsync(X.f() + b * cells, q.f, cells * 8, cudaMemcpyHostToDevice, l.st), "server copy f");
        sck(cudaMemcpyAsync(X.a() + b * m, q.a, m * 8, cudaMemcpyHostToDevice, l.st), "server copy a");
        sck(cudaMemcpyAsync(X.r() + b * m, q.r, m * 8, cudaMemcpyHostToDevice, l.st), "server copy r");
    }
    X.solve(B, t.sweeps.load());
    sck(cudaGetLastError(), "server block solve");
    for (int b = 0; b < B; ++b)
        sck(cudaMemcpyAsync(l.batch[b].u, X.u() + b * cells, cells * 8, cudaMemcpyDeviceToHost, l.st), "server copy u");
    sck(cudaEventRecord(l.done, l.st), "server event");
    l.busy = true;
}

void Server::loop() {
    for (;;) {
        bool progress = false, busy = false;
        try {
            // completions
            for (auto& t : trees_)
                for (auto& l : t.lanes) {
                    if (!l.busy) continue;
                    const cudaError_t e = cudaEventQuery(l.done);
                    if (e == cudaErrorNotReady) { busy = true; continue; }
                    sck(e, "server block");
                    int err = l.ms->take_error();
                    if (err) throw std::runtime_error("server: an operator tile copy did not complete");
                    const auto now = Clock::now();
                    {
                        std::lock_guard<std::mutex> g(mu_);
                        for (const Req& q : l.batch) {
                            done_[q.id] = std::chrono::duration<double>(now - q.t0).count();
                            pending_.erase(q.id);
                        }
                        stats_.completed += (long long)l.batch.size();
                    }
                    cv_done_.notify_all();
                    l.batch.clear();
                    l.busy = false;
                    progress = true;
                }
            // root operators waiting for their tree's lanes to be idle
            for (auto& t : trees_) {
                bool pend;
                {
                    std::lock_guard<std::mutex> g(mu_);
                    pend = t.root_pending;
                }
                if (!pend) continue;
                bool idle = true;
                for (auto& l : t.lanes) idle = idle && !l.busy;
                if (!idle) continue;
                for (auto& l : t.lanes) l.ms->set_root_operator(t.root_a.data(), t.root_b.data());
                {
                    std::lock_guard<std::mutex> g(mu_);
                    t.root_pending = false;
                }
                cv_done_.notify_all();
                progress = true;
            }
            // new blocks on free lanes: every request that has arrived, up to bmax
            for (auto& t : trees_)
                for (auto& l : t.lanes) {
                    if (l.busy) continue;
                    {
                        std::lock_guard<std::mutex> g(mu_);
                        while (!t.queue.empty() && int(l.batch.size()) < t.bmax) {
                            l.batch.push_back(t.queue.front());
                            t.queue.pop_front();
                        }
                        if (!l.batch.empty()) {
                            ++stats_.batches;
                            if ((long long)l.batch.size() > stats_.max_batch) stats_.max_batch = (long long)l.batch.size();
                        }
                    }
                    if (l.batch.empty()) continue;
                    launch(t, l);
                    busy = true;
                    progress = true;
                }
        } catch (const std::exception& ex) {
            std::lock_guard<std::mutex> g(mu_);
            error_ = ex.what();
            cv_done_.notify_all();
            return;
        }
        std::unique_lock<std::mutex> g(mu_);
        bool queued = false;
        for (auto& t : trees_)
            if (!t.queue.empty()) queued = true;
        if (stop_ && !busy && !queued) return;
        if (progress) continue;
        if (busy) {
            // blocks in flight: poll their events again shortly
            cv_work_.wait_for(g, std::chrono::microseconds(20));
        } else if (!queued) {
            cv_work_.wait_for(g, std::chrono::milliseconds(5));
        }
    }
}

}  // namespace efgb
