// fbk_workers.cpp — the host thread pool behind host_parallel_for.
#include "fbk_workers.h"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>

namespace fbk {

namespace {

class Pool {
  public:
    Pool() {
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const unsigned n = std::min(8u, hw) - 1;  // the caller is the last thread
        for (unsigned i = 0; i < n; ++i) std::thread([this, i] { loop(i + 1); }).detach();
        n_threads_ = n + 1;
    }
    unsigned threads() const { return n_threads_; }

    void run(uint64_t n, const std::function<void(uint64_t, unsigned)>& fn) {
        if (n == 0) return;
        std::lock_guard<std::mutex> one_at_a_time(run_mu_);
        if (n == 1 || n_threads_ == 1) {
            for (uint64_t i = 0; i < n; ++i) fn(i, 0);
            return;
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            fn_ = &fn;
            n_ = n;
            next_.store(0);
            busy_ = n_threads_ - 1;
            ++gen_;
        }
        cv_.notify_all();
        drain(0);
        std::unique_lock<std::mutex> lk(mu_);
        done_cv_.wait(lk, [this] { return busy_ == 0; });
        fn_ = nullptr;
    }

  private:
    void drain(unsigned t) {
        for (uint64_t i; (i = next_.fetch_add(1)) < n_;) (*fn_)(i, t);
    }
    void loop(unsigned t) {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
            }
            drain(t);
            std::lock_guard<std::mutex> lk(mu_);
            if (--busy_ == 0) done_cv_.notify_all();
        }
    }

    unsigned n_threads_ = 1;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(uint64_t, unsigned)>* fn_ = nullptr;
    uint64_t n_ = 0, gen_ = 0;
    unsigned busy_ = 0;
    std::atomic<uint64_t> next_{0};
};

Pool& pool() {
    static Pool* p = new Pool();  // never destroyed: its threads are detached and idle at exit
    return *p;
}

}  // namespace

void host_parallel_for(uint64_t n, const std::function<void(uint64_t, unsigned)>& fn) { pool().run(n, fn); }

unsigned host_threads() { return pool().threads(); }

}  // namespace fbk
