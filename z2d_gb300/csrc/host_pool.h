// host_pool.h -- a process-wide pool of host threads for the data-parallel
// parts of a call's host work (per-command validation and descriptor
// preparation, staging copies of large arrays).
//
// run(n, fn) calls fn(i) for every i in [0, n) on the workers and on the
// calling thread, and returns when every call has returned.  One run uses
// the workers at a time: a caller that finds them busy (another thread's
// run, or a run nested inside fn) does all its items itself, as does a
// process forked after the workers started (the child has no workers).
#pragma once
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace z2dg {

class HostPool {
  public:
    // Never destroyed: detached workers may still be waiting at exit.
    static HostPool &get() {
        static HostPool *p = new HostPool();
        return *p;
    }
    size_t threads() const { return n_workers_ + 1; }

    void run(size_t n, const std::function<void(size_t)> &fn) {
        if (n == 0) return;
        std::unique_lock<std::mutex> busy(run_mu_, std::defer_lock);
        if (n == 1 || n_workers_ == 0 || getpid() != pid_ || !busy.try_lock()) {
            for (size_t i = 0; i < n; i++) fn(i);
            return;
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            fn_ = &fn;
            n_ = n;
            next_.store(0);
            gen_++;
        }
        cv_.notify_all();
        for (size_t i; (i = next_.fetch_add(1)) < n;) fn(i);
        // every item is claimed; wait for the workers still running theirs.
        // Workers that wake later find fn_ cleared and go back to sleep.
        std::unique_lock<std::mutex> lk(mu_);
        done_cv_.wait(lk, [&] { return in_run_ == 0; });
        fn_ = nullptr;
    }

  private:
    HostPool() : pid_(getpid()) {
        const unsigned hc = std::max(1u, std::thread::hardware_concurrency());
        const unsigned nw = std::min(hc, 16u) - 1;
        for (unsigned t = 0; t < nw; t++) std::thread([this] { loop(); }).detach();
        n_workers_ = nw;
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            const std::function<void(size_t)> *fn;
            size_t n;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
                fn = fn_;
                n = n_;
                if (!fn) continue;
                in_run_++;
            }
            for (size_t i; (i = next_.fetch_add(1)) < n;) (*fn)(i);
            std::lock_guard<std::mutex> lk(mu_);
            if (--in_run_ == 0) done_cv_.notify_one();
        }
    }

    const pid_t pid_;
    size_t n_workers_ = 0;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(size_t)> *fn_ = nullptr;
    size_t n_ = 0;
    std::atomic<size_t> next_{0};
    size_t in_run_ = 0;  // workers inside the current run
    uint64_t gen_ = 0;
};

// memcpy split over the pool in 1 MiB pieces when it is large.
inline void pool_copy(void *dst, const void *src, size_t bytes) {
    constexpr size_t kPiece = (size_t)1 << 20;
    if (bytes < 2 * kPiece) {
        if (bytes) std::memcpy(dst, src, bytes);
        return;
    }
    const size_t n = (bytes + kPiece - 1) / kPiece;
    HostPool::get().run(n, [&](size_t i) {
        const size_t a = i * kPiece, b = std::min(bytes, a + kPiece);
        std::memcpy(static_cast<uint8_t *>(dst) + a, static_cast<const uint8_t *>(src) + a, b - a);
    });
}

}  // namespace z2dg
