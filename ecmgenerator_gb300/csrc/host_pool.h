/*
 * host_pool.h -- the host threads that run the planner calls of a tick.
 */
#ifndef ECMG_HOST_POOL_H
#define ECMG_HOST_POOL_H

#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace ecmg {

/* Host threads for the planner calls of a tick (re-plans, spawned agents):
   started once, idle on a condition variable between ticks.  run(m, fn)
   calls fn(i, w) for i in [0, m) on the calling thread (w = 0) and the
   workers (w = 1..size()), each with its own planner scratch. */
template <class Scratch>
class HostPool {
public:
    ~HostPool()
    {
        {
            std::lock_guard<std::mutex> l(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : th_) t.join();
    }
    int size() const { return (int)th_.size(); }
    std::vector<Scratch> scratch; /* [size() + 1] */
    void start(int n)
    {
        if (!th_.empty() || n < 1) return;
        scratch.resize((size_t)n + 1);
        for (int w = 1; w <= n; w++) th_.emplace_back([this, w] { loop(w); });
    }
    void run(int m, const std::function<void(int, int)>& fn)
    {
        if (th_.empty() || m < 2) {
            for (int i = 0; i < m; i++) fn(i, 0);
            return;
        }
        {
            std::lock_guard<std::mutex> l(mu_);
            job_ = &fn;
            m_ = m;
            next_ = 0;
            busy_ = (int)th_.size();
            gen_++;
        }
        cv_.notify_all();
        for (int i; (i = next_.fetch_add(1)) < m;) fn(i, 0);
        std::unique_lock<std::mutex> l(mu_);
        done_.wait(l, [this] { return busy_ == 0; });
        job_ = nullptr;
    }

private:
    void loop(int w)
    {
        unsigned seen = 0;
        for (;;) {
            const std::function<void(int, int)>* job;
            int m;
            {
                std::unique_lock<std::mutex> l(mu_);
                cv_.wait(l, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
                job = job_;
                m = m_;
            }
            for (int i; (i = next_.fetch_add(1)) < m;) (*job)(i, w);
            std::lock_guard<std::mutex> l(mu_);
            if (--busy_ == 0) done_.notify_one();
        }
    }
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    const std::function<void(int, int)>* job_ = nullptr;
    int m_ = 0, busy_ = 0;
    unsigned gen_ = 0;
    std::atomic<int> next_{0};
    bool stop_ = false;
};

}  // namespace ecmg

#endif
