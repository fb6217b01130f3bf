// Stress test of ecmg::HostPool (the planner threads of a tick): runs of 1 to
// 40 jobs from three caller threads, one run at a time (the library
// serialises its callers with a mutex).  Every job of a run must execute
// exactly once, on a distinct scratch per thread, and every run must return.
#include "host_pool.h"

#include <chrono>
#include <cstdio>
#include <random>

struct Scratch {
    long uses = 0;
};

int main()
{
    ecmg::HostPool<Scratch> pool;
    pool.start(15);
    std::mutex callers;
    std::atomic<long> runs{0}, bad{0};
    auto user = [&](unsigned seed) {
        std::mt19937 rng(seed);
        for (int it = 0; it < 4000; it++) {
            const int m = 1 + (int)(rng() % 40);
            std::vector<std::atomic<int>> hit(m);
            for (auto& h : hit) h = 0;
            std::lock_guard<std::mutex> l(callers);
            pool.run(m, [&](int i, int w) {
                hit[i]++;
                pool.scratch[w].uses++;
            });
            for (auto& h : hit)
                if (h.load() != 1) bad++;
            runs++;
        }
    };
    const auto t0 = std::chrono::steady_clock::now();
    std::thread a(user, 1u), b(user, 2u), c(user, 3u);
    a.join();
    b.join();
    c.join();
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("runs %ld, jobs not run exactly once %ld, %.2f s\n", runs.load(), bad.load(), s);
    return bad.load() == 0 && runs.load() == 12000 ? 0 : 1;
}
