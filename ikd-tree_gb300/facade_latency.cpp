// Per-point Nearest_Search through the drop-in facade (include/ikd_Tree_gb300.h),
// the call shape of a mapping front end that searches point by point
// (ikd_Tree.cpp:366-397, called from several threads at once, :875-884).
//
//   facade_latency <map points> <queries> <threads>
//
// Builds a uniform map in [-50, 50]^3, then runs `queries` single-point
// Nearest_Search calls (k = 5) on 1 thread and on `threads` threads, and
// prints one JSON object: microseconds per call on one thread and calls per
// second with all threads.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <thread>
#include <vector>

#include "ikd_Tree_gb300.h"

int main(int argc, char** argv) {
    const int n = argc > 1 ? std::atoi(argv[1]) : 1000000;
    const int nq = argc > 2 ? std::atoi(argv[2]) : 20000;
    const int nt = argc > 3 ? std::atoi(argv[3]) : 8;
    using Tree = KD_TREE<ikdTree_PointType>;
    std::mt19937_64 rng(1002);
    std::uniform_real_distribution<float> U(-50.f, 50.f);
    Tree::PointVector map(n), q(nq);
    for (auto& p : map) p = ikdTree_PointType(U(rng), U(rng), U(rng));
    for (auto& p : q) p = ikdTree_PointType(U(rng), U(rng), U(rng));
    Tree tree(0.5, 0.6, 0.5);
    tree.Build(map);
    auto run = [&](int lo, int hi) {
        Tree::PointVector nn;
        std::vector<float> d;
        for (int i = lo; i < hi; ++i) tree.Nearest_Search(q[i], 5, nn, d);
    };
    run(0, 200);  // warm-up: search contexts and their buffers
    auto t0 = std::chrono::steady_clock::now();
    run(0, nq);
    auto t1 = std::chrono::steady_clock::now();
    std::vector<std::thread> ts;
    for (int t = 0; t < nt; ++t) ts.emplace_back(run, (int)((long long)nq * t / nt), (int)((long long)nq * (t + 1) / nt));
    for (auto& th : ts) th.join();
    auto t2 = std::chrono::steady_clock::now();
    const double one = std::chrono::duration<double>(t1 - t0).count();
    const double all = std::chrono::duration<double>(t2 - t1).count();
    std::printf("{\"map_points\": %d, \"calls\": %d, \"k\": 5, \"us_per_call_1_thread\": %.3f, "
                "\"calls_per_s_1_thread\": %.1f, \"threads\": %d, \"calls_per_s_threads\": %.1f}\n",
                n, nq, 1e6 * one / nq, nq / one, nt, nq / all);
    return 0;
}
