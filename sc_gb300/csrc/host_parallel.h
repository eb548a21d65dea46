// host_parallel.h -- host loops over particle records, split across threads.
//
// Moving a 65,536-particle state between the caller's records, the host copy and the pinned
// staging block is four passes of about 16 MB each (sc_set_particles, the upload's packing,
// the download's unpacking, sc_get_particles); one core streams them in milliseconds, as long
// as a device sweep of the same system.  parallelRange splits [0, n) into contiguous chunks,
// one per thread, so that the passes run at the host's memory bandwidth instead.  Every index
// is visited exactly once and each chunk writes only its own records, so the result does not
// depend on the number of threads.  Small ranges stay on the calling thread, and when a thread
// cannot be started its chunk runs on the calling thread as well.
#pragma once

#include <algorithm>
#include <thread>
#include <vector>

namespace scg {

// Records per thread below which a range is not split (a thread start costs ~10-20 us).
constexpr int kHostChunkMin = 8192;
// At most this many threads per loop: the passes are bandwidth-bound, and more threads than
// a few memory channels' worth only add start-up time.
constexpr int kHostThreadsMax = 8;

inline int hostThreads(int n) {
    const unsigned hw = std::thread::hardware_concurrency();
    const int byWork = (n + kHostChunkMin - 1) / kHostChunkMin;
    return std::max(1, std::min({(int)(hw ? hw : 1u), kHostThreadsMax, byWork}));
}

// Calls body(lo, hi) on disjoint chunks that cover [0, n) and returns when all have run.
template <class Body>
void parallelRange(int n, const Body& body) {
    if (n <= 0) return;
    const int nt = hostThreads(n);
    if (nt <= 1) {
        body(0, n);
        return;
    }
    const int chunk = (n + nt - 1) / nt;
    std::vector<std::thread> pool;
    int next = 1;                          // chunk 0 runs on the calling thread
    try {
        pool.reserve(nt - 1);
        for (; next < nt; ++next) {
            const int lo = next * chunk, hi = std::min(n, lo + chunk);
            if (lo >= hi) break;
            pool.emplace_back([&body, lo, hi] { body(lo, hi); });
        }
    } catch (...) {
        // no thread could be started for chunk `next`: it and the rest run below
    }
    body(0, std::min(n, chunk));
    for (int c = next; c < nt; ++c) {
        const int lo = c * chunk, hi = std::min(n, lo + chunk);
        if (lo < hi) body(lo, hi);
    }
    for (auto& t : pool) t.join();
}

}  // namespace scg
