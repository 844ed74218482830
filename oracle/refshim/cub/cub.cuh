/* Host shim: stand-in for CUB's BlockReduce, used by the reference's
 * shapeMatchingAlphaOne (brasstower/kernel/shapematching.cuh:17-62).
 *
 * The block runs as an OpenMP team (one OpenMP thread per CUDA thread), so
 * Sum() publishes each thread's value in the shared TempStorage, thread 0
 * adds them in thread order, and barriers on both sides keep back-to-back
 * calls on the same storage race-free.  Like CUB, only thread 0 receives the
 * aggregate.  Summation order differs from CUB's warp tree, so results agree
 * with a GPU build to rounding only. */
#pragma once
#include <omp.h>

namespace cub {
template <class T, int BLOCK_THREADS>
struct BlockReduce {
    struct TempStorage { T vals[BLOCK_THREADS]; T total; };
    TempStorage &s;
    explicit BlockReduce(TempStorage &storage) : s(storage) {}
    T Sum(T v)
    {
        const int t = omp_get_thread_num();
        s.vals[t] = v;
#pragma omp barrier
        if (t == 0) {
            T acc = s.vals[0];
            for (int k = 1; k < BLOCK_THREADS; ++k) acc = acc + s.vals[k];
            s.total = acc;
        }
#pragma omp barrier
        return t == 0 ? s.total : v;
    }
};
}  // namespace cub
