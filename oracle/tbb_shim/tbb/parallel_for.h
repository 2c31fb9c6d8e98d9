// Stand-in for tbb::parallel_for(range, body): splits the range into one
// contiguous chunk per OpenMP thread and calls body on each chunk.  The
// reference's bodies are independent per element, so the result does not
// depend on the split.  Oracle build only.
#pragma once
#include <omp.h>
#include "blocked_range.h"
namespace tbb {
template <typename T, typename Body> void parallel_for(const blocked_range<T> &r, const Body &body) {
    const long n = (long)(r.end() - r.begin());
    if (n <= 0) return;
#pragma omp parallel
    {
        const long nt = omp_get_num_threads(), id = omp_get_thread_num();
        const long lo = n * id / nt, hi = n * (id + 1) / nt;
        if (hi > lo) body(blocked_range<T>(r.begin() + (T)lo, r.begin() + (T)hi));
    }
}
}
