// Host-side parallel loop over a persistent pool of threads.  Used by the
// work-list compilers (enlarged-block builds, sigma plans), whose loops over
// operators are independent and each write their own output slot.
#pragma once
#include <functional>

namespace bgpu {

// Number of pool threads (hardware concurrency, at most 32; the environment
// variable BGPU_HOST_THREADS overrides).
int host_threads();

// Runs fn(i) for every i in [0, n) with a dynamic schedule and returns when
// all calls have finished.  The first exception thrown by fn is rethrown in
// the caller.  Calls made from inside a pool thread run serially.
void parallel_for(int n, const std::function<void(int)>& fn);

}  // namespace bgpu
