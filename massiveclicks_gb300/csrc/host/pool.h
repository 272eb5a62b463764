// A persistent pool of host threads for the library's parallel host loops
// (tiling, log parsing).  Starting a std::thread costs tens of microseconds;
// an upload that spawned one per core spent about half a millisecond on it.
#ifndef MCLICKS_POOL_H
#define MCLICKS_POOL_H

#include <cstddef>
#include <functional>

namespace mch {

// Runs fn(i) for every i in [0, n), on the pool's threads and the calling
// thread, and returns when all calls have returned.  Calls from several
// threads run one after another.  fn must not call parallel_for itself.
void parallel_for(size_t n, const std::function<void(size_t)>& fn);

// Threads that take part in parallel_for (the pool's plus the caller).
size_t pool_threads();

}  // namespace mch

#endif
