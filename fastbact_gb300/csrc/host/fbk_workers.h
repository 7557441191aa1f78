// fbk_workers.h — a process-wide pool of host threads for the library's parallel
// host loops (read-bank scans, staged host<->device copies).
#pragma once
#include <cstdint>
#include <functional>

namespace fbk {

// Calls fn(i, t) for every i in [0, n) on the pool and returns when all calls have
// returned; t in [0, host_threads()) names the thread making the call (0 = the
// caller), so per-thread partial results need no locks.  Calls from several threads
// run one after another.
void host_parallel_for(uint64_t n, const std::function<void(uint64_t, unsigned)>& fn);

// Threads that take part in host_parallel_for, the caller included.
unsigned host_threads();

}  // namespace fbk
