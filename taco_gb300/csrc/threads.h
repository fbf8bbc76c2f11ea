// Host helper threads of the library (page mapping, host index checks, file parsing).
#pragma once

#include <pthread.h>
#include <sched.h>
#include <unistd.h>

namespace tacogb {

// Lets a helper thread run on any online CPU.  Threads inherit the affinity of the thread that
// starts them, and a caller bound to one core (OpenMP's OMP_PROC_BIND binds the initial thread)
// would otherwise crowd every helper onto that core.  The kernel still keeps the thread within
// the process's cpuset; a refusal leaves the inherited affinity.
inline void spread_thread() {
  const long n = sysconf(_SC_NPROCESSORS_ONLN);
  if (n <= 0) return;
  cpu_set_t set;
  CPU_ZERO(&set);
  for (long c = 0; c < n && c < CPU_SETSIZE; c++) CPU_SET((int)c, &set);
  pthread_setaffinity_np(pthread_self(), sizeof(set), &set);
}

}  // namespace tacogb
