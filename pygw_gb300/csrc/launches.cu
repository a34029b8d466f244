// Host-side count of the kernels this library has enqueued (all entry points).
#include <atomic>
#include "launches.h"

static std::atomic<unsigned long long> g_launches{0};

void pg_count_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

extern "C" unsigned long long pg_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }
