// Test-only host-thread emulation of one CUDA thread block: every CUDA thread
// is an OS thread, __syncthreads() is a barrier, shared memory is a heap
// buffer.  Included by capi.cu only when CMGB_HOST_EMULATION is defined (the
// CPU test build in tests/emu); the product never defines it.
#pragma once
#include <atomic>
#include <sched.h>
#include <thread>
#include <vector>

// A generation-counting barrier that spins briefly and then yields the CPU:
// the emulated threads outnumber the cores and meet at a barrier every few
// microseconds, where a futex-based barrier spends its time in the kernel.
struct EmuBarrier {
  std::atomic<int> count{0}, gen{0};
  const int n;
  explicit EmuBarrier(int n_) : n(n_) {}
  void arrive_and_wait()
  {
    const int g = gen.load(std::memory_order_acquire);
    if (count.fetch_add(1, std::memory_order_acq_rel) + 1 == n) {
      count.store(0, std::memory_order_relaxed);
      gen.fetch_add(1, std::memory_order_release);
      return;
    }
    for (int i = 0; gen.load(std::memory_order_acquire) == g; i++)
      if (i > 64) sched_yield();
  }
};

inline thread_local EmuBarrier *cmgb_emu_bar = nullptr;
inline void cmgb_emu_sync() { cmgb_emu_bar->arrive_and_wait(); }
inline unsigned cmgb_emu_maxu(unsigned *p, unsigned v)
{
  unsigned cur = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while (cur < v && !__atomic_compare_exchange_n(p, &cur, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {}
  return cur;
}
inline long long cmgb_emu_minll(long long *p, long long v)
{
  long long cur = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while (cur > v && !__atomic_compare_exchange_n(p, &cur, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {}
  return cur;
}
inline long long cmgb_emu_maxll(long long *p, long long v)
{
  long long cur = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while (cur < v && !__atomic_compare_exchange_n(p, &cur, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {}
  return cur;
}
inline unsigned long long cmgb_emu_maxull(unsigned long long *p, unsigned long long v)
{
  unsigned long long cur = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while (cur < v && !__atomic_compare_exchange_n(p, &cur, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {}
  return cur;
}
#include <cstring>
// warp-level primitives: the 32 threads of an emulated warp meet at a
// per-warp barrier and exchange values through a slot array
struct EmuWarp {
  EmuBarrier bar{32};
  long long slot[32];
};
inline thread_local EmuWarp *cmgb_emu_warp = nullptr;
inline thread_local int cmgb_emu_lane = 0;
template <class T> inline T cmgb_shfl_up(T x, int k)
{
  EmuWarp *w = cmgb_emu_warp;
  std::memcpy(&w->slot[cmgb_emu_lane], &x, sizeof(T));
  w->bar.arrive_and_wait();
  T y = x;
  if (cmgb_emu_lane >= k) std::memcpy(&y, &w->slot[cmgb_emu_lane - k], sizeof(T));
  w->bar.arrive_and_wait();
  return y;
}
inline bool cmgb_any(bool b)
{
  EmuWarp *w = cmgb_emu_warp;
  w->slot[cmgb_emu_lane] = b ? 1 : 0;
  w->bar.arrive_and_wait();
  bool any = false;
  for (int l = 0; l < 32; l++) any = any || w->slot[l];
  w->bar.arrive_and_wait();
  return any;
}
inline void __syncwarp_portable() { cmgb_emu_warp->bar.arrive_and_wait(); }
inline int __ldg_int(const int *p) { return *p; }
// TMA / mbarrier stand-ins: the copy happens at issue; waits always succeed
inline void cmgb_mbar_init(unsigned long long *mb) { *mb = 0; }
inline void cmgb_tma_load(void *dst, const void *src, unsigned bytes, unsigned long long *) { std::memcpy(dst, src, bytes); }
inline bool cmgb_mbar_wait(unsigned long long *, unsigned) { return true; }
#define CMGB_EMU_THREADS 64
