// Test-only host-thread emulation of one CUDA thread block: every CUDA thread
// is an OS thread, __syncthreads() is a std::barrier, shared memory is a
// heap buffer.  Included by capi.cu only when CMGB_HOST_EMULATION is defined
// (the CPU test build in tests/emu); the product never defines it.
#pragma once
#include <barrier>
#include <thread>
#include <vector>

inline thread_local std::barrier<> *cmgb_emu_bar = nullptr;
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
#define CMGB_EMU_THREADS 64
