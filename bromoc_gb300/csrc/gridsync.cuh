// Bounded inter-block synchronisation for cooperative launches.  Every wait
// gives up after kWaitSpins polls, or as soon as another block has given up;
// it then records kErrBarrier in the device state and returns false, so the
// launch ends and the host reads the error instead of a hung context.
#pragma once
#include <cuda/atomic>
#include "common.cuh"

namespace bgpu {

constexpr int kWaitSpins = 1 << 23;  // ~0.5-1 s of polling at most

// Thread 0 of a block: poll until *ctr >= target (acquire ordering), at
// most `limit` polls.
__device__ __forceinline__ bool wait_at_least(unsigned *ctr, unsigned target, DevState *st,
                                              bool sleep = true, int limit = kWaitSpins) {
  cuda::atomic_ref<unsigned, cuda::thread_scope_device> a(*ctr);
  volatile int *err = &st->err;
  for (int spin = 0; a.load(cuda::memory_order_acquire) < target; ++spin) {
    if (spin > limit || ((spin & 1023) == 1023 && (*err & kErrBarrier))) {
      atomicOr(&st->err, kErrBarrier);
      return false;
    }
    if (sleep) __nanosleep(32);
  }
  return true;
}

__device__ __forceinline__ void release_add(unsigned *ctr, unsigned v) {
  cuda::atomic_ref<unsigned, cuda::thread_scope_device> a(*ctr);
  a.fetch_add(v, cuda::memory_order_release);
}

// Block-wide: thread 0 waits (polling without sleeps: the waits of GRAND's
// rounds are a few microseconds, and a sleep's wake-up adds to each),
// everyone learns the outcome.
__device__ __forceinline__ bool block_wait(unsigned *ctr, unsigned target, DevState *st,
                                           int *flag) {
  if (threadIdx.x == 0) *flag = wait_at_least(ctr, target, st, false) ? 1 : 0;
  __syncthreads();
  const bool ok = *flag != 0;
  __syncthreads();
  return ok;
}

// Grid-wide barrier number k (1, 2, ...) on a counter that starts the launch
// at zero: each block arrives once, then waits for k * gridDim.x arrivals.
// The block's writes before the barrier reach every block after it through
// the barrier's own ordering: __syncthreads, thread 0's release increment,
// the other block's acquire load that sees it, its __syncthreads (the PTX
// memory model composes these into happens-before; no full fence is
// needed, and two of them cost ~9 us over a 10-step loop).  *flag: one
// shared int of the block.
__device__ __forceinline__ bool grid_barrier(unsigned *ctr, unsigned k, DevState *st,
                                             int *flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    release_add(ctr, 1u);
    *flag = wait_at_least(ctr, k * gridDim.x, st, false) ? 1 : 0;
  }
  __syncthreads();
  // thread 0 rewrites *flag only after the next barrier's first
  // __syncthreads, which every thread reaches after this read
  return *flag != 0;
}

// End of a cooperative launch that used the counters (every block, every
// thread; also after a wait that gave up): the last block out clears them
// for the next launch on the stream, so no reset runs between launches.
// By then every other block has passed its last wait.
__device__ __forceinline__ void launch_exit(DevState *st) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> x(st->bar_exit);
    if (x.fetch_add(1u, cuda::memory_order_acq_rel) == gridDim.x - 1) {
      cuda::atomic_ref<unsigned, cuda::thread_scope_device>(st->bar_count)
          .store(0u, cuda::memory_order_relaxed);
      cuda::atomic_ref<unsigned, cuda::thread_scope_device>(st->bar_gen)
          .store(0u, cuda::memory_order_relaxed);
      x.store(0u, cuda::memory_order_relaxed);
    }
  }
}

}  // namespace bgpu
