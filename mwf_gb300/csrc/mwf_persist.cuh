// Persistent FP32 time step (sm_103a): the three passes of every run whose passes all have a
// batched form (mwf_xbatch.cuh, mwf_zbatch.cuh) in one launch.
//
// The CTAs of the launch stay resident and take work items one at a time from a ticket counter
// over one list that holds every x-forward, z and x-inverse item of the step.  A z item of a run
// may start once all of the run's x-forward items are done, an x-inverse item once all of its z
// items are done; the host orders the list so that an item's prerequisites always hold lower
// tickets.  Tickets are only taken by CTAs that are running, so every prerequisite of a waiting
// item belongs to a running CTA or is finished: the waits always end.  The host lists the items
// as a three-stage pipeline over groups of runs (the x forward of group g beside the z pass of
// group g-1 and the x inverse of group g-2), so items of different passes share the SMs and a
// group's x-transformed fields are still in L2 when its z items read them.
//
// Counters (device memory, cleared before every launch): [0] ticket; per run r, [1 + 2r] its
// x-forward items done and [2 + 2r] its z items done.  When an item is finished the CTA
// synchronises and thread 0 counts it with a release reduction, which orders every write of the
// CTA before the count; a waiting item's thread 0 reads the counter with acquire semantics, then
// the CTA synchronises (x-inverse items have no consumer in the launch and are not counted).  A
// CTA takes its next ticket while it works on the current item; the lowest ticket that is taken
// and not finished is then always one a CTA is working on, whose prerequisites are all lower.  Every wait gives up after about a second (the step takes milliseconds): it
// then sets MWF_DERR_WAIT_TIMEOUT, skips the item's work and counts it as done, and later waits
// see the flag and do not wait again, so the launch always ends.
#pragma once
#include "mwf_kernels.cuh"
#include "mwf_zbatch.cuh"
#include "mwf_xbatch.cuh"

namespace mwf {

// PersistItem (mwf_common.cuh): code = kind << 8 | size index of MM (x passes) or NN (z pass)
enum { kPxForward = 0, kPzM4 = 1, kPzM6 = 2, kPxInverse = 3 };

__device__ __forceinline__ void red_release_add(int* p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Thread 0 of a CTA: wait until *counter >= target; false if the wait gave up (or an earlier
// wait of the launch did).
__device__ __forceinline__ bool wait_count(const int* counter, int target, int* err) {
  if (ld_acquire(counter) >= target) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (ld_acquire(counter) >= target) return true;
    if (ld_acquire(err) & MWF_DERR_WAIT_TIMEOUT) return false;
    if (global_ns() - t0 > kMbarWaitNs) {
      atomicOr(err, MWF_DERR_WAIT_TIMEOUT);
      return false;
    }
    __nanosleep(256);
  }
}

template <int NT>
__global__ void __launch_bounds__(NT, 2) persistent_step_kernel(const RunDesc* __restrict__ runs,
                                                                const PersistItem* __restrict__ items, int n_items,
                                                                int* counters, int* err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item, s_ok;
  const unsigned smem_bytes = dyn_smem_bytes();
  int next = 0;
  if (threadIdx.x == 0) next = atomicAdd(&counters[0], 1);
  for (;;) {
    if (threadIdx.x == 0) s_item = next;
    __syncthreads();
    const int i = s_item;
    if (i >= n_items) break;
    if (threadIdx.x == 0) next = atomicAdd(&counters[0], 1);    // fetched while this item runs
    const PersistItem it = items[i];
    const int kind = it.code >> 8;
    const RunDesc& R = runs[it.run];
    if (threadIdx.x == 0) {
      bool ok = true;
      if (kind == kPzM4 || kind == kPzM6) ok = wait_count(&counters[1 + 2 * it.run], R.xbf_items, err);
      else if (kind == kPxInverse) ok = wait_count(&counters[2 + 2 * it.run], R.zb_items, err);
      s_ok = ok;
    }
    __syncthreads();
    if (s_ok) {
      const WorkItem wi{it.run, it.a, it.b, 0};
#define MWF_PX(SZ, MM_)                                                                          \
  case (kPxForward << 8) | SZ: xf_batched_item<MM_, NT>(R, wi, smem_raw, smem_bytes, err); break; \
  case (kPzM4 << 8) | SZ: z_batched_item<4, MM_, NT>(R, wi, smem_raw, smem_bytes, err); break;   \
  case (kPxInverse << 8) | SZ: xi_batched_item<MM_, NT>(R, wi, smem_raw, smem_bytes, err); break;
#define MWF_PZ6(SZ, Q_) \
  case (kPzM6 << 8) | SZ: z_batched_item<6, Q_, NT>(R, wi, smem_raw, smem_bytes, err); break;
      switch (it.code) {
        MWF_PX(0, 32) MWF_PX(1, 48) MWF_PX(2, 64) MWF_PX(3, 96) MWF_PX(4, 128) MWF_PX(5, 192) MWF_PX(6, 256)
        MWF_PZ6(0, 32) MWF_PZ6(1, 48) MWF_PZ6(2, 64) MWF_PZ6(3, 96) MWF_PZ6(4, 128)
        default:
          if (threadIdx.x == 0) atomicOr(err, MWF_DERR_BAD_RADIX);
          break;
      }
#undef MWF_PX
#undef MWF_PZ6
    }
    // the whole CTA, then the count with release semantics: a consumer that sees the count sees
    // the item's writes; the shared memory is free for the next item
    __syncthreads();
    if (threadIdx.x == 0 && kind != kPxInverse)
      red_release_add(&counters[kind == kPxForward ? 1 + 2 * it.run : 2 + 2 * it.run], 1);
  }
}

}  // namespace mwf
