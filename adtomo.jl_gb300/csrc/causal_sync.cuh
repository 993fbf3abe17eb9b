// causal_sync.cuh -- the queue and the CTA-scope ordering of the causal-order
// adjoint solves (eik3d_adj_causal.cuh in 3D, eik2d.cu in 2D): one CTA
// evaluates the cells of a solve in an order where every cell follows its
// users, taking cells from a queue that the threads releasing them fill.
#pragma once
#include <cstdint>

namespace adt {

// A wait on one queue slot gives up after this many SM cycles (about two
// seconds; a slot is written once the cells queued before it are evaluated,
// which takes microseconds to milliseconds).
constexpr long long CAUSAL_WAIT_CYCLES = 4000000000LL;

// CTA-scope acquire load / release store / acq_rel atomic AND on global memory.
__device__ __forceinline__ int ld_acquire_cta(const int* p) {
  int v;
  asm volatile("ld.acquire.cta.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_cta(int* p, int v) {
  asm volatile("st.release.cta.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t atom_and_acq_rel_cta(uint32_t* p, uint32_t v) {
  uint32_t old;
  asm volatile("atom.acq_rel.cta.global.and.b32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// The lanes that arrive together take consecutive slots of a shared counter:
// n (0..3) each; one shared atomic per group of lanes.  Callable from
// divergent code (the group is __activemask()).
__device__ __forceinline__ int take_slots(int n, int* counter) {
  const unsigned mask = __activemask();
  const int lane = threadIdx.x & 31;
  const unsigned b0 = __ballot_sync(mask, n & 1), b1 = __ballot_sync(mask, n & 2);
  const unsigned lower = (1u << lane) - 1u;
  const int total = __popc(b0) + 2 * __popc(b1);
  const int leader = __ffs(mask) - 1;
  int base = 0;
  if (lane == leader && total) base = atomicAdd(counter, total);
  base = __shfl_sync(mask, base, leader);
  return base + __popc(b0 & lower) + 2 * __popc(b1 & lower);
}

// All 32 lanes call with their entry counts; returns this lane's first slot
// in a list whose length is counted in *len (one shared atomic per warp).
__device__ __forceinline__ int warp_append(int np, int* len, int lane) {
  int incl = np;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  int wb = 0;
  if (lane == 31 && total) wb = atomicAdd(len, total);
  wb = __shfl_sync(0xffffffffu, wb, 31);
  return wb + incl - np;
}

}  // namespace adt
