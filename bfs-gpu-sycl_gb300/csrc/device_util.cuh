// device_util.cuh -- warp-level helpers shared by the BFS kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace bfsgb {

constexpr uint32_t kFull = 0xFFFFFFFFu;

// ---- device helpers ---------------------------------------------------------

// Edge-array load: read once per BFS, so bypass L1 and mark evict-first in L2
// to keep the L2 for the visited bitmaps and queues.
__device__ __forceinline__ uint32_t ld_stream(const uint32_t *p, uint64_t pol) {
  uint32_t r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.b32 %0, [%1], %2;"
               : "=r"(r)
               : "l"(p), "l"(pol));
  return r;
}
// 16-byte edge-array load (four consecutive entries), same cache policy.
__device__ __forceinline__ uint4 ld_stream4(const uint4 *p, uint64_t pol) {
  uint4 r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p), "l"(pol));
  return r;
}
// 1 << p for p < 32 and 0 for p >= 32 (PTX shl clamps the shift amount;
// C++ would leave p >= 32 undefined).
__device__ __forceinline__ uint32_t bit_or_zero(uint32_t p) {
  uint32_t r;
  asm("shl.b32 %0, 1, %1;" : "=r"(r) : "r"(p));
  return r;
}
// Loads *p into r only when pred != 0 (a predicated load: no branch, and no
// memory request for lanes whose predicate is off); r keeps its value
// otherwise.  Not volatile and without a memory clobber, so the compiler may
// move it freely -- used for visited-bitmap words, where a stale value only
// costs an extra claim (bits only ever go from 0 to 1).
__device__ __forceinline__ void ld_global_if(uint32_t &r, const uint32_t *p, uint32_t pred) {
  asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q ld.global.u32 %0, [%1];\n\t}"
      : "+r"(r)
      : "l"(p), "r"(pred));
}
__device__ __forceinline__ void ld_shared_if(uint32_t &r, uint32_t saddr, uint32_t pred) {
  asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q ld.shared.u32 %0, [%1];\n\t}"
      : "+r"(r)
      : "r"(saddr), "r"(pred));
}
// Fire-and-forget OR into global memory (a reduction: no value comes back,
// so nothing is written back to the registers of the issuing warp).
__device__ __forceinline__ void red_or(uint32_t *p, uint32_t v) {
  asm volatile("red.relaxed.gpu.global.or.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_or(unsigned long long *p, unsigned long long v) {
  asm volatile("red.relaxed.gpu.global.or.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x, uint32_t lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t y = __shfl_up_sync(kFull, x, d);
    if (lane >= (uint32_t)d) x += y;
  }
  return x;
}
__device__ __forceinline__ unsigned long long warp_incl_scan64(unsigned long long x,
                                                               uint32_t lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    unsigned long long y = __shfl_up_sync(kFull, x, d);
    if (lane >= (uint32_t)d) x += y;
  }
  return x;
}

// Last entry j in [0, F) with qp[j] <= x, for a non-decreasing qp with
// qp[0] <= x: a 32-ary search, one probe per lane and round.
__device__ __forceinline__ uint32_t warp_owner_search(const uint32_t *__restrict__ qp,
                                                      uint32_t F, uint32_t x,
                                                      uint32_t lane) {
  uint32_t lo = 0, hi = F;  // qp[lo] <= x < qp[hi] (qp[F] = edge total)
  while (hi - lo > 32u) {
    const uint32_t step = (hi - lo + 31u) >> 5;
    const uint32_t j = lo + lane * step;
    const uint32_t val = (j < hi) ? qp[j] : kFull;
    const uint32_t m = __ballot_sync(kFull, val <= x);
    const uint32_t t = 31u - __clz(m);
    lo = lo + t * step;
    hi = min(hi, lo + step);
  }
  const uint32_t j = lo + lane;
  const uint32_t val = (j < hi) ? qp[j] : kFull;
  const uint32_t m = __ballot_sync(kFull, val <= x);
  return lo + 31u - __clz(m);
}

}  // namespace bfsgb
