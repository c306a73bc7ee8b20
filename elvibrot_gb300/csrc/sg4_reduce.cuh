// sg4_reduce.cuh -- the ordered join of chunk partials shared by the H.psi
// accumulation and the fused propagation stages.
#pragma once
#include <cuda_runtime.h>

namespace evr {

// sum over chunks ch0..ch1-1 of part[ch * nrhs_v + v] = (s, c) partials,
// joined in chunk order with TwoSum (the second phase of the ordered
// reduction of the Smolyak-term contributions).
__device__ __forceinline__ double join_chunks(const double2* __restrict__ part, long long ch0, long long ch1,
                                              int nrhs_v, int v) {
  double s = 0.0, c = 0.0;
  for (long long ch = ch0; ch < ch1; ++ch) {
    const double2 pc = part[ch * nrhs_v + v];
    const double u = s + pc.x;  // TwoSum(s, pc.x)
    const double bp = u - s;
    c += ((s - (u - bp)) + (pc.x - bp)) + pc.y;
    s = u;
  }
  return s + c;
}

}  // namespace evr
