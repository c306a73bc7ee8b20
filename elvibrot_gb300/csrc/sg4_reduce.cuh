// sg4_reduce.cuh -- the ordered join of chunk partials shared by the H.psi
// accumulation and the fused propagation stages.
#pragma once
#include <cuda_runtime.h>

namespace evr {

// sum over chunks ch0..ch1-1 of part[ch * nrhs_v + v] = (s, c) partials,
// joined in chunk order with TwoSum (the second phase of the ordered
// reduction of the Smolyak-term contributions).
// The partials are loaded four at a time ahead of the additions (a short
// list is latency-bound: its loads, not its additions, set the time); the
// additions run in the same order, so the bits do not change.
__device__ __forceinline__ void two_sum_add(double& s, double& c, double2 pc) {
  const double u = s + pc.x;  // TwoSum(s, pc.x)
  const double bp = u - s;
  c += ((s - (u - bp)) + (pc.x - bp)) + pc.y;
  s = u;
}

__device__ __forceinline__ double join_chunks(const double2* __restrict__ part, long long ch0, long long ch1,
                                              int nrhs_v, int v) {
  double s = 0.0, c = 0.0;
  long long ch = ch0;
  for (; ch + 4 <= ch1; ch += 4) {
    double2 pc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) pc[k] = part[(ch + k) * nrhs_v + v];
#pragma unroll
    for (int k = 0; k < 4; ++k) two_sum_add(s, c, pc[k]);
  }
  for (; ch < ch1; ++ch) two_sum_add(s, c, part[ch * nrhs_v + v]);
  return s + c;
}

}  // namespace evr
