// reduce.cuh -- deterministic block and grid reductions.
//
// A reducing kernel stores one partial per block, takes a ticket from a
// counter, and the block that takes the last ticket sums the partials in a
// fixed order (so results are bitwise reproducible) and resets the counter
// for the next launch.  This folds the final pass of a dot product into the
// kernel that produces it.
#pragma once

namespace ifemgpu {

// sum over the block, valid in thread 0; sh holds 32 doubles
__device__ inline double blockReduceSum(double v, double* sh)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sh[i];
  __syncthreads();
  return s;
}

// FP32 partials: warp and block sums in FP32, widened once per block (valid
// in thread 0); the blocks' partials are then summed in FP64.  FP64
// instructions issued by one lane cost the FP64 pipe a full warp on this GPU,
// so per-element work stays in FP32.
__device__ inline double blockReduceSumF(float v, double* sh)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float* shf = reinterpret_cast<float*>(sh);
  if (lane == 0) shf[w] = v;
  __syncthreads();
  float s = 0.f;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += shf[i];
  __syncthreads();
  return (double)s;  // one widening per block
}

// after thread 0 has stored this block's partials: true in the block that
// finishes last of nblocks (every thread of it), which also resets the counter
__device__ inline bool lastBlockOf(unsigned* counter, unsigned nblocks)
{
  __shared__ unsigned ticket;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) ticket = atomicAdd(counter, 1u);
  __syncthreads();
  const bool last = ticket == nblocks - 1;
  if (last) {
    __threadfence();
    if (threadIdx.x == 0) *counter = 0u;
  }
  return last;
}

__device__ inline bool lastBlock(unsigned* counter) { return lastBlockOf(counter, gridDim.x); }

// stores the partial t (thread 0's value) of this block in part[blockIdx.x]
__device__ inline bool lastBlockDone(double* part, double t, unsigned* counter)
{
  if (threadIdx.x == 0) part[blockIdx.x] = t;
  return lastBlock(counter);
}

// sum of part[0..n) in fixed order, valid in thread 0 (call from the last block)
__device__ inline double finalSum(const double* part, int n, double* sh)
{
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += __ldcg(part + i);
  return blockReduceSum(s, sh);
}

}  // namespace ifemgpu
