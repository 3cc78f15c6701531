// solver.cu -- linear solve of the assembled system on the GPU.
//
// IFEM solves K x = b with SuperLU (SparseMatrix::solveSLUx,
// src/LinAlg/SparseMatrix.C:1147-1296) or, with PETSc/ISTL, a Krylov method.
// Here the solve is Jacobi-preconditioned CG:
//   IFEMGPU_PCG_MIXED  FP32 PCG on an FP32 copy of K inside an FP64 iterative
//                      refinement loop; the refinement residual r = b - K x
//                      is formed from the FP64 matrix, so the reported
//                      relative residual is an FP64 quantity.
//   IFEMGPU_PCG_FP64   FP64 PCG.
// The matrix is symmetric, so its compressed-column arrays are also its
// compressed-row arrays: SpMV reads one column per output entry (warp per
// row).  Dot products reduce through fixed-size per-block partial sums and a
// single-block final pass, so results are bitwise reproducible run to run.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <unordered_map>
#include <vector>

#include "ifemgpu_internal.h"
#include "reduce.cuh"

namespace ifemgpu {

namespace {

constexpr int kRedBlocks = 1024;   // blocks of the reducing kernels
constexpr int kThreads = 256;

// Partial sums -> scalar (single block, fixed order).
__global__ void k_finish(const double* __restrict__ part, int nparts, int nvals,
                         double* __restrict__ out)
{
  __shared__ double sh[kThreads];
  for (int v = 0; v < nvals; v++) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += part[(size_t)v * nparts + i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[v] = sh[0];
    __syncthreads();
  }
}

__device__ inline double blockSum(double v, double* sh)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sh[i];
  __syncthreads();
  return s;  // valid in thread 0
}

template <typename T>
__global__ void k_convert(const double* __restrict__ a, T* __restrict__ b, int64_t n)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (T)a[i];
}

// inverse diagonal
__global__ void k_diag(const int* __restrict__ colptr, const int* __restrict__ rowidx,
                       const double* __restrict__ K, int n, double* __restrict__ d64,
                       float* __restrict__ d32)
{
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    int lo = colptr[j], hi = colptr[j + 1] - 1;
    double v = 1.0;
    while (lo <= hi) {
      int mid = (lo + hi) >> 1;
      int r = rowidx[mid];
      if (r == j) { v = K[mid]; break; }
      if (r < j) lo = mid + 1; else hi = mid - 1;
    }
    double di = v != 0.0 ? 1.0 / v : 1.0;
    d64[j] = di;
    d32[j] = (float)di;
  }
}

// y = A x (warp per row), partial of dot(x, y) per block when part != null
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_spmv(const int* __restrict__ colptr, const int* __restrict__ rowidx, const T* __restrict__ A,
       const T* __restrict__ x, T* __restrict__ y, int n, double* __restrict__ part)
{
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31;
  const int warpsPerGrid = gridDim.x * (blockDim.x >> 5);
  double dot = 0.0;
  for (int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < n; row += warpsPerGrid) {
    const int b = colptr[row], e = colptr[row + 1];
    T s = 0;
    for (int k = b + lane; k < e; k += 32) s += A[k] * x[rowidx[k]];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) {
      y[row] = s;
      dot += (double)s * (double)x[row];
    }
  }
  if (part) {
    double t = blockSum(dot, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}

// r = b - A x in FP64, partial of ||r||^2; column indices from rowidx, or
// (rowPat != nullptr) from the row-pattern dictionary
__global__ void __launch_bounds__(kThreads)
k_residual(const int* __restrict__ colptr, const int* __restrict__ rowidx,
           const double* __restrict__ A, const double* __restrict__ x,
           const double* __restrict__ b, double* __restrict__ r, int n, double* __restrict__ part,
           const int* __restrict__ rowPat = nullptr, const int* __restrict__ patStart = nullptr,
           const short* __restrict__ patOff = nullptr)
{
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31;
  const int warpsPerGrid = gridDim.x * (blockDim.x >> 5);
  double acc = 0.0;
  for (int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < n; row += warpsPerGrid) {
    const int c0 = colptr[row], c1 = colptr[row + 1];
    double s = 0.0;
    if (rowPat) {
      const int so = patStart[rowPat[row]] - c0;  // offset of entry k: patOff[k + so]
      for (int k = c0 + lane; k < c1; k += 32) s += A[k] * x[row + patOff[k + so]];
    } else {
      for (int k = c0 + lane; k < c1; k += 32) s += A[k] * x[rowidx[k]];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) {
      const double v = b[row] - s;
      r[row] = v;
      acc += v * v;
    }
  }
  double t = blockSum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// partial of ||v||^2
template <typename T>
__global__ void k_norm2(const T* __restrict__ v, int n, double* __restrict__ part)
{
  __shared__ double sh[32];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    acc += (double)v[i] * (double)v[i];
  double t = blockSum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// rhs32 = r / rn ; x32 = 0 ; z = Dinv r ; p = z ; partial of (r, z)
template <typename T>
__global__ void k_pcg_start(const double* __restrict__ r64, const double* __restrict__ scal,
                            int scalIdx, T* __restrict__ r, T* __restrict__ x, T* __restrict__ z,
                            T* __restrict__ p, const T* __restrict__ dinv, int n,
                            double* __restrict__ part)
{
  __shared__ double sh[32];
  const double inv = 1.0 / sqrt(scal[scalIdx]);
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const T ri = (T)(r64[i] * inv);
    const T zi = dinv[i] * ri;
    r[i] = ri;
    x[i] = 0;
    z[i] = zi;
    p[i] = zi;
    acc += (double)ri * (double)zi;
  }
  double t = blockSum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// scalars: s[0]=rz, s[1]=pq, s[2]=rz_new, s[3]=rr
template <typename T>
__global__ void k_pcg_update(T* __restrict__ x, T* __restrict__ r, T* __restrict__ z,
                             const T* __restrict__ p, const T* __restrict__ q,
                             const T* __restrict__ dinv, const double* __restrict__ s, int n,
                             double* __restrict__ part)
{
  __shared__ double sh[32];
  const T alpha = (T)(s[0] / s[1]);
  double a1 = 0.0, a2 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    const T ri = r[i] - alpha * q[i];
    const T zi = dinv[i] * ri;
    r[i] = ri;
    z[i] = zi;
    a1 += (double)ri * (double)zi;
    a2 += (double)ri * (double)ri;
  }
  double t1 = blockSum(a1, sh);
  double t2 = blockSum(a2, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = t1;
    part[gridDim.x + blockIdx.x] = t2;
  }
}

template <typename T>
__global__ void k_pcg_dir(T* __restrict__ p, const T* __restrict__ z, double* __restrict__ s, int n)
{
  const T beta = (T)(s[2] / s[0]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = z[i] + beta * p[i];
}

__global__ void k_shift_scalars(double* s)
{
  // rz <- rz_new after the direction update has consumed both
  s[0] = s[2];
}

// x64 += scale * d
template <typename T>
__global__ void k_accumulate(double* __restrict__ x, const T* __restrict__ d,
                             const double* __restrict__ scal, int scalIdx, int n)
{
  const double sc = sqrt(scal[scalIdx]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] += sc * (double)d[i];
}

// ---- kernels of the captured inner loops --------------------------------------
// The loops run as CUDA graphs of kLoopBlock iterations.  Their scalars live
// on the device; the kernel that updates the residual sets S_DONE once the
// recurrence residual reaches the tolerance (or the iteration cap, or NaN),
// after which every later kernel of the graph returns at once.  Dot products
// finish inside the kernel that forms them (last-block reduction).
enum : int {
  S_RZ = 0, S_PQ = 1, S_RZN = 2, S_RR = 3, S_DONE = 4, S_ITS = 5, S_TOL2 = 6, S_MAXIT = 7,
  // [8] ||b||^2 and [9] the refinement residual^2 belong to runSolve
  S_PR = 10, S_ZQ = 11,
  S_STAG = 12, S_RREF = 13, S_ITREF = 14,  // stagnation test (learned loops)
  S_CNT = 24  // [24..28): eight unsigned ticket counters
};
constexpr int kScal = 32;
constexpr int kLoopBlock = 8;
constexpr int kStagWindow = 32;      // iterations per stagnation test
constexpr double kStagFactor = 0.25; // required reduction of ||r||^2 per window

// S_DONE: 1 converged or capped, 2 NaN, 3 stagnated
__device__ inline unsigned* tickets(double* s) { return reinterpret_cast<unsigned*>(s + S_CNT); }
__device__ inline bool loopStopped(const double* s) { return s[S_DONE] != 0.0; }

// FP32 step ratios [0] alpha, [1] beta in scalar slot 16, formed once by the
// last block of the kernel that finishes their numerator or denominator (an
// FP64 division per thread or per block would keep the FP64 pipe busy)
constexpr int S_RAT = 16;
__device__ inline float* ratios(double* s) { return reinterpret_cast<float*>(s + S_RAT); }
__device__ inline const float* ratios(const double* s)
{
  return reinterpret_cast<const float*>(s + S_RAT);
}

__global__ void k_loop_init(double* s, double tol2, double maxit, double stagnation)
{
  s[S_DONE] = 0.0;
  s[S_ITS] = 0.0;
  s[S_TOL2] = tol2;
  s[S_MAXIT] = maxit;
  s[S_PQ] = 1.0;
  s[S_ZQ] = 0.0;
  s[S_STAG] = stagnation;
  s[S_RREF] = 1.0;  // the loops start from a unit right-hand side
  s[S_ITREF] = 0.0;
  ratios(s)[0] = ratios(s)[1] = 0.f;
  unsigned* c = tickets(s);
  for (int i = 0; i < 8; i++) c[i] = 0u;
}

// after a residual update: count the iteration, stop on convergence, cap,
// NaN or (when enabled) too little progress over the last window
__device__ inline void loopCheck(double* s, double rr)
{
  s[S_RR] = rr;
  const double its = s[S_ITS] + 1.0;
  s[S_ITS] = its;
  if (!(rr == rr)) {
    s[S_DONE] = 2.0;
  } else if (rr <= s[S_TOL2] || its >= s[S_MAXIT]) {
    s[S_DONE] = 1.0;
  } else if (s[S_STAG] != 0.0 && its - s[S_ITREF] >= kStagWindow) {
    if (rr > kStagFactor * s[S_RREF]) {
      s[S_DONE] = 3.0;
    } else {
      s[S_RREF] = rr;
      s[S_ITREF] = its;
    }
  }
}

// rhs = r64 / sqrt(scal[9]); x = 0; z = Dinv r; p = z; rz -> S_RZ, S_RZN
template <typename T>
__global__ void __launch_bounds__(kThreads)
g_pcg_start(const double* __restrict__ r64, double* s, T* __restrict__ r, T* __restrict__ x,
            T* __restrict__ z, T* __restrict__ p, const T* __restrict__ dinv, int n,
            double* __restrict__ part)
{
  __shared__ double sh[32];
  const double inv = 1.0 / sqrt(s[9]);
  float acc = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const T ri = (T)(r64[i] * inv);
    const T zi = dinv[i] * ri;
    r[i] = ri;
    x[i] = 0;
    z[i] = zi;
    p[i] = zi;
    acc += (float)(ri * zi);
  }
  const double t = blockReduceSumF(acc, sh);
  if (lastBlockDone(part, t, tickets(s) + 4)) {
    const double v = finalSum(part, gridDim.x, sh);
    if (threadIdx.x == 0) s[S_RZ] = s[S_RZN] = v;
  }
}

// q = A p (warp per row); (p, q) -> S_PQ; with shift also S_RZ <- S_RZN
template <typename T>
__global__ void __launch_bounds__(kThreads)
g_spmv(const int* __restrict__ colptr, const int* __restrict__ rowidx, const T* __restrict__ A,
       const T* __restrict__ p, T* __restrict__ q, int n, double* __restrict__ part, double* s,
       int shift)
{
  if (loopStopped(s)) return;
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31;
  const int warpsPerGrid = gridDim.x * (blockDim.x >> 5);
  float dot = 0.f;
  for (int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < n; row += warpsPerGrid) {
    const int b = colptr[row], e = colptr[row + 1];
    T acc = 0;
    for (int k = b + lane; k < e; k += 32) acc += A[k] * p[rowidx[k]];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      q[row] = acc;
      dot += (float)(acc * p[row]);
    }
  }
  if (shift < 0) return;  // plain product: no dot, no scalars
  const double t = blockReduceSumF(dot, sh);
  if (lastBlockDone(part, t, tickets(s) + 0)) {
    const double v = finalSum(part, gridDim.x, sh);
    if (threadIdx.x == 0) {
      s[S_PQ] = v;
      if (shift) s[S_RZ] = s[S_RZN];
      ratios(s)[0] = (float)((shift ? s[S_RZ] : s[S_PR]) / v);  // alpha
    }
  }
}

// q = A p with 16-bit column offsets relative to the row (banded spline
// patterns), four independent load chains per lane; (p, q) -> S_PQ, alpha,
// with shift > 0 also S_RZ <- S_RZN, with shift < 0 the product only.  kPat: the offsets of row r are pattern
// rowPat[r] of the row-pattern dictionary (4 bytes per entry from HBM, the
// dictionary stays in L2); otherwise one offset per entry (6 bytes per entry).
template <bool kPat>
__global__ void __launch_bounds__(kThreads)
g_spmvOff(const int* __restrict__ colptr, const int* __restrict__ rowPat,
          const int* __restrict__ patStart, const short* __restrict__ off,
          const float* __restrict__ A, const float* __restrict__ p, float* __restrict__ q, int n,
          double* __restrict__ part, double* s, int shift)
{
  if (loopStopped(s)) return;
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31;
  const int warpsPerGrid = gridDim.x * (blockDim.x >> 5);
  float dot = 0.f;
  for (int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < n; row += warpsPerGrid) {
    const int b = colptr[row], e = colptr[row + 1];
    const int so = kPat ? patStart[rowPat[row]] - b : 0;  // offset of entry k: off[k + so]
    float acc = 0.f, acc1 = 0.f, acc2 = 0.f, acc3 = 0.f;
    int k = b + lane;
    // values stream (no L1 allocation: the offsets and p stay in L1); two
    // rounds unrolled so that their loads are issued together (-4% per
    // product on the 64^3 p=3 Poisson system)
#pragma unroll 2
    for (; k + 96 < e; k += 128) {
      const int o0 = off[k + so], o1 = off[k + so + 32], o2 = off[k + so + 64], o3 = off[k + so + 96];
      const float a0 = __ldcs(A + k), a1 = __ldcs(A + k + 32), a2 = __ldcs(A + k + 64),
                  a3 = __ldcs(A + k + 96);
      acc += a0 * p[row + o0];
      acc1 += a1 * p[row + o1];
      acc2 += a2 * p[row + o2];
      acc3 += a3 * p[row + o3];
    }
    // the remainder (at most three 32-wide slices) in one round of loads
    if (k < e) {
      const bool h1 = k + 32 < e, h2 = k + 64 < e;
      const int o0 = off[k + so];
      const int o1 = h1 ? off[k + so + 32] : 0, o2 = h2 ? off[k + so + 64] : 0;
      const float a0 = __ldcs(A + k);
      const float a1 = h1 ? __ldcs(A + k + 32) : 0.f, a2 = h2 ? __ldcs(A + k + 64) : 0.f;
      const float p0 = p[row + o0];
      const float p1 = h1 ? p[row + o1] : 0.f, p2 = h2 ? p[row + o2] : 0.f;
      acc += a0 * p0;
      acc1 += a1 * p1;
      acc2 += a2 * p2;
    }
    acc += (acc1 + acc2) + acc3;
    for (int w = 16; w > 0; w >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, w);
    if (lane == 0) {
      q[row] = acc;
      dot += acc * p[row];
    }
  }
  if (shift < 0) return;  // plain product: no dot, no scalars
  const double t = blockReduceSumF(dot, sh);
  if (lastBlockDone(part, t, tickets(s) + 0)) {
    const double v = finalSum(part, gridDim.x, sh);
    if (threadIdx.x == 0) {
      s[S_PQ] = v;
      if (shift) s[S_RZ] = s[S_RZN];
      ratios(s)[0] = (float)((shift ? s[S_RZ] : s[S_PR]) / v);  // alpha
    }
  }
}

// off[k] = rowidx[k] - row (warp per row); *bad = 1 when an offset needs more than 16 bits
__global__ void k_make_off16(const int* __restrict__ colptr, const int* __restrict__ rowidx, int n,
                             short* __restrict__ off, int* __restrict__ bad)
{
  const int lane = threadIdx.x & 31;
  const int warpsPerGrid = gridDim.x * (blockDim.x >> 5);
  for (int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < n; row += warpsPerGrid)
    for (int k = colptr[row] + lane; k < colptr[row + 1]; k += 32) {
      const int d = rowidx[k] - row;
      if (d < -32768 || d > 32767) *bad = 1;
      off[k] = (short)d;
    }
}

// x += a p; r -= a q; z = Dinv r with a = rz / pq; (r, z) -> S_RZN, (r, r) -> check
template <typename T>
__global__ void __launch_bounds__(kThreads)
g_pcg_update(T* __restrict__ x, T* __restrict__ r, T* __restrict__ z, const T* __restrict__ p,
             const T* __restrict__ q, const T* __restrict__ dinv, double* s, int n,
             double* __restrict__ part)
{
  if (loopStopped(s)) return;
  __shared__ double sh[32];
  const T alpha = (T)ratios(s)[0];
  float a1 = 0.f, a2 = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    const T ri = r[i] - alpha * q[i];
    const T zi = dinv[i] * ri;
    r[i] = ri;
    z[i] = zi;
    a1 += (float)(ri * zi);
    a2 += (float)(ri * ri);
  }
  const double t1 = blockReduceSumF(a1, sh);
  const double t2 = blockReduceSumF(a2, sh);
  if (threadIdx.x == 0) part[gridDim.x + blockIdx.x] = t2;
  if (lastBlockDone(part, t1, tickets(s) + 1)) {
    const double rz = finalSum(part, gridDim.x, sh);
    const double rr = finalSum(part + gridDim.x, gridDim.x, sh);
    if (threadIdx.x == 0) {
      s[S_RZN] = rz;
      ratios(s)[1] = (float)(rz / s[S_RZ]);  // beta of the PCG direction
      loopCheck(s, rr);
    }
  }
}

// p = z + (rz_new / rz) p
template <typename T>
__global__ void g_pcg_dir(T* __restrict__ p, const T* __restrict__ z, const double* s, int n)
{
  if (loopStopped(s)) return;
  const T beta = (T)ratios(s)[1];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = z[i] + beta * p[i];
}

// flexible CG (Notay's FCG(1)): rhs = r64 / sqrt(scal[9]); x = p = q = 0; z = Dinv r
__global__ void g_fcg_start(const double* __restrict__ r64, const double* s, float* __restrict__ r,
                            float* __restrict__ x, float* __restrict__ z, float* __restrict__ p,
                            float* __restrict__ q, const float* __restrict__ dinv, int n)
{
  const double inv = 1.0 / sqrt(s[9]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float ri = (float)(r64[i] * inv);
    r[i] = ri;
    x[i] = 0.f;
    z[i] = dinv[i] * ri;
    p[i] = 0.f;
    q[i] = 0.f;
  }
}

// x += a p; r -= a q; z = Dinv r with a = (p, r) / (p, q); (r, r) -> check
__global__ void __launch_bounds__(kThreads)
g_fcg_update(float* __restrict__ x, float* __restrict__ r, float* __restrict__ z,
             const float* __restrict__ p, const float* __restrict__ q,
             const float* __restrict__ dinv, double* s, int n, double* __restrict__ part)
{
  if (loopStopped(s)) return;
  __shared__ double sh[32];
  const float alpha = ratios(s)[0];
  float acc = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    const float ri = r[i] - alpha * q[i];
    r[i] = ri;
    if (z) z[i] = dinv[i] * ri;  // Jacobi fine level (null when another preconditioner writes z)
    acc += ri * ri;
  }
  const double t = blockReduceSumF(acc, sh);
  if (lastBlockDone(part, t, tickets(s) + 1)) {
    const double rr = finalSum(part, gridDim.x, sh);
    if (threadIdx.x == 0) loopCheck(s, rr);
  }
}

// p = z - ((z, q) / (p, q)) p, q = A p of the previous direction; (p, r) -> S_PR
__global__ void __launch_bounds__(kThreads)
g_fcg_dir(float* __restrict__ p, const float* __restrict__ z, const float* __restrict__ r,
          double* s, int n, double* __restrict__ part)
{
  if (loopStopped(s)) return;
  __shared__ double sh[32];
  const float beta = ratios(s)[1];
  float acc = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float pi = z[i] + beta * p[i];
    p[i] = pi;
    acc += pi * r[i];
  }
  const double t = blockReduceSumF(acc, sh);
  if (lastBlockDone(part, t, tickets(s) + 3)) {
    const double v = finalSum(part, gridDim.x, sh);
    if (threadIdx.x == 0) s[S_PR] = v;
  }
}

// (z, q) -> S_ZQ and the flexible-CG beta = -(z, q) / (p, q)
__global__ void __launch_bounds__(kThreads)
g_dot(const float* __restrict__ a, const float* __restrict__ b, int n, double* __restrict__ part,
      unsigned* counter, double* s)
{
  if (loopStopped(s)) return;
  __shared__ double sh[32];
  float acc = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    acc += a[i] * b[i];
  const double t = blockReduceSumF(acc, sh);
  if (lastBlockDone(part, t, counter)) {
    const double v = finalSum(part, gridDim.x, sh);
    if (threadIdx.x == 0) {
      s[S_ZQ] = v;
      ratios(s)[1] = (float)(-v / s[S_PQ]);
    }
  }
}

__global__ void k_copy_d(const double* __restrict__ a, double* __restrict__ b, int n)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = a[i];
}

}  // namespace

// Workspace layout (doubles): x64, r64, dinv64 | part (2*kRedBlocks) | scal(kScal)
// then typed vectors for the inner PCG (FP32: 6 n floats; FP64: 5 n doubles)
struct Work {
  double *x64, *r64, *d64, *part, *scal;
  float *r32, *x32, *z32, *p32, *q32, *dinv32;
  double *rD, *xD, *zD, *pD, *qD;
};

static Work carve(ifemgpu_ctx* ctx)
{
  const size_t n = ctx->neq;
  Work w{};
  double* base = ctx->d_work;
  w.x64 = base; base += n;
  w.r64 = base; base += n;
  w.d64 = base; base += n;
  w.part = base; base += 2 * kRedBlocks;
  w.scal = base; base += kScal;
  w.rD = base; base += n;
  w.xD = base; base += n;
  w.zD = base; base += n;
  w.pD = base; base += n;
  w.qD = base; base += n;
  float* fb = reinterpret_cast<float*>(base);
  w.r32 = fb; fb += n;
  w.x32 = fb; fb += n;
  w.z32 = fb; fb += n;
  w.p32 = fb; fb += n;
  w.q32 = fb; fb += n;
  w.dinv32 = fb; fb += n;
  return w;
}

static void dropLoopGraphs(ifemgpu_ctx* ctx)
{
  for (int g = 0; g < ifemgpu_ctx::kLoops; g++) {  // every captured inner loop
    if (ctx->loopExec[g]) cudaGraphExecDestroy(ctx->loopExec[g]);
    ctx->loopExec[g] = nullptr;
    ctx->loopKey[g] = nullptr;
  }
  ctx->workGen++;
}

void freeSolver(ifemgpu_ctx* ctx)
{
  dropLoopGraphs(ctx);
  if (ctx->d_K32) cudaFree(ctx->d_K32);
  if (ctx->d_off16) cudaFree(ctx->d_off16);
  if (ctx->d_rowPat) cudaFree(ctx->d_rowPat);
  if (ctx->d_patStart) cudaFree(ctx->d_patStart);
  if (ctx->d_patOff) cudaFree(ctx->d_patOff);
  if (ctx->d_work) cudaFree(ctx->d_work);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  ctx->d_off16 = nullptr;
  ctx->off16State = 0;
  ctx->d_rowPat = ctx->d_patStart = nullptr;
  ctx->d_patOff = nullptr;
  ctx->patState = 0;
  ctx->numPatterns = 0;
  ctx->d_K32 = nullptr;
  ctx->d_work = nullptr;
  ctx->h_pinned = nullptr;
  ctx->work_len = 0;
}

template <typename T>
static ifemgpu_status innerPCG(ifemgpu_ctx* ctx, const Work& w, const T* A, const T* dinv,
                               T* r, T* x, T* z, T* p, T* q, int scalIdx, double rtol,
                               int maxit, int* iters)
{
  cudaStream_t s = ctx->stream;
  const int n = ctx->neq;
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  const int sb = std::min(kRedBlocks, (n + 7) / 8);
  k_pcg_start<T><<<vb, kThreads, 0, s>>>(w.r64, w.scal, scalIdx, r, x, z, p, dinv, n, w.part);
  k_finish<<<1, kThreads, 0, s>>>(w.part, vb, 1, w.scal + 0);
  int it = 0;
  const int checkEvery = 16;
  double* h = ctx->h_pinned;
  while (it < maxit) {
    for (int k = 0; k < checkEvery && it < maxit; k++, it++) {
      k_spmv<T><<<sb, kThreads, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, A, p, q, n, w.part);
      k_finish<<<1, kThreads, 0, s>>>(w.part, sb, 1, w.scal + 1);
      k_pcg_update<T><<<vb, kThreads, 0, s>>>(x, r, z, p, q, dinv, w.scal, n, w.part);
      k_finish<<<1, kThreads, 0, s>>>(w.part, vb, 2, w.scal + 2);
      k_pcg_dir<T><<<vb, kThreads, 0, s>>>(p, z, w.scal, n);
      k_shift_scalars<<<1, 1, 0, s>>>(w.scal);
    }
    IFEMGPU_CUDA(ctx, cudaGetLastError());
    IFEMGPU_CUDA(ctx, cudaMemcpyAsync(h, w.scal + 3, sizeof(double), cudaMemcpyDeviceToHost, s));
    IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
    const double rr = h[0];
    if (!(rr == rr)) { *iters = it; return setError(ctx, IFEMGPU_NOT_CONVERGED, "PCG breakdown (NaN)"); }
    if (std::sqrt(rr) <= rtol) break;  // the right-hand side has unit norm
  }
  *iters = it;
  return IFEMGPU_OK;
}

// Captures kLoopBlock iterations of body into the slot's graph, once per
// workspace (and network) generation.
template <typename Body>
static ifemgpu_status captureLoop(ifemgpu_ctx* ctx, int slot, int gen, Body body)
{
  if (ctx->loopExec[slot] && ctx->loopKey[slot] == ctx->d_work && ctx->loopGen[slot] == gen)
    return IFEMGPU_OK;
  if (ctx->loopExec[slot]) cudaGraphExecDestroy(ctx->loopExec[slot]);
  ctx->loopExec[slot] = nullptr;
  cudaStream_t s = ctx->stream;
  IFEMGPU_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  ifemgpu_status st = IFEMGPU_OK;
  for (int k = 0; k < kLoopBlock && st == IFEMGPU_OK; k++) st = body();
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s, &g);
  if (st == IFEMGPU_OK && e != cudaSuccess) st = cudaFail(ctx, e, "cudaStreamEndCapture");
  if (st == IFEMGPU_OK) {
    const cudaError_t e2 = cudaGraphInstantiate(&ctx->loopExec[slot], g, 0);
    if (e2 != cudaSuccess) {
      ctx->loopExec[slot] = nullptr;
      st = cudaFail(ctx, e2, "cudaGraphInstantiate");
    }
  }
  if (g) cudaGraphDestroy(g);
  if (st != IFEMGPU_OK) return st;
  ctx->loopKey[slot] = ctx->d_work;
  ctx->loopGen[slot] = gen;
  return IFEMGPU_OK;
}

// Replays a captured loop until its stop flag is set (bounded by the cap).
static ifemgpu_status replayLoop(ifemgpu_ctx* ctx, const Work& w, int slot, int maxit,
                                 int* iters, int* flag)
{
  cudaStream_t s = ctx->stream;
  double* h = ctx->h_pinned;
  h[1] = 0.0;
  h[2] = 0.0;
  const int maxLaunch = maxit / kLoopBlock + 2;
  for (int l = 0; l < maxLaunch; l++) {
    IFEMGPU_CUDA(ctx, cudaGraphLaunch(ctx->loopExec[slot], s));
    IFEMGPU_CUDA(ctx, cudaMemcpyAsync(h, w.scal + S_RR, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
    if (h[1] != 0.0) break;  // S_DONE
  }
  *iters = (int)h[2];        // S_ITS
  *flag = (int)h[1];
  return IFEMGPU_OK;
}

static inline unsigned* hostTickets(const Work& w)
{
  return reinterpret_cast<unsigned*>(w.scal + S_CNT);
}

static void spmv32(ifemgpu_ctx* ctx, const Work& w, const float* p, float* q, int shift);

// One FP32 Jacobi-PCG iteration (the body of the captured loop), and its start
// on rhs r64 / sqrt(scal[9]) from x = 0.
static ifemgpu_status pcgIteration(ifemgpu_ctx* ctx, const Work& w)
{
  cudaStream_t s = ctx->stream;
  const int n = ctx->neq;
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  spmv32(ctx, w, w.p32, w.q32, 1);
  g_pcg_update<float><<<vb, kThreads, 0, s>>>(w.x32, w.r32, w.z32, w.p32, w.q32, w.dinv32, w.scal,
                                              n, w.part);
  g_pcg_dir<float><<<vb, kThreads, 0, s>>>(w.p32, w.z32, w.scal, n);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  return IFEMGPU_OK;
}

static ifemgpu_status pcgStart(ifemgpu_ctx* ctx, const Work& w, double rtol, int maxit)
{
  cudaStream_t s = ctx->stream;
  const int n = ctx->neq;
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  k_loop_init<<<1, 1, 0, s>>>(w.scal, rtol * rtol, (double)maxit, 0.0);
  g_pcg_start<float><<<vb, kThreads, 0, s>>>(w.r64, w.scal, w.r32, w.x32, w.z32, w.p32, w.dinv32,
                                             n, w.part);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  return IFEMGPU_OK;
}

// FP32 Jacobi-PCG on rhs r64 / sqrt(scal[9]) from x = 0 (captured loop)
static ifemgpu_status loopPCG32(ifemgpu_ctx* ctx, const Work& w, double rtol, int maxit,
                                int* iters)
{
  ifemgpu_status st = captureLoop(ctx, 0, ctx->workGen, [&]() { return pcgIteration(ctx, w); });
  if (st != IFEMGPU_OK) return st;
  if ((st = pcgStart(ctx, w, rtol, maxit)) != IFEMGPU_OK) return st;
  int flag = 0;
  if ((st = replayLoop(ctx, w, 0, maxit, iters, &flag)) != IFEMGPU_OK) return st;
  if (flag == 2) return setError(ctx, IFEMGPU_NOT_CONVERGED, "PCG breakdown (NaN)");
  return IFEMGPU_OK;
}

// z = M r of flexible CG after the Jacobi step of the update kernel: the fine
// level z1 (Jacobi, or the Kronecker preconditioner when kron) and, when
// learned, the network's coarse direction added with its energy-optimal
// coefficient (a multiplicative two-level step); withDot: (z, q) -> S_ZQ
// and beta
static ifemgpu_status fcgPrecondition(ifemgpu_ctx* ctx, const Work& w, bool kron, bool learned,
                                      bool withDot)
{
  cudaStream_t s = ctx->stream;
  const int n = ctx->neq;
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  unsigned* tk = hostTickets(w);
  const double* guard = w.scal + S_DONE;
  ifemgpu_status st2;
  if (kron && !learned && withDot && fdCanDot(ctx)) {  // (z, q) inside the last FD kernel
    FdDot dot;
    dot.q = w.q32;
    dot.part = w.part;
    dot.counter = tk + 2;
    dot.out = w.scal + S_ZQ;
    dot.pq = w.scal + S_PQ;
    dot.beta = reinterpret_cast<float*>(w.scal + S_RAT) + 1;
    return fdApply(ctx, w.r32, w.z32, guard, &dot);
  }
  if (kron && (st2 = fdApply(ctx, w.r32, w.z32, guard)) != IFEMGPU_OK) return st2;
  if (learned) {  // two-level step: t = A z1, then z = z1 + alpha R^T y
    float* t = learnT(ctx);
    spmv32(ctx, w, w.z32, t, -1);
    return learnApply(ctx, w.r32, w.z32, t, withDot ? w.q32 : nullptr, w.part, vb, tk + 2,
                      tk + 5, w.scal + S_ZQ, w.scal + S_PQ,
                      reinterpret_cast<float*>(w.scal + S_RAT) + 1, guard);
  }
  if (withDot) g_dot<<<vb, kThreads, 0, s>>>(w.z32, w.q32, n, w.part, tk + 2, w.scal);
  return IFEMGPU_OK;
}

// one flexible-CG iteration (the body of the captured loop)
static ifemgpu_status fcgIteration(ifemgpu_ctx* ctx, const Work& w, bool kron, bool learned)
{
  cudaStream_t s = ctx->stream;
  const int n = ctx->neq;
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  spmv32(ctx, w, w.p32, w.q32, 0);
  g_fcg_update<<<vb, kThreads, 0, s>>>(w.x32, w.r32, kron ? nullptr : w.z32, w.p32, w.q32,
                                       w.dinv32, w.scal, n, w.part);
  ifemgpu_status st2 = fcgPrecondition(ctx, w, kron, learned, true);
  if (st2 != IFEMGPU_OK) return st2;
  g_fcg_dir<<<vb, kThreads, 0, s>>>(w.p32, w.z32, w.r32, w.scal, n, w.part);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  return IFEMGPU_OK;
}

// flexible CG start on rhs r64 / sqrt(scal[9]) from x = p = q = 0
static ifemgpu_status fcgStart(ifemgpu_ctx* ctx, const Work& w, bool kron, bool learned,
                               double rtol, int maxit)
{
  cudaStream_t s = ctx->stream;
  const int n = ctx->neq;
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  // a learned loop must keep shrinking its residual or it stops (and the
  // caller continues without the network)
  k_loop_init<<<1, 1, 0, s>>>(w.scal, rtol * rtol, (double)maxit, learned ? 1.0 : 0.0);
  g_fcg_start<<<vb, kThreads, 0, s>>>(w.r64, w.scal, w.r32, w.x32, w.z32, w.p32, w.q32, w.dinv32, n);
  ifemgpu_status st = fcgPrecondition(ctx, w, kron, learned, false);  // p = q = 0: (z, q) = 0
  if (st != IFEMGPU_OK) return st;
  g_fcg_dir<<<vb, kThreads, 0, s>>>(w.p32, w.z32, w.r32, w.scal, n, w.part);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  return IFEMGPU_OK;
}

// FP32 flexible CG (captured loop).  *nan is set when the recurrence produced
// NaN or (learned) stagnated.
static ifemgpu_status loopFCG(ifemgpu_ctx* ctx, const Work& w, bool kron, bool learned,
                              double rtol, int maxit, int* iters, bool* nan)
{
  const int slot = 1 + (kron ? 1 : 0) + (learned ? 2 : 0);
  ifemgpu_status st = captureLoop(ctx, slot, ctx->workGen * 65536 + (learned ? ctx->learnGen : 0),
                                  [&]() { return fcgIteration(ctx, w, kron, learned); });
  if (st != IFEMGPU_OK) return st;
  if ((st = fcgStart(ctx, w, kron, learned, rtol, maxit)) != IFEMGPU_OK) return st;
  int flag = 0;
  if ((st = replayLoop(ctx, w, slot, maxit, iters, &flag)) != IFEMGPU_OK) return st;
  *nan = flag >= 2;  // NaN or stagnation
  return IFEMGPU_OK;
}

// SplitMix64 finaliser (Steele, Lea and Flood 2014) as the mixing step of a
// hash over a row's column offsets
static inline uint64_t mix64(uint64_t x)
{
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// Row-pattern dictionary of the compressed rows: rows whose column offsets
// (col - row) are the same sequence share one entry.  A structured patch has
// a few hundred distinct rows (interior, and each distance to each face), so
// the dictionary is a few hundred KB against 2 bytes per stored entry for
// per-entry offsets.  Returns false when an offset needs more than 16 bits,
// the dictionary would exceed 1/16 of the entries, or two different rows
// share a hash (then per-entry offsets are used).
static bool buildRowPatterns(const ifemgpu_ctx* ctx, std::vector<int>& rowPat,
                             std::vector<int>& patStart, std::vector<short>& patOff)
{
  const int n = ctx->neq;
  const int* cp = ctx->colptr.data();
  const int* ri = ctx->rowidx.data();
  std::vector<uint64_t> h(n);
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int r = 0; r < n; r++) {
    uint64_t x = mix64(0x9e3779b97f4a7c15ull + (uint64_t)(cp[r + 1] - cp[r]));
    for (int k = cp[r]; k < cp[r + 1]; k++) {
      const int d = ri[k] - r;
      bad |= d < -32768 || d > 32767;
      x = mix64(x ^ (uint32_t)d);
    }
    h[r] = x;
  }
  if (bad) return false;
  std::unordered_map<uint64_t, int> ids;
  std::vector<int> rep;
  rowPat.resize(n);
  for (int r = 0; r < n; r++) {
    auto it = ids.find(h[r]);
    if (it == ids.end()) {
      it = ids.emplace(h[r], (int)rep.size()).first;
      rep.push_back(r);
    }
    rowPat[r] = it->second;
  }
  patStart.assign(rep.size() + 1, 0);
  for (size_t i = 0; i < rep.size(); i++)
    patStart[i + 1] = patStart[i] + (cp[rep[i] + 1] - cp[rep[i]]);
  if ((int64_t)patStart.back() * 16 > ctx->nnz) return false;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int r = 0; r < n; r++) {
    const int q = rep[rowPat[r]];
    if (cp[r + 1] - cp[r] != cp[q + 1] - cp[q]) {
      bad = 1;
      continue;
    }
    for (int k = 0; k < cp[r + 1] - cp[r]; k++)
      bad |= ri[cp[r] + k] - r != ri[cp[q] + k] - q;
  }
  if (bad) return false;
  patOff.resize(patStart.back());
  for (size_t i = 0; i < rep.size(); i++) {
    const int q = rep[i];
    for (int k = cp[q]; k < cp[q + 1]; k++) patOff[patStart[i] + k - cp[q]] = (short)(ri[k] - q);
  }
  return true;
}

// workspace, pinned scalars and (mixed) the FP32 matrix copy
static ifemgpu_status ensureWork(ifemgpu_ctx* ctx, bool mixed)
{
  const size_t n = ctx->neq;
  const size_t need = sizeof(double) * (n * 8 + 2 * kRedBlocks + kScal) + sizeof(float) * n * 6;
  if (ctx->work_len < need) {
    dropLoopGraphs(ctx);
    if (ctx->d_work) cudaFree(ctx->d_work);
    ctx->d_work = nullptr;
    ctx->work_len = 0;
    IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_work, need));
    ctx->work_len = need;
  }
  if (!ctx->h_pinned) IFEMGPU_CUDA(ctx, cudaMallocHost(&ctx->h_pinned, 64));
  if (mixed && !ctx->d_K32) IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_K32, sizeof(float) * ctx->nnz));
  if (ctx->patState == 0) {  // row-pattern dictionary when the rows repeat
    ctx->patState = -1;
    std::vector<int> rowPat, patStart;
    std::vector<short> patOff;
    if (buildRowPatterns(ctx, rowPat, patStart, patOff)) {
      bool ok = cudaMalloc(&ctx->d_rowPat, sizeof(int) * rowPat.size()) == cudaSuccess &&
                cudaMalloc(&ctx->d_patStart, sizeof(int) * patStart.size()) == cudaSuccess &&
                cudaMalloc(&ctx->d_patOff, sizeof(short) * std::max<size_t>(patOff.size(), 1)) ==
                    cudaSuccess;
      ok = ok &&
           cudaMemcpy(ctx->d_rowPat, rowPat.data(), sizeof(int) * rowPat.size(),
                      cudaMemcpyHostToDevice) == cudaSuccess &&
           cudaMemcpy(ctx->d_patStart, patStart.data(), sizeof(int) * patStart.size(),
                      cudaMemcpyHostToDevice) == cudaSuccess &&
           cudaMemcpy(ctx->d_patOff, patOff.data(), sizeof(short) * patOff.size(),
                      cudaMemcpyHostToDevice) == cudaSuccess;
      if (ok) {
        ctx->patState = 1;
        ctx->numPatterns = (int)patStart.size() - 1;
      } else {
        cudaGetLastError();
        if (ctx->d_rowPat) cudaFree(ctx->d_rowPat);
        if (ctx->d_patStart) cudaFree(ctx->d_patStart);
        if (ctx->d_patOff) cudaFree(ctx->d_patOff);
        ctx->d_rowPat = ctx->d_patStart = nullptr;
        ctx->d_patOff = nullptr;
      }
      dropLoopGraphs(ctx);
    }
  }
  if (mixed && ctx->off16State == 0 && ctx->patState != 1) {  // 16-bit column offsets when the band allows
    ctx->off16State = -1;
    if (cudaMalloc(&ctx->d_off16, sizeof(short) * std::max<int64_t>(ctx->nnz, 1)) == cudaSuccess) {
      int* d_bad = reinterpret_cast<int*>(carve(ctx).scal + 30);  // unused scalar slot
      IFEMGPU_CUDA(ctx, cudaMemsetAsync(d_bad, 0, sizeof(int), ctx->stream));
      k_make_off16<<<1024, kThreads, 0, ctx->stream>>>(ctx->d_colptr, ctx->d_rowidx, (int)n,
                                                        ctx->d_off16, d_bad);
      int bad = 1;
      IFEMGPU_CUDA(ctx, cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      if (bad == 0) {
        ctx->off16State = 1;
      } else {
        cudaFree(ctx->d_off16);
        ctx->d_off16 = nullptr;
      }
      dropLoopGraphs(ctx);
    } else {
      cudaGetLastError();
      ctx->d_off16 = nullptr;
    }
  }
  return IFEMGPU_OK;
}

// q = A p of the FP32 loops (16-bit offsets when available)
static void spmv32(ifemgpu_ctx* ctx, const Work& w, const float* p, float* q, int shift)
{
  const int n = ctx->neq;
  const int sb = std::min(kRedBlocks, (n + 7) / 8);
  if (ctx->d_rowPat)
    g_spmvOff<true><<<sb, kThreads, 0, ctx->stream>>>(ctx->d_colptr, ctx->d_rowPat, ctx->d_patStart,
                                                      ctx->d_patOff, ctx->d_K32, p, q, n, w.part,
                                                      w.scal, shift);
  else if (ctx->d_off16)
    g_spmvOff<false><<<sb, kThreads, 0, ctx->stream>>>(ctx->d_colptr, nullptr, nullptr,
                                                       ctx->d_off16, ctx->d_K32, p, q, n, w.part,
                                                       w.scal, shift);
  else
    g_spmv<float><<<sb, kThreads, 0, ctx->stream>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K32, p, q,
                                                    n, w.part, w.scal, shift);
}

// FP32 matrix copy, inverse diagonal, x64 = 0, r64 = b, ||b||^2 in scal[8]
// and scal[9]; returns ||b||
static ifemgpu_status solvePrologue(ifemgpu_ctx* ctx, const Work& w, const double* b, bool mixed,
                                    double* bn)
{
  cudaStream_t s = ctx->stream;
  const int n = ctx->neq;
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  if (mixed) k_convert<float><<<1024, kThreads, 0, s>>>(ctx->d_K, ctx->d_K32, ctx->nnz);
  k_diag<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K,
                                                              n, w.d64, w.dinv32);
  IFEMGPU_CUDA(ctx, cudaMemsetAsync(w.x64, 0, sizeof(double) * n, s));
  k_norm2<double><<<vb, kThreads, 0, s>>>(b, n, w.part);
  k_finish<<<1, kThreads, 0, s>>>(w.part, vb, 1, w.scal + 8);
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(w.r64, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(w.scal + 9, w.scal + 8, sizeof(double), cudaMemcpyDeviceToDevice, s));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, w.scal + 8, sizeof(double), cudaMemcpyDeviceToHost, s));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  *bn = std::sqrt(ctx->h_pinned[0]);
  return IFEMGPU_OK;
}

// r64 = b - A x64 in FP64; returns ||r64||
static ifemgpu_status refineResidual(ifemgpu_ctx* ctx, const Work& w, const double* b, double* rn)
{
  cudaStream_t s = ctx->stream;
  const int n = ctx->neq;
  const int sb = std::min(kRedBlocks, (n + 7) / 8);
  k_residual<<<sb, kThreads, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K, w.x64, b, w.r64, n,
                                     w.part, ctx->d_rowPat, ctx->d_patStart, ctx->d_patOff);
  k_finish<<<1, kThreads, 0, s>>>(w.part, sb, 1, w.scal + 9);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, w.scal + 9, sizeof(double), cudaMemcpyDeviceToHost, s));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  *rn = std::sqrt(ctx->h_pinned[0]);
  return IFEMGPU_OK;
}

ifemgpu_status runSolve(ifemgpu_ctx* ctx, const ifemgpu_solver_options* o, double* xh,
                        ifemgpu_solve_info* info, const double* bdev)
{
  const int n = ctx->neq;
  cudaStream_t s = ctx->stream;
  const double* b = bdev ? bdev : ctx->d_b;
  if (n == 0) {
    if (info) *info = ifemgpu_solve_info{0, 0, 0.0, 0.0, 0};
    return IFEMGPU_OK;
  }
  if (o->method != IFEMGPU_PCG_MIXED && o->method != IFEMGPU_PCG_FP64 &&
      o->method != IFEMGPU_FCG_LEARNED)
    return setError(ctx, IFEMGPU_INVALID_ARG, "solve: unknown method");
  bool learned = o->method == IFEMGPU_FCG_LEARNED;
  if (learned && !learnReady(ctx))
    return setError(ctx, IFEMGPU_NOT_READY, "solve: no trained coarse correction");
  const bool mixed = o->method != IFEMGPU_PCG_FP64;
  if (o->precond != IFEMGPU_PRECOND_JACOBI && o->precond != IFEMGPU_PRECOND_KRONECKER)
    return setError(ctx, IFEMGPU_INVALID_ARG, "solve: unknown preconditioner");
  const bool kron = o->precond == IFEMGPU_PRECOND_KRONECKER;
  if (kron && !mixed)
    return setError(ctx, IFEMGPU_INVALID_ARG, "solve: the FP64 method takes the Jacobi preconditioner");
  ifemgpu_status st = ensureWork(ctx, mixed);
  if (st != IFEMGPU_OK) return st;
  if (kron && (st = fdSetup(ctx)) != IFEMGPU_OK) return st;
  if (learned && (st = learnPrepare(ctx)) != IFEMGPU_OK) return st;
  Work w = carve(ctx);
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
  // the coarse Galerkin matrix of this assembly (timed with the solve)
  if (learned && (st = learnGalerkin(ctx)) != IFEMGPU_OK) return st;
  double bn = 0.0;
  if ((st = solvePrologue(ctx, w, b, mixed, &bn)) != IFEMGPU_OK) return st;
  if (kron && (st = fdRescale(ctx, w.d64)) != IFEMGPU_OK) return st;
  int outer = 0, inner = 0, fallbacks = 0;
  double relres = bn > 0 ? 1.0 : 0.0;
  const int maxOuter = mixed ? std::max(1, o->max_outer) : 1;
  const double innerTol = mixed ? (o->inner_rtol > 0 ? o->inner_rtol : 1e-4) : o->rtol;
  while (bn > 0 && relres > o->rtol && outer < maxOuter) {
    int it = 0;
    bool nan = false;
    if (learned || kron) {
      st = loopFCG(ctx, w, kron, learned, innerTol, o->max_inner, &it, &nan);
    } else if (mixed) {
      st = loopPCG32(ctx, w, innerTol, o->max_inner, &it);
    } else {
      st = innerPCG<double>(ctx, w, ctx->d_K, w.d64, w.rD, w.xD, w.zD, w.pD, w.qD, 9, innerTol,
                            o->max_inner, &it);
    }
    inner += it;
    outer++;
    if (st != IFEMGPU_OK) break;
    if (nan) {  // the learned step broke down: continue without the network
      if (!learned) {
        st = setError(ctx, IFEMGPU_NOT_CONVERGED, "flexible CG breakdown (NaN)");
        break;
      }
      learned = false;
      fallbacks++;
      continue;
    }
    if (learned) k_copy_d<<<vb, kThreads, 0, s>>>(w.x64, w.rD, n);  // x before the step
    if (mixed)
      k_accumulate<float><<<vb, kThreads, 0, s>>>(w.x64, w.x32, w.scal, 9, n);
    else
      k_accumulate<double><<<vb, kThreads, 0, s>>>(w.x64, w.xD, w.scal, 9, n);
    double rn = 0.0;
    if ((st = refineResidual(ctx, w, b, &rn)) != IFEMGPU_OK) return st;
    const double next = rn / bn;
    if (learned && !(next < relres)) {
      // the FP64 residual judges the learned step: no progress -> undo it
      // and continue with plain Jacobi-PCG
      k_copy_d<<<vb, kThreads, 0, s>>>(w.rD, w.x64, n);
      if ((st = refineResidual(ctx, w, b, &rn)) != IFEMGPU_OK) return st;
      learned = false;
      fallbacks++;
      relres = rn / bn;
      continue;
    }
    relres = next;
  }
  IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(xh, w.x64, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
  if (info) *info = ifemgpu_solve_info{outer, inner, relres, (double)ms, fallbacks};
  if (st != IFEMGPU_OK) return st;
  if (bn > 0 && relres > o->rtol)
    return setError(ctx, IFEMGPU_NOT_CONVERGED, "relative residual above tolerance");
  return IFEMGPU_OK;
}

// ---------------------------------------------------------------------------
// One captured assemble -> solve step (ifemgpu_graph_capture / _launch): the
// pair SIMbase::assembleSystem -> SIMbase::solveEqSystem as a single CUDA
// graph.  Its nodes: the assembly's kernels, the solver prologue, and the
// FP64 refinement loop as a conditional WHILE node whose body runs one FP32
// inner solve -- itself a WHILE node over blocks of kLoopBlock iterations --
// then the FP64 residual.  Kernels decide both loop conditions from the same
// device scalars the host-driven solve reads (same FP64 operations), so a
// replay takes the same decisions as ifemgpu_assemble + ifemgpu_solve and
// gives the same bits.  Both loops end by construction: the inner stop flag
// is set at max_inner iterations (or NaN), the outer loop stops after
// max_outer refinement steps or on a failed inner solve.
namespace {

enum : int { S_OUT = 20, S_INN = 21, S_REL = 22, S_FAIL = 23 };

__global__ void k_step_init(cudaGraphConditionalHandle outer, double* s, double rtol, int maxOuter)
{
  s[S_OUT] = 0.0;
  s[S_INN] = 0.0;
  s[S_FAIL] = 0.0;
  const double bn = sqrt(s[8]);
  const double rel = bn > 0.0 ? 1.0 : 0.0;
  s[S_REL] = rel;
  cudaGraphSetConditional(outer, (bn > 0.0 && rel > rtol && maxOuter > 0) ? 1u : 0u);
}

__global__ void k_step_inner_cond(cudaGraphConditionalHandle inner, const double* s)
{
  cudaGraphSetConditional(inner, s[S_DONE] == 0.0 ? 1u : 0u);
}

// after an inner solve: count it; a breakdown (NaN or stagnation) ends the step
__global__ void k_step_inner_done(double* s)
{
  s[S_OUT] += 1.0;
  s[S_INN] += s[S_ITS];
  if (s[S_DONE] >= 2.0) s[S_FAIL] = 1.0;
}

// x64 += sqrt(scal[9]) x32 unless the inner solve failed
__global__ void k_step_accumulate(double* __restrict__ x64, const float* __restrict__ x32,
                                  const double* __restrict__ s, int n)
{
  if (s[S_FAIL] != 0.0) return;
  const double sc = sqrt(s[9]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x64[i] += sc * (double)x32[i];
}

// relative FP64 residual of the step and the outer loop condition
__global__ void k_step_outer_cond(cudaGraphConditionalHandle outer, double* s, double rtol,
                                  int maxOuter)
{
  if (s[S_FAIL] == 0.0) s[S_REL] = sqrt(s[9]) / sqrt(s[8]);
  const bool more = s[S_FAIL] == 0.0 && s[S_REL] > rtol && s[S_OUT] < (double)maxOuter;
  cudaGraphSetConditional(outer, more ? 1u : 0u);
}

}  // namespace

void dropStep(ifemgpu_ctx* ctx)
{
  if (ctx->stepExec) cudaGraphExecDestroy(ctx->stepExec);
  if (ctx->stepGraph) cudaGraphDestroy(ctx->stepGraph);
  ctx->stepExec = nullptr;
  ctx->stepGraph = nullptr;
  ctx->stepKey = nullptr;
  ctx->stepGen = -1;
}

// the current capture's dependency set -> a new node of `params` -> the new
// dependency set (the node itself)
static ifemgpu_status addNodeToCapture(ifemgpu_ctx* ctx, cudaGraphNodeParams* params,
                                       cudaGraphNode_t* node)
{
  cudaStream_t s = ctx->stream;
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  IFEMGPU_CUDA(ctx, cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &ndeps));
  if (cs != cudaStreamCaptureStatusActive)
    return setError(ctx, IFEMGPU_CUDA_ERROR, "internal: stream not capturing");
  IFEMGPU_CUDA(ctx, cudaGraphAddNode(node, g, deps, nullptr, ndeps, params));
  IFEMGPU_CUDA(ctx, cudaStreamUpdateCaptureDependencies(s, node, nullptr, 1,
                                                        cudaStreamSetCaptureDependencies));
  return IFEMGPU_OK;
}

// a WHILE node on `handle` appended to the capture; *body receives its body graph
static ifemgpu_status addWhile(ifemgpu_ctx* ctx, cudaGraphConditionalHandle handle,
                               cudaGraph_t* body)
{
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = handle;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  IFEMGPU_TRY(addNodeToCapture(ctx, &p, &node));
  *body = p.conditional.phGraph_out[0];
  return IFEMGPU_OK;
}

ifemgpu_status captureStep(ifemgpu_ctx* ctx, const ifemgpu_solver_options* o)
{
  if (o->method != IFEMGPU_PCG_MIXED)
    return setError(ctx, IFEMGPU_UNSUPPORTED,
                    "graph_capture: the captured step takes the mixed-precision method");
  if (o->precond != IFEMGPU_PRECOND_JACOBI && o->precond != IFEMGPU_PRECOND_KRONECKER)
    return setError(ctx, IFEMGPU_INVALID_ARG, "graph_capture: unknown preconditioner");
  if (o->max_inner < 1) return setError(ctx, IFEMGPU_INVALID_ARG, "graph_capture: max_inner < 1");
  const int n = ctx->neq;
  if (n == 0) return setError(ctx, IFEMGPU_INVALID_ARG, "graph_capture: no equations");
  const bool kron = o->precond == IFEMGPU_PRECOND_KRONECKER;
  dropStep(ctx);
  // settle everything a capture cannot do: the assembly's tuning, the
  // workspace, the inner-loop variants and the preconditioner set-up
  if (!ctx->tuned) {
    IFEMGPU_TRY(launchAssembly(ctx));
    IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  ifemgpu_status st = ensureWork(ctx, true);
  if (st != IFEMGPU_OK) return st;
  if (kron && (st = fdSetup(ctx)) != IFEMGPU_OK) return st;
  const Work w = carve(ctx);
  const int maxOuter = std::max(1, o->max_outer);
  const double innerTol = o->inner_rtol > 0 ? o->inner_rtol : 1e-4;
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  const int sb = std::min(kRedBlocks, (n + 7) / 8);
  cudaStream_t s = ctx->stream;
  cudaGraph_t g = nullptr;
  IFEMGPU_CUDA(ctx, cudaGraphCreate(&g, 0));
  ctx->stepGraph = g;
  cudaGraphConditionalHandle hOuter, hInner;  // each made on the graph that holds its node
  IFEMGPU_CUDA(ctx, cudaGraphConditionalHandleCreate(&hOuter, g, 0, 0));
  auto fail = [&](ifemgpu_status e) {
    cudaGraph_t junk = nullptr;
    cudaStreamCaptureStatus cs;
    if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
      cudaStreamEndCapture(s, &junk);
    cudaGetLastError();
    dropStep(ctx);
    return e;
  };
  // assembly, prologue, refinement loop
  IFEMGPU_CUDA(ctx, cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal));
  if ((st = enqueueAssembly(ctx)) != IFEMGPU_OK) return fail(st);
  k_convert<float><<<1024, kThreads, 0, s>>>(ctx->d_K, ctx->d_K32, ctx->nnz);
  k_diag<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K,
                                                              n, w.d64, w.dinv32);
  cudaMemsetAsync(w.x64, 0, sizeof(double) * n, s);
  k_norm2<double><<<vb, kThreads, 0, s>>>(ctx->d_b, n, w.part);
  k_finish<<<1, kThreads, 0, s>>>(w.part, vb, 1, w.scal + 8);
  cudaMemcpyAsync(w.r64, ctx->d_b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(w.scal + 9, w.scal + 8, sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (kron && (st = fdRescale(ctx, w.d64)) != IFEMGPU_OK) return fail(st);
  k_step_init<<<1, 1, 0, s>>>(hOuter, w.scal, o->rtol, maxOuter);
  if (cudaGetLastError() != cudaSuccess) return fail(setError(ctx, IFEMGPU_CUDA_ERROR, "graph_capture: prologue"));
  cudaGraph_t outerBody = nullptr;
  if ((st = addWhile(ctx, hOuter, &outerBody)) != IFEMGPU_OK) return fail(st);
  cudaGraph_t top = nullptr;
  IFEMGPU_CUDA(ctx, cudaStreamEndCapture(s, &top));
  IFEMGPU_CUDA(ctx, cudaGraphConditionalHandleCreate(&hInner, outerBody, 0, 0));
  // outer body: inner start, inner WHILE, accumulate, FP64 residual, condition
  IFEMGPU_CUDA(ctx, cudaStreamBeginCaptureToGraph(s, outerBody, nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal));
  st = kron ? fcgStart(ctx, w, true, false, innerTol, o->max_inner)
            : pcgStart(ctx, w, innerTol, o->max_inner);
  if (st != IFEMGPU_OK) return fail(st);
  k_step_inner_cond<<<1, 1, 0, s>>>(hInner, w.scal);
  cudaGraph_t innerBody = nullptr;
  if ((st = addWhile(ctx, hInner, &innerBody)) != IFEMGPU_OK) return fail(st);
  k_step_inner_done<<<1, 1, 0, s>>>(w.scal);
  k_step_accumulate<<<vb, kThreads, 0, s>>>(w.x64, w.x32, w.scal, n);
  k_residual<<<sb, kThreads, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K, w.x64, ctx->d_b, w.r64,
                                     n, w.part, ctx->d_rowPat, ctx->d_patStart, ctx->d_patOff);
  k_finish<<<1, kThreads, 0, s>>>(w.part, sb, 1, w.scal + 9);
  k_step_outer_cond<<<1, 1, 0, s>>>(hOuter, w.scal, o->rtol, maxOuter);
  if (cudaGetLastError() != cudaSuccess) return fail(setError(ctx, IFEMGPU_CUDA_ERROR, "graph_capture: outer body"));
  cudaGraph_t ob = nullptr;
  IFEMGPU_CUDA(ctx, cudaStreamEndCapture(s, &ob));
  // inner body: kLoopBlock iterations, then the inner condition
  IFEMGPU_CUDA(ctx, cudaStreamBeginCaptureToGraph(s, innerBody, nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < kLoopBlock && st == IFEMGPU_OK; k++)
    st = kron ? fcgIteration(ctx, w, true, false) : pcgIteration(ctx, w);
  if (st != IFEMGPU_OK) return fail(st);
  k_step_inner_cond<<<1, 1, 0, s>>>(hInner, w.scal);
  if (cudaGetLastError() != cudaSuccess) return fail(setError(ctx, IFEMGPU_CUDA_ERROR, "graph_capture: inner body"));
  cudaGraph_t ib = nullptr;
  IFEMGPU_CUDA(ctx, cudaStreamEndCapture(s, &ib));
  const cudaError_t e = cudaGraphInstantiate(&ctx->stepExec, g, 0);
  if (e != cudaSuccess) return fail(cudaFail(ctx, e, "cudaGraphInstantiate (assemble -> solve step)"));
  ctx->stepOpts = *o;
  ctx->stepKey = ctx->d_work;
  ctx->stepGen = ctx->workGen;
  return IFEMGPU_OK;
}

ifemgpu_status launchStep(ifemgpu_ctx* ctx, double* xh, ifemgpu_solve_info* info)
{
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  if (!ctx->stepExec) return setError(ctx, IFEMGPU_NOT_READY, "graph_launch before graph_capture");
  if (ctx->stepKey != ctx->d_work || ctx->stepGen != ctx->workGen) {  // the workspace moved
    const ifemgpu_solver_options o = ctx->stepOpts;
    IFEMGPU_TRY(captureStep(ctx, &o));
  }
  cudaStream_t s = ctx->stream;
  const int n = ctx->neq;
  const Work w = carve(ctx);
  IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
  IFEMGPU_CUDA(ctx, cudaGraphLaunch(ctx->stepExec, s));
  ctx->assemblies++;
  IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, w.scal + S_OUT, 4 * sizeof(double),
                                    cudaMemcpyDeviceToHost, s));
  if (xh) IFEMGPU_CUDA(ctx, cudaMemcpyAsync(xh, w.x64, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  ctx->assembled = true;
  ctx->checkPending = true;
  IFEMGPU_TRY(verifyAssembly(ctx));
  const double* h = ctx->h_pinned;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
  const double relres = h[2];
  if (info) *info = ifemgpu_solve_info{(int)h[0], (int)h[1], relres, (double)ms, 0};
  if (h[3] != 0.0) return setError(ctx, IFEMGPU_NOT_CONVERGED, "graph step: inner solve broke down");
  if (relres > ctx->stepOpts.rtol)
    return setError(ctx, IFEMGPU_NOT_CONVERGED, "relative residual above tolerance");
  return IFEMGPU_OK;
}

// z = M r for the FP32 preconditioner precond of the assembled matrix (host
// vectors; diagnostic)
ifemgpu_status applyPreconditioner(ifemgpu_ctx* ctx, int precond, const double* r, double* z)
{
  const int n = ctx->neq;
  cudaStream_t s = ctx->stream;
  if (precond != IFEMGPU_PRECOND_JACOBI && precond != IFEMGPU_PRECOND_KRONECKER)
    return setError(ctx, IFEMGPU_INVALID_ARG, "apply_preconditioner: unknown preconditioner");
  ifemgpu_status st = ensureWork(ctx, true);
  if (st != IFEMGPU_OK) return st;
  if (precond == IFEMGPU_PRECOND_KRONECKER && (st = fdSetup(ctx)) != IFEMGPU_OK) return st;
  if (n == 0) return IFEMGPU_OK;
  Work w = carve(ctx);
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  k_diag<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K,
                                                              n, w.d64, w.dinv32);
  const double one = 1.0;
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(w.scal + 9, &one, sizeof(double), cudaMemcpyHostToDevice, s));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(w.r64, r, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  g_fcg_start<<<vb, kThreads, 0, s>>>(w.r64, w.scal, w.r32, w.x32, w.z32, w.p32, w.q32, w.dinv32, n);
  if (precond == IFEMGPU_PRECOND_KRONECKER) {
    if ((st = fdRescale(ctx, w.d64)) != IFEMGPU_OK) return st;
    if ((st = fdApply(ctx, w.r32, w.z32, nullptr)) != IFEMGPU_OK) return st;
  }
  std::vector<float> zf(n);
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(zf.data(), w.z32, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  for (int i = 0; i < n; i++) z[i] = zf[i];
  return IFEMGPU_OK;
}

// Training pairs from one FP32 solve of A x = rhs (the assembled b when rhs
// is null) from x = 0 -- Jacobi-PCG, or flexible CG with the Kronecker
// preconditioner (the iteration the network will serve): every stride-th
// iterate gives one pair (learnRecord).  x* is the caller's reference
// solution, or the FP64-refined mixed solve to 1e-12 with the same
// preconditioner when xstar is null.
ifemgpu_status collectPairs(ifemgpu_ctx* ctx, const double* rhs, const double* xstar, int stride,
                            int maxit, double rtol, int precond)
{
  if (precond != IFEMGPU_PRECOND_JACOBI && precond != IFEMGPU_PRECOND_KRONECKER)
    return setError(ctx, IFEMGPU_INVALID_ARG, "learn_collect: unknown preconditioner");
  const int n = ctx->neq;
  cudaStream_t s = ctx->stream;
  double* xs = learnXstar(ctx);
  if (!xs) return setError(ctx, IFEMGPU_NOT_READY, "learn_collect before learn_setup");
  if (n == 0) return IFEMGPU_OK;
  const double* b = ctx->d_b;
  if (rhs) {
    if (!ctx->d_rhsAlt) IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_rhsAlt, sizeof(double) * n));
    IFEMGPU_CUDA(ctx, cudaMemcpy(ctx->d_rhsAlt, rhs, sizeof(double) * n, cudaMemcpyHostToDevice));
    b = ctx->d_rhsAlt;
  }
  ifemgpu_status st;
  if (xstar) {
    IFEMGPU_CUDA(ctx, cudaMemcpy(xs, xstar, sizeof(double) * n, cudaMemcpyHostToDevice));
  } else {
    std::vector<double> xh(n);
    ifemgpu_solver_options so{IFEMGPU_PCG_MIXED, 1e-12, 40, 100000, 1e-5, precond};
    ifemgpu_solve_info si{};
    st = runSolve(ctx, &so, xh.data(), &si, b);
    if (st != IFEMGPU_OK && !(st == IFEMGPU_NOT_CONVERGED && si.relres < 1e-9)) return st;
    IFEMGPU_CUDA(ctx, cudaMemcpy(xs, xh.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  }
  if ((st = ensureWork(ctx, true)) != IFEMGPU_OK) return st;
  if ((st = learnPrepare(ctx)) != IFEMGPU_OK) return st;
  Work w = carve(ctx);
  double bn = 0.0;
  if ((st = solvePrologue(ctx, w, b, true, &bn)) != IFEMGPU_OK) return st;
  if (!(bn > 0)) return IFEMGPU_OK;
  const bool kron = precond == IFEMGPU_PRECOND_KRONECKER;
  // complement pairs take the collecting iteration's fine preconditioner
  // output for r_k (z: Kronecker along flexible CG, Jacobi along PCG) and
  // its product t = A z
  const bool complement = learnTarget(ctx) == IFEMGPU_LEARN_TARGET_COMPLEMENT;
  if (kron) {
    if ((st = fdSetup(ctx)) != IFEMGPU_OK) return st;
    if ((st = fdRescale(ctx, w.d64)) != IFEMGPU_OK) return st;
  }
  const double sx = 1.0 / bn;  // the loop solves the system scaled by 1/||b||
  auto record = [&]() -> ifemgpu_status {
    float* t = nullptr;
    if (complement) {
      t = learnT(ctx);
      spmv32(ctx, w, w.z32, t, -1);
    }
    return learnRecord(ctx, w.r32, w.x32, sx, complement ? w.z32 : nullptr, t);
  };
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  unsigned* tk = hostTickets(w);
  k_loop_init<<<1, 1, 0, s>>>(w.scal, rtol * rtol, (double)maxit, 0.0);
  if (kron) {  // flexible CG with the Kronecker preconditioner
    g_fcg_start<<<vb, kThreads, 0, s>>>(w.r64, w.scal, w.r32, w.x32, w.z32, w.p32, w.q32, w.dinv32, n);
    if ((st = fdApply(ctx, w.r32, w.z32, w.scal + S_DONE)) != IFEMGPU_OK) return st;
    g_fcg_dir<<<vb, kThreads, 0, s>>>(w.p32, w.z32, w.r32, w.scal, n, w.part);
  } else {
    g_pcg_start<float><<<vb, kThreads, 0, s>>>(w.r64, w.scal, w.r32, w.x32, w.z32, w.p32, w.dinv32,
                                               n, w.part);
  }
  if ((st = record()) != IFEMGPU_OK) return st;
  stride = std::max(1, stride);
  for (int l = 0; l <= maxit / stride; l++) {
    for (int k = 0; k < stride; k++) {
      if (kron) {
        spmv32(ctx, w, w.p32, w.q32, 0);
        g_fcg_update<<<vb, kThreads, 0, s>>>(w.x32, w.r32, w.z32, w.p32, w.q32, w.dinv32, w.scal,
                                             n, w.part);
        if ((st = fdApply(ctx, w.r32, w.z32, w.scal + S_DONE)) != IFEMGPU_OK) return st;
        g_dot<<<vb, kThreads, 0, s>>>(w.z32, w.q32, n, w.part, tk + 2, w.scal);
        g_fcg_dir<<<vb, kThreads, 0, s>>>(w.p32, w.z32, w.r32, w.scal, n, w.part);
      } else {
        spmv32(ctx, w, w.p32, w.q32, 1);
        g_pcg_update<float><<<vb, kThreads, 0, s>>>(w.x32, w.r32, w.z32, w.p32, w.q32, w.dinv32,
                                                    w.scal, n, w.part);
        g_pcg_dir<float><<<vb, kThreads, 0, s>>>(w.p32, w.z32, w.scal, n);
      }
    }
    IFEMGPU_CUDA(ctx, cudaGetLastError());
    IFEMGPU_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, w.scal + S_DONE, sizeof(double),
                                      cudaMemcpyDeviceToHost, s));
    IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
    if (ctx->h_pinned[0] != 0.0) break;
    if ((st = record()) != IFEMGPU_OK) return st;
  }
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  return IFEMGPU_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free FP64 solve (ifemgpu_solve_noalloc).  Its workspace is one
// file-scope device array, the same on every call: 11 * 65,536 doubles for
// the vectors plus the reduction partials, about 5.8 MB, held by every GPU
// that loads the library.  Host code reaches it through the address that
// cudaGetSymbolAddress returns for the current device (the array's name in
// host code is only a host-side stand-in).  The address is looked up at the
// first call on a device and kept; the primary context of that device must
// not be reset (cudaDeviceReset) while the library is in use.  The scalars
// read back during a solve go through a stack variable of the call (a
// pageable copy followed by a stream synchronisation allocates nothing), so
// calls from several host threads share no host memory.
constexpr int kNoAllocMaxEq = 65536;
constexpr size_t kNoAllocWords = (size_t)kNoAllocMaxEq * 11 + 2 * kRedBlocks + 16;
static __device__ __align__(256) double g_noallocWork[kNoAllocWords];
constexpr int kMaxDevices = 64;
static double* g_noallocAddr[kMaxDevices] = {};  // device address per device ordinal

static Work carveFrom(double* base, size_t n)
{
  Work w{};
  w.x64 = base; base += n;
  w.r64 = base; base += n;
  w.d64 = base; base += n;
  w.part = base; base += 2 * kRedBlocks;
  w.scal = base; base += 16;
  w.rD = base; base += n;
  w.xD = base; base += n;
  w.zD = base; base += n;
  w.pD = base; base += n;
  w.qD = base; base += n;
  float* fb = reinterpret_cast<float*>(base);
  w.r32 = fb; fb += n;
  w.x32 = fb; fb += n;
  w.z32 = fb; fb += n;
  w.p32 = fb; fb += n;
  w.q32 = fb; fb += n;
  w.dinv32 = fb; fb += n;
  return w;
}

// FP64 Jacobi-PCG of innerPCG with the convergence scalar read through a
// caller-given host buffer instead of the context's pinned buffer.
static ifemgpu_status innerPCG64(ifemgpu_ctx* ctx, const Work& w, double rtol, int maxit,
                                 double* hostScalar, int* iters)
{
  cudaStream_t s = ctx->stream;
  const int n = ctx->neq;
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  const int sb = std::min(kRedBlocks, (n + 7) / 8);
  k_pcg_start<double><<<vb, kThreads, 0, s>>>(w.r64, w.scal, 9, w.rD, w.xD, w.zD, w.pD, w.d64, n,
                                              w.part);
  k_finish<<<1, kThreads, 0, s>>>(w.part, vb, 1, w.scal + 0);
  int it = 0;
  while (it < maxit) {
    for (int k = 0; k < 16 && it < maxit; k++, it++) {
      k_spmv<double><<<sb, kThreads, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K, w.pD, w.qD, n,
                                             w.part);
      k_finish<<<1, kThreads, 0, s>>>(w.part, sb, 1, w.scal + 1);
      k_pcg_update<double><<<vb, kThreads, 0, s>>>(w.xD, w.rD, w.zD, w.pD, w.qD, w.d64, w.scal, n,
                                                   w.part);
      k_finish<<<1, kThreads, 0, s>>>(w.part, vb, 2, w.scal + 2);
      k_pcg_dir<double><<<vb, kThreads, 0, s>>>(w.pD, w.zD, w.scal, n);
      k_shift_scalars<<<1, 1, 0, s>>>(w.scal);
    }
    IFEMGPU_CUDA(ctx, cudaGetLastError());
    IFEMGPU_CUDA(ctx, cudaMemcpyAsync(hostScalar, w.scal + 3, sizeof(double),
                                      cudaMemcpyDeviceToHost, s));
    IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
    const double rr = hostScalar[0];
    if (!(rr == rr)) { *iters = it; return setError(ctx, IFEMGPU_NOT_CONVERGED, "PCG breakdown (NaN)"); }
    if (std::sqrt(rr) <= rtol) break;
  }
  *iters = it;
  return IFEMGPU_OK;
}

ifemgpu_status solveNoAlloc(ifemgpu_ctx* ctx, double rtol, int maxit, double* xh,
                            ifemgpu_solve_info* info)
{
  const int n = ctx->neq;
  if (n > kNoAllocMaxEq)
    return setError(ctx, IFEMGPU_INVALID_ARG,
                    "ifemgpu_solve_noalloc: more than 65536 equations (its fixed workspace)");
  if (ctx->opts.device < 0 || ctx->opts.device >= kMaxDevices)
    return setError(ctx, IFEMGPU_INVALID_ARG, "ifemgpu_solve_noalloc: unsupported device ordinal");
  if (n == 0) {
    if (info) *info = ifemgpu_solve_info{0, 0, 0.0, 0.0};
    return IFEMGPU_OK;
  }
  double*& base = g_noallocAddr[ctx->opts.device];
  if (!base) IFEMGPU_CUDA(ctx, cudaGetSymbolAddress((void**)&base, g_noallocWork));
  cudaStream_t s = ctx->stream;
  const Work w = carveFrom(base, (size_t)n);
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  const int sb = std::min(kRedBlocks, (n + 7) / 8);
  IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
  k_diag<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K,
                                                              n, w.d64, w.dinv32);
  // the accumulated solution starts at zero; every other workspace entry is
  // written before it is read
  IFEMGPU_CUDA(ctx, cudaMemsetAsync(w.x64, 0, sizeof(double) * n, s));
  k_norm2<double><<<vb, kThreads, 0, s>>>(ctx->d_b, n, w.part);
  k_finish<<<1, kThreads, 0, s>>>(w.part, vb, 1, w.scal + 8);
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(w.r64, ctx->d_b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(w.scal + 9, w.scal + 8, sizeof(double), cudaMemcpyDeviceToDevice, s));
  double hostScalar = 0.0;  // pageable, per call
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(&hostScalar, w.scal + 8, sizeof(double), cudaMemcpyDeviceToHost, s));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  const double bn = std::sqrt(hostScalar);
  int inner = 0, outer = 0;
  double relres = bn > 0 ? 1.0 : 0.0;
  ifemgpu_status st = IFEMGPU_OK;
  if (bn > 0) {
    st = innerPCG64(ctx, w, rtol, maxit, &hostScalar, &inner);
    outer = 1;
    if (st == IFEMGPU_OK) {
      k_accumulate<double><<<vb, kThreads, 0, s>>>(w.x64, w.xD, w.scal, 9, n);
      k_residual<<<sb, kThreads, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K, w.x64, ctx->d_b,
                                         w.r64, n, w.part);
      k_finish<<<1, kThreads, 0, s>>>(w.part, sb, 1, w.scal + 9);
      IFEMGPU_CUDA(ctx, cudaGetLastError());
      IFEMGPU_CUDA(ctx, cudaMemcpyAsync(&hostScalar, w.scal + 9, sizeof(double),
                                        cudaMemcpyDeviceToHost, s));
      IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
      relres = std::sqrt(hostScalar) / bn;
    }
  }
  IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(xh, w.x64, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
  if (info) *info = ifemgpu_solve_info{outer, inner, relres, (double)ms};
  if (st != IFEMGPU_OK) return st;
  if (bn > 0 && relres > rtol)
    return setError(ctx, IFEMGPU_NOT_CONVERGED, "relative residual above tolerance");
  return IFEMGPU_OK;
}

}  // namespace ifemgpu

extern "C" ifemgpu_status ifemgpu_apply_preconditioner(ifemgpu_ctx* ctx, int precond,
                                                       const double* r, double* z)
{
  if (!ctx || !r || !z) return IFEMGPU_INVALID_ARG;
  if (!ctx->assembled)
    return ifemgpu::setError(ctx, IFEMGPU_NOT_READY, "apply_preconditioner before assemble");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  return ifemgpu::applyPreconditioner(ctx, precond, r, z);
}

extern "C" ifemgpu_status ifemgpu_solve_noalloc(ifemgpu_ctx* ctx, double rtol, int max_iter,
                                                double* x, ifemgpu_solve_info* info)
{
  if (!ctx || !x || max_iter < 1) return IFEMGPU_INVALID_ARG;
  if (!ctx->assembled)
    return ifemgpu::setError(ctx, IFEMGPU_NOT_READY, "solve before assemble");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  return ifemgpu::solveNoAlloc(ctx, rtol, max_iter, x, info);
}

extern "C" ifemgpu_status ifemgpu_graph_capture(ifemgpu_ctx* ctx, const ifemgpu_solver_options* opts)
{
  if (!ctx || !opts) return IFEMGPU_INVALID_ARG;
  if (!ctx->preprocessed || ctx->opts.device < 0)
    return ifemgpu::setError(ctx, IFEMGPU_NOT_READY, "graph_capture before preprocess");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  return ifemgpu::captureStep(ctx, opts);
}

extern "C" ifemgpu_status ifemgpu_graph_launch(ifemgpu_ctx* ctx, double* x, ifemgpu_solve_info* info)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  return ifemgpu::launchStep(ctx, x, info);
}
