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

#include "ifemgpu_internal.h"

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

// r = b - A x in FP64, partial of ||r||^2
__global__ void __launch_bounds__(kThreads)
k_residual(const int* __restrict__ colptr, const int* __restrict__ rowidx,
           const double* __restrict__ A, const double* __restrict__ x,
           const double* __restrict__ b, double* __restrict__ r, int n, double* __restrict__ part)
{
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31;
  const int warpsPerGrid = gridDim.x * (blockDim.x >> 5);
  double acc = 0.0;
  for (int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < n; row += warpsPerGrid) {
    const int c0 = colptr[row], c1 = colptr[row + 1];
    double s = 0.0;
    for (int k = c0 + lane; k < c1; k += 32) s += A[k] * x[rowidx[k]];
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

}  // namespace

// Workspace layout (doubles): x64, r64, dinv64 | part (2*kRedBlocks) | scal(16)
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

void freeSolver(ifemgpu_ctx* ctx)
{
  if (ctx->d_K32) cudaFree(ctx->d_K32);
  if (ctx->d_work) cudaFree(ctx->d_work);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
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

ifemgpu_status runSolve(ifemgpu_ctx* ctx, const ifemgpu_solver_options* o, double* xh,
                        ifemgpu_solve_info* info)
{
  const int n = ctx->neq;
  cudaStream_t s = ctx->stream;
  if (n == 0) {
    if (info) *info = ifemgpu_solve_info{0, 0, 0.0, 0.0};
    return IFEMGPU_OK;
  }
  const size_t need = sizeof(double) * ((size_t)n * 8 + 2 * kRedBlocks + 16) + sizeof(float) * (size_t)n * 6;
  if (ctx->work_len < need) {
    if (ctx->d_work) cudaFree(ctx->d_work);
    IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_work, need));
    ctx->work_len = need;
  }
  if (!ctx->h_pinned) IFEMGPU_CUDA(ctx, cudaMallocHost(&ctx->h_pinned, 64));
  const bool mixed = o->method != IFEMGPU_PCG_FP64;
  if (mixed && !ctx->d_K32) IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_K32, sizeof(float) * ctx->nnz));
  Work w = carve(ctx);
  const int vb = std::min(kRedBlocks, (n + kThreads - 1) / kThreads);
  const int sb = std::min(kRedBlocks, (n + 7) / 8);
  IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
  if (mixed) k_convert<float><<<1024, kThreads, 0, s>>>(ctx->d_K, ctx->d_K32, ctx->nnz);
  k_diag<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K,
                                                              n, w.d64, w.dinv32);
  IFEMGPU_CUDA(ctx, cudaMemsetAsync(w.x64, 0, sizeof(double) * n, s));
  // ||b||^2 -> scal[8]
  k_norm2<double><<<vb, kThreads, 0, s>>>(ctx->d_b, n, w.part);
  k_finish<<<1, kThreads, 0, s>>>(w.part, vb, 1, w.scal + 8);
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(w.r64, ctx->d_b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(w.scal + 9, w.scal + 8, sizeof(double), cudaMemcpyDeviceToDevice, s));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, w.scal + 8, sizeof(double), cudaMemcpyDeviceToHost, s));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  const double bn = std::sqrt(ctx->h_pinned[0]);
  int outer = 0, inner = 0;
  double relres = bn > 0 ? 1.0 : 0.0;
  ifemgpu_status st = IFEMGPU_OK;
  const int maxOuter = mixed ? std::max(1, o->max_outer) : 1;
  const double innerTol = mixed ? (o->inner_rtol > 0 ? o->inner_rtol : 1e-4) : o->rtol;
  while (bn > 0 && relres > o->rtol && outer < maxOuter) {
    int it = 0;
    if (mixed)
      st = innerPCG<float>(ctx, w, ctx->d_K32, w.dinv32, w.r32, w.x32, w.z32, w.p32, w.q32, 9,
                           innerTol, o->max_inner, &it);
    else
      st = innerPCG<double>(ctx, w, ctx->d_K, w.d64, w.rD, w.xD, w.zD, w.pD, w.qD, 9, innerTol,
                            o->max_inner, &it);
    inner += it;
    outer++;
    if (st != IFEMGPU_OK) break;
    if (mixed)
      k_accumulate<float><<<vb, kThreads, 0, s>>>(w.x64, w.x32, w.scal, 9, n);
    else
      k_accumulate<double><<<vb, kThreads, 0, s>>>(w.x64, w.xD, w.scal, 9, n);
    k_residual<<<sb, kThreads, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K, w.x64, ctx->d_b,
                                       w.r64, n, w.part);
    k_finish<<<1, kThreads, 0, s>>>(w.part, sb, 1, w.scal + 9);
    IFEMGPU_CUDA(ctx, cudaGetLastError());
    IFEMGPU_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, w.scal + 9, sizeof(double), cudaMemcpyDeviceToHost, s));
    IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
    relres = std::sqrt(ctx->h_pinned[0]) / bn;
  }
  IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(xh, w.x64, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
  if (info) *info = ifemgpu_solve_info{outer, inner, relres, (double)ms};
  if (st != IFEMGPU_OK) return st;
  if (bn > 0 && relres > o->rtol)
    return setError(ctx, IFEMGPU_NOT_CONVERGED, "relative residual above tolerance");
  return IFEMGPU_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free FP64 solve (ifemgpu_solve_noalloc).  Its workspace is one
// file-scope device array, the same on every call: 11 * 65,536 doubles for
// the vectors plus the reduction partials, about 5.8 MB, held by every GPU
// that loads the library.  Host code reaches it through the address that
// cudaGetSymbolAddress returns for the current device (the array's name in
// host code is only a host-side stand-in).
constexpr int kNoAllocMaxEq = 65536;
constexpr size_t kNoAllocWords = (size_t)kNoAllocMaxEq * 11 + 2 * kRedBlocks + 16;
static __device__ __align__(256) double g_noallocWork[kNoAllocWords];
constexpr int kMaxDevices = 64;
static double* g_noallocAddr[kMaxDevices] = {};  // device address per device ordinal
static double g_noallocScalar[2];                // pageable host copy of one reduced scalar

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
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(g_noallocScalar, w.scal + 8, sizeof(double), cudaMemcpyDeviceToHost, s));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  const double bn = std::sqrt(g_noallocScalar[0]);
  int inner = 0, outer = 0;
  double relres = bn > 0 ? 1.0 : 0.0;
  ifemgpu_status st = IFEMGPU_OK;
  if (bn > 0) {
    st = innerPCG64(ctx, w, rtol, maxit, g_noallocScalar, &inner);
    outer = 1;
    if (st == IFEMGPU_OK) {
      k_accumulate<double><<<vb, kThreads, 0, s>>>(w.x64, w.xD, w.scal, 9, n);
      k_residual<<<sb, kThreads, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K, w.x64, ctx->d_b,
                                         w.r64, n, w.part);
      k_finish<<<1, kThreads, 0, s>>>(w.part, sb, 1, w.scal + 9);
      IFEMGPU_CUDA(ctx, cudaGetLastError());
      IFEMGPU_CUDA(ctx, cudaMemcpyAsync(g_noallocScalar, w.scal + 9, sizeof(double),
                                        cudaMemcpyDeviceToHost, s));
      IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
      relres = std::sqrt(g_noallocScalar[0]) / bn;
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

extern "C" ifemgpu_status ifemgpu_solve_noalloc(ifemgpu_ctx* ctx, double rtol, int max_iter,
                                                double* x, ifemgpu_solve_info* info)
{
  if (!ctx || !x || max_iter < 1) return IFEMGPU_INVALID_ARG;
  if (!ctx->assembled)
    return ifemgpu::setError(ctx, IFEMGPU_NOT_READY, "solve before assemble");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  return ifemgpu::solveNoAlloc(ctx, rtol, max_iter, x, info);
}
