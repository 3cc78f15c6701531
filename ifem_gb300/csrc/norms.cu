// norms.cu -- solution norms and the secondary solution at the Gauss points.
//
// IFEM integrates norms through NormBase integrands driven by
// SIMbase::solutionNorms (src/SIM/SIMbase.C:1838-1967) and evaluates the
// secondary solution through ASMs3D::evalSolution (src/ASM/ASMs3D.C:
// 3179-3500); the applications' integrands define
//   Poisson:     a(u, u) = int kappa grad u . grad u,  secondary: flux -kappa grad u
//   elasticity:  a(u, u) = int sigma(u) : eps(u),      secondary: stress sigma
//                (Voigt order xx yy zz xy yz zx)
// and the L2 norm int u . u.  One CTA integrates one element with the Gauss
// rules and 1D basis tables of the last assembly: point arithmetic in FP32
// (split mode) or FP64, the Jacobian determinant and inverse in FP64,
// element sums in FP64, the totals by one fixed-order block (deterministic).
#include <algorithm>
#include <vector>

#include "ifemgpu_internal.h"

namespace ifemgpu {

namespace {

constexpr int kNT = 128;

__device__ inline int normElemNode(const DevPatch& P, int e, int a)
{
  const int q1 = P.p[0] + 1, q2 = P.p[1] + 1;
  const int e1 = e % P.nel[0], e2 = (e / P.nel[0]) % P.nel[1], e3 = e / (P.nel[0] * P.nel[1]);
  const int i = a % q1, j = (a / q1) % q2, k = a / (q1 * q2);
  return ((e3 + k) * P.n[1] + e2 + j) * P.n[0] + e1 + i;
}

template <typename T> __device__ inline const T* tabN(const DevPatch& P, int d);
template <typename T> __device__ inline const T* tabD(const DevPatch& P, int d);
template <> __device__ inline const double* tabN<double>(const DevPatch& P, int d) { return P.tabN[d]; }
template <> __device__ inline const double* tabD<double>(const DevPatch& P, int d) { return P.tabD[d]; }
template <> __device__ inline const float* tabN<float>(const DevPatch& P, int d) { return P.tabNf[d]; }
template <> __device__ inline const float* tabD<float>(const DevPatch& P, int d) { return P.tabDf[d]; }

// Shared memory: Xn[nen][4] (relative coordinates, weight), U[nen][npv],
// G[nen] (log-conductivity), red[2][kNT / 32]
template <typename T>
__global__ void __launch_bounds__(kNT)
k_norms(const DevPatch* __restrict__ patches, const Item* __restrict__ items,
        const int* __restrict__ madof, const double* __restrict__ u, double* __restrict__ elemOut,
        double* __restrict__ secOut, int secPatch)
{
  extern __shared__ __align__(16) unsigned char smraw[];
  const Item it = items[blockIdx.x];
  const DevPatch& P = patches[it.patch];
  const int nen = P.nen, nq = P.nq, dim = P.dim, npv = P.npv, e = it.elem;
  T* Xn = reinterpret_cast<T*>(smraw);
  T* U = Xn + 4 * nen;
  T* Gk = U + 3 * nen;
  double* red = reinterpret_cast<double*>(Gk + nen);  // 8 nen values: 8-byte aligned
  const double* c00 = P.ctrl + (size_t)normElemNode(P, e, 0) * 4;
  for (int a = threadIdx.x; a < nen; a += blockDim.x) {
    const int node = normElemNode(P, e, a);
    for (int c = 0; c < 3; c++) Xn[a * 4 + c] = (T)(P.ctrl[(size_t)node * 4 + c] - c00[c]);
    Xn[a * 4 + 3] = (T)P.ctrl[(size_t)node * 4 + 3];
    const int d0 = madof[globalNode(P, node)] - 1;
    for (int c = 0; c < 3; c++) U[a * 3 + c] = c < npv ? (T)u[d0 + c] : T(0);
    Gk[a] = P.logk ? (T)P.logk[node] : T(0);
  }
  __syncthreads();

  const int e1 = e % P.nel[0], e2 = (e / P.nel[0]) % P.nel[1], e3 = e / (P.nel[0] * P.nel[1]);
  const int q1 = P.p[0] + 1, q2 = P.p[1] + 1, q3 = dim == 3 ? P.p[2] + 1 : 1;
  const double lam = P.lam, mu = P.mu;
  double eSum = 0.0, lSum = 0.0;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    const int gi = q % P.ng[0], gj = (q / P.ng[0]) % P.ng[1], gz = q / (P.ng[0] * P.ng[1]);
    const T* n0 = tabN<T>(P, 0) + ((size_t)e1 * P.ng[0] + gi) * q1;
    const T* d0 = tabD<T>(P, 0) + ((size_t)e1 * P.ng[0] + gi) * q1;
    const T* n1 = tabN<T>(P, 1) + ((size_t)e2 * P.ng[1] + gj) * q2;
    const T* d1 = tabD<T>(P, 1) + ((size_t)e2 * P.ng[1] + gj) * q2;
    const T* n2 = dim == 3 ? tabN<T>(P, 2) + ((size_t)e3 * P.ng[2] + gz) * q3 : nullptr;
    const T* d2 = dim == 3 ? tabD<T>(P, 2) + ((size_t)e3 * P.ng[2] + gz) * q3 : nullptr;
    // homogeneous sums over the element's functions: weight, position,
    // solution and log-conductivity with their parametric derivatives
    T W = 0, Wd[3] = {0, 0, 0}, SX[3] = {0, 0, 0}, SXd[3][3] = {}, SU[3] = {0, 0, 0},
      SUd[3][3] = {}, SG = 0;
    for (int a = 0; a < nen; a++) {
      const int i = a % q1, j = (a / q1) % q2, k = a / (q1 * q2);
      const T nz = dim == 3 ? n2[k] : T(1), dz = dim == 3 ? d2[k] : T(0);
      const T w = Xn[a * 4 + 3];
      const T N = w * n0[i] * n1[j] * nz;
      const T D[3] = {w * d0[i] * n1[j] * nz, w * n0[i] * d1[j] * nz, w * n0[i] * n1[j] * dz};
      W += N;
      SG += N * Gk[a];
      for (int d = 0; d < 3; d++) Wd[d] += D[d];
      for (int r = 0; r < 3; r++) {
        SX[r] += N * Xn[a * 4 + r];
        SU[r] += N * U[a * 3 + r];
        for (int d = 0; d < 3; d++) {
          SXd[r][d] += D[d] * Xn[a * 4 + r];
          SUd[r][d] += D[d] * U[a * 3 + r];
        }
      }
    }
    const T iW = T(1) / W;
    T uh[3], Gu[3][3];
    double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 1};  // J[d*3 + r] = dX_r/du_d
    for (int r = 0; r < 3; r++) {
      const T X = SX[r] * iW;
      uh[r] = SU[r] * iW;
      for (int d = 0; d < dim; d++) {
        if (r < dim) J[d * 3 + r] = (double)((SXd[r][d] - X * Wd[d]) * iW);
        Gu[r][d] = (SUd[r][d] - uh[r] * Wd[d]) * iW;
      }
      for (int d = dim; d < 3; d++) Gu[r][d] = 0;
    }
    // FP64 determinant and inverse: Bi[r*3 + d] = du_d/dX_r
    double det, Bi[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (dim == 3) {
      const double c0 = J[4] * J[8] - J[5] * J[7], c1 = J[1] * J[8] - J[2] * J[7],
                   c2 = J[1] * J[5] - J[2] * J[4];
      det = J[0] * c0 - J[3] * c1 + J[6] * c2;
      if (fabs(det) > kEpsZ) {
        const double id = 1.0 / det;
        Bi[0] = c0 * id;
        Bi[3] = -(J[3] * J[8] - J[5] * J[6]) * id;
        Bi[6] = (J[3] * J[7] - J[4] * J[6]) * id;
        Bi[1] = -c1 * id;
        Bi[4] = (J[0] * J[8] - J[2] * J[6]) * id;
        Bi[7] = -(J[0] * J[7] - J[1] * J[6]) * id;
        Bi[2] = c2 * id;
        Bi[5] = -(J[0] * J[5] - J[2] * J[3]) * id;
        Bi[8] = (J[0] * J[4] - J[1] * J[3]) * id;
      }
    } else {
      det = J[0] * J[4] - J[1] * J[3];
      if (fabs(det) > kEpsZ) {
        const double id = 1.0 / det;
        Bi[0] = J[4] * id;
        Bi[1] = -J[1] * id;
        Bi[3] = -J[3] * id;
        Bi[4] = J[0] * id;
      }
    }
    if (!(fabs(det) > kEpsZ)) continue;  // singular point: skipped as in the assembly
    double dV = (dim == 3 ? 0.125 : 0.25) * P.span[0][e1] * P.span[1][e2];
    if (dim == 3) dV *= P.span[2][e3] * P.gw[2][gz];
    const double wq = det * dV * P.gw[0][gi] * P.gw[1][gj];
    // grad u: gu[c][r] = sum_d (du_c/du_d) (du_d/dX_r)
    double gu[3][3];
    for (int c = 0; c < 3; c++)
      for (int r = 0; r < 3; r++) {
        double v = 0.0;
        for (int d = 0; d < dim; d++) v += (double)Gu[c][d] * Bi[r * 3 + d];
        gu[c][r] = v;
      }
    double energy, sec[6] = {0, 0, 0, 0, 0, 0};
    if (P.kind == IFEMGPU_POISSON) {
      double kap = P.kappa;
      if (P.logk) kap *= exp((double)(SG * iW));
      energy = kap * (gu[0][0] * gu[0][0] + gu[0][1] * gu[0][1] + gu[0][2] * gu[0][2]);
      for (int r = 0; r < dim; r++) sec[r] = -kap * gu[0][r];
    } else {
      const double exx = gu[0][0], eyy = gu[1][1], ezz = gu[2][2];
      const double gxy = gu[0][1] + gu[1][0], gyz = gu[1][2] + gu[2][1], gzx = gu[2][0] + gu[0][2];
      const double tr = exx + eyy + ezz;
      sec[0] = lam * tr + 2.0 * mu * exx;
      sec[1] = lam * tr + 2.0 * mu * eyy;
      sec[2] = lam * tr + 2.0 * mu * ezz;
      sec[3] = mu * gxy;
      sec[4] = mu * gyz;
      sec[5] = mu * gzx;
      energy = sec[0] * exx + sec[1] * eyy + sec[2] * ezz + sec[3] * gxy + sec[4] * gyz + sec[5] * gzx;
    }
    double l2 = 0.0;
    for (int c = 0; c < npv; c++) l2 += (double)uh[c] * (double)uh[c];
    eSum += wq * energy;
    lSum += wq * l2;
    if (secOut && it.patch == secPatch) {
      const int nc = P.kind == IFEMGPU_POISSON ? dim : 6;
      for (int c = 0; c < nc; c++) secOut[((size_t)e * nq + q) * nc + c] = sec[c];
    }
  }
  // fixed-order block sums
  for (int o = 16; o > 0; o >>= 1) {
    eSum += __shfl_down_sync(0xffffffffu, eSum, o);
    lSum += __shfl_down_sync(0xffffffffu, lSum, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    red[warp] = eSum;
    red[kNT / 32 + warp] = lSum;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < kNT / 32; w++) {
      a += red[w];
      b += red[kNT / 32 + w];
    }
    elemOut[2 * (size_t)it.bc] = a;
    elemOut[2 * (size_t)it.bc + 1] = b;
  }
}

// totals of the element values in a fixed order: one block, strided partial
// sums per thread, then a fixed-order tree
__global__ void __launch_bounds__(256) k_norm_totals(const double* __restrict__ elem, int n,
                                                     double* __restrict__ out)
{
  __shared__ double s0[256], s1[256];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    a += elem[2 * (size_t)i];
    b += elem[2 * (size_t)i + 1];
  }
  s0[threadIdx.x] = a;
  s1[threadIdx.x] = b;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      s0[threadIdx.x] += s0[threadIdx.x + h];
      s1[threadIdx.x] += s1[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s0[0];
    out[1] = s1[0];
  }
}

size_t normSmem(const DevPatch& D, bool fp64)
{
  const size_t t = fp64 ? sizeof(double) : sizeof(float);
  return t * (8 * (size_t)D.nen + 2) + sizeof(double) * (2 * (kNT / 32) + 1);
}

ifemgpu_status prepareNorms(ifemgpu_ctx* ctx)
{
  if (ctx->d_normItems) return IFEMGPU_OK;
  std::vector<Item> items;
  ctx->normBase.assign(ctx->patches.size(), 0);
  int slot = 0;
  for (size_t pi = 0; pi < ctx->patches.size(); pi++) {
    const HostPatch& pc = ctx->patches[pi];
    ctx->normBase[pi] = slot;
    for (int e = 0; e < pc.nelAll; e++)
      if (pc.active[e]) items.push_back({(int)pi, e, 0, slot + e});
    slot += pc.nelAll;
  }
  ctx->nNormItems = (int)items.size();
  ctx->nNormSlots = slot;
  IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_normItems, sizeof(Item) * std::max<size_t>(items.size(), 1)));
  IFEMGPU_CUDA(ctx, cudaMemcpy(ctx->d_normItems, items.data(), sizeof(Item) * items.size(),
                               cudaMemcpyHostToDevice));
  const size_t len = (size_t)ctx->ndof + 2 * (size_t)slot + 2;
  IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_normBuf, sizeof(double) * len));
  IFEMGPU_CUDA(ctx, cudaMemset(ctx->d_normBuf, 0, sizeof(double) * len));
  ctx->normBufLen = len;
  return IFEMGPU_OK;
}

// Uploads u, runs the element kernel (secondary output for one patch when
// secDev != nullptr) and the totals.
ifemgpu_status runNorms(ifemgpu_ctx* ctx, const double* u, double* secDev, int secPatch)
{
  if (!ctx->assembled) return setError(ctx, IFEMGPU_NOT_READY, "norms: assemble first (basis tables)");
  ifemgpu_status st = prepareNorms(ctx);
  if (st != IFEMGPU_OK) return st;
  cudaStream_t s = ctx->stream;
  double* dU = ctx->d_normBuf;
  double* dElem = dU + ctx->ndof;
  double* dTot = dElem + 2 * (size_t)ctx->nNormSlots;
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(dU, u, sizeof(double) * ctx->ndof, cudaMemcpyHostToDevice, s));
  IFEMGPU_CUDA(ctx, cudaMemsetAsync(dElem, 0, sizeof(double) * 2 * ctx->nNormSlots, s));
  const bool fp64 = ctx->opts.ke_precision == IFEMGPU_KE_FP64;
  size_t smem = 0;
  for (const DevPatch& D : ctx->h_devpatches) smem = std::max(smem, normSmem(D, fp64));
  if (ctx->nNormItems > 0) {
    if (fp64)
      k_norms<double><<<ctx->nNormItems, kNT, smem, s>>>(ctx->d_patches, ctx->d_normItems,
                                                         ctx->d_madof, dU, dElem, secDev, secPatch);
    else
      k_norms<float><<<ctx->nNormItems, kNT, smem, s>>>(ctx->d_patches, ctx->d_normItems,
                                                        ctx->d_madof, dU, dElem, secDev, secPatch);
  }
  k_norm_totals<<<1, 256, 0, s>>>(dElem, ctx->nNormSlots, dTot);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  return IFEMGPU_OK;
}

}  // namespace

void freeNorms(ifemgpu_ctx* ctx)
{
  if (ctx->d_normItems) cudaFree(ctx->d_normItems);
  if (ctx->d_normBuf) cudaFree(ctx->d_normBuf);
  ctx->d_normItems = nullptr;
  ctx->d_normBuf = nullptr;
  ctx->nNormItems = ctx->nNormSlots = 0;
  ctx->normBufLen = 0;
  ctx->normBase.clear();
}

}  // namespace ifemgpu

using namespace ifemgpu;

extern "C" ifemgpu_status ifemgpu_solution_norms(ifemgpu_ctx* ctx, const double* u_dof,
                                                 double* totals, double* element)
{
  if (!ctx || !u_dof || !totals) return IFEMGPU_INVALID_ARG;
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  ifemgpu_status st = runNorms(ctx, u_dof, nullptr, -1);
  if (st != IFEMGPU_OK) return st;
  const double* dElem = ctx->d_normBuf + ctx->ndof;
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(totals, dElem + 2 * (size_t)ctx->nNormSlots, 2 * sizeof(double),
                                    cudaMemcpyDeviceToHost, ctx->stream));
  if (element)
    IFEMGPU_CUDA(ctx, cudaMemcpyAsync(element, dElem, 2 * sizeof(double) * ctx->nNormSlots,
                                      cudaMemcpyDeviceToHost, ctx->stream));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return IFEMGPU_OK;
}

extern "C" ifemgpu_status ifemgpu_secondary_solution(ifemgpu_ctx* ctx, int patch_id,
                                                     const double* u_dof, double* out)
{
  if (!ctx || !u_dof || !out || patch_id < 1 || patch_id > (int)ctx->patches.size())
    return IFEMGPU_INVALID_ARG;
  if (!ctx->assembled) return setError(ctx, IFEMGPU_NOT_READY, "secondary solution: assemble first");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  const DevPatch& D = ctx->h_devpatches[patch_id - 1];
  const int nc = D.kind == IFEMGPU_POISSON ? D.dim : 6;
  const size_t count = (size_t)ctx->patches[patch_id - 1].nelAll * D.nq * nc;
  double* dSec = nullptr;
  IFEMGPU_CUDA(ctx, cudaMalloc(&dSec, sizeof(double) * std::max<size_t>(count, 1)));
  ifemgpu_status st = IFEMGPU_OK;
  if (cudaMemsetAsync(dSec, 0, sizeof(double) * count, ctx->stream) != cudaSuccess)
    st = setError(ctx, IFEMGPU_CUDA_ERROR, "secondary solution: memset");
  if (st == IFEMGPU_OK) st = runNorms(ctx, u_dof, dSec, patch_id - 1);
  if (st == IFEMGPU_OK &&
      (cudaMemcpyAsync(out, dSec, sizeof(double) * count, cudaMemcpyDeviceToHost, ctx->stream) !=
           cudaSuccess ||
       cudaStreamSynchronize(ctx->stream) != cudaSuccess))
    st = setError(ctx, IFEMGPU_CUDA_ERROR, "secondary solution: copy");
  cudaFree(dSec);
  return st;
}
