// fdprec.cu -- Kronecker-product (fast-diagonalisation) preconditioner.
//
// No IFEM counterpart (IFEM's iterative solvers take algebraic
// preconditioners from PETSc/ISTL).  For a 3D spline patch the free DOFs of
// each solution component form a box of control points when Dirichlet
// conditions cover whole faces.  On that box the Laplacian of the parameter
// cube, K0 (x) M1 (x) M2 + M0 (x) K1 (x) M2 + M0 (x) M1 (x) K2 with the 1D
// spline stiffness K_d and mass M_d, is inverted exactly through the 1D
// generalised eigenproblems K_d U_d = M_d U_d diag(lam_d), U_d^T M_d U_d = I:
//   P^-1 = (U2 (x) U1 (x) U0) diag(1 / (lam0_a + lam1_b + lam2_c)) (U2 (x) U1 (x) U0)^T
// (Lynch, Rice and Thomas 1964; for splines Sangalli and Tani 2016).  The
// geometry and the coefficient enter through a diagonal scaling,
// z = S P^-1 S r with S = sqrt(diag(P) / diag(A)).  Unlike point Jacobi it
// also handles the high-frequency modes that are small for spline degree
// p >= 2, so the iteration count barely grows with p or the mesh size.
//
// Device work per application of one block (n0 x n1 x n2): two slab kernels
// (mode products along u and v of one w-slab, in shared memory) around one
// column kernel (mode product along w, the eigenvalue division and the
// inverse mode product); everything stays in L2 for the sizes used here.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ifemgpu_internal.h"
#include "reduce.cuh"

namespace ifemgpu {

void gaussLegendre(int n, double* x, double* w);  // assembly.cu

constexpr int kFdMax = 112;   // largest box extent (shared-memory slabs)
constexpr int kFdCols = 16;   // columns per block of the w-direction kernel

struct FdBlock {
  int n[3];
  int* map = nullptr;         // box position (i fastest) -> equation (0-based)
  int base = -1, stride = 0;  // map[o] = base + stride o when base >= 0 (no map reads)
  float* U[3] = {nullptr, nullptr, nullptr};    // n_d x n_d, row-major U[i][a]
  float* Ut[3] = {nullptr, nullptr, nullptr};   // transposes
  float* lam[3] = {nullptr, nullptr, nullptr};
};

struct FdState {
  std::vector<FdBlock> blocks;
  float* dP = nullptr;        // neq: diagonal of the Kronecker operator
  float* scale = nullptr;     // neq: sqrt(dP / A_ee) of the current matrix
  float* tmp = nullptr;       // largest box
  size_t smemSlab = 0;
  std::vector<void*> allocs;
};

namespace {

constexpr int kT = 256;

__device__ inline bool fdStopped(const double* guard) { return guard && guard[0] != 0.0; }

// Asynchronous staging (cp.async, 4-byte copies): every thread issues all of
// its copies before waiting once, so a block's whole staging costs about one
// L2 round trip instead of one per batch of loads.
__device__ inline void cpAsync4(float* dst, const float* src)
{
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;"
               :
               : "r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst))), "l"(src)
               : "memory");
}

__device__ inline void cpAsyncWaitAll()
{
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" : : : "memory");
}

// n floats global -> shared (issued only)
__device__ inline void stageAsync(float* __restrict__ dst, const float* __restrict__ src, int n)
{
  for (int o = threadIdx.x; o < n; o += blockDim.x) cpAsync4(dst + o, src + o);
}

// equation of box position o (affine maps need no map read)
__device__ inline int boxEq(const int* __restrict__ map, int base, int stride, size_t o)
{
  return base >= 0 ? base + stride * (int)o : map[o];
}

// S[o] <- r[e(o)], X[o] <- scale[e(o)] for the positions [first, first + n) (issued only)
__device__ inline void stageGatherAsync(float* __restrict__ S, float* __restrict__ X,
                                        const int* __restrict__ map, int base, int stride,
                                        size_t first, const float* __restrict__ scale,
                                        const float* __restrict__ r, int n)
{
#pragma unroll 4
  for (int o = threadIdx.x; o < n; o += blockDim.x) {
    const int e = boxEq(map, base, stride, first + o);
    cpAsync4(S + o, r + e);
    cpAsync4(X + o, scale + e);
  }
}

// Every thread of the three kernels below forms kFdTile outputs of one
// column at once (independent FMA chains sharing each loaded coefficient);
// rows past the end are clamped on load and dropped on store.
constexpr int kFdTile = 8;
constexpr int kFdSplit = 4;   // blocks per w-slab in the slab kernels

// out[k][b][a] = sum_j U1[j][b] sum_i U0[i][a] scale_e r_e for one w-slab k
// and the block's share of the columns a
__global__ void __launch_bounds__(kT)
k_fd_fwd(const float* __restrict__ r, const float* __restrict__ scale, const int* __restrict__ map,
         int base, int stride, int n0, int n1, const float* __restrict__ U0,
         const float* __restrict__ U1, float* __restrict__ out, const double* guard)
{
  if (fdStopped(guard)) return;
  extern __shared__ float sm[];
  const int ns = n0 * n1;
  float* S = sm;
  float* T = S + ns;
  float* u0 = T + ns;
  float* u1 = u0 + n0 * n0;
  const int k = blockIdx.x;
  const int per = (n0 + gridDim.y - 1) / gridDim.y;
  const int a0 = blockIdx.y * per, na = min(n0, a0 + per) - a0;
  if (na <= 0) return;
  // r and the scaling of the slab (the scaling into T, free until the first
  // product), both eigenvector matrices; then S = scale r on own elements
  stageGatherAsync(S, T, map, base, stride, (size_t)k * ns, scale, r, ns);
  stageAsync(u0, U0, n0 * n0);
  stageAsync(u1, U1, n1 * n1);
  cpAsyncWaitAll();
  for (int o = threadIdx.x; o < ns; o += blockDim.x) S[o] *= T[o];
  __syncthreads();
  const int nt = (n1 + kFdTile - 1) / kFdTile;
  for (int w = threadIdx.x; w < nt * na; w += blockDim.x) {
    const int jt = w / na, a = a0 + (w - jt * na), j0 = jt * kFdTile;
    const float* srow[kFdTile];
#pragma unroll
    for (int q = 0; q < kFdTile; q++) srow[q] = S + min(j0 + q, n1 - 1) * n0;
    float acc[kFdTile] = {};
#pragma unroll 4
    for (int i = 0; i < n0; i++) {
      const float u = u0[i * n0 + a];
#pragma unroll
      for (int q = 0; q < kFdTile; q++) acc[q] = fmaf(srow[q][i], u, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < kFdTile; q++)
      if (j0 + q < n1) T[(j0 + q) * n0 + a] = acc[q];
  }
  __syncthreads();
  for (int w = threadIdx.x; w < nt * na; w += blockDim.x) {
    const int bt = w / na, a = a0 + (w - bt * na), b0 = bt * kFdTile;
    int bq[kFdTile];
#pragma unroll
    for (int q = 0; q < kFdTile; q++) bq[q] = min(b0 + q, n1 - 1);
    float acc[kFdTile] = {};
#pragma unroll 4
    for (int j = 0; j < n1; j++) {
      const float t = T[j * n0 + a];
      const float* u = u1 + j * n1;
#pragma unroll
      for (int q = 0; q < kFdTile; q++) acc[q] = fmaf(u[bq[q]], t, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < kFdTile; q++)
      if (b0 + q < n1) out[((size_t)k * n1 + b0 + q) * n0 + a] = acc[q];
  }
}

// along w for kFdCols columns (b, a): V = U2^T X / (lam0 + lam1 + lam2), X <- U2 V
__global__ void __launch_bounds__(kT)
k_fd_mid(float* __restrict__ tmp, int n0, int n1, int n2, const float* __restrict__ U2,
         const float* __restrict__ lam0, const float* __restrict__ lam1,
         const float* __restrict__ lam2, const double* guard)
{
  if (fdStopped(guard)) return;
  extern __shared__ float sm[];
  float* X = sm;                   // n2 x kFdCols
  float* V = X + n2 * kFdCols;     // n2 x kFdCols
  float* u2 = V + n2 * kFdCols;    // n2 x n2
  const int ncol = n0 * n1, col0 = blockIdx.x * kFdCols;
  for (int o = threadIdx.x; o < n2 * kFdCols; o += blockDim.x) {
    const int k = o / kFdCols, t = o - k * kFdCols;
    if (col0 + t < ncol) cpAsync4(X + o, tmp + (size_t)k * ncol + col0 + t);
    else X[o] = 0.f;
  }
  stageAsync(u2, U2, n2 * n2);
  cpAsyncWaitAll();
  __syncthreads();
  const int nt = (n2 + kFdTile - 1) / kFdTile;
  for (int w = threadIdx.x; w < nt * kFdCols; w += blockDim.x) {
    const int ct = w / kFdCols, t = w - ct * kFdCols, c0 = ct * kFdTile;
    int cq[kFdTile];
#pragma unroll
    for (int q = 0; q < kFdTile; q++) cq[q] = min(c0 + q, n2 - 1);
    float acc[kFdTile] = {};
#pragma unroll 4
    for (int k = 0; k < n2; k++) {
      const float x = X[k * kFdCols + t];
      const float* u = u2 + k * n2;
#pragma unroll
      for (int q = 0; q < kFdTile; q++) acc[q] = fmaf(u[cq[q]], x, acc[q]);
    }
    const int col = min(col0 + t, ncol - 1), b = col / n0, a = col - b * n0;
    const float lab = lam0[a] + lam1[b];
#pragma unroll
    for (int q = 0; q < kFdTile; q++)
      if (c0 + q < n2) V[(c0 + q) * kFdCols + t] = acc[q] / (lab + lam2[c0 + q]);
  }
  __syncthreads();
  for (int w = threadIdx.x; w < nt * kFdCols; w += blockDim.x) {
    const int kt = w / kFdCols, t = w - kt * kFdCols, k0 = kt * kFdTile;
    const float* urow[kFdTile];
#pragma unroll
    for (int q = 0; q < kFdTile; q++) urow[q] = u2 + min(k0 + q, n2 - 1) * n2;
    float acc[kFdTile] = {};
#pragma unroll 4
    for (int c = 0; c < n2; c++) {
      const float v = V[c * kFdCols + t];
#pragma unroll
      for (int q = 0; q < kFdTile; q++) acc[q] = fmaf(urow[q][c], v, acc[q]);
    }
    if (col0 + t >= ncol) continue;
#pragma unroll
    for (int q = 0; q < kFdTile; q++)
      if (k0 + q < n2) tmp[(size_t)(k0 + q) * ncol + col0 + t] = acc[q];
  }
}

// z_e = scale_e sum_a U0[i][a] sum_b U1[j][b] tmp[k][b][a] for one w-slab k
// and the block's share of the rows j
__global__ void __launch_bounds__(kT)
k_fd_inv(const float* __restrict__ tmp, int n0, int n1, const float* __restrict__ U0t,
         const float* __restrict__ U1, const float* __restrict__ scale,
         const int* __restrict__ map, int base, int stride, float* __restrict__ z, FdDot dot,
         const double* guard)
{
  if (fdStopped(guard)) return;
  extern __shared__ float sm[];
  const int ns = n0 * n1;
  float* W = sm;
  float* T = W + ns;
  float* u0t = T + ns;    // u0t[a][i] = U0[i][a]
  float* u1 = u0t + n0 * n0;
  const int k = blockIdx.x;
  const int per = (n1 + gridDim.y - 1) / gridDim.y;
  const int jb = blockIdx.y * per, nj = max(min(n1, jb + per) - jb, 0);
  stageAsync(W, tmp + (size_t)k * ns, ns);
  stageAsync(u0t, U0t, n0 * n0);
  stageAsync(u1, U1, n1 * n1);
  cpAsyncWaitAll();
  __syncthreads();
  const int nt = (nj + kFdTile - 1) / kFdTile, je = jb + nj;
  for (int w = threadIdx.x; w < nt * n0; w += blockDim.x) {
    const int jt = w / n0, a = w - jt * n0, j0 = jb + jt * kFdTile;
    const float* urow[kFdTile];
#pragma unroll
    for (int q = 0; q < kFdTile; q++) urow[q] = u1 + min(j0 + q, je - 1) * n1;
    float acc[kFdTile] = {};
#pragma unroll 4
    for (int b = 0; b < n1; b++) {
      const float x = W[b * n0 + a];
#pragma unroll
      for (int q = 0; q < kFdTile; q++) acc[q] = fmaf(urow[q][b], x, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < kFdTile; q++)
      if (j0 + q < je) T[(j0 + q) * n0 + a] = acc[q];
  }
  __syncthreads();
  float zq = 0.f;
  for (int w = threadIdx.x; w < nt * n0; w += blockDim.x) {
    const int jt = w / n0, i = w - jt * n0, j0 = jb + jt * kFdTile;
    const float* trow[kFdTile];
#pragma unroll
    for (int q = 0; q < kFdTile; q++) trow[q] = T + min(j0 + q, je - 1) * n0;
    float acc[kFdTile] = {};
#pragma unroll 4
    for (int a = 0; a < n0; a++) {
      const float u = u0t[a * n0 + i];
#pragma unroll
      for (int q = 0; q < kFdTile; q++) acc[q] = fmaf(trow[q][a], u, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < kFdTile; q++) {
      const int j = j0 + q;
      if (j >= je) continue;
      const int e = boxEq(map, base, stride, (size_t)k * ns + j * n0 + i);
      const float ze = scale[e] * acc[q];
      z[e] = ze;
      if (dot.q) zq = fmaf(ze, dot.q[e], zq);
    }
  }
  // (z, q) of the flexible-CG step and beta = -(z, q) / (p, q), folded into
  // this (single-box) product
  if (dot.q) {
    __shared__ double sh[32];
    const double t = blockReduceSumF(zq, sh);
    const unsigned nb = gridDim.x * gridDim.y;
    if (threadIdx.x == 0) dot.part[blockIdx.y * gridDim.x + blockIdx.x] = t;
    if (lastBlockOf(dot.counter, nb)) {
      const double v = finalSum(dot.part, (int)nb, sh);
      if (threadIdx.x == 0) {
        *dot.out = v;
        *dot.beta = (float)(-v / *dot.pq);
      }
    }
  }
}

__global__ void k_fd_scale(const float* __restrict__ dP, const double* __restrict__ dinv,
                           float* __restrict__ scale, int n)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    scale[i] = sqrtf(fmaxf(dP[i] * (float)dinv[i], 0.f));
}

// ---- host: 1D spline matrices and the generalised eigenproblem ----------------

// the deg+1 B-splines of degree deg non-zero on knot span s, at u
// (Cox-de Boor recursion in the triangular form of Piegl and Tiller, A2.2)
void basisFuns(const std::vector<double>& U, int deg, int s, double u, double* N)
{
  std::vector<double> left(deg + 1), right(deg + 1);
  N[0] = 1.0;
  for (int j = 1; j <= deg; j++) {
    left[j] = u - U[s + 1 - j];
    right[j] = U[s + j] - u;
    double saved = 0.0;
    for (int r = 0; r < j; r++) {
      const double temp = N[r] / (right[r + 1] + left[j - r]);
      N[r] = saved + right[r + 1] * temp;
      saved = left[j - r] * temp;
    }
    N[j] = saved;
  }
}

// values and first derivatives of the p+1 B-splines non-zero on span s, from
// dN_i/du = p N_(i,p-1) / (U_(i+p) - U_i) - p N_(i+1,p-1) / (U_(i+p+1) - U_(i+1))
void splineDers(const std::vector<double>& U, int p, int s, double u, double* N, double* dN)
{
  basisFuns(U, p, s, u, N);
  if (p == 0) {
    dN[0] = 0.0;
    return;
  }
  std::vector<double> Nm(p);  // degree p-1: functions s-p+1 .. s
  basisFuns(U, p - 1, s, u, Nm.data());
  for (int r = 0; r <= p; r++) {
    double d = 0.0;
    if (r >= 1) d += p * Nm[r - 1] / (U[s + r] - U[s - p + r]);
    if (r <= p - 1) d -= p * Nm[r] / (U[s + r + 1] - U[s - p + r + 1]);
    dN[r] = d;
  }
}

// 1D stiffness and mass of all n basis functions of (U, p), Gauss rule of p+1 points
void splineMatrices1D(const std::vector<double>& U, int p, int n, std::vector<double>& K,
                      std::vector<double>& M)
{
  K.assign((size_t)n * n, 0.0);
  M.assign((size_t)n * n, 0.0);
  const int ng = p + 1;
  std::vector<double> gx(ng), gw(ng), N(p + 1), dN(p + 1);
  gaussLegendre(ng, gx.data(), gw.data());
  for (int s = p; s < n; s++) {
    const double a = U[s], b = U[s + 1];
    if (!(b > a)) continue;
    for (int q = 0; q < ng; q++) {
      const double u = 0.5 * (a + b) + 0.5 * (b - a) * gx[q];
      const double w = 0.5 * (b - a) * gw[q];
      splineDers(U, p, s, u, N.data(), dN.data());
      for (int r = 0; r <= p; r++)
        for (int c = 0; c <= p; c++) {
          const size_t idx = (size_t)(s - p + r) * n + (s - p + c);
          K[idx] += w * dN[r] * dN[c];
          M[idx] += w * N[r] * N[c];
        }
    }
  }
}

// K U = M U diag(lam), U^T M U = I for symmetric K and SPD M (n x n,
// row-major): Cholesky M = L L^T, cyclic Jacobi rotations on L^-1 K L^-T,
// back substitution U = L^-T V.  Returns false when M is not SPD.
bool generalisedEigen(int n, std::vector<double> K, std::vector<double> M, std::vector<double>& U,
                      std::vector<double>& lam)
{
  std::vector<double> L((size_t)n * n, 0.0);
  for (int j = 0; j < n; j++) {
    double d = M[(size_t)j * n + j];
    for (int k = 0; k < j; k++) d -= L[(size_t)j * n + k] * L[(size_t)j * n + k];
    if (!(d > 0.0)) return false;
    L[(size_t)j * n + j] = std::sqrt(d);
    for (int i = j + 1; i < n; i++) {
      double v = M[(size_t)i * n + j];
      for (int k = 0; k < j; k++) v -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
      L[(size_t)i * n + j] = v / L[(size_t)j * n + j];
    }
  }
  // Y = L^-1 K (forward substitution per column), C = Y L^-T = (L^-1 Y^T)^T
  auto lowerSolveColumns = [&](std::vector<double>& B) {
    for (int c = 0; c < n; c++)
      for (int i = 0; i < n; i++) {
        double v = B[(size_t)i * n + c];
        for (int k = 0; k < i; k++) v -= L[(size_t)i * n + k] * B[(size_t)k * n + c];
        B[(size_t)i * n + c] = v / L[(size_t)i * n + i];
      }
  };
  std::vector<double> C = K;
  lowerSolveColumns(C);
  for (int i = 0; i < n; i++)
    for (int j = i + 1; j < n; j++) std::swap(C[(size_t)i * n + j], C[(size_t)j * n + i]);
  lowerSolveColumns(C);
  for (int i = 0; i < n; i++)  // symmetrise rounding
    for (int j = i + 1; j < n; j++) {
      const double v = 0.5 * (C[(size_t)i * n + j] + C[(size_t)j * n + i]);
      C[(size_t)i * n + j] = C[(size_t)j * n + i] = v;
    }
  std::vector<double> V((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) V[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        const double v = C[(size_t)i * n + j] * C[(size_t)i * n + j];
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-30 * tot) break;
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = C[(size_t)p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double app = C[(size_t)p * n + p], aqq = C[(size_t)q * n + q];
        const double theta = 0.5 * (aqq - app) / apq;
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; k++) {  // C <- C J (columns p, q)
          const double ckp = C[(size_t)k * n + p], ckq = C[(size_t)k * n + q];
          C[(size_t)k * n + p] = c * ckp - s * ckq;
          C[(size_t)k * n + q] = s * ckp + c * ckq;
        }
        for (int k = 0; k < n; k++) {  // C <- J^T C (rows p, q)
          const double cpk = C[(size_t)p * n + k], cqk = C[(size_t)q * n + k];
          C[(size_t)p * n + k] = c * cpk - s * cqk;
          C[(size_t)q * n + k] = s * cpk + c * cqk;
        }
        for (int k = 0; k < n; k++) {  // V <- V J
          const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = c * vkp - s * vkq;
          V[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  lam.resize(n);
  for (int i = 0; i < n; i++) lam[i] = C[(size_t)i * n + i];
  // U = L^-T V: back substitution per column
  U = V;
  for (int c = 0; c < n; c++)
    for (int i = n - 1; i >= 0; i--) {
      double v = U[(size_t)i * n + c];
      for (int k = i + 1; k < n; k++) v -= L[(size_t)k * n + i] * U[(size_t)k * n + c];
      U[(size_t)i * n + c] = v / L[(size_t)i * n + i];
    }
  return true;
}

}  // namespace

void destroyFd(ifemgpu_ctx* ctx)
{
  if (!ctx->fd) return;
  for (void* p : ctx->fd->allocs) cudaFree(p);
  delete ctx->fd;
  ctx->fd = nullptr;
}

ifemgpu_status fdSetup(ifemgpu_ctx* ctx)
{
  if (ctx->fd) return IFEMGPU_OK;
  const int neq = ctx->neq;
  FdState* F = new FdState;
  auto fail = [&](ifemgpu_status st, const char* msg) {
    for (void* p : F->allocs) cudaFree(p);
    delete F;
    return setError(ctx, st, msg);
  };
  std::vector<int> covered(neq, 0);
  std::vector<float> dP(neq, 0.f);
  size_t maxVol = 0;
  struct HostBlock { int n[3]; std::vector<int> map; std::vector<float> U[3], Ut[3], lam[3]; };
  std::vector<HostBlock> hb;
  for (const HostPatch& pc : ctx->patches) {
    if (pc.dim != 3)
      return fail(IFEMGPU_UNSUPPORTED, "Kronecker preconditioner: 3D patches only");
    std::vector<double> K1[3], M1[3];
    for (int d = 0; d < 3; d++) splineMatrices1D(pc.knots[d], pc.p[d], pc.n[d], K1[d], M1[d]);
    for (int comp = 0; comp < pc.npv; comp++) {
      auto eqOf = [&](int i, int j, int k) {
        const int node = (k * pc.n[1] + j) * pc.n[0] + i;
        return ctx->meqn[ctx->madof[pc.mlgn[node]] - 1 + comp];
      };
      int lo[3] = {pc.n[0], pc.n[1], pc.n[2]}, hi[3] = {-1, -1, -1};
      long nfree = 0;
      for (int k = 0; k < pc.n[2]; k++)
        for (int j = 0; j < pc.n[1]; j++)
          for (int i = 0; i < pc.n[0]; i++)
            if (eqOf(i, j, k) > 0) {
              nfree++;
              const int ijk[3] = {i, j, k};
              for (int d = 0; d < 3; d++) {
                lo[d] = std::min(lo[d], ijk[d]);
                hi[d] = std::max(hi[d], ijk[d]);
              }
            }
      if (nfree == 0) continue;
      HostBlock B;
      for (int d = 0; d < 3; d++) B.n[d] = hi[d] - lo[d] + 1;
      if ((long)B.n[0] * B.n[1] * B.n[2] != nfree)
        return fail(IFEMGPU_UNSUPPORTED,
                    "Kronecker preconditioner: free DOFs of a patch component are not a box");
      if (std::max({B.n[0], B.n[1], B.n[2]}) > kFdMax)
        return fail(IFEMGPU_UNSUPPORTED, "Kronecker preconditioner: more than 112 coefficients per direction");
      std::vector<double> Kd[3], Md[3];
      for (int d = 0; d < 3; d++) {
        const int nd = B.n[d], n = pc.n[d];
        Kd[d].resize((size_t)nd * nd);
        Md[d].resize((size_t)nd * nd);
        for (int r = 0; r < nd; r++)
          for (int c = 0; c < nd; c++) {
            Kd[d][(size_t)r * nd + c] = K1[d][(size_t)(lo[d] + r) * n + lo[d] + c];
            Md[d][(size_t)r * nd + c] = M1[d][(size_t)(lo[d] + r) * n + lo[d] + c];
          }
        std::vector<double> U, lam;
        if (!generalisedEigen(nd, Kd[d], Md[d], U, lam))
          return fail(IFEMGPU_INVALID_ARG, "Kronecker preconditioner: singular 1D mass matrix");
        B.U[d].resize((size_t)nd * nd);
        B.Ut[d].resize((size_t)nd * nd);
        B.lam[d].resize(nd);
        for (int r = 0; r < nd; r++) {
          B.lam[d][r] = (float)lam[r];
          for (int c = 0; c < nd; c++) {
            B.U[d][(size_t)r * nd + c] = (float)U[(size_t)r * nd + c];
            B.Ut[d][(size_t)c * nd + r] = (float)U[(size_t)r * nd + c];
          }
        }
      }
      B.map.resize(nfree);
      for (int k = 0; k < B.n[2]; k++)
        for (int j = 0; j < B.n[1]; j++)
          for (int i = 0; i < B.n[0]; i++) {
            const int eq = eqOf(lo[0] + i, lo[1] + j, lo[2] + k) - 1;
            if (covered[eq]++)
              return fail(IFEMGPU_UNSUPPORTED, "Kronecker preconditioner: patches share equations");
            B.map[((size_t)k * B.n[1] + j) * B.n[0] + i] = eq;
            const double k0 = Kd[0][(size_t)i * B.n[0] + i], m0 = Md[0][(size_t)i * B.n[0] + i];
            const double k1 = Kd[1][(size_t)j * B.n[1] + j], m1 = Md[1][(size_t)j * B.n[1] + j];
            const double k2 = Kd[2][(size_t)k * B.n[2] + k], m2 = Md[2][(size_t)k * B.n[2] + k];
            dP[eq] = (float)(k0 * m1 * m2 + m0 * k1 * m2 + m0 * m1 * k2);
          }
      maxVol = std::max(maxVol, (size_t)nfree);
      hb.push_back(std::move(B));
    }
  }
  for (int e = 0; e < neq; e++)
    if (!covered[e]) return fail(IFEMGPU_UNSUPPORTED, "Kronecker preconditioner: equation outside every box");
  auto up = [&](auto** dst, const auto* src, size_t n) -> bool {
    if (cudaMalloc((void**)dst, sizeof(**dst) * std::max<size_t>(n, 1)) != cudaSuccess) return false;
    F->allocs.push_back((void*)*dst);
    return !src || !n ||
           cudaMemcpy(*dst, src, sizeof(**dst) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  };
  for (HostBlock& B : hb) {
    FdBlock D;
    for (int d = 0; d < 3; d++) D.n[d] = B.n[d];
    // equations numbered in box order with a fixed stride (one component of a
    // box-shaped free set): the kernels form them without reading the map
    const int stride = B.map.size() > 1 ? B.map[1] - B.map[0] : 1;
    bool affine = stride > 0;
    for (size_t o = 0; affine && o < B.map.size(); o++)
      affine = B.map[o] == B.map[0] + stride * (int)o;
    if (affine) {
      D.base = B.map[0];
      D.stride = stride;
    }
    bool ok = up(&D.map, B.map.data(), B.map.size());
    for (int d = 0; d < 3; d++) {
      ok = ok && up(&D.U[d], B.U[d].data(), B.U[d].size());
      ok = ok && up(&D.Ut[d], B.Ut[d].data(), B.Ut[d].size());
      ok = ok && up(&D.lam[d], B.lam[d].data(), B.lam[d].size());
    }
    if (!ok) return fail(IFEMGPU_OUT_OF_MEMORY, "Kronecker preconditioner: device allocation");
    const size_t slab = sizeof(float) * (2 * (size_t)B.n[0] * B.n[1] + (size_t)B.n[0] * B.n[0] +
                                         (size_t)B.n[1] * B.n[1]);
    const size_t mid = sizeof(float) * (2 * (size_t)B.n[2] * kFdCols + (size_t)B.n[2] * B.n[2]);
    F->smemSlab = std::max({F->smemSlab, slab, mid});
    F->blocks.push_back(D);
  }
  bool ok = up(&F->dP, dP.data(), dP.size());
  ok = ok && up(&F->scale, (float*)nullptr, (size_t)neq);
  ok = ok && up(&F->tmp, (float*)nullptr, maxVol);
  if (!ok) return fail(IFEMGPU_OUT_OF_MEMORY, "Kronecker preconditioner: device allocation");
  if (F->smemSlab > 48 * 1024) {
    cudaFuncSetAttribute(k_fd_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)F->smemSlab);
    cudaFuncSetAttribute(k_fd_mid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)F->smemSlab);
    cudaFuncSetAttribute(k_fd_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)F->smemSlab);
  }
  ctx->fd = F;
  return IFEMGPU_OK;
}

// scaling of the current matrix from its inverse diagonal (FP64, neq)
ifemgpu_status fdRescale(ifemgpu_ctx* ctx, const double* dinv)
{
  FdState* F = ctx->fd;
  k_fd_scale<<<std::min(4096, (ctx->neq + kT - 1) / kT), kT, 0, ctx->stream>>>(F->dP, dinv, F->scale,
                                                                              ctx->neq);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  return IFEMGPU_OK;
}

bool fdCanDot(const ifemgpu_ctx* ctx)
{
  return ctx->fd && ctx->fd->blocks.size() == 1 && ctx->fd->blocks[0].n[2] * kFdSplit <= 1024;
}

// z = S P^-1 S r over every block; each kernel returns at once when *guard != 0.
// With dot (one box only, fdCanDot), the last kernel also forms (z, q) and beta.
ifemgpu_status fdApply(ifemgpu_ctx* ctx, const float* r, float* z, const double* guard,
                       const FdDot* dot)
{
  FdState* F = ctx->fd;
  cudaStream_t s = ctx->stream;
  if (dot && !fdCanDot(ctx))
    return setError(ctx, IFEMGPU_INVALID_ARG, "internal: fused (z, q) needs a single box");
  const FdDot none{};
  for (const FdBlock& B : F->blocks) {
    const size_t slab = sizeof(float) * (2 * (size_t)B.n[0] * B.n[1] + (size_t)B.n[0] * B.n[0] +
                                         (size_t)B.n[1] * B.n[1]);
    const size_t mid = sizeof(float) * (2 * (size_t)B.n[2] * kFdCols + (size_t)B.n[2] * B.n[2]);
    const int ncol = B.n[0] * B.n[1];
    const dim3 slabs(B.n[2], kFdSplit);
    k_fd_fwd<<<slabs, kT, slab, s>>>(r, F->scale, B.map, B.base, B.stride, B.n[0], B.n[1], B.U[0],
                                     B.U[1], F->tmp, guard);
    k_fd_mid<<<(ncol + kFdCols - 1) / kFdCols, kT, mid, s>>>(F->tmp, B.n[0], B.n[1], B.n[2], B.U[2],
                                                             B.lam[0], B.lam[1], B.lam[2], guard);
    k_fd_inv<<<slabs, kT, slab, s>>>(F->tmp, B.n[0], B.n[1], B.Ut[0], B.U[1], F->scale, B.map,
                                     B.base, B.stride, z, dot ? *dot : none, guard);
  }
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  return IFEMGPU_OK;
}

int fdLaunches(const ifemgpu_ctx* ctx) { return ctx->fd ? 3 * (int)ctx->fd->blocks.size() : 0; }

}  // namespace ifemgpu
