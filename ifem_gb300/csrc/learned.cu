// learned.cu -- learned coarse correction of the flexible PCG solve.
//
// No IFEM counterpart (IFEM solves with SuperLU or a PETSc/ISTL Krylov
// method).  For a patch with npv unknowns per node the correction works on a
// coarse grid of (m+1)^3 vertices over the patch's parameter domain, npv
// values per vertex (nc = npv (m+1)^3 coarse unknowns):
//   restriction   rc_(v,c) = sum_e w_ve r_e     over the free equations e of
//                                               component c; w_ve is the
//                                               trilinear weight of vertex v
//                                               at e's Greville point (R)
//   network       y = MLP([rc / |rc|, g])       3 layers, width nh, ReLU;
//                                               BF16 tcgen05 inference with
//                                               FP32 accumulation
//   two-level step  after the fine step z1 and t = A z1, rc = R (r - t):
//                 z = z1 + alpha R^T y, alpha = (y, rc) / (y, Ac y) with the
//                 Galerkin coarse matrix Ac = R A R^T of the assembly
// g (optional) is the patch's log-conductivity field restricted to the
// coarse vertices, so that one network can serve many coefficient fields.
// The network is trained by the kernels of this file (3xTF32 tcgen05 GEMMs,
// FP32 elsewhere) on pairs
// ([rc/|rc|, g], ec/|rc|), ec the weight-normalised restriction of the error
// of the method's own iterates (learnRecord); S, the RMS of the targets,
// keeps the network's outputs of order one.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "ifemgpu_internal.h"
#include "reduce.cuh"
#include "tc_common.cuh"

namespace ifemgpu {

constexpr int kGemmTiles = 1024;  // output tiles of one training product with split K

struct LearnState {
  int m = 8;             // coarse cells per direction
  int npv = 1;           // unknowns per node
  int nc = 0;            // coarse unknowns, npv (m+1)^3
  int nf = 0;            // field inputs: (m+1)^3 or 0
  int nin = 0;           // network inputs, nc + nf
  int nh = 256;          // hidden width
  float* feat = nullptr; // nf: coarse log-conductivity of the current field
  int featVersion = -1;  // field version the features were computed from
  std::vector<int> featEq;     // per feature weight list: equations (component 0)
  std::vector<float> featW;
  std::vector<int> featPtr;
  int nparam = 0;
  int oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0;
  // transfer operators
  int* eqCell = nullptr;      // neq: coarse cell of the equation's Greville point
  float4* eqFrac = nullptr;   // neq: position inside the cell (x, y, z), component (w)
  int* vPtr = nullptr;        // nc+1: equations in the support of each coarse unknown
  int* vEq = nullptr;
  float* vW = nullptr;        // trilinear weights
  float* vWn = nullptr;       // weights divided by their sum per coarse unknown
  // network: FP32 master weights; for the solve a BF16 copy packed in
  // 128 x 64 tensor-core operand tiles per layer (layer l: Mt[l] row tiles x
  // nKT[l] K tiles at element offset pOff[l]), per-tile partial sums and the
  // tickets of the row tiles' last CTAs
  float* theta = nullptr;
  float* grad = nullptr;
  float* am = nullptr;
  float* av = nullptr;
  __nv_bfloat16* wtc = nullptr;
  size_t pOff[3] = {0, 0, 0};
  int Mt[3] = {0, 0, 0}, nKT[3] = {0, 0, 0};
  float* tpart = nullptr;
  unsigned* tick = nullptr;
  // split-K partial tiles and tile tickets of the training products
  float* gws = nullptr;
  size_t gwsCap = 0;
  unsigned* gtick = nullptr;
  int adamStep = 0;
  float scale = 1.f;          // S
  bool trained = false;
  // dataset
  float* X = nullptr;
  float* Y = nullptr;
  int cap = 0, count = 0;
  double* xstar = nullptr;    // neq: reference solution of the collecting solve
  int target = IFEMGPU_LEARN_TARGET_ERROR;
  // training scratch (batch B)
  int B = 0;
  float *Xb = nullptr, *Yb = nullptr, *H1 = nullptr, *H2 = nullptr, *Yp = nullptr;
  float *dH1 = nullptr, *dH2 = nullptr, *dY = nullptr, *loss = nullptr;
  int* perm = nullptr;
  // solve scratch
  float *rc = nullptr, *h1 = nullptr, *h2 = nullptr, *yc = nullptr;
  float* nrm = nullptr;        // [0] |rc| of the last restriction, [1] S, [2] alpha
  // energy-optimal step: t = A z1, rc1 = R (r - t), the Galerkin coarse
  // matrix Ac = R A R^T (banded: 125 npv entries per row, columns at vertex
  // offsets -2..2 per direction) and its factor B = A R^T (per equation a
  // box of 4^3 vertices per component, from the equation's cell - 1)
  int reach = 0;               // max cell distance of two coupled equations
  float* t = nullptr;
  float* rc1 = nullptr;
  float* Bm = nullptr;
  float* Ac = nullptr;
  int acAssembly = -1;         // assembly count Ac was formed from
};

namespace {

constexpr int kT = 256;

__device__ inline bool stopped(const double* guard) { return guard && guard[0] != 0.0; }

// ---- transfer kernels --------------------------------------------------------

// rc = R r: warp per coarse unknown, fixed order (deterministic)
__global__ void k_restrict(const int* __restrict__ vPtr, const int* __restrict__ vEq,
                           const float* __restrict__ vW, const float* __restrict__ r,
                           float* __restrict__ rc, int nc, const double* guard)
{
  if (stopped(guard)) return;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nc) return;
  float s = 0.f;
  for (int k = vPtr[warp] + lane; k < vPtr[warp + 1]; k += 32) s += vW[k] * r[vEq[k]];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) rc[warp] = s;
}

// rc1 = R (r - t), and rc = R r (sub = 0) or rc1 (sub != 0): warp per coarse
// unknown, fixed order
__global__ void k_restrict2(const int* __restrict__ vPtr, const int* __restrict__ vEq,
                            const float* __restrict__ vW, const float* __restrict__ r,
                            const float* __restrict__ t, int sub, float* __restrict__ rc,
                            float* __restrict__ rc1, int nc, const double* guard)
{
  if (stopped(guard)) return;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nc) return;
  float a = 0.f, b = 0.f;
  for (int k = vPtr[warp] + lane; k < vPtr[warp + 1]; k += 32) {
    const int e = vEq[k];
    const float w = vW[k], re = r[e];
    a += w * re;
    b += w * (re - t[e]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  if (lane == 0) {
    rc[warp] = sub ? b : a;
    rc1[warp] = b;
  }
}

// B = A R^T, one row block per (equation i, component c): warp per item,
// lanes over the row's entries.  Slot (sx, sy, sz) of the item's 4^3 box is
// the coarse vertex cell(i) - 1 + (sx, sy, sz); an entry j of component c
// adds A_ij times its trilinear weights, which sit at the slots
// cell(j) - cell(i) + 1 + {0, 1} per direction (coupled equations lie at most
// one cell apart: checked on the host).  Per-lane sums, then a butterfly:
// the same order on every run.
__global__ void __launch_bounds__(kT)
k_galerkin_rows(const int* __restrict__ colptr, const int* __restrict__ rowidx,
                const double* __restrict__ A, const int* __restrict__ eqCell,
                const float4* __restrict__ eqFrac, int m, int npv, int n, float* __restrict__ Bm)
{
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int item = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); item < n * npv;
       item += warps) {
    const int i = item / npv, c = item - i * npv;
    const int ci = eqCell[i];
    const int cix = ci % m, ciy = (ci / m) % m, ciz = ci / (m * m);
    float acc[64];
#pragma unroll
    for (int q = 0; q < 64; q++) acc[q] = 0.f;
    for (int k = colptr[i] + lane; k < colptr[i + 1]; k += 32) {
      const int j = rowidx[k];
      const float4 f = eqFrac[j];
      if ((int)f.w != c) continue;
      const int cj = eqCell[j];
      const int dx = cj % m - cix + 1, dy = (cj / m) % m - ciy + 1, dz = cj / (m * m) - ciz + 1;
      const float a = (float)A[k];
      float hx[4], hy[4], hz[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        hx[q] = q == dx ? a * (1.f - f.x) : (q == dx + 1 ? a * f.x : 0.f);
        hy[q] = q == dy ? 1.f - f.y : (q == dy + 1 ? f.y : 0.f);
        hz[q] = q == dz ? 1.f - f.z : (q == dz + 1 ? f.z : 0.f);
      }
#pragma unroll
      for (int qz = 0; qz < 4; qz++)
#pragma unroll
        for (int qy = 0; qy < 4; qy++) {
          const float yz = hy[qy] * hz[qz];
#pragma unroll
          for (int qx = 0; qx < 4; qx++)
            acc[(qz * 4 + qy) * 4 + qx] = fmaf(hx[qx], yz, acc[(qz * 4 + qy) * 4 + qx]);
        }
    }
    float v0 = 0.f, v1 = 0.f;
#pragma unroll
    for (int q = 0; q < 32; q++) {
      float a0 = acc[q], a1 = acc[q + 32];
      for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      }
      if (q == lane) {
        v0 = a0;
        v1 = a1;
      }
    }
    float* out = Bm + (size_t)item * 64;
    out[lane] = v0;
    out[lane + 32] = v1;
  }
}

// Ac = R B, banded: warp per coarse unknown (vertex v, component c); the
// equations of v's support in list order, lanes over the slots of their B
// rows.  Column (v + o - 2, c') is stored at o npv + c' with o the vertex
// offset (0..4 per direction); the slots of one B row land on distinct
// columns, so every column is summed in list order.
__global__ void __launch_bounds__(kT)
k_galerkin_coarse(const int* __restrict__ vPtr, const int* __restrict__ vEq,
                  const float* __restrict__ vW, const int* __restrict__ eqCell,
                  const float* __restrict__ Bm, int m, int npv, int nc, float* __restrict__ Ac)
{
  extern __shared__ float gacc[];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int band = 125 * npv;
  float* acc = gacc + wib * band;
  const int row = blockIdx.x * (blockDim.x >> 5) + wib;
  if (row >= nc) return;
  for (int q = lane; q < band; q += 32) acc[q] = 0.f;
  __syncwarp();
  const int m1 = m + 1, v = row / npv;
  const int vx = v % m1, vy = (v / m1) % m1, vz = v / (m1 * m1);
  for (int k = vPtr[row]; k < vPtr[row + 1]; k++) {
    const int i = vEq[k];
    const float w = vW[k];
    const int ci = eqCell[i];
    // offset of slot 0 from v, plus 2: in 0..1 since v is a corner of cell(i)
    const int bx = ci % m + 1 - vx, by = (ci / m) % m + 1 - vy, bz = ci / (m * m) + 1 - vz;
    const float* Bi = Bm + (size_t)i * npv * 64;
    for (int q = lane; q < 64 * npv; q += 32) {
      const int cp = q >> 6, sl = q & 63;
      const int o = ((bz + (sl >> 4)) * 5 + by + ((sl >> 2) & 3)) * 5 + bx + (sl & 3);
      acc[o * npv + cp] += w * Bi[q];
    }
    __syncwarp();
  }
  float* out = Ac + (size_t)row * band;
  for (int q = lane; q < band; q += 32) out[q] = acc[q];
}

// alpha = (y, rc1) / (y, Ac y) for the coarse direction y (0 when the
// denominator is not positive or not finite): warp per coarse row, per-block
// partials of both sums in part[b] and part[nb + b], the last block sums
// them in fixed order.  With y = R^T-prolonged network output c, alpha is
// the coefficient that minimises the energy norm of the error after
// z = z1 + alpha c.
__global__ void __launch_bounds__(kT)
k_coarse_alpha(const float* __restrict__ Ac, const float* __restrict__ y,
               const float* __restrict__ rc1, int m, int npv, int nc, double* __restrict__ part,
               unsigned* counter, float* alphaOut, const double* guard)
{
  if (stopped(guard)) return;
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, m1 = m + 1, band = 125 * npv;
  const int warps = gridDim.x * (blockDim.x >> 5);
  float num = 0.f, den = 0.f;
  for (int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < nc; row += warps) {
    const int v = row / npv;
    const int vx = v % m1, vy = (v / m1) % m1, vz = v / (m1 * m1);
    const float* a = Ac + (size_t)row * band;
    float e = 0.f;
    for (int q = lane; q < band; q += 32) {
      const int o = q / npv, cp = q - o * npv;
      const int ux = vx + o % 5 - 2, uy = vy + (o / 5) % 5 - 2, uz = vz + o / 25 - 2;
      if (ux < 0 || ux > m || uy < 0 || uy > m || uz < 0 || uz > m) continue;
      e += a[q] * y[((uz * m1 + uy) * m1 + ux) * npv + cp];
    }
    for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
    if (lane == 0) {
      den += y[row] * e;
      num += y[row] * rc1[row];
    }
  }
  const double tn = blockReduceSumF(num, sh);
  const double td = blockReduceSumF(den, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = tn;
    part[gridDim.x + blockIdx.x] = td;
  }
  if (lastBlock(counter)) {
    const double n2 = finalSum(part, gridDim.x, sh);
    const double d2 = finalSum(part + gridDim.x, gridDim.x, sh);
    if (threadIdx.x == 0) {
      const double al = n2 / d2;
      *alphaOut = (d2 > 0.0 && al == al && al < 1e30 && al > -1e30) ? (float)al : 0.f;
    }
  }
}

// ec = Rn (x* sx - x) for the error of an iterate
__global__ void k_restrict_err(const int* __restrict__ vPtr, const int* __restrict__ vEq,
                               const float* __restrict__ vWn, const double* __restrict__ xs,
                               double sx, const float* __restrict__ x,
                               const float* __restrict__ fine, float* __restrict__ ec, int nc)
{
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nc) return;
  float s = 0.f;
  for (int k = vPtr[warp] + lane; k < vPtr[warp + 1]; k += 32) {
    const int e = vEq[k];
    float d = (float)(xs[e] * sx - (double)x[e]);
    if (fine) d -= fine[e];  // what the fine preconditioner already supplies
    s += vWn[k] * d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) ec[warp] = s;
}

__device__ float blockSumF(float v, float* sh)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  float s = 0.f;
  for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sh[i];
  __syncthreads();
  return s;  // every thread
}

// dataset row: X = [rc/|rc|, feat], Y = ec/|rc| (single block)
__global__ void k_store_pair(const float* __restrict__ rc, const float* __restrict__ ec,
                             const float* __restrict__ feat, float* __restrict__ X,
                             float* __restrict__ Y, int nc, int nf)
{
  __shared__ float sh[32];
  float s = 0.f;
  for (int i = threadIdx.x; i < nc; i += blockDim.x) s += rc[i] * rc[i];
  const float n = sqrtf(blockSumF(s, sh));
  const float inv = n > 0.f ? 1.f / n : 0.f;
  for (int i = threadIdx.x; i < nc; i += blockDim.x) {
    X[i] = rc[i] * inv;
    Y[i] = ec[i] * inv;
  }
  for (int i = threadIdx.x; i < nf; i += blockDim.x) X[nc + i] = feat[i];
}

// z_e += alpha sum_v w_ve y_(v,c); with q != 0 also (z, q): per-block
// partials, summed in fixed order by the last block into *dotOut
__global__ void __launch_bounds__(kT)
k_prolong_add(const int* __restrict__ eqCell, const float4* __restrict__ eqFrac,
              const float* __restrict__ y, const float* __restrict__ nrm, int m, int npv,
              float* __restrict__ z, int n, const float* __restrict__ q, double* __restrict__ part,
              unsigned* counter, double* dotOut, const double* pq, float* betaOut,
              const double* guard)
{
  if (stopped(guard)) return;
  __shared__ double sh[32];
  const float sc = nrm[2];  // the energy-optimal coefficient of the direction
  const int m1 = m + 1;
  float dot = 0.f;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int c = eqCell[e];
    const int ci = c % m, cj = (c / m) % m, ck = c / (m * m);
    const float4 f = eqFrac[e];
    const int comp = (int)f.w;
    float s = 0.f;
#pragma unroll
    for (int d = 0; d < 8; d++) {
      const int di = d & 1, dj = (d >> 1) & 1, dk = d >> 2;
      const float w = (di ? f.x : 1.f - f.x) * (dj ? f.y : 1.f - f.y) * (dk ? f.z : 1.f - f.z);
      s += w * y[(((ck + dk) * m1 + cj + dj) * m1 + ci + di) * npv + comp];
    }
    const float zi = z[e] + sc * s;
    z[e] = zi;
    if (q) dot += zi * q[e];
  }
  if (!q) return;
  const double t = blockReduceSumF(dot, sh);
  if (lastBlockDone(part, t, counter)) {
    const double v = finalSum(part, gridDim.x, sh);
    if (threadIdx.x == 0) {
      *dotOut = v;
      *betaOut = (float)(-v / *pq);  // flexible-CG beta
    }
  }
}

// ---- network kernels -----------------------------------------------------------

// ---- tensor-core inference ----------------------------------------------------
// One network layer y = act(W [x / |x|, x2] + b) on tcgen05 (kind::f16: BF16
// operands, FP32 accumulation in tensor memory).  W is packed in BF16 as
// 128 x 64 operand tiles (K-major core matrices, no swizzle), row tile major;
// the input vector is the MMA's B operand with N = 16 (row 0, zero rows
// 1..15): one right-hand side per solve iteration.  CTA (m, t) multiplies row
// tile m by K tile t (one bulk copy of 16 KB, four MMAs of K = 16) and stores
// its 128 partial sums; the last CTA of row tile m sums the partials of all K
// tiles in tile order, adds the bias and applies the activation.
constexpr int kTileRows = 128, kTileK = 64;
constexpr int kTileElems = kTileRows * kTileK;

struct InferSmem {
  __nv_bfloat16 A[kTileElems];   // one packed W tile (16 KB)
  __nv_bfloat16 B[16 * kTileK];  // the input slice as row 0 of 16
  unsigned long long mbarA, mbarD;
  uint32_t tmemSlot;
  int ok, last;
  float red[4];
};

// element offset of (row r, k) inside a packed tile (r < 128, k < 64)
__device__ __forceinline__ int tileOff(int r, int k)
{
  return (r >> 3) * 512 + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
}

// W (rows x cols, FP32 row-major) -> packed BF16 tiles (zero padding)
__global__ void k_pack_bf16(const float* __restrict__ W, int rows, int cols, int nKT,
                            __nv_bfloat16* __restrict__ out, size_t total)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t tile = i / kTileElems;
    const int e = (int)(i - tile * kTileElems);
    const int mt = (int)(tile / nKT), kt = (int)(tile - (size_t)mt * nKT);
    const int rem = e & 511, rem2 = rem & 63;
    const int r = ((e >> 9) << 3) | (rem2 >> 3), k = ((rem >> 6) << 3) | (rem2 & 7);
    const int row = mt * kTileRows + r, col = kt * kTileK + k;
    out[i] = __float2bfloat16(row < rows && col < cols ? W[(size_t)row * cols + col] : 0.f);
  }
}

__global__ void __launch_bounds__(128)
k_mlp_tc(const __nv_bfloat16* __restrict__ Wp, int nKT, const float* __restrict__ bias,
         const float* __restrict__ x, int cols1, const float* __restrict__ x2, int cols2,
         int normFirst, float* __restrict__ part, unsigned* __restrict__ tick,
         float* __restrict__ y, int rows, int relu, float* normOut, unsigned spin,
         const double* guard)
{
  if (stopped(guard)) return;
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char smraw[];
  InferSmem& sm = *reinterpret_cast<InferSmem*>(smraw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = blockIdx.x, kt = blockIdx.y;
  const uint32_t mbarA = smemAddr(&sm.mbarA), mbarD = smemAddr(&sm.mbarD);
  if (tid == 0) {
    mbarInit(mbarA, 1);
    mbarInit(mbarD, 1);
  }
  if (warp == 0) tmemAlloc(&sm.tmemSlot, 32);
  float inv = 1.f;
  if (normFirst) {  // |x| over the first cols1 inputs
    float q = 0.f;
    for (int i = tid; i < cols1; i += blockDim.x) q += x[i] * x[i];
    for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
    if (lane == 0) sm.red[warp] = q;
  }
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = sm.tmemSlot;
  if (normFirst) {
    const float nx = sqrtf((sm.red[0] + sm.red[1]) + (sm.red[2] + sm.red[3]));
    inv = nx > 0.f ? 1.f / nx : 0.f;
    if (mt == 0 && kt == 0 && tid == 0 && normOut) *normOut = nx;
  }
  if (tid == 0) {
    mbarExpectTx(mbarA, kTileElems * 2);
    bulkLoad(smemAddr(sm.A), Wp + ((size_t)mt * nKT + kt) * kTileElems, kTileElems * 2, mbarA);
  }
  // the input slice in BF16 as row 0 of the B operand
  for (int e = tid; e < 16 * kTileK; e += blockDim.x) {
    const int rem = e & 511, rem2 = rem & 63;
    const int n = ((e >> 9) << 3) | (rem2 >> 3), k = ((rem >> 6) << 3) | (rem2 & 7);
    float v = 0.f;
    if (n == 0) {
      const int col = kt * kTileK + k;
      v = col < cols1 ? x[col] * inv : (col < cols1 + cols2 ? x2[col - cols1] : 0.f);
    }
    sm.B[e] = __float2bfloat16(v);
  }
  fenceProxyAsync();
  __syncthreads();
  if (tid == 0) {
    int ok = mbarWait(mbarA, 0, spin) ? 1 : 0;
    if (ok) {
      tcFenceAfter();
      const uint32_t idesc = instrDescBF16(kTileRows, 16);
      const uint32_t a0 = smemAddr(sm.A), b0 = smemAddr(sm.B);
#pragma unroll
      for (int s = 0; s < kTileK / 16; s++)  // K = 16 BF16 = 32 bytes: two core matrices
        mmaBF16(tmem, smemDesc(a0 + s * 256), smemDesc(b0 + s * 256), idesc, s > 0 ? 1u : 0u);
      mmaCommit(mbarD);
      ok = mbarWait(mbarD, 0, spin) ? 2 : 0;
    }
    sm.ok = ok;
  }
  __syncthreads();
  tcFenceAfter();
  float v[16];
  if (sm.ok == 2) {
    tmemLoad16(tmem + ((uint32_t)(32 * warp) << 16), v);
  } else {
    v[0] = __int_as_float(0x7FC00000);  // a wait gave up: NaN ends the solve's learned step
  }
  const int row = mt * kTileRows + warp * 32 + lane;
  if (row < rows) part[(size_t)kt * rows + row] = v[0];
  __threadfence();
  __syncthreads();
  if (tid == 0) sm.last = atomicAdd(tick + mt, 1u) == gridDim.y - 1;
  __syncthreads();
  if (sm.last) {
    __threadfence();
    if (row < rows) {
      float acc = 0.f;
      for (int t = 0; t < (int)gridDim.y; t++) acc += __ldcg(part + (size_t)t * rows + row);
      acc += bias[row];
      y[row] = relu ? fmaxf(acc, 0.f) : acc;
    }
    if (tid == 0) tick[mt] = 0u;
  }
  // a copy still in flight after a give-up lands before the CTA exits
  if (tid == 0 && sm.ok == 0) mbarWait(mbarA, 0, spin);
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (warp == 0) tmemDealloc(tmem, 32);
}

// C (M x N) = op(A) op(B) (+ C when accumulate); row-major; op transposes
// when its flag is set (A is M x K or K x M, B is K x N or N x K).  On the
// tensor cores in 3xTF32 (hi hi + hi lo + lo hi, FP32 accumulation in tensor
// memory), so the training keeps FP32 accuracy: one CTA of 128 threads per
// 128 x 128 tile of C and slice of K (gridDim.z slices of kChunks chunks of
// 32), each chunk staged by the threads (the loads follow the operand's
// contiguous direction; split into TF32 hi/lo parts in the K-major
// core-matrix layout) and contracted by twelve MMAs, the accumulator read
// back by the four warps (32 rows each).  With several slices every CTA
// stores its partial tile and the last CTA of a tile (ticket) sums the
// slices in order: the result does not depend on which CTA finishes first.
constexpr int kGT = 128;  // tile of C: rows and columns
struct GemmSmem {
  float Ahi[kGT * tc::kK], Alo[kGT * tc::kK], Bhi[kGT * tc::kK], Blo[kGT * tc::kK];
  unsigned long long mbar;
  uint32_t tmemSlot;
  int ok, last;
};

__global__ void __launch_bounds__(128)
k_gemm_tc(const float* __restrict__ A, const float* __restrict__ B, float* __restrict__ C, int M,
          int N, int K, int lda, int ldb, int ldc, int transA, int transB, int accumulate,
          int kChunks, float* __restrict__ P, unsigned* __restrict__ tick, unsigned spin)
{
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char smraw[];
  GemmSmem& sm = *reinterpret_cast<GemmSmem*>(smraw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kGT, n0 = blockIdx.x * kGT;
  const int kBeg = blockIdx.z * kChunks * kK, kEnd = min(K, kBeg + kChunks * kK);
  const int slices = gridDim.z;
  const uint32_t mbar = smemAddr(&sm.mbar);
  if (tid == 0) {
    mbarInit(mbar, 1);
    sm.ok = 1;
  }
  if (warp == 0) tmemAlloc(&sm.tmemSlot, kGT);
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = sm.tmemSlot;
  const uint32_t idesc = instrDescTF32(kGT, kGT);
  uint32_t phase = 0;
  bool ok = true;
  for (int k0 = kBeg; k0 < kEnd && ok; k0 += kK) {
    // op(A)[m0 + r][k0 + k] and op(B)[k0 + k][n0 + r] for r < 128, k < 32
    for (int i = tid; i < kGT * kK; i += blockDim.x) {
      int r, k;
      if (transA) { k = i / kGT; r = i % kGT; }  // A stored K x M: consecutive threads along m
      else { r = i / kK; k = i % kK; }          // A stored M x K: along k
      const int gm = m0 + r, gk = k0 + k;
      float va = 0.f;
      if (gm < M && gk < kEnd) va = transA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
      float hi, lo;
      splitTF32(va, hi, lo);
      sm.Ahi[kmaj(r, k)] = hi;
      sm.Alo[kmaj(r, k)] = lo;
      if (transB) { r = i / kK; k = i % kK; }   // B stored N x K: along k
      else { k = i / kGT; r = i % kGT; }        // B stored K x N: along n
      const int gn = n0 + r, gkb = k0 + k;
      float vb = 0.f;
      if (gn < N && gkb < kEnd) vb = transB ? B[(size_t)gn * ldb + gkb] : B[(size_t)gkb * ldb + gn];
      splitTF32(vb, hi, lo);
      sm.Bhi[kmaj(r, k)] = hi;
      sm.Blo[kmaj(r, k)] = lo;
    }
    fenceProxyAsync();
    __syncthreads();
    if (tid == 0) {
      tcFenceAfter();
      const uint32_t ah = smemAddr(sm.Ahi), al = smemAddr(sm.Alo);
      const uint32_t bh = smemAddr(sm.Bhi), bl = smemAddr(sm.Blo);
#pragma unroll
      for (int st = 0; st < kK / 8; st++) {
        const uint32_t off = st * 256;
        const uint32_t acc = (k0 > kBeg || st > 0) ? 1u : 0u;
        mmaTF32(tmem, smemDesc(ah + off), smemDesc(bh + off), idesc, acc);
        mmaTF32(tmem, smemDesc(ah + off), smemDesc(bl + off), idesc, 1u);
        mmaTF32(tmem, smemDesc(al + off), smemDesc(bh + off), idesc, 1u);
      }
      mmaCommit(mbar);
      if (!mbarWait(mbar, phase, spin)) sm.ok = 0;
    }
    phase ^= 1u;
    __syncthreads();  // the operand tiles are free again (or the wait gave up)
    ok = sm.ok != 0;
    tcFenceAfter();
  }
  // this CTA's tile: to C (one slice) or to its partial slot; an empty slice
  // is zero, a wait that gave up NaN
  const int r = warp * 32 + lane, gm = m0 + r;
  const bool any = kEnd > kBeg;
  float* Pt = P + ((size_t)blockIdx.z * gridDim.x * gridDim.y + blockIdx.y * gridDim.x + blockIdx.x) *
                  kGT * kGT;
  for (int c16 = 0; c16 < kGT / 16; c16++) {
    float v[16];
    if (any && ok) {
      tmemLoad16(tmem + ((uint32_t)(32 * warp) << 16) + 16 * c16, v);
    } else {
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = any ? __int_as_float(0x7FC00000) : 0.f;
    }
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const int c = 16 * c16 + j, gn = n0 + c;
      if (slices > 1) {
        Pt[(size_t)r * kGT + c] = v[j];
      } else if (gm < M && gn < N) {
        float* cp = C + (size_t)gm * ldc + gn;
        *cp = accumulate ? *cp + v[j] : v[j];
      }
    }
  }
  if (!ok && tid == 0) mbarWait(mbar, phase ^ 1u, spin);  // the MMAs given up on finish first
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (warp == 0) tmemDealloc(tmem, kGT);
  if (slices == 1) return;
  __threadfence();
  __syncthreads();
  const int tile = blockIdx.y * gridDim.x + blockIdx.x;
  if (tid == 0) sm.last = atomicAdd(tick + tile, 1u) == (unsigned)slices - 1;
  __syncthreads();
  if (!sm.last) return;
  __threadfence();
  if (gm < M) {
    const size_t tstride = (size_t)gridDim.x * gridDim.y * kGT * kGT;
    const float* P0 = P + (size_t)tile * kGT * kGT + (size_t)r * kGT;
    for (int c = 0; c < kGT && n0 + c < N; c++) {
      float acc = 0.f;
      for (int z = 0; z < slices; z++) acc += __ldcg(P0 + z * tstride + c);
      float* cp = C + (size_t)gm * ldc + n0 + c;
      *cp = accumulate ? *cp + acc : acc;
    }
  }
  if (tid == 0) tick[tile] = 0u;
}

// H = act(H + b) row-wise
__global__ void k_bias_act(float* __restrict__ H, const float* __restrict__ b, int rows, int cols,
                           int relu)
{
  const size_t n = (size_t)rows * cols;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float v = H[i] + b[i % cols];
    H[i] = relu ? fmaxf(v, 0.f) : v;
  }
}

// dH *= (H > 0)
__global__ void k_relu_back(float* __restrict__ dH, const float* __restrict__ H, size_t n)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    if (!(H[i] > 0.f)) dH[i] = 0.f;
}

// g = column sums of D (rows x cols), fixed order per column
__global__ void k_colsum(const float* __restrict__ D, float* __restrict__ g, int rows, int cols)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; r++) s += D[(size_t)r * cols + c];
  g[c] = s;
}

// dY = 2 (Yp - Y/S) / n (when dY != 0), per-block partial sums of (Yp - Y/S)^2
__global__ void k_mse(const float* __restrict__ Yp, const float* __restrict__ Y, float invS,
                      float* __restrict__ dY, size_t n, float* __restrict__ part)
{
  __shared__ float sh[32];
  float s = 0.f;
  const float g = 2.f / (float)n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float d = Yp[i] - Y[i] * invS;
    if (dY) dY[i] = d * g;
    s += d * d;
  }
  const float t = blockSumF(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void k_adam(float* __restrict__ th, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float c1,
                       float c2, float eps)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    th[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// batch rows gathered through a permutation
__global__ void k_gather_rows(const float* __restrict__ src, const int* __restrict__ idx,
                              float* __restrict__ dst, int rows, int cols)
{
  const size_t n = (size_t)rows * cols;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    dst[i] = src[(size_t)idx[r] * cols + c];
  }
}

__global__ void k_sum_sq(const float* __restrict__ v, size_t n, float* __restrict__ part)
{
  __shared__ float sh[32];
  float s = 0.f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    s += v[i] * v[i];
  const float t = blockSumF(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// K is split into up to 8 slices, for about 96 CTAs per product (the
// training products have few 128 x 128 tiles and long K; the last CTA of a
// tile reads every slice's partial tile, which bounds the useful split)
void sgemm(cudaStream_t s, LearnState* L, const float* A, const float* B, float* C, int M, int N,
           int K, int lda, int ldb, int ldc, int tA, int tB, int acc)
{
  const int tn = (N + kGT - 1) / kGT, tm = (M + kGT - 1) / kGT;
  const int chunks = std::max(1, (K + tc::kK - 1) / tc::kK);
  int slices = std::min(std::min(chunks, 8), std::max(1, 96 / (tn * tm)));
  const int per = (chunks + slices - 1) / slices;
  slices = (chunks + per - 1) / per;
  if ((size_t)slices * tn * tm * kGT * kGT > L->gwsCap || tn * tm > kGemmTiles) slices = 1;
  k_gemm_tc<<<dim3(tn, tm, slices), 128, sizeof(GemmSmem), s>>>(
      A, B, C, M, N, K, lda, ldb, ldc, tA, tB, acc, slices > 1 ? per : chunks, L->gws, L->gtick,
      tc::kSpinLimit);
}

void freeLearn(LearnState* L)
{
  void* ptrs[] = {L->eqCell, L->eqFrac, L->vPtr, L->vEq, L->vW, L->vWn, L->theta, L->grad,
                  L->am, L->av, L->wtc, L->tpart, L->tick, L->X, L->Y, L->xstar, L->Xb, L->Yb, L->H1, L->H2,
                  L->Yp, L->dH1, L->dH2, L->dY, L->loss, L->perm, L->rc, L->h1, L->h2,
                  L->yc, L->nrm, L->feat, L->t, L->rc1, L->Bm, L->Ac, L->gws, L->gtick};
  for (void* p : ptrs)
    if (p) cudaFree(p);
}

constexpr int kLossParts = 128;

// forward (+ backward when grad) of one batch of Bn rows in Xb/Yb; the
// per-block loss partials go to L->loss[0..kLossParts)
void batchPass(cudaStream_t s, LearnState* L, int Bn, float invS, bool grad)
{
  const int nc = L->nc, nh = L->nh, nin = L->nin;
  const float* th = L->theta;
  float* g = L->grad;
  sgemm(s, L, L->Xb, th + L->oW1, L->H1, Bn, nh, nin, nin, nin, nh, 0, 1, 0);
  k_bias_act<<<256, kT, 0, s>>>(L->H1, th + L->ob1, Bn, nh, 1);
  sgemm(s, L, L->H1, th + L->oW2, L->H2, Bn, nh, nh, nh, nh, nh, 0, 1, 0);
  k_bias_act<<<256, kT, 0, s>>>(L->H2, th + L->ob2, Bn, nh, 1);
  sgemm(s, L, L->H2, th + L->oW3, L->Yp, Bn, nc, nh, nh, nh, nc, 0, 1, 0);
  k_bias_act<<<256, kT, 0, s>>>(L->Yp, th + L->ob3, Bn, nc, 0);
  k_mse<<<kLossParts, kT, 0, s>>>(L->Yp, L->Yb, invS, grad ? L->dY : nullptr, (size_t)Bn * nc,
                                  L->loss);
  if (!grad) return;
  sgemm(s, L, L->dY, L->H2, g + L->oW3, nc, nh, Bn, nc, nh, nh, 1, 0, 0);
  k_colsum<<<(nc + kT - 1) / kT, kT, 0, s>>>(L->dY, g + L->ob3, Bn, nc);
  sgemm(s, L, L->dY, th + L->oW3, L->dH2, Bn, nh, nc, nc, nh, nh, 0, 0, 0);
  k_relu_back<<<256, kT, 0, s>>>(L->dH2, L->H2, (size_t)Bn * nh);
  sgemm(s, L, L->dH2, L->H1, g + L->oW2, nh, nh, Bn, nh, nh, nh, 1, 0, 0);
  k_colsum<<<(nh + kT - 1) / kT, kT, 0, s>>>(L->dH2, g + L->ob2, Bn, nh);
  sgemm(s, L, L->dH2, th + L->oW2, L->dH1, Bn, nh, nh, nh, nh, nh, 0, 0, 0);
  k_relu_back<<<256, kT, 0, s>>>(L->dH1, L->H1, (size_t)Bn * nh);
  sgemm(s, L, L->dH1, L->Xb, g + L->oW1, nh, nin, Bn, nh, nin, nin, 1, 0, 0);
  k_colsum<<<(nh + kT - 1) / kT, kT, 0, s>>>(L->dH1, g + L->ob1, Bn, nh);
}

// the BF16 operand tiles of the three layers from the FP32 master weights
void packWeights(cudaStream_t s, LearnState* L)
{
  const int rows[3] = {L->nh, L->nh, L->nc}, cols[3] = {L->nin, L->nh, L->nh};
  const int off[3] = {L->oW1, L->oW2, L->oW3};
  for (int l = 0; l < 3; l++) {
    const size_t total = (size_t)L->Mt[l] * L->nKT[l] * kTileElems;
    k_pack_bf16<<<512, kT, 0, s>>>(L->theta + off[l], rows[l], cols[l], L->nKT[l],
                                   L->wtc + L->pOff[l], total);
  }
}

ifemgpu_status readLoss(ifemgpu_ctx* ctx, LearnState* L, double denom, double* out)
{
  float part[kLossParts];
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(part, L->loss, sizeof(part), cudaMemcpyDeviceToHost, ctx->stream));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double sl = 0.0;
  for (float v : part) sl += v;
  *out = sl / denom;
  return IFEMGPU_OK;
}

ifemgpu_status ensureBatch(ifemgpu_ctx* ctx, LearnState* L, int B)
{
  if (L->B >= B) return IFEMGPU_OK;
  float** bufs[] = {&L->Xb, &L->Yb, &L->H1, &L->H2, &L->Yp, &L->dH1, &L->dH2, &L->dY};
  for (float** p : bufs)
    if (*p) { cudaFree(*p); *p = nullptr; }
  L->B = 0;
  const size_t nc = L->nc, nh = L->nh, nin = L->nin;
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->Xb, sizeof(float) * B * nin));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->Yb, sizeof(float) * B * nc));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->Yp, sizeof(float) * B * nc));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->dY, sizeof(float) * B * nc));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->H1, sizeof(float) * B * nh));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->H2, sizeof(float) * B * nh));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->dH1, sizeof(float) * B * nh));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->dH2, sizeof(float) * B * nh));
  // split-K workspace: up to 96 CTAs of 128 x 128 partial tiles
  if (!L->gws) {
    L->gwsCap = (size_t)96 * 128 * 128;
    IFEMGPU_CUDA(ctx, cudaMalloc(&L->gws, sizeof(float) * L->gwsCap));
    IFEMGPU_CUDA(ctx, cudaMalloc(&L->gtick, sizeof(unsigned) * kGemmTiles));
    IFEMGPU_CUDA(ctx, cudaMemset(L->gtick, 0, sizeof(unsigned) * kGemmTiles));
  }
  L->B = B;
  return IFEMGPU_OK;
}

}  // namespace

void destroyLearn(ifemgpu_ctx* ctx)
{
  if (!ctx->learn) return;
  freeLearn(ctx->learn);
  delete ctx->learn;
  ctx->learn = nullptr;
}

ifemgpu_status learnSetup(ifemgpu_ctx* ctx, int m, int nh, int capacity, unsigned seed,
                          int fieldInputs)
{
  if (ctx->patches.size() != 1)
    return setError(ctx, IFEMGPU_UNSUPPORTED, "learned correction: one patch per context");
  const HostPatch& pc = ctx->patches[0];
  if (pc.dim != 3)
    return setError(ctx, IFEMGPU_UNSUPPORTED, "learned correction: 3D patches");
  if (m < 1 || m > 32 || nh < 8 || nh > 1024 || capacity < 1)
    return setError(ctx, IFEMGPU_INVALID_ARG, "learned correction: bad sizes");
  if (fieldInputs && pc.logk.empty())
    return setError(ctx, IFEMGPU_NOT_READY, "learned correction: field inputs without a log-conductivity field");
  destroyLearn(ctx);
  LearnState* L = new LearnState;
  ctx->learn = L;
  ctx->learnGen++;
  L->m = m;
  L->nh = nh;
  L->npv = pc.npv;
  const int nv = (m + 1) * (m + 1) * (m + 1);
  L->nc = nv * pc.npv;
  L->nf = fieldInputs ? nv : 0;
  L->nin = L->nc + L->nf;
  const int nc = L->nc, neq = ctx->neq, npv = pc.npv, nin = L->nin;
  std::vector<std::vector<std::pair<int, float>>> flist(L->nf);
  // coarse cell and trilinear weights of every free equation's Greville point
  std::vector<double> gr[3];
  for (int d = 0; d < 3; d++) {
    const auto& U = pc.knots[d];
    const int p = pc.p[d], n = pc.n[d];
    const double u0 = U[p], u1 = U[n];
    gr[d].resize(n);
    for (int i = 0; i < n; i++) {
      double s = 0.0;
      for (int k = 1; k <= p; k++) s += U[i + k];
      gr[d][i] = p > 0 ? (s / p - u0) / (u1 - u0) : 0.0;
    }
  }
  // coupling reach in coarse cells: nodes at most p apart in one direction
  // (the box couplings of one patch) lie in cells at most `reach` apart
  L->reach = 0;
  for (int d = 0; d < 3; d++) {
    auto cellOf = [&](int i) {
      return std::min(m - 1, std::max(0, (int)std::floor(gr[d][i] * m)));
    };
    for (int i = 0; i < pc.n[d]; i++)
      for (int j = i + 1; j <= std::min(pc.n[d] - 1, i + pc.p[d]); j++)
        L->reach = std::max(L->reach, std::abs(cellOf(j) - cellOf(i)));
  }
  std::vector<int> cell(neq, 0);
  std::vector<float4> frac(neq, make_float4(0.f, 0.f, 0.f, 0.f));
  std::vector<std::vector<std::pair<int, float>>> vlist(nc);
  for (int node = 0; node < pc.nnod; node++) {
    const int ii = node % pc.n[0], jj = (node / pc.n[0]) % pc.n[1],
              kk = node / (pc.n[0] * pc.n[1]);
    const double t[3] = {gr[0][ii] * m, gr[1][jj] * m, gr[2][kk] * m};
    int c[3];
    float f[3];
    for (int d = 0; d < 3; d++) {
      c[d] = std::min(m - 1, std::max(0, (int)std::floor(t[d])));
      f[d] = (float)std::min(1.0, std::max(0.0, t[d] - c[d]));
    }
    for (int dd = 0; dd < 8 && L->nf; dd++) {  // field inputs: every control point
      const int di = dd & 1, dj = (dd >> 1) & 1, dk = dd >> 2;
      const float w = (di ? f[0] : 1.f - f[0]) * (dj ? f[1] : 1.f - f[1]) *
                      (dk ? f[2] : 1.f - f[2]);
      flist[((c[2] + dk) * (m + 1) + c[1] + dj) * (m + 1) + c[0] + di].push_back({node, w});
    }
    const int first = ctx->madof[pc.mlgn[node]] - 1;
    for (int comp = 0; comp < npv; comp++) {
      const int eq = ctx->meqn[first + comp];
      if (eq <= 0) continue;
      cell[eq - 1] = (c[2] * m + c[1]) * m + c[0];
      frac[eq - 1] = make_float4(f[0], f[1], f[2], (float)comp);
      for (int dd = 0; dd < 8; dd++) {
        const int di = dd & 1, dj = (dd >> 1) & 1, dk = dd >> 2;
        const float w = (di ? f[0] : 1.f - f[0]) * (dj ? f[1] : 1.f - f[1]) *
                        (dk ? f[2] : 1.f - f[2]);
        const int v = ((c[2] + dk) * (m + 1) + c[1] + dj) * (m + 1) + c[0] + di;
        vlist[v * npv + comp].push_back({eq - 1, w});
      }
    }
  }
  std::vector<int> vptr(nc + 1, 0), veq;
  std::vector<float> vw, vwn;
  for (int v = 0; v < nc; v++) {
    double sw = 0.0;
    for (auto& pr : vlist[v]) sw += pr.second;
    for (auto& pr : vlist[v]) {
      veq.push_back(pr.first);
      vw.push_back(pr.second);
      vwn.push_back(sw > 0 ? (float)(pr.second / sw) : 0.f);
    }
    vptr[v + 1] = (int)veq.size();
  }
  L->featPtr.assign(L->nf + 1, 0);
  for (int v = 0; v < L->nf; v++) {
    double sw = 0.0;
    for (auto& pr : flist[v]) sw += pr.second;
    for (auto& pr : flist[v]) {
      L->featEq.push_back(pr.first);
      L->featW.push_back(sw > 0 ? (float)(pr.second / sw) : 0.f);
    }
    L->featPtr[v + 1] = (int)L->featEq.size();
  }
  auto up = [&](auto** dst, const auto* src, size_t n) -> ifemgpu_status {
    IFEMGPU_CUDA(ctx, cudaMalloc((void**)dst, sizeof(**dst) * std::max<size_t>(n, 1)));
    if (n) IFEMGPU_CUDA(ctx, cudaMemcpy(*dst, src, sizeof(**dst) * n, cudaMemcpyHostToDevice));
    return IFEMGPU_OK;
  };
  ifemgpu_status st;
  if ((st = up(&L->eqCell, cell.data(), cell.size())) != IFEMGPU_OK) return st;
  if ((st = up(&L->eqFrac, frac.data(), frac.size())) != IFEMGPU_OK) return st;
  if ((st = up(&L->vPtr, vptr.data(), vptr.size())) != IFEMGPU_OK) return st;
  if ((st = up(&L->vEq, veq.data(), veq.size())) != IFEMGPU_OK) return st;
  if ((st = up(&L->vW, vw.data(), vw.size())) != IFEMGPU_OK) return st;
  if ((st = up(&L->vWn, vwn.data(), vwn.size())) != IFEMGPU_OK) return st;
  // parameters: W1 (nh x nin), b1, W2 (nh x nh), b2, W3 (nc x nh), b3; He
  // initialisation from the seed, zero biases
  L->oW1 = 0;
  L->ob1 = L->oW1 + nh * nin;
  L->oW2 = L->ob1 + nh;
  L->ob2 = L->oW2 + nh * nh;
  L->oW3 = L->ob2 + nh;
  L->ob3 = L->oW3 + nc * nh;
  L->nparam = L->ob3 + nc;
  std::vector<float> th(L->nparam, 0.f);
  std::mt19937 rng(seed);
  auto fill = [&](int off, int count, double sd) {
    std::normal_distribution<double> nd(0.0, sd);
    for (int i = 0; i < count; i++) th[off + i] = (float)nd(rng);
  };
  fill(L->oW1, nh * nin, std::sqrt(2.0 / nin));
  fill(L->oW2, nh * nh, std::sqrt(2.0 / nh));
  fill(L->oW3, nc * nh, std::sqrt(1.0 / nh));
  if ((st = up(&L->theta, th.data(), th.size())) != IFEMGPU_OK) return st;
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->grad, sizeof(float) * L->nparam));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->am, sizeof(float) * L->nparam));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->av, sizeof(float) * L->nparam));
  IFEMGPU_CUDA(ctx, cudaMemset(L->am, 0, sizeof(float) * L->nparam));
  IFEMGPU_CUDA(ctx, cudaMemset(L->av, 0, sizeof(float) * L->nparam));
  {
    const int rows[3] = {nh, nh, nc}, cols[3] = {nin, nh, nh};
    size_t at = 0;
    int parts = 0, tiles = 0;
    for (int l = 0; l < 3; l++) {
      L->Mt[l] = (rows[l] + kTileRows - 1) / kTileRows;
      L->nKT[l] = (cols[l] + kTileK - 1) / kTileK;
      L->pOff[l] = at;
      at += (size_t)L->Mt[l] * L->nKT[l] * kTileElems;
      parts = std::max(parts, L->nKT[l] * rows[l]);
      tiles = std::max(tiles, L->Mt[l]);
    }
    IFEMGPU_CUDA(ctx, cudaMalloc(&L->wtc, sizeof(__nv_bfloat16) * at));
    IFEMGPU_CUDA(ctx, cudaMalloc(&L->tpart, sizeof(float) * parts));
    IFEMGPU_CUDA(ctx, cudaMalloc(&L->tick, sizeof(unsigned) * tiles));
    IFEMGPU_CUDA(ctx, cudaMemset(L->tick, 0, sizeof(unsigned) * tiles));
    IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)sizeof(GemmSmem)));
  }
  L->cap = capacity;
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->X, sizeof(float) * (size_t)capacity * nin));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->Y, sizeof(float) * (size_t)capacity * nc));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->feat, sizeof(float) * std::max(L->nf, 1)));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->xstar, sizeof(double) * std::max(neq, 1)));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->perm, sizeof(int) * capacity));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->loss, sizeof(float) * kLossParts));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->rc, sizeof(float) * nc));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->rc1, sizeof(float) * nc));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->t, sizeof(float) * std::max(neq, 1)));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->yc, sizeof(float) * nc));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->h1, sizeof(float) * nh));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->h2, sizeof(float) * nh));
  IFEMGPU_CUDA(ctx, cudaMalloc(&L->nrm, sizeof(float) * 4));
  IFEMGPU_CUDA(ctx, cudaMemset(L->nrm, 0, sizeof(float) * 4));
  IFEMGPU_CUDA(ctx, cudaMemcpy(L->nrm + 1, &L->scale, sizeof(float), cudaMemcpyHostToDevice));
  return IFEMGPU_OK;
}

double* learnXstar(ifemgpu_ctx* ctx) { return ctx->learn ? ctx->learn->xstar : nullptr; }

// field inputs of the current log-conductivity field (host restriction,
// uploaded when the field changed); call outside stream capture
ifemgpu_status learnPrepare(ifemgpu_ctx* ctx)
{
  LearnState* L = ctx->learn;
  if (!L || !L->nf || L->featVersion == ctx->fieldVersion) return IFEMGPU_OK;
  const std::vector<double>& g = ctx->patches[0].logk;
  std::vector<float> f(L->nf, 0.f);
  for (int v = 0; v < L->nf; v++) {
    double s = 0.0;
    for (int k = L->featPtr[v]; k < L->featPtr[v + 1]; k++) s += L->featW[k] * g[L->featEq[k]];
    f[v] = (float)s;
  }
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  IFEMGPU_CUDA(ctx, cudaMemcpy(L->feat, f.data(), sizeof(float) * L->nf, cudaMemcpyHostToDevice));
  L->featVersion = ctx->fieldVersion;
  return IFEMGPU_OK;
}

// one iterate (r, x of the system scaled by sx; fine = the fine
// preconditioner's output for r, t = A fine) -> one pair: input R r (target
// ERROR) or R (r - t) (target COMPLEMENT), target Rn (x* sx - x) or
// Rn (x* sx - x - fine)
ifemgpu_status learnRecord(ifemgpu_ctx* ctx, const float* r, const float* x, double sx,
                           const float* fine, const float* t)
{
  LearnState* L = ctx->learn;
  if (!L || L->count >= L->cap) return IFEMGPU_OK;
  cudaStream_t s = ctx->stream;
  const int nc = L->nc;
  const int blocks = (nc * 32 + kT - 1) / kT;
  const bool comp = L->target == IFEMGPU_LEARN_TARGET_COMPLEMENT;
  if (comp && (!fine || !t))
    return setError(ctx, IFEMGPU_INVALID_ARG, "internal: complement pair without the fine step");
  if (comp)
    k_restrict2<<<blocks, kT, 0, s>>>(L->vPtr, L->vEq, L->vW, r, t, 1, L->rc, L->rc1, nc, nullptr);
  else
    k_restrict<<<blocks, kT, 0, s>>>(L->vPtr, L->vEq, L->vW, r, L->rc, nc, nullptr);
  k_restrict_err<<<blocks, kT, 0, s>>>(L->vPtr, L->vEq, L->vWn, L->xstar, sx, x,
                                       comp ? fine : nullptr, L->yc, nc);
  k_store_pair<<<1, kT, 0, s>>>(L->rc, L->yc, L->feat, L->X + (size_t)L->count * L->nin,
                                L->Y + (size_t)L->count * nc, nc, L->nf);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  L->count++;
  return IFEMGPU_OK;
}

float* learnT(ifemgpu_ctx* ctx) { return ctx->learn ? ctx->learn->t : nullptr; }

// The Galerkin coarse matrix Ac = R A R^T of the assembled matrix (through
// B = A R^T), formed once per assembly; it prices the network's direction in
// the energy norm.
ifemgpu_status learnGalerkin(ifemgpu_ctx* ctx)
{
  LearnState* L = ctx->learn;
  if (L->acAssembly == ctx->assemblies) return IFEMGPU_OK;
  if (L->reach > 1)
    return setError(ctx, IFEMGPU_UNSUPPORTED,
                    "learned correction: coarse cells narrower than the matrix coupling "
                    "(use fewer coarse cells)");
  const int n = ctx->neq, npv = L->npv, nc = L->nc;
  if (!L->Bm) {
    IFEMGPU_CUDA(ctx, cudaMalloc(&L->Bm, sizeof(float) * 64 * (size_t)npv * std::max(n, 1)));
    IFEMGPU_CUDA(ctx, cudaMalloc(&L->Ac, sizeof(float) * 125 * (size_t)npv * nc));
  }
  cudaStream_t s = ctx->stream;
  int sms = 0;
  IFEMGPU_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->opts.device));
  const long long items = (long long)n * npv;
  const int wpb = kT / 32;
  const int rb = (int)std::min<long long>((items + wpb - 1) / wpb, (long long)sms * 16);
  if (rb > 0)
    k_galerkin_rows<<<rb, kT, 0, s>>>(ctx->d_colptr, ctx->d_rowidx, ctx->d_K, L->eqCell, L->eqFrac,
                                      L->m, npv, n, L->Bm);
  const size_t sm = sizeof(float) * wpb * 125 * npv;
  k_galerkin_coarse<<<(nc + wpb - 1) / wpb, kT, sm, s>>>(L->vPtr, L->vEq, L->vW, L->eqCell, L->Bm,
                                                         L->m, npv, nc, L->Ac);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  L->acAssembly = ctx->assemblies;
  return IFEMGPU_OK;
}

// the network's three layers on the tensor cores: L->rc (and the field
// features) -> L->yc
void inferTC(ifemgpu_ctx* ctx, const double* guard)
{
  LearnState* L = ctx->learn;
  cudaStream_t s = ctx->stream;
  const int nc = L->nc, nh = L->nh;
  const unsigned spin = ctx->dbg.mbarSpin ? ctx->dbg.mbarSpin : tc::kSpinLimit;
  const size_t sm = sizeof(InferSmem);
  k_mlp_tc<<<dim3(L->Mt[0], L->nKT[0]), 128, sm, s>>>(
      L->wtc + L->pOff[0], L->nKT[0], L->theta + L->ob1, L->rc, nc, L->feat, L->nf, 1, L->tpart,
      L->tick, L->h1, nh, 1, L->nrm, spin, guard);
  k_mlp_tc<<<dim3(L->Mt[1], L->nKT[1]), 128, sm, s>>>(
      L->wtc + L->pOff[1], L->nKT[1], L->theta + L->ob2, L->h1, nh, nullptr, 0, 0, L->tpart,
      L->tick, L->h2, nh, 1, nullptr, spin, guard);
  k_mlp_tc<<<dim3(L->Mt[2], L->nKT[2]), 128, sm, s>>>(
      L->wtc + L->pOff[2], L->nKT[2], L->theta + L->ob3, L->h2, nh, nullptr, 0, 0, L->tpart,
      L->tick, L->yc, nc, 0, nullptr, spin, guard);
}

// z = z1 + alpha R^T y: y the BF16 network's coarse direction for the input
// R r (target ERROR) or R (r - t) (target COMPLEMENT), t = A z1 computed by
// the caller, alpha = (y, R (r - t)) / (y, Ac y) the coefficient that
// minimises the energy norm of the error after the step (0 when the
// direction carries no energy).  With q != 0 the prolongation also forms
// (z, q) over its grid of nparts blocks and the last block stores it in
// *dotOut and -(z, q) / *pq in *betaOut.  Every kernel returns at once when
// *guard != 0.
ifemgpu_status learnApply(ifemgpu_ctx* ctx, const float* r, float* z, const float* t,
                          const float* q, double* part, int nparts, unsigned* counter,
                          unsigned* counter2, double* dotOut, const double* pq, float* betaOut,
                          const double* guard)
{
  LearnState* L = ctx->learn;
  cudaStream_t s = ctx->stream;
  const int nc = L->nc, nh = L->nh;
  const int comp = L->target == IFEMGPU_LEARN_TARGET_COMPLEMENT ? 1 : 0;
  k_restrict2<<<(nc * 32 + kT - 1) / kT, kT, 0, s>>>(L->vPtr, L->vEq, L->vW, r, t, comp, L->rc,
                                                     L->rc1, nc, guard);
  inferTC(ctx, guard);
  const int ab = std::min(nparts, (nc + 7) / 8);
  k_coarse_alpha<<<ab, kT, 0, s>>>(L->Ac, L->yc, L->rc1, L->m, L->npv, nc, part, counter2,
                                   L->nrm + 2, guard);
  k_prolong_add<<<nparts, kT, 0, s>>>(L->eqCell, L->eqFrac, L->yc, L->nrm, L->m, L->npv,
                                      z, ctx->neq, q, part, counter, dotOut, pq, betaOut, guard);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  return IFEMGPU_OK;
}

ifemgpu_status learnTrain(ifemgpu_ctx* ctx, int epochs, int B, float lr, unsigned seed,
                          float* lossOut)
{
  LearnState* L = ctx->learn;
  if (!L || L->count < 1) return setError(ctx, IFEMGPU_NOT_READY, "no training pairs collected");
  if (epochs < 0 || B < 1 || !(lr > 0.f))
    return setError(ctx, IFEMGPU_INVALID_ARG, "learn_train: bad arguments");
  const int N = L->count, nc = L->nc;
  B = std::min(B, N);
  ifemgpu_status st = ensureBatch(ctx, L, B);
  if (st != IFEMGPU_OK) return st;
  cudaStream_t s = ctx->stream;
  // S = RMS of the targets
  k_sum_sq<<<kLossParts, kT, 0, s>>>(L->Y, (size_t)N * nc, L->loss);
  double ms = 0.0;
  if ((st = readLoss(ctx, L, (double)N * nc, &ms)) != IFEMGPU_OK) return st;
  L->scale = ms > 0 ? (float)std::sqrt(ms) : 1.f;
  IFEMGPU_CUDA(ctx, cudaMemcpy(L->nrm + 1, &L->scale, sizeof(float), cudaMemcpyHostToDevice));
  std::mt19937 rng(seed);
  std::vector<int> perm(N);
  double lastLoss = 0.0;
  const float b1 = 0.9f, b2 = 0.999f;
  for (int ep = 0; ep < epochs; ep++) {
    for (int i = 0; i < N; i++) perm[i] = i;
    std::shuffle(perm.begin(), perm.end(), rng);
    IFEMGPU_CUDA(ctx, cudaMemcpyAsync(L->perm, perm.data(), sizeof(int) * N, cudaMemcpyHostToDevice, s));
    for (int b0 = 0; b0 + B <= N; b0 += B) {
      k_gather_rows<<<256, kT, 0, s>>>(L->X, L->perm + b0, L->Xb, B, L->nin);
      k_gather_rows<<<256, kT, 0, s>>>(L->Y, L->perm + b0, L->Yb, B, nc);
      batchPass(s, L, B, 1.f / L->scale, true);
      L->adamStep++;
      const float c1 = 1.f - std::pow(b1, (float)L->adamStep);
      const float c2 = 1.f - std::pow(b2, (float)L->adamStep);
      k_adam<<<512, kT, 0, s>>>(L->theta, L->grad, L->am, L->av, L->nparam, lr, b1, b2, c1, c2, 1e-8f);
    }
    if (ep == epochs - 1) {  // loss of the epoch's last batch
      if ((st = readLoss(ctx, L, (double)B * nc, &lastLoss)) != IFEMGPU_OK) return st;
    }
    // the host permutation is rewritten next epoch: wait for its copy
    IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  }
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  packWeights(s, L);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(s));
  L->trained = true;
  if (lossOut) *lossOut = (float)lastLoss;
  return IFEMGPU_OK;
}

// mean squared error of the FP32 network on the collected pairs, targets in units of S
ifemgpu_status learnEvaluate(ifemgpu_ctx* ctx, float* mse)
{
  LearnState* L = ctx->learn;
  if (!L || L->count < 1) return setError(ctx, IFEMGPU_NOT_READY, "no pairs collected");
  const int N = L->count, nc = L->nc;
  const int B = std::min(N, 1024);
  ifemgpu_status st = ensureBatch(ctx, L, B);
  if (st != IFEMGPU_OK) return st;
  cudaStream_t s = ctx->stream;
  double total = 0.0;
  std::vector<int> idx(B);
  for (int b0 = 0; b0 < N; b0 += B) {
    const int nb = std::min(B, N - b0);
    for (int i = 0; i < nb; i++) idx[i] = b0 + i;
    IFEMGPU_CUDA(ctx, cudaMemcpyAsync(L->perm, idx.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, s));
    k_gather_rows<<<256, kT, 0, s>>>(L->X, L->perm, L->Xb, nb, L->nin);
    k_gather_rows<<<256, kT, 0, s>>>(L->Y, L->perm, L->Yb, nb, nc);
    batchPass(s, L, nb, 1.f / L->scale, false);
    double l = 0.0;
    if ((st = readLoss(ctx, L, 1.0, &l)) != IFEMGPU_OK) return st;  // also waits for idx
    total += l;
  }
  if (mse) *mse = (float)(total / ((double)N * nc));
  return IFEMGPU_OK;
}

// loss mean((Yp - Y)^2) and its gradient for host pairs (targets unscaled)
ifemgpu_status learnGradients(ifemgpu_ctx* ctx, const float* X, const float* Y, int n,
                              float* gradOut, float* lossOut)
{
  LearnState* L = ctx->learn;
  if (!L) return setError(ctx, IFEMGPU_NOT_READY, "learned correction not set up");
  if (n < 1 || !X || !Y) return setError(ctx, IFEMGPU_INVALID_ARG, "learn_gradients: bad arguments");
  ifemgpu_status st = ensureBatch(ctx, L, n);
  if (st != IFEMGPU_OK) return st;
  cudaStream_t s = ctx->stream;
  const int nc = L->nc;
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(L->Xb, X, sizeof(float) * (size_t)n * L->nin, cudaMemcpyHostToDevice, s));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(L->Yb, Y, sizeof(float) * (size_t)n * nc, cudaMemcpyHostToDevice, s));
  batchPass(s, L, n, 1.f, true);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  double l = 0.0;
  if ((st = readLoss(ctx, L, (double)n * nc, &l)) != IFEMGPU_OK) return st;
  if (gradOut)
    IFEMGPU_CUDA(ctx, cudaMemcpy(gradOut, L->grad, sizeof(float) * L->nparam, cudaMemcpyDeviceToHost));
  if (lossOut) *lossOut = (float)l;
  return IFEMGPU_OK;
}

ifemgpu_status learnWeights(ifemgpu_ctx* ctx, float* theta, int* count, float* scale, int set)
{
  LearnState* L = ctx->learn;
  if (!L) return setError(ctx, IFEMGPU_NOT_READY, "learned correction not set up");
  if (set && count && *count != L->nparam)
    return setError(ctx, IFEMGPU_INVALID_ARG, "learn_weights: parameter count mismatch");
  if (count) *count = L->nparam;
  if (!theta) return IFEMGPU_OK;
  if (set) {
    IFEMGPU_CUDA(ctx, cudaMemcpy(L->theta, theta, sizeof(float) * L->nparam, cudaMemcpyHostToDevice));
    if (scale) L->scale = *scale;
    IFEMGPU_CUDA(ctx, cudaMemcpy(L->nrm + 1, &L->scale, sizeof(float), cudaMemcpyHostToDevice));
    packWeights(ctx->stream, L);
    IFEMGPU_CUDA(ctx, cudaGetLastError());
    IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    L->trained = true;
  } else {
    IFEMGPU_CUDA(ctx, cudaMemcpy(theta, L->theta, sizeof(float) * L->nparam, cudaMemcpyDeviceToHost));
    if (scale) *scale = L->scale;
  }
  return IFEMGPU_OK;
}

int learnCount(const ifemgpu_ctx* ctx) { return ctx->learn ? ctx->learn->count : 0; }
int learnTarget(const ifemgpu_ctx* ctx)
{
  return ctx->learn ? ctx->learn->target : IFEMGPU_LEARN_TARGET_ERROR;
}
ifemgpu_status learnSetTarget(ifemgpu_ctx* ctx, int mode)
{
  if (!ctx->learn) return setError(ctx, IFEMGPU_NOT_READY, "learn_set_target before learn_setup");
  if (ctx->learn->target != mode) ctx->learn->count = 0;
  ctx->learn->target = mode;
  return IFEMGPU_OK;
}
bool learnReady(const ifemgpu_ctx* ctx) { return ctx->learn && ctx->learn->trained; }
void learnClear(ifemgpu_ctx* ctx)
{
  if (ctx->learn) ctx->learn->count = 0;
}

}  // namespace ifemgpu

extern "C" ifemgpu_status ifemgpu_learn_forward(ifemgpu_ctx* ctx, const float* rc, float* y)
{
  using namespace ifemgpu;
  if (!ctx || !rc || !y) return IFEMGPU_INVALID_ARG;
  if (!ctx->learn || !ctx->learn->trained)
    return setError(ctx, IFEMGPU_NOT_READY, "learn_forward without a trained network");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  IFEMGPU_TRY(learnPrepare(ctx));
  LearnState* L = ctx->learn;
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(L->rc, rc, sizeof(float) * L->nc, cudaMemcpyHostToDevice,
                                    ctx->stream));
  inferTC(ctx, nullptr);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(y, L->yc, sizeof(float) * L->nc, cudaMemcpyDeviceToHost,
                                    ctx->stream));
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return IFEMGPU_OK;
}

extern "C" ifemgpu_status ifemgpu_learn_coarse_matrix(ifemgpu_ctx* ctx, float* Ac)
{
  using namespace ifemgpu;
  if (!ctx || !Ac) return IFEMGPU_INVALID_ARG;
  if (!ctx->learn) return setError(ctx, IFEMGPU_NOT_READY, "learn_coarse_matrix before learn_setup");
  if (!ctx->assembled) return setError(ctx, IFEMGPU_NOT_READY, "learn_coarse_matrix before assemble");
  IFEMGPU_CUDA(ctx, cudaSetDevice(ctx->opts.device));
  IFEMGPU_TRY(verifyAssembly(ctx));
  IFEMGPU_TRY(learnGalerkin(ctx));
  LearnState* L = ctx->learn;
  const int nc = L->nc, npv = L->npv, m1 = L->m + 1, band = 125 * npv;
  std::vector<float> b((size_t)nc * band);
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  IFEMGPU_CUDA(ctx, cudaMemcpy(b.data(), L->Ac, sizeof(float) * b.size(), cudaMemcpyDeviceToHost));
  std::fill(Ac, Ac + (size_t)nc * nc, 0.f);
  for (int row = 0; row < nc; row++) {
    const int v = row / npv;
    const int vx = v % m1, vy = (v / m1) % m1, vz = v / (m1 * m1);
    for (int q = 0; q < band; q++) {
      const int o = q / npv, cp = q % npv;
      const int ux = vx + o % 5 - 2, uy = vy + (o / 5) % 5 - 2, uz = vz + o / 25 - 2;
      if (ux < 0 || ux >= m1 || uy < 0 || uy >= m1 || uz < 0 || uz >= m1) continue;
      Ac[(size_t)row * nc + ((uz * m1 + uy) * m1 + ux) * npv + cp] = b[(size_t)row * band + q];
    }
  }
  return IFEMGPU_OK;
}

extern "C" ifemgpu_status ifemgpu_learn_info(const ifemgpu_ctx* ctx, int* coarse_unknowns,
                                             int* inputs, int* hidden, int* nparam, int* pairs)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  const ifemgpu::LearnState* L = ctx->learn;
  if (!L) return IFEMGPU_NOT_READY;
  if (coarse_unknowns) *coarse_unknowns = L->nc;
  if (inputs) *inputs = L->nin;
  if (hidden) *hidden = L->nh;
  if (nparam) *nparam = L->nparam;
  if (pairs) *pairs = L->count;
  return IFEMGPU_OK;
}

extern "C" ifemgpu_status ifemgpu_learn_get_pairs(ifemgpu_ctx* ctx, int first, int count,
                                                  float* X, float* Y)
{
  if (!ctx) return IFEMGPU_INVALID_ARG;
  const ifemgpu::LearnState* L = ctx->learn;
  if (!L) return ifemgpu::setError(ctx, IFEMGPU_NOT_READY, "learned correction not set up");
  if (first < 0 || count < 0 || first + count > L->count || !X || !Y)
    return ifemgpu::setError(ctx, IFEMGPU_INVALID_ARG, "learn_get_pairs: bad range or arrays");
  IFEMGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  IFEMGPU_CUDA(ctx, cudaMemcpy(X, L->X + (size_t)first * L->nin, sizeof(float) * (size_t)count * L->nin,
                               cudaMemcpyDeviceToHost));
  IFEMGPU_CUDA(ctx, cudaMemcpy(Y, L->Y + (size_t)first * L->nc, sizeof(float) * (size_t)count * L->nc,
                               cudaMemcpyDeviceToHost));
  return IFEMGPU_OK;
}
