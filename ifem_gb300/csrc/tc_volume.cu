// tc_volume.cu -- tensor-core (tcgen05, sm_103a) element kernel for 3D
// isotropic linear elasticity with quadratic (p=2) spline patches and 3x3x3
// Gauss points: the hot loop of ASMs3D::integrate (src/ASM/ASMs3D.C:2266-2312)
// with the linear-elasticity integrand, and the scatter of assemSparse
// (src/LinAlg/SparseMatrix.C:614-688).
//
// Per element (one CTA of 128 threads processes the elements of a colour):
//   1. rational basis and Jacobian at the 27 Gauss points (FP32 sums of the
//      homogeneous control net; determinant and inverse in FP64);
//   2. Gram matrix G = A^T B on the tensor cores, A[(a,k),q] = w_q dN_a/dx_k,
//      B[(b,l),q] = dN_b/dx_l (rows m = 32k + a), in 3xTF32 split precision:
//      G = Ahi Bhi + Ahi Blo + Alo Bhi, FP32 accumulation in tensor memory;
//   3. Ke[(a,k),(b,l)] = lambda G[(a,k),(b,l)] + mu G[(a,l),(b,k)]
//                        + mu delta_kl sum_m G[(a,m),(b,m)]
//      -- the B^T D B product of isotropic elasticity regrouped so that the
//      tensor cores contract over Gauss points once;
//   4. FP64 reductions of Ke into the compressed-column matrix in L2
//      (red.global.add.f64).  Elements of one colour share no node, so no
//      address is reduced twice within a launch and the sum order is fixed.
#include <algorithm>
#include <cstdio>

#include "ifemgpu_internal.h"
#include "tc_common.cuh"

namespace ifemgpu {

using namespace tc;

namespace {

constexpr int kNen = 27;      // p = 2: 3x3x3 functions
constexpr int kNq = 27;       // 3x3x3 Gauss points
constexpr int kM = 128;       // MMA M (rows 32k + a, k < 3, a < 27)
constexpr int kN = 96;        // MMA N (columns 32l + b)
constexpr int kGld = 97;      // row stride of the staged Gram matrix (floats)

struct TcSmem {
  // operand tiles (K-major core-matrix layout); the staged Gram matrix
  // G[96][97] aliases the first 37 KB once the MMAs have completed
  float Ahi[kM * kK];
  float Alo[kM * kK];
  float Bhi[kN * kK];
  float Blo[kN * kK];
  float N[kNq][kNen];      // weighted basis wN, later the rational basis R
  float Du[kNq][kNen];     // weighted parametric derivatives w dN/du_d
  float Dv[kNq][kNen];
  float Dw[kNq][kNen];
  float P[kNq][4][4];      // homogeneous sums: [q][x,y,z,w][value, d/du, d/dv, d/dw]
  float Jinv[kNq][9];      // column-major inverse Jacobian
  float Wq[kNq][4];        // W and dW/du_d
  float wq[kNq];           // detJ * dV * Gauss weights (0 at skipped points)
  float X[kNen][4];        // control points relative to the element's first, weight
  int eq[kNen * 3];
  int colStart[kNen * 3];  // colptr of the element's free columns
  int Fa[kNen];            // F(a): free DOFs before node a
  int lo[kNen][9];         // line offset of row node line (j + 3k) in column node b
  unsigned long long mbar;
  uint32_t tmemSlot;
  int fail;
};

__device__ inline int findRowTc(const int* __restrict__ colptr, const int* __restrict__ rowidx,
                                int c, int r)
{
  int lo = colptr[c], hi = colptr[c + 1] - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    const int v = rowidx[mid];
    if (v == r) return mid;
    if (v < r) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

__device__ __forceinline__ void redAdd(double* p, double v)
{
  atomicAdd(p, v);  // result unused: compiles to an L2 reduction
}

}  // namespace

struct TcSys {
  const int* madof;
  const int* meqn;
  const int* F;
  const double* c0;
  const int* colptr;
  const int* rowidx;
  double* K;
  double* b;
  unsigned long long* counters;  // [0] singular points, [1] pattern misses, [2] device timeouts
};

__global__ void __launch_bounds__(128)
k_volume_tc_elast_p2(const DevPatch* __restrict__ patches, const Item* __restrict__ items,
                     int count, TcSys S)
{
  extern __shared__ __align__(1024) unsigned char smraw[];
  TcSmem& sm = *reinterpret_cast<TcSmem*>(smraw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t mbar = smemAddr(&sm.mbar);
  if (tid == 0) {
    mbarInit(mbar, 1);
    sm.fail = 0;
  }
  if (warp == 0) tmemAlloc(&sm.tmemSlot, 128);
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = sm.tmemSlot;
  constexpr uint32_t idesc = instrDescTF32(kM, kN);
  const uint32_t aHi = smemAddr(sm.Ahi), aLo = smemAddr(sm.Alo);
  const uint32_t bHi = smemAddr(sm.Bhi), bLo = smemAddr(sm.Blo);
  float* G = sm.Ahi;  // staged Gram matrix, [96][kGld]
  uint32_t phase = 0;

  for (int it = blockIdx.x; it < count; it += gridDim.x) {
    const Item item = items[it];
    const DevPatch& P = patches[item.patch];
    const int e = item.elem;
    const int e1 = e % P.nel[0], e2 = (e / P.nel[0]) % P.nel[1], e3 = e / (P.nel[0] * P.nel[1]);
    const int n0 = (e3 * P.n[1] + e2) * P.n[0] + e1;

    // ---- 1. element nodes ------------------------------------------------
    if (tid < kNen) {
      const int a = tid;
      const int node = n0 + ((a / 9) * P.n[1] + (a / 3) % 3) * P.n[0] + a % 3;
      const double* c = P.ctrl + (size_t)node * 4;
      const double* c00 = P.ctrl + (size_t)n0 * 4;
      sm.X[a][0] = (float)(c[0] - c00[0]);
      sm.X[a][1] = (float)(c[1] - c00[1]);
      sm.X[a][2] = (float)(c[2] - c00[2]);
      sm.X[a][3] = (float)c[3];
      const int d0 = S.madof[P.firstNode + node] - 1;
      sm.eq[3 * a] = S.meqn[d0];
      sm.eq[3 * a + 1] = S.meqn[d0 + 1];
      sm.eq[3 * a + 2] = S.meqn[d0 + 2];
      sm.Fa[a] = S.F[P.firstNode + node];
    }
    if (P.lineOff) {
      // line offsets of the 9 row lines of the element in each column node
      for (int idx = tid; idx < kNen * 9; idx += blockDim.x) {
        const int bn = idx / 9, la = idx % 9;
        const int nodeb = n0 + ((bn / 9) * P.n[1] + (bn / 3) % 3) * P.n[0] + bn % 3;
        const int dy = la % 3 - (bn / 3) % 3, dz = la / 3 - bn / 9;
        sm.lo[bn][la] = P.lineOff[(size_t)nodeb * 25 + (dz + 2) * 5 + dy + 2];
      }
    }
    // zero padding of the operand tiles (rows a >= 27 per component block,
    // rows >= 96 of A, columns q >= 27)
    for (int idx = tid; idx < kM * kK; idx += blockDim.x) {
      const int r = idx >> 5, k = idx & 31;
      if ((r & 31) >= kNen || r >= 96 || k >= kNq) {
        const int o = kmaj(r, k);
        sm.Ahi[o] = 0.f;
        sm.Alo[o] = 0.f;
        if (r < kN) {
          sm.Bhi[o] = 0.f;
          sm.Blo[o] = 0.f;
        }
      }
    }
    __syncthreads();

    if (tid < kNen * 3) sm.colStart[tid] = sm.eq[tid] > 0 ? S.colptr[sm.eq[tid] - 1] : 0;

    // ---- 2. weighted tensor-product basis at every (Gauss point, function)
    for (int idx = tid; idx < kNq * kNen; idx += blockDim.x) {
      const int q = idx / kNen, a = idx % kNen;
      const int gi = q % 3, gj = (q / 3) % 3, gk = q / 9;
      const int i = a % 3, j = (a / 3) % 3, k = a / 9;
      const double* t0 = P.tabN[0] + (e1 * 3 + gi) * 3;
      const double* t1 = P.tabN[1] + (e2 * 3 + gj) * 3;
      const double* t2 = P.tabN[2] + (e3 * 3 + gk) * 3;
      const double* d0 = P.tabD[0] + (e1 * 3 + gi) * 3;
      const double* d1 = P.tabD[1] + (e2 * 3 + gj) * 3;
      const double* d2 = P.tabD[2] + (e3 * 3 + gk) * 3;
      const float nx = (float)t0[i], ny = (float)t1[j], nz = (float)t2[k];
      const float w = sm.X[a][3];
      sm.N[q][a] = w * nx * ny * nz;
      sm.Du[q][a] = w * (float)d0[i] * ny * nz;
      sm.Dv[q][a] = w * nx * (float)d1[j] * nz;
      sm.Dw[q][a] = w * nx * ny * (float)d2[k];
    }
    __syncthreads();

    // ---- 3. homogeneous sums per Gauss point: sum_a (wN)_a (X_a, 1) and derivatives
    if (tid < kNq * 4) {
      const int q = tid >> 2, c = tid & 3;
      float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll 9
      for (int a = 0; a < kNen; a++) {
        const float x = c < 3 ? sm.X[a][c] : 1.f;
        s0 = fmaf(sm.N[q][a], x, s0);
        s1 = fmaf(sm.Du[q][a], x, s1);
        s2 = fmaf(sm.Dv[q][a], x, s2);
        s3 = fmaf(sm.Dw[q][a], x, s3);
      }
      sm.P[q][c][0] = s0;
      sm.P[q][c][1] = s1;
      sm.P[q][c][2] = s2;
      sm.P[q][c][3] = s3;
    }
    __syncthreads();

    // ---- 4. Jacobian, FP64 determinant and inverse, integration weight
    if (tid < kNq) {
      const int q = tid;
      const float W = sm.P[q][3][0];
      const float iW = 1.f / W;
      double J[9];  // column-major: J[d*3 + r] = dX_r/du_d
      for (int r = 0; r < 3; r++) {
        const float Xr = sm.P[q][r][0] * iW;
        for (int d = 0; d < 3; d++)
          J[d * 3 + r] = (double)((sm.P[q][r][1 + d] - Xr * sm.P[q][3][1 + d]) * iW);
      }
      const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[3] * (J[1] * J[8] - J[2] * J[7]) +
                         J[6] * (J[1] * J[5] - J[2] * J[4]);
      float w = 0.f;
      float B[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (det > kEpsZ || det < -kEpsZ) {
        const double id = 1.0 / det;
        B[0] = (float)((J[4] * J[8] - J[5] * J[7]) * id);
        B[1] = (float)(-(J[1] * J[8] - J[2] * J[7]) * id);
        B[2] = (float)((J[1] * J[5] - J[2] * J[4]) * id);
        B[3] = (float)(-(J[3] * J[8] - J[5] * J[6]) * id);
        B[4] = (float)((J[0] * J[8] - J[2] * J[6]) * id);
        B[5] = (float)(-(J[0] * J[5] - J[2] * J[3]) * id);
        B[6] = (float)((J[3] * J[7] - J[4] * J[6]) * id);
        B[7] = (float)(-(J[0] * J[7] - J[1] * J[6]) * id);
        B[8] = (float)((J[0] * J[4] - J[1] * J[3]) * id);
        const double dV = 0.125 * P.span[0][e1] * P.span[1][e2] * P.span[2][e3];
        w = (float)(det * dV * P.gw[0][q % 3] * P.gw[1][(q / 3) % 3] * P.gw[2][q / 9]);
      } else {
        atomicAdd(S.counters, 1ull);
      }
      sm.wq[q] = w;
      for (int c = 0; c < 9; c++) sm.Jinv[q][c] = B[c];
      sm.Wq[q][0] = iW;
      sm.Wq[q][1] = sm.P[q][3][1];
      sm.Wq[q][2] = sm.P[q][3][2];
      sm.Wq[q][3] = sm.P[q][3][3];
    }
    __syncthreads();

    // ---- 5. dN/dX into the split-TF32 operand tiles
    for (int idx = tid; idx < kNq * kNen; idx += blockDim.x) {
      const int q = idx / kNen, a = idx % kNen;
      const float iW = sm.Wq[q][0];
      const float R = sm.N[q][a] * iW;
      const float ru = (sm.Du[q][a] - R * sm.Wq[q][1]) * iW;
      const float rv = (sm.Dv[q][a] - R * sm.Wq[q][2]) * iW;
      const float rw = (sm.Dw[q][a] - R * sm.Wq[q][3]) * iW;
      const float* B = sm.Jinv[q];
      const float w = sm.wq[q];
      const float g[3] = {ru * B[0] + rv * B[1] + rw * B[2], ru * B[3] + rv * B[4] + rw * B[5],
                          ru * B[6] + rv * B[7] + rw * B[8]};
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const int o = kmaj(32 * c + a, q);
        float hi, lo;
        splitTF32(g[c], hi, lo);
        sm.Bhi[o] = hi;
        sm.Blo[o] = lo;
        splitTF32(w * g[c], hi, lo);
        sm.Ahi[o] = hi;
        sm.Alo[o] = lo;
      }
      sm.N[q][a] = R;
    }
    fenceProxyAsync();
    __syncthreads();

    // ---- 6. tensor cores: G = Ahi Bhi + Ahi Blo + Alo Bhi over 4 K-steps
    if (tid == 0) {
      tcFenceAfter();
      for (int s = 0; s < kK / 8; s++) {
        const uint32_t off = s * 256;
        mmaTF32(tmem, smemDesc(aHi + off), smemDesc(bHi + off), idesc, s > 0);
        mmaTF32(tmem, smemDesc(aHi + off), smemDesc(bLo + off), idesc, 1);
        mmaTF32(tmem, smemDesc(aLo + off), smemDesc(bHi + off), idesc, 1);
      }
      mmaCommit(mbar);
    }

    // element load vector (body force), overlapping the MMAs
    float fe = 0.f;
    if (tid < kNen * 3) {
      const int a = tid / 3, k = tid % 3;
      const double bk = P.body[k];
      if (bk != 0.0) {
        float s = 0.f;
        for (int q = 0; q < kNq; q++) s = fmaf(sm.N[q][a], sm.wq[q], s);
        fe = (float)bk * s;
      }
    }

    // ---- 7. wait for the MMAs (bounded), stage G in shared memory
    const bool ok = mbarWait(mbar, phase);
    phase ^= 1u;
    if (!ok) {
      if (tid == 0) {
        atomicAdd(S.counters + 2, 1ull);
        sm.fail = 1;
      }
    }
    tcFenceAfter();
    if (ok && warp < 3) {
      float v[16];
      for (int c16 = 0; c16 < kN / 16; c16++) {
        tmemLoad16(tmem + ((uint32_t)(32 * warp) << 16) + 16 * c16, v);
#pragma unroll
        for (int i = 0; i < 16; i++) G[(32 * warp + lane) * kGld + 16 * c16 + i] = v[i];
      }
    }
    tcFenceBefore();
    __syncthreads();
    if (sm.fail) break;

    // ---- 8. element matrix and scatter, node pair by node pair (FP32
    //         arithmetic; the FP64 additions happen in the L2 reductions)
    const double lam = P.E * P.nu / ((1.0 + P.nu) * (1.0 - 2.0 * P.nu));
    const double mu = P.E / (2.0 * (1.0 + P.nu));
    const float lamf = (float)lam, muf = (float)mu;
    for (int pr = tid; pr < kNen * kNen; pr += blockDim.x) {
      const int a = pr % kNen, bn = pr / kNen;
      int firstCol = -1, firstRow = -1;
      for (int l = 0; l < 3 && firstCol < 0; l++)
        if (sm.eq[3 * bn + l] > 0) firstCol = sm.eq[3 * bn + l] - 1;
      for (int k = 0; k < 3 && firstRow < 0; k++)
        if (sm.eq[3 * a + k] > 0) firstRow = sm.eq[3 * a + k] - 1;
      if (firstCol < 0 || firstRow < 0) continue;
      float g[3][3];
#pragma unroll
      for (int k = 0; k < 3; k++)
#pragma unroll
        for (int l = 0; l < 3; l++) g[k][l] = G[(32 * k + a) * kGld + 32 * l + bn];
      const float trm = muf * (g[0][0] + g[1][1] + g[2][2]);
      int off;
      if (P.lineOff) {
        off = sm.lo[bn][(a / 3) % 3 + 3 * (a / 9)] + sm.Fa[a];
      } else {
        const int pos0 = findRowTc(S.colptr, S.rowidx, firstCol, firstRow);
        if (pos0 < 0) {
          atomicAdd(S.counters + 1, 1ull);
          continue;
        }
        off = pos0 - S.colptr[firstCol];
      }
      for (int l = 0; l < 3; l++) {
        const int ce = sm.eq[3 * bn + l];
        if (ce <= 0) continue;
        double* col = S.K + sm.colStart[3 * bn + l] + off;
        int rank = 0;
        for (int k = 0; k < 3; k++) {
          if (sm.eq[3 * a + k] <= 0) continue;
          const float ke = fmaf(lamf, g[k][l], fmaf(muf, g[l][k], k == l ? trm : 0.f));
          redAdd(col + rank, widenF32(ke));
          rank++;
        }
      }
    }

    // ---- 9. right-hand side: load vector minus prescribed-DOF terms
    if (tid < kNen * 3) {
      const int a = tid / 3, k = tid % 3;
      const int r = sm.eq[tid];
      if (r > 0) {
        double acc = widenF32(fe);
        if (S.c0) {
          for (int j = 0; j < kNen * 3; j++) {
            const int ce = sm.eq[j];
            if (ce >= 0) continue;
            const int bn = j / 3, l = j % 3;
            double tr = 0.0;
            for (int m = 0; m < 3; m++) tr += G[(32 * m + a) * kGld + 32 * m + bn];
            const double ke = lam * G[(32 * k + a) * kGld + 32 * l + bn] +
                              mu * G[(32 * l + a) * kGld + 32 * k + bn] + (k == l ? mu * tr : 0.0);
            acc -= S.c0[-ce - 1] * ke;
          }
        }
        if (acc != 0.0) redAdd(S.b + r - 1, acc);
      }
    }
    __syncthreads();
  }

  // after a timed-out wait, give the MMAs in flight one more bounded wait
  if (sm.fail) mbarWait(mbar, phase ^ 1u);
  // release tensor memory (all tcgen05 traffic of this CTA has completed)
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (warp == 0) tmemDealloc(tmem, 128);
}

// ---------------------------------------------------------------------------
// Self-test of the MMA building blocks: D (128x96) = A (128x32) B^T (96x32)^T
// with the same operand layout, descriptors and 3xTF32 split as the kernel.
__global__ void __launch_bounds__(128)
k_selftest_gemm(const float* __restrict__ A, const float* __restrict__ B, float* __restrict__ D,
                unsigned long long* status)
{
  extern __shared__ __align__(1024) unsigned char smraw[];
  float* Ahi = reinterpret_cast<float*>(smraw);
  float* Alo = Ahi + kM * kK;
  float* Bhi = Alo + kM * kK;
  float* Blo = Bhi + kN * kK;
  unsigned long long* mb = reinterpret_cast<unsigned long long*>(Blo + kN * kK);
  uint32_t* slot = reinterpret_cast<uint32_t*>(mb + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t mbar = smemAddr(mb);
  if (tid == 0) mbarInit(mbar, 1);
  if (warp == 0) tmemAlloc(slot, 128);
  for (int idx = tid; idx < kM * kK; idx += blockDim.x) {
    float hi, lo;
    splitTF32(A[idx], hi, lo);
    Ahi[kmaj(idx >> 5, idx & 31)] = hi;
    Alo[kmaj(idx >> 5, idx & 31)] = lo;
    if (idx < kN * kK) {
      splitTF32(B[idx], hi, lo);
      Bhi[kmaj(idx >> 5, idx & 31)] = hi;
      Blo[kmaj(idx >> 5, idx & 31)] = lo;
    }
  }
  fenceProxyAsync();
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = *slot;
  constexpr uint32_t idesc = instrDescTF32(kM, kN);
  if (tid == 0) {
    for (int s = 0; s < kK / 8; s++) {
      const uint32_t off = s * 256;
      mmaTF32(tmem, smemDesc(smemAddr(Ahi) + off), smemDesc(smemAddr(Bhi) + off), idesc, s > 0);
      mmaTF32(tmem, smemDesc(smemAddr(Ahi) + off), smemDesc(smemAddr(Blo) + off), idesc, 1);
      mmaTF32(tmem, smemDesc(smemAddr(Alo) + off), smemDesc(smemAddr(Bhi) + off), idesc, 1);
    }
    mmaCommit(mbar);
  }
  const bool ok = mbarWait(mbar, 0);
  if (!ok && tid == 0) atomicAdd(status, 1ull);
  tcFenceAfter();
  if (ok) {
    float v[16];
    for (int c16 = 0; c16 < kN / 16; c16++) {
      tmemLoad16(tmem + ((uint32_t)(32 * warp) << 16) + 16 * c16, v);
      for (int i = 0; i < 16; i++) D[(32 * warp + lane) * kN + 16 * c16 + i] = v[i];
    }
  }
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (warp == 0) tmemDealloc(tmem, 128);
}

size_t tcVolumeSmem() { return sizeof(TcSmem) + 1024; }

bool tcSupports(const DevPatch& P)
{
  return P.dim == 3 && P.kind == IFEMGPU_ELASTICITY && P.p[0] == 2 && P.p[1] == 2 && P.p[2] == 2 &&
         P.ng[0] == 3 && P.ng[1] == 3 && P.ng[2] == 3 && P.npv == 3;
}

ifemgpu_status tcPrepare(ifemgpu_ctx* ctx)
{
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_volume_tc_elast_p2,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tcVolumeSmem()));
  return IFEMGPU_OK;
}

ifemgpu_status tcLaunchVolume(ifemgpu_ctx* ctx, const Pass& p, int grid)
{
  TcSys S{ctx->d_madof, ctx->d_meqn, ctx->d_freeBefore, ctx->nceq ? ctx->d_c0 : nullptr,
          ctx->d_colptr, ctx->d_rowidx, ctx->d_K, ctx->d_b, ctx->d_counters};
  // dynamic shared memory is 1024-aligned by the __align__ of the buffer
  k_volume_tc_elast_p2<<<grid, 128, tcVolumeSmem(), ctx->stream>>>(ctx->d_patches,
                                                                   ctx->d_items + p.first,
                                                                   p.count, S);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  return IFEMGPU_OK;
}

}  // namespace ifemgpu

extern "C" ifemgpu_status ifemgpu_selftest_tc_gemm(const float* A, const float* B, float* D)
{
  using namespace ifemgpu;
  if (!A || !B || !D) return IFEMGPU_INVALID_ARG;
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  unsigned long long* dS = nullptr;
  const size_t smem = sizeof(float) * (2 * kM * kK + 2 * kN * kK) + 64;
  ifemgpu_status st = IFEMGPU_OK;
  if (cudaMalloc(&dA, sizeof(float) * kM * kK) != cudaSuccess ||
      cudaMalloc(&dB, sizeof(float) * kN * kK) != cudaSuccess ||
      cudaMalloc(&dD, sizeof(float) * kM * kN) != cudaSuccess ||
      cudaMalloc(&dS, sizeof(unsigned long long)) != cudaSuccess) {
    st = IFEMGPU_OUT_OF_MEMORY;
  } else {
    cudaMemcpy(dA, A, sizeof(float) * kM * kK, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B, sizeof(float) * kN * kK, cudaMemcpyHostToDevice);
    cudaMemset(dS, 0, sizeof(unsigned long long));
    cudaFuncSetAttribute(k_selftest_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_selftest_gemm<<<1, 128, smem>>>(dA, dB, dD, dS);
    unsigned long long s = 0;
    if (cudaDeviceSynchronize() != cudaSuccess) st = IFEMGPU_CUDA_ERROR;
    else {
      cudaMemcpy(D, dD, sizeof(float) * kM * kN, cudaMemcpyDeviceToHost);
      cudaMemcpy(&s, dS, sizeof(s), cudaMemcpyDeviceToHost);
      if (s) st = IFEMGPU_DEVICE_TIMEOUT;
    }
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(dS);
  return st;
}
