// tc_volume.cu -- tensor-core (tcgen05, sm_103a) element kernel for 3D
// isotropic linear elasticity with quadratic (p=2) spline patches and 3x3x3
// Gauss points: the hot loop of ASMs3D::integrate (src/ASM/ASMs3D.C:2266-2312)
// with the linear-elasticity integrand.  Its element matrices go to the
// element scratch, which the node-wise gather (gather.cu) sums into the
// compressed-column matrix (the scatter of assemSparse,
// src/LinAlg/SparseMatrix.C:614-688).
//
// One persistent launch processes every element of the eligible patches.
// Per element (one CTA of 128 threads; elements in index order, no element
// waits for another):
//   0. the element's 3x3x3 control points staged in shared memory by TMA,
//      the next element's requested as soon as the current one has read its
//      own;
//   1. rational basis and Jacobian at the 27 Gauss points (FP32 sums of the
//      homogeneous control net; determinant and inverse in FP64);
//   2. operand tile T[(a,k), q] = sqrt|w_q| dN_a/dx_k (rows m = 32k + a), so
//      that the Gram matrix G = sum_q w_q dN dN^T = s T^T T with the sign s of
//      the weights.  Elements whose weights change sign (folded geometry) run
//      one pass per sign, the negative one with the negate-A bit of the MMA;
//   3. G on the tensor cores in 3xTF32 split precision,
//      G = Thi^T Thi + Thi^T Tlo + Tlo^T Thi, FP32 accumulation in tensor memory;
//   4. G made exactly symmetric in shared memory (the upper triangle mirrored)
//      and written, with the element load vector (body force, Neumann
//      traction), as the element's scratch block G[a][k][l][b], F[a][k]; the
//      gather forms Ke[(a,k),(b,l)] = lambda G_kl + mu G_lk + delta_kl mu tr G
//      -- B^T D B of isotropic elasticity regrouped so the tensor cores
//      contract over the Gauss points once.
#include <algorithm>
#include <cstdio>
#include <vector>

#include <cuda.h>  // CUtensorMap and its encoder's types (entry point fetched at run time)

#include "ifemgpu_internal.h"
#include "tc_common.cuh"

namespace ifemgpu {

using namespace tc;

namespace {

constexpr int kNen = 27;      // p = 2: 3x3x3 functions
constexpr int kNq = 27;       // 3x3x3 Gauss points
constexpr int kM = 128;       // MMA M (rows 32k + a, k < 3, a < 27)
constexpr int kN = 96;        // MMA N (columns 32l + b)
constexpr int kGs = 81;       // row stride of the Gram matrix in the element block
constexpr int kBlock = 81 * 81 + 81 + 2;  // element block: G, F, padding to 16 bytes
constexpr int kTcPerSM = 4;   // CTAs per SM at most: 4 x 128 tensor-memory columns

// The operand tile has 96 rows (32k + a for k < 3, a < 27, the rest zero);
// the MMA's A operand reads M = 128 rows from the tile start, so the reads of
// rows 96..127 run into the next 4 KB (Tlo after Thi, the union after Tlo).
// Those rows only feed accumulator lanes 96..127, which are never read, and
// nothing writes shared memory while an MMA runs.
constexpr int kRowsT = 96;

// per-element front-end arrays (dead before the element block is formed)
struct Front {
  float wX[4][kNen];          // weighted control net: w x, w y, w z, w (x relative)
  float A[2][4][3][9];        // x contracted: [N/D][field][gx][j + 3k]
  float B[3][4][9][3];        // y contracted: [NN/DN/ND][field][gx + 3gy][k]
  float S[kNq][4][4];         // [q][field][value, d/du, d/dv, d/dw]: homogeneous sums
  float E[kNq][12];           // du_d/dx_k / W at [k 3 + d], then e_k = sum_d dW_d/W E_kd
  float Es[kNq][12];          // E scaled by sqrt(max(s w_q, 0)) for the current sign pass
  float iW[kNq];              // 1 / W
  float face[9 * 27 + 9];     // Neumann face points: rational basis, dS weights
};

struct TcSmem {
  float Thi[kRowsT * kK];  // operand tile, K-major core-matrix layout
  float Tlo[kRowsT * kK];
  union {
    Front f;
    // the element's scratch block, written once the front-end data is dead:
    // G[a][k][l][b] at (3a + k) 81 + 27 l + b, then F[a][k], 2 floats padding
    float Gc[kBlock];
  } u;
  float tb[3][2][9];       // 1D tables of the element: [direction][N, dN/du][g 3 + i]
  float wq[kNq];           // signed integration weight (0 at skipped points)
  float X[kNen][4];        // control points relative to the element's first, weight
  // the element's node box, written by TMA (node a = i + 3 j + 9 k)
  alignas(128) double ctrlT[kNen][4];  // control points x, y, z, w
  unsigned long long mbar;
  unsigned long long ctrlbar;  // TMA completion of ctrlT
  uint32_t tmemSlot;
  int fail;
  int signs;               // bit 0: some w_q > 0, bit 1: some w_q < 0
  float dVf;               // span volume / 8 of the element
};

constexpr uint32_t kCtrlBytes = sizeof(double) * kNen * 4;
static_assert(sizeof(TcSmem) <= 56320, "4 CTAs per SM: 4 x (56 KB + 1 KB reserved) shared memory");
static_assert(offsetof(TcSmem, u) % 16 == 0 && (kBlock * sizeof(float)) % 16 == 0,
              "element blocks are copied in 16-byte pieces");
static_assert(offsetof(TcSmem, Tlo) == offsetof(TcSmem, Thi) + sizeof(float) * kRowsT * kK &&
                  offsetof(TcSmem, u) == offsetof(TcSmem, Tlo) + sizeof(float) * kRowsT * kK &&
                  sizeof(TcSmem::u) >= sizeof(float) * (kM - kRowsT) * kK,
              "A-operand reads of rows 96..127 must stay inside the tile and the union");

}  // namespace

struct TcSys {
  unsigned long long* counters;  // [0] singular points, [2] device timeouts
  unsigned mbarSpin;             // polls per wait for a copy
  int wPatch, wElem;             // element whose copy is never issued (test hook), -1 none
};

__global__ void __launch_bounds__(128)
k_volume_tc_elast_p2(const DevPatch* __restrict__ patches, const Item* __restrict__ items,
                     int count, TcSys S)
{
  extern __shared__ __align__(1024) unsigned char smraw[];
  TcSmem& sm = *reinterpret_cast<TcSmem*>(smraw);
  Front& F = sm.u.f;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t mbar = smemAddr(&sm.mbar);
  const uint32_t ctrlbar = smemAddr(&sm.ctrlbar);
  if (tid == 0) {
    mbarInit(mbar, 1);
    mbarInit(ctrlbar, 1);
    sm.fail = 0;
  }
  // the padding of the operand tile (rows with a >= 27, q >= 27) is written
  // with zeros only
  for (int i = tid; i < kRowsT * kK; i += blockDim.x) {
    sm.Thi[i] = 0.f;
    sm.Tlo[i] = 0.f;
  }
  if (warp == 0) tmemAlloc(&sm.tmemSlot, 128);
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = sm.tmemSlot;
  const uint32_t tHi = smemAddr(sm.Thi), tLo = smemAddr(sm.Tlo);
  uint32_t phase = 0;
  // thread 0: control points of item itn into the TMA buffer, requested as
  // soon as the current element has read its own (step 1) and waited for
  // only where they are first read
  int mapPatch = -1;        // patch whose tensor map was last acquired
  bool ctrlOut = false;     // copy in flight (thread 0)
  auto stageCtrl = [&](int itn) {
    const Item nx = items[itn];
    const DevPatch& Pn = patches[nx.patch];
    const int f1 = nx.elem % Pn.nel[0];
    const int f2 = (nx.elem / Pn.nel[0]) % Pn.nel[1];
    const int f3 = nx.elem / (Pn.nel[0] * Pn.nel[1]);
    const char* tm = static_cast<const char*>(Pn.tmaps);
    if (nx.patch == S.wPatch && nx.elem == S.wElem) return;  // withheld: the wait runs out
    if (nx.patch != mapPatch) {
      tmapAcquire(tm);
      mapPatch = nx.patch;
    }
    mbarExpectTx(ctrlbar, kCtrlBytes);
    tmaLoad4d(smemAddr(sm.ctrlT), tm, 0, f1, f2, f3, ctrlbar);
    ctrlOut = true;
  };
  if (tid == 0 && (int)blockIdx.x < count) stageCtrl(blockIdx.x);
  uint32_t cphase = 0;

  // the next element's item is read during the current element's store
  Item nextItem{};
  if ((int)blockIdx.x < count) nextItem = items[blockIdx.x];
  for (int it = blockIdx.x; it < count; it += gridDim.x) {
    const Item item = nextItem;
    const DevPatch& P = patches[item.patch];
    const int e = item.elem;
    const int e1 = e % P.nel[0], e2 = (e / P.nel[0]) % P.nel[1], e3 = e / (P.nel[0] * P.nel[1]);

    // ---- 1. element nodes from the TMA box: coordinates relative to the
    //         first node, weights, the weighted net; the 1D table rows and
    //         the span volume are read from L2 while the control points arrive
    double dV = 0.0;
    if (tid == 96) dV = P.span[0][e1] * P.span[1][e2] * P.span[2][e3];
    float tbv = 0.f;
    if (tid < 54) {
      const int d = tid / 18, dd = (tid / 9) & 1, g = tid % 9;
      tbv = (dd ? P.tabDf[d] : P.tabNf[d])[(d == 0 ? e1 : d == 1 ? e2 : e3) * 9 + g];
    }
    if (mbarWait(ctrlbar, cphase, S.mbarSpin)) {
      cphase ^= 1u;
      ctrlOut = false;
    } else {
      atomicAdd(S.counters + 2, 1ull);
      sm.fail = 1;
    }
    if (tid < kNen) {
      const int a = tid;
      const float x0 = (float)(sm.ctrlT[a][0] - sm.ctrlT[0][0]);
      const float x1 = (float)(sm.ctrlT[a][1] - sm.ctrlT[0][1]);
      const float x2 = (float)(sm.ctrlT[a][2] - sm.ctrlT[0][2]);
      const float w = (float)sm.ctrlT[a][3];
      sm.X[a][0] = x0;
      sm.X[a][1] = x1;
      sm.X[a][2] = x2;
      sm.X[a][3] = w;
      F.wX[0][a] = w * x0;
      F.wX[1][a] = w * x1;
      F.wX[2][a] = w * x2;
      F.wX[3][a] = w;
    }
    if (tid < 54) sm.tb[tid / 18][(tid / 9) & 1][tid % 9] = tbv;
    if (tid == 96) {
      sm.signs = 0;
      sm.dVf = (float)(0.125 * dV);
    }
    __syncthreads();  // ctrlT read, node data and tables visible
    if (sm.fail) break;
    if (tid == 0 && it + (int)gridDim.x < count) stageCtrl(it + gridDim.x);

    // ---- 2. homogeneous sums at the Gauss points by sum factorisation:
    //         S[q][c][d] = sum_a (d_d N_a)(q) w_a X_a^c (X^3 = 1); three
    //         contractions of 3 terms instead of 27 per (point, field, d)
    for (int t = tid; t < 2 * 4 * 3 * 9; t += blockDim.x) {        // x: [N/D][c][gx][jk]
      const int jk = t % 9, gx = (t / 9) % 3, c = (t / 27) % 4, dd = t / 108;
      const float* tbx = sm.tb[0][dd] + gx * 3;
      const float* w = F.wX[c] + 3 * jk;
      (&F.A[0][0][0][0])[t] = fmaf(tbx[0], w[0], fmaf(tbx[1], w[1], tbx[2] * w[2]));
    }
    __syncthreads();
    for (int t = tid; t < 3 * 4 * 9 * 3; t += blockDim.x) {        // y: [NN/DN/ND][c][gx gy][k]
      const int k = t % 3, gxy = (t / 3) % 9, c = (t / 27) % 4, v = t / 108;
      const int gx = gxy % 3, gy = gxy / 3;
      const float* tby = sm.tb[1][v == 2] + gy * 3;
      const float* a = F.A[v == 1][c][gx] + 3 * k;
      (&F.B[0][0][0][0])[t] = fmaf(tby[0], a[0], fmaf(tby[1], a[1], tby[2] * a[2]));
    }
    __syncthreads();
    for (int t = tid; t < kNq * 16; t += blockDim.x) {              // z: S[q][c][d]
      const int d = t % 4, c = (t / 4) % 4, q = t / 16;
      const int gxy = q % 9, gz = q / 9;
      const int src = d == 1 ? 1 : d == 2 ? 2 : 0;                   // DN, ND, else NN
      const float* tbz = sm.tb[2][d == 3] + gz * 3;
      const float* b = F.B[src][c][gxy];
      (&F.S[0][0][0])[t] = fmaf(tbz[0], b[0], fmaf(tbz[1], b[1], tbz[2] * b[2]));
    }
    __syncthreads();

    // ---- 3. per Gauss point: Jacobian, determinant and cofactors in FP64
    //         (from exactly widened FP32 entries), the rest in FP32
    if (tid < kNq) {
      const int q = tid;
      const float* Sq = F.S[q][0];
      const float iW = 1.f / Sq[12];
      double J[9];  // J[d*3 + r] = dX_r/du_d, formed in FP32 and widened exactly
#pragma unroll
      for (int r = 0; r < 3; r++) {
        const float Xr = Sq[r * 4] * iW;
#pragma unroll
        for (int d = 0; d < 3; d++)
          J[d * 3 + r] = widenF32((Sq[r * 4 + 1 + d] - Xr * Sq[12 + 1 + d]) * iW);
      }
      const double c0 = J[4] * J[8] - J[5] * J[7], c1 = J[1] * J[8] - J[2] * J[7],
                   c2 = J[1] * J[5] - J[2] * J[4];
      const double det = J[0] * c0 - J[3] * c1 + J[6] * c2;
      float w = 0.f;
      float B[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // du_d/dx_k at k 3 + d
      if (fabs(det) > kEpsZ) {
        const float detf = narrowF64(det);
        const float id = 1.f / detf;
        B[0] = narrowF64(c0) * id;
        B[1] = -narrowF64(c1) * id;
        B[2] = narrowF64(c2) * id;
        B[3] = -narrowF64(J[3] * J[8] - J[5] * J[6]) * id;
        B[4] = narrowF64(J[0] * J[8] - J[2] * J[6]) * id;
        B[5] = -narrowF64(J[0] * J[5] - J[2] * J[3]) * id;
        B[6] = narrowF64(J[3] * J[7] - J[4] * J[6]) * id;
        B[7] = -narrowF64(J[0] * J[7] - J[1] * J[6]) * id;
        B[8] = narrowF64(J[0] * J[4] - J[1] * J[3]) * id;
        // |J| dV w_i w_j w_k in FP32 (dV = span volume / 8)
        w = detf * sm.dVf * P.gwf[0][q % 3] * P.gwf[1][(q / 3) % 3] * P.gwf[2][q / 9];
        atomicOr(&sm.signs, w > 0.f ? 1 : 2);
      } else {
        atomicAdd(S.counters, 1ull);
      }
      sm.wq[q] = w;
      F.iW[q] = iW;
      // dR_a/dx_k = w_a (sum_d dN_a/du_d E_kd - N_a e_k) with N_a the
      // B-spline products, E_kd = (du_d/dx_k) / W, e_k = sum_d (dW/du_d / W) E_kd
      const float g0 = Sq[13] * iW, g1 = Sq[14] * iW, g2 = Sq[15] * iW;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const float E0 = B[3 * k] * iW, E1 = B[3 * k + 1] * iW, E2 = B[3 * k + 2] * iW;
        F.E[q][3 * k] = E0;
        F.E[q][3 * k + 1] = E1;
        F.E[q][3 * k + 2] = E2;
        F.E[q][9 + k] = fmaf(g0, E0, fmaf(g1, E1, g2 * E2));
      }
    }
    __syncthreads();

    // ---- 4. operand tile and tensor-core Gram matrix, one pass per weight sign
    const int signs = sm.signs;
    bool first = true, ok = true;
    for (int pass = 0; pass < 2 && ok; pass++) {
      const float s = pass == 0 ? 1.f : -1.f;
      if (!(signs & (1 << pass))) continue;
      for (int t = tid; t < kNq * 12; t += blockDim.x) {
        const int q = t / 12;
        const float ws = s * sm.wq[q];
        (&F.Es[0][0])[t] = (ws > 0.f ? sqrtf(ws) : 0.f) * (&F.E[0][0])[t];
      }
      __syncthreads();
      // task (a, g): function a, Gauss points 4g..4g+3 (16-byte stores of
      // each row 32k + a); the three rows k of a from one basis evaluation
      for (int task = tid; task < kNen * 7; task += blockDim.x) {
        const int a = task % kNen, g = task / kNen;
        const int ia = a % 3, ja = (a / 3) % 3, ka = a / 9;
        const float wa = sm.X[a][3];
        float hi[3][4], lo[3][4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int q = 4 * g + u;
          float t0 = 0.f, t1 = 0.f, t2 = 0.f;
          if (q < kNq) {
            const int gx = q % 3, gy = (q / 3) % 3, gz = q / 9;
            const float nx = sm.tb[0][0][3 * gx + ia], dx = sm.tb[0][1][3 * gx + ia];
            const float ny = sm.tb[1][0][3 * gy + ja], dy = sm.tb[1][1][3 * gy + ja];
            const float nz = sm.tb[2][0][3 * gz + ka], dz = sm.tb[2][1][3 * gz + ka];
            const float nyz = wa * ny * nz;
            const float du = dx * nyz, dv = wa * nx * dy * nz, dw = wa * nx * ny * dz;
            const float n = nx * nyz;
            const float4 E0 = *reinterpret_cast<const float4*>(F.Es[q]);
            const float4 E1 = *reinterpret_cast<const float4*>(F.Es[q] + 4);
            const float4 E2 = *reinterpret_cast<const float4*>(F.Es[q] + 8);
            // E_kd at 3k + d, e_k at 9 + k
            t0 = fmaf(du, E0.x, fmaf(dv, E0.y, fmaf(dw, E0.z, -n * E2.y)));
            t1 = fmaf(du, E0.w, fmaf(dv, E1.x, fmaf(dw, E1.y, -n * E2.z)));
            t2 = fmaf(du, E1.z, fmaf(dv, E1.w, fmaf(dw, E2.x, -n * E2.w)));
          }
          splitTF32(t0, hi[0][u], lo[0][u]);
          splitTF32(t1, hi[1][u], lo[1][u]);
          splitTF32(t2, hi[2][u], lo[2][u]);
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
          const int o = kmaj(32 * k + a, 4 * g);
          *reinterpret_cast<float4*>(sm.Thi + o) = make_float4(hi[k][0], hi[k][1], hi[k][2], hi[k][3]);
          *reinterpret_cast<float4*>(sm.Tlo + o) = make_float4(lo[k][0], lo[k][1], lo[k][2], lo[k][3]);
        }
      }
      fenceProxyAsync();
      __syncthreads();
      if (tid == 0) {
        tcFenceAfter();
        const uint32_t idesc = instrDescTF32(kM, kN) | (s < 0.f ? (1u << 13) : 0u);
        for (int st = 0; st < kK / 8; st++) {
          const uint32_t off = st * 256;
          mmaTF32(tmem, smemDesc(tHi + off), smemDesc(tHi + off), idesc, first ? 0u : 1u);
          mmaTF32(tmem, smemDesc(tHi + off), smemDesc(tLo + off), idesc, 1);
          mmaTF32(tmem, smemDesc(tLo + off), smemDesc(tHi + off), idesc, 1);
          first = false;
        }
        mmaCommit(mbar);
      }
      first = false;
      ok = mbarWait(mbar, phase);
      phase ^= 1u;
      tcFenceAfter();
    }
    if (!ok && tid == 0) {
      atomicAdd(S.counters + 2, 1ull);
      sm.fail = 1;
    }

    // ---- 5. element load vector: body force, Fe[a][k] = b_k sum_q R_a w_q
    //         (R_a = w_a N_a / W), and Neumann traction on the patch faces
    //         this element touches
    float fe = 0.f;
    if (tid < kNen * 3) {
      const int a = tid / 3, k = tid % 3;
      const float bk = P.bodyf[k];
      if (bk != 0.f) {
        const int ia = a % 3, ja = (a / 3) % 3, ka = a / 9;
        float acc = 0.f;
        for (int q = 0; q < kNq; q++) {
          const float n = sm.tb[0][0][3 * (q % 3) + ia] * sm.tb[1][0][3 * ((q / 3) % 3) + ja] *
                          sm.tb[2][0][3 * (q / 9) + ka];
          acc = fmaf(n * F.iW[q], sm.wq[q], acc);
        }
        fe = bk * sm.X[a][3] * acc;
      }
    }
    // constant traction t: Fe += t R dS w at the 3x3 face points (face
    // overload of ASMs3D::integrate, src/ASM/ASMs3D.C:2547-2812)
    for (int f = 0; f < P.nneu; f++) {
      const int face = P.neuFace[f];
      const int nd0 = (face - 1) >> 1, side = (face - 1) & 1;
      const int ee[3] = {e1, e2, e3};
      if (ee[nd0] != (side ? P.nel[nd0] - 1 : 0)) continue;  // uniform in the CTA
      float* fR = F.face;            // [9][27] rational basis at the face points
      float* fW = F.face + 9 * 27;   // [9] dS * weights
      if (tid < 9) {
        const int ta = nd0 == 0 ? 1 : 0, tb = nd0 == 2 ? 1 : 2;
        int g[3] = {0, 0, 0};
        g[ta] = tid % 3;
        g[tb] = tid / 3;
        float Nd[3][3], Dd[3][3];
        for (int d = 0; d < 3; d++)
          for (int r = 0; r < 3; r++) {
            if (d == nd0) {
              Nd[d][r] = (float)P.tabB[d][side * 6 + r];
              Dd[d][r] = (float)P.tabB[d][side * 6 + 3 + r];
            } else {
              Nd[d][r] = P.tabNf[d][ee[d] * 9 + g[d] * 3 + r];
              Dd[d][r] = P.tabDf[d][ee[d] * 9 + g[d] * 3 + r];
            }
          }
        float S4[4][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f},
                          {0.f, 0.f, 0.f, 0.f}};
        for (int a = 0; a < kNen; a++) {
          const int i = a % 3, j = (a / 3) % 3, k = a / 9;
          const float w = sm.X[a][3];
          const float wN = w * Nd[0][i] * Nd[1][j] * Nd[2][k];
          const float w0 = w * Dd[0][i] * Nd[1][j] * Nd[2][k];
          const float w1 = w * Nd[0][i] * Dd[1][j] * Nd[2][k];
          const float w2 = w * Nd[0][i] * Nd[1][j] * Dd[2][k];
          fR[tid * 27 + a] = wN;
#pragma unroll
          for (int c = 0; c < 4; c++) {
            const float x = c < 3 ? sm.X[a][c] : 1.f;
            S4[c][0] = fmaf(wN, x, S4[c][0]);
            S4[c][1] = fmaf(w0, x, S4[c][1]);
            S4[c][2] = fmaf(w1, x, S4[c][2]);
            S4[c][3] = fmaf(w2, x, S4[c][3]);
          }
        }
        const float iW = 1.f / S4[3][0];
        float J[9];  // J[d*3 + c] = dX_c/du_d
        for (int c = 0; c < 3; c++)
          for (int d = 0; d < 3; d++)
            J[d * 3 + c] = (S4[c][1 + d] - S4[c][0] * iW * S4[3][1 + d]) * iW;
        const int t1 = 1 + (nd0 + 1) % 3, t2 = 1 + t1 % 3;
        const float* u = J + 3 * (t1 - 1);
        const float* v = J + 3 * (t2 - 1);
        const float nx = u[1] * v[2] - u[2] * v[1], ny = u[2] * v[0] - u[0] * v[2],
                    nz = u[0] * v[1] - u[1] * v[0];
        const double det = (double)J[0] * ((double)J[4] * J[8] - (double)J[5] * J[7]) -
                           (double)J[3] * ((double)J[1] * J[8] - (double)J[2] * J[7]) +
                           (double)J[6] * ((double)J[1] * J[5] - (double)J[2] * J[4]);
        float wgt = 0.f;
        if (det > kEpsZ || det < -kEpsZ)
          wgt = sqrtf(nx * nx + ny * ny + nz * nz) * 0.25f * (float)P.span[ta][ee[ta]] *
                (float)P.span[tb][ee[tb]] * (float)P.fw[ta][g[ta]] * (float)P.fw[tb][g[tb]];
        for (int a = 0; a < kNen; a++) fR[tid * 27 + a] *= iW;
        fW[tid] = wgt;
      }
      __syncthreads();
      if (tid < kNen * 3) {
        const int a = tid / 3, c = tid % 3;
        float acc = 0.f;
        for (int gq = 0; gq < 9; gq++) acc = fmaf(fR[gq * 27 + a], fW[gq], acc);
        fe = fmaf(P.neuT[f][c], acc, fe);
      }
      __syncthreads();
    }
    __syncthreads();  // the element block below overlays the front-end arrays

    // ---- 6. tensor memory -> exactly symmetric Gram matrix in the element
    //         block layout: row r = 3a + k keeps its entries at and right of
    //         the diagonal (c = 3b + l >= r) and mirrors them (the MMA's FP32
    //         sums of G_rc and G_cr need not agree), so the element matrix and
    //         the assembled matrix are exactly symmetric
    float* Gc = sm.u.Gc;
    if (ok && warp < 3 && signs) {
      float v[16];
      const int a = lane, k = warp, r = 3 * lane + warp;
#pragma unroll
      for (int c16 = 0; c16 < kN / 16; c16++) {
        tmemLoad16(tmem + ((uint32_t)(32 * warp) << 16) + 16 * c16, v);
        if (lane < kNen) {
#pragma unroll
          for (int i = 0; i < 16; i++) {
            const int n = 16 * c16 + i, l = n >> 5, bcol = n & 31, c = 3 * bcol + l;
            if (bcol < kNen && c >= r) {
              Gc[r * kGs + 27 * l + bcol] = v[i];
              Gc[c * kGs + 27 * k + a] = v[i];
            }
          }
        }
      }
    } else if (!signs) {
      for (int i = tid; i < 81 * kGs; i += blockDim.x) Gc[i] = 0.f;
    }
    if (tid < kNen * 3) Gc[81 * kGs + tid] = fe;  // F[a][k] at 3a + k = tid
    if (tid < kBlock - 82 * 81) Gc[82 * 81 + tid] = 0.f;
    tcFenceBefore();
    __syncthreads();
    if (sm.fail) break;
    if (it + (int)gridDim.x < count) nextItem = items[it + gridDim.x];

    // ---- 7. the element block to the scratch (16-byte stores)
    {
      float4* dst = reinterpret_cast<float4*>(P.elm + (size_t)e * P.elmStride);
      const float4* src = reinterpret_cast<const float4*>(Gc);
      for (int i = tid; i < kBlock / 4; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();  // the next element's step 1 overwrites the block
  }
  // after a timeout: a copy still in flight lands before the CTA exits
  if (tid == 0 && ctrlOut) mbarWait(ctrlbar, cphase, S.mbarSpin);

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

size_t tcVolumeSmem() { return sizeof(TcSmem); }

namespace {

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encodeTiled()
{
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

}  // namespace

// Tensor map (128 bytes at out) of a node-major array with `inner` values of
// `esize` bytes (4: INT32, 8: FLOAT64) per node of an n0 x n1 x n2 control
// net; boxes of inner x q x q x q (one element's nodes for degree q - 1).
// Row pitches and the inner extent are multiples of 16 bytes.
bool nodeBoxMap(void* out, size_t esize, void* base, int inner, const int n[3], int q)
{
  const EncodeTiledFn enc = encodeTiled();
  if (!enc || (esize * inner) % 16 != 0 || reinterpret_cast<uintptr_t>(base) % 16 != 0 ||
      (esize != 4 && esize != 8) || q < 1 || q > 8)
    return false;
  const CUtensorMapDataType type =
      esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_INT32;
  const cuuint64_t dims[4] = {(cuuint64_t)inner, (cuuint64_t)n[0], (cuuint64_t)n[1], (cuuint64_t)n[2]};
  const cuuint64_t strides[3] = {esize * inner, esize * inner * n[0],
                                 esize * inner * (cuuint64_t)n[0] * n[1]};
  const cuuint32_t box[4] = {(cuuint32_t)inner, (cuuint32_t)q, (cuuint32_t)q, (cuuint32_t)q};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(static_cast<CUtensorMap*>(out), type, 4, base, dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The tensor map of the control net of a tensor-core patch (3x3x3 node
// boxes); false leaves the patch to the generic kernel.
bool tcUploadPatch(ifemgpu_ctx* ctx, HostPatch& pc, DevPatch& D)
{
  (void)ctx;
  if (!pc.d_ctrl) return false;
  CUtensorMap map;
  const bool ok = nodeBoxMap(&map, 8, (void*)pc.d_ctrl, 4, pc.n, 3) &&
                  cudaMalloc(&pc.d_tmaps, sizeof(map)) == cudaSuccess &&
                  cudaMemcpy(pc.d_tmaps, &map, sizeof(map), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    return false;
  }
  D.tmaps = pc.d_tmaps;
  return true;
}

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
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_volume_tc_elast_p2,
                                         cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared));
  return IFEMGPU_OK;
}

ifemgpu_status tcLaunchVolume(ifemgpu_ctx* ctx, const Pass& p, int)
{
  TcSys S{ctx->d_counters, ctx->dbg.mbarSpin ? ctx->dbg.mbarSpin : kSpinLimit, ctx->dbg.patch,
          ctx->dbg.elem};
  // as many CTAs as fit at once (shared memory, registers and the 4 x 128
  // tensor-memory columns of an SM); no CTA waits for another
  cudaFuncAttributes fa{};
  IFEMGPU_CUDA(ctx, cudaFuncGetAttributes(&fa, k_volume_tc_elast_p2));
  int smemSM = 0, resv = 0, regsSM = 0;
  IFEMGPU_CUDA(ctx, cudaDeviceGetAttribute(&smemSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor,
                                           ctx->opts.device));
  IFEMGPU_CUDA(ctx, cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock,
                                           ctx->opts.device));
  IFEMGPU_CUDA(ctx, cudaDeviceGetAttribute(&regsSM, cudaDevAttrMaxRegistersPerMultiprocessor,
                                           ctx->opts.device));
  const int bySmem = smemSM / (int)(tcVolumeSmem() + resv);
  const int byRegs = regsSM / (((fa.numRegs + 7) / 8) * 8 * 128);
  const int perSM = std::min(std::min(bySmem, byRegs), kTcPerSM);
  const int grid = std::min(p.count, perSM * ctx->numSMs);
  if (ctx->opts.verbose)
    std::printf("tensor-core volume kernel: %zu B shared memory, %d registers, %d blocks/SM, grid %d\n",
                tcVolumeSmem(), fa.numRegs, perSM, grid);
  const DevPatch* patches = ctx->d_patches;
  const Item* items = ctx->d_items + p.first;
  int count = p.count;
  void* args[] = {(void*)&patches, (void*)&items, (void*)&count, (void*)&S};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = tcVolumeSmem();
  cfg.stream = ctx->stream;
  cfg.numAttrs = 0;
  IFEMGPU_CUDA(ctx, cudaLaunchKernelExC(&cfg, (const void*)k_volume_tc_elast_p2, args));
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
