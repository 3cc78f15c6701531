// tc_poisson.cu -- tensor-core (tcgen05, sm_103a) element kernels for the 3D
// Poisson integrand with p = 2 and p = 3 spline patches (Gauss rule p + 1 per
// direction): the hot loop of ASMs3D::integrate (src/ASM/ASMs3D.C:2266-2312)
// with EqualOrderOperators::Weak::LaplacianCoeff and ::Source
// (Apps/Utils/EqualOrderOperators.C:158-265).  The element matrices go to the
// element scratch, which the node-wise gather (gather.cu) sums into the
// compressed-column matrix (the scatter of assemSparse,
// src/LinAlg/SparseMatrix.C:614-688).
//
// One persistent launch per degree processes every element of its patches,
// one CTA of 128 threads per element, elements in index order (no element
// waits for another).  Per element:
//   0. the (p+1)^3 control points staged by TMA, requested as soon as the
//      previous element has read its own;
//   1. geometry at the Gauss points by sum factorisation of the homogeneous
//      control net (w x, w y, w z, w) and of w g, w n (log-conductivity and
//      source noise at the nodes): three contractions of (p+1) terms, FP32;
//      Jacobian determinant and inverse in FP64 from exactly widened sums;
//   2. operand rows T[a, 3q + k] = sqrt|kappa_q w_q| dR_a/dx_k (functions a,
//      Gauss points q, directions k) in chunks of 32 points, so that the
//      element matrix is K = s T T^T with the sign s of kappa w; elements
//      whose weights change sign run one pass per sign (negate-A bit);
//   3. K on the tensor cores in 3xTF32 split precision (M = 128 over the
//      function rows, N = 32 or 64, K = 96 per chunk), FP32 accumulation in
//      tensor memory; the element load vector Fe_a = sum_q R_a f_q w_q on the
//      CUDA cores while the operand rows are formed;
//   4. K from tensor memory to shared memory, exactly symmetric (the upper
//      triangle mirrored), and with Fe to the element's scratch block
//      K[a][b], F[a].
#include <algorithm>
#include <cstdio>
#include <vector>

#include "ifemgpu_internal.h"
#include "tc_common.cuh"

namespace ifemgpu {

using namespace tc;

namespace {

template <int P>
struct PCfg {
  static constexpr int Q = P + 1;                  // functions and Gauss points per direction
  static constexpr int Q2 = Q * Q;
  static constexpr int NEN = Q * Q * Q;            // 27, 64
  static constexpr int NQ = NEN;
  static constexpr int ROWS = P == 2 ? 32 : 64;    // operand rows = MMA N = TMEM columns
  static constexpr int SPLIT = 128 / ROWS;         // thread groups per operand row (4, 2)
  static constexpr int CHUNKS = (NQ + 31) / 32;    // 32 Gauss points per operand chunk
  static constexpr int PTS = 32 / SPLIT;           // points per thread and chunk (8, 16)
  static constexpr int TILE = ROWS * kK;           // floats per 32-wide K tile
  static constexpr int TFL = 3 * TILE;             // floats per chunk and copy (K = 96)
  static constexpr int GS = NEN % 2 ? NEN : NEN + 1;  // odd Gram row stride (conflict-free)
  static constexpr int OVER = (128 - ROWS) * kK;   // floats the A operand reads past Tlo
  static constexpr int PER_SM = P == 2 ? 5 : 3;    // CTAs per SM (shared memory)
  static constexpr int BLOCK = NEN * NEN + NEN;    // element block: K[a][b], F[a] (16-byte multiple)
};

template <int P>
struct PSmem {
  using C = PCfg<P>;
  alignas(128) double ctrlT[C::NEN][4];    // control points x, y, z, w (TMA)
  float X[C::NEN][4];                      // relative control points, weight
  float fv[2][C::NEN];                     // log-conductivity and noise at the nodes
  float tb[3][2][C::Q2];                   // 1D tables [direction][N, dN/du][g (p+1) + i]
  float fePart[C::SPLIT][C::ROWS];         // element load vector, per point group
  double c00[3];                           // first control point of the element
  unsigned long long mbar, ctrlbar;
  uint32_t tmemSlot;
  int fail;
  int signs;                               // bit 0: some kappa w > 0, bit 1: some < 0
  float dVf;                               // span volume / 8
  // operand chunk (K-major core matrices, three 32-wide K tiles); before the
  // MMAs the sum-factorisation arrays live here, after them the element matrix
  alignas(1024) float Thi[C::TFL];
  float Tlo[C::TFL];
  // the MMA's A operand reads 128 rows from each tile start: rows ROWS..127
  // of the last Tlo tile fall into this union, only feeding accumulator lanes
  // that are never read; nothing writes it while an MMA runs
  union {
    struct {
      float Wq[C::NQ][4];   // 1/W and dW/du_d
      float Ji[C::NQ][9];   // column-major inverse Jacobian
      float Cq[C::NQ][9];   // sqrt(max(s kappa w, 0)) Jinv of the current sign pass
      float kw[C::NQ];      // kappa |J| w, signed (0 at singular points)
      float fw[C::NQ];      // f |J| w
    } pt;
    float over[C::OVER];
  } t;
};

static_assert(sizeof(PSmem<3>) + 1024 <= 233472 / 3, "three p = 3 CTAs per SM");
static_assert(sizeof(PSmem<2>) + 1024 <= 233472 / 5, "five p = 2 CTAs per SM");
static_assert(6 * 64 + 10 * 64 + 14 * 64 + 64 * 24 <= PCfg<3>::TFL &&
                  6 * 27 + 10 * 27 + 14 * 27 + 27 * 24 <= PCfg<2>::TFL,
              "sum-factorisation arrays fit in the operand tile");
static_assert(PCfg<3>::NEN * (PCfg<3>::GS + 1) <= PCfg<3>::TFL &&
                  PCfg<2>::NEN * (PCfg<2>::GS + 1) <= PCfg<2>::TFL,
              "element matrix and load vector fit in the operand tile");
static_assert(PCfg<3>::BLOCK % 4 == 0 && PCfg<2>::BLOCK % 4 == 0, "16-byte element blocks");

}  // namespace

struct PoisSys {
  unsigned long long* counters;  // [0] singular points, [2] device timeouts
  unsigned mbarSpin;             // polls per wait for a copy
  int wPatch, wElem;             // element whose copy is never issued (test hook), -1 none
};

template <int P>
__global__ void __launch_bounds__(128)
k_volume_tc_poisson(const DevPatch* __restrict__ patches, const Item* __restrict__ items,
                    int count, PoisSys S)
{
  using C = PCfg<P>;
  constexpr int Q = C::Q, Q2 = C::Q2, Q3 = C::NEN;
  extern __shared__ __align__(1024) unsigned char smraw[];
  PSmem<P>& sm = *reinterpret_cast<PSmem<P>*>(smraw);
  static_assert(offsetof(PSmem<P>, Tlo) == offsetof(PSmem<P>, Thi) + sizeof(float) * C::TFL &&
                    offsetof(PSmem<P>, t) == offsetof(PSmem<P>, Tlo) + sizeof(float) * C::TFL,
                "A-operand reads past Tlo must stay inside the union");
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t mbar = smemAddr(&sm.mbar), ctrlbar = smemAddr(&sm.ctrlbar);
  if (tid == 0) {
    mbarInit(mbar, 1);
    mbarInit(ctrlbar, 1);
    sm.fail = 0;
  }
  if (warp == 0) tmemAlloc(&sm.tmemSlot, C::ROWS);
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = sm.tmemSlot;
  const uint32_t tHi = smemAddr(sm.Thi), tLo = smemAddr(sm.Tlo);
  uint32_t phase = 0;
  int mapPatch = -1;
  bool ctrlOut = false;  // copy in flight (thread 0)
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
    mbarExpectTx(ctrlbar, sizeof(double) * C::NEN * 4);
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
    const DevPatch& Pt = patches[item.patch];
    const int e = item.elem;
    const int e1 = e % Pt.nel[0], e2 = (e / Pt.nel[0]) % Pt.nel[1], e3 = e / (Pt.nel[0] * Pt.nel[1]);
    const bool hasG = Pt.logk != nullptr, hasN = Pt.noise != nullptr;

    // ---- 0. node data (control points by TMA), nodal fields, 1D tables (read
    //         from L2 while the control points arrive)
    float tbv = 0.f;
    if (tid < 6 * Q2) {
      const int d = tid / (2 * Q2), dd = (tid / Q2) % 2, gi = tid % Q2;
      const int ed = d == 0 ? e1 : d == 1 ? e2 : e3;
      tbv = (dd ? Pt.tabDf[d] : Pt.tabNf[d])[ed * Q2 + gi];
    }
    double dV = 0.0;  // span volume
    if (tid == 97) dV = Pt.span[0][e1] * Pt.span[1][e2] * Pt.span[2][e3];
    float gv = 0.f, nv = 0.f;  // nodal log-conductivity and noise, also read early
    if (tid < C::NEN) {
      const int node = ((e3 + tid / Q2) * Pt.n[1] + e2 + (tid / Q) % Q) * Pt.n[0] + e1 + tid % Q;
      if (hasG) gv = (float)Pt.logk[node];
      if (hasN) nv = (float)Pt.noise[node];
    }
    if (mbarWait(ctrlbar, cphase, S.mbarSpin)) {
      cphase ^= 1u;
      ctrlOut = false;
    } else {
      atomicAdd(S.counters + 2, 1ull);
      sm.fail = 1;
    }
    float* sFw = sm.Thi;  // weighted nodal fields [6][nen]: w x, w y, w z, w, w g, w n
    if (tid < C::NEN) {
      const int a = tid;
      const float x0 = (float)(sm.ctrlT[a][0] - sm.ctrlT[0][0]);
      const float x1 = (float)(sm.ctrlT[a][1] - sm.ctrlT[0][1]);
      const float x2 = (float)(sm.ctrlT[a][2] - sm.ctrlT[0][2]);
      const float w = (float)sm.ctrlT[a][3];
      sm.X[a][0] = x0;
      sm.X[a][1] = x1;
      sm.X[a][2] = x2;
      sm.X[a][3] = w;
      const float g = gv, nz = nv;
      sm.fv[0][a] = g;
      sm.fv[1][a] = nz;
      sFw[a] = w * x0;
      sFw[C::NEN + a] = w * x1;
      sFw[2 * C::NEN + a] = w * x2;
      sFw[3 * C::NEN + a] = w;
      sFw[4 * C::NEN + a] = w * g;
      sFw[5 * C::NEN + a] = w * nz;
    }
    if (tid >= 64 && tid < 67) sm.c00[tid - 64] = sm.ctrlT[0][tid - 64];
    if (tid == 96) sm.signs = 0;
    if (tid == 97) sm.dVf = (float)(0.125 * dV);
    if (tid < 6 * Q2) sm.tb[tid / (2 * Q2)][(tid / Q2) % 2][tid % Q2] = tbv;
    __syncthreads();  // ctrlT read, node data visible
    if (sm.fail) break;
    if (tid == 0 && it + (int)gridDim.x < count) stageCtrl(it + gridDim.x);

    // ---- 1. sums over the element's functions at every Gauss point by sum
    //         factorisation.  Fields 0..3 (w x, w y, w z, w) with their
    //         derivatives, fields 4, 5 (w g, w n) values only.
    float* sA = sFw + 6 * C::NEN;  // blocks 2f + [N, D] (f < 4), 8 + (f - 4): [k][j][gi]
    float* sB = sA + 10 * Q3;      // blocks 3f + [NN, DN, ND] (f < 4), 12 + (f - 4): [k][gj][gi]
    float* sP = sB + 14 * Q3;      // [6][value, d/du, d/dv, d/dw][q]: slot-major
    for (int t = tid; t < 10 * Q3; t += blockDim.x) {
      const int blk = t / Q3, r = t - blk * Q3;
      const int gi = r % Q, j = (r / Q) % Q, k = r / Q2;
      const int f = blk < 8 ? blk >> 1 : blk - 4, d0 = blk < 8 ? blk & 1 : 0;
      const float* fw = sFw + f * C::NEN + Q * j + Q2 * k;
      const float* tb = sm.tb[0][d0] + gi * Q;
      float acc = 0.f;
#pragma unroll
      for (int i = 0; i < Q; i++) acc = fmaf(tb[i], fw[i], acc);
      sA[t] = acc;
    }
    __syncthreads();
    for (int t = tid; t < 14 * Q3; t += blockDim.x) {
      const int blk = t / Q3, r = t - blk * Q3;
      const int gi = r % Q, gj = (r / Q) % Q, k = r / Q2;
      int src, d1;
      if (blk < 12) {
        const int f = blk / 3, c = blk - 3 * f;
        src = 2 * f + (c == 1);
        d1 = c == 2;
      } else {
        src = blk - 4;  // 12, 13 -> 8, 9
        d1 = 0;
      }
      const float* a = sA + src * Q3 + k * Q2 + gi;
      const float* tb = sm.tb[1][d1] + gj * Q;
      float acc = 0.f;
#pragma unroll
      for (int jj = 0; jj < Q; jj++) acc = fmaf(tb[jj], a[jj * Q], acc);
      sB[t] = acc;
    }
    __syncthreads();
    // lanes over the Gauss points of one output slot: the lanes of a warp
    // read one source block (no bank conflicts) and store consecutive words
    for (int t = tid; t < C::NQ * 18; t += blockDim.x) {
      const int r = t / C::NQ, q = t - r * C::NQ;
      const int gi = q % Q, gj = (q / Q) % Q, gk = q / Q2;
      int src, d2, slot;
      if (r < 16) {
        const int f = r >> 2, c4 = r & 3;
        src = 3 * f + (c4 == 1 ? 1 : c4 == 2 ? 2 : 0);
        d2 = c4 == 3;
        slot = r;
      } else {
        src = r - 4;          // 16, 17 -> 12, 13
        d2 = 0;
        slot = (r - 12) * 4;  // 16, 20
      }
      const float* b = sB + src * Q3 + gj * Q + gi;
      const float* tb = sm.tb[2][d2] + gk * Q;
      float acc = 0.f;
#pragma unroll
      for (int kk = 0; kk < Q; kk++) acc = fmaf(tb[kk], b[kk * Q2], acc);
      sP[slot * C::NQ + q] = acc;
    }
    __syncthreads();

    // ---- 2. per Gauss point: Jacobian (FP64 determinant and inverse),
    //         weight, conductivity kappa = kappa0 exp(sum R g), source
    if (tid < C::NQ) {
      const int q = tid;
      auto Pq = [&](int k) { return sP[k * C::NQ + q]; };
      const float iW = 1.f / Pq(12);
      double J[9];  // J[d*3 + r] = dX_r/du_d, formed in FP32 and widened exactly
#pragma unroll
      for (int r = 0; r < 3; r++) {
        const float Xr = Pq(r * 4) * iW;
#pragma unroll
        for (int d = 0; d < 3; d++)
          J[d * 3 + r] = widenF32((Pq(r * 4 + 1 + d) - Xr * Pq(12 + 1 + d)) * iW);
      }
      const double c0 = J[4] * J[8] - J[5] * J[7], c1 = J[1] * J[8] - J[2] * J[7],
                   c2 = J[1] * J[5] - J[2] * J[4];
      const double det = J[0] * c0 - J[3] * c1 + J[6] * c2;
      float w = 0.f;
      float B[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (fabs(det) > kEpsZ) {
        // cofactors and determinant narrowed on the integer pipe, the
        // quotients in FP32 (an FP64 division and nine FP64 products and
        // conversions would occupy the scarce FP64 units)
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
        w = detf * sm.dVf * Pt.gwf[0][q % Q] * Pt.gwf[1][(q / Q) % Q] * Pt.gwf[2][q / Q2];
      } else {
        atomicAdd(S.counters, 1ull);
      }
      float kap = (float)Pt.kappa;
      if (hasG) kap *= expf(Pq(16) * iW);
      float f = (float)Pt.source;
      if (Pt.source_shape == IFEMGPU_SOURCE_SINE)
        for (int c = 0; c < 3; c++) f *= sinpif((float)((double)(Pq(c * 4) * iW) + sm.c00[c]));
      if (hasN) f *= 1.f + Pq(20) * iW;
      const float kw = kap * w;
      if (kw != 0.f) atomicOr(&sm.signs, kw > 0.f ? 1 : 2);
      sm.t.pt.kw[q] = kw;
      sm.t.pt.fw[q] = f * w;
      sm.t.pt.Wq[q][0] = iW;
      sm.t.pt.Wq[q][1] = Pq(13);
      sm.t.pt.Wq[q][2] = Pq(14);
      sm.t.pt.Wq[q][3] = Pq(15);
      for (int c = 0; c < 9; c++) sm.t.pt.Ji[q][c] = B[c];
    }
    __syncthreads();

    // ---- 3. operand rows and the tensor-core Gram matrix, one pass per sign
    const int signs = sm.signs;
    const int ra = tid % C::ROWS, hg = tid / C::ROWS;  // operand row, point group
    bool first = true, ok = true;
    float fe = 0.f;
    bool feDone = false;
    for (int pass = 0; pass < 2 && ok; pass++) {
      if (!(signs & (1 << pass))) continue;
      const float s = pass == 0 ? 1.f : -1.f;
      if (tid < C::NQ) {
        const float ws = s * sm.t.pt.kw[tid];
        const float sw = ws > 0.f ? sqrtf(ws) : 0.f;
#pragma unroll
        for (int c = 0; c < 9; c++) sm.t.pt.Cq[tid][c] = sw * sm.t.pt.Ji[tid][c];
      }
      __syncthreads();
      for (int ch = 0; ch < C::CHUNKS && ok; ch++) {
        if (ch > 0) {  // the previous chunk's MMAs must have read the tiles
          ok = mbarWait(mbar, phase);
          phase ^= 1u;
          tcFenceAfter();
          if (!ok) break;
        }
        if (ra < C::NEN) {
          const int i = ra % Q, j = (ra / Q) % Q, k = ra / Q2;
          const float wa = sm.X[ra][3];
#pragma unroll 1
          for (int g4 = 0; g4 < C::PTS / 4; g4++) {
            float hi[12], lo[12];
#pragma unroll
            for (int u = 0; u < 4; u++) {
              const int q = ch * 32 + hg * C::PTS + g4 * 4 + u;
              float t0 = 0.f, t1 = 0.f, t2 = 0.f;
              if (q < C::NQ) {
                const int gi = q % Q, gj = (q / Q) % Q, gk = q / Q2;
                const float n0 = sm.tb[0][0][gi * Q + i], d0 = sm.tb[0][1][gi * Q + i];
                const float n1 = sm.tb[1][0][gj * Q + j], d1 = sm.tb[1][1][gj * Q + j];
                const float n2 = sm.tb[2][0][gk * Q + k], d2 = sm.tb[2][1][gk * Q + k];
                const float* Wq = sm.t.pt.Wq[q];
                const float w12 = wa * n1 * n2;
                const float R = w12 * n0 * Wq[0];
                const float du = (w12 * d0 - R * Wq[1]) * Wq[0];
                const float dv = (wa * n0 * d1 * n2 - R * Wq[2]) * Wq[0];
                const float dw = (wa * n0 * n1 * d2 - R * Wq[3]) * Wq[0];
                const float* Cq = sm.t.pt.Cq[q];
                t0 = du * Cq[0] + dv * Cq[1] + dw * Cq[2];
                t1 = du * Cq[3] + dv * Cq[4] + dw * Cq[5];
                t2 = du * Cq[6] + dv * Cq[7] + dw * Cq[8];
                if (!feDone) fe = fmaf(R, sm.t.pt.fw[q], fe);
              }
              splitTF32(t0, hi[3 * u], lo[3 * u]);
              splitTF32(t1, hi[3 * u + 1], lo[3 * u + 1]);
              splitTF32(t2, hi[3 * u + 2], lo[3 * u + 2]);
            }
#pragma unroll
            for (int v = 0; v < 3; v++) {
              const int kk = 3 * (hg * C::PTS + 4 * g4) + 4 * v;  // K index within the chunk
              const int o = (kk >> 5) * C::TILE + kmaj(ra, kk & 31);
              *reinterpret_cast<float4*>(sm.Thi + o) =
                  make_float4(hi[4 * v], hi[4 * v + 1], hi[4 * v + 2], hi[4 * v + 3]);
              *reinterpret_cast<float4*>(sm.Tlo + o) =
                  make_float4(lo[4 * v], lo[4 * v + 1], lo[4 * v + 2], lo[4 * v + 3]);
            }
          }
        }
        fenceProxyAsync();
        __syncthreads();
        if (tid == 0) {
          tcFenceAfter();
          const uint32_t idesc = instrDescTF32(128, C::ROWS) | (s < 0.f ? (1u << 13) : 0u);
          for (int t3 = 0; t3 < 3; t3++)
            for (int st = 0; st < kK / 8; st++) {
              const uint32_t off = (uint32_t)(t3 * C::TILE) * 4u + st * 256u;
              mmaTF32(tmem, smemDesc(tHi + off), smemDesc(tHi + off), idesc, first ? 0u : 1u);
              mmaTF32(tmem, smemDesc(tHi + off), smemDesc(tLo + off), idesc, 1);
              mmaTF32(tmem, smemDesc(tLo + off), smemDesc(tHi + off), idesc, 1);
              first = false;
            }
          mmaCommit(mbar);
        }
        first = false;
      }
      feDone = true;
      if (ok) {
        ok = mbarWait(mbar, phase);
        phase ^= 1u;
        tcFenceAfter();
      }
    }
    if (ra < C::NEN) sm.fePart[hg][ra] = fe;
    if (!ok) sm.fail = 1;
    __syncthreads();  // every MMA complete: the operand tile becomes the element matrix
    if (sm.fail) {
      if (tid == 0) atomicAdd(S.counters + 2, 1ull);
      break;
    }

    // ---- 4. tensor memory -> element matrix G in shared memory (row stride
    //         GS), exactly symmetric: row m keeps its entries at and right of
    //         the diagonal and mirrors them (the MMA's FP32 sums of G_ab and
    //         G_ba need not agree); the load vector after it
    float* G = sm.Thi;
    if (signs && warp < C::ROWS / 32) {
      float v[16];
      const int m = 32 * warp + lane;
#pragma unroll
      for (int c16 = 0; c16 < C::ROWS / 16; c16++) {
        tmemLoad16(tmem + ((uint32_t)(32 * warp) << 16) + 16 * c16, v);
        if (m < C::NEN) {
#pragma unroll
          for (int i = 0; i < 16; i++) {
            const int n = 16 * c16 + i;
            if (n < C::NEN && n >= m) {
              G[m * C::GS + n] = v[i];
              G[n * C::GS + m] = v[i];
            }
          }
        }
      }
    } else if (!signs) {
      for (int i = tid; i < C::NEN * C::GS; i += blockDim.x) G[i] = 0.f;
    }
    if (tid < C::NEN) {
      float fs = 0.f;
#pragma unroll
      for (int g = 0; g < C::SPLIT; g++) fs += sm.fePart[g][tid];
      G[C::NEN * C::GS + tid] = fs;
    }
    tcFenceBefore();
    __syncthreads();
    if (it + (int)gridDim.x < count) nextItem = items[it + gridDim.x];

    // ---- 5. the element block to the scratch: K[a][b] (row stride nen), F[a]
    {
      float4* dst = reinterpret_cast<float4*>(Pt.elm + (size_t)e * Pt.elmStride);
      for (int i4 = tid; i4 < C::BLOCK / 4; i4 += blockDim.x) {
        float v4[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int i = 4 * i4 + u;
          const int a = i / C::NEN, b = i - a * C::NEN;
          v4[u] = a < C::NEN ? G[a * C::GS + b] : G[C::NEN * C::GS + b];
        }
        dst[i4] = make_float4(v4[0], v4[1], v4[2], v4[3]);
      }
    }
    __syncthreads();  // the next element's node data overwrite the tile
  }
  // after a timeout: a copy still in flight lands before the CTA exits
  if (tid == 0 && ctrlOut) mbarWait(ctrlbar, cphase, S.mbarSpin);
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (warp == 0) tmemDealloc(tmem, C::ROWS);
}

// ---------------------------------------------------------------------------
// host side

int tcPoissonDegree(const DevPatch& D, const HostPatch& pc)
{
  if (D.dim != 3 || D.kind != IFEMGPU_POISSON || D.npv != 1 || D.mass != 0.0 || !D.lineOff ||
      !pc.neumann.empty() || !D.tabNf[0] || !D.tabNf[1] || !D.tabNf[2])
    return 0;
  const int p = D.p[0];
  if ((p != 2 && p != 3) || D.p[1] != p || D.p[2] != p) return 0;
  for (int d = 0; d < 3; d++)
    if (D.ng[d] != p + 1 || D.n[d] != D.nel[d] + p) return 0;
  return p;
}

size_t tcPoissonSmem(int deg) { return deg == 2 ? sizeof(PSmem<2>) : sizeof(PSmem<3>); }

// the tensor map of the control net ((p+1)^3 node boxes); false leaves the
// patch to the generic kernel
bool tcPoissonUpload(ifemgpu_ctx* ctx, HostPatch& pc, DevPatch& D, int deg)
{
  (void)ctx;
  if (!pc.d_ctrl) return false;
  alignas(64) unsigned char map[128];
  const bool ok = nodeBoxMap(map, 8, (void*)pc.d_ctrl, 4, pc.n, deg + 1) &&
                  cudaMalloc(&pc.d_tmaps, sizeof(map)) == cudaSuccess &&
                  cudaMemcpy(pc.d_tmaps, map, sizeof(map), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    return false;
  }
  D.tmaps = pc.d_tmaps;
  return true;
}

ifemgpu_status tcPoissonPrepare(ifemgpu_ctx* ctx)
{
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_volume_tc_poisson<2>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(PSmem<2>)));
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_volume_tc_poisson<3>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(PSmem<3>)));
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_volume_tc_poisson<2>,
                                         cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared));
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_volume_tc_poisson<3>,
                                         cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared));
  return IFEMGPU_OK;
}

ifemgpu_status tcPoissonLaunch(ifemgpu_ctx* ctx, const Pass& p, int deg)
{
  if (deg != 2 && deg != 3) return setError(ctx, IFEMGPU_INVALID_ARG, "internal: Poisson kernel degree");
  PoisSys S{ctx->d_counters, ctx->dbg.mbarSpin ? ctx->dbg.mbarSpin : kSpinLimit, ctx->dbg.patch,
          ctx->dbg.elem};
  const void* fn = deg == 2 ? (const void*)k_volume_tc_poisson<2> : (const void*)k_volume_tc_poisson<3>;
  const size_t smem = tcPoissonSmem(deg);
  const int cap = deg == 2 ? PCfg<2>::PER_SM : PCfg<3>::PER_SM;
  // as many CTAs as fit at once (shared memory, registers); no CTA waits
  // for another
  cudaFuncAttributes fa{};
  IFEMGPU_CUDA(ctx, cudaFuncGetAttributes(&fa, fn));
  int smemSM = 0, resv = 0, regsSM = 0;
  IFEMGPU_CUDA(ctx, cudaDeviceGetAttribute(&smemSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor,
                                           ctx->opts.device));
  IFEMGPU_CUDA(ctx, cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock,
                                           ctx->opts.device));
  IFEMGPU_CUDA(ctx, cudaDeviceGetAttribute(&regsSM, cudaDevAttrMaxRegistersPerMultiprocessor,
                                           ctx->opts.device));
  const int bySmem = smemSM / (int)(smem + resv);
  const int byRegs = regsSM / (((fa.numRegs + 7) / 8) * 8 * 128);
  const int perSM = std::max(1, std::min(std::min(bySmem, byRegs), cap));
  const int grid = std::min(p.count, perSM * ctx->numSMs);
  if (ctx->opts.verbose)
    std::printf("tensor-core Poisson kernel p=%d: %zu B shared memory, %d registers, %d blocks/SM, grid %d\n",
                deg, smem, fa.numRegs, perSM, grid);
  const DevPatch* patches = ctx->d_patches;
  const Item* items = ctx->d_items + p.first;
  int count = p.count;
  void* args[] = {(void*)&patches, (void*)&items, (void*)&count, (void*)&S};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream;
  cfg.numAttrs = 0;
  IFEMGPU_CUDA(ctx, cudaLaunchKernelExC(&cfg, fn, args));
  return IFEMGPU_OK;
}

}  // namespace ifemgpu
