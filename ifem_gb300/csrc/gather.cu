// gather.cu -- deterministic assembly of the tensor-core element matrices:
// the second half of the tensor-core assembly.  The element kernels
// (tc_volume.cu, tc_poisson.cu) write each element's matrix (FP32, exactly
// symmetric) and load vector to a block of an element scratch array; here one
// warp per node sums, in ascending element order, the contributions of the
// elements around the node to the node's columns of the compressed-column
// matrix and to its right-hand side entries, and writes every matrix entry
// once.  Together they replace the scatter of assemSparse
// (src/LinAlg/SparseMatrix.C:614-688) driven by SAM::assembleSystem
// (src/LinAlg/SAM.C:430-543), including the right-hand side corrections of
// prescribed DOFs (-c0 K(i, j), SparseMatrix.C:639-687).
//
// Why a gather: every entry is written by one warp, with its contributions
// added in a fixed order (the order of the elements' indices), so the result
// is bitwise reproducible without colouring, flags or atomics, every element
// kernel runs without waiting for its neighbours, and the matrix needs no
// zeroing.  The entry (a, k; b, l) and its mirror (b, l; a, k) are summed by
// different warps from the same exactly symmetric element values in the same
// element order, so the assembled matrix is exactly symmetric.
//
// Element scratch block (floats, per element, `stride` apart):
//   G[a][k][l][b]  element matrix entry of rows (a, k), column (b, l)
//                  (a, b element functions, k, l < npv), at
//                  ((a npv + k) npv + l) nen + b;
//                  elasticity stores the gradient Gram matrix
//                  G_kl(a, b) = sum_q w_q dN_a/dx_k dN_b/dx_l and the entry is
//                  formed here: lambda G_kl + mu G_lk + delta_kl mu tr G;
//   F[a][k]        element load vector, at npv^2 nen^2 + a npv + k.
// Sums are double-float (an FP32 value and its FP32 rounding error, Knuth's
// TwoSum per addition), widened exactly and added once in FP64 at the end:
// the FP32 element values are summed with an error far below their own.
#include <algorithm>
#include <cstdio>
#include <vector>

#include "ifemgpu_internal.h"
#include "tc_common.cuh"

namespace ifemgpu {

namespace {

template <int P, int NPV, bool HALF>
struct GCfg {
  static constexpr int Q = P + 1;
  static constexpr int NEN = Q * Q * Q;
  static constexpr int W = 2 * P + 1;
  static constexpr int NS = W * W * W;           // neighbour slots of a node
  static constexpr int KL = NPV * NPV;
  // neighbour slots summed by a node's warp: all of them, or (HALF) the
  // centre and the slots after it, the offsets (dz, dy, dx) >= 0 in
  // lexicographic order -- each unordered node pair then belongs to exactly
  // one of its two nodes
  static constexpr int SB = HALF ? NS / 2 : 0;
  static constexpr bool E3 = P == 3 && NPV == 3;
  // warps per CTA, elements whose loads are issued together, CTAs per SM:
  // measured on 64^3 (32^3 for p = 3 elasticity) models; more elements in
  // flight only add registers (p = 2 elasticity spilled with three) where
  // the warps of an SM already keep enough loads in flight
  static constexpr int WARPS = E3 ? (HALF ? 6 : 4) : (P == 3 ? 6 : 8);
  static constexpr int NB = (NEN + 31) / 32;           // element functions per lane
  static constexpr int U = NPV == 3 ? (P == 2 || HALF ? 1 : 3) : (P == 3 ? 1 : 6);
  static constexpr int MINB = E3 ? (HALF ? 3 : 2) : (NPV == 3 ? 3 : (P == 3 ? 5 : 4));
  static constexpr size_t SMEM = sizeof(float) * 2 * KL * (NS - SB) * WARPS;
  // MINB CTAs per SM must fit in its 228 KB of shared memory (1 KB of each
  // CTA's share is reserved by the system)
  static_assert(MINB * (SMEM + 1024) <= 228 * 1024, "gather accumulators exceed shared memory");
};

// hi + lo += x (TwoSum: the rounding error of hi + x goes to lo)
__device__ __forceinline__ void dfAdd(float& hi, float& lo, float x)
{
  const float s = __fadd_rn(hi, x);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
  hi = s;
  lo = __fadd_rn(lo, err);
}

// the same on a shared (hi, lo) pair: one 8-byte load and store
__device__ __forceinline__ void dfAdd(float2* acc, float x)
{
  float2 v = *acc;
  dfAdd(v.x, v.y, x);
  *acc = v;
}

}  // namespace

size_t elementBlockFloats(int p, int npv)
{
  const size_t nen = (size_t)(p + 1) * (p + 1) * (p + 1);
  const size_t f = (size_t)npv * npv * nen * nen + nen * npv;
  return (f + 3) & ~(size_t)3;  // 16-byte blocks
}

struct GatherSys {
  const int* madof;
  const int* meqn;
  const int* F;        // free DOFs of the nodes before each global node
  const double* c0;    // prescribed values (null: none)
  const int* colptr;
  double* K;
  double* b;
};

// One warp per node of the patches of one (degree, npv) class; node item t
// belongs to the last range whose start is <= t.  HALF (models without
// prescribed DOFs): the warp of node a sums only the entries of the node
// pairs it owns (slots from the centre on) and writes each of them twice,
// at (a, k; b, l) in its own columns and at (b, l; a, k) in node b's
// columns: half the loads, additions and accumulators, and the matrix is
// exactly symmetric by construction.  Otherwise every warp sums all of its
// node's neighbour entries and writes its own columns, and the prescribed
// neighbours' terms -c0 K(i, j) go to the right-hand side.
template <int P, int NPV, bool HALF>
__global__ void __launch_bounds__(GCfg<P, NPV, HALF>::WARPS * 32, GCfg<P, NPV, HALF>::MINB)
k_gather(const DevPatch* __restrict__ patches, const int* __restrict__ start,
         const int* __restrict__ pidx, int nranges, int total, GatherSys S)
{
  using C = GCfg<P, NPV, HALF>;
  constexpr int Q = C::Q, NEN = C::NEN, W = C::W, NS = C::NS, KL = C::KL;
  constexpr int SB = C::SB, NSH = NS - SB;
  extern __shared__ float gsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2* acc = reinterpret_cast<float2*>(gsm) + warp * KL * NSH;  // [kl][slot - SB] (hi, lo)
  for (int t = blockIdx.x * C::WARPS + warp; t < total; t += gridDim.x * C::WARPS) {
    int r0 = 0, r1 = nranges - 1;
    while (r0 < r1) {
      const int mid = (r0 + r1 + 1) >> 1;
      if (start[mid] <= t) r0 = mid;
      else r1 = mid - 1;
    }
    const DevPatch& Pt = patches[pidx[r0]];
    const int a = t - start[r0];
    const int n0 = Pt.n[0], n1 = Pt.n[1];
    const int ax = a % n0, ay = (a / n0) % n1, az = a / (n0 * n1);
    const int ga = Pt.firstNode + a;
    const int da = S.madof[ga] - 1;
    int eqa[NPV], cpa[NPV];
    bool any = false;
#pragma unroll
    for (int k = 0; k < NPV; k++) {
      eqa[k] = S.meqn[da + k];
      any |= eqa[k] > 0;
      cpa[k] = eqa[k] > 0 ? S.colptr[eqa[k] - 1] : 0;
    }
    if (!any) continue;  // no column: fixed or prescribed DOFs only
    for (int i = lane; i < KL * NSH; i += 32) acc[i] = make_float2(0.f, 0.f);
    float feHi = 0.f, feLo = 0.f;  // lane k < NPV: load vector of DOF k
    const float lamf = Pt.lamf, muf = Pt.muf;
    const int ex0 = max(0, ax - P), cx = min(ax, Pt.nel[0] - 1) - ex0 + 1;
    const int ey0 = max(0, ay - P), cy = min(ay, Pt.nel[1] - 1) - ey0 + 1;
    const int ez0 = max(0, az - P), cz = min(az, Pt.nel[2] - 1) - ez0 + 1;
    const int ne = cx * cy * cz;
    __syncwarp();
    // elements around the node in ascending index order, U at a time: the
    // loads of U elements are issued before any of them is added, so that
    // each warp keeps U row blocks in flight
    int jx = 0, jy = 0, jz = 0;  // next element, offsets from (ex0, ey0, ez0)
    for (int j0 = 0; j0 < ne; j0 += C::U) {
      float g[C::U][C::NB][KL];
      int alU[C::U];
      const float* blkU[C::U];
#pragma unroll
      for (int u = 0; u < C::U; u++) {
        const int j = j0 + u;
        alU[u] = -1;
        blkU[u] = nullptr;
        if (j < ne) {
          const int ex = ex0 + jx, ey = ey0 + jy, ez = ez0 + jz;
          if (++jx == cx) {
            jx = 0;
            if (++jy == cy) {
              jy = 0;
              ++jz;
            }
          }
          const size_t e = ((size_t)ez * Pt.nel[1] + ey) * Pt.nel[0] + ex;
          alU[u] = (ax - ex) + Q * ((ay - ey) + Q * (az - ez));
          blkU[u] = Pt.elm + e * (size_t)Pt.elmStride;
          const float* row = blkU[u] + (size_t)alU[u] * KL * NEN;
#pragma unroll
          for (int bb = 0; bb < C::NB; bb++) {
            const int bl = lane + 32 * bb;
#pragma unroll
            for (int kl = 0; kl < KL; kl++)
              g[u][bb][kl] = (bl < NEN && (!HALF || bl >= alU[u])) ? __ldcs(row + kl * NEN + bl) : 0.f;
          }
        }
      }
#pragma unroll
      for (int u = 0; u < C::U; u++) {
        if (alU[u] < 0) break;
        const int al = alU[u];
        const int alx = al % Q, aly = (al / Q) % Q, alz = al / (Q * Q);  // constant divisors
#pragma unroll
        for (int bb = 0; bb < C::NB; bb++) {
          const int bl = lane + 32 * bb;
          // (local order = slot order: bl >= al exactly for the owned slots)
          if (bl < NEN && (!HALF || bl >= al)) {
            const int blx = bl % Q, bly = (bl / Q) % Q, blz = bl / (Q * Q);
            const int s = (blx - alx + P) + W * ((bly - aly + P) + W * (blz - alz + P)) - SB;
            const float* gg = g[u][bb];
            if (NPV == 3) {
              const float tr = muf * (gg[0] + gg[4] + gg[8]);
#pragma unroll
              for (int k = 0; k < 3; k++)
#pragma unroll
                for (int l = 0; l < 3; l++) {
                  const float ke = fmaf(lamf, gg[3 * k + l], fmaf(muf, gg[3 * l + k], k == l ? tr : 0.f));
                  dfAdd(acc + (3 * k + l) * NSH + s, ke);
                }
            } else {
              dfAdd(acc + s, gg[0]);
            }
          }
        }
        if (lane < NPV) dfAdd(feHi, feLo, __ldcs(blkU[u] + (size_t)KL * NEN * NEN + al * NPV + lane));
        __syncwarp();
      }
    }
    // write the node's columns (and, HALF, the mirrored entries in the owned
    // neighbours' columns); prescribed neighbours feed the right-hand side
    double corr[NPV];
    int rankA[NPV];  // position of a's DOF k among its free DOFs
    {
      int r = 0;
#pragma unroll
      for (int k = 0; k < NPV; k++) {
        corr[k] = 0.0;
        rankA[k] = r;
        r += eqa[k] > 0;
      }
    }
    const int Fa = S.F[ga];
    const int* lineOff = Pt.lineOff + (size_t)a * W * W;
    for (int s = SB + lane; s < NS; s += 32) {
      const int dx = s % W - P, dy = (s / W) % W - P, dz = s / (W * W) - P;
      const int bx = ax + dx, by = ay + dy, bz = az + dz;
      if (bx < 0 || bx >= n0 || by < 0 || by >= n1 || bz < 0 || bz >= Pt.n[2]) continue;
      const int b = (bz * n1 + by) * n0 + bx;
      const int gb = Pt.firstNode + b;
      const int db = S.madof[gb] - 1;
      const int pos = lineOff[(dz + P) * W + dy + P] + S.F[gb];
      const bool mirror = HALF && s != SB;
      // row (a, k) in node b's columns: b's line towards a, then a's free DOFs
      const int posB = mirror ? Pt.lineOff[(size_t)b * W * W + (P - dz) * W + P - dy] + Fa : 0;
      int rank = 0;
#pragma unroll
      for (int l = 0; l < NPV; l++) {
        const int eqb = S.meqn[db + l];
        if (eqb == 0) continue;
        const int cpb = (mirror && eqb > 0) ? S.colptr[eqb - 1] : 0;
#pragma unroll
        for (int k = 0; k < NPV; k++) {
          if (eqa[k] <= 0) continue;
          const int kl = k * NPV + l;
          const float2 hl = acc[kl * NSH + s - SB];
          const double v = tc::widenF32(hl.x) + tc::widenF32(hl.y);
          if (eqb > 0) {
            S.K[cpa[k] + pos + rank] = v;
            if (mirror) S.K[cpb + posB + rankA[k]] = v;
          } else if (S.c0) {
            corr[k] = fma(S.c0[-eqb - 1], v, corr[k]);
          }
        }
        rank += eqb > 0;
      }
    }
    // right-hand side: load vector minus the prescribed-DOF terms, the lanes'
    // parts added in a fixed order
#pragma unroll
    for (int k = 0; k < NPV; k++) {
      double c = corr[k];
      if (S.c0)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
      const float fh = __shfl_sync(0xffffffffu, feHi, k), fl = __shfl_sync(0xffffffffu, feLo, k);
      if (lane == 0 && eqa[k] > 0) S.b[eqa[k] - 1] = (tc::widenF32(fh) + tc::widenF32(fl)) - c;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// host side

namespace {

template <int P, int NPV, bool HALF>
ifemgpu_status prepareOne(ifemgpu_ctx* ctx, GatherList& g)
{
  using C = GCfg<P, NPV, HALF>;
  const size_t smem = C::SMEM;
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_gather<P, NPV, HALF>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int perSM = 0;
  IFEMGPU_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_gather<P, NPV, HALF>,
                                                                  C::WARPS * 32, smem));
  const int need = (g.total + C::WARPS - 1) / C::WARPS;
  g.grid = std::max(1, std::min(need, std::max(1, perSM) * ctx->numSMs));
  return IFEMGPU_OK;
}

template <int P, int NPV, bool HALF>
ifemgpu_status launchOne(ifemgpu_ctx* ctx, const GatherList& g)
{
  using C = GCfg<P, NPV, HALF>;
  GatherSys S{ctx->d_madof, ctx->d_meqn, ctx->d_freeBefore, ctx->nceq ? ctx->d_c0 : nullptr,
              ctx->d_colptr, ctx->d_K, ctx->d_b};
  k_gather<P, NPV, HALF><<<g.grid, C::WARPS * 32, C::SMEM, ctx->stream>>>(
      ctx->d_patches, g.d_start, g.d_pidx, g.nranges, g.total, S);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  return IFEMGPU_OK;
}

}  // namespace

// kernel attributes and grid of a gather launch (before any capture); the
// half-pair mode is built for p = 3 elasticity only, the one class that
// takes it (for the others the mirrored writes cost more than they save)
ifemgpu_status gatherPrepare(ifemgpu_ctx* ctx, GatherList& g)
{
  if (g.half) {
    if (g.p == 3 && g.npv == 3) return prepareOne<3, 3, true>(ctx, g);
    return setError(ctx, IFEMGPU_INVALID_ARG, "internal: half-pair gather class");
  }
  if (g.p == 2 && g.npv == 3) return prepareOne<2, 3, false>(ctx, g);
  if (g.p == 2 && g.npv == 1) return prepareOne<2, 1, false>(ctx, g);
  if (g.p == 3 && g.npv == 1) return prepareOne<3, 1, false>(ctx, g);
  if (g.p == 3 && g.npv == 3) return prepareOne<3, 3, false>(ctx, g);
  return setError(ctx, IFEMGPU_INVALID_ARG, "internal: gather class");
}

ifemgpu_status gatherLaunch(ifemgpu_ctx* ctx, const GatherList& g)
{
  if (g.total == 0) return IFEMGPU_OK;
  if (g.half) {
    if (g.p == 3 && g.npv == 3) return launchOne<3, 3, true>(ctx, g);
    return setError(ctx, IFEMGPU_INVALID_ARG, "internal: half-pair gather class");
  }
  if (g.p == 2 && g.npv == 3) return launchOne<2, 3, false>(ctx, g);
  if (g.p == 2 && g.npv == 1) return launchOne<2, 1, false>(ctx, g);
  if (g.p == 3 && g.npv == 1) return launchOne<3, 1, false>(ctx, g);
  if (g.p == 3 && g.npv == 3) return launchOne<3, 3, false>(ctx, g);
  return setError(ctx, IFEMGPU_INVALID_ARG, "internal: gather class");
}

}  // namespace ifemgpu
