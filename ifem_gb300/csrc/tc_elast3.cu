// tc_elast3.cu -- tensor-core (tcgen05, sm_103a) element kernel for 3D
// isotropic linear elasticity with cubic (p=3) spline patches and 4x4x4 Gauss
// points: the hot loop of ASMs3D::integrate (src/ASM/ASMs3D.C:2266-2312) with
// the linear-elasticity integrand.  Its element matrices go to the element
// scratch, which the node-wise gather (gather.cu) sums into the
// compressed-column matrix (the scatter of assemSparse,
// src/LinAlg/SparseMatrix.C:614-688).
//
// The element has 64 functions and 192 DOFs.  The gradient Gram matrix
// G[(a,k),(b,l)] = sum_q w_q dR_a/dx_k dR_b/dx_l (rows r = 64k + a) is
// s T^T T with the operand T[(a,k), q] = sqrt|w_q| dR_a/dx_k, formed in two
// chunks of 32 Gauss points and contracted on the tensor cores in 3xTF32:
//   block 1: rows 0..127 (k = 0, 1) against all 192 rows, M = 128, N = 192;
//   block 2: rows 128..191 (k = 2; rows 192..255 of the tile are zero)
//            against rows 128..191, M = 128, N = 64;
// both accumulated in tensor memory over the chunks (256 columns per CTA,
// two CTAs per SM).  Together the blocks hold every entry with c >= r (the
// upper triangle in row order r = 64k + a); each such value is written to the
// element block at (r, c) and at its mirror (c, r) straight from the tensor
// memory read-out, so the block is exactly symmetric.  The element block
// (G[a][k][l][b] at ((3a + k) 3 + l) 64 + b, then F[a][k]) is 148 KB, more
// than shared memory holds, hence the direct global stores; the mirror
// stores of a warp cover 32 consecutive floats.
#include <algorithm>
#include <cstdio>

#include "ifemgpu_internal.h"
#include "tc_common.cuh"

namespace ifemgpu {

using namespace tc;

namespace {

constexpr int kNen = 64;             // functions
constexpr int kNq = 64;              // Gauss points
constexpr int kRows = 256;           // operand rows (192 used, 64 zero)
constexpr int kThreads3 = 256;
constexpr uint32_t kCols3 = 256;     // tensor-memory columns: 192 (block 1) + 64 (block 2)

struct Front3 {
  float wX[4][kNen];        // w x, w y, w z, w (x relative to the element's first node)
  float A[2][4][4][16];     // x contracted: [N/D][field][gx][j + 4k]
  float B[3][4][16][4];     // y contracted: [NN/DN/ND][field][gx + 4gy][k]
  float S[kNq][4][4];       // [q][field][value, d/du, d/dv, d/dw]
  float E[kNq][12];         // (du_d/dx_k) / W at 3k + d, then e_k
  float Es[kNq][12];        // scaled by sqrt(max(s w_q, 0)) for the current sign pass
  float iW[kNq];
  float face[16 * kNen + 16];
};

struct E3Smem {
  float Thi[kRows * kK];    // operand tile of 32 Gauss points, K-major core matrices
  float Tlo[kRows * kK];
  Front3 f;
  float tb[3][2][16];       // 1D tables: [direction][N, dN/du][g 4 + i]
  float wq[kNq];
  float X[kNen][4];
  float fe[kNen * 3];       // element load vector F[a][k] at 3a + k
  alignas(128) double ctrlT[kNen][4];
  unsigned long long mbar;
  unsigned long long ctrlbar;
  uint32_t tmemSlot;
  int fail;
  int signs;
  float dVf;
};

constexpr uint32_t kCtrlBytes3 = sizeof(double) * kNen * 4;
static_assert(2 * (sizeof(E3Smem) + 1024) <= 233472, "two CTAs per SM");
static_assert(offsetof(E3Smem, Tlo) % 1024 == 0 && offsetof(E3Smem, Thi) == 0,
              "operand tiles on 1 KB boundaries");

}  // namespace

struct Tc3Sys {
  unsigned long long* counters;  // [0] singular points, [2] device timeouts
  unsigned mbarSpin;
  int wPatch, wElem;             // element whose copy is never issued (test hook)
  int upper;                     // write only the node pairs b >= a (the gather's half mode)
};

__global__ void __launch_bounds__(kThreads3, 2)
k_volume_tc_elast_p3(const DevPatch* __restrict__ patches, const Item* __restrict__ items,
                     int count, Tc3Sys S)
{
  extern __shared__ __align__(1024) unsigned char smraw[];
  E3Smem& sm = *reinterpret_cast<E3Smem*>(smraw);
  Front3& F = sm.f;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t mbar = smemAddr(&sm.mbar), ctrlbar = smemAddr(&sm.ctrlbar);
  if (tid == 0) {
    mbarInit(mbar, 1);
    mbarInit(ctrlbar, 1);
    sm.fail = 0;
  }
  // rows 192..255 of the operand tiles stay zero (block 2's padding)
  for (int i = tid; i < kRows * kK; i += blockDim.x) {
    sm.Thi[i] = 0.f;
    sm.Tlo[i] = 0.f;
  }
  if (warp == 0) tmemAlloc(&sm.tmemSlot, kCols3);
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = sm.tmemSlot;
  const uint32_t tHi = smemAddr(sm.Thi), tLo = smemAddr(sm.Tlo);
  const uint32_t half = 128 / 8 * 1024;  // byte offset of row 128 in a tile
  uint32_t phase = 0;
  int mapPatch = -1;
  bool ctrlOut = false;
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
    mbarExpectTx(ctrlbar, kCtrlBytes3);
    tmaLoad4d(smemAddr(sm.ctrlT), tm, 0, f1, f2, f3, ctrlbar);
    ctrlOut = true;
  };
  if (tid == 0 && (int)blockIdx.x < count) stageCtrl(blockIdx.x);
  uint32_t cphase = 0;
  Item nextItem{};
  if ((int)blockIdx.x < count) nextItem = items[blockIdx.x];

  for (int it = blockIdx.x; it < count; it += gridDim.x) {
    const Item item = nextItem;
    const DevPatch& P = patches[item.patch];
    const int e = item.elem;
    const int e1 = e % P.nel[0], e2 = (e / P.nel[0]) % P.nel[1], e3 = e / (P.nel[0] * P.nel[1]);

    // ---- 1. control points (TMA box), weighted net, 1D tables, span volume
    double dV = 0.0;
    if (tid == 192) dV = P.span[0][e1] * P.span[1][e2] * P.span[2][e3];
    float tbv = 0.f;
    if (tid < 96) {
      const int d = tid / 32, dd = (tid / 16) & 1, g = tid % 16;
      tbv = (dd ? P.tabDf[d] : P.tabNf[d])[(d == 0 ? e1 : d == 1 ? e2 : e3) * 16 + g];
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
    if (tid < 96) sm.tb[tid / 32][(tid / 16) & 1][tid % 16] = tbv;
    if (tid == 192) {
      sm.signs = 0;
      sm.dVf = (float)(0.125 * dV);
    }
    __syncthreads();
    if (sm.fail) break;
    if (tid == 0 && it + (int)gridDim.x < count) stageCtrl(it + gridDim.x);

    // ---- 2. homogeneous sums at the Gauss points by sum factorisation
    for (int t = tid; t < 2 * 4 * 4 * 16; t += blockDim.x) {        // x: [N/D][c][gx][j + 4k]
      const int jk = t % 16, gx = (t / 16) % 4, c = (t / 64) % 4, dd = t / 256;
      const float* tbx = sm.tb[0][dd] + gx * 4;
      const float* w = F.wX[c] + 4 * jk;
      (&F.A[0][0][0][0])[t] = fmaf(tbx[0], w[0], fmaf(tbx[1], w[1], fmaf(tbx[2], w[2], tbx[3] * w[3])));
    }
    __syncthreads();
    for (int t = tid; t < 3 * 4 * 16 * 4; t += blockDim.x) {       // y: [NN/DN/ND][c][gx + 4gy][k]
      const int k = t % 4, gxy = (t / 4) % 16, c = (t / 64) % 4, v = t / 256;
      const int gx = gxy % 4, gy = gxy / 4;
      const float* tby = sm.tb[1][v == 2] + gy * 4;
      const float* a = F.A[v == 1][c][gx] + 4 * k;
      (&F.B[0][0][0][0])[t] = fmaf(tby[0], a[0], fmaf(tby[1], a[1], fmaf(tby[2], a[2], tby[3] * a[3])));
    }
    __syncthreads();
    for (int t = tid; t < kNq * 16; t += blockDim.x) {              // z: S[q][c][d]
      const int d = t % 4, c = (t / 4) % 4, q = t / 16;
      const int gxy = q % 16, gz = q / 16;
      const int src = d == 1 ? 1 : d == 2 ? 2 : 0;
      const float* tbz = sm.tb[2][d == 3] + gz * 4;
      const float* b = F.B[src][c][gxy];
      (&F.S[0][0][0])[t] = fmaf(tbz[0], b[0], fmaf(tbz[1], b[1], fmaf(tbz[2], b[2], tbz[3] * b[3])));
    }
    __syncthreads();

    // ---- 3. per Gauss point: Jacobian, FP64 cofactors and determinant
    if (tid < kNq) {
      const int q = tid;
      const float* Sq = F.S[q][0];
      const float iW = 1.f / Sq[12];
      double J[9];  // J[d*3 + r] = dX_r/du_d, FP32 sums widened exactly
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
      float B[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // du_d/dx_k at 3k + d
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
        w = detf * sm.dVf * P.gwf[0][q % 4] * P.gwf[1][(q / 4) % 4] * P.gwf[2][q / 16];
        atomicOr(&sm.signs, w > 0.f ? 1 : 2);
      } else {
        atomicAdd(S.counters, 1ull);
      }
      sm.wq[q] = w;
      F.iW[q] = iW;
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

    // ---- 4. operand chunks and the two tensor-core blocks, per weight sign
    const int signs = sm.signs;
    bool first = true, ok = true;
    for (int pass = 0; pass < 2 && ok; pass++) {
      const float s = pass == 0 ? 1.f : -1.f;
      if (!(signs & (1 << pass))) continue;
      for (int t = tid; t < kNq * 12; t += blockDim.x) {
        const float ws = s * sm.wq[t / 12];
        (&F.Es[0][0])[t] = (ws > 0.f ? sqrtf(ws) : 0.f) * (&F.E[0][0])[t];
      }
      __syncthreads();
      for (int ch = 0; ch < 2 && ok; ch++) {
        if (!first) {  // the previous MMAs must have read the tiles
          ok = mbarWait(mbar, phase);
          phase ^= 1u;
          tcFenceAfter();
          if (!ok) break;
        }
        // task (a, g): function a, Gauss points 32 ch + 4g .. +3
        for (int task = tid; task < kNen * 8; task += blockDim.x) {
          const int a = task % kNen, g = task / kNen;
          const int ia = a % 4, ja = (a / 4) % 4, ka = a / 16;
          const float wa = sm.X[a][3];
          float hi[3][4], lo[3][4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const int q = 32 * ch + 4 * g + u;
            const int gx = q % 4, gy = (q / 4) % 4, gz = q / 16;
            const float nx = sm.tb[0][0][4 * gx + ia], dx = sm.tb[0][1][4 * gx + ia];
            const float ny = sm.tb[1][0][4 * gy + ja], dy = sm.tb[1][1][4 * gy + ja];
            const float nz = sm.tb[2][0][4 * gz + ka], dz = sm.tb[2][1][4 * gz + ka];
            const float nyz = wa * ny * nz;
            const float du = dx * nyz, dv = wa * nx * dy * nz, dw = wa * nx * ny * dz;
            const float n = nx * nyz;
            const float4 E0 = *reinterpret_cast<const float4*>(F.Es[q]);
            const float4 E1 = *reinterpret_cast<const float4*>(F.Es[q] + 4);
            const float4 E2 = *reinterpret_cast<const float4*>(F.Es[q] + 8);
            const float t0 = fmaf(du, E0.x, fmaf(dv, E0.y, fmaf(dw, E0.z, -n * E2.y)));
            const float t1 = fmaf(du, E0.w, fmaf(dv, E1.x, fmaf(dw, E1.y, -n * E2.z)));
            const float t2 = fmaf(du, E1.z, fmaf(dv, E1.w, fmaf(dw, E2.x, -n * E2.w)));
            splitTF32(t0, hi[0][u], lo[0][u]);
            splitTF32(t1, hi[1][u], lo[1][u]);
            splitTF32(t2, hi[2][u], lo[2][u]);
          }
#pragma unroll
          for (int k = 0; k < 3; k++) {
            const int o = kmaj(64 * k + a, 4 * g);
            *reinterpret_cast<float4*>(sm.Thi + o) = make_float4(hi[k][0], hi[k][1], hi[k][2], hi[k][3]);
            *reinterpret_cast<float4*>(sm.Tlo + o) = make_float4(lo[k][0], lo[k][1], lo[k][2], lo[k][3]);
          }
        }
        fenceProxyAsync();
        __syncthreads();
        if (tid == 0) {
          tcFenceAfter();
          const uint32_t neg = s < 0.f ? (1u << 13) : 0u;
          const uint32_t id1 = instrDescTF32(128, 192) | neg, id2 = instrDescTF32(128, 64) | neg;
          for (int st = 0; st < kK / 8; st++) {
            const uint32_t off = st * 256;
            const uint32_t acc = first ? 0u : 1u;
            mmaTF32(tmem, smemDesc(tHi + off), smemDesc(tHi + off), id1, acc);
            mmaTF32(tmem, smemDesc(tHi + off), smemDesc(tLo + off), id1, 1);
            mmaTF32(tmem, smemDesc(tLo + off), smemDesc(tHi + off), id1, 1);
            mmaTF32(tmem + 192, smemDesc(tHi + half + off), smemDesc(tHi + half + off), id2, acc);
            mmaTF32(tmem + 192, smemDesc(tHi + half + off), smemDesc(tLo + half + off), id2, 1);
            mmaTF32(tmem + 192, smemDesc(tLo + half + off), smemDesc(tHi + half + off), id2, 1);
            first = false;
          }
          mmaCommit(mbar);
        }
        first = false;
      }
    }
    if (ok && !first) {  // the last chunk's MMAs
      ok = mbarWait(mbar, phase);
      phase ^= 1u;
      tcFenceAfter();
    }
    if (!ok && tid == 0) {
      atomicAdd(S.counters + 2, 1ull);
      sm.fail = 1;
    }

    // ---- 5. element load vector: body force, Neumann traction
    float fe = 0.f;
    if (tid < kNen * 3) {
      const int a = tid / 3, k = tid % 3;
      const float bk = P.bodyf[k];
      if (bk != 0.f) {
        const int ia = a % 4, ja = (a / 4) % 4, ka = a / 16;
        float acc = 0.f;
        for (int q = 0; q < kNq; q++) {
          const float n = sm.tb[0][0][4 * (q % 4) + ia] * sm.tb[1][0][4 * ((q / 4) % 4) + ja] *
                          sm.tb[2][0][4 * (q / 16) + ka];
          acc = fmaf(n * F.iW[q], sm.wq[q], acc);
        }
        fe = bk * sm.X[a][3] * acc;
      }
    }
    // constant traction t: Fe += t R dS w at the 4x4 face points (face
    // overload of ASMs3D::integrate, src/ASM/ASMs3D.C:2547-2812)
    for (int f = 0; f < P.nneu; f++) {
      const int face = P.neuFace[f];
      const int nd0 = (face - 1) >> 1, side = (face - 1) & 1;
      const int ee[3] = {e1, e2, e3};
      if (ee[nd0] != (side ? P.nel[nd0] - 1 : 0)) continue;  // uniform in the CTA
      float* fR = F.face;             // [16][64] rational basis at the face points
      float* fW = F.face + 16 * kNen; // [16] dS * weights
      if (tid < 16) {
        const int ta = nd0 == 0 ? 1 : 0, tb = nd0 == 2 ? 1 : 2;
        int g[3] = {0, 0, 0};
        g[ta] = tid % 4;
        g[tb] = tid / 4;
        float Nd[3][4], Dd[3][4];
        for (int d = 0; d < 3; d++)
          for (int r = 0; r < 4; r++) {
            if (d == nd0) {
              Nd[d][r] = (float)P.tabB[d][side * 8 + r];
              Dd[d][r] = (float)P.tabB[d][side * 8 + 4 + r];
            } else {
              Nd[d][r] = P.tabNf[d][ee[d] * 16 + g[d] * 4 + r];
              Dd[d][r] = P.tabDf[d][ee[d] * 16 + g[d] * 4 + r];
            }
          }
        float S4[4][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f},
                          {0.f, 0.f, 0.f, 0.f}};
        for (int a = 0; a < kNen; a++) {
          const int i = a % 4, j = (a / 4) % 4, k = a / 16;
          const float w = sm.X[a][3];
          const float wN = w * Nd[0][i] * Nd[1][j] * Nd[2][k];
          const float w0 = w * Dd[0][i] * Nd[1][j] * Nd[2][k];
          const float w1 = w * Nd[0][i] * Dd[1][j] * Nd[2][k];
          const float w2 = w * Nd[0][i] * Nd[1][j] * Dd[2][k];
          fR[tid * kNen + a] = wN;
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
        for (int a = 0; a < kNen; a++) fR[tid * kNen + a] *= iW;
        fW[tid] = wgt;
      }
      __syncthreads();
      if (tid < kNen * 3) {
        const int a = tid / 3, c = tid % 3;
        float acc = 0.f;
        for (int gq = 0; gq < 16; gq++) acc = fmaf(fR[gq * kNen + a], fW[gq], acc);
        fe = fmaf(P.neuT[f][c], acc, fe);
      }
      __syncthreads();
    }
    if (tid < kNen * 3) sm.fe[tid] = fe;
    __syncthreads();
    if (sm.fail) break;
    if (it + (int)gridDim.x < count) nextItem = items[it + gridDim.x];

    // ---- 6. tensor memory -> element block: every entry with c >= r at
    //         (r, c) and its mirror (c, r); warps 0..3 block 1, warps 4, 5
    //         block 2, warps 6, 7 the load vector.  With S.upper the gather
    //         reads only the node pairs b >= a of each row block (a row
    //         (a, k), columns (b, l)), so only those positions are written:
    //         half the stores
    float* blk = P.elm + (size_t)e * P.elmStride;
    if (warp < 4) {
      const int r = 32 * warp + lane, k = r >> 6, a = r & 63;
      float* rowOut = blk + (size_t)((3 * a + k) * 3) * 64;  // G[a][k][0][0]
      for (int c16 = 4 * k; c16 < 12; c16++) {  // blocks l < k: written by their mirrors
        float v[16];
        if (signs) tmemLoad16(tmem + ((uint32_t)(32 * warp) << 16) + 16 * c16, v);
        else
#pragma unroll
          for (int i = 0; i < 16; i++) v[i] = 0.f;
        const int l = c16 >> 2, b0 = (c16 & 3) * 16;
        const bool full = l > k && (!S.upper || b0 >= a);  // the 16 direct values, 16-byte stores
        if (full) {
#pragma unroll
          for (int i = 0; i < 16; i += 4)
            *reinterpret_cast<float4*>(rowOut + l * 64 + b0 + i) =
                make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        }
#pragma unroll
        for (int i = 0; i < 16; i++) {
          const int b = b0 + i;
          if (!full && b >= a && l >= k) rowOut[l * 64 + b] = v[i];
          if ((l > k || b > a) && (!S.upper || b <= a))
            blk[(size_t)((3 * b + l) * 3 + k) * 64 + a] = v[i];
        }
      }
    } else if (warp < 6) {
      const int a = 32 * (warp - 4) + lane;  // row 128 + a: k = 2
      float* rowOut = blk + (size_t)((3 * a + 2) * 3 + 2) * 64;
      for (int c16 = 0; c16 < 4; c16++) {
        float v[16];
        if (signs) tmemLoad16(tmem + ((uint32_t)(32 * (warp - 4)) << 16) + 192 + 16 * c16, v);
        else
#pragma unroll
          for (int i = 0; i < 16; i++) v[i] = 0.f;
#pragma unroll
        for (int i = 0; i < 16; i++) {
          const int b = 16 * c16 + i;
          if (b >= a) rowOut[b] = v[i];
          if (b > a && !S.upper) blk[(size_t)((3 * b + 2) * 3 + 2) * 64 + a] = v[i];
        }
      }
    } else {
      for (int i = tid - 192; i < kNen * 3; i += 64) blk[64 * 9 * 64 + i] = sm.fe[i];
    }
    tcFenceBefore();
    __syncthreads();  // tensor memory read before the next element's MMAs
    tcFenceAfter();
  }
  if (tid == 0 && ctrlOut) mbarWait(ctrlbar, cphase, S.mbarSpin);
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (warp == 0) tmemDealloc(tmem, kCols3);
}

// ---------------------------------------------------------------------------
// host side

bool tcElast3Supports(const DevPatch& P)
{
  return P.dim == 3 && P.kind == IFEMGPU_ELASTICITY && P.npv == 3 && P.p[0] == 3 &&
         P.p[1] == 3 && P.p[2] == 3 && P.ng[0] == 4 && P.ng[1] == 4 && P.ng[2] == 4;
}

size_t tcElast3Smem() { return sizeof(E3Smem); }

ifemgpu_status tcElast3Prepare(ifemgpu_ctx* ctx)
{
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_volume_tc_elast_p3,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(E3Smem)));
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_volume_tc_elast_p3,
                                         cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared));
  return IFEMGPU_OK;
}

ifemgpu_status tcElast3Launch(ifemgpu_ctx* ctx, const Pass& p)
{
  // without prescribed values the gather of this class sums each node pair
  // once (half mode) and reads only the pairs b >= a
  Tc3Sys S{ctx->d_counters, ctx->dbg.mbarSpin ? ctx->dbg.mbarSpin : kSpinLimit, ctx->dbg.patch,
           ctx->dbg.elem, ctx->nceq == 0 ? 1 : 0};
  // two CTAs per SM (2 x 256 tensor-memory columns, shared memory)
  const int grid = std::min(p.count, 2 * ctx->numSMs);
  const DevPatch* patches = ctx->d_patches;
  const Item* items = ctx->d_items + p.first;
  int count = p.count;
  void* args[] = {(void*)&patches, (void*)&items, (void*)&count, (void*)&S};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kThreads3);
  cfg.dynamicSmemBytes = sizeof(E3Smem);
  cfg.stream = ctx->stream;
  IFEMGPU_CUDA(ctx, cudaLaunchKernelExC(&cfg, (const void*)k_volume_tc_elast_p3, args));
  return IFEMGPU_OK;
}

}  // namespace ifemgpu
