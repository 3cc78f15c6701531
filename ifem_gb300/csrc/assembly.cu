// assembly.cu -- element integration and scatter kernels of libifemgpu.
//
// Data flow of one assembly (ifemgpu_assemble):
//   1. k_basis_tables   1D B-spline values/derivatives at the Gauss points of
//                       every knot span (Cox-de Boor, FP64), per patch and
//                       direction -- the GPU replacement of IFEM's
//                       BasisFunctionCache (src/ASM/ASMs3D.C:3996-4143).
//   2. volume passes    tensor-core patches: one element-kernel launch per
//                       kernel class (tc_volume.cu, tc_poisson.cu,
//                       tc_elast3.cu), each element's FP32 matrix and load
//                       vector written to the element scratch, then one
//                       node-wise gather per (degree, field) class
//                       (gather.cu) that sums them into the matrix in a fixed
//                       order.  Other patches (2D, p other than 2/3, mass
//                       terms, repeated knots, the FP64 mode): the generic
//                       kernels below, one launch per element colour or one
//                       persistent colour-major launch ordered by done flags;
//                       elements of one colour share no node, so the sum
//                       order is fixed (deterministic).  Replaces the element
//                       loop of ASMs3D::integrate (src/ASM/ASMs3D.C:2118-2325)
//                       and the scatter of assemSparse
//                       (src/LinAlg/SparseMatrix.C:614-688).
//   3. face passes      Neumann (traction / flux) integration on the faces of
//                       generic patches (src/ASM/ASMs3D.C:2547-2812), colour
//                       by colour; tensor-core elasticity kernels integrate
//                       their tractions in the element kernel.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "ifemgpu_internal.h"
#include "tc_common.cuh"

namespace ifemgpu {

namespace {

// ---------------------------------------------------------------------------
// Gauss-Legendre rule on [-1,1] (ascending), Newton iteration on P_n.
void gaussRule(int n, double* x, double* w)
{
  for (int i = 0; i < (n + 1) / 2; i++) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; k++) {
        double pk = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      if (n == 1) { p0 = 1.0; p1 = z; }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; k++) {
      double pk = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
      p0 = p1;
      p1 = pk;
    }
    if (n == 1) { p0 = 1.0; p1 = z; }
    dp = n * (z * p1 - p0) / (z * z - 1.0);
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
  if (n % 2) x[n / 2] = 0.0;
}

}  // namespace

void gaussLegendre(int n, double* x, double* w) { gaussRule(n, x, w); }

namespace {

int gaussCount(int nGauss, int order, bool neumann)
{
  // ASMbase::getNoGaussPt semantics (src/ASM/ASMbase.C:1788-1798)
  if (nGauss <= -order) return 0;
  if (nGauss > 0 && nGauss < 11) return nGauss;
  if (neumann) return order;
  return order + nGauss % 10;
}

}  // namespace

// ---------------------------------------------------------------------------
// Device Cox-de Boor: values N[0..p] and first derivatives D[0..p] of the
// degree-p B-splines that are non-zero on span k (U[k] <= u < U[k+1]).
__device__ void bsplineDers(const double* __restrict__ U, int p, int k, double u,
                            double* N, double* D)
{
  double left[kMaxDeg + 1], right[kMaxDeg + 1], lo[kMaxDeg + 1];
  N[0] = 1.0;
  for (int j = 1; j <= p; j++) {
    if (j == p) {
      for (int r = 0; r < p; r++) lo[r] = N[r];  // degree p-1 values
    }
    left[j] = u - U[k + 1 - j];
    right[j] = U[k + j] - u;
    double saved = 0.0;
    for (int r = 0; r < j; r++) {
      double temp = N[r] / (right[r + 1] + left[j - r]);
      N[r] = saved + right[r + 1] * temp;
      saved = left[j - r] * temp;
    }
    N[j] = saved;
  }
  if (p == 0) { D[0] = 0.0; return; }
  // d/du N_{i,p} = p (N_{i,p-1}/(U_{i+p}-U_i) - N_{i+1,p-1}/(U_{i+p+1}-U_{i+1}))
  for (int r = 0; r <= p; r++) {
    const int i = k - p + r;
    double a = 0.0, b = 0.0;
    if (r >= 1) {
      double den = U[i + p] - U[i];
      a = den > 0.0 ? lo[r - 1] / den : 0.0;
    }
    if (r <= p - 1) {
      double den = U[i + p + 1] - U[i + 1];
      b = den > 0.0 ? lo[r] / den : 0.0;
    }
    D[r] = p * (a - b);
  }
}

// 1D tables of one patch: thread per (direction, span, Gauss point).
__device__ void basisItem(const DevPatch& P, int t)
{
  for (int d = 0; d < P.dim; d++) {
    const int cnt = P.nel[d] * P.ng[d];
    if (t < cnt) {
      const int e = t / P.ng[d], g = t % P.ng[d];
      const double* U = P.knots[d];
      const int k = P.p[d] + e;
      const double u0 = U[k], u1 = U[k + 1];
      const double u = 0.5 * ((u1 - u0) * P.gx[d][g] + u1 + u0);
      double N[kMaxDeg + 1], D[kMaxDeg + 1];
      bsplineDers(U, P.p[d], k, u, N, D);
      double* tn = P.tabN[d] + (size_t)t * (P.p[d] + 1);
      double* td = P.tabD[d] + (size_t)t * (P.p[d] + 1);
      for (int r = 0; r <= P.p[d]; r++) { tn[r] = N[r]; td[r] = D[r]; }
      if (P.tabNf[d]) {
        float* fn = P.tabNf[d] + (size_t)t * (P.p[d] + 1);
        float* fd = P.tabDf[d] + (size_t)t * (P.p[d] + 1);
        for (int r = 0; r <= P.p[d]; r++) { fn[r] = (float)N[r]; fd[r] = (float)D[r]; }
      }
      if (g == 0) P.span[d][e] = u1 - u0;
      return;
    }
    t -= cnt;
  }
  // boundary tables: the first and last span evaluated at the patch ends
  if (t < 2 * P.dim) {
    const int d = t >> 1, side = t & 1;
    const double* U = P.knots[d];
    const int k = side ? P.n[d] - 1 : P.p[d];
    const double u = side ? U[P.n[d]] : U[P.p[d]];
    double N[kMaxDeg + 1], D[kMaxDeg + 1];
    bsplineDers(U, P.p[d], k, u, N, D);
    double* tb = P.tabB[d] + side * 2 * (P.p[d] + 1);
    for (int r = 0; r <= P.p[d]; r++) {
      tb[r] = N[r];
      tb[P.p[d] + 1 + r] = D[r];
    }
  }
}

// every patch's tables in one launch: item t of the concatenated work lists
// belongs to the last patch whose start[] is <= t
__global__ void k_basis_tables(const DevPatch* __restrict__ patches, const int* __restrict__ start,
                               int np)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= start[np]) return;
  int lo = 0, hi = np - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  basisItem(patches[lo], t - start[lo]);
}

// ---------------------------------------------------------------------------
// FP64 volume kernel: one CTA per element of one colour.
//
// Shared memory (doubles): Xn[nen*4] | N[nq*nen] | dX[3][nq*nen] | Jinv[nq*9]
//                          | wq[nq] | kq[nq] | fq[nq]   then  eq[nd] (int)
__device__ inline int elemNode(const DevPatch& P, int e, int a)
{
  const int q1 = P.p[0] + 1, q2 = P.p[1] + 1;
  const int e1 = e % P.nel[0], e2 = (e / P.nel[0]) % P.nel[1], e3 = e / (P.nel[0] * P.nel[1]);
  const int i = a % q1, j = (a / q1) % q2, k = a / (q1 * q2);
  return ((e3 + k) * P.n[1] + e2 + j) * P.n[0] + e1 + i;
}

// Position of row `r` (0-based) in column `c` (0-based) of the CSC pattern.
__device__ inline int findRow(const int* __restrict__ colptr, const int* __restrict__ rowidx,
                              int c, int r)
{
  int lo = colptr[c], hi = colptr[c + 1] - 1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    int v = rowidx[mid];
    if (v == r) return mid;
    if (v < r) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

struct SysView {
  const int* madof;
  const int* meqn;
  const double* c0;
  const int* colptr;
  const int* rowidx;
  double* K;
  double* b;
  unsigned long long* counters;  // [0] singular points [1] pattern misses [2] timeouts [3] work
  const int* F;  // free DOFs before each node
  int* flags;    // per-element done flags of the persistent pass
  unsigned flagSpin;  // polls per flag wait
  int withhold;       // flag slot that is never published (test hook), -1 none
};

constexpr uint32_t kGenFlagSpin = 1u << 20;  // x 64 ns sleeps: about 0.1 s per wait

// flags are polled with relaxed loads (served by L2); a thread that saw a
// flag issues one acquire fence before the block's scatter
__device__ __forceinline__ int genLoadRelaxed(const int* p)
{
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void genFenceAcquire()
{
  asm volatile("fence.acq_rel.gpu;" : : : "memory");
}

__device__ __forceinline__ void genStoreRelease(int* p, int v)
{
  asm volatile("st.release.gpu.global.b32 [%0], %1;" : : "l"(p), "r"(v) : "memory");
}

// Generic element kernel, one CTA per element of one colour; T = double is
// the exact-parity mode (FP64 arithmetic, plain adds: no two CTAs of a colour
// touch one entry), T = float the split mode on the CUDA cores (FP32
// arithmetic, FP64 determinant/inverse, FP64 additions in L2 reductions).
// Node pairs a <= b are computed once; the (b, a) block is the transpose.
//
// Shared memory (T): Xn[nen*4] | N[nq*nen] | dX[3][nq*nen] | Jinv[nq*9]
//                    | wq[nq] | kq[nq] | fq[nq]   then  eq[nd] (int)
// FP64 values: plain adds within a colour pass (no two elements of a colour
// share an entry), L2 reductions in the persistent pass (ordered by flags);
// FP32 values: widened exactly and added by L2 reductions.
__device__ __forceinline__ void addEntry(double* p, double v, bool red)
{
  if (red) atomicAdd(p, v);
  else *p += v;
}
__device__ __forceinline__ void addEntry(double* p, float v, bool)
{
  atomicAdd(p, tc::widenF32(v));
}

template <typename V>
__device__ __forceinline__ V warpAllSum(V v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// 1D basis tables in the element kernel's precision
template <typename T> __device__ __forceinline__ const T* tableN(const DevPatch& P, int d);
template <typename T> __device__ __forceinline__ const T* tableD(const DevPatch& P, int d);
template <> __device__ __forceinline__ const double* tableN<double>(const DevPatch& P, int d) { return P.tabN[d]; }
template <> __device__ __forceinline__ const double* tableD<double>(const DevPatch& P, int d) { return P.tabD[d]; }
template <> __device__ __forceinline__ const float* tableN<float>(const DevPatch& P, int d) { return P.tabNf[d]; }
template <> __device__ __forceinline__ const float* tableD<float>(const DevPatch& P, int d) { return P.tabDf[d]; }

// Waits until every lower-colour neighbour of element e (the elements within
// p spans in each direction share nodes with it) has published its flag.
// Bounded: a wait that runs out counts in counters[2] and lets the element go
// on (the host then reports IFEMGPU_DEVICE_TIMEOUT).
__device__ void waitNeighbours(const DevPatch& P, int e, const SysView& S)
{
  const int q[3] = {P.p[0] + 1, P.p[1] + 1, P.dim == 3 ? P.p[2] + 1 : 1};
  const int w[3] = {2 * P.p[0] + 1, 2 * P.p[1] + 1, P.dim == 3 ? 2 * P.p[2] + 1 : 1};
  const int ee[3] = {e % P.nel[0], (e / P.nel[0]) % P.nel[1], e / (P.nel[0] * P.nel[1])};
  const int myc = ee[0] % q[0] + q[0] * (ee[1] % q[1] + q[1] * (ee[2] % q[2]));
  const int total = w[0] * w[1] * w[2];
  bool waited = false;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int f[3] = {ee[0] + t % w[0] - P.p[0], ee[1] + (t / w[0]) % w[1] - P.p[1],
                      ee[2] + (P.dim == 3 ? t / (w[0] * w[1]) - P.p[2] : 0)};
    bool inside = true;
    for (int d = 0; d < 3; d++) inside = inside && f[d] >= 0 && f[d] < P.nel[d];
    if (!inside) continue;
    const int nc = f[0] % q[0] + q[0] * (f[1] % q[1] + q[1] * (f[2] % q[2]));
    if (nc >= myc) continue;  // the element itself and later colours
    const int* flag = S.flags + P.flagBase + (f[2] * P.nel[1] + f[1]) * P.nel[0] + f[0];
    uint32_t spin = 0;
    waited = true;
    while (genLoadRelaxed(flag) == 0) {
      if (++spin > S.flagSpin) {
        atomicAdd(S.counters + 2, 1ull);
        break;
      }
      __nanosleep(64);
    }
  }
  if (waited) genFenceAcquire();
}

// FP32 Poisson element matrix in TS x TS register tiles of node pairs
// (ta <= tb): Ke[a][b] = sum over (Gauss point, direction) of kq dX_a dX_b,
// scattered as the (a, b) block and its transpose.
template <int TS>
__device__ void poissonTiles(const DevPatch& P, const SysView& S, const float* dX,
                             const float* kq, const int* eq, const int* nodeA, const int* Fa)
{
  const int nen = P.nen, nq = P.nq, dim = P.dim;
  const int q1 = P.p[0] + 1, q2 = P.p[1] + 1;
  const int nt = (nen + TS - 1) / TS, ntp = nt * (nt + 1) / 2;
  for (int t = threadIdx.x; t < ntp; t += blockDim.x) {
    int tb = (int)((sqrtf(8.f * t + 1.f) - 1.f) * 0.5f);
    while (tb * (tb + 1) / 2 > t) tb--;
    while ((tb + 1) * (tb + 2) / 2 <= t) tb++;
    const int ta = t - tb * (tb + 1) / 2;
    // functions past nen are clamped to the last one; their sums are dropped
    int ia[TS], ib[TS];
#pragma unroll
    for (int i = 0; i < TS; i++) {
      ia[i] = min(TS * ta + i, nen - 1);
      ib[i] = min(TS * tb + i, nen - 1);
    }
    float acc[TS][TS];
#pragma unroll
    for (int i = 0; i < TS; i++)
#pragma unroll
      for (int j = 0; j < TS; j++) acc[i][j] = 0.f;
    for (int c = 0; c < dim; c++) {
      const float* plane = dX + c * nq * nen;
      for (int q = 0; q < nq; q++) {
        const float* row = plane + q * nen;
        const float s = kq[q];
        float va[TS], vb[TS];
#pragma unroll
        for (int i = 0; i < TS; i++) {
          va[i] = row[ia[i]] * s;
          vb[i] = row[ib[i]];
        }
#pragma unroll
        for (int i = 0; i < TS; i++)
#pragma unroll
          for (int j = 0; j < TS; j++) acc[i][j] = fmaf(va[i], vb[j], acc[i][j]);
      }
    }
#pragma unroll
    for (int i = 0; i < TS; i++)
#pragma unroll
      for (int j = 0; j < TS; j++) {
        const int a = TS * ta + i, bn = TS * tb + j;
        if (a >= nen || bn >= nen || a > bn) continue;
        for (int side = 0; side < (a == bn ? 1 : 2); side++) {
          const int ra = side ? bn : a, cb = side ? a : bn;
          const int r = eq[ra], ce = eq[cb];
          if (r <= 0 || ce <= 0) continue;
          int off;
          if (P.lineOff) {
            const int w1 = 2 * P.p[1] + 1, w2 = 2 * P.p[2] + 1;
            const int dy = (ra / q1) % q2 - (cb / q1) % q2, dz = ra / (q1 * q2) - cb / (q1 * q2);
            off = P.lineOff[(size_t)nodeA[cb] * w1 * w2 + (dz + P.p[2]) * w1 + dy + P.p[1]] +
                  Fa[ra];
          } else {
            const int pos0 = findRow(S.colptr, S.rowidx, ce - 1, r - 1);
            if (pos0 < 0) { atomicAdd(S.counters + 1, 1ull); continue; }
            off = pos0 - S.colptr[ce - 1];
          }
          atomicAdd(S.K + S.colptr[ce - 1] + off, tc::widenF32(acc[i][j]));
        }
      }
  }
}

// One element: basis, geometry, element matrix and load, scatter.  With
// kFlow the element waits for its lower-colour neighbours before it
// scatters and publishes its own done flag afterwards.
template <typename T, bool kFlow>
__device__ void volumeElement(const DevPatch& P, const Item it, const SysView& S,
                              unsigned char* smraw)
{
  T* sm = reinterpret_cast<T*>(smraw);
  const int nen = P.nen, nq = P.nq, dim = P.dim, npv = P.npv, nd = nen * npv;
  const int e = it.elem;
  T* Xn = sm;
  T* Nq = Xn + nen * 4;
  T* dX = Nq + nq * nen;          // 3 planes of nq*nen
  T* Ji = dX + 3 * nq * nen;      // nq * 9
  T* wq = Ji + nq * 9;
  T* kq = wq + nq;
  T* fq = kq + nq;
  double* gsum = reinterpret_cast<double*>(fq + nq);  // per point: log-kappa, noise sums
  int* eq = reinterpret_cast<int*>(gsum + 2 * nq);
  int* nodeA = eq + nd;     // patch-local node of each element function
  int* Fa = nodeA + nen;    // free DOFs before that node
  const int e1 = e % P.nel[0], e2 = (e / P.nel[0]) % P.nel[1], e3 = e / (P.nel[0] * P.nel[1]);
  const int q1 = P.p[0] + 1, q2 = P.p[1] + 1;
  const double* c00 = P.ctrl + (size_t)elemNode(P, e, 0) * 4;

  // element nodes: coordinates (relative to the first node) and equation numbers
  for (int a = threadIdx.x; a < nen; a += blockDim.x) {
    const int node = elemNode(P, e, a);
    for (int c = 0; c < 3; c++) Xn[a * 4 + c] = (T)(P.ctrl[(size_t)node * 4 + c] - c00[c]);
    Xn[a * 4 + 3] = (T)P.ctrl[(size_t)node * 4 + 3];
    const int g = globalNode(P, node);
    const int d0 = S.madof[g] - 1;
    for (int c = 0; c < npv; c++) eq[a * npv + c] = S.meqn[d0 + c];
    nodeA[a] = node;
    Fa[a] = S.F[g];
  }
  __syncthreads();

  // tensor-product basis at every (Gauss point, function), from the 1D
  // tables in the kernel's precision
  for (int t = threadIdx.x; t < nq * nen; t += blockDim.x) {
    const int q = t / nen, a = t % nen;
    const int gi = q % P.ng[0], gj = (q / P.ng[0]) % P.ng[1], gk = q / (P.ng[0] * P.ng[1]);
    const int i = a % q1, j = (a / q1) % q2, k = a / (q1 * q2);
    const T* n0 = tableN<T>(P, 0) + ((size_t)e1 * P.ng[0] + gi) * q1;
    const T* d0 = tableD<T>(P, 0) + ((size_t)e1 * P.ng[0] + gi) * q1;
    const T* n1 = tableN<T>(P, 1) + ((size_t)e2 * P.ng[1] + gj) * q2;
    const T* d1 = tableD<T>(P, 1) + ((size_t)e2 * P.ng[1] + gj) * q2;
    T N, du, dv, dw = 0;
    if (dim == 3) {
      const int q3 = P.p[2] + 1;
      const T* n2 = tableN<T>(P, 2) + ((size_t)e3 * P.ng[2] + gk) * q3;
      const T* d2 = tableD<T>(P, 2) + ((size_t)e3 * P.ng[2] + gk) * q3;
      N = n0[i] * n1[j] * n2[k];
      du = d0[i] * n1[j] * n2[k];
      dv = n0[i] * d1[j] * n2[k];
      dw = n0[i] * n1[j] * d2[k];
    } else {
      N = n0[i] * n1[j];
      du = d0[i] * n1[j];
      dv = n0[i] * d1[j];
    }
    Nq[t] = N;
    dX[t] = du;
    dX[nq * nen + t] = dv;
    dX[2 * nq * nen + t] = dw;
  }
  __syncthreads();

  // per Gauss point, one warp each (lanes over the basis functions, sums by
  // butterfly shuffles): rational weighting, Jacobian, material sums; lane 0
  // forms the FP64 determinant and inverse
  const int lane = threadIdx.x & 31;
  for (int q = threadIdx.x >> 5; q < nq; q += blockDim.x >> 5) {
    T* Nr = Nq + q * nen;
    T* Du = dX + q * nen;
    T* Dv = dX + nq * nen + q * nen;
    T* Dw = dX + 2 * nq * nen + q * nen;
    if (P.rational) {
      T W = 0, Wu = 0, Wv = 0, Ww = 0;
      for (int a = lane; a < nen; a += 32) {
        const T w = Xn[a * 4 + 3];
        W += w * Nr[a];
        Wu += w * Du[a];
        Wv += w * Dv[a];
        Ww += w * Dw[a];
      }
      W = warpAllSum(W);
      Wu = warpAllSum(Wu);
      Wv = warpAllSum(Wv);
      Ww = warpAllSum(Ww);
      for (int a = lane; a < nen; a += 32) {
        const T w = Xn[a * 4 + 3];
        const T R = w * Nr[a] / W;
        Du[a] = (w * Du[a] - R * Wu) / W;
        Dv[a] = (w * Dv[a] - R * Wv) / W;
        Dw[a] = (w * Dw[a] - R * Ww) / W;
        Nr[a] = R;
      }
      __syncwarp();
    }
    T Jt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // column-major J(r,c) = dX_r/du_c
    T Xt[3] = {0, 0, 0};
    T gk = 0, sn = 0;                        // log-conductivity and noise sums
    for (int a = lane; a < nen; a += 32) {
      const T x = Xn[a * 4], y = Xn[a * 4 + 1], z = Xn[a * 4 + 2];
      Jt[0] += x * Du[a]; Jt[1] += y * Du[a]; Jt[2] += z * Du[a];
      Jt[3] += x * Dv[a]; Jt[4] += y * Dv[a]; Jt[5] += z * Dv[a];
      Jt[6] += x * Dw[a]; Jt[7] += y * Dw[a]; Jt[8] += z * Dw[a];
      Xt[0] += x * Nr[a]; Xt[1] += y * Nr[a]; Xt[2] += z * Nr[a];
      if (P.kind == IFEMGPU_POISSON && P.logk) gk += Nr[a] * (T)P.logk[nodeA[a]];
      if (P.kind == IFEMGPU_POISSON && P.noise) sn += Nr[a] * (T)P.noise[nodeA[a]];
    }
#pragma unroll
    for (int c = 0; c < 9; c++) Jt[c] = warpAllSum(Jt[c]);
#pragma unroll
    for (int c = 0; c < 3; c++) Xt[c] = warpAllSum(Xt[c]);
    if (P.kind == IFEMGPU_POISSON && P.logk) gk = warpAllSum(gk);
    if (P.kind == IFEMGPU_POISSON && P.noise) sn = warpAllSum(sn);
    // park the sums (every lane holds them) for the thread-per-point FP64 stage
#pragma unroll
    for (int c = 0; c < 9; c++)
      if (lane == c) Ji[q * 9 + c] = Jt[c];
    if (lane == 9) wq[q] = Xt[0];
    if (lane == 10) kq[q] = Xt[1];
    if (lane == 11) fq[q] = Xt[2];
    if (lane == 12) gsum[2 * q] = gk;
    if (lane == 13) gsum[2 * q + 1] = sn;
  }
  __syncthreads();
  // thread per Gauss point (FP64 instructions with every lane busy)
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    T Jt[9], Xt[3];
    for (int c = 0; c < 9; c++) Jt[c] = Ji[q * 9 + c];
    Xt[0] = wq[q];
    Xt[1] = kq[q];
    Xt[2] = fq[q];
    const double gk = gsum[2 * q], sn = gsum[2 * q + 1];
    double J[9], X[3];
    for (int c = 0; c < 9; c++) J[c] = (double)Jt[c];
    for (int c = 0; c < 3; c++) X[c] = (double)Xt[c] + c00[c];
    double det, B[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (dim == 3) {
      // matrix<T>::det / inverse (src/LinAlg/matrix.h:790-850), T(i,j)=J[(j-1)*3+i-1];
      // cofactors times one reciprocal of det (FP64 divisions are costly here)
      det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[3] * (J[1] * J[8] - J[2] * J[7]) +
            J[6] * (J[1] * J[5] - J[2] * J[4]);
      if (det > kEpsZ || det < -kEpsZ) {
        const double id = 1.0 / det;
        B[0] = (J[4] * J[8] - J[5] * J[7]) * id;
        B[1] = -(J[1] * J[8] - J[2] * J[7]) * id;
        B[2] = (J[1] * J[5] - J[2] * J[4]) * id;
        B[3] = -(J[3] * J[8] - J[5] * J[6]) * id;
        B[4] = (J[0] * J[8] - J[2] * J[6]) * id;
        B[5] = -(J[0] * J[5] - J[2] * J[3]) * id;
        B[6] = (J[3] * J[7] - J[4] * J[6]) * id;
        B[7] = -(J[0] * J[7] - J[1] * J[6]) * id;
        B[8] = (J[0] * J[4] - J[1] * J[3]) * id;
      }
    } else {
      // 2x2: J(r,c) at J[c*3+r] in the 3x3 storage above
      det = J[0] * J[4] - J[1] * J[3];
      if (det > kEpsZ || det < -kEpsZ) {
        const double id = 1.0 / det;
        B[0] = J[4] * id; B[1] = -J[1] * id;
        B[3] = -J[3] * id; B[4] = J[0] * id;
      }
    }
    double w = 0.0;
    if (det > kEpsZ || det < -kEpsZ) {
      const int gi = q % P.ng[0], gj = (q / P.ng[0]) % P.ng[1], gz = q / (P.ng[0] * P.ng[1]);
      double dV = (dim == 3 ? 0.125 : 0.25) * P.span[0][e1] * P.span[1][e2];
      if (dim == 3) dV *= P.span[2][e3];
      w = det * dV * P.gw[0][gi] * P.gw[1][gj];
      if (dim == 3) w *= P.gw[2][gz];
    } else {
      atomicAdd(S.counters, 1ull);
    }
    wq[q] = (T)w;
    for (int c = 0; c < 9; c++) Ji[q * 9 + c] = (T)B[c];
    // material data at the point
    double kap = P.kappa, f = P.source;
    if (P.kind == IFEMGPU_POISSON) {
      if (P.logk) kap *= sizeof(T) == sizeof(float) ? (double)expf((float)gk) : exp(gk);
      if (P.source_shape == IFEMGPU_SOURCE_SINE)
        for (int c = 0; c < dim; c++) f *= sin(M_PI * X[c]);
      if (P.noise) f *= 1.0 + sn;
    }
    kq[q] = (T)(kap * w);
    fq[q] = (T)f;
  }
  __syncthreads();

  // dNdX = dNdu * J^-1 in place
  for (int t = threadIdx.x; t < nq * nen; t += blockDim.x) {
    const int q = t / nen;
    const T* B = Ji + q * 9;
    const T du = dX[t], dv = dX[nq * nen + t], dw = dX[2 * nq * nen + t];
    // (dNdX)_c = sum_k dNdu_k * Jinv(k,c), Jinv column-major B[c*3+k]
    dX[t] = du * B[0] + dv * B[1] + dw * B[2];
    dX[nq * nen + t] = du * B[3] + dv * B[4] + dw * B[5];
    dX[2 * nq * nen + t] = du * B[6] + dv * B[7] + dw * B[8];
  }
  __syncthreads();

  if (kFlow) {
    waitNeighbours(P, e, S);
    __syncthreads();
  }

  // Poisson in split mode: register tiles of node pairs, tile size per patch
  if constexpr (sizeof(T) == sizeof(float)) {
    if (P.kind == IFEMGPU_POISSON && S.c0 == nullptr && P.mass == 0.0) {
      if (P.tile == 2) poissonTiles<2>(P, S, dX, kq, eq, nodeA, Fa);
      else poissonTiles<4>(P, S, dX, kq, eq, nodeA, Fa);
    }
  }

  // element matrix for node pairs a <= bn, scattered as the (a, bn) block and
  // its transpose (bn, a)
  const T lam = sizeof(T) == sizeof(float) ? (T)P.lamf : (T)P.lam;
  const T mu = sizeof(T) == sizeof(float) ? (T)P.muf : (T)P.mu;
  const bool tiled =
      sizeof(T) == sizeof(float) && P.kind == IFEMGPU_POISSON && S.c0 == nullptr && P.mass == 0.0;
  const T ms = (T)P.mass;  // consistent mass: Ke += ms sum_q N_a N_b w_q per component
  const int npairs = tiled ? 0 : nen * (nen + 1) / 2;
  for (int t = threadIdx.x; t < npairs; t += blockDim.x) {
    int bn = (int)((sqrtf(8.f * t + 1.f) - 1.f) * 0.5f);
    while (bn * (bn + 1) / 2 > t) bn--;
    while ((bn + 1) * (bn + 2) / 2 <= t) bn++;
    const int a = t - bn * (bn + 1) / 2;
    T Ke[9];
    if (P.kind == IFEMGPU_POISSON) {
      T acc = 0;
      for (int q = 0; q < nq; q++) {
        const T s = kq[q];
        if (s == T(0)) continue;
        T v = 0;
        for (int c = 0; c < dim; c++)
          v += dX[c * nq * nen + q * nen + a] * s * dX[c * nq * nen + q * nen + bn];
        acc += v;
      }
      Ke[0] = acc;
    } else {
      T G[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int q = 0; q < nq; q++) {
        const T w = wq[q];
        if (w == T(0)) continue;
        const T ax = dX[q * nen + a] * w, ay = dX[nq * nen + q * nen + a] * w,
                az = dX[2 * nq * nen + q * nen + a] * w;
        const T bx = dX[q * nen + bn], by = dX[nq * nen + q * nen + bn],
                bz = dX[2 * nq * nen + q * nen + bn];
        G[0] += ax * bx; G[1] += ax * by; G[2] += ax * bz;
        G[3] += ay * bx; G[4] += ay * by; G[5] += ay * bz;
        G[6] += az * bx; G[7] += az * by; G[8] += az * bz;
      }
      const T tr = G[0] + G[4] + G[8];
      for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++)
          Ke[k * 3 + l] = lam * G[k * 3 + l] + mu * G[l * 3 + k] + (k == l ? mu * tr : T(0));
    }
    if (ms != T(0)) {  // EqualOrderOperators::Weak::Mass
      T m = 0;
      for (int q = 0; q < nq; q++) m += Nq[q * nen + a] * Nq[q * nen + bn] * wq[q];
      for (int k = 0; k < npv; k++) Ke[k * npv + k] += ms * m;
    }
    // scatter: block (rows of a, columns of bn), then (rows of bn, columns of a)
    for (int side = 0; side < (a == bn ? 1 : 2); side++) {
      const int ra = side ? bn : a, cb = side ? a : bn;
      int firstCol = -1, firstRow = -1;
      for (int l = 0; l < npv && firstCol < 0; l++)
        if (eq[cb * npv + l] > 0) firstCol = eq[cb * npv + l] - 1;
      for (int k = 0; k < npv && firstRow < 0; k++)
        if (eq[ra * npv + k] > 0) firstRow = eq[ra * npv + k] - 1;
      if (firstCol < 0 || firstRow < 0) continue;
      int off;
      if (P.lineOff) {  // structured patch: position from the line-offset table
        const int w1 = 2 * P.p[1] + 1, w2 = 2 * P.p[2] + 1;
        const int dy = (ra / q1) % q2 - (cb / q1) % q2, dz = ra / (q1 * q2) - cb / (q1 * q2);
        off = P.lineOff[(size_t)nodeA[cb] * w1 * w2 + (dz + P.p[2]) * w1 + dy + P.p[1]] + Fa[ra];
      } else {
        const int pos0 = findRow(S.colptr, S.rowidx, firstCol, firstRow);
        if (pos0 < 0) { atomicAdd(S.counters + 1, 1ull); continue; }
        off = pos0 - S.colptr[firstCol];
      }
      for (int l = 0; l < npv; l++) {
        const int ce = eq[cb * npv + l];
        if (ce <= 0) continue;
        int rank = 0;
        for (int k = 0; k < npv; k++) {
          const int re = eq[ra * npv + k];
          if (re <= 0) continue;
          addEntry(S.K + S.colptr[ce - 1] + off + rank, side ? Ke[l * npv + k] : Ke[k * npv + l],
                   kFlow);
          rank++;
        }
      }
    }
  }

  // element load vector and prescribed-DOF corrections, row by row
  for (int i = threadIdx.x; i < nd; i += blockDim.x) {
    const int r = eq[i];
    if (r <= 0) continue;
    const int a = i / npv, k = i % npv;
    T fe = 0;
    for (int q = 0; q < nq; q++) {
      if (wq[q] == T(0)) continue;
      const T Na = Nq[q * nen + a];
      if (P.kind == IFEMGPU_POISSON) fe += Na * fq[q] * wq[q];
      else fe += (sizeof(T) == sizeof(float) ? (T)P.bodyf[k] : (T)P.body[k]) * Na * wq[q];
    }
    double acc = (double)fe;
    if (S.c0 != nullptr) {
      for (int j = 0; j < nd; j++) {
        const int ce = eq[j];
        if (ce >= 0) continue;
        const int bn = j / npv, l = j % npv;
        T kij = 0;
        for (int q = 0; q < nq; q++) {
          const T w = wq[q];
          if (w == T(0)) continue;
          if (P.kind == IFEMGPU_POISSON) {
            T v = 0;
            for (int c = 0; c < dim; c++)
              v += dX[c * nq * nen + q * nen + a] * kq[q] * dX[c * nq * nen + q * nen + bn];
            kij += v;
          } else {
            const T ak = dX[k * nq * nen + q * nen + a] * w;
            const T al = dX[l * nq * nen + q * nen + a] * w;
            T g = 0;
            for (int c = 0; c < 3; c++)
              g += dX[c * nq * nen + q * nen + a] * w * dX[c * nq * nen + q * nen + bn];
            kij += lam * ak * dX[l * nq * nen + q * nen + bn] +
                   mu * al * dX[k * nq * nen + q * nen + bn] + (k == l ? mu * g : T(0));
          }
          if (k == l && ms != T(0)) kij += ms * Nq[q * nen + a] * Nq[q * nen + bn] * w;
        }
        acc -= S.c0[-ce - 1] * (double)kij;
      }
    }
    if (sizeof(T) == sizeof(double) && !kFlow) S.b[r - 1] += acc;
    else atomicAdd(S.b + r - 1, acc);
  }
  if (kFlow) {  // publish: this element's contributions are all issued
    __syncthreads();
    if (threadIdx.x == 0 && P.flagBase + e != S.withhold) {
      __threadfence();
      genStoreRelease(S.flags + P.flagBase + e, 1);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256, 3)
k_volume_gen(const DevPatch* __restrict__ patches, const Item* __restrict__ items, SysView S)
{
  extern __shared__ __align__(16) unsigned char smraw[];
  const Item it = items[blockIdx.x];
  volumeElement<T, false>(patches[it.patch], it, S, smraw);
}

// Persistent colour-major pass over many patches: blocks claim elements in
// item order through counters[3], so an element only ever waits for elements
// claimed before it by running blocks, whatever the grid size.
template <typename T>
__global__ void __launch_bounds__(256, 3)  // three blocks per SM, as the per-colour kernel
k_volume_gen_flow(const DevPatch* __restrict__ patches, const Item* __restrict__ items, int count,
                  SysView S)
{
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int claimed;
  for (;;) {
    __syncthreads();  // the previous element is done with shared memory
    if (threadIdx.x == 0) claimed = (int)atomicAdd(S.counters + 3, 1ull);
    __syncthreads();
    const int idx = claimed;
    if (idx >= count) break;
    const Item it = items[idx];
    volumeElement<T, true>(patches[it.patch], it, S, smraw);
  }
}

// ---------------------------------------------------------------------------
// Face (Neumann) kernel: one CTA per face element of one colour, FP64.
// Shared memory (doubles): Xn[nen*4] | Nf[nqf*nen] | wf[nqf]  then eq[nd] (int)
__global__ void __launch_bounds__(128)
k_face_fp64(const DevPatch* __restrict__ patches, const Item* __restrict__ items,
            const double* __restrict__ neumann, SysView S)
{
  extern __shared__ double sm[];
  const Item it = items[blockIdx.x];
  const DevPatch& P = patches[it.patch];
  const int nen = P.nen, npv = P.npv, nd = nen * npv, e = it.elem;
  const int face = it.face;
  const int faceDir = (face % 10 + 1) / ((face % 2) ? -2 : 2);
  const int nd0 = abs(faceDir) - 1;
  const int t1 = 1 + abs(faceDir) % 3, t2 = 1 + t1 % 3;
  int ng[3];
  for (int d = 0; d < 3; d++) ng[d] = d == nd0 ? 1 : P.ngf[d];
  const int nqf = ng[0] * ng[1] * ng[2];
  double* Xn = sm;
  double* Nf = Xn + nen * 4;
  double* wf = Nf + nqf * nen;
  int* eq = reinterpret_cast<int*>(wf + nqf);
  const int ee[3] = {e % P.nel[0], (e / P.nel[0]) % P.nel[1], e / (P.nel[0] * P.nel[1])};
  const int q1 = P.p[0] + 1, q2 = P.p[1] + 1;
  for (int a = threadIdx.x; a < nen; a += blockDim.x) {
    const int node = elemNode(P, e, a);
    for (int c = 0; c < 4; c++) Xn[a * 4 + c] = P.ctrl[(size_t)node * 4 + c];
    const int d0 = S.madof[globalNode(P, node)] - 1;
    for (int c = 0; c < npv; c++) eq[a * npv + c] = S.meqn[d0 + c];
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nqf; q += blockDim.x) {
    const int gi[3] = {q % ng[0], (q / ng[0]) % ng[1], q / (ng[0] * ng[1])};
    double Nd[3][kMaxDeg + 1], Dd[3][kMaxDeg + 1];
    double wt = 0.25;
    for (int d = 0; d < 3; d++) {
      const int p1 = P.p[d] + 1;
      if (d == nd0) {  // normal direction: the boundary table of this side
        const double* tb = P.tabB[d] + (faceDir < 0 ? 0 : 2 * p1);
        for (int r = 0; r < p1; r++) {
          Nd[d][r] = tb[r];
          Dd[d][r] = tb[p1 + r];
        }
        continue;
      }
      wt *= P.span[d][ee[d]] * P.fw[d][gi[d]];
      if (P.faceTables) {  // face rule = volume rule: the volume tables apply
        const size_t o = ((size_t)ee[d] * P.ng[d] + gi[d]) * p1;
        for (int r = 0; r < p1; r++) {
          Nd[d][r] = P.tabN[d][o + r];
          Dd[d][r] = P.tabD[d][o + r];
        }
      } else {
        const double* U = P.knots[d];
        const int k = P.p[d] + ee[d];
        const double u0 = U[k], u1 = U[k + 1];
        bsplineDers(U, P.p[d], k, 0.5 * ((u1 - u0) * P.fx[d][gi[d]] + u1 + u0), Nd[d], Dd[d]);
      }
    }
    // homogeneous sums S[c][0] = sum_a wN_a X_a,c, S[c][1+d] = sum_a w dN_a/du_d X_a,c
    // (X_a,3 = 1 gives W and its derivatives); one reciprocal per point
    double Sm[4][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
    double* Nr = Nf + q * nen;
    for (int a = 0; a < nen; a++) {
      const int i = a % q1, j = (a / q1) % q2, k = a / (q1 * q2);
      const double w = Xn[a * 4 + 3];
      const double wN = w * (Nd[0][i] * Nd[1][j] * Nd[2][k]);
      const double w0 = w * (Dd[0][i] * Nd[1][j] * Nd[2][k]);
      const double w1 = w * (Nd[0][i] * Dd[1][j] * Nd[2][k]);
      const double w2 = w * (Nd[0][i] * Nd[1][j] * Dd[2][k]);
      Nr[a] = wN;
      for (int c = 0; c < 4; c++) {
        const double x = c < 3 ? Xn[a * 4 + c] : 1.0;
        Sm[c][0] += wN * x;
        Sm[c][1] += w0 * x;
        Sm[c][2] += w1 * x;
        Sm[c][3] += w2 * x;
      }
    }
    const double iW = 1.0 / Sm[3][0];
    for (int a = 0; a < nen; a++) Nr[a] *= iW;
    double J[9];  // J[d*3 + c] = dX_c/du_d
    for (int c = 0; c < 3; c++) {
      const double Xc = Sm[c][0] * iW;
      for (int d = 0; d < 3; d++) J[d * 3 + c] = (Sm[c][1 + d] - Xc * Sm[3][1 + d]) * iW;
    }
    const double* ta = J + 3 * (t1 - 1);
    const double* tb = J + 3 * (t2 - 1);
    const double nx = ta[1] * tb[2] - ta[2] * tb[1], ny = ta[2] * tb[0] - ta[0] * tb[2],
                 nz = ta[0] * tb[1] - ta[1] * tb[0];
    const double dS = sqrt(nx * nx + ny * ny + nz * nz);
    const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[3] * (J[1] * J[8] - J[2] * J[7]) +
                       J[6] * (J[1] * J[5] - J[2] * J[4]);
    wf[q] = (det > kEpsZ || det < -kEpsZ) ? dS * wt : 0.0;
  }
  __syncthreads();
  const double* t = neumann + 3 * it.bc;
  for (int i = threadIdx.x; i < nd; i += blockDim.x) {
    const int r = eq[i];
    if (r <= 0) continue;
    const int a = i / npv, c = i % npv;
    double fe = 0.0;
    for (int q = 0; q < nqf; q++)
      if (wf[q] != 0.0) fe += t[c] * Nf[q * nen + a] * wf[q];
    S.b[r - 1] += fe;
  }
}

// ---------------------------------------------------------------------------
size_t volumeSmem(const DevPatch& P, size_t real)
{
  return real * ((size_t)P.nen * 4 + (size_t)P.nq * P.nen * 4 + (size_t)P.nq * 12) +
         sizeof(double) * 2 * (size_t)P.nq + sizeof(int) * (size_t)P.nen * (P.npv + 2);
}

size_t faceSmem(const DevPatch& P, int nqf)
{
  return sizeof(double) * ((size_t)P.nen * 4 + (size_t)nqf * P.nen + nqf) +
         sizeof(int) * (size_t)P.nen * P.npv;
}

template <typename T>
ifemgpu_status upload(ifemgpu_ctx* ctx, T** dst, const T* src, size_t n)
{
  IFEMGPU_CUDA(ctx, cudaMalloc((void**)dst, sizeof(T) * std::max<size_t>(n, 1)));
  if (n) IFEMGPU_CUDA(ctx, cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice));
  return IFEMGPU_OK;
}


ifemgpu_status uploadAssemblyModel(ifemgpu_ctx* ctx)
{
  const int np = (int)ctx->patches.size();
  const size_t realBytes = ctx->opts.ke_precision == IFEMGPU_KE_SPLIT_TF32 ? sizeof(float)
                                                                          : sizeof(double);
  ctx->h_devpatches.assign(np, DevPatch{});
  std::vector<Item> vol, face;
  std::vector<double> neuVals;
  int maxColours = 0;
  for (int pi = 0; pi < np; pi++) {
    HostPatch& pc = ctx->patches[pi];
    DevPatch& D = ctx->h_devpatches[pi];
    std::memset(&D, 0, sizeof(D));
    D.dim = pc.dim;
    D.nen = pc.nen();
    D.npv = pc.npv;
    D.kind = pc.mat.kind;
    D.rational = pc.rational;
    D.firstNode = pc.firstNode;
    D.mlgn = nullptr;
    if (!ctx->conns.empty()) {  // connected model: global node table
      IFEMGPU_TRY(upload(ctx, &pc.d_mlgn, pc.mlgn.data(), pc.mlgn.size()));
      D.mlgn = pc.d_mlgn;
    }
    D.kappa = pc.mat.kappa;
    D.source = pc.mat.source;
    D.source_shape = pc.mat.source_shape;
    D.E = pc.mat.E;
    D.nu = pc.mat.nu;
    D.lam = D.E * D.nu / ((1.0 + D.nu) * (1.0 - 2.0 * D.nu));
    D.mu = D.E / (2.0 * (1.0 + D.nu));
    D.lamf = (float)D.lam;
    D.muf = (float)D.mu;
    D.mass = pc.mass;
    for (int c = 0; c < 3; c++) {
      D.body[c] = pc.mat.body[c];
      D.bodyf[c] = (float)D.body[c];
    }
    D.nq = 1;
    D.faceTables = 1;
    for (int d = 0; d < 3; d++) {
      D.p[d] = pc.p[d];
      D.n[d] = pc.n[d];
      D.nel[d] = pc.nel[d];
      D.ng[d] = 1;
      if (d < pc.dim) {
        int ng = gaussCount(ctx->opts.n_gauss, pc.p[d] + 1, false);
        int ngf = gaussCount(ctx->opts.n_gauss, pc.p[d] + 1, true);
        if (ng < 1 || ng > kMaxGauss || ngf < 1 || ngf > kMaxGauss)
          return setError(ctx, IFEMGPU_UNSUPPORTED, "Gauss point count outside 1..6");
        D.ng[d] = ng;
        D.ngf[d] = ngf;
        gaussRule(ng, D.gx[d], D.gw[d]);
        gaussRule(ngf, D.fx[d], D.fw[d]);
        for (int g = 0; g < ng; g++) D.gwf[d][g] = (float)D.gw[d][g];
        IFEMGPU_TRY(upload(ctx, &pc.d_knots[d], pc.knots[d].data(), pc.knots[d].size()));
        size_t tab = (size_t)pc.nel[d] * ng * (pc.p[d] + 1);
        IFEMGPU_CUDA(ctx, cudaMalloc(&pc.d_tabN[d], sizeof(double) * tab));
        IFEMGPU_CUDA(ctx, cudaMalloc(&pc.d_tabD[d], sizeof(double) * tab));
        IFEMGPU_CUDA(ctx, cudaMalloc(&pc.d_span[d], sizeof(double) * pc.nel[d]));
        IFEMGPU_CUDA(ctx, cudaMalloc(&pc.d_tabB[d], sizeof(double) * 4 * (pc.p[d] + 1)));
        IFEMGPU_CUDA(ctx, cudaMalloc(&pc.d_tabNf[d], sizeof(float) * tab));
        IFEMGPU_CUDA(ctx, cudaMalloc(&pc.d_tabDf[d], sizeof(float) * tab));
        if (ngf != ng) D.faceTables = 0;
      }
      D.nq *= D.ng[d];
      D.knots[d] = pc.d_knots[d];
      D.tabN[d] = pc.d_tabN[d];
      D.tabD[d] = pc.d_tabD[d];
      D.span[d] = pc.d_span[d];
      D.tabB[d] = pc.d_tabB[d];
      D.tabNf[d] = pc.d_tabNf[d];
      D.tabDf[d] = pc.d_tabDf[d];
    }
    IFEMGPU_TRY(upload(ctx, &pc.d_ctrl, pc.ctrl4.data(), pc.ctrl4.size()));
    if (!pc.lineOff.empty()) {
      IFEMGPU_TRY(upload(ctx, &pc.d_lineOff, pc.lineOff.data(), pc.lineOff.size()));
      D.lineOff = pc.d_lineOff;
    }
    D.ctrl = pc.d_ctrl;
    if (!pc.logk.empty()) {
      IFEMGPU_TRY(upload(ctx, &pc.d_logk, pc.logk.data(), pc.logk.size()));
      D.logk = pc.d_logk;
    }
    if (!pc.noise.empty()) {
      IFEMGPU_TRY(upload(ctx, &pc.d_noise, pc.noise.data(), pc.noise.size()));
      D.noise = pc.d_noise;
    }
    if (volumeSmem(D, realBytes) > 227 * 1024)
      return setError(ctx, IFEMGPU_UNSUPPORTED, "element too large for the element kernel");
    const int nc = (pc.p[0] + 1) * (pc.p[1] + 1) * (pc.dim == 3 ? pc.p[2] + 1 : 1);
    maxColours = std::max(maxColours, nc);
  }
  // Patches on the tensor-core path: all their elements in one colour-major
  // pass (one persistent launch ordered by per-element done flags); the
  // other patches: one FP64 launch per colour.
  // colour = (e1 mod q1) + q1 (e2 mod q2) + q1 q2 (e3 mod q3)
  std::vector<char> onTc(np, 0);
  std::vector<int> tcDeg(np, 0);  // 0: elasticity p = 2 kernel; 2, 3: Poisson kernel
  int nflags = 0;
  // the other patches share one persistent pass when every element has a
  // volume (the done flags assume a full element grid)
  bool flow = ctx->opts.colour_passes != 1 && ctx->conns.empty();
  for (int pi = 0; pi < np; pi++) {
    DevPatch& D = ctx->h_devpatches[pi];
    onTc[pi] = ctx->opts.ke_precision == IFEMGPU_KE_SPLIT_TF32 && tcSupports(D) && D.mass == 0.0 &&
               D.lineOff != nullptr && D.faceTables && ctx->patches[pi].neumann.size() <= 6;
    if (onTc[pi]) onTc[pi] = tcUploadPatch(ctx, ctx->patches[pi], D);  // control-net TMA map
    if (!onTc[pi] && ctx->opts.ke_precision == IFEMGPU_KE_SPLIT_TF32 && tcElast3Supports(D) &&
        D.mass == 0.0 && D.lineOff != nullptr && D.faceTables &&
        ctx->patches[pi].neumann.size() <= 6 &&
        tcPoissonUpload(ctx, ctx->patches[pi], D, 3)) {  // (p+1)^3 control-net boxes
      onTc[pi] = 1;
      tcDeg[pi] = kTcElast3;
    }
    if (!onTc[pi] && ctx->opts.ke_precision == IFEMGPU_KE_SPLIT_TF32) {
      const int deg = tcPoissonDegree(D, ctx->patches[pi]);
      if (deg && tcPoissonUpload(ctx, ctx->patches[pi], D, deg)) {
        onTc[pi] = 1;
        tcDeg[pi] = deg;
      }
    }
    if (!onTc[pi] && ctx->patches[pi].nelActive != ctx->patches[pi].nelAll) flow = false;
  }
  // element scratch of the tensor-core patches (one block per element, read
  // back by the node-wise gather) and the gather launches per (degree, npv)
  ctx->elmFloats = 0;
  for (int pi = 0; pi < np; pi++)
    if (onTc[pi])
      ctx->elmFloats += (size_t)ctx->patches[pi].nelAll *
                        elementBlockFloats(ctx->h_devpatches[pi].p[0], ctx->h_devpatches[pi].npv);
  if (ctx->elmFloats)
    IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_elm, sizeof(float) * ctx->elmFloats));
  {
    size_t at = 0;
    for (int pi = 0; pi < np; pi++) {
      DevPatch& D = ctx->h_devpatches[pi];
      D.elm = nullptr;
      D.elmStride = 0;
      if (!onTc[pi]) continue;
      D.elmStride = (int)elementBlockFloats(D.p[0], D.npv);
      D.elm = ctx->d_elm + at;
      at += (size_t)ctx->patches[pi].nelAll * D.elmStride;
    }
  }
  ctx->gathers.clear();
  ctx->zeroSystem = false;
  for (int pi = 0; pi < np; pi++) ctx->zeroSystem |= !onTc[pi];
  for (const auto& cls : {std::make_pair(2, 3), std::make_pair(3, 3), std::make_pair(2, 1),
                          std::make_pair(3, 1)}) {
    std::vector<int> start, pidx;
    int total = 0;
    for (int pi = 0; pi < np; pi++) {
      const DevPatch& D = ctx->h_devpatches[pi];
      if (!onTc[pi] || D.p[0] != cls.first || D.npv != cls.second) continue;
      start.push_back(total);
      pidx.push_back(pi);
      total += ctx->patches[pi].nnod;
    }
    if (!total) continue;
    GatherList g;
    g.p = cls.first;
    g.npv = cls.second;
    // each node pair once, mirrored writes: pays where the element work
    // dominates the scattered mirrored writes (p = 3 elasticity, 32^3: 5.14 ->
    // 4.78 ms per assembly); p = 2 elasticity and p = 3 Poisson run slower
    // with it (64^3: 6.80 -> 7.72 and 12.5 -> 13.5 ms); prescribed values
    // need every warp's full neighbourhood
    g.half = ctx->nceq == 0 && g.p == 3 && g.npv == 3;
    g.nranges = (int)start.size();
    g.total = total;
    IFEMGPU_TRY(upload(ctx, &g.d_start, start.data(), start.size()));
    IFEMGPU_TRY(upload(ctx, &g.d_pidx, pidx.data(), pidx.size()));
    ctx->gathers.push_back(g);
  }
  for (int pi = 0; pi < np; pi++) {
    DevPatch& D = ctx->h_devpatches[pi];
    D.flagBase = nflags;
    D.tile = 4;
    if (!onTc[pi] && flow) nflags += ctx->patches[pi].nelAll;
    if (onTc[pi] && (tcDeg[pi] == 0 || tcDeg[pi] == kTcElast3)) {
      // the element kernel integrates this patch's Neumann faces itself
      D.nneu = (int)ctx->patches[pi].neumann.size();
      for (int f = 0; f < D.nneu; f++) {
        D.neuFace[f] = ctx->patches[pi].neumann[f].face;
        for (int c = 0; c < 3; c++) D.neuT[f][c] = (float)ctx->patches[pi].neumann[f].t[c];
      }
    }
  }
  auto colourItems = [&](int pi, int c, std::vector<Item>& out) {
    const HostPatch& pc = ctx->patches[pi];
    const int q1 = pc.p[0] + 1, q2 = pc.p[1] + 1, q3 = pc.dim == 3 ? pc.p[2] + 1 : 1;
    if (c >= q1 * q2 * q3) return;
    const int c1 = c % q1, c2 = (c / q1) % q2, c3 = c / (q1 * q2);
    for (int e3 = c3; e3 < pc.nel[2]; e3 += q3)
      for (int e2 = c2; e2 < pc.nel[1]; e2 += q2)
        for (int e1 = c1; e1 < pc.nel[0]; e1 += q1) {
          const int e = (e3 * pc.nel[1] + e2) * pc.nel[0] + e1;
          if (pc.active[e]) out.push_back({pi, e, 0, 0});
        }
  };
  for (int deg : {0, kTcElast3, 2, 3}) {  // one persistent launch per tensor-core kernel
    const size_t smem = deg == 0 ? tcVolumeSmem() : deg == kTcElast3 ? tcElast3Smem()
                                                                      : tcPoissonSmem(deg);
    Pass pass{(int)vol.size(), 0, 0, deg == 0 ? 81 : deg == kTcElast3 ? 192 : 1, smem, true};
    pass.tcDeg = deg;
    for (int pi = 0; pi < np; pi++)
      if (onTc[pi] && tcDeg[pi] == deg)
        for (int e = 0; e < ctx->patches[pi].nelAll; e++) vol.push_back({pi, e, 0, 0});
    pass.count = (int)vol.size() - pass.first;
    if (pass.count) ctx->passes.push_back(pass);
  }
  ctx->onFlow.assign(np, 0);
  for (int pi = 0; pi < np; pi++) ctx->onFlow[pi] = flow && !onTc[pi];
  if (flow) {  // one colour-major launch over every other patch
    Pass pass{(int)vol.size(), 0, 0, 0, 0, false};
    pass.persistent = true;
    for (int c = 0; c < maxColours; c++)
      for (int pi = 0; pi < np; pi++)
        if (!onTc[pi]) colourItems(pi, c, vol);
    for (int pi = 0; pi < np; pi++) {
      if (onTc[pi]) continue;
      pass.maxNd = std::max(pass.maxNd, ctx->patches[pi].nen() * ctx->patches[pi].npv);
      pass.smem = std::max(pass.smem, volumeSmem(ctx->h_devpatches[pi], realBytes));
    }
    pass.count = (int)vol.size() - pass.first;
    if (pass.count) {
      ctx->passes.push_back(pass);
      // the same items as one launch per colour (the autotuner picks the faster)
      int at = pass.first;
      for (int c = 0; c < maxColours; c++) {
        Pass cp{at, 0, 0, pass.maxNd, pass.smem, false};
        cp.altColour = true;
        for (int pi = 0; pi < np; pi++) {
          if (onTc[pi]) continue;
          const HostPatch& pc = ctx->patches[pi];
          const int q1 = pc.p[0] + 1, q2 = pc.p[1] + 1, q3 = pc.dim == 3 ? pc.p[2] + 1 : 1;
          if (c >= q1 * q2 * q3) continue;
          const int c1 = c % q1, c2 = (c / q1) % q2, c3 = c / (q1 * q2);
          cp.count += ((pc.nel[0] - c1 + q1 - 1) / q1) * ((pc.nel[1] - c2 + q2 - 1) / q2) *
                      ((pc.nel[2] - c3 + q3 - 1) / q3);
        }
        at += cp.count;
        if (cp.count) ctx->passes.push_back(cp);
      }
      if (at != pass.first + pass.count)
        return setError(ctx, IFEMGPU_CUDA_ERROR, "internal: colour ranges of the persistent pass");
    }
  } else {
    // one launch per colour; in a connected model elements of two patches
    // may share nodes, so there one launch per (colour, patch), in order
    const bool perPatch = !ctx->conns.empty();
    for (int c = 0; c < maxColours; c++) {
      Pass pass{(int)vol.size(), 0, 0, 0, 0, false};
      for (int pi = 0; pi < np; pi++) {
        if (onTc[pi]) continue;
        const HostPatch& pc = ctx->patches[pi];
        colourItems(pi, c, vol);
        pass.maxNd = std::max(pass.maxNd, pc.nen() * pc.npv);
        pass.smem = std::max(pass.smem, volumeSmem(ctx->h_devpatches[pi], realBytes));
        if (perPatch) {
          pass.count = (int)vol.size() - pass.first;
          if (pass.count) ctx->passes.push_back(pass);
          pass = Pass{(int)vol.size(), 0, 0, 0, 0, false};
        }
      }
      pass.count = (int)vol.size() - pass.first;
      if (pass.count) ctx->passes.push_back(pass);
    }
  }
  ctx->nflags = nflags;
  if (nflags) IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_flags, sizeof(int) * nflags));
  // face items: per Neumann condition, face elements coloured in 2D
  const int nVol = (int)vol.size();
  std::vector<Pass> facePasses;
  for (int pi = 0; pi < np; pi++) {
    const HostPatch& pc = ctx->patches[pi];
    if (onTc[pi]) continue;  // integrated by the tensor-core element kernel
    for (const auto& nm : pc.neumann) {
      const int bc = (int)neuVals.size() / 3;
      for (int c = 0; c < 3; c++) neuVals.push_back(nm.t[c]);
      const int faceDir = (nm.face + 1) / ((nm.face % 2) ? -2 : 2);
      const int nd0 = std::abs(faceDir) - 1;
      const int fixedIdx = faceDir < 0 ? 0 : pc.nel[nd0] - 1;
      int ta = nd0 == 0 ? 1 : 0, tb = nd0 == 2 ? 1 : 2;
      const int qa = pc.p[ta] + 1, qb = pc.p[tb] + 1;
      int nqf = 1;
      for (int d = 0; d < 3; d++)
        if (d != nd0) nqf *= gaussCount(ctx->opts.n_gauss, pc.p[d] + 1, true);
      for (int c = 0; c < qa * qb; c++) {
        Pass pass{0, 0, nm.face, pc.nen() * pc.npv, faceSmem(ctx->h_devpatches[pi], nqf), false};
        std::vector<Item> lst;
        for (int e = 0; e < pc.nelAll; e++) {
          if (!pc.active[e]) continue;
          int ee[3] = {e % pc.nel[0], (e / pc.nel[0]) % pc.nel[1], e / (pc.nel[0] * pc.nel[1])};
          if (ee[nd0] != fixedIdx) continue;
          if ((ee[ta] % qa) + qa * (ee[tb] % qb) != c) continue;
          lst.push_back({pi, e, nm.face, bc});
        }
        pass.first = (int)(vol.size() + face.size());
        pass.count = (int)lst.size();
        face.insert(face.end(), lst.begin(), lst.end());
        if (pass.count) facePasses.push_back(pass);
      }
    }
  }
  (void)nVol;
  ctx->passes.insert(ctx->passes.end(), facePasses.begin(), facePasses.end());
  vol.insert(vol.end(), face.begin(), face.end());
  IFEMGPU_TRY(upload(ctx, &ctx->d_items, vol.data(), vol.size()));
  IFEMGPU_TRY(upload(ctx, &ctx->d_neumann, neuVals.data(), neuVals.size()));
  IFEMGPU_TRY(upload(ctx, &ctx->d_patches, ctx->h_devpatches.data(), np));
  // work lists of the basis-table launch: per patch nel*ng points per
  // direction plus the boundary tables
  {
    std::vector<int> start(np + 1, 0);
    for (int pi = 0; pi < np; pi++) {
      const DevPatch& D = ctx->h_devpatches[pi];
      int work = 2 * D.dim;
      for (int d = 0; d < D.dim; d++) work += D.nel[d] * D.ng[d];
      start[pi + 1] = start[pi] + work;
    }
    ctx->basisWork = start[np];
    IFEMGPU_TRY(upload(ctx, &ctx->d_basisStart, start.data(), start.size()));
  }
  // system arrays
  IFEMGPU_TRY(upload(ctx, &ctx->d_madof, ctx->madof.data(), ctx->madof.size()));
  IFEMGPU_TRY(upload(ctx, &ctx->d_meqn, ctx->meqn.data(), ctx->meqn.size()));
  if (!ctx->c0.empty()) IFEMGPU_TRY(upload(ctx, &ctx->d_c0, ctx->c0.data(), ctx->c0.size()));
  IFEMGPU_TRY(upload(ctx, &ctx->d_colptr, ctx->colptr.data(), ctx->colptr.size()));
  IFEMGPU_TRY(upload(ctx, &ctx->d_rowidx, ctx->rowidx.data(), ctx->rowidx.size()));
  IFEMGPU_TRY(upload(ctx, &ctx->d_freeBefore, ctx->freeBefore.data(), ctx->freeBefore.size()));
  IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_K, sizeof(double) * std::max<int64_t>(ctx->nnz, 1)));
  IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_b, sizeof(double) * std::max(ctx->neq, 1)));
  IFEMGPU_CUDA(ctx, cudaMalloc(&ctx->d_counters, sizeof(unsigned long long) * 4));
  size_t maxSmem = 0;
  for (auto& p : ctx->passes) maxSmem = std::max(maxSmem, p.smem);
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_volume_gen<double>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::min<size_t>(maxSmem, 227 * 1024)));
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_volume_gen<float>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::min<size_t>(maxSmem, 227 * 1024)));
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_face_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::min<size_t>(maxSmem, 227 * 1024)));
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_volume_gen_flow<double>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::min<size_t>(maxSmem, 227 * 1024)));
  IFEMGPU_CUDA(ctx, cudaFuncSetAttribute(k_volume_gen_flow<float>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::min<size_t>(maxSmem, 227 * 1024)));
  IFEMGPU_CUDA(ctx, cudaDeviceGetAttribute(&ctx->numSMs, cudaDevAttrMultiProcessorCount,
                                           ctx->opts.device));
  // default grid of the persistent pass: as many blocks as fit at once
  ctx->genGrid = 0;
  ctx->tuned = false;
  for (auto& p : ctx->passes)
    if (p.persistent) {
      int perSM = 0;
      if (ctx->opts.ke_precision == IFEMGPU_KE_SPLIT_TF32)
        IFEMGPU_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                              &perSM, k_volume_gen_flow<float>, 256, p.smem));
      else
        IFEMGPU_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                              &perSM, k_volume_gen_flow<double>, 256, p.smem));
      ctx->genGrid = std::max(1, perSM) * ctx->numSMs;
    }
  for (auto& p : ctx->passes)
    if (p.tc) {
      IFEMGPU_TRY(tcPrepare(ctx));
      IFEMGPU_TRY(tcPoissonPrepare(ctx));
      IFEMGPU_TRY(tcElast3Prepare(ctx));
      break;
    }
  for (auto& g : ctx->gathers) IFEMGPU_TRY(gatherPrepare(ctx, g));
  return IFEMGPU_OK;
}

// raw (dim coordinates [+ weight]) -> (x, y, z, w) control net layout
__global__ void k_pack_coefs(const double* __restrict__ raw, double* __restrict__ ctrl,
                             int nnod, int dim, int rational)
{
  const int stride = dim + rational;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnod; i += gridDim.x * blockDim.x) {
    double v[4] = {0.0, 0.0, 0.0, 1.0};
    for (int c = 0; c < dim; c++) v[c] = raw[(size_t)i * stride + c];
    if (rational) v[3] = raw[(size_t)i * stride + dim];
    for (int c = 0; c < 4; c++) ctrl[(size_t)i * 4 + c] = v[c];
  }
}

ifemgpu_status updateCoefs(ifemgpu_ctx* ctx, int pi, const double* coefs)
{
  HostPatch& pc = ctx->patches[pi];
  const int stride = pc.dim + (pc.rational ? 1 : 0);
  const size_t n = (size_t)pc.nnod * stride;
  if (!pc.d_stage) IFEMGPU_CUDA(ctx, cudaMalloc(&pc.d_stage, sizeof(double) * n));
  IFEMGPU_CUDA(ctx, cudaMemcpyAsync(pc.d_stage, coefs, sizeof(double) * n,
                                    cudaMemcpyHostToDevice, ctx->stream));
  const int blocks = std::min(1024, (pc.nnod + 255) / 256);
  k_pack_coefs<<<blocks, 256, 0, ctx->stream>>>(pc.d_stage, pc.d_ctrl, pc.nnod, pc.dim,
                                                pc.rational ? 1 : 0);
  IFEMGPU_CUDA(ctx, cudaGetLastError());
  return IFEMGPU_OK;
}

static SysView sysView(ifemgpu_ctx* ctx)
{
  int withhold = -1;
  if (ctx->dbg.patch >= 0 && ctx->dbg.patch < (int)ctx->h_devpatches.size() && ctx->dbg.elem >= 0)
    withhold = ctx->h_devpatches[ctx->dbg.patch].flagBase + ctx->dbg.elem;
  return SysView{ctx->d_madof, ctx->d_meqn, ctx->nceq ? ctx->d_c0 : nullptr, ctx->d_colptr,
                 ctx->d_rowidx, ctx->d_K, ctx->d_b, ctx->d_counters, ctx->d_freeBefore,
                 ctx->d_flags, ctx->dbg.flagSpin ? ctx->dbg.flagSpin : kGenFlagSpin, withhold};
}

// The kernel sequence of one assembly in four segments -- prologue (zeroing,
// basis tables), element kernels and generic volume passes, gathers, face
// passes -- each captured once into a CUDA graph; the timing events are
// recorded between the graph launches.
static ifemgpu_status enqueueSegment(ifemgpu_ctx* ctx, int seg)
{
  cudaStream_t s = ctx->stream;
  if (seg == 0) {
    // the gather writes every entry of the tensor-core patches' columns; the
    // generic kernels add into a zeroed system
    if (ctx->zeroSystem) {
      IFEMGPU_CUDA(ctx, cudaMemsetAsync(ctx->d_K, 0, sizeof(double) * ctx->nnz, s));
      IFEMGPU_CUDA(ctx, cudaMemsetAsync(ctx->d_b, 0, sizeof(double) * ctx->neq, s));
    }
    IFEMGPU_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, sizeof(unsigned long long) * 4, s));
    if (ctx->nflags)
      IFEMGPU_CUDA(ctx, cudaMemsetAsync(ctx->d_flags, 0, sizeof(int) * ctx->nflags, s));
    const int np = (int)ctx->h_devpatches.size();
    if (np)
      k_basis_tables<<<(ctx->basisWork + 127) / 128, 128, 0, s>>>(ctx->d_patches, ctx->d_basisStart,
                                                                  np);
    IFEMGPU_CUDA(ctx, cudaGetLastError());
    return IFEMGPU_OK;
  }
  SysView S = sysView(ctx);
  const bool split = ctx->opts.ke_precision == IFEMGPU_KE_SPLIT_TF32;
  if (seg == 1) {  // element kernels of the tensor-core patches
    for (const Pass& p : ctx->passes) {
      if (!p.tc) continue;
      if (p.tcDeg == kTcElast3) IFEMGPU_TRY(tcElast3Launch(ctx, p));
      else if (p.tcDeg) IFEMGPU_TRY(tcPoissonLaunch(ctx, p, p.tcDeg));
      else IFEMGPU_TRY(tcLaunchVolume(ctx, p, 0));
    }
  }
  if (seg == 2) {  // their gathers
    for (const GatherList& g : ctx->gathers) IFEMGPU_TRY(gatherLaunch(ctx, g));
    return IFEMGPU_OK;
  }
  for (const Pass& p : ctx->passes) {
    if (p.tc) continue;
    if ((p.face != 0) != (seg == 3)) continue;
    if ((p.persistent && !ctx->useFlow) || (p.altColour && ctx->useFlow)) continue;
    if (p.persistent && split)
      k_volume_gen_flow<float><<<std::min(p.count, ctx->genGrid), 256, p.smem, s>>>(
          ctx->d_patches, ctx->d_items + p.first, p.count, S);
    else if (p.persistent)
      k_volume_gen_flow<double><<<std::min(p.count, ctx->genGrid), 256, p.smem, s>>>(
          ctx->d_patches, ctx->d_items + p.first, p.count, S);
    else if (!p.face && split)
      k_volume_gen<float><<<p.count, 256, p.smem, s>>>(ctx->d_patches, ctx->d_items + p.first, S);
    else if (!p.face)
      k_volume_gen<double><<<p.count, 256, p.smem, s>>>(ctx->d_patches, ctx->d_items + p.first, S);
    else
      k_face_fp64<<<p.count, 128, p.smem, s>>>(ctx->d_patches, ctx->d_items + p.first,
                                               ctx->d_neumann, S);
    IFEMGPU_CUDA(ctx, cudaGetLastError());
  }
  return IFEMGPU_OK;
}

// Autotuner of the persistent pass, run once before the first assembly is
// captured: for every (degree, dim) group of FP32 Poisson patches the register
// tile of the element matrix (2 x 2 or 4 x 4 node pairs per thread), then the
// grid (1 .. the occupancy limit of blocks per SM), each candidate timed with
// device events on a full pass (prologue untimed); the fastest is kept.
static ifemgpu_status autotune(ifemgpu_ctx* ctx)
{
  ctx->tuned = true;
  ctx->tuneLog.clear();
  const Pass* pp = nullptr;
  for (const Pass& p : ctx->passes)
    if (p.persistent) pp = &p;
  if (!pp) return IFEMGPU_OK;
  const bool split = ctx->opts.ke_precision == IFEMGPU_KE_SPLIT_TF32;
  cudaStream_t s = ctx->stream;
  SysView S = sysView(ctx);
  const int np = (int)ctx->h_devpatches.size();
  // grid > 0: the persistent pass with that grid; grid = 0: its colour passes
  auto timePass = [&](int grid, float* ms) -> ifemgpu_status {
    float best = 1e30f;
    for (int rep = 0; rep < 2; rep++) {
      IFEMGPU_TRY(enqueueSegment(ctx, 0));
      IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
      if (grid > 0 && split)
        k_volume_gen_flow<float><<<std::min(pp->count, grid), 256, pp->smem, s>>>(
            ctx->d_patches, ctx->d_items + pp->first, pp->count, S);
      else if (grid > 0)
        k_volume_gen_flow<double><<<std::min(pp->count, grid), 256, pp->smem, s>>>(
            ctx->d_patches, ctx->d_items + pp->first, pp->count, S);
      else
        for (const Pass& p : ctx->passes) {
          if (!p.altColour) continue;
          if (split)
            k_volume_gen<float><<<p.count, 256, p.smem, s>>>(ctx->d_patches, ctx->d_items + p.first, S);
          else
            k_volume_gen<double><<<p.count, 256, p.smem, s>>>(ctx->d_patches, ctx->d_items + p.first, S);
        }
      IFEMGPU_CUDA(ctx, cudaGetLastError());
      IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
      IFEMGPU_CUDA(ctx, cudaEventSynchronize(ctx->ev[1]));
      float t = 0.f;
      IFEMGPU_CUDA(ctx, cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[1]));
      best = std::min(best, t);
    }
    *ms = best;
    return IFEMGPU_OK;
  };
  auto pushPatches = [&]() -> ifemgpu_status {
    IFEMGPU_CUDA(ctx, cudaMemcpy(ctx->d_patches, ctx->h_devpatches.data(),
                                 sizeof(DevPatch) * np, cudaMemcpyHostToDevice));
    return IFEMGPU_OK;
  };
  // groups of FP32 Poisson patches by (degree, dim)
  std::vector<std::pair<int, int>> keys;
  for (int pi = 0; pi < np; pi++) {
    const DevPatch& D = ctx->h_devpatches[pi];
    if (!split || !ctx->onFlow[pi] || D.kind != IFEMGPU_POISSON || ctx->nceq) continue;
    const std::pair<int, int> k{std::max({D.p[0], D.p[1], D.p[2]}), D.dim};
    if (std::find(keys.begin(), keys.end(), k) == keys.end()) keys.push_back(k);
  }
  for (const auto& k : keys) {
    int bestTile = 4;
    float bestMs = 1e30f;
    for (int tile : {4, 2}) {
      for (int pi = 0; pi < np; pi++) {
        DevPatch& D = ctx->h_devpatches[pi];
        if (ctx->onFlow[pi] && D.kind == IFEMGPU_POISSON &&
            std::max({D.p[0], D.p[1], D.p[2]}) == k.first && D.dim == k.second)
          D.tile = tile;
      }
      IFEMGPU_TRY(pushPatches());
      float ms = 0.f;
      IFEMGPU_TRY(timePass(ctx->genGrid, &ms));
      if (ms < bestMs) { bestMs = ms; bestTile = tile; }
    }
    for (int pi = 0; pi < np; pi++) {
      DevPatch& D = ctx->h_devpatches[pi];
      if (ctx->onFlow[pi] && D.kind == IFEMGPU_POISSON &&
          std::max({D.p[0], D.p[1], D.p[2]}) == k.first && D.dim == k.second)
        D.tile = bestTile;
    }
    ctx->tuneLog.insert(ctx->tuneLog.end(), {k.first, k.second, bestTile});
  }
  IFEMGPU_TRY(pushPatches());
  const int maxPerSM = std::max(1, ctx->genGrid / std::max(1, ctx->numSMs));
  int bestGrid = ctx->genGrid;
  float bestMs = 1e30f;
  for (int perSM = 1; perSM <= maxPerSM; perSM++) {
    float ms = 0.f;
    IFEMGPU_TRY(timePass(perSM * ctx->numSMs, &ms));
    if (ms < bestMs) { bestMs = ms; bestGrid = perSM * ctx->numSMs; }
  }
  ctx->genGrid = bestGrid;
  ctx->tuneLog.insert(ctx->tuneLog.end(), {0, 0, bestGrid});
  // persistent launch or one launch per colour (forced by the context option)
  float colourMs = 0.f;
  IFEMGPU_TRY(timePass(0, &colourMs));
  ctx->useFlow = ctx->opts.colour_passes == 2 || (ctx->opts.colour_passes == 0 && bestMs <= colourMs);
  ctx->tuneLog.insert(ctx->tuneLog.end(), {-1, (int)(bestMs * 1000.f), (int)(colourMs * 1000.f)});
  if (ctx->opts.verbose) {
    for (size_t i = 0; i + 2 < ctx->tuneLog.size(); i += 3) {
      const int* t = ctx->tuneLog.data() + i;
      if (t[0] > 0) std::printf("ifemgpu autotune: p=%d dim=%d tile %d\n", t[0], t[1], t[2]);
      else if (t[0] == 0) std::printf("ifemgpu autotune: persistent grid %d\n", t[2]);
      else std::printf("ifemgpu autotune: persistent %.3f ms, per colour %.3f ms -> %s\n",
                       t[1] * 1e-3, t[2] * 1e-3, ctx->useFlow ? "persistent" : "per colour");
    }
  }
  return IFEMGPU_OK;
}

// Every kernel of one assembly on the context's stream, without timing events
// (for the capture of a whole assemble -> solve step); the autotuner has run.
ifemgpu_status enqueueAssembly(ifemgpu_ctx* ctx)
{
  if (!ctx->tuned) return setError(ctx, IFEMGPU_NOT_READY, "internal: assembly not tuned");
  bool hasSeg[4] = {true, false, !ctx->gathers.empty(), false};
  for (const Pass& p : ctx->passes) hasSeg[p.face ? 3 : 1] = true;
  for (int seg = 0; seg < 4; seg++)
    if (hasSeg[seg]) IFEMGPU_TRY(enqueueSegment(ctx, seg));
  return IFEMGPU_OK;
}

ifemgpu_status launchAssembly(ifemgpu_ctx* ctx)
{
  cudaStream_t s = ctx->stream;
  if (!ctx->tuned) IFEMGPU_TRY(autotune(ctx));
  bool hasSeg[4] = {true, false, !ctx->gathers.empty(), false};
  for (const Pass& p : ctx->passes) hasSeg[p.face ? 3 : 1] = true;
  for (int seg = 0; seg < 4; seg++) {
    if (ctx->graphExec[seg] || !hasSeg[seg]) continue;
    IFEMGPU_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    ifemgpu_status st = enqueueSegment(ctx, seg);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (st != IFEMGPU_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    IFEMGPU_CUDA(ctx, e);
    ctx->graph[seg] = g;
    IFEMGPU_CUDA(ctx, cudaGraphInstantiate(&ctx->graphExec[seg], g, 0));
  }
  for (int seg = 0; seg < 4; seg++) {
    IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->ev[seg], s));
    if (hasSeg[seg]) IFEMGPU_CUDA(ctx, cudaGraphLaunch(ctx->graphExec[seg], s));
  }
  IFEMGPU_CUDA(ctx, cudaEventRecord(ctx->ev[4], s));
  ctx->assemblies++;
  int used = 0;
  for (const Pass& p : ctx->passes)
    used += !((p.persistent && !ctx->useFlow) || (p.altColour && ctx->useFlow));
  ctx->launches_per_assembly = (ctx->h_devpatches.empty() ? 0 : 1) + used + (int)ctx->gathers.size();
  return IFEMGPU_OK;
}

}  // namespace ifemgpu
