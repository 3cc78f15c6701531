// tc_common.cuh -- inline-PTX building blocks for the sm_103a tensor-core
// path: tcgen05 MMA (kind::tf32, and kind::f16 with BF16 operands;
// cta_group::1), tensor-memory allocation and loads, mbarrier waits with an
// iteration bound, bulk copies, and the shared-memory operand layout.
//
// Operand layout ("K-major, no swizzle"): a tile of R rows x 128 bytes of K
// (32 FP32/TF32 or 64 BF16 elements) is stored as core matrices of 8 rows x
// 16 bytes; the core matrices of one 8-row group are adjacent along K
// (leading byte offset 128 B) and the 8-row groups follow each other every
// 1024 B (stride byte offset).
#pragma once

#include <cstdint>

namespace ifemgpu {
namespace tc {

constexpr int kK = 32;                 // K extent of one operand tile (elements)
constexpr uint32_t kLBO = 128;         // bytes between K-adjacent core matrices
constexpr uint32_t kSBO = 1024;        // bytes between 8-row groups
constexpr uint32_t kSpinLimit = 1u << 22;  // bounded mbarrier polling

__device__ __forceinline__ uint32_t smemAddr(const void* p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// float offset of (row r, k) in a K-major tile with kK = 32
__device__ __forceinline__ int kmaj(int r, int k)
{
  return (r >> 3) * 256 + (k >> 2) * 32 + (r & 7) * 4 + (k & 3);
}

// shared-memory matrix descriptor (sm_100 family): start address, LBO, SBO
// (all >> 4), descriptor version 1 at bit 46, no swizzle, base offset 0.
__device__ __forceinline__ uint64_t smemDesc(uint32_t saddr)
{
  return static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4) |
         (static_cast<uint64_t>(kLBO >> 4) << 16) |
         (static_cast<uint64_t>(kSBO >> 4) << 32) | (1ull << 46);
}

// instruction descriptor, kind::tf32: D f32 (bits 4-5 = 1), A and B tf32
// (bits 7-9 and 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t instrDescTF32(int M, int N)
{
  return (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void mmaTF32(uint32_t tmemD, uint64_t adesc, uint64_t bdesc,
                                        uint32_t idesc, uint32_t accumulate)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n"
      :
      : "r"(tmemD), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// instruction descriptor, kind::f16 with BF16 A and B (format 1 at bits 7-9
// and 10-12), D f32, both K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t instrDescBF16(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void mmaBF16(uint32_t tmemD, uint64_t adesc, uint64_t bdesc,
                                        uint32_t idesc, uint32_t accumulate)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
      :
      : "r"(tmemD), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mmaCommit(uint32_t mbar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :
               : "r"(mbar)
               : "memory");
}

__device__ __forceinline__ void mbarInit(uint32_t mbar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" : : "r"(mbar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" : : : "memory");
}

__device__ __forceinline__ bool mbarTryWait(uint32_t mbar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Polls the barrier phase at most `limit` times (each try_wait may suspend
// the thread for a while); false on give-up.
__device__ __forceinline__ bool mbarWait(uint32_t mbar, uint32_t parity, uint32_t limit = kSpinLimit)
{
  for (uint32_t i = 0; i < limit; i++)
    if (mbarTryWait(mbar, parity)) return true;
  return false;
}

// TMA: one tiled 4D box global -> shared (destination 128-byte aligned,
// innermost coordinate 0), completing on an mbarrier that expects `bytes`.
__device__ __forceinline__ void mbarExpectTx(uint32_t mbar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
               : : "r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tmaLoad4d(uint32_t dst, const void* tmap, int c0, int c1, int c2,
                                          int c3, uint32_t mbar)
{
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];"
      : : "r"(dst), "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(mbar) : "memory");
}

// untiled bulk copy global -> shared of `bytes` (both addresses 16-byte
// aligned, bytes a multiple of 16), completing on an mbarrier
__device__ __forceinline__ void bulkLoad(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t mbar)
{
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      : : "r"(dst), "l"(src), "r"(bytes), "r"(mbar) : "memory");
}

// tensor maps written to global memory by copies before the launch: order
// them before their first use by the tensor-map proxy
__device__ __forceinline__ void tmapAcquire(const void* tmap)
{
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" : : "l"(tmap) : "memory");
}

__device__ __forceinline__ void fenceProxyAsync()
{
  asm volatile("fence.proxy.async.shared::cta;" : : : "memory");
}

__device__ __forceinline__ void tcFenceBefore()
{
  asm volatile("tcgen05.fence::before_thread_sync;" : : : "memory");
}

__device__ __forceinline__ void tcFenceAfter()
{
  asm volatile("tcgen05.fence::after_thread_sync;" : : : "memory");
}

// one warp: allocate ncols TMEM columns, base address written to smem slot
__device__ __forceinline__ void tmemAlloc(uint32_t* slot, uint32_t ncols)
{
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
               :
               : "r"(smemAddr(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" : : : "memory");
}

__device__ __forceinline__ void tmemDealloc(uint32_t taddr, uint32_t ncols)
{
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
               :
               : "r"(taddr), "r"(ncols)
               : "memory");
}

// 32 lanes x 16 columns of 32-bit words: thread t of the warp receives lane
// (quadrant base + t), columns col..col+15
__device__ __forceinline__ void tmemLoad16(uint32_t taddr, float* v)
{
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" : : : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Exact float -> double widening on the integer pipe (GB300's FP64 units run
// at a small fraction of the FP32 rate, and the conversion instruction uses
// them).  Normal numbers and zero are exact; subnormal floats (< 1.2e-38)
// flush to a signed zero; infinities and NaN keep their class.
__device__ __forceinline__ double widenF32(float f)
{
  const uint32_t b = __float_as_uint(f);
  const uint32_t mag = b & 0x7FFFFFFFu;
  // normal numbers: exponent rebias by 896 and mantissa shift by 29; zero and
  // subnormals to a signed zero; infinities and NaN keep their class
  uint32_t hi = (b & 0x80000000u) | ((mag >> 3) + (896u << 20));
  hi = mag < 0x00800000u ? (b & 0x80000000u) : hi;
  hi = mag >= 0x7F800000u ? ((b & 0x80000000u) | 0x7FF00000u | (mag & 0x007FFFFFu ? 0x80000u : 0u)) : hi;
  const uint32_t lo = mag < 0x00800000u ? 0u : (b << 29);
  return __hiloint2double((int)hi, (int)lo);
}

// Double -> float narrowing on the integer pipe, rounded to nearest even (the
// conversion instruction runs on the FP64 units, which are scarce on this
// GPU).  Results below the smallest normal float flush to a signed zero,
// results beyond the largest finite float become infinity, NaN stays NaN.
__device__ __forceinline__ float narrowF64(double d)
{
  const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
  const uint32_t sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FFu);
  const int ef = e - 1023 + 127;
  const uint32_t m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // top 23 mantissa bits
  const uint32_t rest = lo & 0x1FFFFFFFu;                  // the 29 bits rounded away
  uint32_t bits = ((uint32_t)(ef & 0xFF) << 23) | m;
  bits += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
  bits = ef <= 0 ? 0u : bits;
  bits = ef >= 255 ? 0x7F800000u : bits;
  bits = (e == 0x7FF && (((hi & 0xFFFFFu) | lo) != 0u)) ? 0x7FC00000u : bits;
  return __uint_as_float(sign | bits);
}

__device__ __forceinline__ void redAdd(double* p, double v)
{
  atomicAdd(p, v);  // result unused: compiles to an L2 reduction
}

// neighbour flags are polled with relaxed loads (served by L2); a thread that
// saw one issues a single acquire fence before the block's scatter
__device__ __forceinline__ int loadRelaxed(const int* p)
{
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void fenceAcquire()
{
  asm volatile("fence.acq_rel.gpu;" : : : "memory");
}

// acquire load of a flag already seen set: synchronises with the release
// store that set it without draining this thread's own outstanding
// reductions (which a full fence.acq_rel would wait for)
__device__ __forceinline__ int loadAcquire(const int* p)
{
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void storeRelease(int* p, int v)
{
  asm volatile("st.release.gpu.global.b32 [%0], %1;" : : "l"(p), "r"(v) : "memory");
}

// x = hi + lo with hi rounded to TF32 (10 explicit mantissa bits)
__device__ __forceinline__ void splitTF32(float x, float& hi, float& lo)
{
  const uint32_t b = __float_as_uint(x);
  hi = __uint_as_float((b + 0x1000u) & 0xFFFFE000u);
  lo = x - hi;
}

}  // namespace tc
}  // namespace ifemgpu
