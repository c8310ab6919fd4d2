// umma.cuh - inline-PTX wrappers for the Blackwell (sm_100 family) tensor-core path:
// mbarriers, bulk async copies (TMA engine), tensor memory (TMEM) and tcgen05.mma.
//
// All waits are bounded: a wait that exceeds its iteration limit returns false
// and the caller records an error word and winds down; nothing traps.
#pragma once

#include <stdint.h>

namespace gdft {
namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// One bounded wait step: the thread suspends until the phase completes or
// kWaitHintNs nanoseconds pass (the suspend-time hint of try_wait), then
// reports whether the phase completed.
constexpr uint32_t kWaitHintNs = 1000;
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(kWaitHintNs)
      : "memory");
  return ok != 0;
}

// Iteration limit of every wait: with each step suspending for up to
// kWaitHintNs, about a second before a wait gives up; a healthy pipeline's
// hand-offs complete within microseconds.  (An earlier form polled and slept
// 64 ns between polls after the 64th: the wake-up latency cost 1-2 % of the
// tensor-core kernels' time.)
constexpr uint32_t kWaitLimit = 1u << 20;

// Returns false when `limit` steps pass without the phase completing.
__device__ __forceinline__ bool mbar_wait_n(uint64_t *bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) { return mbar_wait_n(bar, parity, kWaitLimit); }
__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Warp-uniform bounded wait: every lane waits on the phase itself (and so has
// acquire ordering); all lanes return the same value.
__device__ __forceinline__ bool warp_wait(uint64_t *bar, uint32_t parity) {
  const bool ok = mbar_wait(bar, parity);
  return __all_sync(0xffffffffu, ok) != 0;
}

// ------------------------------------------------------- bulk async copies
// One contiguous global -> shared copy through the TMA engine, completing
// `bytes` of transaction count on `bar`.  Both addresses 16-byte aligned,
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// ---------------------------------------------------------------- TMEM
// Allocate `ncols` (power of two >= 32) TMEM columns; one full warp executes
// this; the base address is written to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive 32-bit TMEM columns of this thread's lane (warp-collective).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Issue a 32-column TMEM load without waiting (pair with tmem_ld_wait()).
__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// Wait, then route the destination registers through ordered empty asm
// statements so that no use of them can be scheduled before the wait.
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&a)[32]) {
  tmem_ld_wait();
#pragma unroll
  for (int i = 0; i < 32; ++i) asm volatile("" : "+r"(a[i]));
}
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&a)[32], uint32_t (&b)[32]) {
  tmem_ld_wait();
#pragma unroll
  for (int i = 0; i < 32; ++i) asm volatile("" : "+r"(a[i]), "+r"(b[i]));
}

// 16 consecutive 32-bit TMEM columns of this thread's lane (warp-collective).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Issue a 16-column TMEM load without waiting.
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&a)[16]) {
  tmem_ld_wait();
#pragma unroll
  for (int i = 0; i < 16; ++i) asm volatile("" : "+r"(a[i]));
}
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&a)[16], uint32_t (&b)[16]) {
  tmem_ld_wait();
#pragma unroll
  for (int i = 0; i < 16; ++i) asm volatile("" : "+r"(a[i]), "+r"(b[i]));
}

// Store 32 consecutive 32-bit TMEM columns of this thread's lane (warp-collective).
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float (&v)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
      "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
      "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])),
      "r"(__float_as_uint(v[11])), "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])),
      "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15])), "r"(__float_as_uint(v[16])),
      "r"(__float_as_uint(v[17])), "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])),
      "r"(__float_as_uint(v[20])), "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])),
      "r"(__float_as_uint(v[23])), "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])),
      "r"(__float_as_uint(v[26])), "r"(__float_as_uint(v[27])), "r"(__float_as_uint(v[28])),
      "r"(__float_as_uint(v[29])), "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
      : "memory");
}
// Store 16 consecutive 32-bit TMEM columns of this thread's lane (warp-collective).
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// ------------------------------------------------------------- descriptors
// Shared-memory matrix descriptor, no swizzle, K-major canonical layout:
// core matrices of 8 rows x 16 bytes (128 contiguous bytes); `lbo` is the byte
// distance between core matrices adjacent along K, `sbo` between core
// matrices adjacent along M/N.  Bits 46-47 hold the descriptor version (1).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor for kind::tf32 with FP32 accumulation, both operands
// K-major: D format F32 (bits 4-5 = 1), A/B format TF32 (bits 7-9, 10-12 = 2),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive once on `bar` when all previously issued tcgen05.mma of this thread complete.
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// ------------------------------------------------------------ TF32 split
// Round an FP32 value to TF32 (10 explicit mantissa bits), nearest-even.
__device__ __forceinline__ float tf32_rn(float x) {
  uint32_t u = __float_as_uint(x);
  if ((u & 0x7F800000u) != 0x7F800000u) {  // finite
    u += 0x0FFFu + ((u >> 13) & 1u);
    u &= 0xFFFFE000u;
  }
  return __uint_as_float(u);
}
// x ~= hi + lo with hi, lo TF32 (about 22 significant bits together).
__device__ __forceinline__ void split_tf32(double x, float &hi, float &lo) {
  hi = tf32_rn((float)x);
  lo = tf32_rn((float)(x - (double)hi));
}
__device__ __forceinline__ void split_tf32f(float x, float &hi, float &lo) {
  hi = tf32_rn(x);
  lo = tf32_rn(x - hi);
}

// ------------------------------------------------------ packed FP32 pairs
// Two FP32 values in one 64-bit register, added or subtracted by one
// instruction (add/sub.rn.f32x2), each lane rounded to nearest like the scalar op.
__device__ __forceinline__ uint64_t pk2(uint32_t lo, uint32_t hi) {
  uint64_t d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "r"(lo), "r"(hi));
  return d;
}
__device__ __forceinline__ void unpk2(uint64_t v, uint32_t &lo, uint32_t &hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// ------------------------------------------- block-scaled three-slice split
// x = hi + lo + lo2 (+ about 2^-33 of the block row's largest magnitude m),
// where hi is x rounded to the row's quantum q = 2^(E - 9), 2^(E-1) <= m < 2^E
// (|hi| <= 512 q: at most ten significant bits), and lo, lo2 are TF32
// roundings of the remainders.  All hi values of a row share q, so a sum of
// 32 products hi_a * hi_b of two such rows is a multiple of q_a q_b below
// 2^23 q_a q_b: exact in an FP32 accumulator, whatever the tensor core's
// alignment and truncation.  Rows whose quantum would leave the FP32 normal
// range keep hi = 0.
struct Quant {
  float q, inv;
};
__device__ __forceinline__ Quant quant(float m) {
  const uint32_t eb = (__float_as_uint(m) >> 23) & 0xFFu;  // m in [2^(eb-127), 2^(eb-126))
  Quant u;
  if (eb >= 9u && eb < 255u) {
    u.q = __uint_as_float((eb - 8u) << 23);     // 2^(eb - 135)
    u.inv = __uint_as_float((262u - eb) << 23);  // 2^(135 - eb)
  } else {
    u.q = 0.0f;
    u.inv = 0.0f;
  }
  return u;
}
// The same from the biased FP32 exponent field of the row maximum alone.
__device__ __forceinline__ Quant quant_eb(uint32_t eb) {
  Quant u;
  if (eb >= 9u && eb < 255u) {
    u.q = __uint_as_float((eb - 8u) << 23);
    u.inv = __uint_as_float((262u - eb) << 23);
  } else {
    u.q = 0.0f;
    u.inv = 0.0f;
  }
  return u;
}
// FP32 source: every step is exact except the two TF32 roundings.
__device__ __forceinline__ void split3(float x, Quant u, float &hi, float &lo, float &lo2) {
  hi = rintf(x * u.inv) * u.q;
  const float r = x - hi;
  lo = tf32_rn(r);
  lo2 = tf32_rn(r - lo);
}
// FP64 source (the remainders are taken in FP64).
__device__ __forceinline__ void split3(double x, Quant u, float &hi, float &lo, float &lo2) {
  hi = (float)(rint(x * (double)u.inv) * (double)u.q);
  const double r = x - (double)hi;
  lo = tf32_rn((float)r);
  lo2 = tf32_rn((float)(r - (double)lo));
}

// Byte offset of element (row, k) inside a K-major no-swizzle block of
// `rows` x 32 fp32 (core matrices 8 rows x 4 elements; row-groups of 8 at
// 1024 bytes, k-groups of 4 at 128 bytes): LBO = 128, SBO = 1024.
__host__ __device__ constexpr uint32_t kblock_off(int row, int k) {
  return (uint32_t)(((row >> 3) * 8 + (k >> 2)) * 128 + (row & 7) * 16 + (k & 3) * 4);
}
constexpr uint32_t kBlockLBO = 128, kBlockSBO = 1024;
// A block of 128 rows x 32 fp32 = 16 KB.
constexpr uint32_t kBlockBytes = 128 * 32 * 4;

// Writes one row (32 K values) of a three-slice block set [hi | lo | lo2]
// (three consecutive 16 KB blocks), quantised on the row's own maximum.
template <class T>
__device__ __forceinline__ void store_row3(float *blk3, int row, const T (&v)[32]) {
  T m = 0;
#pragma unroll
  for (int k = 0; k < 32; ++k) m = fmax(m, fabs(v[k]));
  const Quant u = quant((float)m);
#pragma unroll
  for (int k4 = 0; k4 < 8; ++k4) {
    float4 h, l, l2;
    split3(v[4 * k4 + 0], u, h.x, l.x, l2.x);
    split3(v[4 * k4 + 1], u, h.y, l.y, l2.y);
    split3(v[4 * k4 + 2], u, h.z, l.z, l2.z);
    split3(v[4 * k4 + 3], u, h.w, l.w, l2.w);
    const uint32_t off = kblock_off(row, 4 * k4) / 4;
    *(float4 *)(blk3 + off) = h;
    *(float4 *)(blk3 + kBlockBytes / 4 + off) = l;
    *(float4 *)(blk3 + kBlockBytes / 2 + off) = l2;
  }
}

}  // namespace umma
}  // namespace gdft
