// tcgen05.cuh -- building blocks of the tensor-core kernels (sm_103a):
// inline-PTX wrappers for mbarriers, TMEM allocation, tcgen05.mma / commit /
// ld, bulk L2 prefetch, the 128-byte-swizzled K-major operand layout and its
// descriptors, bounded waits, and the host-side split-BF16 image of a block
// matrix.
#pragma once

#include <stdint.h>
#include <string.h>

#include "common.cuh"

namespace qcs {

constexpr int kTcM = 128;                       // state columns per tile = UMMA M = TMEM lanes
// The final drain of a kernel's MMAs always waits this long (its MMAs
// complete in microseconds); the pipeline waits take the launch's limit.
constexpr long long kWaitCycles = kDefaultWaitCycles;  // ~2 s at 2 GHz

// Byte offset of bf16 element (r, k) in a K-major operand of R rows laid out
// in 128-byte swizzle atoms (8 rows x 64 elements, 16-byte chunks permuted by
// XOR with the row), atoms along K R*128 bytes apart.
__host__ __device__ __forceinline__ int sw128_offset(int r, int k, int R) {
  const int kb = k >> 6, chunk = (k >> 3) & 7, e = k & 7;
  return kb * (R * 128) + (r >> 3) * 1024 + (r & 7) * 128 + ((chunk ^ (r & 7)) << 4) + e * 2;
}

// The same for 64-byte swizzle atoms (8 rows x 32 elements, 16-byte chunks
// permuted by XOR with bits 1-2 of the row): an operand whose K extent is 32.
__host__ __device__ __forceinline__ int sw64_offset(int r, int k) {
  const int chunk = (k >> 3) & 3, e = k & 7;
  return (r >> 3) * 512 + (r & 7) * 64 + ((chunk ^ ((r >> 1) & 3)) << 4) + e * 2;
}

// ---- PTX wrappers ---------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
// Bulk prefetch of [p, p + bytes) into L2 (p 16-byte aligned, bytes a
// multiple of 16); no destination, no completion to wait for.
__device__ __forceinline__ void prefetch_l2(const void *p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ uint32_t mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok;
}
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
// D (TMEM) [+]= A (smem desc) * B (smem desc)^T, bf16 in, fp32 accumulate.
__device__ __forceinline__ void umma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrive on `bar` once every MMA issued so far by this thread has completed.
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}
// 32 consecutive TMEM columns of this warp's 32 lanes; waits for completion
// inside the same statement so the registers are never read early.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *out) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) out[i] = __uint_as_float(r[i]);
}

// 16 consecutive TMEM columns of this warp's 32 lanes (for kernels with few
// registers a thread).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *out) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) out[i] = __uint_as_float(r[i]);
}

// Two loads of 16 columns (at ta and tb) under one completion wait.
__device__ __forceinline__ void tmem_ld16x2(uint32_t ta, uint32_t tb, float *a, float *b) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%32];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,"
      "%28,%29,%30,%31}, [%33];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(ta), "r"(tb)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) {
    a[i] = __uint_as_float(r[i]);
    b[i] = __uint_as_float(r[16 + i]);
  }
}

// 64 consecutive TMEM columns of this warp's 32 lanes in one instruction,
// again waiting inside the same statement (half the waits of two x32 loads).
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float *out) {
  uint32_t r[64];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 64; i++) out[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO); the leading offset is unused for this layout.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;             // LBO (ignored for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;   // SBO
  d |= (uint64_t)1 << 46;             // descriptor version for tcgen05
  d |= (uint64_t)2 << 61;             // SWIZZLE_128B
  return d;
}

// The same for the 64-byte swizzle: 8-row groups 512 bytes apart.
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;             // LBO (ignored for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;    // SBO
  d |= (uint64_t)1 << 46;             // descriptor version for tcgen05
  d |= (uint64_t)4 << 61;             // SWIZZLE_64B
  return d;
}

// Instruction descriptor: kind::f16, A = B = bf16, D = fp32, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// Bounded mbarrier wait: at most `limit` clock cycles (the launch's wait
// limit, kWaitCycles unless a debug override shortened it).  Returns false
// when the CTA is aborting.
static __device__ __noinline__ bool wait_bar(uint32_t bar, uint32_t parity, volatile int *abort_flag,
                                      int *err, int where, long long limit) {
  long long t0 = clock64();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (clock64() - t0 > limit) {
      *abort_flag = 1;
      atomicExch(err, where);
      return false;
    }
  }
}

// ---- host: split-BF16 images of block matrices ------------------------------

static inline uint16_t bf16_rn(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

static inline float bf16_to_float(uint16_t h) {
  uint32_t u = (uint32_t)h << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

// Block matrix u (K x K complex, row-major) -> swizzled hi/lo image of B.
template <int KA>
static void make_image(const double *u, uint8_t *img) {
  constexpr int N = 2 * KA, B_BYTES = N * 2 * KA * 2;
  memset(img, 0, 2 * B_BYTES);
  uint16_t *hi = reinterpret_cast<uint16_t *>(img);
  uint16_t *lo = reinterpret_cast<uint16_t *>(img + B_BYTES);
  for (int ao = 0; ao < KA; ao++)
    for (int ai = 0; ai < KA; ai++) {
      const double re = u[2 * (ao * KA + ai)], im = u[2 * (ao * KA + ai) + 1];
      const double blk[2][2] = {{re, -im}, {im, re}};
      for (int co = 0; co < 2; co++)
        for (int ci = 0; ci < 2; ci++) {
          const int o = 2 * ao + co, i = 2 * ai + ci;
          const double x = blk[co][ci];
          const uint16_t h = bf16_rn((float)x);
          const uint16_t l = bf16_rn((float)(x - (double)bf16_to_float(h)));
          const int off = sw128_offset(o, i, N) / 2;
          hi[off] = h;
          lo[off] = l;
        }
    }
}

// Block matrix u (128 x 128 complex, row-major) -> the four swizzled
// operands of the k = 7 kernel: Re U hi, Re U lo, Im U hi, Im U lo, each
// N = 128 output rows x K = 128 inputs.
static void make_image7(const double *u, uint8_t *img) {
  constexpr int KA = 128, U_BYTES = KA * KA * 2;
  memset(img, 0, 4 * U_BYTES);
  uint16_t *op[4];
  for (int o = 0; o < 4; o++) op[o] = reinterpret_cast<uint16_t *>(img + o * U_BYTES);
  for (int ao = 0; ao < KA; ao++)
    for (int ai = 0; ai < KA; ai++) {
      const int off = sw128_offset(ao, ai, KA) / 2;
      for (int part = 0; part < 2; part++) {
        const double x = u[2 * (ao * KA + ai) + part];
        const uint16_t h = bf16_rn((float)x);
        op[2 * part][off] = h;
        op[2 * part + 1][off] = bf16_rn((float)(x - (double)bf16_to_float(h)));
      }
    }
}

}  // namespace qcs
