// hp3dg_tc.cuh -- inline-PTX helpers for the tcgen05 kernels (sm_103a):
// mbarriers with bounded waits, bulk async copies, UMMA shared-memory
// descriptors, BF16 MMA issue / commit and TMEM loads.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hp3dg {

constexpr long TC_WAIT_LIMIT = 1L << 24;  // bounded mbarrier waits

// ---------------------------------------------------------------------------
// PTX helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false if the limit was hit or another role aborted
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, volatile int* abort_) {
  for (long it = 0; it < TC_WAIT_LIMIT; ++it) {
    if (mbar_try(a, parity)) return true;
    if ((it & 255) == 255 && *abort_) return false;
  }
  return false;
}
// the same with a caller-chosen iteration limit
__device__ __forceinline__ bool mbar_wait_n(uint32_t a, uint32_t parity, volatile int* abort_,
                                            long limit) {
  for (long it = 0; it < limit; ++it) {
    if (mbar_try(a, parity)) return true;
    if ((it & 255) == 255 && *abort_) return false;
  }
  return false;
}
// wait without the abort test (draining a role's own asynchronous work)
__device__ __forceinline__ bool mbar_drain(uint32_t a, uint32_t parity, long limit) {
  for (long it = 0; it < limit; ++it)
    if (mbar_try(a, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes,
                                          uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(dst), "l"((uint64_t)src), "r"(bytes), "r"(mbar)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// shared-memory matrix descriptor: K-major, no swizzle (canonical interleaved
// layout): 8-row x 16-byte core matrices, K-direction core matrices 128 bytes
// apart (LBO), 8-row groups 256 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc_kmajor(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)(128 >> 4) << 16;        // LBO
  d |= (uint64_t)(256 >> 4) << 32;        // SBO
  d |= (uint64_t)1 << 46;                 // descriptor version
  return d;                               // layout type 0 = no swizzle
}
__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
      : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}


// TMEM load of 16 columns without waiting: issue several, then tmem_wait()
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// TMEM load of 8 columns without waiting
__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
}

// ---------------------------------------------------------------------------
// split-BF16 digit operands
// ---------------------------------------------------------------------------
// exponent e with max |v| = m 2^e, m in [0.5, 1), from the largest magnitude
// bit pattern (magnitudes of finite doubles order like their bits); 0 for 0
__device__ __forceinline__ int row_exponent(unsigned long long maxbits) {
  return maxbits ? (int)(maxbits >> 52) - 1022 : 0;
}
__device__ __forceinline__ unsigned long long mag_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

// X = round(v 2^(radix*digits - e)) for |v| < 2^e, as an integer, from the bits
__device__ __forceinline__ long long fixed_of(double v, int e, int fbits) {
  const long long bits = __double_as_longlong(v);
  const int E = (int)((bits >> 52) & 0x7ff);
  if (E == 0) return 0;
  const long long M = (bits & 0xfffffffffffffLL) | (1LL << 52);
  const int sh = E - 1075 - e + fbits;
  long long x = 0;
  if (sh >= 0) x = M << sh;
  else if (sh > -54) x = (M + (1LL << (-sh - 1))) >> (-sh);
  return bits < 0 ? -x : x;
}

// V 2^sc rounded to nearest (ties to even), assembled from the bits of V
// without an FP64 instruction (GB300 issues FP64 and its conversions at
// about 2 per clock per SM); scales outside the normal range take ldexp
__device__ __forceinline__ double scaled_i64(long long V, int sc) {
  if (V == 0) return 0.0;
  const unsigned long long sb = (unsigned long long)V & 0x8000000000000000ull;
  unsigned long long u = V < 0 ? (unsigned long long)(-V) : (unsigned long long)V;
  const int lz = __clzll((long long)u);
  const int eb = 63 - lz + sc + 1023;  // biased exponent of the leading bit
  if (eb < 1 || eb > 2045) return ldexp((double)V, sc);
  u <<= lz;
  unsigned long long m = u >> 11;  // 53 bits, leading bit at 52
  const unsigned long long r = u & 0x7ffull;
  m += (r > 0x400ull || (r == 0x400ull && (m & 1ull))) ? 1ull : 0ull;
  return __longlong_as_double((long long)(sb | (((unsigned long long)(eb - 1) << 52) + m)));
}

// balanced radix-2^R digits of 8 fixed-point integers, written as one
// 16-byte core-matrix row per digit (least significant digit first)
__device__ __forceinline__ void store_digits8(long long* X, int R, int D, uint8_t* dst,
                                              size_t digit_stride) {
  const long long half = 1LL << (R - 1);
  for (int dg = D - 1; dg >= 0; --dg) {
    uint32_t h[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      long long d;
      if (dg > 0) {
        const long long q = (X[t] + half) >> R;
        d = X[t] - (q << R);
        X[t] = q;
      } else {
        d = X[t];
      }
      h[t] = __float_as_uint((float)(int)d) >> 16;  // exact in BF16
    }
    uint4 w;
    w.x = h[0] | (h[1] << 16);
    w.y = h[2] | (h[3] << 16);
    w.z = h[4] | (h[5] << 16);
    w.w = h[6] | (h[7] << 16);
    *(uint4*)(dst + (size_t)dg * digit_stride) = w;
  }
}

// byte offset of (row, 8-wide K group g) in a canonical tile set with `nrows` rows
__host__ __device__ __forceinline__ size_t tile_off(int row, int g, int nrows) {
  return (size_t)(g >> 1) * nrows * 32 + (size_t)(row >> 3) * 256 + (size_t)(g & 1) * 128 +
         (size_t)(row & 7) * 16;
}

}  // namespace hp3dg
