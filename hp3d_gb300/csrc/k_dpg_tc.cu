// k_dpg_tc.cu -- the dense algebra of the DPG Maxwell element on tcgen05
// tensor cores: the steps ZPPTRF / ZTPTRS / ZHERK of elem_maxwell.F90:590-639
// and the condensation of the L2 fields (stc_fwd_herm, stc.F90:338-416) as one
// partial Cholesky factorization of the augmented Hermitian matrix
//     [[G, S], [S^H, 0]],  S = [B | l] with the trial unknowns ordered [Q | E | l],
// column panel by column panel (64 wide).  Eliminating the test unknowns
// leaves -Z = -X^H X (X = L^-1 S) in the trailing block; after the sign
// flip and the impedance penalty, eliminating the L2 fields Q leaves the
// Schur complement of the interface unknowns with its load.
//
// Per panel the FP64 work is the 64 x 64 diagonal block: its Cholesky factor
// L11 and W = L11^-H.  Every O(n^3) product -- the panel solve P := P W and
// the trailing update T -= P P^H, and the blocked backward substitution for
// ASchur -- is one kind of update
//     C (FP64 complex) = or -= A B^T,   K = 64 complex per step,
// computed from split-BF16 digits: each complex row vector of A and B is
// written as a real vector of length 128 (its real and imaginary parts in a
// "form": [re|im], [-im|re], [re|-im], [im|re] or [im|-re]) with one
// power-of-two scale per row and 7 balanced radix-2^7 digits of a 48-bit
// fixed-point value (every digit at most 2^6 in magnitude, exact in BF16).
// The real part of the product is A(form [re|im]) . B(one form), the
// imaginary part A . B(another form); each digit pair (p, q) with p + q <= 6
// lands in the FP32 TMEM accumulator of its level (sums below 2^22, exact).
// For A digit p one MMA (N up to 256) covers the B digits q = 0..6-p of both
// forms, whose levels p..6 are contiguous in TMEM.  The levels are
// recombined exactly in 64-bit integers and added to C with one rounding.
#include "hp3dg_kernels.h"
#include "hp3dg_tc.cuh"
#include "hp3dg_zla.cuh"

#include <string.h>

namespace hp3dg {

namespace {
using namespace zla;

constexpr int ZD = 7, ZR = 7;          // digits per operand, bits per digit
constexpr int ZK = 128;                // real-expanded K of one update (64 complex)
constexpr int ZGROUPS = ZK / 8;        // 8-wide K groups
constexpr int ZM = 128, ZN = 32;       // output tile
constexpr int ZA_BLK = ZM * ZK * 2;    // one A digit block (bytes)
constexpr int ZB_BLK = ZN * ZK * 2;    // one B digit block
constexpr int ZB_TILE = 2 * ZD * ZB_BLK;  // both B forms of one column tile
constexpr int ZFB = 48;                // fraction bits of the split (|v| < 2^e -> |X| <= 2^48)
constexpr int ZBROWS = 2 * ZD * ZN;    // rows of one B K-step: [digit q][form][32 rows]
constexpr int ZU_THREADS = 576;        // loader, MMA, 16 epilogue warps (4 per TMEM lane quarter)
constexpr int ZEPI = ZU_THREADS / 32 - 2;  // epilogue warps
constexpr int ZCG = ZN / 8 / (ZEPI / 4);   // 8-column groups per epilogue warp
constexpr int ZNABUF = 2;              // A digit buffers
constexpr uint32_t ZU_TMEM = 512;      // 7 levels x 2 parts x 32 columns = 448
constexpr size_t ZU_SMEM = ZNABUF * ZA_BLK + ZB_TILE + 1024;  // 177 KB: one CTA per SM

__host__ __device__ constexpr uint32_t zidesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

// value of the real-expanded vector of form f at position kk (kc complex
// entries; positions beyond them are zero)
__device__ __forceinline__ double form_value(const double2* s, int64_t sk, int kc, int f, int kk) {
  const int half = kk >= 64, k = kk & 63;
  if (k >= kc) return 0.0;
  const double2 z = s[(int64_t)k * sk];
  switch (f) {
    case 0: return half ? z.y : z.x;     // [re | im]
    case 1: return half ? z.x : -z.y;    // [-im | re]
    case 2: return half ? -z.y : z.x;    // [re | -im]
    case 3: return half ? z.x : z.y;     // [im | re]
    default: return half ? -z.x : z.y;   // [im | -re]
  }
}

struct ZSlice {
  const double2* src;
  int64_t src_estride;  // complex entries per element
  int64_t srow, sk;     // strides of the row index and of k
  int rows, rows_pad, kc;
  int nt;               // rows per tile block (128: A operand, 32: B operand)
  int nforms, form0, form1;
  uint8_t* dst;
  int64_t dst_estride;  // bytes per element
  int* ex;
  int ex_estride;
};

// one thread per (padded row, element): row exponent and the digits of each form
__global__ void k_zslice(ZSlice a) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  const int e = blockIdx.y;
  if (row >= a.rows_pad) return;
  const bool valid = row < a.rows;
  const double2* s = a.src + (int64_t)e * a.src_estride + (int64_t)row * a.srow;
  unsigned long long mx = 0;
  if (valid)
    for (int k = 0; k < a.kc; ++k) {
      const double2 z = s[(int64_t)k * a.sk];
      mx = max(mx, max(mag_bits(z.x), mag_bits(z.y)));
    }
  const int ex = row_exponent(mx);
  a.ex[(int64_t)e * a.ex_estride + row] = valid ? ex : 0;
  const int r = row % a.nt;
  const bool isB = a.nt == ZN;
  // A: [row tile][digit][canonical 128 x 128]; B: [column tile][canonical
  // 448 x 128], row (digit q, form, r) = 64 q + 32 form + r, so that the
  // digits q = 0..6-p of both forms are one N = (7 - p) 64 operand
  const size_t tile_bytes = isB ? (size_t)ZB_TILE : (size_t)ZD * a.nt * ZK * 2;
  const size_t dstride = isB ? (size_t)(2 * ZN / 8) * 256 : (size_t)a.nt * ZK * 2;
  uint8_t* base = a.dst + (int64_t)e * a.dst_estride + (size_t)(row / a.nt) * tile_bytes;
  for (int fi = 0; fi < a.nforms; ++fi) {
    const int f = fi == 0 ? a.form0 : a.form1;
    for (int g = 0; g < ZGROUPS; ++g) {
      long long X[8];
#pragma unroll
      for (int t = 0; t < 8; ++t)
        X[t] = valid ? fixed_of(form_value(s, a.sk, a.kc, f, 8 * g + t), ex, ZFB) : 0;
      uint8_t* dst = base + (isB ? tile_off(fi * ZN + r, g, ZBROWS) : tile_off(r, g, a.nt));
      store_digits8(X, ZR, ZD, dst, dstride);
    }
  }
}

// digits of 8 fixed-point integers (most significant first), as BF16 bits
__device__ __forceinline__ void digits8(long long* X, uint32_t (*h)[8]) {
  const long long half = 1LL << (ZR - 1);
  for (int dg = ZD - 1; dg >= 0; --dg)
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      long long d;
      if (dg > 0) {
        const long long q = (X[t] + half) >> ZR;
        d = X[t] - (q << ZR);
        X[t] = q;
      } else {
        d = X[t];
      }
      h[dg][t] = __float_as_uint((float)(int)d) >> 16;
    }
}
__device__ __forceinline__ uint4 pack8(const uint32_t* h, uint32_t sign) {
  uint4 w;
  w.x = (h[0] | (h[1] << 16)) ^ sign;
  w.y = (h[2] | (h[3] << 16)) ^ sign;
  w.z = (h[4] | (h[5] << 16)) ^ sign;
  w.w = (h[6] | (h[7] << 16)) ^ sign;
  return w;
}

// one source row -> the A operand (form [re|im]) and the B operand (forms
// [re|im] and [-im|re]) with one exponent and one digit expansion: the
// digits of [-im|re] are those of [re|im] negated and swapped in halves
// (a negated balanced expansion is again one, digits still <= 2^6)
struct ZSliceAB {
  const double2* src;
  int64_t src_estride, srow, sk;
  int rows, kc;
  uint8_t *a, *b;
  int64_t a_estride, b_estride;
  int *ea, *eb;
  int ex_estride;
};
__global__ void k_zslice_ab(ZSliceAB a) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  const int e = blockIdx.y;
  const int pa = (a.rows + ZM - 1) / ZM * ZM, pb = (a.rows + ZN - 1) / ZN * ZN;
  if (row >= pa) return;
  const bool valid = row < a.rows, inb = row < pb;
  const double2* s = a.src + (int64_t)e * a.src_estride + (int64_t)row * a.srow;
  unsigned long long mx = 0;
  if (valid)
    for (int k = 0; k < a.kc; ++k) {
      const double2 z = s[(int64_t)k * a.sk];
      mx = max(mx, max(mag_bits(z.x), mag_bits(z.y)));
    }
  const int ex = row_exponent(mx);
  a.ea[(int64_t)e * a.ex_estride + row] = valid ? ex : 0;
  if (inb) a.eb[(int64_t)e * a.ex_estride + row] = valid ? ex : 0;
  uint8_t* abase = a.a + (int64_t)e * a.a_estride + (size_t)(row / ZM) * ZD * ZA_BLK;
  uint8_t* bbase = a.b + (int64_t)e * a.b_estride + (size_t)(row / ZN) * ZB_TILE;
  const int ra = row % ZM, rb = row % ZN;
  const size_t bdig = (size_t)(2 * ZN / 8) * 256;  // B digit stride (64 rows)
  for (int g = 0; g < ZGROUPS / 2; ++g) {  // K positions 8g.. (re) and 64 + 8g.. (im)
    long long Xr[8], Xi[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int k = 8 * g + t;
      const double2 z = (valid && k < a.kc) ? s[(int64_t)k * a.sk] : make_double2(0.0, 0.0);
      Xr[t] = fixed_of(z.x, ex, ZFB);
      Xi[t] = fixed_of(z.y, ex, ZFB);
    }
    uint32_t hr[ZD][8], hi[ZD][8];
    digits8(Xr, hr);
    digits8(Xi, hi);
    for (int dg = 0; dg < ZD; ++dg) {
      const uint4 wr = pack8(hr[dg], 0u), wi = pack8(hi[dg], 0u);
      const uint4 wmi = pack8(hi[dg], 0x80008000u);  // -im (BF16 sign bits)
      uint8_t* ad = abase + (size_t)dg * ZA_BLK;
      *(uint4*)(ad + tile_off(ra, g, ZM)) = wr;
      *(uint4*)(ad + tile_off(ra, g + ZGROUPS / 2, ZM)) = wi;
      if (inb) {
        uint8_t* bd = bbase + (size_t)dg * bdig;
        *(uint4*)(bd + tile_off(rb, g, ZBROWS)) = wr;                   // form [re|im]
        *(uint4*)(bd + tile_off(rb, g + ZGROUPS / 2, ZBROWS)) = wi;
        *(uint4*)(bd + tile_off(ZN + rb, g, ZBROWS)) = wmi;             // form [-im|re]
        *(uint4*)(bd + tile_off(ZN + rb, g + ZGROUPS / 2, ZBROWS)) = wr;
      }
    }
  }
}

struct ZUpd {
  const uint8_t* a;
  int64_t a_estride;
  const uint8_t* b;
  int64_t b_estride;
  const int* ea;
  int ea_estride;
  const int* eb;
  int eb_estride;
  double2* C;
  int64_t c_estride;
  int ldc;
  int m, n;
  int lower;
  int beta0;  // 1: C = sgn A B^T (C is not read)
  double sgn;
  int nrt;
  int* err;
};

constexpr int ZX_SKIP = -0x40000000;  // column exponent slot of a skipped output


// one 128 x 32 tile of one element per CTA
__global__ void __launch_bounds__(ZU_THREADS) k_zupd(ZUpd a) {
  const int e = blockIdx.y;
  const int rt = blockIdx.x % a.nrt, ct = blockIdx.x / a.nrt;
  if (a.lower && ct * ZN > rt * ZM + ZM - 1) return;  // tile above the diagonal
  extern __shared__ __align__(1024) uint8_t zsm_raw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)zsm_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* regA0 = sm;
  uint8_t* regB = sm + ZNABUF * ZA_BLK;
  // levfin[p]: the MMAs of A digit p are complete, so the levels 0..p are final
  __shared__ __align__(8) uint64_t ldB_bar, ldA_bar[ZNABUF], afree_bar[ZNABUF], levfin[ZD];
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&ldB_bar), 1);
    for (int i = 0; i < ZNABUF; ++i) {
      mbar_init(smem_u32(&ldA_bar[i]), 1);
      mbar_init(smem_u32(&afree_bar[i]), 1);
    }
    for (int l = 0; l < ZD; ++l) mbar_init(smem_u32(&levfin[l]), 1);
    abort_ = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(ZU_TMEM));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base;
  if (warp == 0) {
    if (lane == 0) {
      const uint8_t* bsrc = a.b + (int64_t)e * a.b_estride + (size_t)ct * ZB_TILE;
      mbar_expect_tx(smem_u32(&ldB_bar), ZB_TILE);
      bulk_load(smem_u32(regB), bsrc, ZB_TILE, smem_u32(&ldB_bar));
      const uint8_t* asrc = a.a + (int64_t)e * a.a_estride + (size_t)rt * ZD * ZA_BLK;
      for (int p = 0; p < ZD; ++p) {
        const int buf = p % ZNABUF;
        if (p >= ZNABUF) {
          if (!mbar_wait(smem_u32(&afree_bar[buf]), ((p - ZNABUF) / ZNABUF) & 1, &abort_)) {
            abort_ = 1;
            atomicExch(a.err, 41);
            break;
          }
        }
        mbar_expect_tx(smem_u32(&ldA_bar[buf]), ZA_BLK);
        bulk_load(smem_u32(regA0 + buf * ZA_BLK), asrc + (size_t)p * ZA_BLK, ZA_BLK,
                  smem_u32(&ldA_bar[buf]));
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      bool ok = mbar_wait(smem_u32(&ldB_bar), 0, &abort_);
      if (!ok) { abort_ = 1; atomicExch(a.err, 42); }
      const uint64_t dB0 = sdesc_kmajor(smem_u32(regB));
      for (int p = 0; p < ZD && ok; ++p) {
        const int buf = p % ZNABUF;
        if (!mbar_wait(smem_u32(&ldA_bar[buf]), (p / ZNABUF) & 1, &abort_)) {
          abort_ = 1;
          atomicExch(a.err, 43);
          ok = false;
          break;
        }
        tc_fence_after();
        const uint64_t dA = sdesc_kmajor(smem_u32(regA0 + buf * ZA_BLK));
        // all pairs (p, q), q = 0..6-p, and both parts: B rows [0, 2 ZN (7 - p))
        // into the TMEM levels p..6 (2 ZN columns each), at most 256 per MMA
        constexpr int QMAX = 256 / (2 * ZN);
        for (int kb = 0; kb < ZK / 16; ++kb) {
          const uint64_t a_kb = dA + (uint64_t)((kb * ZM * 32) >> 4);
          for (int q0 = 0; q0 + p < ZD;) {
            const int nq = (ZD - p - q0) < QMAX ? (ZD - p - q0) : QMAX;
            const uint32_t dt = tbase + (uint32_t)((p + q0) * 2 * ZN);
            const uint64_t db = dB0 + (uint64_t)(((size_t)kb * ZBROWS * 32 + (size_t)q0 * 2 * ZN * 32) >> 4);
            umma_bf16(dt, a_kb, db, zidesc(nq * 2 * ZN), (p > 0 || kb > 0) ? 1u : 0u);
            q0 += nq;
          }
        }
        umma_commit(smem_u32(&afree_bar[buf]));
        umma_commit(smem_u32(&levfin[p]));
      }
    }
  } else {
    // epilogue: warps 2..; TMEM lane quarter warp % 4 = rows of the tile,
    // (warp - 2) / 4 = which ZCG 8-column groups.  Level p takes only the
    // digit pairs (p', p - p') with p' <= p, so it is final once the MMAs of
    // A digit p are (levfin[p]): each level is read and folded into the
    // running integer while the MMAs of the later digits proceed.
    const int quarter = warp & 3, half = (warp - 2) >> 2;
    const int i = rt * ZM + quarter * 32 + lane;
    const bool rowok = i < a.m;
    const int ea = rowok ? a.ea[(int64_t)e * a.ea_estride + i] : 0;
    const double2* crow = a.C + (int64_t)e * a.c_estride + i;
    const int* ebp = a.eb + (int64_t)e * a.eb_estride;
    const uint32_t tl = tbase + ((uint32_t)(quarter * 32) << 16);
    double2* C = a.C + (int64_t)e * a.c_estride;
    for (int cg = ZCG * half; cg < ZCG * (half + 1); ++cg) {
      // C and the column exponents, loaded while the MMAs run
      double2 cv[8];
      int xs[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int j = ct * ZN + cg * 8 + c;
        const bool ok = rowok && j < a.n && !(a.lower && j > i);
        cv[c] = (ok && !a.beta0) ? crow[(int64_t)j * a.ldc] : make_double2(0.0, 0.0);
        xs[c] = ok ? ebp[j] : ZX_SKIP;
      }
      // exact recombination in integers.  Digits are at most 2^6 (48-bit
      // split), so each level sum s_L (at most 7 pairs x 128 terms) is an
      // integer below 2^21.8 and (s_L + 1.5 2^23) has it in its low mantissa
      // bits.  V = sum_{L<=3} s_L 2^(7(3-L)+19) + sum_{L>=4} s_L 2^(7(6-L)-2)
      // (< 2^61.1; the last level rounded down to a unit) carries the
      // product in units of 2^(sx - 52), below the 2^(sx - 48) of the split
      long long V[2][8];
#pragma unroll
      for (int part = 0; part < 2; ++part)
#pragma unroll
        for (int c = 0; c < 8; ++c) V[part][c] = 0;
      bool okw = true;
#pragma unroll
      for (int L = 0; L < ZD; ++L) {
        if (!mbar_wait(smem_u32(&levfin[L]), 0, &abort_)) {
          abort_ = 1;
          atomicExch(a.err, 44);
          okw = false;
          break;
        }
        tc_fence_after();
        uint32_t r0[8], r1[8];
        tmem_ld8_nowait(tl + (uint32_t)((L * 2 + 0) * ZN + cg * 8), r0);
        tmem_ld8_nowait(tl + (uint32_t)((L * 2 + 1) * ZN + cg * 8), r1);
        tmem_wait();
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const long long s0 = __float_as_int(__uint_as_float(r0[c]) + 12582912.0f) - 0x4B400000;
          const long long s1 = __float_as_int(__uint_as_float(r1[c]) + 12582912.0f) - 0x4B400000;
          if (L <= 3) {
            V[0][c] += s0 << (ZR * (3 - L) + 19);
            V[1][c] += s1 << (ZR * (3 - L) + 19);
          } else if (L < 6) {
            V[0][c] += s0 << (ZR * (6 - L) - 2);
            V[1][c] += s1 << (ZR * (6 - L) - 2);
          } else {
            V[0][c] += s0 >> 2;
            V[1][c] += s1 >> 2;
          }
        }
      }
      if (!okw || !rowok) continue;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        if (xs[c] == ZX_SKIP) continue;
        const int sc = ea + xs[c] - 52;
        const long long v0 = a.sgn < 0.0 ? -V[0][c] : V[0][c];
        const long long v1 = a.sgn < 0.0 ? -V[1][c] : V[1][c];
        cv[c].x += scaled_i64(v0, sc);
        cv[c].y += scaled_i64(v1, sc);
        C[i + (int64_t)(ct * ZN + cg * 8 + c) * a.ldc] = cv[c];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(ZU_TMEM));
  }
}

int rows_pad(int rows, int nt) { return (rows + nt - 1) / nt * nt; }

// ---------------------------------------------------------------------------
// the augmented partial factorization
// ---------------------------------------------------------------------------
// FP64 step of one panel of the augmented matrix, one warp per element:
// the Cholesky factor L11 of the kb x kb diagonal block at (k0, k0) and
// W = L11^-H (upper, 64 x 64 column-major, zero outside kb x kb).  Right-
// looking Cholesky, then the inverse in place by right-looking forward
// substitution (column k of L kept in a scratch vector), in one packed lower
// triangle per warp (34 KB: six warps per SM), warp-synchronous.  Each step's
// update runs over a flat index, so every lane of an FP64 instruction has
// work (GB300 issues FP64 at about 1.6 per clock per SM); complex updates are
// 4 fused multiply-adds.  Only W is written: nothing reads the diagonal block
// of the augmented matrix after its panel step.
constexpr int ZDG_WARPS = 2;
constexpr int ZDG_TRI = 64 * 65 / 2;
constexpr size_t ZDG_SMEM = ZDG_WARPS * (ZDG_TRI + 64) * sizeof(double2);

__device__ __forceinline__ int tri(int i, int j) { return i * (i + 1) / 2 + j; }
// c - a b and c - a conj(b)
__device__ __forceinline__ double2 zfms(double2 c, double2 a, double2 b) {
  return make_double2(fma(a.y, b.y, fma(-a.x, b.x, c.x)), fma(-a.y, b.x, fma(-a.x, b.y, c.y)));
}
__device__ __forceinline__ double2 zfms_c(double2 c, double2 a, double2 b) {
  return make_double2(fma(-a.y, b.y, fma(-a.x, b.x, c.x)), fma(-a.y, b.x, fma(a.x, b.y, c.y)));
}

__global__ void __launch_bounds__(ZDG_WARPS * 32) k_zdiag(const double2* M, int64_t estride, int ld,
                                                          int k0, int kb, double2* W,
                                                          int64_t wstride, int* bad, int nel) {
  extern __shared__ double2 zdg[];
  const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * ZDG_WARPS + wp;
  if (e >= nel) return;
  double2* A = zdg + (size_t)wp * (ZDG_TRI + 64);  // L, then X = L^-1 (packed lower)
  double2* col = A + ZDG_TRI;
  const double2* D = M + (int64_t)e * estride + k0 + (int64_t)k0 * ld;
  for (int j = 0; j < kb; ++j)
    for (int i = j + lane; i < kb; i += 32) A[tri(i, j)] = D[i + (int64_t)j * ld];
  __syncwarp();
  bool ok = true;
  for (int k = 0; k < kb; ++k) {
    double dd = A[tri(k, k)].x;
    if (!(dd > 0.0)) { ok = false; dd = 1.0; }
    const double sq = sqrt(dd), rs = 1.0 / sq;
    __syncwarp();
    if (lane == 0) A[tri(k, k)] = make_double2(sq, 0.0);
    for (int i = k + 1 + lane; i < kb; i += 32) A[tri(i, k)] = zscale(rs, A[tri(i, k)]);
    __syncwarp();
    const int m = kb - k - 1;
    for (int x = lane; x < m * (m + 1) / 2; x += 32) {
      int ip = (int)((sqrtf(8.0f * x + 1.0f) - 1.0f) * 0.5f);
      while (tri(ip + 1, 0) <= x) ++ip;
      while (tri(ip, 0) > x) --ip;
      const int i = k + 1 + ip, jj = k + 1 + (x - tri(ip, 0));
      A[tri(i, jj)] = zfms_c(A[tri(i, jj)], A[tri(i, k)], A[tri(jj, k)]);
    }
    __syncwarp();
  }
  if (!ok && lane == 0) atomicMin(bad, e);
  for (int k = 0; k < kb; ++k) {
    for (int i = k + 1 + lane; i < kb; i += 32) col[i] = A[tri(i, k)];
    const double dk = 1.0 / A[tri(k, k)].x;
    __syncwarp();
    if (lane == 0) A[tri(k, k)] = make_double2(dk, 0.0);
    for (int jj = lane; jj < k; jj += 32) A[tri(k, jj)] = zscale(dk, A[tri(k, jj)]);
    __syncwarp();
    const int w = k + 1, m = kb - k - 1;
    for (int x = lane; x < m * w; x += 32) {
      const int ip = x / w, jj = x - ip * w, i = k + 1 + ip;
      const double2 lik = col[i];
      A[tri(i, jj)] = jj == k ? make_double2(-lik.x * dk, -lik.y * dk)
                              : zfms(A[tri(i, jj)], lik, A[tri(k, jj)]);
    }
    __syncwarp();
  }
  double2* w = W + (int64_t)e * wstride;
  for (int j = 0; j < 64; ++j)
    for (int i = lane; i < 64; i += 32)  // W(i, j) = conj(X(j, i))
      w[i + 64 * j] = (j >= i && j < kb) ? zconj(A[tri(j, i)]) : make_double2(0.0, 0.0);
}

// the n x n trailing block at (o, o), lower triangle: T := -T
__global__ void k_zneg(double2* M, int64_t estride, int ld, int o, int n) {
  double2* m = M + (int64_t)blockIdx.y * estride + o + (int64_t)o * ld;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < (int64_t)n * n;
       x += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(x % n), c = (int)(x / n);
    if (r >= c) {
      const double2 v = m[r + (int64_t)c * ld];
      m[r + (int64_t)c * ld] = make_double2(-v.x, -v.y);
    }
  }
}

// position of trial unknown c (interface order [E | Q | l]) in the augmented
// order [Q | E | l]
__device__ __forceinline__ int aug_pos(int c, int ni, int nq) {
  return c < ni ? nq + c : (c < ni + nq ? c - ni : c);
}

// Z (n1 x n1, full, interface order) from the lower trailing block at (o, o)
__global__ void k_zkeep(const double2* M, int64_t estride, int ld, int o, int n1, int nq,
                        double2* Z) {
  const int e = blockIdx.y, ni = n1 - 1 - nq;
  const double2* m = M + (int64_t)e * estride + o + (int64_t)o * ld;
  double2* z = Z + (int64_t)e * n1 * n1;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < (int64_t)n1 * n1;
       x += (int64_t)gridDim.x * blockDim.x) {
    const int ar = aug_pos((int)(x % n1), ni, nq), ac = aug_pos((int)(x / n1), ni, nq);
    z[x] = ar >= ac ? m[ar + (int64_t)ac * ld] : zconj(m[ac + (int64_t)ar * ld]);
  }
}

// Y (nq x ni1, column-major) = L_EQ^H, L_EQ the panel below the L2 block
// (rows o + nq .. o + nq + ni1, columns o .. o + nq)
__global__ void k_zcopyT(const double2* M, int64_t estride, int ld, int o, int nq, int ni1,
                         double2* Y) {
  const int e = blockIdx.y;
  const double2* m = M + (int64_t)e * estride;
  double2* y = Y + (int64_t)e * nq * ni1;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < (int64_t)nq * ni1;
       x += (int64_t)gridDim.x * blockDim.x) {
    const int q = (int)(x % nq), j = (int)(x / nq);
    y[x] = zconj(m[(o + nq + j) + (int64_t)(o + q) * ld]);
  }
}

// outputs: the compressed Schur complement and load (row-major over the
// extraction list, celem_systemI with ISYM_FLAG = 2) from the lower trailing
// block at (o, o) in the order [E | l]; ASchur and BSchur from Y
__global__ void k_dpg_aug_out(const double2* M, int64_t estride, int ld, int o, int ni,
                              const double2* Y, int nq, const int* nextract,
                              const int64_t* lcon_off, const int64_t* elem_nnz,
                              const int64_t* schur_off, const int64_t* bub_off, double2* zastif,
                              double2* zbload, double2* aschur, double2* bschur) {
  const int e = blockIdx.x;
  const double2* m = M + (int64_t)e * estride + o + (int64_t)o * ld;
  const double2* y = Y + (int64_t)e * nq * (ni + 1);
  const int64_t lo = lcon_off[e];
  const int nc = (int)(lcon_off[e + 1] - lo);
  const int* nx = nextract + lo;
  double2* za = zastif + elem_nnz[e];
  for (int64_t x = threadIdx.x; x < (int64_t)nc * nc; x += blockDim.x) {
    const int r = nx[x / nc], c = nx[x % nc];
    za[x] = r >= c ? m[r + (int64_t)c * ld] : zconj(m[c + (int64_t)r * ld]);
  }
  for (int l1 = threadIdx.x; l1 < nc; l1 += blockDim.x)
    zbload[lo + l1] = zconj(m[ni + (int64_t)nx[l1] * ld]);
  double2* as = aschur + schur_off[e];
  for (int64_t x = threadIdx.x; x < (int64_t)nq * ni; x += blockDim.x) as[x] = y[x];
  for (int i = threadIdx.x; i < nq; i += blockDim.x) bschur[bub_off[e] + i] = y[i + (int64_t)ni * nq];
}

}  // namespace

size_t dpg_tc_ex_slots(int rows) { return (size_t)rows_pad(rows, ZM); }
size_t dpg_tc_a_bytes(int rows) { return (size_t)rows_pad(rows, ZM) / ZM * ZD * ZA_BLK; }
size_t dpg_tc_b_bytes(int rows) { return (size_t)rows_pad(rows, ZN) / ZN * ZB_TILE; }

int dpg_aug_wslots(int nt, int nq) { return 1 + (nq + 63) / 64; }

// the augmented Hermitian matrix [[G, S], [S^H, 0]] (na = nt + n1, trial
// order [Q | E | l]) factored column panel by column panel:
//   1: the nt test columns; the trailing block becomes -Z, then Z (negated);
//   2: the nq L2-field columns of Z; the trailing block becomes the Schur
//      complement and the panel below holds Y^H, Y = L_QQ^-1 Z_Q[E|l]; then
//      ASchur | BSchur = L_QQ^-H Y by blocked backward substitution;
//   3: Z in the interface order to zkeep.
// Per panel: FP64 L11 and W = L11^-H (k_zdiag), then on tensor cores the
// panel solve P := P W and the trailing update T -= P P^H.
int launch_dpg_aug_tc(int part, int nel, int nt, int n1, int nq, const DpgWork& w, double* zkeep,
                      int* bad, int* err, cudaStream_t st) {
  if (nel <= 0) return 0;
  if (raise_smem_limit((const void*)k_zupd, ZU_SMEM) != cudaSuccess ||
      raise_smem_limit((const void*)k_zdiag, ZDG_SMEM) != cudaSuccess)
    return -1;
  const int na = nt + n1, ni1 = n1 - nq;
  int nk = 0;  // kernel launches
  double2* M = (double2*)w.M;
  double2* W = (double2*)w.W;
  double2* Y = (double2*)w.Y;
  const int64_t mst = (int64_t)na * na, wst = (int64_t)dpg_aug_wslots(nt, nq) * 4096;
  const int64_t yst = (int64_t)nq * ni1;
  const DpgTcBufs& tb = w.tb;
  const int exst = rows_pad(na, ZM);
  const int64_t ast = (int64_t)dpg_tc_a_bytes(na), bst = (int64_t)dpg_tc_b_bytes(na);
  auto slice = [&](const double2* src, int64_t estr, int64_t srow, int64_t sk, int rows, int kc,
                   bool isA, int f0, int f1) {
    ZSlice a;
    a.src = src; a.src_estride = estr; a.srow = srow; a.sk = sk;
    a.rows = rows; a.kc = kc;
    a.nt = isA ? ZM : ZN;
    a.rows_pad = rows_pad(rows, a.nt);
    a.nforms = isA ? 1 : 2; a.form0 = f0; a.form1 = f1;
    a.dst = isA ? tb.a : tb.b;
    a.dst_estride = isA ? ast : bst;
    a.ex = isA ? tb.ea : tb.eb;
    a.ex_estride = exst;
    k_zslice<<<dim3((a.rows_pad + 127) / 128, nel), 128, 0, st>>>(a);
    ++nk;
  };
  auto update = [&](double2* C, int64_t cst, int ldc, int m, int n, bool lower, double sgn,
                    bool beta0) {
    ZUpd u;
    u.a = tb.a; u.a_estride = ast; u.b = tb.b; u.b_estride = bst;
    u.ea = tb.ea; u.ea_estride = exst; u.eb = tb.eb; u.eb_estride = exst;
    u.C = C; u.c_estride = cst; u.ldc = ldc; u.m = m; u.n = n;
    u.lower = lower ? 1 : 0; u.sgn = sgn; u.beta0 = beta0 ? 1 : 0;
    u.nrt = (m + ZM - 1) / ZM;
    u.err = err;
    const int nct = (n + ZN - 1) / ZN;
    k_zupd<<<dim3(u.nrt * nct, nel), ZU_THREADS, ZU_SMEM, st>>>(u);
    ++nk;
  };
  auto panel = [&](int k0, int kb, int slot) {
    double2* ws = W + (int64_t)slot * 4096;
    k_zdiag<<<(nel + ZDG_WARPS - 1) / ZDG_WARPS, ZDG_WARPS * 32, ZDG_SMEM, st>>>(
        M, mst, na, k0, kb, ws, wst, bad, nel);
    ++nk;
    const int rem = na - k0 - kb;  // > 0: the load row is never a pivot
    double2* P = M + (k0 + kb) + (int64_t)k0 * na;
    slice(P, mst, 1, na, rem, kb, true, 0, 0);
    slice(ws, wst, 64, 1, kb, kb, false, 2, 3);  // B row j = column j of W
    update(P, mst, na, rem, kb, false, 1.0, true);
    ZSliceAB ab;
    ab.src = P; ab.src_estride = mst; ab.srow = 1; ab.sk = na; ab.rows = rem; ab.kc = kb;
    ab.a = tb.a; ab.b = tb.b; ab.a_estride = ast; ab.b_estride = bst;
    ab.ea = tb.ea; ab.eb = tb.eb; ab.ex_estride = exst;
    k_zslice_ab<<<dim3((rem + ZM - 1) / ZM, nel), ZM, 0, st>>>(ab);
    ++nk;
    update(M + (k0 + kb) + (int64_t)(k0 + kb) * na, mst, na, rem, rem, true, -1.0, false);
  };
  if (part == 1) {
    for (int k0 = 0; k0 < nt; k0 += 64) panel(k0, nt - k0 < 64 ? nt - k0 : 64, 0);
    k_zneg<<<dim3(64, nel), 256, 0, st>>>(M, mst, na, nt, n1);
    ++nk;
  } else if (part == 2) {
    for (int k0 = nt; k0 < nt + nq; k0 += 64)
      panel(k0, nt + nq - k0 < 64 ? nt + nq - k0 : 64, 1 + (k0 - nt) / 64);
    k_zcopyT<<<dim3(64, nel), 256, 0, st>>>(M, mst, na, nt, nq, ni1, Y);
    ++nk;
    for (int kq = (nq + 63) / 64 - 1; kq >= 0; --kq) {
      const int q0 = 64 * kq, qb = nq - q0 < 64 ? nq - q0 : 64;
      const double2* ws = W + (int64_t)(1 + kq) * 4096;
      // Y_k := W_k Y_k
      slice(ws, wst, 1, 64, qb, qb, true, 0, 0);
      slice(Y + q0, yst, nq, 1, ni1, qb, false, 2, 3);
      update(Y + q0, yst, nq, qb, ni1, false, 1.0, true);
      if (q0 > 0) {  // Y_i -= L_ki^H Y_k for the blocks i above
        slice(M + (nt + q0) + (int64_t)nt * na, mst, na, 1, q0, qb, true, 0, 0);
        slice(Y + q0, yst, nq, 1, ni1, qb, false, 0, 4);
        update(Y, yst, nq, q0, ni1, false, -1.0, false);
      }
    }
  } else if (part == 3) {
    k_zkeep<<<dim3(64, nel), 256, 0, st>>>(M, mst, na, nt, n1, nq, (double2*)zkeep);
    ++nk;
  }
  return cudaPeekAtLastError() == cudaSuccess ? nk : -1;
}

int launch_dpg_aug_out(int nel, int nt, int n1, int nq, const DpgWork& w, const int* nextract,
                        const int64_t* lcon_off, const int64_t* elem_nnz,
                        const int64_t* schur_off, const int64_t* bub_off, double* zastif,
                        double* zbload, double* aschur, double* bschur, cudaStream_t st) {
  if (nel <= 0) return 0;
  const int na = nt + n1, ni = n1 - 1 - nq;
  k_dpg_aug_out<<<nel, 256, 0, st>>>((const double2*)w.M, (int64_t)na * na, na, nt + nq, ni,
                                     (const double2*)w.Y, nq, nextract, lcon_off, elem_nnz,
                                     schur_off, bub_off, (double2*)zastif, (double2*)zbload,
                                     (double2*)aschur, (double2*)bschur);
  return 1;
}

}  // namespace hp3dg
