// k_dpg_tc.cu -- the dense algebra of the DPG Maxwell element on tcgen05
// tensor cores: Gram Cholesky G = L L^H, forward solve X = L^-1 [B | l] and
// Z = X^H X (the steps ZPPTRF / ZTPTRS / ZHERK of elem_maxwell.F90:590-639),
// blocked in 64-column panels.
//
// The FP64 work that stays on the CUDA cores is the 64-wide diagonal blocks:
// the Cholesky of each diagonal block with the solve of the panel below it,
// and the triangular solve of each 64-row block of X.  Every O(n^3) product
// -- the trailing updates of the Cholesky, the block updates of the solve
// and X^H X -- is one kind of update
//     C (FP64 complex) -= A B^T,   K = 64 complex per step,
// computed from split-BF16 digits: each complex row vector of A and B is
// written as a real vector of length 128 (its real and imaginary parts in a
// "form": [re|im], [-im|re], [re|-im], [im|re] or [im|-re]) with one
// power-of-two scale per row and 7 balanced radix-2^7 digits (49 bits).  The
// real part of the product is A(form [re|im]) . B(one form), the imaginary
// part A . B(another form); each digit pair (p, q) with p + q <= 8 lands in
// the FP32 TMEM accumulator of its level, where the sums of at most
// 7 * 128 products of digits below 2^14 stay below 2^24 (exact); the levels
// are recombined in FP64 and scaled by the two row exponents, one rounding
// per term.
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
constexpr int ZU_THREADS = 192;        // loader, MMA, 4 epilogue warps
constexpr uint32_t ZU_TMEM = 512;      // 7 levels x 2 parts x 32 columns = 448
constexpr size_t ZU_SMEM = 2 * ZA_BLK + ZB_TILE + 1024;

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
  const size_t dstride = (size_t)a.nt * ZK * 2;
  uint8_t* base = a.dst + (int64_t)e * a.dst_estride +
                  (size_t)(row / a.nt) * a.nforms * ZD * dstride;
  const int r = row % a.nt;
  for (int fi = 0; fi < a.nforms; ++fi) {
    const int f = fi == 0 ? a.form0 : a.form1;
    uint8_t* fb = base + (size_t)fi * ZD * dstride;
    for (int g = 0; g < ZGROUPS; ++g) {
      long long X[8];
#pragma unroll
      for (int t = 0; t < 8; ++t)
        X[t] = valid ? fixed_of(form_value(s, a.sk, a.kc, f, 8 * g + t), ex, ZR * ZD) : 0;
      store_digits8(X, ZR, ZD, fb + tile_off(r, g, a.nt), dstride);
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
  double sgn;
  int nrt;
  int* err;
};

// one 128 x 32 tile of one element per CTA
__global__ void __launch_bounds__(ZU_THREADS) k_zupd(ZUpd a) {
  const int e = blockIdx.y;
  const int rt = blockIdx.x % a.nrt, ct = blockIdx.x / a.nrt;
  if (a.lower && ct * ZN > rt * ZM + ZM - 1) return;  // tile above the diagonal
  extern __shared__ __align__(1024) uint8_t zsm_raw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)zsm_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* regA0 = sm;
  uint8_t* regB = sm + 2 * ZA_BLK;
  __shared__ __align__(8) uint64_t ldB_bar, ldA_bar[2], afree_bar[2], accf_bar;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&ldB_bar), 1);
    for (int i = 0; i < 2; ++i) {
      mbar_init(smem_u32(&ldA_bar[i]), 1);
      mbar_init(smem_u32(&afree_bar[i]), 1);
    }
    mbar_init(smem_u32(&accf_bar), 1);
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
        const int buf = p & 1;
        if (p >= 2) {
          if (!mbar_wait(smem_u32(&afree_bar[buf]), ((p - 2) >> 1) & 1, &abort_)) {
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
      const uint32_t idesc = zidesc(ZN);
      const uint64_t dB0 = sdesc_kmajor(smem_u32(regB));
      for (int p = 0; p < ZD && ok; ++p) {
        const int buf = p & 1;
        if (!mbar_wait(smem_u32(&ldA_bar[buf]), (p >> 1) & 1, &abort_)) {
          abort_ = 1;
          atomicExch(a.err, 43);
          ok = false;
          break;
        }
        tc_fence_after();
        const uint64_t dA = sdesc_kmajor(smem_u32(regA0 + buf * ZA_BLK));
        for (int q = 0; q + p < ZD; ++q) {
          for (int part = 0; part < 2; ++part) {
            const uint32_t dt = tbase + (uint32_t)(((p + q) * 2 + part) * ZN);
            const uint64_t db = dB0 + (uint64_t)(((size_t)part * ZD * ZB_BLK + (size_t)q * ZB_BLK) >> 4);
            for (int kb = 0; kb < ZK / 16; ++kb)
              umma_bf16(dt, dA + (uint64_t)((kb * ZM * 32) >> 4), db + (uint64_t)((kb * ZN * 32) >> 4),
                        idesc, (p > 0 || kb > 0) ? 1u : 0u);
          }
        }
        umma_commit(smem_u32(&afree_bar[buf]));
      }
      umma_commit(smem_u32(&accf_bar));
    }
  } else {
    // epilogue: warps 2..5 -> TMEM lane quarter warp % 4 = rows of the tile
    const int quarter = warp & 3;
    const int i = rt * ZM + quarter * 32 + lane;
    const bool okw = mbar_wait(smem_u32(&accf_bar), 0, &abort_);
    if (!okw) { abort_ = 1; atomicExch(a.err, 44); }
    tc_fence_after();
    const uint32_t tl = tbase + ((uint32_t)(quarter * 32) << 16);
    const int ea = (i < a.m) ? a.ea[(int64_t)e * a.ea_estride + i] : 0;
    double2* C = a.C + (int64_t)e * a.c_estride;
    for (int cg = 0; cg < ZN / 8; ++cg) {
      // exact recombination in integers: levels L = 0..3 (weights 2^7(3-L)) and
      // L = 4..6 (weights 2^7(6-L)) as two 64-bit sums (below 2^45 / 2^38),
      // then one FP64 fma per part: v = hi 2^-35 + lo 2^-56
      long long hi[2][8], lo[2][8];
#pragma unroll
      for (int part = 0; part < 2; ++part)
#pragma unroll
        for (int c = 0; c < 8; ++c) hi[part][c] = lo[part][c] = 0;
#pragma unroll
      for (int L = 0; L < ZD; ++L) {
        uint32_t r0[8], r1[8];
        tmem_ld8_nowait(tl + (uint32_t)((L * 2 + 0) * ZN + cg * 8), r0);
        tmem_ld8_nowait(tl + (uint32_t)((L * 2 + 1) * ZN + cg * 8), r1);
        tmem_wait();
        const int sh = ZR * ((L < 4 ? 3 : 6) - L);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const long long a0 = (long long)__float2int_rn(__uint_as_float(r0[c])) << sh;
          const long long a1 = (long long)__float2int_rn(__uint_as_float(r1[c])) << sh;
          if (L < 4) { hi[0][c] += a0; hi[1][c] += a1; }
          else { lo[0][c] += a0; lo[1][c] += a1; }
        }
      }
      if (!okw || i >= a.m) continue;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int j = ct * ZN + cg * 8 + c;
        if (j >= a.n || (a.lower && j > i)) continue;
        const int sx = ea + a.eb[(int64_t)e * a.eb_estride + j];
        // 2^(sx - 35) and 2^(sx - 56) from the bits, with the sign of the update
        const double sh1 = a.sgn * __longlong_as_double((long long)(1023 + sx - 5 * ZR) << 52);
        const double sh2 = a.sgn * __longlong_as_double((long long)(1023 + sx - 8 * ZR) << 52);
        double2* cp = &C[i + (int64_t)j * a.ldc];
        double2 cv = *cp;
        if (sx > -960 && sx < 960) {
          cv.x = fma(__ll2double_rn(hi[0][c]), sh1, fma(__ll2double_rn(lo[0][c]), sh2, cv.x));
          cv.y = fma(__ll2double_rn(hi[1][c]), sh1, fma(__ll2double_rn(lo[1][c]), sh2, cv.y));
        } else {  // scales outside the normal range of the bit-built powers
          cv.x += a.sgn * (ldexp(__ll2double_rn(hi[0][c]), sx - 5 * ZR) +
                           ldexp(__ll2double_rn(lo[0][c]), sx - 8 * ZR));
          cv.y += a.sgn * (ldexp(__ll2double_rn(hi[1][c]), sx - 5 * ZR) +
                           ldexp(__ll2double_rn(lo[1][c]), sx - 8 * ZR));
        }
        *cp = cv;
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

// FP64 diagonal step of the Cholesky: L11 of the 64-wide block at k0 and the
// panel below it, x L11^H = a for every row (two 32-column halves)
constexpr size_t ZP_SMEM = (2 * TK * TM + 64 * 65) * sizeof(double2) + 64 * sizeof(double);
#define LSM(i, j) Ls[(i) * 65 + (j)]

__global__ void __launch_bounds__(LA_THREADS) k_zpanel(double2* G, int64_t estride, int n, int k0,
                                                       int kb, int* bad) {
  extern __shared__ double2 zp_dyn[];
  double2* sm = zp_dyn;
  double2* Ls = zp_dyn + 2 * TK * TM;
  const int e = blockIdx.x;
  double2* A = G + (int64_t)e * estride;
  double2* D = A + k0 + (int64_t)k0 * n;
  if (cta_zpotrf(D, n, kb, sm) && threadIdx.x == 0) atomicMin(bad, e);
  double* rd = (double*)(Ls + 64 * 65);  // reciprocals of the diagonal
  for (int x = threadIdx.x; x < kb * kb; x += LA_THREADS) {
    const int i = x % kb, j = x / kb;
    LSM(i, j) = i >= j ? D[i + (int64_t)j * n] : make_double2(0.0, 0.0);
    if (i == j) rd[i] = 1.0 / D[i + (int64_t)i * n].x;
  }
  __syncthreads();
  const int h1 = kb < 32 ? kb : 32;
  for (int r = k0 + kb + threadIdx.x; r < n; r += LA_THREADS) {
    double2 x[32];
    for (int j = 0; j < h1; ++j) {
      double2 t = A[r + (int64_t)(k0 + j) * n];
      for (int q = 0; q < j; ++q) t = zsub(t, zmul(x[q], zconj(LSM(j, q))));
      x[j] = zscale(rd[j], t);
    }
    for (int j = 0; j < h1; ++j) A[r + (int64_t)(k0 + j) * n] = x[j];
    if (kb > 32) {
      double2 y[32];
      for (int j = 32; j < kb; ++j) {
        double2 t = A[r + (int64_t)(k0 + j) * n];
        for (int q = 0; q < 32; ++q) t = zsub(t, zmul(x[q], zconj(LSM(j, q))));
        for (int q = 32; q < j; ++q) t = zsub(t, zmul(y[q - 32], zconj(LSM(j, q))));
        y[j - 32] = zscale(rd[j], t);
      }
      for (int j = 32; j < kb; ++j) A[r + (int64_t)(k0 + j) * n] = y[j - 32];
    }
  }
}

// FP64 diagonal step of the forward solve: X[k0:k0+kb, :] = L11^-1 X[k0:k0+kb, :]
__global__ void __launch_bounds__(LA_THREADS) k_zfsolve(const double2* G, int64_t gstride,
                                                        double2* S, int64_t sstride, int n,
                                                        int m, int k0, int kb) {
  extern __shared__ double2 zp_dyn[];
  double2* Ls = zp_dyn + 2 * TK * TM;
  const int e = blockIdx.x;
  const double2* A = G + (int64_t)e * gstride;
  double2* X = S + (int64_t)e * sstride;
  double* rd = (double*)(Ls + 64 * 65);
  for (int x = threadIdx.x; x < kb * kb; x += LA_THREADS) {
    const int i = x % kb, j = x / kb;
    LSM(i, j) = i >= j ? A[(k0 + i) + (int64_t)(k0 + j) * n] : make_double2(0.0, 0.0);
    if (i == j) rd[i] = 1.0 / A[(k0 + i) + (int64_t)(k0 + i) * n].x;
  }
  __syncthreads();
  const int h1 = kb < 32 ? kb : 32;
  for (int c = threadIdx.x; c < m; c += LA_THREADS) {
    double2* xc = X + k0 + (int64_t)c * n;
    double2 x[32];
    for (int i = 0; i < h1; ++i) {
      double2 t = xc[i];
      for (int q = 0; q < i; ++q) t = zsub(t, zmul(LSM(i, q), x[q]));
      x[i] = zscale(rd[i], t);
    }
    for (int i = 0; i < h1; ++i) xc[i] = x[i];
    if (kb > 32) {
      double2 y[32];
      for (int i = 32; i < kb; ++i) {
        double2 t = xc[i];
        for (int q = 0; q < 32; ++q) t = zsub(t, zmul(LSM(i, q), x[q]));
        for (int q = 32; q < i; ++q) t = zsub(t, zmul(LSM(i, q), y[q - 32]));
        y[i - 32] = zscale(rd[i], t);
      }
      for (int i = 32; i < kb; ++i) xc[i] = y[i - 32];
    }
  }
}

// Z (lower) -> full Hermitian
__global__ void k_zmirror(double2* Z, int64_t estride, int n1) {
  double2* z = Z + (int64_t)blockIdx.y * estride;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < (int64_t)n1 * n1;
       x += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(x % n1), j = (int)(x / n1);
    if (i < j) z[x] = zconj(z[j + (int64_t)i * n1]);
  }
}

int rows_pad(int rows, int nt) { return (rows + nt - 1) / nt * nt; }

}  // namespace

size_t dpg_tc_ex_slots(int rows) { return (size_t)rows_pad(rows, ZM); }
size_t dpg_tc_a_bytes(int rows) { return (size_t)rows_pad(rows, ZM) / ZM * ZD * ZA_BLK; }
size_t dpg_tc_b_bytes(int rows) { return (size_t)rows_pad(rows, ZN) / ZN * ZB_TILE; }

// the dense DPG algebra of nel elements on tensor cores: G (nt x nt) ->
// L (lower), S (nt x n1) -> X = L^-1 S, Z = X^H X (n1 x n1, full)
int launch_dpg_solve_tc(int nel, int nt, int n1, double* G, double* S, double* Z,
                        const DpgTcBufs& tb, int* bad, int* err, cudaStream_t st) {
  if (nel <= 0) return 0;
  if (raise_smem_limit((const void*)k_zupd, ZU_SMEM) != cudaSuccess ||
      raise_smem_limit((const void*)k_zpanel, ZP_SMEM) != cudaSuccess ||
      raise_smem_limit((const void*)k_zfsolve, ZP_SMEM) != cudaSuccess)
    return -1;
  double2* g = (double2*)G;
  double2* s = (double2*)S;
  double2* z = (double2*)Z;
  const int64_t gst = (int64_t)nt * nt, sst = (int64_t)nt * n1, zst = (int64_t)n1 * n1;
  const int rmax = nt > n1 ? nt : n1;
  const int exst = rows_pad(rmax, ZM);  // exponent slots per element (>= every padded row count)
  const int64_t ast = (int64_t)dpg_tc_a_bytes(rmax), bst = (int64_t)dpg_tc_b_bytes(rmax);
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
  };
  auto update = [&](double2* C, int64_t cst, int ldc, int m, int n, bool lower, double sgn) {
    ZUpd u;
    u.a = tb.a; u.a_estride = ast; u.b = tb.b; u.b_estride = bst;
    u.ea = tb.ea; u.ea_estride = exst; u.eb = tb.eb; u.eb_estride = exst;
    u.C = C; u.c_estride = cst; u.ldc = ldc; u.m = m; u.n = n;
    u.lower = lower ? 1 : 0; u.sgn = sgn;
    u.nrt = (m + ZM - 1) / ZM;
    u.err = err;
    const int nct = (n + ZN - 1) / ZN;
    k_zupd<<<dim3(u.nrt * nct, nel), ZU_THREADS, ZU_SMEM, st>>>(u);
  };
  // 1. G = L L^H: diagonal blocks in FP64, trailing updates on tensor cores
  for (int k0 = 0; k0 < nt; k0 += 64) {
    const int kb = nt - k0 < 64 ? nt - k0 : 64, rem = nt - k0 - kb;
    k_zpanel<<<nel, LA_THREADS, ZP_SMEM, st>>>(g, gst, nt, k0, kb, bad);
    if (rem > 0) {
      const double2* p = g + (k0 + kb) + (int64_t)k0 * nt;
      slice(p, gst, 1, nt, rem, kb, true, 0, 0);
      slice(p, gst, 1, nt, rem, kb, false, 0, 1);
      update(g + (k0 + kb) + (int64_t)(k0 + kb) * nt, gst, nt, rem, rem, true, -1.0);
    }
  }
  // 2. X = L^-1 S: diagonal solves in FP64, block updates on tensor cores
  for (int k0 = 0; k0 < nt; k0 += 64) {
    const int kb = nt - k0 < 64 ? nt - k0 : 64, rem = nt - k0 - kb;
    k_zfsolve<<<nel, LA_THREADS, ZP_SMEM, st>>>(g, gst, s, sst, nt, n1, k0, kb);
    if (rem > 0) {
      slice(g + (k0 + kb) + (int64_t)k0 * nt, gst, 1, nt, rem, kb, true, 0, 0);
      slice(s + k0, sst, nt, 1, n1, kb, false, 2, 3);
      update(s + (k0 + kb), sst, nt, rem, n1, false, -1.0);
    }
  }
  // 3. Z = X^H X over 64-row chunks of X
  if (cudaMemsetAsync(z, 0, (size_t)nel * zst * sizeof(double2), st) != cudaSuccess) return -1;
  for (int k0 = 0; k0 < nt; k0 += 64) {
    const int kb = nt - k0 < 64 ? nt - k0 : 64;
    slice(s + k0, sst, nt, 1, n1, kb, true, 0, 0);
    slice(s + k0, sst, nt, 1, n1, kb, false, 0, 4);
    update(z, zst, n1, n1, n1, true, 1.0);
  }
  k_zmirror<<<dim3(64, nel), 256, 0, st>>>(z, zst, n1);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace hp3dg
