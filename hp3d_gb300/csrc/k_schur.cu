// k_schur.cu -- the Schur-complement update of the static condensation on
// tcgen05 tensor cores (mixed-precision pass).
//
// stc_fwd (modules/stc.F90:338-416, 443-509) forms, per element,
//   S = K_ii - K_ib K_bb^-1 K_bi = K_ii - Y^T Y,   Y = L^-1 K_bi,  K_bb = L L^T.
// The FP64 kernel (k_condense, factor mode) computes L and Y and writes Y as
// balanced BF16 digits (one power-of-two scale per column a of Y):
//   Y[:, a] = 2^e_a sum_{i=1..D} y_i[:, a] 2^(-radix i),  |y_1| <= 2^radix,
//   |y_i| <= 2^(radix-1) for i >= 2,
// stored as UMMA canonical K-major tiles: rows = interface dof a (padded to
// nr >= 128), K = bubble dof (16 per k-block).  This kernel forms
//   W_ab = sum_r Y_ra Y_rb = 2^(e_a+e_b-radix(D+1)) sum_s L_s 2^(radix(D+1-s)),
//   L_s = sum_{i+j=s} y_i^T y_j,  s = 2..D+1,
// with one FP32 TMEM accumulator per level s.  With K <= 128 bubble dof every
// level sum is an integer below 2^24 (at most 2^14 + 5 * 2^12 per product
// row times K), so the accumulators are exact; the levels are recombined as
// two exact 64-bit integers and one FP64 addition (one rounding).  The
// epilogue writes W_ab (a <= b, element dof order) into the packed upper
// scratch; the compression kernel forms S = K_ii - W while it gathers K_ii.
//
// One persistent CTA per SM walks the elements of a bin: warp 0 copies the
// element's digits into shared memory (one bulk copy), warp 1 owns the TMEM
// (512 columns) and issues the MMAs, warps 2-5 drain the accumulators.  The
// product is computed in chunks of 128 rows x <= 64 columns with all levels
// resident (levels x 64 <= 512 TMEM columns); rows are one 128-row tile, or
// two (0..127 and nr-128..nr-1) when nr > 128.
#include "hp3dg_internal.cuh"
#include "hp3dg_kernels.h"
#include "hp3dg_tc.cuh"

#include <string.h>

namespace hp3dg {

namespace {
constexpr int SC_NC = 64;         // TMEM columns per level slot (max chunk width)
constexpr int SC_MAXDIG = 7;
constexpr int SC_MAXCHUNK = 8;
constexpr int SC_MAXPAIR = 28;
constexpr int SC_THREADS = 192;
constexpr uint32_t SC_TMEM_COLS = 512;

struct SchurParams {
  int digits, radix;
  int nr, nkb;            // digit tile rows (>= 128, multiple of 16), k-blocks
  int nif, nbf, nfull;    // bin sizes (packed element matrix layout)
  int nel;
  int nchunk;
  int ch_m0[SC_MAXCHUNK], ch_c0[SC_MAXCHUNK], ch_nc[SC_MAXCHUNK], ch_rmin[SC_MAXCHUNK];
  int npair;
  int8_t pi[SC_MAXPAIR], pj[SC_MAXPAIR], pfirst[SC_MAXPAIR];
};

__host__ __device__ constexpr uint32_t idesc_bf16_m128(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}
}  // namespace

__global__ void __launch_bounds__(SC_THREADS, 1)
    k_schur_tc(const uint8_t* __restrict__ Ydig, const int* __restrict__ Yexp, const SchurParams P,
               const int* __restrict__ elist, const int* __restrict__ ni_e,
               double* __restrict__ Wbuf, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smraw[];
  uint8_t* ybuf = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t load_bar, free_bar, acc_full, acc_empty;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ebytes = (uint32_t)P.digits * P.nkb * P.nr * 32;
  const uint32_t dstride = (uint32_t)P.nkb * P.nr * 32;  // bytes per digit
  const uint32_t kstride = (uint32_t)P.nr * 32;           // bytes per k-block

  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&load_bar), 1);
    mbar_init(smem_u32(&free_bar), 1);
    mbar_init(smem_u32(&acc_full), 1);
    mbar_init(smem_u32(&acc_empty), 128);
    abort_ = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(SC_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base;

  if (warp == 0) {
    // ---------------- loader ----------------
    if (lane == 0) {
      uint32_t fph = 0;
      for (int j = blockIdx.x; j < P.nel && !abort_; j += gridDim.x) {
        // the MMAs of the previous element must be done with the buffer
        if (!mbar_wait(smem_u32(&free_bar), fph ^ 1, &abort_)) { abort_ = 1; atomicExch(err, 11); break; }
        fph ^= 1;
        const uint32_t lb = smem_u32(&load_bar);
        mbar_expect_tx(lb, ebytes);
        bulk_load(smem_u32(ybuf), Ydig + (size_t)j * ebytes, ebytes, lb);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      uint32_t lph = 0, eph = 0;
      const uint32_t ybase = smem_u32(ybuf);
      for (int j = blockIdx.x; j < P.nel && !abort_; j += gridDim.x) {
        if (!mbar_wait(smem_u32(&load_bar), lph, &abort_)) { abort_ = 1; atomicExch(err, 12); break; }
        lph ^= 1;
        tc_fence_after();
        for (int ch = 0; ch < P.nchunk && !abort_; ++ch) {
          if (!mbar_wait(smem_u32(&acc_empty), eph ^ 1, &abort_)) { abort_ = 1; atomicExch(err, 13); break; }
          eph ^= 1;
          tc_fence_after();
          const uint32_t idesc = idesc_bf16_m128(P.ch_nc[ch]);
          const uint32_t aoff = (uint32_t)(P.ch_m0[ch] >> 3) * 256;
          const uint32_t boff = (uint32_t)(P.ch_c0[ch] >> 3) * 256;
          for (int p = 0; p < P.npair; ++p) {
            const uint32_t dt = tbase + (uint32_t)(P.pi[p] + P.pj[p] - 2) * SC_NC;
            const uint32_t abase = ybase + (uint32_t)(P.pi[p] - 1) * dstride + aoff;
            const uint32_t bbase = ybase + (uint32_t)(P.pj[p] - 1) * dstride + boff;
            for (int kb = 0; kb < P.nkb; ++kb) {
              const uint32_t acc = (kb > 0 || !P.pfirst[p]) ? 1u : 0u;
              umma_bf16(dt, sdesc_kmajor(abase + kb * kstride), sdesc_kmajor(bbase + kb * kstride),
                        idesc, acc);
            }
          }
          umma_commit(smem_u32(&acc_full));
        }
        umma_commit(smem_u32(&free_bar));  // the buffer may be refilled once these MMAs retire
      }
    }
  } else {
    // ---------------- epilogue (warps 2..5, one TMEM lane quarter each) ----------------
    const int quarter = warp & 3;
    const uint32_t tlane = tbase + ((uint32_t)(quarter * 32) << 16);
    const int D = P.digits, kh = D < 4 ? D : 4;
    uint32_t aph = 0;
    for (int j = blockIdx.x; j < P.nel && !abort_; j += gridDim.x) {
      const int e = elist[j];
      const int ni = ni_e[e];
      const int* ex = Yexp + (size_t)j * P.nr;
      double* W = Wbuf + (size_t)j * ((size_t)P.nif * (P.nif + 1) / 2);
      for (int ch = 0; ch < P.nchunk; ++ch) {
        if (!mbar_wait(smem_u32(&acc_full), aph, &abort_)) { abort_ = 1; atomicExch(err, 14); break; }
        aph ^= 1;
        tc_fence_after();
        const int a = P.ch_m0[ch] + quarter * 32 + lane;
        const bool arow = a >= P.ch_rmin[ch] && a < ni;
        const int ea = arow ? ex[a] : 0;
        for (int cc = 0; cc < P.ch_nc[ch] / 16; ++cc) {
          uint32_t v[SC_MAXDIG][16];
#pragma unroll
          for (int k = 0; k < SC_MAXDIG; ++k)
            if (k < D) tmem_ld16_nowait(tlane + (uint32_t)(k * SC_NC + cc * 16), v[k]);
          tmem_wait();
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int b = P.ch_c0[ch] + cc * 16 + q;
            if (!(arow && b < ni && a <= b)) continue;
            long long hi = 0, lo = 0;
#pragma unroll
            for (int k = 0; k < SC_MAXDIG; ++k) {
              if (k >= D) break;
              long long l = (long long)__float2int_rn(__uint_as_float(v[k][q]));
              if (k < kh) hi = hi * (1LL << P.radix) + l;
              else lo = lo * (1LL << P.radix) + l;
            }
            // W = (hi 2^(radix(D-kh)) + lo) 2^(e_a + e_b - radix(D+1)); the power
            // of two is built from its exponent bits (exact, normal range)
            const int sx = ea + ex[b] - P.radix * (D + 1);
            const double sc = __longlong_as_double((long long)(1023 + sx) << 52);
            const double sch = __longlong_as_double((long long)(1023 + sx + P.radix * (D - kh)) << 52);
            W[(int64_t)b * (b + 1) / 2 + a] = fma(__ll2double_rn(hi), sch, __ll2double_rn(lo) * sc);
          }
        }
        tc_fence_before();
        mbar_arrive(smem_u32(&acc_empty));
      }
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase),
                 "r"(SC_TMEM_COLS));
  }
}

// Layout of an element's Y digits: digit-major, then k-block, then the
// canonical K-major tile of nr rows x 16 bubble dof.
int schur_tc_rows(int nif) {
  int nr = (nif + 15) / 16 * 16;
  return nr < 128 ? 128 : nr;
}
int schur_tc_kblocks(int nbf) { return (nbf + 15) / 16; }
size_t schur_tc_elem_bytes(int nif, int nbf, int digits) {
  return (size_t)digits * schur_tc_kblocks(nbf) * schur_tc_rows(nif) * 32;
}
// usable when the digits of one element fit in shared memory, the bubble
// block is non-empty and at most 128 (exactness bound), and rows fit in two
// 128-row tiles
bool schur_tc_supported(int nif, int nbf, int digits) {
  return nbf > 0 && nbf <= 128 && schur_tc_rows(nif) <= 256 && digits <= SC_MAXDIG &&
         schur_tc_elem_bytes(nif, nbf, digits) + 1024 <= 220 * 1024;
}

int launch_schur_tc(int nel, int nfull, int nif, int nbf, int radix, int digits,
                    const uint8_t* d_ydig, const int* d_yexp, const int* d_elist,
                    const int* d_ni_e, double* d_W, int* d_flag, cudaStream_t st) {
  if (nel <= 0) return 0;
  if (!schur_tc_supported(nif, nbf, digits)) return -2;
  static int num_sms = 0;
  if (!num_sms) {
    int dev;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  SchurParams P;
  memset(&P, 0, sizeof(P));
  P.digits = digits;
  P.radix = radix;
  P.nr = schur_tc_rows(nif);
  P.nkb = schur_tc_kblocks(nbf);
  P.nif = nif; P.nbf = nbf; P.nfull = nfull; P.nel = nel;
  // chunks: tile 0 rows 0..127 over all columns; tile 1 rows nr-128..nr-1,
  // kept for rows >= 128, over columns 128..nr-1
  int nch = 0;
  for (int c0 = 0; c0 < P.nr; c0 += SC_NC) {
    P.ch_m0[nch] = 0; P.ch_c0[nch] = c0; P.ch_rmin[nch] = 0;
    P.ch_nc[nch] = (P.nr - c0) < SC_NC ? (P.nr - c0) : SC_NC;
    ++nch;
  }
  if (P.nr > 128)
    for (int c0 = 128; c0 < P.nr; c0 += SC_NC) {
      P.ch_m0[nch] = P.nr - 128; P.ch_c0[nch] = c0; P.ch_rmin[nch] = 128;
      P.ch_nc[nch] = (P.nr - c0) < SC_NC ? (P.nr - c0) : SC_NC;
      ++nch;
    }
  P.nchunk = nch;
  // digit pairs (i, j), i + j <= digits + 1, grouped by level; the first
  // pair of a level starts its accumulator
  int np = 0;
  for (int s = 2; s <= digits + 1; ++s)
    for (int i = 1; i < s; ++i) {
      P.pi[np] = (int8_t)i; P.pj[np] = (int8_t)(s - i); P.pfirst[np] = (int8_t)(i == 1);
      ++np;
    }
  P.npair = np;
  size_t smem = schur_tc_elem_bytes(nif, nbf, digits) + 1024;
  if (raise_smem_limit((const void*)k_schur_tc, smem) != cudaSuccess) return -1;
  int grid = nel < num_sms ? nel : num_sms;
  k_schur_tc<<<grid, SC_THREADS, smem, st>>>(d_ydig, d_yexp, P, d_elist, d_ni_e, d_W, d_flag);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace hp3dg
