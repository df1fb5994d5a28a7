// k_ozaki.cu -- mixed-precision B^T D B contraction on tcgen05 tensor cores.
//
// The stiffness of every element of a bin is one row of a GEMM with a shared
// operand (elem_opt.F90:86-137 computes it per element as A_TEST*A_TEST^T):
//
//   PK[e, c] = sum_q D[e, q] M[q, c],   q = (point l, component pair ij),
//   c = packed (a <= b) entry,  M[(l,ij), (a,b)] = G_i[l,a] G_j[l,b] (+ sym).
//
// Both operands are FP64.  They are split into balanced integer digits of
// `radix` bits (scaled per element row / per column by powers of two):
//   D = s_e * sum_i d_i 2^(-radix*i),   M = t_c * sum_j m_j 2^(-radix*j),
// every digit an integer |d| <= 2^radix, exact in BF16.  The digit products
// d_i * m_j are exact and, grouped by level s = i + j, their sums over q stay
// below 2^24 and are therefore exact in the FP32 TMEM accumulators.  The
// levels s = 2 .. digits+1 are recombined exactly as 64-bit integers and
// scaled to FP64 in the epilogue (the FP64 residual correction of the
// split): the result carries ~radix*digits bits.
//
// Kernel structure (one CTA per SM, persistent over 128 x 128 output tiles):
//   warp 0   producer: per k-block one contiguous bulk copy (cp.async.bulk)
//            of the A = M digit tiles (128 packed columns x 16 q each) and one
//            of the B = D digit tiles (128 elements x 16 q); the digits are
//            stored in HBM already in the UMMA canonical K-major layout
//            (8-row x 16-byte core matrices), 4-stage ring
//   warp 1   TMEM allocation (512 columns) and the single MMA-issuing thread;
//            the pairs (i, j), (i, j+1) of an A digit read consecutive B digit
//            tiles into consecutive level slots, so they run as one
//            128 x 256 x 16 MMA (the A tile read once for both)
//   warps 2-5 epilogue: tcgen05.ld of up to 4 level accumulators, exact
//            integer recombination, FP64 scaling, coalesced stores of PK
// Levels are processed in passes of <= 4 accumulators (4 x 128 TMEM
// columns); pass > 1 adds into the FP64 tile written by pass 1.
#include "hp3dg_internal.cuh"
#include "hp3dg_kernels.h"
#include "hp3dg_tc.cuh"

#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

namespace hp3dg {

namespace {
constexpr int BM = 128;       // packed columns per tile (MMA M, TMEM lanes)
constexpr int BN = 128;       // elements per tile (MMA N, TMEM columns per level)
constexpr int BK = 16;        // q per k-block (one MMA K step), 32-byte rows
constexpr int MAXDIG = 7;
constexpr int MAXPASS = 4;
constexpr int MAXPAIR = 40;
constexpr int NSTAGE = 4;
#ifndef KGROUP
#define KGROUP 2  // k-blocks per accumulator run (NSTAGE / KGROUP groups in flight)
#endif
constexpr int TILE_BYTES = BM * BK * 2;  // 4096, A and B tiles have the same size
constexpr int STAGE_BYTES = 2 * MAXDIG * TILE_BYTES;  // room for all digits
constexpr int NTHREADS = 192;
constexpr uint32_t TMEM_COLS = 512;


struct PassDesc {
  int first_level;  // level of accumulator slot 0
  int nlev;         // accumulator slots used (<= 4)
  int nA, nB;       // digits of A (M) and B (D) needed: 1..nA, 1..nB
  int pair0, npair; // range in the pair table
};
struct GemmParams {
  int npass;
  PassDesc pass[MAXPASS];
  int npairs;
  int8_t pi[MAXPAIR], pj[MAXPAIR], pslot[MAXPAIR], pfirst[MAXPAIR];
  int radix;
  int s1;           // two-pass recombination shift (see epi_chunk)
  int scale_shift;  // radix*last level of pass 0 (+ s1) : final power-of-two shift
  int digits;
  int nk;        // k-blocks
  int ncb, neb;  // column / element blocks
  int nel, ncols;
};
}  // namespace

// tile t -> (column block, element block): groups of 8 column blocks sweep
// all element blocks, so the digit tiles of a group stay resident in L2.
__device__ __forceinline__ void tile_coords(int t, const GemmParams& P, int& cb, int& eb) {
  const int grp = 8;
  int g = t / (grp * P.neb);
  int r = t - g * grp * P.neb;
  int gw = P.ncb - g * grp;
  if (gw > grp) gw = grp;
  cb = g * grp + r % gw;
  eb = r / gw;
}

// instruction descriptor: kind::f16, A = B = BF16, D = F32, K-major, M=128, N=128
__host__ __device__ constexpr uint32_t idesc_bf16_m128_n128() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}
// the same with N = 256: two consecutive B digit tiles into two slots
__host__ __device__ constexpr uint32_t idesc_bf16_m128_n256() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(2 * BN >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

// exponent k of an exact power of two 2^k (the digit scales)
__device__ __forceinline__ int pow2_exponent(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7ff) - 1023;
}
// x * 2^k for normal results (k within the normal range), exact
__device__ __forceinline__ double times_pow2(double x, int k) {
  if (k >= -1022 && k <= 1023) return x * __longlong_as_double((long long)(k + 1023) << 52);
  return ldexp(x, k);
}

// Epilogue of one 16-element chunk of one pass.  The level accumulators are
// exact integers (< 2^24) in FP32; they are recombined exactly as 64-bit
// integers.  With two passes, pass 0 stores its integer V1 in the output
// slot and the last pass forms W = V1 * 2^S1 + V2 * 2^(S1 - radix*nlev2)
// (|W| < 2^63) before the single conversion to FP64 and the power-of-two
// scaling by the element and column scales.
template <int NLEV>
__device__ __forceinline__ void epi_chunk(const GemmParams& P, int ps, uint32_t tlane, int ch,
                                          int e0, int c, bool cok, int kc,
                                          const double* __restrict__ dscale,
                                          double* __restrict__ PK, int lane) {
  uint32_t v[NLEV][16];
#pragma unroll
  for (int k = 0; k < NLEV; ++k) tmem_ld16(tlane + (uint32_t)(k * BN + ch * 16), v[k]);
  const int el = e0 + (lane & 15);
  const int ke_lane = (el < P.nel) ? pow2_exponent(dscale[el]) : 0;
  long long* out = (long long*)PK;
  const bool two = P.npass == 2;
  const bool last = ps == P.npass - 1;
  long long prev[16];
  if (two && last) {
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int e = e0 + q;
      prev[q] = (cok && e < P.nel) ? out[(size_t)e * P.ncols + c] : 0;
    }
  }
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    long long s = 0;
#pragma unroll
    for (int k = 0; k < NLEV; ++k)
      s = s * (1LL << P.radix) + (long long)__float2int_rn(__uint_as_float(v[k][q]));
    const int e = e0 + q;
    const int ke = __shfl_sync(0xffffffffu, ke_lane, q);
    if (!(cok && e < P.nel)) continue;
    const size_t idx = (size_t)e * P.ncols + c;
    if (two && !last) {
      out[idx] = s;  // exact partial sum V1
    } else if (two) {
      const int sh = P.radix * P.pass[1].nlev - P.s1;
      long long w = prev[q] * (1LL << P.s1) + (sh >= 0 ? (s >> sh) : s * (1LL << (-sh)));
      PK[idx] = times_pow2((double)w, ke + kc - P.scale_shift);
    } else {
      PK[idx] = times_pow2((double)s, ke + kc - P.scale_shift);
    }
  }
}

// ---------------------------------------------------------------------------
// the GEMM
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS, 1)
    k_ozaki_gemm(const uint8_t* __restrict__ Atiles, const uint8_t* __restrict__ Btiles,
                 const GemmParams P, const double* __restrict__ dscale,
                 const double* __restrict__ mscale, double* __restrict__ PK,
                 int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smraw[];
  // align the ring to 1024 bytes (swizzle repeat)
  uint8_t* ring = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full_bar[NSTAGE], empty_bar[NSTAGE], acc_full, acc_empty;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = P.ncb * P.neb;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    mbar_init(smem_u32(&acc_full), 1);
    mbar_init(smem_u32(&acc_empty), 128);
    abort_ = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      for (int t = blockIdx.x; t < ntiles && !abort_; t += gridDim.x) {
        int cb, eb;
        tile_coords(t, P, cb, eb);
        for (int ps = 0; ps < P.npass && !abort_; ++ps) {
          const PassDesc& pd = P.pass[ps];
          for (int kb = 0; kb < P.nk; ++kb) {
            if (!mbar_wait(smem_u32(&empty_bar[stage]), phase ^ 1, &abort_)) {
              abort_ = 1; atomicExch(err, 1); break;
            }
            uint32_t fb = smem_u32(&full_bar[stage]);
            mbar_expect_tx(fb, (uint32_t)(pd.nA + pd.nB) * TILE_BYTES);
            uint8_t* st = ring + (size_t)stage * STAGE_BYTES;
            // digits 0..nA-1 of (column block, k-block) are contiguous, likewise for B
            const size_t ablk = ((size_t)cb * P.nk + kb) * P.digits;
            const size_t bblk = ((size_t)eb * P.nk + kb) * P.digits;
            bulk_load(smem_u32(st), Atiles + ablk * TILE_BYTES, (uint32_t)pd.nA * TILE_BYTES, fb);
            bulk_load(smem_u32(st + MAXDIG * TILE_BYTES), Btiles + bblk * TILE_BYTES,
                      (uint32_t)pd.nB * TILE_BYTES, fb);
            if (++stage == NSTAGE) { stage = 0; phase ^= 1; }
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_m128_n128();
      const uint32_t idesc2 = idesc_bf16_m128_n256();
      int stage = 0;
      uint32_t phase = 0, accph = 0;
      for (int t = blockIdx.x; t < ntiles && !abort_; t += gridDim.x) {
        for (int ps = 0; ps < P.npass && !abort_; ++ps) {
          const PassDesc& pd = P.pass[ps];
          // the epilogue must have drained the accumulators
          if (!mbar_wait(smem_u32(&acc_empty), accph ^ 1, &abort_)) {
            abort_ = 1; atomicExch(err, 2); break;
          }
          accph ^= 1;
          tc_fence_after();
          // k-blocks are consumed in groups of KGROUP stages so that each level
          // accumulator receives a run of (pairs of the level) x KGROUP MMAs:
          // switching the accumulator between MMAs stalls the tensor pipe.
          for (int kb0 = 0; kb0 < P.nk && !abort_; kb0 += KGROUP) {
            const int ng = (P.nk - kb0) < KGROUP ? (P.nk - kb0) : KGROUP;
            uint32_t sbase[KGROUP];
            for (int g = 0; g < ng; ++g) {
              int sg = stage + g;
              uint32_t pg = phase;
              if (sg >= NSTAGE) { sg -= NSTAGE; pg ^= 1; }
              if (!mbar_wait(smem_u32(&full_bar[sg]), pg, &abort_)) {
                abort_ = 1; atomicExch(err, 3); break;
              }
              sbase[g] = smem_u32(ring + (size_t)sg * STAGE_BYTES);
            }
            if (abort_) break;
            tc_fence_after();
            // the pass's pairs by A digit i: its B digits j = jlo..jhi are
            // consecutive 128-row tiles of the stage and their levels i + j
            // consecutive 128-column accumulator slots, so two of them make
            // one N = 256 MMA (A read once from shared memory for both).
            // Digit i = 1 is the first to write every slot of a pass.
            for (int i = 1; i <= pd.nA; ++i) {
              const int jlo = pd.first_level - i > 1 ? pd.first_level - i : 1;
              const int jtop = pd.first_level + pd.nlev - 1 - i;
              const int jhi = jtop < P.digits ? jtop : P.digits;
              const uint32_t aoff = (uint32_t)(i - 1) * TILE_BYTES;
              for (int j = jlo; j <= jhi; j += 2) {
                const bool two = j + 1 <= jhi;
                const uint32_t boff = (uint32_t)(MAXDIG + j - 1) * TILE_BYTES;
                const uint32_t dt = tbase + (uint32_t)(i + j - pd.first_level) * BN;
                for (int g = 0; g < ng; ++g) {
                  const uint32_t acc = (kb0 + g > 0 || i > 1) ? 1u : 0u;
                  umma_bf16(dt, sdesc_kmajor(sbase[g] + aoff), sdesc_kmajor(sbase[g] + boff),
                            two ? idesc2 : idesc, acc);
                }
              }
            }
            for (int g = 0; g < ng; ++g) {
              int sg = stage + g;
              if (sg >= NSTAGE) sg -= NSTAGE;
              umma_commit(smem_u32(&empty_bar[sg]));  // frees the stage when done
            }
            stage += ng;
            if (stage >= NSTAGE) { stage -= NSTAGE; phase ^= 1; }
          }
          umma_commit(smem_u32(&acc_full));  // accumulators complete
        }
      }
    }
  } else {
    // ---------------- epilogue (warps 2..5, one TMEM lane quarter each) ----------------
    const int quarter = warp & 3;
    const int row = quarter * 32 + lane;  // TMEM lane = packed column within the tile
    const uint32_t tlane = tbase + ((uint32_t)(quarter * 32) << 16);
    uint32_t accph = 0;
    for (int t = blockIdx.x; t < ntiles && !abort_; t += gridDim.x) {
      int cb, eb;
      tile_coords(t, P, cb, eb);
      const int c = cb * BM + row;
      const bool cok = c < P.ncols;
      const int kc = cok ? pow2_exponent(mscale[c]) : 0;
      for (int ps = 0; ps < P.npass; ++ps) {
        const PassDesc& pd = P.pass[ps];
        if (!mbar_wait(smem_u32(&acc_full), accph, &abort_)) {
          abort_ = 1; atomicExch(err, 4); break;
        }
        accph ^= 1;
        tc_fence_after();
        for (int ch = 0; ch < BN / 16; ++ch) {
          const int e0 = eb * BN + ch * 16;
          switch (pd.nlev) {
            case 1: epi_chunk<1>(P, ps, tlane, ch, e0, c, cok, kc, dscale, PK, lane); break;
            case 2: epi_chunk<2>(P, ps, tlane, ch, e0, c, cok, kc, dscale, PK, lane); break;
            case 3: epi_chunk<3>(P, ps, tlane, ch, e0, c, cok, kc, dscale, PK, lane); break;
            default: epi_chunk<4>(P, ps, tlane, ch, e0, c, cok, kc, dscale, PK, lane); break;
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
                 "r"(TMEM_COLS));
  }
}

// ---------------------------------------------------------------------------
// digit builders
// ---------------------------------------------------------------------------
// Digit tiles in HBM: tile (block, k-block, digit) = 128 rows x 16 q in the
// UMMA canonical K-major layout; byte offset of (row r, q-in-block k):
//   (r/8)*256 + (k/8)*128 + (r%8)*16 + (k%8)*2
// Tiles of one (block, k-block) are consecutive over the digits.
__host__ __device__ __forceinline__ size_t tile_base(int blk, int kb, int dig, int nk, int ndig) {
  return (((size_t)blk * nk + kb) * ndig + dig) * (size_t)TILE_BYTES;
}

__device__ __forceinline__ double pow2_ceil_scale(double mx) {
  if (!(mx > 0.0)) return 1.0;
  int ex;
  frexp(mx, &ex);  // mx = m 2^ex, m in [0.5, 1)
  return ldexp(1.0, ex);
}

__device__ __forceinline__ uint32_t bf16pair(double lo, double hi) {
  __nv_bfloat16 a = __float2bfloat16_rn((float)lo), b = __float2bfloat16_rn((float)hi);
  return (uint32_t)(*(uint16_t*)&a) | ((uint32_t)(*(uint16_t*)&b) << 16);
}

// M[q, c] for q = (l, comp), c = packed index (pk_index order)
__device__ __forceinline__ double m_entry(const double* __restrict__ grad, int n, int l, int comp,
                                          int a, int b) {
  const double* g = grad + (size_t)l * 3 * n;
  int i = comp < 3 ? comp : (comp == 5 ? 1 : 0);
  int j = comp < 3 ? comp : (comp == 3 ? 1 : 2);
  double v = g[i * n + a] * g[j * n + b];
  if (i != j) v += g[j * n + a] * g[i * n + b];
  return v;
}

__device__ inline void pk_decode(int64_t c, int ni, int nb, int& a, int& b) {
  int64_t nbb = (int64_t)nb * (nb + 1) / 2, nbi = (int64_t)nb * ni;
  if (c < nbb) {
    int cc = (int)((sqrt(8.0 * (double)c + 1.0) - 1.0) * 0.5);
    while ((int64_t)(cc + 1) * (cc + 2) / 2 <= c) ++cc;
    while ((int64_t)cc * (cc + 1) / 2 > c) --cc;
    a = ni + (int)(c - (int64_t)cc * (cc + 1) / 2);
    b = ni + cc;
  } else if (c < nbb + nbi) {
    int64_t r = c - nbb;
    a = (int)(r / nb);           // interface
    b = ni + (int)(r % nb);      // bubble
  } else {
    int64_t r = c - nbb - nbi;
    int bb = (int)((sqrt(8.0 * (double)r + 1.0) - 1.0) * 0.5);
    while ((int64_t)(bb + 1) * (bb + 2) / 2 <= r) ++bb;
    while ((int64_t)bb * (bb + 1) / 2 > r) --bb;
    a = (int)(r - (int64_t)bb * (bb + 1) / 2);
    b = bb;
  }
}

// column scales of M: 2^ceil(log2 max_q |M[q,c]|)
__global__ void k_m_scale(int nint, int n, int ni, int nb, int ncols, int ncols_pad,
                          const double* __restrict__ grad, double* __restrict__ mscale) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols_pad) return;
  if (c >= ncols) { mscale[c] = 1.0; return; }
  int a, b;
  pk_decode(c, ni, nb, a, b);
  double mx = 0.0;
  for (int q = 0; q < 6 * nint; ++q) mx = fmax(mx, fabs(m_entry(grad, n, q / 6, q % 6, a, b)));
  mscale[c] = pow2_ceil_scale(mx);
}

// row scales of D: 2^ceil(log2 max_q |D[e,q]|); one block per element row
__global__ void k_d_scale(int K, int nel, const double* __restrict__ D, double* __restrict__ dscale) {
  int e = blockIdx.x;
  __shared__ double red[256];
  double mx = 0.0;
  if (e < nel)
    for (int q = threadIdx.x; q < K; q += blockDim.x) mx = fmax(mx, fabs(D[(size_t)e * K + q]));
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) dscale[e] = (e < nel) ? pow2_ceil_scale(red[0]) : 1.0;
}

// digits of 8 consecutive values -> one 16-byte core-matrix row per digit
__device__ __forceinline__ void write_digits8(const double* vals, double rs, int radix, int digits,
                                              uint8_t* __restrict__ base, int nk, int blk, int kb,
                                              int r, int kg) {
  double up = ldexp(1.0, radix);
  double rr[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) rr[t] = vals[t] * rs;
  const size_t off = (size_t)(r >> 3) * 256 + (size_t)kg * 128 + (size_t)(r & 7) * 16;
  for (int s = 0; s < digits; ++s) {
    double d[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      rr[t] *= up;
      d[t] = rint(rr[t]);
      rr[t] -= d[t];
    }
    uint4 w;
    w.x = bf16pair(d[0], d[1]);
    w.y = bf16pair(d[2], d[3]);
    w.z = bf16pair(d[4], d[5]);
    w.w = bf16pair(d[6], d[7]);
    *(uint4*)(base + tile_base(blk, kb, s, nk, digits) + off) = w;
  }
}

// M digit tiles: grid (k-blocks, column blocks), 256 threads = 128 rows x 2 q-groups
__global__ void k_build_m(int nint, int n, int ni, int nb, int ncols, int nk, int radix,
                          int digits, const double* __restrict__ grad,
                          const double* __restrict__ mscale, uint8_t* __restrict__ mdig) {
  const int kb = blockIdx.x, cb = blockIdx.y;
  const int r = threadIdx.x >> 1, kg = threadIdx.x & 1;
  const int c = cb * 128 + r;
  const int K = 6 * nint;
  double vals[8];
  int a = 0, b = 0;
  if (c < ncols) pk_decode(c, ni, nb, a, b);
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    int q = kb * 16 + kg * 8 + t;
    vals[t] = (c < ncols && q < K) ? m_entry(grad, n, q / 6, q % 6, a, b) : 0.0;
  }
  double rs = (c < ncols) ? 1.0 / mscale[c] : 0.0;
  write_digits8(vals, rs, radix, digits, mdig, nk, cb, kb, r, kg);
}

// dense M (K x ncols, row-major): column scales and digit tiles
__global__ void k_m_scale_dense(int K, int ncols, int ncols_pad, const double* __restrict__ Md,
                                double* __restrict__ mscale) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols_pad) return;
  if (c >= ncols) { mscale[c] = 1.0; return; }
  double mx = 0.0;
  for (int q = 0; q < K; ++q) mx = fmax(mx, fabs(Md[(size_t)q * ncols + c]));
  mscale[c] = pow2_ceil_scale(mx);
}

__global__ void k_build_m_dense(int K, int ncols, int nk, int radix, int digits,
                                const double* __restrict__ Md, const double* __restrict__ mscale,
                                uint8_t* __restrict__ mdig) {
  const int kb = blockIdx.x, cb = blockIdx.y;
  const int r = threadIdx.x >> 1, kg = threadIdx.x & 1;
  const int c = cb * 128 + r;
  double vals[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    const int q = kb * 16 + kg * 8 + t;
    vals[t] = (c < ncols && q < K) ? Md[(size_t)q * ncols + c] : 0.0;
  }
  const double rs = (c < ncols) ? 1.0 / mscale[c] : 0.0;
  write_digits8(vals, rs, radix, digits, mdig, nk, cb, kb, r, kg);
}

// D digit tiles: grid (k-blocks, element blocks), 256 threads
__global__ void k_slice_d(int K, int nk, int nel, int radix, int digits,
                          const double* __restrict__ D, const double* __restrict__ dscale,
                          uint8_t* __restrict__ ddig) {
  const int kb = blockIdx.x, eb = blockIdx.y;
  const int r = threadIdx.x >> 1, kg = threadIdx.x & 1;
  const int e = eb * 128 + r;
  double vals[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    int q = kb * 16 + kg * 8 + t;
    vals[t] = (e < nel && q < K) ? D[(size_t)e * K + q] : 0.0;
  }
  double rs = (e < nel) ? 1.0 / dscale[e] : 0.0;
  write_digits8(vals, rs, radix, digits, ddig, nk, eb, kb, r, kg);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {
int round_up(int v, int m) { return (v + m - 1) / m * m; }
}  // namespace

int ozaki_plan(int nint, int n, int radix, int digits, OzakiPlan* plan) {
  if (radix <= 0) radix = 7;
  if (digits <= 0) digits = 7;
  if (radix < 4 || radix > 8 || digits < 2 || digits > MAXDIG) return -1;
  plan->radix = radix;
  plan->digits = digits;
  plan->levels = digits;  // levels 2 .. digits+1
  plan->kdim = round_up(6 * nint, BK);
  plan->ncols = round_up(n * (n + 1) / 2, BM);
  return 0;
}

int ozaki_plan_dense(int K, int ncols, int radix, int digits, OzakiPlan* plan) {
  if (radix < 4 || radix > 8 || digits < 2 || digits > MAXDIG || K <= 0 || ncols <= 0) return -1;
  plan->radix = radix;
  plan->digits = digits;
  plan->levels = digits;
  plan->kdim = round_up(K, BK);
  plan->ncols = round_up(ncols, BM);
  plan->kreal = K;
  plan->nreal = ncols;
  return 0;
}

size_t ozaki_m_bytes(const OzakiPlan& p) { return (size_t)p.digits * p.ncols * p.kdim * 2; }
size_t ozaki_d_bytes(const OzakiPlan& p, int nel) {
  return (size_t)p.digits * round_up(nel, BN) * p.kdim * 2;
}

int launch_ozaki_build_m(const OzakiPlan& p, int nint, int n, int ni, int nb, const double* d_grad,
                         uint16_t* d_mdig, double* d_mscale, double* d_work, cudaStream_t st) {
  (void)d_work;
  int ncols = n * (n + 1) / 2;
  k_m_scale<<<p.ncols / 128, 128, 0, st>>>(nint, n, ni, nb, ncols, p.ncols, d_grad, d_mscale);
  dim3 g(p.kdim / BK, p.ncols / BM);
  k_build_m<<<g, 256, 0, st>>>(nint, n, ni, nb, ncols, p.kdim / BK, p.radix, p.digits, d_grad,
                               d_mscale, (uint8_t*)d_mdig);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_ozaki_slice_d(const OzakiPlan& p, int nel, int nint, const double* d_D,
                         uint16_t* d_ddig, double* d_dscale, cudaStream_t st) {
  int nel_pad = round_up(nel, BN);
  if (nel_pad == 0) return 0;
  k_d_scale<<<nel_pad, 256, 0, st>>>(6 * nint, nel, d_D, d_dscale);
  dim3 g(p.kdim / BK, nel_pad / BN);
  k_slice_d<<<g, 256, 0, st>>>(6 * nint, p.kdim / BK, nel, p.radix, p.digits, d_D, d_dscale,
                               (uint8_t*)d_ddig);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_ozaki_build_m_dense(const OzakiPlan& p, const double* d_M, uint16_t* d_mdig,
                               double* d_mscale, cudaStream_t st) {
  k_m_scale_dense<<<p.ncols / 128, 128, 0, st>>>(p.kreal, p.nreal, p.ncols, d_M, d_mscale);
  dim3 g(p.kdim / BK, p.ncols / BM);
  k_build_m_dense<<<g, 256, 0, st>>>(p.kreal, p.nreal, p.kdim / BK, p.radix, p.digits, d_M,
                                     d_mscale, (uint8_t*)d_mdig);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_ozaki_slice_d_dense(const OzakiPlan& p, int nrows, const double* d_D, uint16_t* d_ddig,
                               double* d_dscale, cudaStream_t st) {
  int nel_pad = round_up(nrows, BN);
  if (nel_pad == 0) return 0;
  k_d_scale<<<nel_pad, 256, 0, st>>>(p.kreal, nrows, d_D, d_dscale);
  dim3 g(p.kdim / BK, nel_pad / BN);
  k_slice_d<<<g, 256, 0, st>>>(p.kreal, p.kdim / BK, nrows, p.radix, p.digits, d_D, d_dscale,
                               (uint8_t*)d_ddig);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

// pass / pair table: levels 2..digits+1 in passes of <= 4 accumulators
static void build_params(const OzakiPlan& p, GemmParams* G) {
  memset(G, 0, sizeof(*G));
  G->radix = p.radix;
  int lev_lo = 2, lev_hi = p.digits + 1;
  int np = 0, npair = 0;
  for (int L0 = lev_lo; L0 <= lev_hi; L0 += 4) {
    PassDesc& pd = G->pass[np++];
    pd.first_level = L0;
    pd.nlev = (lev_hi - L0 + 1) < 4 ? (lev_hi - L0 + 1) : 4;
    pd.pair0 = npair;
    pd.nA = pd.nB = 0;
    for (int s = L0; s < L0 + pd.nlev; ++s) {
      bool first = true;
      for (int i = 1; i <= p.digits; ++i) {
        int j = s - i;
        if (j < 1 || j > p.digits) continue;
        G->pi[npair] = (int8_t)i;
        G->pj[npair] = (int8_t)j;
        G->pslot[npair] = (int8_t)(s - L0);
        G->pfirst[npair] = first ? 1 : 0;
        first = false;
        pd.nA = pd.nA > i ? pd.nA : i;
        pd.nB = pd.nB > j ? pd.nB : j;
        ++npair;
      }
    }
    pd.npair = npair - pd.pair0;
  }
  G->npass = np;
  G->npairs = npair;
  const PassDesc& p0 = G->pass[0];
  int last0 = p0.first_level + p0.nlev - 1;
  if (np == 2) {
    G->s1 = 62 - (24 + p.radix * (p0.nlev - 1));
    G->scale_shift = p.radix * last0 + G->s1;
  } else {
    G->s1 = 0;
    G->scale_shift = p.radix * last0;
  }
}

int ozaki_pairs(const OzakiPlan& p) {
  GemmParams G;
  build_params(p, &G);
  return G.npairs;
}

static int ozaki_gemm_cols(const OzakiPlan& p, int nel, int ncols_real, const uint16_t* d_ddig,
                           const double* d_dscale, const uint16_t* d_mdig, const double* d_mscale,
                           double* d_PK, int* d_flag, cudaStream_t st);

int launch_ozaki_gemm(const OzakiPlan& p, int nel, int n, const uint16_t* d_ddig,
                      const double* d_dscale, const uint16_t* d_mdig, const double* d_mscale,
                      double* d_PK, int* d_flag, cudaStream_t st) {
  return ozaki_gemm_cols(p, nel, n * (n + 1) / 2, d_ddig, d_dscale, d_mdig, d_mscale, d_PK, d_flag,
                         st);
}

int launch_ozaki_gemm_dense(const OzakiPlan& p, int nrows, const uint16_t* d_ddig,
                            const double* d_dscale, const uint16_t* d_mdig, const double* d_mscale,
                            double* d_out, int* d_flag, cudaStream_t st) {
  return ozaki_gemm_cols(p, nrows, p.nreal, d_ddig, d_dscale, d_mdig, d_mscale, d_out, d_flag, st);
}

static int ozaki_gemm_cols(const OzakiPlan& p, int nel, int ncols_real, const uint16_t* d_ddig,
                           const double* d_dscale, const uint16_t* d_mdig, const double* d_mscale,
                           double* d_PK, int* d_flag, cudaStream_t st) {
  if (nel <= 0) return 0;
  static int num_sms = 0;
  if (!num_sms) {
    int dev;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  GemmParams G;
  build_params(p, &G);
  int nel_pad = round_up(nel, BN);
  G.nk = p.kdim / BK;
  G.digits = p.digits;
  G.ncb = p.ncols / BM;
  G.neb = nel_pad / BN;
  G.nel = nel;
  G.ncols = ncols_real;
  size_t smem = (size_t)NSTAGE * STAGE_BYTES + 1024;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_ozaki_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return -1;
    attr = true;
  }
  int ntiles = G.ncb * G.neb;
  int grid = ntiles < num_sms ? ntiles : num_sms;
  k_ozaki_gemm<<<grid, NTHREADS, smem, st>>>((const uint8_t*)d_mdig, (const uint8_t*)d_ddig, G,
                                              d_dscale, d_mscale, d_PK, d_flag);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace hp3dg
