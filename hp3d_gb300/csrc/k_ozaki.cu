// k_ozaki.cu -- mixed-precision B^T D B contraction on tcgen05 tensor cores.
//
// The stiffness of every element of a bin is one row of a GEMM with a shared
// operand (elem_opt.F90:86-137 computes it per element as A_TEST*A_TEST^T):
//
//   PK[e, c] = sum_q D[e, q] M[q, c],   q = (point l, component pair ij),
//   c = packed (a <= b) entry,  M[(l,ij), (a,b)] = G_i[l,a] G_j[l,b] (+ sym).
//
// Both operands are FP64.  They are split into balanced integer digits of R
// = `radix` bits, scaled per element row / per column by powers of two:
//   D = s_e * sum_i d_i 2^(-R i),   M = t_c * sum_j m_j 2^(-R j),
// with |d_1|, |m_1| <= 2^R and every later digit <= 2^(R-1), all exact in
// BF16.  A digit product d_i m_j is exact in FP32; the products of one level
// s = i + j (s = 2 .. digits+1) are summed into one FP32 TMEM accumulator.
//
// Exactness, a priori: the accumulators are restarted every `kchunk`
// k-blocks (16 q each), with kchunk * 16 * max_s sum_{i+j=s} b_i b_j <= 2^24
// (b_1 = 2^R, b_i = 2^(R-1)): every partial sum of every level, in any order
// of accumulation, is an integer of magnitude below 2^24 and therefore exact
// in FP32.  At R = 7 and 7 digits the largest level bound per q is
// 2 * 2^13 + 5 * 2^12 = 36864, so kchunk = 28 (448 q; K = 2058 at p = 5 with
// INTEGRATION = 1 is five runs).  After each run the epilogue adds the levels
// exactly into one 64-bit integer per output, V += sum_s L_s 2^(R(S-s) - t)
// (S = the last level, t >= 0 chosen so that |V| < 2^62 over all runs; only
// the last level loses its t low bits), and at the end forms the FP64 result
// V 2^(ke + kc - R S + t) with one rounding (the FP64 recombination of the
// split): the result carries about R * digits bits.
//
// Kernel structure (one CTA per SM, persistent over 128 x 64 output tiles):
//   warp 0    producer: per k-block one contiguous bulk copy (cp.async.bulk)
//             of the A = M digit tiles (128 packed columns x 16 q each) and
//             one of the B = D digit tiles (64 elements x 16 q each); digits
//             are stored in HBM already in the UMMA canonical K-major layout
//             (8-row x 16-byte core matrices), ring of 5 stages
//   warp 1    TMEM allocation (512 columns) and the single MMA-issuing thread:
//             every level has its own 64-column slot, all levels of a tile in
//             one pass (7 x 64 = 448 columns); the B digits j of one A digit i
//             are consecutive tiles in shared memory and their levels i + j
//             consecutive slots, so up to four pairs run as one
//             128 x 256 x 16 MMA (A read once for all of them)
//   warps 2-17 epilogue: after each accumulation run tcgen05.ld of the level
//             accumulators (warp w reads TMEM lane quarter w % 4, elements
//             16 (w - 2) / 4 ..), exact integer accumulation; after the last
//             run FP64 assembly from the bits and coalesced stores of PK
// Every mbarrier wait is bounded; a role that gives up sets the error flag and
// the abort word, the MMA thread and the producer wait (bounded) for their own
// tensor-core and copy work in flight, and TMEM is freed before the CTA exits.
#include "../../include/hp3dg.h"
#include "hp3dg_internal.cuh"
#include "hp3dg_kernels.h"
#include "hp3dg_tc.cuh"

#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

namespace hp3dg {

namespace {
constexpr int BM = 128;       // packed columns per tile (MMA M, TMEM lanes)
constexpr int BN = 64;        // elements per tile (TMEM columns per level slot)
constexpr int BK = 16;        // q per k-block (one MMA K step), 32-byte rows
constexpr int MAXDIG = 7;
constexpr int MAXSTAGE = 8;
constexpr int KGROUP = 2;     // k-blocks per accumulator run between slot switches
constexpr int A_TILE = BM * BK * 2;          // 4096 bytes: one M digit tile
constexpr int B_TILE = BN * BK * 2;          // 2048 bytes: one D digit tile
constexpr int B_OFF = MAXDIG * A_TILE;       // B digits after the A digits in a stage
constexpr int STAGE_BYTES = MAXDIG * (A_TILE + B_TILE);  // 43008
constexpr int NEPI = 16;                     // epilogue warps
constexpr int EPI_ELEMS = BN / (NEPI / 4);   // 16 elements per epilogue warp
constexpr int NTHREADS = 64 + 32 * NEPI;     // 576
constexpr uint32_t TMEM_COLS = 512;
constexpr int MAXMMA = 16;

// One bin of a grouped launch: its operands, outputs and tile space.
struct GemmBin {
  const uint8_t* A;          // M digit tiles
  const uint8_t* B;          // D digit tiles
  const double* dscale;
  const double* mscale;
  double* PK;
  int nk;                    // k-blocks
  int nchunk;                // exact accumulation runs per tile
  int ncb, neb;              // column / element blocks
  int nel, ncols;
  int grp;                   // column blocks per raster group
  int tile0;                 // first tile of the bin in the launch's tile space
  int shift0;                // slot s: V += L << (shift0 - radix s), or >> when negative
  int scale_shift;           // PK = V * 2^(ke + kc - scale_shift)
};
constexpr int MAXBINS = OZAKI_MAXBINS;
struct GemmParams {
  int radix, digits, nlev;  // levels 2 .. digits+1 in slots 0 .. nlev-1
  int kchunk;               // k-blocks per exact accumulation run
  int nstage;
  long wait_limit;          // bounded mbarrier waits (iterations)
  int fault;                // testing: 1 = the producer withholds one stage
  int nmma;                 // MMAs per k-block, in issue order:
  uint32_t mma[MAXMMA];     // A digit i | first B digit j0 << 4 | B digit count << 8
  int nbins, ntiles;
  GemmBin bin[MAXBINS];
};
static_assert(sizeof(GemmParams) <= 32764, "kernel parameter space");
}  // namespace

// the bin of tile t (bins in tile order)
__device__ __forceinline__ int find_bin(const GemmParams& P, int t) {
  int lo = 0, hi = P.nbins - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (P.bin[mid].tile0 <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// local tile t of bin B -> (column block, element block): groups of `grp`
// column blocks sweep all element blocks, so the M digit strips of a group
// stay resident in L2.
__device__ __forceinline__ void tile_coords(int t, const GemmBin& B, int& cb, int& eb) {
  const int grp = B.grp;
  int g = t / (grp * B.neb);
  int r = t - g * grp * B.neb;
  int gw = B.ncb - g * grp;
  if (gw > grp) gw = grp;
  cb = g * grp + r % gw;
  eb = r / gw;
}

// instruction descriptor: kind::f16, A = B = BF16, D = F32, both K-major, M = 128
__host__ __device__ constexpr uint32_t idesc_bf16_m128(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

// exponent k of an exact power of two 2^k (the digit scales)
__device__ __forceinline__ int pow2_exponent(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7ff) - 1023;
}

// ---------------------------------------------------------------------------
// the GEMM
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS, 1)
    k_ozaki_gemm(const __grid_constant__ GemmParams P, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smraw[];
  uint8_t* ring = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full_bar[MAXSTAGE], empty_bar[MAXSTAGE];
  __shared__ __align__(8) uint64_t acc_full, acc_empty, drain_bar;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = P.ntiles;
  const long lim = P.wait_limit;

  if (threadIdx.x == 0) {
    for (int s = 0; s < P.nstage; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    mbar_init(smem_u32(&acc_full), 1);
    mbar_init(smem_u32(&acc_empty), NEPI);
    mbar_init(smem_u32(&drain_bar), 1);
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
    // ---------------- producer ----------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      uint32_t issued = 0, last_par = 0;  // per stage: a copy issued / its phase parity
      const uint32_t bytes = (uint32_t)P.digits * (A_TILE + B_TILE);
      bool withheld = false;
      for (int t = blockIdx.x; t < ntiles && !abort_; t += gridDim.x) {
        const GemmBin& B = P.bin[find_bin(P, t)];
        int cb, eb;
        tile_coords(t - B.tile0, B, cb, eb);
        for (int kb = 0; kb < B.nk; ++kb) {
          if (!mbar_wait_n(smem_u32(&empty_bar[stage]), phase ^ 1, &abort_, lim)) {
            abort_ = 1; atomicExch(err, 1); break;
          }
          if (P.fault == 1 && !withheld && kb == 1) {
            // testing: this stage is never filled, so the MMA thread's bounded
            // wait on it runs out
            withheld = true;
            issued &= ~(1u << stage);
          } else {
            const uint32_t fb = smem_u32(&full_bar[stage]);
            mbar_expect_tx(fb, bytes);
            uint8_t* st = ring + (size_t)stage * STAGE_BYTES;
            // digits 0..D-1 of (column block, k-block) are contiguous, likewise for B
            const size_t ablk = ((size_t)cb * B.nk + kb) * P.digits;
            const size_t bblk = ((size_t)eb * B.nk + kb) * P.digits;
            bulk_load(smem_u32(st), B.A + ablk * A_TILE, (uint32_t)P.digits * A_TILE, fb);
            bulk_load(smem_u32(st + B_OFF), B.B + bblk * B_TILE, (uint32_t)P.digits * B_TILE, fb);
            issued |= 1u << stage;
            last_par = (last_par & ~(1u << stage)) | (phase << stage);
          }
          if (++stage == P.nstage) { stage = 0; phase ^= 1; }
        }
      }
      // the copies this thread started have landed before the CTA exits
      for (int s = 0; s < P.nstage; ++s)
        if (issued >> s & 1u) mbar_drain(smem_u32(&full_bar[s]), (last_par >> s) & 1u, lim);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0, accph = 0;
      bool any = false;
      for (int t = blockIdx.x; t < ntiles && !abort_; t += gridDim.x) {
        const GemmBin& B = P.bin[find_bin(P, t)];
        const int nk = B.nk, nchunk = B.nchunk;
        for (int ch = 0; ch < nchunk && !abort_; ++ch) {
          const int kc0 = ch * P.kchunk;
          const int kc1 = (kc0 + P.kchunk) < nk ? (kc0 + P.kchunk) : nk;
          // the epilogue must have drained the accumulators
          if (!mbar_wait_n(smem_u32(&acc_empty), accph ^ 1, &abort_, lim)) {
            abort_ = 1; atomicExch(err, 2); break;
          }
          accph ^= 1;
          tc_fence_after();
          for (int kb0 = kc0; kb0 < kc1 && !abort_; kb0 += KGROUP) {
            const int ng = (kc1 - kb0) < KGROUP ? (kc1 - kb0) : KGROUP;
            uint32_t sbase[KGROUP];
#pragma unroll
            for (int g = 0; g < KGROUP; ++g) {
              sbase[g] = 0;
              if (g >= ng || abort_) continue;
              int sg = stage + g;
              uint32_t pg = phase;
              if (sg >= P.nstage) { sg -= P.nstage; pg ^= 1; }
              if (!mbar_wait_n(smem_u32(&full_bar[sg]), pg, &abort_, lim)) {
                abort_ = 1; atomicExch(err, 3); continue;
              }
              sbase[g] = smem_u32(ring + (size_t)sg * STAGE_BYTES);
            }
            if (abort_) break;
            tc_fence_after();
            // A digit i pairs with B digits j = 1 .. min(D, S - i) (levels
            // i + j <= S = D + 1); their slots i + j - 2 are consecutive, so
            // up to four B tiles make one MMA of N = 64 * count.  The MMAs
            // come in the host's order (no MMA follows one whose accumulator
            // range overlaps its own without being equal); the two of digit
            // i = 1 come first, cover every slot and start each run.
#pragma unroll
            for (int ci = 0; ci < MAXMMA; ++ci) {
              if (ci >= P.nmma) break;
              const uint32_t m = P.mma[ci];
              const int i = (int)(m & 15u), j0 = (int)((m >> 4) & 15u), nd = (int)(m >> 8);
              const uint32_t aoff = (uint32_t)(i - 1) * A_TILE;
              const uint32_t idesc = idesc_bf16_m128(BN * nd);
              const uint32_t boff = (uint32_t)(B_OFF + (j0 - 1) * B_TILE);
              const uint32_t dt = tbase + (uint32_t)(i + j0 - 2) * BN;
#pragma unroll
              for (int g = 0; g < KGROUP; ++g) {
                if (g >= ng) continue;
                const uint32_t acc = (kb0 + g > kc0 || i > 1) ? 1u : 0u;
                umma_bf16(dt, sdesc_kmajor(sbase[g] + aoff), sdesc_kmajor(sbase[g] + boff),
                          idesc, acc);
              }
            }
            any = true;
            for (int g = 0; g < ng; ++g) {
              int sg = stage + g;
              if (sg >= P.nstage) sg -= P.nstage;
              umma_commit(smem_u32(&empty_bar[sg]));  // frees the stage when done
            }
            stage += ng;
            if (stage >= P.nstage) { stage -= P.nstage; phase ^= 1; }
          }
          if (abort_) break;
          umma_commit(smem_u32(&acc_full));  // this run's level sums are complete
        }
      }
      // every MMA this thread issued has completed before TMEM is freed
      if (any) {
        umma_commit(smem_u32(&drain_bar));
        mbar_drain(smem_u32(&drain_bar), 0, lim);
      }
    }
  } else {
    // ---------------- epilogue (warps 2..17) ----------------
    const int quarter = warp & 3;              // TMEM lanes this warp may read
    const int eg = (warp - 2) >> 2;            // its 16 elements of the tile
    const int row = quarter * 32 + lane;       // TMEM lane = packed column in the tile
    const uint32_t tlane = tbase + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(eg * EPI_ELEMS);
    uint32_t accph = 0;
    for (int t = blockIdx.x; t < ntiles && !abort_; t += gridDim.x) {
      const GemmBin& B = P.bin[find_bin(P, t)];
      int cb, eb;
      tile_coords(t - B.tile0, B, cb, eb);
      const int c = cb * BM + row;
      const bool cok = c < B.ncols;
      const int e0 = eb * BN + eg * EPI_ELEMS;
      const int el = e0 + (lane & 15);
      // exponents of the element scale (of element lane & 15) and of this
      // lane's column scale, less the recombination shift
      const int ke_lane = (el < B.nel) ? pow2_exponent(B.dscale[el]) : 0;
      const int kcs = (cok ? pow2_exponent(B.mscale[c]) : 0) - B.scale_shift;
      long long V[EPI_ELEMS];
#pragma unroll
      for (int q = 0; q < EPI_ELEMS; ++q) V[q] = 0;
      bool ok = true;
      for (int ch = 0; ch < B.nchunk; ++ch) {
        if (!mbar_wait_n(smem_u32(&acc_full), accph, &abort_, lim)) {
          abort_ = 1; atomicExch(err, 4); ok = false; break;
        }
        accph ^= 1;
        tc_fence_after();
        for (int s = 0; s < P.nlev; ++s) {
          uint32_t v[EPI_ELEMS];
          tmem_ld16(tlane + (uint32_t)(s * BN), v);
          const int sh = B.shift0 - P.radix * s;
          if (sh >= 0) {
#pragma unroll
            for (int q = 0; q < EPI_ELEMS; ++q)
              V[q] += (long long)__float2int_rn(__uint_as_float(v[q])) << sh;
          } else {
#pragma unroll
            for (int q = 0; q < EPI_ELEMS; ++q)
              V[q] += (long long)__float2int_rn(__uint_as_float(v[q])) >> (-sh);
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&acc_empty));
      }
      if (!ok) break;
      double* PK = B.PK;
      const int nel = B.nel, ncols = B.ncols;
#pragma unroll
      for (int q = 0; q < EPI_ELEMS; ++q) {
        const int ke = __shfl_sync(0xffffffffu, ke_lane, q);
        const int e = e0 + q;
        if (cok && e < nel) PK[(size_t)e * ncols + c] = scaled_i64(V[q], ke + kcs);
      }
    }
  }
  tc_fence_before();
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
// Digit tiles in HBM: tile (block, k-block, digit) = rows x 16 q in the UMMA
// canonical K-major layout (M: 128 packed columns per block, 4 KB tiles; D:
// 64 elements per block, 2 KB tiles); byte offset of (row r, q-in-block k):
//   (r/8)*256 + (k/8)*128 + (r%8)*16 + (k%8)*2
// Tiles of one (block, k-block) are consecutive over the digits, so the 64-row
// D tiles of consecutive digits form one canonical operand of 64 * count rows.
__host__ __device__ __forceinline__ size_t tile_base(int blk, int kb, int dig, int nk, int ndig,
                                                     int tile_bytes) {
  return (((size_t)blk * nk + kb) * ndig + dig) * (size_t)tile_bytes;
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
__device__ __forceinline__ void d_scale_row(int e, int K, int nel, const double* __restrict__ D,
                                            double* __restrict__ dscale) {
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

__global__ void k_d_scale(int K, int nel, const double* __restrict__ D, double* __restrict__ dscale) {
  d_scale_row(blockIdx.x, K, nel, D, dscale);
}

// digits of 8 consecutive values -> one 16-byte core-matrix row per digit
__device__ __forceinline__ void write_digits8(const double* vals, double rs, int radix, int digits,
                                              uint8_t* __restrict__ base, int nk, int blk, int kb,
                                              int r, int kg, int tile_bytes) {
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
    *(uint4*)(base + tile_base(blk, kb, s, nk, digits, tile_bytes) + off) = w;
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
  write_digits8(vals, rs, radix, digits, mdig, nk, cb, kb, r, kg, A_TILE);
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
  write_digits8(vals, rs, radix, digits, mdig, nk, cb, kb, r, kg, A_TILE);
}

// D digit tiles: grid (k-blocks, 64-element blocks), 128 threads = 64 rows x 2 q-groups
__device__ __forceinline__ void slice_d_tile(int kb, int eb, int K, int nk, int nel, int radix,
                                             int digits, const double* __restrict__ D,
                                             const double* __restrict__ dscale,
                                             uint8_t* __restrict__ ddig) {
  const int r = threadIdx.x >> 1, kg = threadIdx.x & 1;
  const int e = eb * BN + r;
  double vals[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    int q = kb * 16 + kg * 8 + t;
    vals[t] = (e < nel && q < K) ? D[(size_t)e * K + q] : 0.0;
  }
  // the row scale is 2^ex: each value becomes the integer round(v 2^(R D - ex))
  // from its bits, split into balanced digits in integer arithmetic (GB300
  // issues FP64 and its conversions at about 2 per clock per SM)
  const int ex = (e < nel) ? (int)((__double_as_longlong(dscale[e]) >> 52) & 0x7ff) - 1023 : 0;
  long long X[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) X[t] = (e < nel) ? fixed_of(vals[t], ex, radix * digits) : 0;
  const size_t off = (size_t)(r >> 3) * 256 + (size_t)kg * 128 + (size_t)(r & 7) * 16;
  store_digits8(X, radix, digits, ddig + tile_base(eb, kb, 0, nk, digits, B_TILE) + off, B_TILE);
}

__global__ void k_slice_d(int K, int nk, int nel, int radix, int digits,
                          const double* __restrict__ D, const double* __restrict__ dscale,
                          uint8_t* __restrict__ ddig) {
  slice_d_tile(blockIdx.x, blockIdx.y, K, nk, nel, radix, digits, D, dscale, ddig);
}

// the same over the bins of a group: one block per (padded) element row, and
// one per (k-block, 64-element block) of each bin
__device__ __forceinline__ int group_seg(const int* __restrict__ pre, int nseg, int b) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
__global__ void k_d_scale_grp(const StageSeg* __restrict__ segs, const int* __restrict__ pre,
                              int nseg, int off) {
  const int blk = blockIdx.x + off;
  const int s = group_seg(pre, nseg, blk);
  const StageSeg& G = segs[s];
  d_scale_row(blk - pre[s], G.K, G.nel, G.D, G.dscale);
}
__global__ void k_slice_d_grp(const StageSeg* __restrict__ segs, const int* __restrict__ pre,
                              int nseg, int off) {
  const int blk = blockIdx.x + off;
  const int s = group_seg(pre, nseg, blk);
  const StageSeg& G = segs[s];
  const int loc = blk - pre[s];
  slice_d_tile(loc % G.nk, loc / G.nk, G.K, G.nk, G.nel, G.radix, G.digits, G.D, G.dscale,
               (uint8_t*)G.ddig);
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
  k_slice_d<<<g, 2 * BN, 0, st>>>(6 * nint, p.kdim / BK, nel, p.radix, p.digits, d_D, d_dscale,
                                  (uint8_t*)d_ddig);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_slice_d_grouped(const StageGroup& g, int k0, int k1, cudaStream_t st) {
  if (k1 <= k0) return 0;
  const int* h = g.h_pre.data();
  const int ns = g.nseg + 1;
  const int d0 = h[2 * ns + k0], d1 = h[2 * ns + k1], s0 = h[3 * ns + k0], s1 = h[3 * ns + k1];
  if (d1 > d0) k_d_scale_grp<<<d1 - d0, 256, 0, st>>>(g.segs, g.pre_dsc, g.nseg, d0);
  if (s1 > s0) k_slice_d_grp<<<s1 - s0, 2 * BN, 0, st>>>(g.segs, g.pre_slice, g.nseg, s0);
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
  k_slice_d<<<g, 2 * BN, 0, st>>>(p.kreal, p.kdim / BK, nrows, p.radix, p.digits, d_D, d_dscale,
                                  (uint8_t*)d_ddig);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

// MMA order of a k-block.  Slots of A digit i: [i-1, D-1], split at slot
// h = min(D, 4) into a low MMA [i-1, h-1] and a high MMA [max(i-1, h), D-1]
// (at most four B tiles each).  An MMA that accumulates into a range that
// overlaps the previous MMA's without being equal waits for it to finish, so
// the order is searched (depth first, a few thousand nodes at 7 digits) for
// the fewest such neighbours, the last MMA counted against the first of the
// next k-block.  The i = 1 MMAs come first: they restart every slot.
namespace {
struct MmaChunk { int i, lo, hi; };
struct OrderSearch {
  std::vector<MmaChunk> c;
  std::vector<int> best, cur;
  std::vector<char> used;
  int best_cost = 1 << 30;
  long nodes = 0;
  static int hazard(const MmaChunk& a, const MmaChunk& b) {
    const bool same = a.lo == b.lo && a.hi == b.hi;
    const bool disjoint = a.hi < b.lo || b.hi < a.lo;
    return (same || disjoint) ? 0 : 1;
  }
  void dfs(int cost) {
    if (cost >= best_cost || ++nodes > 200000) return;
    if (cur.size() == c.size()) {
      const int total = cost + hazard(c[cur.back()], c[cur.front()]);
      if (total < best_cost) { best_cost = total; best = cur; }
      return;
    }
    for (size_t k = 0; k < c.size(); ++k) {
      if (used[k]) continue;
      used[k] = 1;
      const int add = cur.empty() ? 0 : hazard(c[cur.back()], c[k]);
      cur.push_back((int)k);
      dfs(cost + add);
      cur.pop_back();
      used[k] = 0;
    }
  }
};
}  // namespace

static void build_mma_order(int D, GemmParams* G) {
  const int h = D < 4 ? D : 4;
  OrderSearch S;
  std::vector<MmaChunk> first;
  for (int i = 1; i <= D; ++i) {
    if (i - 1 < h) (i == 1 ? first : S.c).push_back({i, i - 1, h - 1});
    if (D > h) (i == 1 ? first : S.c).push_back({i, i - 1 > h ? i - 1 : h, D - 1});
  }
  // the i = 1 MMAs are disjoint; they open the order, the rest is searched
  S.c.insert(S.c.begin(), first.begin(), first.end());
  S.used.assign(S.c.size(), 0);
  for (size_t k = 0; k < first.size(); ++k) {
    S.used[k] = 1;
    S.cur.push_back((int)k);
  }
  S.dfs(0);
  G->nmma = (int)S.best.size();
  for (int k = 0; k < G->nmma; ++k) {
    const MmaChunk& m = S.c[S.best[k]];
    const int j0 = m.lo - m.i + 2, nd = m.hi - m.lo + 1;
    G->mma[k] = (uint32_t)m.i | ((uint32_t)j0 << 4) | ((uint32_t)nd << 8);
  }
}

// Exactness parameters shared by every bin of a plan's digits (file header).
static void build_params(const OzakiPlan& p, GemmParams* G) {
  memset(G, 0, sizeof(*G));
  const int R = p.radix, D = p.digits, S = D + 1;
  G->radix = R;
  G->digits = D;
  G->nlev = D;
  // largest level bound per q: sum over i + j = s of b_i b_j
  double worst = 0.0;
  for (int s = 2; s <= S; ++s) {
    double b = 0.0;
    for (int i = 1; i <= D; ++i) {
      const int j = s - i;
      if (j < 1 || j > D) continue;
      b += ldexp(1.0, i == 1 ? R : R - 1) * ldexp(1.0, j == 1 ? R : R - 1);
    }
    worst = b > worst ? b : worst;
  }
  int kchunk = (int)floor(ldexp(1.0, 24) / (BK * worst));
  kchunk = kchunk / KGROUP * KGROUP;
  G->kchunk = kchunk < KGROUP ? KGROUP : kchunk;
  // (a kchunk of KGROUP always satisfies the bound for R <= 8: 2 * 16 * 147456 < 2^24)
  build_mma_order(D, G);
}

// One bin's tile space and recombination shifts.
static void build_bin(const OzakiGemmItem& it, int kchunk, GemmBin* b) {
  const OzakiPlan& p = *it.plan;
  const int R = p.radix, D = p.digits, S = D + 1;
  b->A = (const uint8_t*)it.mdig;
  b->B = (const uint8_t*)it.ddig;
  b->dscale = it.dscale;
  b->mscale = it.mscale;
  b->PK = it.out;
  b->nk = p.kdim / BK;
  b->nchunk = (b->nk + kchunk - 1) / kchunk;
  b->ncb = p.ncols / BM;
  b->neb = round_up(it.nrows, BN) / BN;
  b->nel = it.nrows;
  b->ncols = it.ncols_real;
  // raster groups whose M digit strips take about 48 MB of L2 (or the
  // tuned width)
  const double strip = (double)b->nk * D * A_TILE;
  const int grp = it.grp > 0 ? it.grp : (int)(48.0 * 1024 * 1024 / strip);
  b->grp = grp < 1 ? 1 : (grp > b->ncb ? b->ncb : grp);
  // V = sum over runs and levels of L_s 2^(R(S-s) - t) stays below 2^62
  const double vmax = log2((double)b->nchunk) + 24.0 + R * (D - 1) - log2(1.0 - ldexp(1.0, -R));
  int t = (int)ceil(vmax - 62.0);
  if (t < 0) t = 0;
  b->shift0 = R * (S - 2) - t;
  b->scale_shift = R * S - t;
}

int ozaki_pairs(const OzakiPlan& p) {
  int n = 0;
  for (int i = 1; i <= p.digits; ++i)
    for (int j = 1; j <= p.digits; ++j) n += (i + j <= p.digits + 1) ? 1 : 0;
  return n;
}

int ozaki_kchunk(const OzakiPlan& p) {
  GemmParams* G = new GemmParams;
  build_params(p, G);
  const int k = G->kchunk;
  delete G;
  return k;
}

int launch_ozaki_gemm_group(const OzakiGemmItem* items, int nitems, int* d_flag,
                            cudaStream_t st, int fault) {
  std::vector<int> order;
  for (int k = 0; k < nitems; ++k)
    if (items[k].nrows > 0) order.push_back(k);
  if (order.empty()) return 0;
  for (int k : order)
    if (items[k].plan->radix != items[order[0]].plan->radix ||
        items[k].plan->digits != items[order[0]].plan->digits)
      return -1;
  int dev = 0, num_sms = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return -1;
  // the longest tiles (most k-blocks) first, so the persistent CTAs end together
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return items[a].plan->kdim > items[b].plan->kdim;
  });
  std::vector<GemmParams> groups;  // one launch per MAXBINS bins
  GemmParams* G = new GemmParams;
  build_params(*items[order[0]].plan, G);
  // as many ring stages as fit next to the static shared memory (barriers),
  // or the tuned depth
  int nst = (optin - 1024 - 1024) / STAGE_BYTES;
  const int tuned = tune_nstage();
  if (tuned > 0 && tuned < nst) nst = tuned < KGROUP + 1 ? KGROUP + 1 : tuned;
  G->nstage = nst > MAXSTAGE ? MAXSTAGE : nst;
  if (G->nstage < KGROUP + 1) { delete G; return -1; }
  G->fault = fault;
  // bounded waits: about a second or more at the normal limit; a fault test
  // runs out quickly
  G->wait_limit = fault ? (1L << 14) : TC_WAIT_LIMIT;
  const size_t smem = (size_t)G->nstage * STAGE_BYTES + 1024;
  if (raise_smem_limit((const void*)k_ozaki_gemm, smem) != cudaSuccess) { delete G; return -1; }
  int rc = 0;
  for (size_t k0 = 0; k0 < order.size() && rc == 0; k0 += MAXBINS) {
    const size_t k1 = std::min(order.size(), k0 + (size_t)MAXBINS);
    G->nbins = (int)(k1 - k0);
    int tiles = 0;
    for (size_t k = k0; k < k1; ++k) {
      GemmBin& b = G->bin[k - k0];
      build_bin(items[order[k]], G->kchunk, &b);
      b.tile0 = tiles;
      tiles += b.ncb * b.neb;
    }
    G->ntiles = tiles;
    const int grid = tiles < num_sms ? tiles : num_sms;
    k_ozaki_gemm<<<grid, NTHREADS, smem, st>>>(*G, d_flag);
    if (cudaPeekAtLastError() != cudaSuccess) rc = -1;
  }
  delete G;
  return rc;
}

int launch_ozaki_gemm(const OzakiPlan& p, int nel, int n, const uint16_t* d_ddig,
                      const double* d_dscale, const uint16_t* d_mdig, const double* d_mscale,
                      double* d_PK, int* d_flag, cudaStream_t st, int fault, int grp) {
  OzakiGemmItem it{&p, nel, n * (n + 1) / 2, d_ddig, d_dscale, d_mdig, d_mscale, d_PK, grp};
  return launch_ozaki_gemm_group(&it, 1, d_flag, st, fault);
}

int launch_ozaki_gemm_dense(const OzakiPlan& p, int nrows, const uint16_t* d_ddig,
                            const double* d_dscale, const uint16_t* d_mdig, const double* d_mscale,
                            double* d_out, int* d_flag, cudaStream_t st) {
  OzakiGemmItem it{&p, nrows, p.nreal, d_ddig, d_dscale, d_mdig, d_mscale, d_out};
  return launch_ozaki_gemm_group(&it, 1, d_flag, st, 0);
}

}  // namespace hp3dg

// ---------------------------------------------------------------------------
// C ABI: the contraction on caller-supplied operands
// ---------------------------------------------------------------------------
extern "C" int hp3dg_mixed_contract(int32_t nrows, int32_t K, int32_t ncols, const double* D,
                                    const double* M, double* out, int32_t radix, int32_t digits,
                                    void* stream) {
  using namespace hp3dg;
  if (nrows < 0 || K <= 0 || ncols <= 0 || (nrows > 0 && (!D || !M || !out)))
    return HP3DG_ERR_ARG;
  if (nrows == 0) return HP3DG_OK;
  OzakiPlan p;
  if (ozaki_plan_dense(K, ncols, radix > 0 ? radix : 7, digits > 0 ? digits : 7, &p))
    return HP3DG_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  uint8_t *mdig = nullptr, *ddig = nullptr;
  double *mscale = nullptr, *dscale = nullptr;
  int* flag = nullptr;
  int rc = HP3DG_OK;
  if (cudaMalloc(&mdig, ozaki_m_bytes(p)) != cudaSuccess ||
      cudaMalloc(&ddig, ozaki_d_bytes(p, nrows)) != cudaSuccess ||
      cudaMalloc(&mscale, (size_t)p.ncols * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&dscale, (size_t)(nrows + 128) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&flag, sizeof(int)) != cudaSuccess) {
    rc = HP3DG_ERR_ALLOC;
  } else if (cudaMemsetAsync(flag, 0x7f, sizeof(int), st) != cudaSuccess ||
             launch_ozaki_build_m_dense(p, M, (uint16_t*)mdig, mscale, st) ||
             launch_ozaki_slice_d_dense(p, nrows, D, (uint16_t*)ddig, dscale, st) ||
             launch_ozaki_gemm_dense(p, nrows, (const uint16_t*)ddig, dscale,
                                     (const uint16_t*)mdig, mscale, out, flag, st)) {
    rc = HP3DG_ERR_CUDA;
  } else {
    int h = 0;
    if (cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = HP3DG_ERR_CUDA;
    else if (h != 0x7f7f7f7f)
      rc = HP3DG_ERR_TIMEOUT;
  }
  if (rc != HP3DG_OK) cudaStreamSynchronize(st);
  cudaFree(mdig);
  cudaFree(ddig);
  cudaFree(mscale);
  cudaFree(dscale);
  cudaFree(flag);
  return rc;
}

