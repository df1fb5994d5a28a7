// k_cond_tc.cu -- static condensation of the mixed pass with every
// triangular solve and product on tcgen05 tensor cores.
//
// stc_fwd (modules/stc.F90:338-416 Hermitian branch, 443-509) per element:
//   K_bb = L L^T,  Y = L^-1 K_bi,  S = K_ii - Y^T Y,  ASchur = L^-T Y,
//   BSchur = K_bb^-1 b_b,  condensed load b_i - K_ib BSchur.
// The FP64 kernel k_cond_chol gathers K_bb through the element's dof map,
// factors it, forms the explicit inverse Li = L^-1 (nb^3/6 FMAs, against
// 2 nb^2 ni for the two triangular solves it replaces) and BSchur; k_cond_kbi
// gathers K_bi per interface column and forms the condensed load.  Both write
// their operands as balanced BF16 digits (integer arithmetic from the
// mantissa bits; one power-of-two scale per row):
//   K_bi^T (rows = interface dof c, K = bubble dof), Li and Li^T (rows = bubble
//   dof, K = bubble dof), each as UMMA canonical K-major tiles.
// The fused kernel k_cond_tc then works on one element at a time with its
// digits in shared memory:
//   1. Y^T = K_bi^T Li^T       (rows c, columns = bubble dof)  -> Y's digits are
//      formed in the epilogue straight from the exact level sums (integer
//      arithmetic) and written over the K_bi^T digits in shared memory;
//   2. W = Y^T Y               (128-row x <= 64-column chunks) -> packed upper W;
//   3. ASchur^T = Y^T Li       (B = Li^T digits, loaded over Li's)
//                              -> ASchur (nb x ni, column-major) in FP64.
// Every product accumulates its digit-pair levels s = i + j in separate FP32
// TMEM accumulators; with K = nb <= 64 and radix-8 digits (6 per operand,
// 48 bits) the level sums are integers below 2^23 (exact); they are
// recombined as two exact 64-bit partial sums.
#include "hp3dg_internal.cuh"
#include "hp3dg_kernels.h"
#include "hp3dg_tc.cuh"

#include <string.h>

#include <algorithm>
#include <vector>

namespace hp3dg {

namespace {
constexpr int CT_NC = 64;          // TMEM columns per level slot
constexpr int CT_MAXDIG = 7;
constexpr int CT_MAXCHUNK = 8;
constexpr int CT_MAXPAIR = 28;
constexpr int CT_THREADS = 320;  // loader, MMA, 8 epilogue warps (2 per TMEM lane quarter)
constexpr int CT_EPI = 256;
constexpr uint32_t CT_TMEM_COLS = 512;

struct CondTcParams {
  int digits, radix;
  int nr, nbr, nkb;        // rows of the K_bi^T / Y tiles, rows of the Li tiles, k-blocks
  int nif, nbf;
  int nel;
  uint32_t bytes_a, bytes_b;  // per element: K_bi^T digits, Li (and Li^T) digits
  int nchunk;
  int ch_m0[CT_MAXCHUNK], ch_c0[CT_MAXCHUNK], ch_nc[CT_MAXCHUNK], ch_rmin[CT_MAXCHUNK];
  int npair;
  int8_t pi[CT_MAXPAIR], pj[CT_MAXPAIR], pfirst[CT_MAXPAIR];
};

__host__ __device__ constexpr uint32_t idesc_m128(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

}  // namespace

// ---------------------------------------------------------------------------
// FP64 part: gather, Cholesky, explicit inverse, load vectors, digit operands
// ---------------------------------------------------------------------------
struct CondTcOut {
  uint8_t *kbd, *lid, *ltd;     // digits: K_bi^T, Li, Li^T
  int *ekb, *eli, *elt;         // row exponents
  double* bi;                   // condensed load (nif per element)
  int nr, nbr, nkb, digits, radix;
  uint32_t bytes_a, bytes_b;
};

// Per element, one warp: gather K_bb (lower triangle, packed) and b_b through
// the dof map; right-looking Cholesky K_bb = L L^T and the inverse Li = L^-1
// in place (right-looking forward substitution, one column of L kept in a
// scratch vector); BSchur = Li^T (Li b_b); the digits of Li and Li^T.
// Warp-synchronous: no block barrier.
constexpr int CH_WARPS = 4;
__device__ __forceinline__ int tri(int i, int j) { return i * (i + 1) / 2 + j; }

__device__ __forceinline__ void cond_chol_body(
    int bx, int nfull, int nif, int nbf, const int* __restrict__ elist, const int* __restrict__ ni_e,
    const int* __restrict__ nb_e, const double* __restrict__ PK, const double* __restrict__ b0,
    const uint32_t* __restrict__ perm, const int64_t* __restrict__ bub_off,
    double* __restrict__ bschur, CondTcOut o, int nel, int* __restrict__ bad_spd) {
  extern __shared__ double sm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = bx * CH_WARPS + w;
  if (j >= nel) return;
  const int e = elist[j];
  const int ni = ni_e[e], nb = nb_e[e];
  const double* PKj = PK + (size_t)j * ((size_t)nfull * (nfull + 1) / 2);
  const uint32_t* pm = perm + (size_t)j * nfull;
  const double* bj = b0 + (size_t)j * nfull;
  const size_t per = (size_t)nbf * (nbf + 1) / 2 + 3 * (size_t)nbf;
  double* A = sm + (size_t)w * per;        // packed lower triangle
  double* col = A + (size_t)nbf * (nbf + 1) / 2;
  double* bb = col + nbf;
  double* yv = bb + nbf;
  for (int idx = lane; idx < nb * (nb + 1) / 2; idx += 32) {
    int i = (int)((sqrtf(8.0f * idx + 1.0f) - 1.0f) * 0.5f);
    while (tri(i + 1, 0) <= idx) ++i;
    while (tri(i, 0) > idx) --i;
    const int c = idx - tri(i, 0);
    A[idx] = pk_get(PKj, pm, ni + i, ni + c, nif, nbf);
  }
  for (int r = lane; r < nb; r += 32) {
    uint32_t m = pm[ni + r];
    double v = bj[m & 0x7fffffffu];
    bb[r] = (m & 0x80000000u) ? -v : v;
  }
  __syncwarp();
  bool fail = false;
  // Cholesky, right-looking.  The trailing update of step k runs over the
  // packed triangle of the m = nb - k - 1 remaining rows as one flat index,
  // so every lane of each FP64 instruction has work (GB300 issues FP64 at
  // about 2 per clock per SM: idle lanes cost the same as busy ones).
  for (int k = 0; k < nb; ++k) {
    double d = A[tri(k, k)];
    if (!(d > 0.0)) { fail = true; d = 1.0; }
    d = sqrt(d);
    const double rk = 1.0 / d;
    __syncwarp();
    if (lane == 0) A[tri(k, k)] = d;
    for (int i = k + 1 + lane; i < nb; i += 32) A[tri(i, k)] *= rk;
    __syncwarp();
    const int m = nb - k - 1;
    for (int x = lane; x < m * (m + 1) / 2; x += 32) {
      int ip = (int)((sqrtf(8.0f * x + 1.0f) - 1.0f) * 0.5f);
      while (tri(ip + 1, 0) <= x) ++ip;
      while (tri(ip, 0) > x) --ip;
      const int i = k + 1 + ip, jj = k + 1 + (x - tri(ip, 0));
      A[tri(i, jj)] = fma(-A[tri(i, k)], A[tri(jj, k)], A[tri(i, jj)]);
    }
    __syncwarp();
  }
  if (fail && lane == 0) atomicMin(bad_spd, e);
  // inverse in place, right-looking forward substitution L Li = I: at step k
  // row k of Li is final once scaled by 1 / L(k,k); the rows i > k then take
  // -L(i,k) Li(k, 0..k) (column k of L kept in col[] first), again one flat
  // index over the (nb - k - 1) x (k + 1) block
  for (int k = 0; k < nb; ++k) {
    for (int i = k + 1 + lane; i < nb; i += 32) col[i] = A[tri(i, k)];
    const double dk = 1.0 / A[tri(k, k)];
    __syncwarp();
    if (lane == 0) A[tri(k, k)] = dk;
    for (int jj = lane; jj < k; jj += 32) A[tri(k, jj)] *= dk;
    __syncwarp();
    const int w = k + 1, m = nb - k - 1;
    for (int x = lane; x < m * w; x += 32) {
      const int ip = x / w, jj = x - ip * w, i = k + 1 + ip;
      const double lik = col[i];
      A[tri(i, jj)] = jj == k ? -lik * A[tri(k, k)] : fma(-lik, A[tri(k, jj)], A[tri(i, jj)]);
    }
    __syncwarp();
  }
  // y = Li b_b, BSchur = Li^T y
  for (int r = lane; r < nb; r += 32) {
    double s = 0.0;
    for (int k = 0; k <= r; ++k) s += A[tri(r, k)] * bb[k];
    yv[r] = s;
  }
  __syncwarp();
  for (int r = lane; r < nb; r += 32) {
    double s = 0.0;
    for (int k = r; k < nb; ++k) s += A[tri(k, r)] * yv[k];
    bschur[bub_off[e] + r] = s;
  }
  // row exponents and digits of Li (row r: A[r][0..r]) and Li^T (row r: A[r..][r])
  const int fb = o.radix * o.digits;
  uint8_t* bl = o.lid + (size_t)j * o.bytes_b;
  uint8_t* bt = o.ltd + (size_t)j * o.bytes_b;
  const size_t dstride = (size_t)o.nkb * o.nbr * 32;
  for (int r = lane; r < o.nbr; r += 32) {
    unsigned long long m1 = 0, m2 = 0;
    if (r < nb) {
      for (int k = 0; k <= r; ++k) { unsigned long long b = mag_bits(A[tri(r, k)]); m1 = b > m1 ? b : m1; }
      for (int k = r; k < nb; ++k) { unsigned long long b = mag_bits(A[tri(k, r)]); m2 = b > m2 ? b : m2; }
    }
    const int e1 = row_exponent(m1), e2 = row_exponent(m2);
    o.eli[(size_t)j * o.nbr + r] = e1;
    o.elt[(size_t)j * o.nbr + r] = e2;
    for (int g = 0; g < o.nkb * 2; ++g) {
      long long X[8], Z[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int k = g * 8 + t;
        X[t] = (r < nb && k <= r) ? fixed_of(A[tri(r, k)], e1, fb) : 0;
        Z[t] = (r < nb && k >= r && k < nb) ? fixed_of(A[tri(k, r)], e2, fb) : 0;
      }
      store_digits8(X, o.radix, o.digits, bl + tile_off(r, g, o.nbr), dstride);
      store_digits8(Z, o.radix, o.digits, bt + tile_off(r, g, o.nbr), dstride);
    }
  }
}


__global__ void __launch_bounds__(CH_WARPS * 32) k_cond_chol(
    int nfull, int nif, int nbf, const int* __restrict__ elist, const int* __restrict__ ni_e,
    const int* __restrict__ nb_e, const double* __restrict__ PK, const double* __restrict__ b0,
    const uint32_t* __restrict__ perm, const int64_t* __restrict__ bub_off,
    double* __restrict__ bschur, CondTcOut o, int nel, int* __restrict__ bad_spd) {
  cond_chol_body(blockIdx.x, nfull, nif, nbf, elist, ni_e, nb_e, PK, b0, perm, bub_off, bschur, o,
                 nel, bad_spd);
}

size_t cond_chol_smem(int nbf) {
  return (size_t)CH_WARPS * ((size_t)nbf * (nbf + 1) / 2 + 3 * (size_t)nbf) * sizeof(double);
}

// Per (element, 128 interface columns): K_bi column c gathered through the
// dof map (twice: the row exponent first, then the digits), the condensed
// load b_i - K_ib BSchur, and the digits of K_bi^T (rows = interface dof).
__device__ __forceinline__ void cond_kbi_body(
    int bx, int by, int nfull, int nif, int nbf, const int* __restrict__ elist, const int* __restrict__ ni_e,
    const int* __restrict__ nb_e, const double* __restrict__ PK, const double* __restrict__ b0,
    const uint32_t* __restrict__ perm, const int64_t* __restrict__ bub_off,
    const double* __restrict__ bschur, CondTcOut o) {
  const int j = bx, e = elist[j];
  const int c = by * 128 + threadIdx.x;
  if (c >= o.nr) return;
  const int ni = ni_e[e], nb = nb_e[e];
  const double* PKj = PK + (size_t)j * ((size_t)nfull * (nfull + 1) / 2);
  const uint32_t* pm = perm + (size_t)j * nfull;
  const double* bs = bschur + bub_off[e];
  const bool col = c < ni;
  const uint32_t mc = col ? pm[c] : 0u;
  const int rc = (int)(mc & 0x7fffffffu);
  // K_bi[r][c] from the packed bin matrix (BI block: interface rc < bubble rb)
  auto kbi = [&](int r) -> double {
    const uint32_t mr = pm[ni + r];
    const int rb = (int)(mr & 0x7fffffffu);
    const double v = PKj[pk_index(rc, rb, nif, nbf)];
    return ((mc ^ mr) & 0x80000000u) ? -v : v;
  };
  unsigned long long mb = 0;
  if (col) {
    double s = 0.0;
    for (int r = 0; r < nb; ++r) {
      const double v = kbi(r);
      const unsigned long long b = mag_bits(v);
      mb = b > mb ? b : mb;
      s += v * bs[r];
    }
    const double* bj = b0 + (size_t)j * nfull;
    double bv = bj[rc];
    if (mc & 0x80000000u) bv = -bv;
    o.bi[(size_t)j * nif + c] = bv - s;
  }
  const int ec = row_exponent(mb);
  o.ekb[(size_t)j * o.nr + c] = ec;
  const int fb = o.radix * o.digits;
  uint8_t* base = o.kbd + (size_t)j * o.bytes_a;
  const size_t dstride = (size_t)o.nkb * o.nr * 32;
  for (int g = 0; g < o.nkb * 2; ++g) {
    long long X[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int r = g * 8 + t;
      X[t] = (col && r < nb) ? fixed_of(kbi(r), ec, fb) : 0;
    }
    store_digits8(X, o.radix, o.digits, base + tile_off(c, g, o.nr), dstride);
  }
}


__global__ void __launch_bounds__(128) k_cond_kbi(
    int nfull, int nif, int nbf, const int* __restrict__ elist, const int* __restrict__ ni_e,
    const int* __restrict__ nb_e, const double* __restrict__ PK, const double* __restrict__ b0,
    const uint32_t* __restrict__ perm, const int64_t* __restrict__ bub_off,
    const double* __restrict__ bschur, CondTcOut o) {
  cond_kbi_body(blockIdx.x, blockIdx.y, nfull, nif, nbf, elist, ni_e, nb_e, PK, b0, perm, bub_off,
                bschur, o);
}

// ---------------------------------------------------------------------------
// tensor-core part
// ---------------------------------------------------------------------------
// Level sums of 8 consecutive TMEM columns (slot k at column k*CT_NC + col)
// folded into the two exact partial sums: hi over levels 2..kh+1, lo over the
// rest.  One level is loaded at a time to keep the register footprint small.
__device__ __forceinline__ void load_levels8(uint32_t taddr, int D, int R, long long* hi,
                                             long long* lo) {
  const int kh = D < 4 ? D : 4;
#pragma unroll
  for (int q = 0; q < 8; ++q) { hi[q] = 0; lo[q] = 0; }
#pragma unroll
  for (int k = 0; k < CT_MAXDIG; ++k) {
    if (k >= D) break;
    uint32_t v[8];
    tmem_ld8_nowait(taddr + (uint32_t)(k * CT_NC), v);
    tmem_wait();
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const long long l = (long long)__float2int_rn(__uint_as_float(v[q]));
      if (k < kh) hi[q] = hi[q] * (1LL << R) + l;
      else lo[q] = lo[q] * (1LL << R) + l;
    }
  }
}

// upper bound on the bit length of |hi 2^s + lo| (s = R(D-kh))
__device__ __forceinline__ int bitlen_bound(long long hi, long long lo, int s) {
  if (hi != 0) {
    unsigned long long a = (unsigned long long)(hi < 0 ? -hi : hi);
    return 64 - __clzll((long long)a) + s + 1;
  }
  unsigned long long b = (unsigned long long)(lo < 0 ? -lo : lo);
  return b ? 64 - __clzll((long long)b) + 1 : 0;
}
// round((hi 2^s + lo) 2^-sh) as a 64-bit integer.  The caller guarantees
// |result| < 2^(radix*digits) <= 2^49, so every left shift below is small;
// right shifts beyond the value's length give 0.
__device__ __forceinline__ long long shift_round(long long hi, long long lo, int s, int sh) {
  if (hi == 0 && lo == 0) return 0;
  if (sh <= 0) {
    const int ls = -sh;
    const long long a = hi ? hi * (1LL << (s + ls)) : 0;
    const long long b = lo ? lo * (1LL << ls) : 0;
    return a + b;
  }
  if (sh < s) {
    const long long lr = (lo + (1LL << (sh - 1))) >> sh;
    return (hi ? hi * (1LL << (s - sh)) : 0) + lr;
  }
  // sh >= s: fold lo into hi at the 2^s scale (drops < one unit), then shift
  const long long t = hi + ((lo + (1LL << (s - 1))) >> s);
  const int r = sh - s;
  if (r == 0) return t;
  if (r >= 62) return 0;
  return (t + (1LL << (r - 1))) >> r;
}

__global__ void __launch_bounds__(CT_THREADS, 1)
    k_cond_tc(const uint8_t* __restrict__ kbd, const uint8_t* __restrict__ lid,
              const uint8_t* __restrict__ ltd, const int* __restrict__ ekb,
              const int* __restrict__ eli, const int* __restrict__ elt, const CondTcParams P,
              const int* __restrict__ elist, const int* __restrict__ ni_e,
              const int* __restrict__ nb_e, const int64_t* __restrict__ schur_off,
              double* __restrict__ Wbuf, double* __restrict__ aschur, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smraw[];
  uint8_t* regA = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);  // K_bi^T, then Y
  uint8_t* regB = regA + P.bytes_a;                                            // Li, then Li^T
  __shared__ __align__(8) uint64_t ldA_bar, ldT_bar, bfree_bar, sfree_bar, acc_full, acc_empty,
      ydone_bar, p1_bar;
  __shared__ int pmax[2][256];  // per half of the columns: partial row exponents of Y
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_;
  __shared__ int ey[256];  // row exponents of Y
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // the digit layout is fixed at compile time (constant shifts, unrolled levels)
  constexpr int D = COND_TC_DIGITS, R = COND_TC_RADIX;
  const uint32_t dstrA = (uint32_t)P.nkb * P.nr * 32, kstrA = (uint32_t)P.nr * 32;
  const uint32_t dstrB = (uint32_t)P.nkb * P.nbr * 32, kstrB = (uint32_t)P.nbr * 32;

  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&ldA_bar), 1);
    mbar_init(smem_u32(&ldT_bar), 1);
    mbar_init(smem_u32(&bfree_bar), 1);
    mbar_init(smem_u32(&sfree_bar), 1);
    mbar_init(smem_u32(&acc_full), 1);
    mbar_init(smem_u32(&acc_empty), CT_EPI);
    mbar_init(smem_u32(&ydone_bar), CT_EPI);
    mbar_init(smem_u32(&p1_bar), CT_EPI);
    abort_ = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(CT_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base;
  const int ntile = P.nr > 128 ? 2 : 1;

  if (warp == 0) {
    // ---------------- loader ----------------
    if (lane == 0) {
      uint32_t sph = 0, bph = 0;
      for (int j = blockIdx.x; j < P.nel && !abort_; j += gridDim.x) {
        if (!mbar_wait(smem_u32(&sfree_bar), sph ^ 1, &abort_)) { abort_ = 1; atomicExch(err, 21); break; }
        sph ^= 1;
        const uint32_t la = smem_u32(&ldA_bar);
        mbar_expect_tx(la, P.bytes_a + P.bytes_b);
        bulk_load(smem_u32(regA), kbd + (size_t)j * P.bytes_a, P.bytes_a, la);
        bulk_load(smem_u32(regB), lid + (size_t)j * P.bytes_b, P.bytes_b, la);
        // Li^T over Li once the Y products have read Li
        if (!mbar_wait(smem_u32(&bfree_bar), bph, &abort_)) { abort_ = 1; atomicExch(err, 22); break; }
        bph ^= 1;
        const uint32_t lt = smem_u32(&ldT_bar);
        mbar_expect_tx(lt, P.bytes_b);
        bulk_load(smem_u32(regB), ltd + (size_t)j * P.bytes_b, P.bytes_b, lt);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      uint32_t aph = 0, tph = 0, eph = 0, yph = 0;
      const uint32_t A0 = smem_u32(regA), B0 = smem_u32(regB);
      const uint32_t idB = idesc_m128(P.nbr);
      // one 128-row product with B = the Li / Li^T tiles (N = nbr): all pairs
      // descriptors are affine in the address: one base per region, byte
      // offsets added in units of 16 bytes
      const uint64_t dA0 = sdesc_kmajor(A0), dB0 = sdesc_kmajor(B0);
      auto prod_b = [&](int m0) {
        const uint64_t a0 = dA0 + (uint64_t)((m0 >> 3) * 256 >> 4);
        for (int p = 0; p < P.npair; ++p) {
          const uint32_t dt = tbase + (uint32_t)(P.pi[p] + P.pj[p] - 2) * CT_NC;
          const uint64_t ap = a0 + (uint64_t)((P.pi[p] - 1) * dstrA >> 4);
          const uint64_t bp = dB0 + (uint64_t)((P.pj[p] - 1) * dstrB >> 4);
          const uint32_t first = P.pfirst[p] ? 0u : 1u;
          for (int kb = 0; kb < P.nkb; ++kb)
            umma_bf16(dt, ap + (uint64_t)(kb * kstrA >> 4), bp + (uint64_t)(kb * kstrB >> 4), idB,
                      kb > 0 ? 1u : first);
        }
      };
      for (int j = blockIdx.x; j < P.nel && !abort_; j += gridDim.x) {
        if (!mbar_wait(smem_u32(&ldA_bar), aph, &abort_)) { abort_ = 1; atomicExch(err, 23); break; }
        aph ^= 1;
        tc_fence_after();
        // 1. Y^T = K_bi^T Li^T: the upper tile (rows nr-128..) first, so that its
        //    epilogue can overwrite rows >= 128 while the lower tile still reads
        //    rows < 128
        for (int t = ntile - 1; t >= 0 && !abort_; --t) {
          if (!mbar_wait(smem_u32(&acc_empty), eph ^ 1, &abort_)) { abort_ = 1; atomicExch(err, 24); break; }
          eph ^= 1;
          tc_fence_after();
          prod_b(t == 1 ? P.nr - 128 : 0);
          umma_commit(smem_u32(&acc_full));
        }
        umma_commit(smem_u32(&bfree_bar));  // Li is free once the Y products retire
        // 2. W = Y^T Y once the epilogue has written Y's digits
        if (!mbar_wait(smem_u32(&ydone_bar), yph, &abort_)) { abort_ = 1; atomicExch(err, 25); break; }
        yph ^= 1;
        tc_fence_after();
        for (int ch = 0; ch < P.nchunk && !abort_; ++ch) {
          if (!mbar_wait(smem_u32(&acc_empty), eph ^ 1, &abort_)) { abort_ = 1; atomicExch(err, 26); break; }
          eph ^= 1;
          tc_fence_after();
          const uint32_t idesc = idesc_m128(P.ch_nc[ch]);
          const uint64_t a0 = dA0 + (uint64_t)((P.ch_m0[ch] >> 3) * 256 >> 4);
          const uint64_t b0 = dA0 + (uint64_t)((P.ch_c0[ch] >> 3) * 256 >> 4);
          for (int p = 0; p < P.npair; ++p) {
            const uint32_t dt = tbase + (uint32_t)(P.pi[p] + P.pj[p] - 2) * CT_NC;
            const uint64_t ap = a0 + (uint64_t)((P.pi[p] - 1) * dstrA >> 4);
            const uint64_t bp = b0 + (uint64_t)((P.pj[p] - 1) * dstrA >> 4);
            const uint32_t first = P.pfirst[p] ? 0u : 1u;
            for (int kb = 0; kb < P.nkb; ++kb)
              umma_bf16(dt, ap + (uint64_t)(kb * kstrA >> 4), bp + (uint64_t)(kb * kstrA >> 4), idesc,
                        kb > 0 ? 1u : first);
          }
          umma_commit(smem_u32(&acc_full));
        }
        // 3. ASchur^T = Y^T Li with B = the Li^T tiles
        if (!mbar_wait(smem_u32(&ldT_bar), tph, &abort_)) { abort_ = 1; atomicExch(err, 27); break; }
        tph ^= 1;
        tc_fence_after();
        for (int t = ntile - 1; t >= 0 && !abort_; --t) {
          if (!mbar_wait(smem_u32(&acc_empty), eph ^ 1, &abort_)) { abort_ = 1; atomicExch(err, 28); break; }
          eph ^= 1;
          tc_fence_after();
          prod_b(t == 1 ? P.nr - 128 : 0);
          umma_commit(smem_u32(&acc_full));
        }
        umma_commit(smem_u32(&sfree_bar));  // shared memory free for the next element
      }
    }
  } else {
    // ---------------- epilogue (warps 2..9: TMEM lane quarter warp%4, half h of
    // the 8-column groups) ----------------
    const int quarter = warp & 3, h = (warp - 2) >> 2;
    const uint32_t tlane = tbase + ((uint32_t)(quarter * 32) << 16);
    const int kh = D < 4 ? D : 4, s = R * (D - kh), fb = R * D;
    uint32_t fph = 0, yph = 0, p1ph = 0;
    auto wait_full = [&]() -> bool {
      if (!mbar_wait(smem_u32(&acc_full), fph, &abort_)) { abort_ = 1; atomicExch(err, 29); return false; }
      fph ^= 1;
      tc_fence_after();
      return true;
    };
    auto release = [&]() {
      tc_fence_before();
      mbar_arrive(smem_u32(&acc_empty));
    };
    for (int j = blockIdx.x; j < P.nel && !abort_; j += gridDim.x) {
      const int e = elist[j];
      const int ni = ni_e[e], nb = nb_e[e];
      const int* ekbj = ekb + (size_t)j * P.nr;
      const int* eL = eli + (size_t)j * P.nbr;
      // ---- 1. Y^T tiles -> Y digits in shared memory (over K_bi^T) ----
      for (int t = ntile - 1; t >= 0; --t) {
        if (!wait_full()) break;
        const int m0 = t == 1 ? P.nr - 128 : 0;
        const int c = m0 + quarter * 32 + lane;
        const bool mine = (t == 1) ? (c >= 128) : true;  // rows >= 128 come from the upper tile
        const int q0 = mine && c < ni ? ekbj[c] - R * (D + 1) : 0;
        // pass 1: exponent of the row (upper bound of log2 |Y[:, c]|); each half
        // scans its column groups, the halves meet on p1_bar
        int erow = -100000;
        for (int g = h; g < P.nbr / 8; g += 2) {
          long long hi[8], lo[8];
          load_levels8(tlane + (uint32_t)(g * 8), D, R, hi, lo);
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int bl = bitlen_bound(hi[q], lo[q], s);
            if (bl) erow = max(erow, bl + q0 + eL[g * 8 + q]);
          }
        }
        pmax[h][quarter * 32 + lane] = erow;
        mbar_arrive(smem_u32(&p1_bar));
        if (!mbar_wait(smem_u32(&p1_bar), p1ph, &abort_)) { abort_ = 1; atomicExch(err, 31); }
        p1ph ^= 1;
        erow = max(pmax[0][quarter * 32 + lane], pmax[1][quarter * 32 + lane]);
        if (!(mine && c < ni) || erow == -100000) erow = 0;
        // pass 2: Y[r, c] 2^(fb - erow) as fixed point, balanced digits
        for (int g = h; g < P.nkb * 2; g += 2) {
          long long hi[8], lo[8];
          load_levels8(tlane + (uint32_t)(g * 8), D, R, hi, lo);
          if (!mine) continue;
          long long X[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int r = g * 8 + q;
            // value = (hi 2^s + lo) 2^(q0 + eL[r]);  X = value 2^(fb - erow)
            const int sh = erow - fb - q0 - eL[r];
            X[q] = (c < ni && r < nb) ? shift_round(hi[q], lo[q], s, sh) : 0;
          }
          store_digits8(X, R, D, regA + tile_off(c, g, P.nr), (size_t)dstrA);
        }
        if (mine && h == 0) ey[c] = erow;
        if (t == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        release();
      }
      mbar_arrive(smem_u32(&ydone_bar));
      // every row exponent of Y is written once all 128 threads have arrived
      if (!mbar_wait(smem_u32(&ydone_bar), yph, &abort_)) { abort_ = 1; atomicExch(err, 30); }
      yph ^= 1;
      // ---- 2. W chunks ----
      double* W = Wbuf + (size_t)j * ((size_t)P.nif * (P.nif + 1) / 2);
      for (int ch = 0; ch < P.nchunk; ++ch) {
        if (!wait_full()) break;
        const int a = P.ch_m0[ch] + quarter * 32 + lane;
        const bool arow = a >= P.ch_rmin[ch] && a < ni;
        const int ea = arow ? ey[a] : 0;
        for (int g = h; g < P.ch_nc[ch] / 8; g += 2) {
          long long hi[8], lo[8];
          load_levels8(tlane + (uint32_t)(g * 8), D, R, hi, lo);
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int b = P.ch_c0[ch] + g * 8 + q;
            if (!(arow && b < ni && a <= b)) continue;
            const int sx = ea + ey[b] - R * (D + 1);
            const double sc = __longlong_as_double((long long)(1023 + sx) << 52);
            const double sch = __longlong_as_double((long long)(1023 + sx + s) << 52);
            W[(int64_t)b * (b + 1) / 2 + a] = fma(__ll2double_rn(hi[q]), sch, __ll2double_rn(lo[q]) * sc);
          }
        }
        release();
      }
      // ---- 3. ASchur^T tiles ----
      const int* eT = elt + (size_t)j * P.nbr;
      double* AS = aschur + schur_off[e];
      for (int t = ntile - 1; t >= 0; --t) {
        if (!wait_full()) break;
        const int m0 = t == 1 ? P.nr - 128 : 0;
        const int c = m0 + quarter * 32 + lane;
        const bool mine = ((t == 1) ? (c >= 128) : (ntile == 1 || c < 128)) && c < ni;
        for (int g = h; g < P.nbr / 8; g += 2) {
          long long hi[8], lo[8];
          load_levels8(tlane + (uint32_t)(g * 8), D, R, hi, lo);
          if (!mine) continue;
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int r = g * 8 + q;
            if (r >= nb) continue;
            const int sx = ey[c] + eT[r] - R * (D + 1);
            const double sc = __longlong_as_double((long long)(1023 + sx) << 52);
            const double sch = __longlong_as_double((long long)(1023 + sx + s) << 52);
            AS[(size_t)c * nb + r] = fma(__ll2double_rn(hi[q]), sch, __ll2double_rn(lo[q]) * sc);
          }
        }
        release();
      }
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase),
                 "r"(CT_TMEM_COLS));
  }
}


// ---------------------------------------------------------------------------
// grouped launches: the condensation of many bins (or element chunks) at once
// ---------------------------------------------------------------------------
struct CondSegDev {
  int nfull, nif, nbf, nel;
  const int* elist;
  const double *PK, *b0;
  const uint32_t* perm;
  double* W;          // the Schur scratch W / S, nif(nif+1)/2 per element
  CondTcOut o;        // the digit operands of the segment's elements
  CondTcParams P;     // the fused kernel's tiles, chunks and digit pairs
};

__device__ __forceinline__ int grp_seg(const int* __restrict__ pre, int nseg, int b) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(CH_WARPS * 32) k_cond_chol_grp(
    const CondSegDev* __restrict__ segs, const int* __restrict__ pre, int nseg, int off,
    const int* __restrict__ ni_e, const int* __restrict__ nb_e, const int64_t* __restrict__ bub_off,
    double* __restrict__ bschur, int* __restrict__ bad_spd) {
  const int blk = blockIdx.x + off;
  const int s = grp_seg(pre, nseg, blk);
  const CondSegDev& G = segs[s];
  cond_chol_body(blk - pre[s], G.nfull, G.nif, G.nbf, G.elist, ni_e, nb_e, G.PK, G.b0, G.perm,
                 bub_off, bschur, G.o, G.nel, bad_spd);
}

__global__ void __launch_bounds__(128) k_cond_kbi_grp(
    const CondSegDev* __restrict__ segs, const int* __restrict__ pre, int nseg, int off,
    const int* __restrict__ ni_e, const int* __restrict__ nb_e, const int64_t* __restrict__ bub_off,
    const double* __restrict__ bschur) {
  const int blk = blockIdx.x + off;
  const int s = grp_seg(pre, nseg, blk);
  const CondSegDev& G = segs[s];
  const int nby = (G.o.nr + 127) / 128;
  const int loc = blk - pre[s];
  cond_kbi_body(loc / nby, loc % nby, G.nfull, G.nif, G.nbf, G.elist, ni_e, nb_e, G.PK, G.b0,
                G.perm, bub_off, bschur, G.o);
}

__global__ void __launch_bounds__(CT_THREADS, 1)
    k_cond_tc_grp(const CondSegDev* __restrict__ segs, const int* __restrict__ pre, int nseg,
                  int el0, int el1, const int* __restrict__ ni_e, const int* __restrict__ nb_e,
                  const int64_t* __restrict__ schur_off, double* __restrict__ aschur,
                  int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smraw[];
  uint8_t* regA = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);  // K_bi^T, then Y
  __shared__ __align__(8) uint64_t ldA_bar, ldT_bar, bfree_bar, sfree_bar, acc_full, acc_empty,
      ydone_bar, p1_bar;
  __shared__ int pmax[2][256];  // per half of the columns: partial row exponents of Y
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_;
  __shared__ int ey[256];  // row exponents of Y
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // the digit layout is fixed at compile time (constant shifts, unrolled levels)
  constexpr int D = COND_TC_DIGITS, R = COND_TC_RADIX;

  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&ldA_bar), 1);
    mbar_init(smem_u32(&ldT_bar), 1);
    mbar_init(smem_u32(&bfree_bar), 1);
    mbar_init(smem_u32(&sfree_bar), 1);
    mbar_init(smem_u32(&acc_full), 1);
    mbar_init(smem_u32(&acc_empty), CT_EPI);
    mbar_init(smem_u32(&ydone_bar), CT_EPI);
    mbar_init(smem_u32(&p1_bar), CT_EPI);
    abort_ = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(CT_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base;
  // the segment (bin or chunk) of element J, its parameters, digit buffers and
  // the element's position in it
#define CT_SEGMENT(J)                                                                   \
  const int seg_ = grp_seg(pre, nseg, J);                                               \
  const CondSegDev& G_ = segs[seg_];                                                    \
  const CondTcParams& P = G_.P;                                                         \
  const int j = (J) - pre[seg_];                                                        \
  uint8_t* regB = regA + P.bytes_a; /* Li, then Li^T */                                 \
  const uint32_t dstrA = (uint32_t)P.nkb * P.nr * 32, kstrA = (uint32_t)P.nr * 32;      \
  const uint32_t dstrB = (uint32_t)P.nkb * P.nbr * 32, kstrB = (uint32_t)P.nbr * 32;    \
  const int ntile = P.nr > 128 ? 2 : 1;                                                 \
  (void)dstrB; (void)kstrB; (void)kstrA; (void)ntile; (void)regB

  if (warp == 0) {
    // ---------------- loader ----------------
    if (lane == 0) {
      uint32_t sph = 0, bph = 0;
      for (int J = el0 + blockIdx.x; J < el1 && !abort_; J += gridDim.x) {
        CT_SEGMENT(J);
        if (!mbar_wait(smem_u32(&sfree_bar), sph ^ 1, &abort_)) { abort_ = 1; atomicExch(err, 21); break; }
        sph ^= 1;
        const uint32_t la = smem_u32(&ldA_bar);
        mbar_expect_tx(la, P.bytes_a + P.bytes_b);
        bulk_load(smem_u32(regA), G_.o.kbd + (size_t)j * P.bytes_a, P.bytes_a, la);
        bulk_load(smem_u32(regB), G_.o.lid + (size_t)j * P.bytes_b, P.bytes_b, la);
        // Li^T over Li once the Y products have read Li
        if (!mbar_wait(smem_u32(&bfree_bar), bph, &abort_)) { abort_ = 1; atomicExch(err, 22); break; }
        bph ^= 1;
        const uint32_t lt = smem_u32(&ldT_bar);
        mbar_expect_tx(lt, P.bytes_b);
        bulk_load(smem_u32(regB), G_.o.ltd + (size_t)j * P.bytes_b, P.bytes_b, lt);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      uint32_t aph = 0, tph = 0, eph = 0, yph = 0;
      const uint32_t A0 = smem_u32(regA);
      const uint64_t dA0 = sdesc_kmajor(A0);
      for (int J = el0 + blockIdx.x; J < el1 && !abort_; J += gridDim.x) {
        CT_SEGMENT(J);
        (void)j;
        const uint32_t B0 = smem_u32(regB);
        const uint32_t idB = idesc_m128(P.nbr);
        // one 128-row product with B = the Li / Li^T tiles (N = nbr): all pairs
        // descriptors are affine in the address: one base per region, byte
        // offsets added in units of 16 bytes
        const uint64_t dB0 = sdesc_kmajor(B0);
        auto prod_b = [&](int m0) {
        const uint64_t a0 = dA0 + (uint64_t)((m0 >> 3) * 256 >> 4);
        for (int p = 0; p < P.npair; ++p) {
          const uint32_t dt = tbase + (uint32_t)(P.pi[p] + P.pj[p] - 2) * CT_NC;
          const uint64_t ap = a0 + (uint64_t)((P.pi[p] - 1) * dstrA >> 4);
          const uint64_t bp = dB0 + (uint64_t)((P.pj[p] - 1) * dstrB >> 4);
          const uint32_t first = P.pfirst[p] ? 0u : 1u;
          for (int kb = 0; kb < P.nkb; ++kb)
            umma_bf16(dt, ap + (uint64_t)(kb * kstrA >> 4), bp + (uint64_t)(kb * kstrB >> 4), idB,
                      kb > 0 ? 1u : first);
        }
      };
        if (!mbar_wait(smem_u32(&ldA_bar), aph, &abort_)) { abort_ = 1; atomicExch(err, 23); break; }
        aph ^= 1;
        tc_fence_after();
        // 1. Y^T = K_bi^T Li^T: the upper tile (rows nr-128..) first, so that its
        //    epilogue can overwrite rows >= 128 while the lower tile still reads
        //    rows < 128
        for (int t = ntile - 1; t >= 0 && !abort_; --t) {
          if (!mbar_wait(smem_u32(&acc_empty), eph ^ 1, &abort_)) { abort_ = 1; atomicExch(err, 24); break; }
          eph ^= 1;
          tc_fence_after();
          prod_b(t == 1 ? P.nr - 128 : 0);
          umma_commit(smem_u32(&acc_full));
        }
        umma_commit(smem_u32(&bfree_bar));  // Li is free once the Y products retire
        // 2. W = Y^T Y once the epilogue has written Y's digits
        if (!mbar_wait(smem_u32(&ydone_bar), yph, &abort_)) { abort_ = 1; atomicExch(err, 25); break; }
        yph ^= 1;
        tc_fence_after();
        for (int ch = 0; ch < P.nchunk && !abort_; ++ch) {
          if (!mbar_wait(smem_u32(&acc_empty), eph ^ 1, &abort_)) { abort_ = 1; atomicExch(err, 26); break; }
          eph ^= 1;
          tc_fence_after();
          const uint32_t idesc = idesc_m128(P.ch_nc[ch]);
          const uint64_t a0 = dA0 + (uint64_t)((P.ch_m0[ch] >> 3) * 256 >> 4);
          const uint64_t b0 = dA0 + (uint64_t)((P.ch_c0[ch] >> 3) * 256 >> 4);
          for (int p = 0; p < P.npair; ++p) {
            const uint32_t dt = tbase + (uint32_t)(P.pi[p] + P.pj[p] - 2) * CT_NC;
            const uint64_t ap = a0 + (uint64_t)((P.pi[p] - 1) * dstrA >> 4);
            const uint64_t bp = b0 + (uint64_t)((P.pj[p] - 1) * dstrA >> 4);
            const uint32_t first = P.pfirst[p] ? 0u : 1u;
            for (int kb = 0; kb < P.nkb; ++kb)
              umma_bf16(dt, ap + (uint64_t)(kb * kstrA >> 4), bp + (uint64_t)(kb * kstrA >> 4), idesc,
                        kb > 0 ? 1u : first);
          }
          umma_commit(smem_u32(&acc_full));
        }
        // 3. ASchur^T = Y^T Li with B = the Li^T tiles
        if (!mbar_wait(smem_u32(&ldT_bar), tph, &abort_)) { abort_ = 1; atomicExch(err, 27); break; }
        tph ^= 1;
        tc_fence_after();
        for (int t = ntile - 1; t >= 0 && !abort_; --t) {
          if (!mbar_wait(smem_u32(&acc_empty), eph ^ 1, &abort_)) { abort_ = 1; atomicExch(err, 28); break; }
          eph ^= 1;
          tc_fence_after();
          prod_b(t == 1 ? P.nr - 128 : 0);
          umma_commit(smem_u32(&acc_full));
        }
        umma_commit(smem_u32(&sfree_bar));  // shared memory free for the next element
      }
    }
  } else {
    // ---------------- epilogue (warps 2..9: TMEM lane quarter warp%4, half h of
    // the 8-column groups) ----------------
    const int quarter = warp & 3, h = (warp - 2) >> 2;
    const uint32_t tlane = tbase + ((uint32_t)(quarter * 32) << 16);
    const int kh = D < 4 ? D : 4, s = R * (D - kh), fb = R * D;
    uint32_t fph = 0, yph = 0, p1ph = 0;
    auto wait_full = [&]() -> bool {
      if (!mbar_wait(smem_u32(&acc_full), fph, &abort_)) { abort_ = 1; atomicExch(err, 29); return false; }
      fph ^= 1;
      tc_fence_after();
      return true;
    };
    auto release = [&]() {
      tc_fence_before();
      mbar_arrive(smem_u32(&acc_empty));
    };
    for (int J = el0 + blockIdx.x; J < el1 && !abort_; J += gridDim.x) {
      CT_SEGMENT(J);
      const int e = G_.elist[j];
      const int ni = ni_e[e], nb = nb_e[e];
      const int* ekbj = G_.o.ekb + (size_t)j * P.nr;
      const int* eL = G_.o.eli + (size_t)j * P.nbr;
      // ---- 1. Y^T tiles -> Y digits in shared memory (over K_bi^T) ----
      for (int t = ntile - 1; t >= 0; --t) {
        if (!wait_full()) break;
        const int m0 = t == 1 ? P.nr - 128 : 0;
        const int c = m0 + quarter * 32 + lane;
        const bool mine = (t == 1) ? (c >= 128) : true;  // rows >= 128 come from the upper tile
        const int q0 = mine && c < ni ? ekbj[c] - R * (D + 1) : 0;
        // pass 1: exponent of the row (upper bound of log2 |Y[:, c]|); each half
        // scans its column groups, the halves meet on p1_bar
        int erow = -100000;
        for (int g = h; g < P.nbr / 8; g += 2) {
          long long hi[8], lo[8];
          load_levels8(tlane + (uint32_t)(g * 8), D, R, hi, lo);
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int bl = bitlen_bound(hi[q], lo[q], s);
            if (bl) erow = max(erow, bl + q0 + eL[g * 8 + q]);
          }
        }
        pmax[h][quarter * 32 + lane] = erow;
        mbar_arrive(smem_u32(&p1_bar));
        if (!mbar_wait(smem_u32(&p1_bar), p1ph, &abort_)) { abort_ = 1; atomicExch(err, 31); }
        p1ph ^= 1;
        erow = max(pmax[0][quarter * 32 + lane], pmax[1][quarter * 32 + lane]);
        if (!(mine && c < ni) || erow == -100000) erow = 0;
        // pass 2: Y[r, c] 2^(fb - erow) as fixed point, balanced digits
        for (int g = h; g < P.nkb * 2; g += 2) {
          long long hi[8], lo[8];
          load_levels8(tlane + (uint32_t)(g * 8), D, R, hi, lo);
          if (!mine) continue;
          long long X[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int r = g * 8 + q;
            // value = (hi 2^s + lo) 2^(q0 + eL[r]);  X = value 2^(fb - erow)
            const int sh = erow - fb - q0 - eL[r];
            X[q] = (c < ni && r < nb) ? shift_round(hi[q], lo[q], s, sh) : 0;
          }
          store_digits8(X, R, D, regA + tile_off(c, g, P.nr), (size_t)dstrA);
        }
        if (mine && h == 0) ey[c] = erow;
        if (t == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        release();
      }
      mbar_arrive(smem_u32(&ydone_bar));
      // every row exponent of Y is written once all 128 threads have arrived
      if (!mbar_wait(smem_u32(&ydone_bar), yph, &abort_)) { abort_ = 1; atomicExch(err, 30); }
      yph ^= 1;
      // ---- 2. W chunks ----
      double* W = G_.W + (size_t)j * ((size_t)P.nif * (P.nif + 1) / 2);
      for (int ch = 0; ch < P.nchunk; ++ch) {
        if (!wait_full()) break;
        const int a = P.ch_m0[ch] + quarter * 32 + lane;
        const bool arow = a >= P.ch_rmin[ch] && a < ni;
        const int ea = arow ? ey[a] : 0;
        for (int g = h; g < P.ch_nc[ch] / 8; g += 2) {
          long long hi[8], lo[8];
          load_levels8(tlane + (uint32_t)(g * 8), D, R, hi, lo);
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int b = P.ch_c0[ch] + g * 8 + q;
            if (!(arow && b < ni && a <= b)) continue;
            const int sx = ea + ey[b] - R * (D + 1);
            const double sc = __longlong_as_double((long long)(1023 + sx) << 52);
            const double sch = __longlong_as_double((long long)(1023 + sx + s) << 52);
            W[(int64_t)b * (b + 1) / 2 + a] = fma(__ll2double_rn(hi[q]), sch, __ll2double_rn(lo[q]) * sc);
          }
        }
        release();
      }
      // ---- 3. ASchur^T tiles ----
      const int* eT = G_.o.elt + (size_t)j * P.nbr;
      double* AS = aschur + schur_off[e];
      for (int t = ntile - 1; t >= 0; --t) {
        if (!wait_full()) break;
        const int m0 = t == 1 ? P.nr - 128 : 0;
        const int c = m0 + quarter * 32 + lane;
        const bool mine = ((t == 1) ? (c >= 128) : (ntile == 1 || c < 128)) && c < ni;
        for (int g = h; g < P.nbr / 8; g += 2) {
          long long hi[8], lo[8];
          load_levels8(tlane + (uint32_t)(g * 8), D, R, hi, lo);
          if (!mine) continue;
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int r = g * 8 + q;
            if (r >= nb) continue;
            const int sx = ey[c] + eT[r] - R * (D + 1);
            const double sc = __longlong_as_double((long long)(1023 + sx) << 52);
            const double sch = __longlong_as_double((long long)(1023 + sx + s) << 52);
            AS[(size_t)c * nb + r] = fma(__ll2double_rn(hi[q]), sch, __ll2double_rn(lo[q]) * sc);
          }
        }
        release();
      }
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase),
                 "r"(CT_TMEM_COLS));
  }
#undef CT_SEGMENT
}


// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int cond_tc_rows(int nif) { int nr = (nif + 15) / 16 * 16; return nr < 128 ? 128 : nr; }
int cond_tc_brows(int nbf) { return (nbf + 15) / 16 * 16; }
size_t cond_tc_bytes_a(int nif, int nbf, int digits) {
  return (size_t)digits * cond_tc_brows(nbf) / 16 * cond_tc_rows(nif) * 32;
}
size_t cond_tc_bytes_b(int nbf, int digits) {
  return (size_t)digits * cond_tc_brows(nbf) / 16 * cond_tc_brows(nbf) * 32;
}
// the fused condensation: K = nb <= 64 (exact level sums, one TMEM slot of
// 64 columns per level), rows in two 128-row tiles, digits of one element in
// shared memory
bool cond_tc_supported(int nif, int nbf, int digits) {
  if (nbf <= 0 || nbf > 64 || digits > CT_MAXDIG || cond_tc_rows(nif) > 256) return false;
  size_t sm = cond_tc_bytes_a(nif, nbf, digits) + cond_tc_bytes_b(nbf, digits) + 1024;
  return sm <= 226 * 1024;
}

void cond_tc_make_out(int nif, int nbf, int radix, int digits, CondTcBufs& b) {
  b.nr = cond_tc_rows(nif);
  b.nbr = cond_tc_brows(nbf);
  b.nkb = b.nbr / 16;
  b.digits = digits;
  b.radix = radix;
  b.bytes_a = cond_tc_bytes_a(nif, nbf, digits);
  b.bytes_b = cond_tc_bytes_b(nbf, digits);
}

// the fused kernel's tiles, W chunks and digit pairs for one bin
static void cond_tc_params(int nif, int nbf, int nel, const CondTcBufs& b, CondTcParams* Q) {
  CondTcParams& P = *Q;
  memset(&P, 0, sizeof(P));
  P.digits = b.digits; P.radix = b.radix;
  P.nr = b.nr; P.nbr = b.nbr; P.nkb = b.nkb;
  P.nif = nif; P.nbf = nbf; P.nel = nel;
  P.bytes_a = (uint32_t)b.bytes_a; P.bytes_b = (uint32_t)b.bytes_b;
  int nch = 0;
  for (int c0 = 0; c0 < P.nr; c0 += CT_NC) {
    P.ch_m0[nch] = 0; P.ch_c0[nch] = c0; P.ch_rmin[nch] = 0;
    P.ch_nc[nch] = (P.nr - c0) < CT_NC ? (P.nr - c0) : CT_NC;
    ++nch;
  }
  if (P.nr > 128)
    for (int c0 = 128; c0 < P.nr; c0 += CT_NC) {
      P.ch_m0[nch] = P.nr - 128; P.ch_c0[nch] = c0; P.ch_rmin[nch] = 128;
      P.ch_nc[nch] = (P.nr - c0) < CT_NC ? (P.nr - c0) : CT_NC;
      ++nch;
    }
  P.nchunk = nch;
  int np = 0;
  for (int s = 2; s <= b.digits + 1; ++s)
    for (int i = 1; i < s; ++i) {
      P.pi[np] = (int8_t)i; P.pj[np] = (int8_t)(s - i); P.pfirst[np] = (int8_t)(i == 1);
      ++np;
    }
  P.npair = np;
}

static CondTcOut cond_tc_out(const CondTcBufs& b) {
  CondTcOut o;
  o.kbd = b.kbd; o.lid = b.lid; o.ltd = b.ltd;
  o.ekb = b.ekb; o.eli = b.eli; o.elt = b.elt; o.bi = b.bi;
  o.nr = b.nr; o.nbr = b.nbr; o.nkb = b.nkb; o.digits = b.digits; o.radix = b.radix;
  o.bytes_a = (uint32_t)b.bytes_a; o.bytes_b = (uint32_t)b.bytes_b;
  return o;
}

int cond_tc_group_build(const std::vector<CondSegIn>& in, CondGroup* g,
                        std::vector<void*>* allocs) {
  *g = CondGroup{};
  if (in.empty()) return 0;
  std::vector<CondSegDev> segs;
  std::vector<CompressSeg> cs;
  std::vector<int> pch{0}, pkb{0}, pel{0};
  bool plain_seen = false;
  for (const CondSegIn& q : in) {
    CondSegDev d;
    memset(&d, 0, sizeof(d));
    d.nfull = q.nfull; d.nif = q.nif; d.nbf = q.nbf; d.nel = q.nel;
    d.elist = q.elist; d.PK = q.PK; d.b0 = q.b0; d.perm = q.perm; d.W = q.W;
    if (q.nbf == 0) {
      // compression only: no blocks of the tensor-core kernels
      plain_seen = true;
      segs.push_back(d);
      cs.push_back({q.nfull, q.nif, 0, q.elist, q.PK, q.perm, q.W, nullptr, q.dmask, q.b0});
      pch.push_back(pch.back());
      pkb.push_back(pkb.back());
      pel.push_back(pel.back() + q.nel);
      g->smem_plain = std::max(g->smem_plain, (size_t)q.nif * sizeof(double));
      continue;
    }
    if (plain_seen || !cond_tc_supported(q.nif, q.nbf, q.t.digits) ||
        q.t.digits != COND_TC_DIGITS || q.t.radix != COND_TC_RADIX)
      return -2;
    d.o = cond_tc_out(q.t);
    cond_tc_params(q.nif, q.nbf, q.nel, q.t, &d.P);
    segs.push_back(d);
    cs.push_back({q.nfull, q.nif, q.nbf, q.elist, q.PK, q.perm, q.W, q.t.bi, q.dmask, nullptr});
    pch.push_back(pch.back() + (q.nel + CH_WARPS - 1) / CH_WARPS);
    pkb.push_back(pkb.back() + q.nel * ((q.t.nr + 127) / 128));
    pel.push_back(pel.back() + q.nel);
    g->smem_chol = std::max(g->smem_chol, cond_chol_smem(q.nbf));
    g->smem_tc = std::max(g->smem_tc, q.t.bytes_a + q.t.bytes_b + 1024);
    ++g->ntc;
  }
  auto dput = [&](const void* src, size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    allocs->push_back(p);
    if (cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    return p;
  };
  g->segs = dput(segs.data(), segs.size() * sizeof(CondSegDev));
  g->csegs = (CompressSeg*)dput(cs.data(), cs.size() * sizeof(CompressSeg));
  g->pre_chol = (int*)dput(pch.data(), pch.size() * 4);
  g->pre_kbi = (int*)dput(pkb.data(), pkb.size() * 4);
  g->pre_el = (int*)dput(pel.data(), pel.size() * 4);
  if (!g->segs || !g->csegs || !g->pre_chol || !g->pre_kbi || !g->pre_el) {
    *g = CondGroup{};
    return -1;
  }
  g->nseg = (int)segs.size();
  for (auto* v : {&pch, &pkb, &pel}) g->h_pre.insert(g->h_pre.end(), v->begin(), v->end());
  g->h_in = in;
  return 0;
}

int launch_cond_tc_group(const CondGroup& g, int k0, int k1, const int* d_ni_e, const int* d_nb_e,
                         const int64_t* d_schur_off, const int64_t* d_bub_off, double* d_aschur,
                         double* d_bschur, int* d_bad_spd, int* d_flag, cudaStream_t st) {
  k1 = std::min(k1, g.ntc);
  if (k1 <= k0) return 0;
  if (k1 == k0 + 1) {
    // one bin or chunk: the kernels with the segment's parameters in the
    // launch arguments (same device bodies and arithmetic as the grouped ones)
    const CondSegIn& q = g.h_in[k0];
    return launch_cond_tc(q.nel, q.nfull, q.nif, q.nbf, q.elist, d_ni_e, d_nb_e, q.PK, q.b0,
                          q.perm, d_schur_off, d_bub_off, q.W, d_aschur, d_bschur, q.t, d_bad_spd,
                          d_flag, st);
  }
  const int ns = g.nseg + 1;
  const int* h = g.h_pre.data();
  const int c0 = h[k0], c1 = h[k1], b0 = h[ns + k0], b1 = h[ns + k1];
  const int e0 = h[2 * ns + k0], e1 = h[2 * ns + k1];
  if (e1 <= e0) return 0;
  int dev = 0, num_sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return -1;
  const CondSegDev* segs = (const CondSegDev*)g.segs;
  if (raise_smem_limit((const void*)k_cond_chol_grp, g.smem_chol) != cudaSuccess) return -1;
  k_cond_chol_grp<<<c1 - c0, CH_WARPS * 32, g.smem_chol, st>>>(segs, g.pre_chol, g.nseg, c0,
                                                                 d_ni_e, d_nb_e, d_bub_off,
                                                                 d_bschur, d_bad_spd);
  k_cond_kbi_grp<<<b1 - b0, 128, 0, st>>>(segs, g.pre_kbi, g.nseg, b0, d_ni_e, d_nb_e, d_bub_off,
                                          d_bschur);
  if (raise_smem_limit((const void*)k_cond_tc_grp, g.smem_tc) != cudaSuccess) return -1;
  const int grid = (e1 - e0) < num_sms ? (e1 - e0) : num_sms;
  k_cond_tc_grp<<<grid, CT_THREADS, g.smem_tc, st>>>(segs, g.pre_el, g.nseg, e0, e1, d_ni_e,
                                                     d_nb_e, d_schur_off, d_aschur, d_flag);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_cond_tc(int nel, int nfull, int nif, int nbf, const int* d_elist, const int* d_ni_e,
                   const int* d_nb_e, const double* d_PK, const double* d_b0,
                   const uint32_t* d_perm, const int64_t* d_schur_off, const int64_t* d_bub_off,
                   double* d_W, double* d_aschur, double* d_bschur, const CondTcBufs& b,
                   int* d_bad_spd, int* d_flag, cudaStream_t st) {
  if (nel <= 0) return 0;
  if (!cond_tc_supported(nif, nbf, b.digits) || b.digits != COND_TC_DIGITS ||
      b.radix != COND_TC_RADIX)
    return -2;
  static int num_sms = 0;
  if (!num_sms) {
    int dev;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  CondTcOut o;
  o.kbd = b.kbd; o.lid = b.lid; o.ltd = b.ltd;
  o.ekb = b.ekb; o.eli = b.eli; o.elt = b.elt; o.bi = b.bi;
  o.nr = b.nr; o.nbr = b.nbr; o.nkb = b.nkb; o.digits = b.digits; o.radix = b.radix;
  o.bytes_a = (uint32_t)b.bytes_a; o.bytes_b = (uint32_t)b.bytes_b;
  size_t sm1 = cond_chol_smem(nbf);
  if (raise_smem_limit((const void*)k_cond_chol, sm1) != cudaSuccess) return -1;
  k_cond_chol<<<(nel + CH_WARPS - 1) / CH_WARPS, CH_WARPS * 32, sm1, st>>>(
      nfull, nif, nbf, d_elist, d_ni_e, d_nb_e, d_PK, d_b0, d_perm, d_bub_off, d_bschur, o, nel,
      d_bad_spd);
  k_cond_kbi<<<dim3(nel, (o.nr + 127) / 128), 128, 0, st>>>(nfull, nif, nbf, d_elist, d_ni_e,
                                                            d_nb_e, d_PK, d_b0, d_perm, d_bub_off,
                                                            d_bschur, o);
  CondTcParams P;
  cond_tc_params(nif, nbf, nel, b, &P);
  size_t sm2 = b.bytes_a + b.bytes_b + 1024;
  if (raise_smem_limit((const void*)k_cond_tc, sm2) != cudaSuccess) return -1;
  int grid = nel < num_sms ? nel : num_sms;
  k_cond_tc<<<grid, CT_THREADS, sm2, st>>>(b.kbd, b.lid, b.ltd, b.ekb, b.eli, b.elt, P, d_elist,
                                           d_ni_e, d_nb_e, d_schur_off, d_W, d_aschur, d_flag);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace hp3dg
