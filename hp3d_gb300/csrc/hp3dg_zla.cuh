// hp3dg_zla.cuh -- complex FP64 dense algebra for one CTA on global memory
// (column-major): a tiled complex GEMM, a blocked right-looking Cholesky and
// forward / backward triangular solves.  Used by the DPG Maxwell kernels,
// one element per CTA of LA_THREADS threads; the shared buffer `sm` holds
// 2 * TK * TM double2.
#pragma once
#include <cuda_runtime.h>

namespace hp3dg {
namespace zla {

__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 zscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
// acc += a * b
__device__ __forceinline__ void zfma(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}

constexpr int LA_THREADS = 256;
constexpr int TM = 64, TN = 64, TK = 16, NB = 32;

// C (M x N) = beta C + sgn op(A) op(B), column-major; op = as stored or
// conjugate transpose.  lower: only entries i >= j of C are written.  The
// whole CTA cooperates; ends with a barrier.
static __device__ void cta_zgemm(int M, int N, int K, const double2* A, int lda, bool cA, const double2* B,
                          int ldb, bool cB, double2* C, int ldc, double sgn, bool beta1, bool lower,
                          double2* sm) {
  double2* As = sm;             // [TK][TM]
  double2* Bs = sm + TK * TM;   // [TK][TN]
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  for (int t0 = 0; t0 < M; t0 += TM)
    for (int u0 = 0; u0 < N; u0 += TN) {
      if (lower && u0 > t0 + TM - 1) continue;
      double2 acc[4][4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = make_double2(0.0, 0.0);
      for (int k0 = 0; k0 < K; k0 += TK) {
        for (int x = tid; x < TK * TM; x += LA_THREADS) {
          int kk, ii;
          if (!cA) { kk = x / TM; ii = x % TM; } else { ii = x / TK; kk = x % TK; }
          const int gi = t0 + ii, gk = k0 + kk;
          double2 v = make_double2(0.0, 0.0);
          if (gi < M && gk < K) v = cA ? zconj(A[gk + (size_t)gi * lda]) : A[gi + (size_t)gk * lda];
          As[kk * TM + ii] = v;
        }
        for (int x = tid; x < TK * TN; x += LA_THREADS) {
          int kk, jj;
          if (!cB) { jj = x / TK; kk = x % TK; } else { kk = x / TN; jj = x % TN; }
          const int gj = u0 + jj, gk = k0 + kk;
          double2 v = make_double2(0.0, 0.0);
          if (gj < N && gk < K) v = cB ? zconj(B[gj + (size_t)gk * ldb]) : B[gk + (size_t)gj * ldb];
          Bs[kk * TN + jj] = v;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < TK; ++kk) {
          double2 a[4], b[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) a[r] = As[kk * TM + ty * 4 + r];
#pragma unroll
          for (int c = 0; c < 4; ++c) b[c] = Bs[kk * TN + tx * 4 + c];
#pragma unroll
          for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) zfma(acc[r][c], a[r], b[c]);
        }
        __syncthreads();
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int i = t0 + ty * 4 + r, j = u0 + tx * 4 + c;
          if (i >= M || j >= N || (lower && i < j)) continue;
          double2* cp = &C[i + (size_t)j * ldc];
          double2 v = zscale(sgn, acc[r][c]);
          *cp = beta1 ? zadd(*cp, v) : v;
        }
    }
  __syncthreads();
}

// A = L L^H in place (lower triangle), n x n.  Returns 0, or 1 + the column
// of a non-positive pivot (the factorisation continues with pivot 1).
static __device__ int cta_zpotrf(double2* A, int lda, int n, double2* sm) {
  __shared__ int bad;
  double2* D = sm;  // [NB][NB+1], aliases the GEMM tiles (phases are separate)
  if (threadIdx.x == 0) bad = 0;
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int kb = min(NB, n - k0);
    for (int x = threadIdx.x; x < kb * kb; x += LA_THREADS) {
      const int i = x % kb, j = x / kb;
      if (i >= j) D[i * (NB + 1) + j] = A[(k0 + i) + (size_t)(k0 + j) * lda];
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      for (int j = 0; j < kb; ++j) {
        if (lane == j) {
          double d = D[j * (NB + 1) + j].x;
          if (!(d > 0.0)) { if (!bad) bad = k0 + j + 1; d = 1.0; }
          D[j * (NB + 1) + j] = make_double2(sqrt(d), 0.0);
        }
        __syncwarp();
        const double rd = 1.0 / D[j * (NB + 1) + j].x;
        if (lane > j && lane < kb) D[lane * (NB + 1) + j] = zscale(rd, D[lane * (NB + 1) + j]);
        __syncwarp();
        for (int c = j + 1; c < kb; ++c)
          if (lane >= c && lane < kb)
            D[lane * (NB + 1) + c] =
                zsub(D[lane * (NB + 1) + c], zmul(D[lane * (NB + 1) + j], zconj(D[c * (NB + 1) + j])));
        __syncwarp();
      }
    }
    __syncthreads();
    for (int x = threadIdx.x; x < kb * kb; x += LA_THREADS) {
      const int i = x % kb, j = x / kb;
      if (i >= j) A[(k0 + i) + (size_t)(k0 + j) * lda] = D[i * (NB + 1) + j];
    }
    // panel rows below: x L11^H = a (reciprocals of the diagonal: one division each)
    __shared__ double rdg[NB];
    if (threadIdx.x < kb) rdg[threadIdx.x] = 1.0 / D[threadIdx.x * (NB + 1) + threadIdx.x].x;
    __syncthreads();
    for (int r = k0 + kb + threadIdx.x; r < n; r += LA_THREADS) {
      double2 x[NB];
      for (int j = 0; j < kb; ++j) {
        double2 t = A[r + (size_t)(k0 + j) * lda];
        for (int q = 0; q < j; ++q) t = zsub(t, zmul(x[q], zconj(D[j * (NB + 1) + q])));
        x[j] = zscale(rdg[j], t);
      }
      for (int j = 0; j < kb; ++j) A[r + (size_t)(k0 + j) * lda] = x[j];
    }
    __syncthreads();
    const int m = n - k0 - kb;
    if (m > 0)
      cta_zgemm(m, m, kb, &A[(k0 + kb) + (size_t)k0 * lda], lda, false,
                &A[(k0 + kb) + (size_t)k0 * lda], lda, true,
                &A[(k0 + kb) + (size_t)(k0 + kb) * lda], lda, -1.0, true, true, sm);
  }
  __syncthreads();
  return bad;
}

// X = L^-1 X (forward) with L lower n x n, X n x m.
static __device__ void cta_ztrsm_fwd(const double2* L, int ldl, int n, double2* X, int ldx, int m,
                              double2* sm) {
  double2* D = sm;
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int kb = min(NB, n - k0);
    for (int x = threadIdx.x; x < kb * kb; x += LA_THREADS) {
      const int i = x % kb, j = x / kb;
      if (i >= j) D[i * (NB + 1) + j] = L[(k0 + i) + (size_t)(k0 + j) * ldl];
    }
    __shared__ double rdf[NB];
    if (threadIdx.x < kb) rdf[threadIdx.x] = 1.0 / L[(k0 + threadIdx.x) + (size_t)(k0 + threadIdx.x) * ldl].x;
    __syncthreads();
    for (int c = threadIdx.x; c < m; c += LA_THREADS) {
      double2 x[NB];
      for (int i = 0; i < kb; ++i) {
        double2 t = X[(k0 + i) + (size_t)c * ldx];
        for (int q = 0; q < i; ++q) t = zsub(t, zmul(D[i * (NB + 1) + q], x[q]));
        x[i] = zscale(rdf[i], t);
      }
      for (int i = 0; i < kb; ++i) X[(k0 + i) + (size_t)c * ldx] = x[i];
    }
    __syncthreads();
    const int rows = n - k0 - kb;
    if (rows > 0)
      cta_zgemm(rows, m, kb, &L[(k0 + kb) + (size_t)k0 * ldl], ldl, false, &X[k0], ldx, false,
                &X[k0 + kb], ldx, -1.0, true, false, sm);
  }
}

// X = L^-H X (backward) with L lower n x n, X n x m.
static __device__ void cta_ztrsm_bwd(const double2* L, int ldl, int n, double2* X, int ldx, int m,
                              double2* sm) {
  double2* D = sm;
  const int nblk = (n + NB - 1) / NB;
  for (int b = nblk - 1; b >= 0; --b) {
    const int k0 = b * NB, kb = min(NB, n - k0);
    for (int x = threadIdx.x; x < kb * kb; x += LA_THREADS) {
      const int i = x % kb, j = x / kb;
      if (i >= j) D[i * (NB + 1) + j] = L[(k0 + i) + (size_t)(k0 + j) * ldl];
    }
    __shared__ double rdb[NB];
    if (threadIdx.x < kb) rdb[threadIdx.x] = 1.0 / L[(k0 + threadIdx.x) + (size_t)(k0 + threadIdx.x) * ldl].x;
    __syncthreads();
    // L11^H x = b: x_j = (b_j - sum_{t>j} conj(L11[t][j]) x_t) / L11[j][j]
    for (int c = threadIdx.x; c < m; c += LA_THREADS) {
      double2 x[NB];
      for (int j = kb - 1; j >= 0; --j) {
        double2 t = X[(k0 + j) + (size_t)c * ldx];
        for (int q = j + 1; q < kb; ++q) t = zsub(t, zmul(zconj(D[q * (NB + 1) + j]), x[q]));
        x[j] = zscale(rdb[j], t);
      }
      for (int j = 0; j < kb; ++j) X[(k0 + j) + (size_t)c * ldx] = x[j];
    }
    __syncthreads();
    // rows above: X[0:k0] -= (L[k0:k0+kb, 0:k0])^H X[k0:k0+kb]
    if (k0 > 0)
      cta_zgemm(k0, m, kb, &L[k0], ldl, true, &X[k0], ldx, false, X, ldx, -1.0, true, false, sm);
  }
}


}  // namespace zla
}  // namespace hp3dg
