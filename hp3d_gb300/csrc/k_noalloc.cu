// k_noalloc.cu -- static condensation entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc: element loops that run inside an
// OpenMP region of a host solver (the reference's mumps_sc loop is one),
// where a device allocation would serialise every thread on the CUDA context
// and synchronise the device; applications whose device memory is owned by
// their own pool allocator or by a solver sharing the GPU, with no room left
// for a library's private buffers; and repeated small calls whose cost an
// allocation per call would dominate.  For them this file provides
// hp3dg_condense_noalloc: the static condensation of caller-supplied dense
// element matrices (stc_fwd of modules/stc.F90:182-509 restated on the GPU).
// The caller passes inputs and outputs as device pointers; the only scratch
// the kernel needs -- the packed upper triangle of each Schur complement --
// lives in a file-scope __device__ array of fixed size, so no call allocates.
//
// The scratch array holds HP3DG_NOALLOC_SCRATCH_DOUBLES doubles (8 MiB) and
// stays resident on every GPU that loads this library until the process
// exits.  All calls share it and it keeps the previous call's contents: the
// kernel writes every scratch entry it reads before reading it, so nothing
// needs clearing, but two calls whose kernels overlap on the GPU (different
// streams, or different host threads) race on the array and must be ordered
// by the caller.  The first call on each device takes the device address of
// the array with cudaGetSymbolAddress; make that first call before any stream
// capture begins.
#include "../../include/hp3dg.h"
#include "hp3dg_internal.cuh"
#include "hp3dg_kernels.h"

#include <cuda_runtime.h>

#include <mutex>

namespace {

constexpr long long kScratchDoubles = HP3DG_NOALLOC_SCRATCH_DOUBLES;
__device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

// Device address of the scratch array on the current device.  In host code
// g_noalloc_scratch is only a host-side stand-in, so the address is taken
// once per device with cudaGetSymbolAddress (first call on that device).
int scratch_for_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return HP3DG_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return HP3DG_ERR_CUDA;
    g_scratch_ptr[dev] = (double*)p;
  }
  *out = g_scratch_ptr[dev];
  return HP3DG_OK;
}

constexpr int NT = 256;

// One CTA per element: Cholesky of the SPD bubble block in shared memory,
// Y = L^-1 [K_bi | b_b], Schur upper triangle S = K_ii - Y^T Y into the
// scratch array, then the full symmetric Aii written from S, condensed load,
// ASchur = L^-T Y, BSchur = L^-T y_b.  Interface dof first, bubbles last,
// as the split of stc_fwd_wrapper (stc.F90:227-261).
__global__ void __launch_bounds__(NT) k_condense_dense(int n, int ni, int nb,
                                                       const double* __restrict__ K,
                                                       const double* __restrict__ b,
                                                       double* __restrict__ scratch,
                                                       double* __restrict__ aii,
                                                       double* __restrict__ bi_out,
                                                       double* __restrict__ aschur,
                                                       double* __restrict__ bschur,
                                                       int* __restrict__ status) {
  extern __shared__ double sm[];
  const int e = blockIdx.x, tid = threadIdx.x;
  const double* Ke = K + (size_t)e * n * n;  // column-major, ld n
  const double* be = b + (size_t)e * n;
  const int ld = ni + 1;
  double* L = sm;
  double* Ys = sm + (size_t)nb * nb;
  double* bi = Ys + (size_t)nb * ld;
  double* S = scratch + (size_t)e * ((size_t)ni * (ni + 1) / 2);
  __shared__ int fail;
  if (tid == 0) fail = 0;
  for (int idx = tid; idx < nb * nb; idx += NT) {
    int r = idx / nb, c = idx % nb;
    L[idx] = Ke[(size_t)(ni + c) * n + ni + r];
  }
  for (int idx = tid; idx < nb * ni; idx += NT) {
    int c = idx / nb, r = idx % nb;
    Ys[r * ld + c] = Ke[(size_t)c * n + ni + r];
  }
  for (int r = tid; r < nb; r += NT) Ys[r * ld + ni] = be[ni + r];
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    if (tid == 0) {
      double d = L[k * nb + k];
      if (!(d > 0.0)) { fail = 1; d = 1.0; }
      L[k * nb + k] = sqrt(d);
    }
    __syncthreads();
    double dk = L[k * nb + k];
    for (int i = k + 1 + tid; i < nb; i += NT) L[i * nb + k] /= dk;
    __syncthreads();
    int m = nb - k - 1;
    for (int idx = tid; idx < m * m; idx += NT) {
      int ii = k + 1 + idx / m, jj = k + 1 + idx % m;
      if (jj <= ii) L[ii * nb + jj] -= L[ii * nb + k] * L[jj * nb + k];
    }
    __syncthreads();
  }
  if (fail && tid == 0) atomicMin(status, e);
  for (int c = tid; c < ld; c += NT)
    for (int r = 0; r < nb; ++r) {
      double s = Ys[r * ld + c];
      for (int k = 0; k < r; ++k) s -= L[r * nb + k] * Ys[k * ld + c];
      Ys[r * ld + c] = s / L[r * nb + r];
    }
  __syncthreads();
  for (int a = tid; a < ni; a += NT) {
    double s = 0.0;
    for (int r = 0; r < nb; ++r) s += Ys[r * ld + a] * Ys[r * ld + ni];
    bi[a] = be[a] - s;
    bi_out[(size_t)e * ni + a] = bi[a];
  }
  const long long nup = (long long)ni * (ni + 1) / 2;
  for (long long idx = tid; idx < nup; idx += NT) {
    int bb = (int)((sqrtf(8.0f * (float)idx + 1.0f) - 1.0f) * 0.5f);
    while ((long long)(bb + 1) * (bb + 2) / 2 <= idx) ++bb;
    while ((long long)bb * (bb + 1) / 2 > idx) --bb;
    int a = (int)(idx - (long long)bb * (bb + 1) / 2);
    double s = 0.0;
    for (int r = 0; r < nb; ++r) s += Ys[r * ld + a] * Ys[r * ld + bb];
    S[idx] = Ke[(size_t)bb * n + a] - s;
  }
  __syncthreads();
  double* A = aii + (size_t)e * ni * ni;  // column-major full
  for (long long idx = tid; idx < (long long)ni * ni; idx += NT) {
    int c = (int)(idx / ni), r = (int)(idx % ni);
    int lo = r < c ? r : c, hi = r < c ? c : r;
    A[idx] = S[(long long)hi * (hi + 1) / 2 + lo];
  }
  for (int c = tid; c < ld; c += NT)
    for (int r = nb - 1; r >= 0; --r) {
      double s = Ys[r * ld + c];
      for (int k = r + 1; k < nb; ++k) s -= L[k * nb + r] * Ys[k * ld + c];
      Ys[r * ld + c] = s / L[r * nb + r];
    }
  __syncthreads();
  for (int idx = tid; idx < nb * ni; idx += NT) {
    int c = idx / nb, r = idx % nb;
    aschur[(size_t)e * nb * ni + idx] = Ys[r * ld + c];
  }
  for (int r = tid; r < nb; r += NT) bschur[(size_t)e * nb + r] = Ys[r * ld + ni];
}

}  // namespace

extern "C" int hp3dg_condense_noalloc(int32_t n_elem, int32_t n, int32_t nb, const double* K,
                                      const double* b, double* aii, double* bi, double* aschur,
                                      double* bschur, int32_t* bad_element, void* stream) {
  if (bad_element) *bad_element = -1;
  if (n_elem < 0 || nb < 1 || n <= nb || !K || !b || !aii || !bi || !aschur || !bschur)
    return HP3DG_ERR_ARG;
  const int ni = n - nb;
  if ((long long)n_elem * ((long long)ni * (ni + 1) / 2) > kScratchDoubles - 1) return HP3DG_ERR_ARG;
  if (n_elem == 0) return HP3DG_OK;
  // one element's bubble block, [K_bi | b_b] and condensed load sit in shared
  // memory next to the kernel's static shared word: hexahedra up to p = 5
  // (nb = 64, ni = 152: 112 KB) fit, p = 6 (nb = 125, ni = 218: 345 KB) does not
  const size_t smem = ((size_t)nb * nb + (size_t)nb * (ni + 1) + ni) * sizeof(double);
  int dev = 0, optin = 0;
  cudaFuncAttributes fa;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
      cudaFuncGetAttributes(&fa, (const void*)k_condense_dense) != cudaSuccess)
    return HP3DG_ERR_CUDA;
  if (smem + fa.sharedSizeBytes > (size_t)optin) return HP3DG_ERR_UNSUPPORTED;
  double* scratch = nullptr;
  int rc = scratch_for_device(&scratch);
  if (rc != HP3DG_OK) return rc;
  // the status word is the last scratch slot (outside every element's part)
  int* status = (int*)(scratch + kScratchDoubles - 1);
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(status, 0x7f, sizeof(int), st) != cudaSuccess) return HP3DG_ERR_CUDA;
  if (hp3dg::raise_smem_limit((const void*)k_condense_dense, smem) != cudaSuccess) return HP3DG_ERR_CUDA;
  k_condense_dense<<<n_elem, NT, smem, st>>>(n, ni, nb, K, b, scratch, aii, bi, aschur, bschur,
                                             status);
  if (cudaPeekAtLastError() != cudaSuccess) return HP3DG_ERR_CUDA;
  int h = 0x7f7f7f7f;
  if (cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return HP3DG_ERR_CUDA;
  if (bad_element) *bad_element = (h == 0x7f7f7f7f) ? -1 : h;
  return (h == 0x7f7f7f7f) ? HP3DG_OK : HP3DG_ERR_NOT_SPD;
}
