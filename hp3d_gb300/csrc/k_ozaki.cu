// k_ozaki.cu -- mixed-precision contraction (placeholder until the tcgen05 kernel lands).
#include "hp3dg_kernels.h"
namespace hp3dg {
int ozaki_plan(int, int, int, int, OzakiPlan*) { return -1; }
int launch_ozaki_build_m(const OzakiPlan&, int, int, int, int, const double*, uint16_t*, double*,
                         double*, cudaStream_t) { return -1; }
size_t ozaki_m_bytes(const OzakiPlan&) { return 0; }
int launch_ozaki_slice_d(const OzakiPlan&, int, int, const double*, uint16_t*, double*,
                         cudaStream_t) { return -1; }
size_t ozaki_d_bytes(const OzakiPlan&, int) { return 0; }
int launch_ozaki_gemm(const OzakiPlan&, int, int, const uint16_t*, const double*, const uint16_t*,
                      const double*, double*, int*, cudaStream_t) { return -1; }
}  // namespace hp3dg
