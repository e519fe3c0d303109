// Instantiations of the fused kernel (rg_fused_kernel.cuh) for
// 45..52 assets.
#include "rg_fused_kernel.cuh"

namespace rg {

cudaError_t launch_fused_c(const PlainArgs &a, const float *Lp_host, const float *hmu, const float *w,
                         int sm_count, cudaStream_t s)
{
    switch ((a.n + 3) / 4) {
    case 12: return launch_fused_nq<12>(a, Lp_host, hmu, w, sm_count, s);
    case 13: return launch_fused_nq<13>(a, Lp_host, hmu, w, sm_count, s);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace rg
