// Instantiations of the fused kernel (rg_fused_kernel.cuh) for
// 53..56 assets.
#include "rg_fused_kernel.cuh"

namespace rg {

cudaError_t launch_fused_d(const PlainArgs &a, const float *Lp_host, const float *hmu, const float *w,
                         int sm_count, cudaStream_t s)
{
    if ((a.n + 3) / 4 != 14) return cudaErrorInvalidValue;
    return launch_fused_nq<14>(a, Lp_host, hmu, w, sm_count, s);
}

} // namespace rg
