// Instantiations of the fused kernel (rg_fused_kernel.cuh) for
// 61..64 assets.
#include "rg_fused_kernel.cuh"

namespace rg {

cudaError_t launch_fused_f(const PlainArgs &a, const float *Lp_host, const float *hmu, const float *w,
                         int sm_count, cudaStream_t s)
{
    if ((a.n + 3) / 4 != 16) return cudaErrorInvalidValue;
    return launch_fused_nq<16>(a, Lp_host, hmu, w, sm_count, s);
}

} // namespace rg
