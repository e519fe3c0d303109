// Instantiations of the fused kernel (rg_fused_kernel.cuh) for
// 53..64 assets.
#include "rg_fused_kernel.cuh"

namespace rg {

cudaError_t launch_fused_d(const PlainArgs &a, const float *Lp_host, const float *hmu, const float *w,
                         int sm_count, cudaStream_t s)
{
    switch ((a.n + 3) / 4) {
    case 14: return launch_fused_nq<14>(a, Lp_host, hmu, w, sm_count, s);
    case 15: return launch_fused_nq<15>(a, Lp_host, hmu, w, sm_count, s);
    case 16: return launch_fused_nq<16>(a, Lp_host, hmu, w, sm_count, s);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace rg
