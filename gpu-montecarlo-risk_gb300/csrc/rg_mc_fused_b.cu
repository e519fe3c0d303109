// Instantiations of the fused kernel (rg_fused_kernel.cuh) for
// 33..44 assets.
#include "rg_fused_kernel.cuh"

namespace rg {

cudaError_t launch_fused_b(const PlainArgs &a, const float *Lp_host, const float *hmu, const float *w,
                         int sm_count, cudaStream_t s)
{
    switch ((a.n + 3) / 4) {
    case 9: return launch_fused_nq<9>(a, Lp_host, hmu, w, sm_count, s);
    case 10: return launch_fused_nq<10>(a, Lp_host, hmu, w, sm_count, s);
    case 11: return launch_fused_nq<11>(a, Lp_host, hmu, w, sm_count, s);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace rg
