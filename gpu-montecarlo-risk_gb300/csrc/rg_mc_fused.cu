// Instantiations of the fused kernel (rg_fused_kernel.cuh) for 1..32
// assets and the dispatcher by asset count.  The larger instantiations are
// split over rg_mc_fused_b/c/d/e/f.cu so they compile in parallel (a
// 64-asset instantiation alone takes about a minute).
#include "rg_fused_kernel.cuh"

namespace rg {

cudaError_t launch_fused_b(const PlainArgs &a, const float *Lp_host, const float *hmu, const float *w,
                         int sm_count, cudaStream_t s);
cudaError_t launch_fused_c(const PlainArgs &a, const float *Lp_host, const float *hmu, const float *w,
                         int sm_count, cudaStream_t s);
cudaError_t launch_fused_d(const PlainArgs &a, const float *Lp_host, const float *hmu, const float *w,
                         int sm_count, cudaStream_t s);
cudaError_t launch_fused_e(const PlainArgs &a, const float *Lp_host, const float *hmu, const float *w,
                         int sm_count, cudaStream_t s);
cudaError_t launch_fused_f(const PlainArgs &a, const float *Lp_host, const float *hmu, const float *w,
                         int sm_count, cudaStream_t s);

int fused_max_n() { return 64; }

cudaError_t launch_fused(const PlainArgs &a, const float *Lp_host, const float *hmu, const float *w,
                         int sm_count, cudaStream_t s)
{
    const int nq = (a.n + 3) / 4;
    if (nq >= 16) return launch_fused_f(a, Lp_host, hmu, w, sm_count, s);
    if (nq >= 15) return launch_fused_e(a, Lp_host, hmu, w, sm_count, s);
    if (nq >= 14) return launch_fused_d(a, Lp_host, hmu, w, sm_count, s);
    if (nq >= 12) return launch_fused_c(a, Lp_host, hmu, w, sm_count, s);
    if (nq >= 9) return launch_fused_b(a, Lp_host, hmu, w, sm_count, s);
    switch (nq) {
    case 1: return launch_fused_nq<1>(a, Lp_host, hmu, w, sm_count, s);
    case 2: return launch_fused_nq<2>(a, Lp_host, hmu, w, sm_count, s);
    case 3: return launch_fused_nq<3>(a, Lp_host, hmu, w, sm_count, s);
    case 4: return launch_fused_nq<4>(a, Lp_host, hmu, w, sm_count, s);
    case 5: return launch_fused_nq<5>(a, Lp_host, hmu, w, sm_count, s);
    case 6: return launch_fused_nq<6>(a, Lp_host, hmu, w, sm_count, s);
    case 7: return launch_fused_nq<7>(a, Lp_host, hmu, w, sm_count, s);
    case 8: return launch_fused_nq<8>(a, Lp_host, hmu, w, sm_count, s);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace rg
