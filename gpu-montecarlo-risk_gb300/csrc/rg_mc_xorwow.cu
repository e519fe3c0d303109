// Instantiations of the plain fused kernel (rg_plain_kernel.cuh) for the
// reference kernel's own cuRAND XORWOW stream (monte_carlos_cuda.cu:30-31,
// 45-47), kept in their own translation unit so they compile in parallel.
#include "rg_plain_kernel.cuh"

namespace rg {

cudaError_t launch_plain_small_xorwow(const PlainArgs &a, int sm_count, cudaStream_t s)
{
    if (a.n <= 16) return launch_np<16, RG_RNG_XORWOW_REF>(a, sm_count, s);
    if (a.n <= 32) return launch_np<32, RG_RNG_XORWOW_REF>(a, sm_count, s);
    if (a.n <= 64) return launch_np<64, RG_RNG_XORWOW_REF>(a, sm_count, s);
    return cudaErrorInvalidValue;
}

} // namespace rg
