// Instantiations of the plain fused kernel (rg_plain_kernel.cuh) for the
// engine's Philox layout, and the dispatcher over both layouts.
#include "rg_plain_kernel.cuh"

namespace rg {

cudaError_t launch_plain_small_xorwow(const PlainArgs &a, int sm_count, cudaStream_t s);

int plain_small_max_n() { return 64; }

cudaError_t launch_plain_small(const PlainArgs &a, int rng, int sm_count, cudaStream_t s)
{
    if (rng != RG_RNG_PHILOX) return launch_plain_small_xorwow(a, sm_count, s);
    if (a.n <= 16) return launch_np<16, RG_RNG_PHILOX>(a, sm_count, s);
    if (a.n <= 32) return launch_np<32, RG_RNG_PHILOX>(a, sm_count, s);
    if (a.n <= 64) return launch_np<64, RG_RNG_PHILOX>(a, sm_count, s);
    return cudaErrorInvalidValue;
}

} // namespace rg
