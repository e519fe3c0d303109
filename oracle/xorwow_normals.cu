// ORACLE TEST INFRASTRUCTURE -- not the engine.
//
// cuRAND draws for the parity tests.  The reference kernel's normals come
// from cuRAND's device API (src/05-GPU/monte_carlos_cuda.cu:30-31,45-47:
// curand_init(seed, idx, 0, &curandState) with the default XORWOW state,
// then curand_normal_double per asset).  That stream exists only on the
// GPU, so the oracle obtains it by making those same library calls here and
// does the rest of the reference's arithmetic on the CPU
// (mc_oracle.c: orc_kernel_from_normals).
//
// It also draws raw cuRAND Philox4_32_10 words (curand_init(seed, path, 0)
// then curand4) so the engine's own Philox stream can be checked against
// cuRAND's seed/subsequence layout.
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>
#include <curand_kernel.h>

__global__ void xorwow_normals_kernel(unsigned long long seed, unsigned long long path0, long long M,
                                      int n_per_path, double *out)
{
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= M) return;
    curandState st;
    curand_init(seed, path0 + (unsigned long long)p, 0ull, &st);
    for (int j = 0; j < n_per_path; j++) out[p * n_per_path + j] = curand_normal_double(&st);
}

__global__ void philox_words_kernel(unsigned long long seed, unsigned long long path0, long long M,
                                    int blocks, uint32_t *out)
{
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= M) return;
    curandStatePhilox4_32_10_t st;
    curand_init(seed, path0 + (unsigned long long)p, 0ull, &st);
    for (int b = 0; b < blocks; b++) {
        uint4 v = curand4(&st);
        uint32_t *o = out + (p * blocks + b) * 4;
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    }
}

template <class F>
static int run_and_copy(size_t bytes, void *host_out, F launch)
{
    void *d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) return -1;
    launch(d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(host_out, d, bytes, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        fprintf(stderr, "oracle cuRAND helper: %s\n", cudaGetErrorString(e));
        return -1;
    }
    return 0;
}

extern "C" int orc_xorwow_normals(unsigned long long seed, unsigned long long path0, long long M,
                                  int n_per_path, double *host_out)
{
    const size_t bytes = sizeof(double) * (size_t)M * (size_t)n_per_path;
    return run_and_copy(bytes, host_out, [&](void *d) {
        xorwow_normals_kernel<<<(unsigned)((M + 127) / 128), 128>>>(seed, path0, M, n_per_path, (double *)d);
    });
}

extern "C" int orc_curand_philox_words(unsigned long long seed, unsigned long long path0, long long M,
                                       int blocks, uint32_t *host_out)
{
    const size_t bytes = sizeof(uint32_t) * 4 * (size_t)M * (size_t)blocks;
    return run_and_copy(bytes, host_out, [&](void *d) {
        philox_words_kernel<<<(unsigned)((M + 127) / 128), 128>>>(seed, path0, M, blocks, (uint32_t *)d);
    });
}
