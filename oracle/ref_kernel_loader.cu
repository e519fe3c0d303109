// ORACLE TEST INFRASTRUCTURE -- not the engine.
//
// Launches the reference's own GPU kernel, monte_carlo_kernel of
// src/05-GPU/monte_carlos_cuda.cu:23-72, compiled unmodified from the
// reference's source for sm_103a into a device-only fatbin
// (oracle/Makefile, target refcuda: _ref/ref_kernel.fatbin).  The fatbin
// holds no host code, so it is loaded here with the CUDA runtime's library
// API and launched the way the reference's host wrapper launches it
// (.cu:121-128: the count zeroed, 256 threads per block,
// ceil(M / 256) blocks, arguments in the kernel's order).
//
// Used by the parity tests (per-path S and the count of the reference
// kernel against the engine's XORWOW layout) and by the benchmark's
// baseline leg (the reference kernel timed on the same GPU).  The engine
// never loads it.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <cuda_runtime.h>

namespace {
std::mutex g_mu;
cudaLibrary_t g_lib = nullptr;
cudaKernel_t g_kernel = nullptr;
char g_path[4096] = "";
// monte_carlo_kernel(int, int, int, double, const double*, const double*,
//                    unsigned long, int*, int*)
const char *kKernelName = "_Z18monte_carlo_kerneliiidPKdS0_mPiS1_";
} // namespace

// Load (once per path) the fatbin and look up the kernel.  0 on success.
extern "C" int orc_ref_kernel_load(const char *fatbin_path)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_kernel && strcmp(g_path, fatbin_path) == 0) return 0;
    if (g_lib) {
        cudaLibraryUnload(g_lib);
        g_lib = nullptr;
        g_kernel = nullptr;
    }
    cudaError_t e = cudaLibraryLoadFromFile(&g_lib, fatbin_path, nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&g_kernel, g_lib, kKernelName);
    if (e != cudaSuccess) {
        fprintf(stderr, "oracle reference-kernel loader: %s: %s\n", fatbin_path, cudaGetErrorString(e));
        if (g_lib) cudaLibraryUnload(g_lib);
        g_lib = nullptr;
        g_kernel = nullptr;
        return -1;
    }
    snprintf(g_path, sizeof(g_path), "%s", fatbin_path);
    return 0;
}

// One launch of the reference kernel over M paths on `stream` (device
// pointers: mu[N], L[N*N] row-major with a zero upper triangle, S[M], count[1]).
// Returns 0 and the launch's device time in *ms (CUDA events on the stream).
extern "C" int orc_ref_kernel_run(int M, int N, int k, double x, const double *d_mu, const double *d_L,
                                  unsigned long seed, int *d_S, int *d_count, void *stream, float *ms)
{
    if (!g_kernel) return -1;
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_count, 0, sizeof(int), s);
    void *args[] = {&M, &N, &k, &x, (void *)&d_mu, (void *)&d_L, &seed, (void *)&d_S, (void *)&d_count};
    const int block = 256;
    const unsigned grid = (unsigned)((M + block - 1) / block);
    if (e == cudaSuccess) e = cudaEventRecord(e0, s);
    if (e == cudaSuccess) e = cudaLaunchKernel((const void *)g_kernel, dim3(grid), dim3(block), args, 0, s);
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess && ms) e = cudaEventElapsedTime(ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        fprintf(stderr, "oracle reference-kernel launch: %s\n", cudaGetErrorString(e));
        return -1;
    }
    return 0;
}
