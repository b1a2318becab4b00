// FP64 / FP32 pipe throughput probe (roofline denominators).
// Independent FMA chains in every thread of a grid that fills every SM; the
// result is flop/s with one FMA counted as two flops.
#include "h4_internal.cuh"

namespace h4 {
namespace {
constexpr int CH = 8;

__global__ void k_probe_dfma(double *out, int iters, double a, double b) {
    double c[CH];
#pragma unroll
    for (int k = 0; k < CH; k++) c[k] = threadIdx.x * 1e-3 + k;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < CH; k++) c[k] = fma(c[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < CH; k++) s += c[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_probe_ffma(float *out, int iters, float a, float b) {
    float c[CH];
#pragma unroll
    for (int k = 0; k < CH; k++) c[k] = threadIdx.x * 1e-3f + k;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < CH; k++) c[k] = fmaf(c[k], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < CH; k++) s += c[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

// One thread waits, bounded, on a flag that nothing sets.
__global__ void k_selftest_wait(const unsigned *flag, unsigned long long timeout_ns, unsigned *result) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    *result = bounded_wait_change(flag, 0u, timeout_ns) ? 0u : 1u;
}

cudaError_t selftest_bounded_wait(double seconds, int *timed_out) {
    unsigned *buf = nullptr;
    cudaError_t e = cudaMalloc(&buf, 2 * sizeof(unsigned));
    if (e != cudaSuccess) return e;
    e = cudaMemset(buf, 0, 2 * sizeof(unsigned));
    if (e == cudaSuccess) {
        k_selftest_wait<<<1, 32>>>(buf, (unsigned long long)(seconds * 1e9), buf + 1);
        e = cudaGetLastError();
    }
    unsigned r = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&r, buf + 1, sizeof(unsigned), cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (e == cudaSuccess && timed_out) *timed_out = (int)r;
    return e;
}

cudaError_t probe_peaks(double *fp64, double *fp32) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int blocks = sms * 8, threads = 256;
    const size_t nt = (size_t)blocks * threads;
    void *buf = nullptr;
    e = cudaMalloc(&buf, nt * sizeof(double));
    if (e != cudaSuccess) return e;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float ms = 0.f, best64 = 1e30f, best32 = 1e30f;
    const int it64 = 2000, it32 = 100000;
    k_probe_dfma<<<blocks, threads>>>((double *)buf, 50, 0.9999999, 1e-9);
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(e0);
        k_probe_dfma<<<blocks, threads>>>((double *)buf, it64, 0.9999999, 1e-9);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best64) best64 = ms;
        cudaEventRecord(e0);
        k_probe_ffma<<<blocks, threads>>>((float *)buf, it32, 0.9999999f, 1e-9f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best32) best32 = ms;
    }
    e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (e != cudaSuccess) return e;
    if (fp64) *fp64 = 2.0 * CH * (double)it64 * (double)nt / (best64 * 1e-3);
    if (fp32) *fp32 = 2.0 * CH * (double)it32 * (double)nt / (best32 * 1e-3);
    return cudaSuccess;
}

}  // namespace h4
