// FP32 FMA throughput probe: the measured ceiling that the count kernels'
// roofline fraction is reported against.  Eight independent FFMA chains per
// thread keep the pipe busy; the result is written only if it equals a value
// it can never take, so the chains are not optimised away.
#include "gbp_internal.cuh"

__global__ void __launch_bounds__(256) k_ffma_probe(float *sink, int iters) {
    float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
    float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
    const float b = 0.9999999f, c = 1e-7f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
            a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
            a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
        }
    }
    float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == -1.0f) sink[blockIdx.x] = s;
}

cudaError_t gbp_run_ffma_probe(int nsm, cudaStream_t st, float *ms_out, double *flops_out) {
    const int blocks = nsm * 8, threads = 256, iters = 4096;
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (e != cudaSuccess) return e;
    e = cudaEventCreate(&e1);
    if (e != cudaSuccess) { cudaEventDestroy(e0); return e; }
    k_ffma_probe<<<blocks, threads, 0, st>>>(nullptr, iters);  // warm-up
    cudaEventRecord(e0, st);
    k_ffma_probe<<<blocks, threads, 0, st>>>(nullptr, iters);
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    float ms = 0;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_out = ms;
    *flops_out = 2.0 * 8.0 * 16.0 * (double)iters * (double)blocks * (double)threads;
    return e;
}
