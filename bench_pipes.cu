// Pipe throughput probes: the denominators of the kernel rooflines, measured
// on the device that runs the propagator.  Each thread runs eight independent
// chains of one operation; the result is written so nothing is elided.
#include <cuda_runtime.h>

#include "cp3_launch.h"

namespace cp3 {

constexpr int kProbeIters = 4096;

// 32x32 -> 64 integer products (mul.wide.s32, the form the Q1.30 chain
// uses): each chain forms two products of its value per iteration and
// continues with the sum of their high words, so every product is used and
// one ALU add per two products rides beside them.  The multipliers change
// every iteration so that no product can be hoisted out of the loop.  (The
// accumulating form, mad.wide.s32 into a 64-bit register, measured about 10 %
// fewer products per second on GB300.)
__global__ void probe_imul_wide(long long* out, int a) {
    int y[8];
    for (int i = 0; i < 8; i++) y[i] = threadIdx.x * 7 + i;
    const int z1 = a | 1, z2 = 3 * a + 1;
    for (int it = 0; it < kProbeIters / 2; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) {
            long long p, q;
            asm volatile("mul.wide.s32 %0, %1, %2;" : "=l"(p) : "r"(y[i]), "r"(z1 ^ it));
            asm volatile("mul.wide.s32 %0, %1, %2;" : "=l"(q) : "r"(y[i]), "r"(z2 ^ it));
            y[i] = (int)(p >> 32) + (int)(q >> 32);
        }
    }
    long long s = 0;
    for (int i = 0; i < 8; i++) s += y[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void probe_ffma(float* out, float a, float b) {
    float x[8];
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-3f + i;
    for (int it = 0; it < kProbeIters; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(x[i]) : "f"(a), "f"(b));
    }
    float s = 0;
    for (int i = 0; i < 8; i++) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void probe_dfma(double* out, double a, double b) {
    double x[8];
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-3 + i;
    for (int it = 0; it < kProbeIters / 16; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(x[i]) : "d"(a), "d"(b));
    }
    double s = 0;
    for (int i = 0; i < 8; i++) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t measure_pipe(int pipe, double* ops) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int threads = 256, blocks = sms * 8;
    void* buf = nullptr;
    if ((e = cudaMalloc(&buf, (size_t)threads * blocks * 8)) != cudaSuccess) return e;
    cudaStream_t s;
    if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) {
        cudaFree(buf);
        return e;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double per_thread = 8.0 * (pipe == 2 ? kProbeIters / 16 : kProbeIters);
    float best = 1e30f;
    for (int r = 0; r < 4 && e == cudaSuccess; r++) {
        cudaEventRecord(e0, s);
        if (pipe == 0)
            probe_imul_wide<<<blocks, threads, 0, s>>>((long long*)buf, 3);
        else if (pipe == 1)
            probe_ffma<<<blocks, threads, 0, s>>>((float*)buf, 0.999f, 0.001f);
        else
            probe_dfma<<<blocks, threads, 0, s>>>((double*)buf, 0.999, 0.001);
        cudaEventRecord(e1, s);
        e = cudaEventSynchronize(e1);
        float ms = 0;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0 && ms < best) best = ms;  // first run is a warm-up
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    *ops = per_thread * threads * (double)blocks / (best * 1e-3);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    cudaFree(buf);
    return e;
}

}  // namespace cp3
