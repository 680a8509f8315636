// Pipe throughput probes of bench.py: the denominators of the kernel
// rooflines, measured on the GPU that runs the propagator.  Each thread runs
// eight independent chains of one operation; the result is written so nothing
// is elided.  Thread 0 of block 0 also records the SM clock (clock64 against
// the global nanosecond timer) over its run, so that a rate can be compared
// per clock and per SM with the GPU's nominal figures.
//
// This is measurement code for the benchmark only: it is built into its own
// library (libbench_pipes.so) and is not part of the propagator's library or
// of its public header.
#include <cuda_runtime.h>

namespace {

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct ClockStamp {
    long long c0, c1;
    unsigned long long t0, t1;
};

__device__ __forceinline__ void stamp_begin(ClockStamp* st) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->t0 = global_ns();
        st->c0 = clock64();
    }
}
__device__ __forceinline__ void stamp_end(ClockStamp* st) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->c1 = clock64();
        st->t1 = global_ns();
    }
}

constexpr int kProbeIters = 4096;

// 32x32 -> 64 integer products (mul.wide.s32, the form the Q1.30 chain
// uses): each chain forms two products of its value per iteration and
// continues with the sum of their high words, so every product is used and
// one ALU add per two products rides beside them.  The multipliers change
// every iteration so that no product can be hoisted out of the loop.  (The
// accumulating form, mad.wide.s32 into a 64-bit register, measured about 10 %
// fewer products per second on GB300.)
__global__ void probe_imul_wide(long long* out, int a, ClockStamp* st) {
    stamp_begin(st);
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
    stamp_end(st);
}

__global__ void probe_ffma(float* out, float a, float b, ClockStamp* st) {
    stamp_begin(st);
    float x[8];
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-3f + i;
    for (int it = 0; it < kProbeIters; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(x[i]) : "f"(a), "f"(b));
    }
    float s = 0;
    for (int i = 0; i < 8; i++) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
    stamp_end(st);
}

__global__ void probe_dfma(double* out, double a, double b, ClockStamp* st) {
    stamp_begin(st);
    double x[8];
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-3 + i;
    for (int it = 0; it < kProbeIters / 16; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(x[i]) : "d"(a), "d"(b));
    }
    double s = 0;
    for (int i = 0; i < 8; i++) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
    stamp_end(st);
}

// Throughput of one pipe on the current device (0 mul.wide.s32, 1 FFMA,
// 2 DFMA) in operations per second, best of three timed runs after a
// warm-up, with the SM clock of that run in MHz and the SM count.
cudaError_t measure_pipe(int pipe, double* ops, double* sm_mhz, int* n_sm) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int threads = 256, blocks = sms * 8;
    void* buf = nullptr;
    if ((e = cudaMalloc(&buf, (size_t)threads * blocks * 8 + sizeof(ClockStamp))) != cudaSuccess) return e;
    ClockStamp* st = (ClockStamp*)((char*)buf + (size_t)threads * blocks * 8);
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
    double best_mhz = 0.0;
    for (int r = 0; r < 4 && e == cudaSuccess; r++) {
        cudaEventRecord(e0, s);
        if (pipe == 0)
            probe_imul_wide<<<blocks, threads, 0, s>>>((long long*)buf, 3, st);
        else if (pipe == 1)
            probe_ffma<<<blocks, threads, 0, s>>>((float*)buf, 0.999f, 0.001f, st);
        else
            probe_dfma<<<blocks, threads, 0, s>>>((double*)buf, 0.999, 0.001, st);
        cudaEventRecord(e1, s);
        e = cudaEventSynchronize(e1);
        float ms = 0;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        ClockStamp h{};
        if (e == cudaSuccess) e = cudaMemcpy(&h, st, sizeof h, cudaMemcpyDeviceToHost);
        if (r > 0 && ms < best && e == cudaSuccess) {  // first run is a warm-up
            best = ms;
            best_mhz = (h.t1 > h.t0) ? 1e3 * (double)(h.c1 - h.c0) / (double)(h.t1 - h.t0) : 0.0;
        }
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    *ops = per_thread * threads * (double)blocks / (best * 1e-3);
    *sm_mhz = best_mhz;
    *n_sm = sms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    cudaFree(buf);
    return e;
}

}  // namespace

// bench_pipe_peak(device, pipe, &ops_per_second, &sm_mhz, &n_sm): 0 on
// success, else the CUDA error code.
extern "C" int bench_pipe_peak(int device, int pipe, double* ops, double* sm_mhz, int* n_sm) {
    if (!ops || !sm_mhz || !n_sm || pipe < 0 || pipe > 2) return (int)cudaErrorInvalidValue;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = measure_pipe(pipe, ops, sm_mhz, n_sm);
    cudaSetDevice(prev);
    return (int)e;
}
