// Test-only loader of the reference's CUDA kernel (oracle/ref_gpu_kernel.cu,
// compiled into oracle/_ref/ref_kernels.cubin) for bench.py's comparison with
// the reference on the GPU.  It contains no physics: it loads the cubin, copies
// the __constant__ data and the device arrays that the reference's own host
// code produced (oracle/ref_gpu_inputs.cpp, one file per precision and
// neutrino type), launches calculateKernel<FLOAT_T> the way
// CudaPropagatorSingle::calculateProbabilitiesAsync does (64-thread blocks,
// SDIV(n_energies, 64) * n_cosines blocks, cudapropagator.cuh:203-209), times
// the launches with CUDA events, and writes every `stride`-th cosine and
// energy of the nine result planes [9][n_cos][n_en] (as doubles) to a file.
//
//     ref_gpu_driver <cubin> <inputs.bin> <reps> <subset_out.bin> <stride>
//
// Prints one JSON line: precision, type, per-launch times (ms), the median,
// the kernel's registers and local memory per thread.  Every size read from
// the inputs is checked before anything is launched; the root order must be a
// permutation of 0, 1, 2 (the kernel indexes with it).
#include <cuda.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

int die(const char* what, CUresult r) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    std::printf("{\"error\": \"%s: %s\"}\n", what, s ? s : "unknown");
    return 1;
}

int die(const char* what) {
    std::printf("{\"error\": \"%s\"}\n", what);
    return 1;
}

struct Inputs {
    int32_t elem = 0, type = 0, n_cos = 0, n_en = 0, n_rows = 0;
    std::vector<unsigned char> cos, en, radii, rhos, height, mix, axfac, mass;
    std::vector<int32_t> maxl;
    int32_t order[3] = {0, 0, 0};
};

bool read_exact(std::FILE* f, void* dst, size_t n) { return std::fread(dst, 1, n, f) == n; }

bool load_inputs(const char* path, Inputs& in) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    char magic[8];
    int32_t head[6];
    bool ok = read_exact(f, magic, 8) && std::memcmp(magic, "CP3RGPU1", 8) == 0 && read_exact(f, head, sizeof head);
    if (ok) {
        in.elem = head[0];
        in.type = head[1];
        in.n_cos = head[2];
        in.n_en = head[3];
        in.n_rows = head[4];
        ok = (in.elem == 4 || in.elem == 8) && (in.type == 0 || in.type == 1) && in.n_cos > 0 && in.n_en > 0 &&
             in.n_cos <= 65536 && in.n_en <= 65536 && in.n_rows > 0 && in.n_rows <= 256;
    }
    auto arr = [&](std::vector<unsigned char>& v, size_t count) {
        v.resize(count * in.elem);
        return read_exact(f, v.data(), v.size());
    };
    if (ok) ok = arr(in.cos, in.n_cos) && arr(in.en, in.n_en) && arr(in.radii, in.n_rows) && arr(in.rhos, in.n_rows);
    if (ok) {
        in.maxl.resize(in.n_cos);
        ok = read_exact(f, in.maxl.data(), sizeof(int32_t) * in.n_cos);
    }
    if (ok) ok = arr(in.height, 1) && arr(in.mix, 18) && arr(in.axfac, 324) && arr(in.mass, 9);
    if (ok) ok = read_exact(f, in.order, sizeof in.order);
    std::fclose(f);
    if (!ok) return false;
    for (int32_t m : in.maxl)  // the kernel reads rows up to M (2n+1 are allocated)
        if (m < 0 || m > in.n_rows) return false;
    int seen = 0;
    for (int32_t o : in.order) {
        if (o < 0 || o > 2) return false;
        seen |= 1 << o;
    }
    return seen == 7;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s cubin inputs.bin reps subset_out.bin stride\n", argv[0]);
        return 2;
    }
    const int reps = std::max(1, std::atoi(argv[3]));
    const int stride = std::max(1, std::atoi(argv[5]));
    Inputs in;
    if (!load_inputs(argv[2], in)) return die("inputs file missing or malformed");
    CUresult r;
    if ((r = cuInit(0))) return die("cuInit", r);
    CUdevice dev;
    CUcontext ctx;
    if ((r = cuDeviceGet(&dev, 0))) return die("cuDeviceGet", r);
    if ((r = cuDevicePrimaryCtxRetain(&ctx, dev))) return die("cuDevicePrimaryCtxRetain", r);
    if ((r = cuCtxSetCurrent(ctx))) return die("cuCtxSetCurrent", r);
    CUmodule mod;
    if ((r = cuModuleLoad(&mod, argv[1]))) return die("cuModuleLoad", r);
    // the kernel instantiation of this precision, by its (mangled) name
    unsigned nf = 0;
    if ((r = cuModuleGetFunctionCount(&nf, mod))) return die("cuModuleGetFunctionCount", r);
    std::vector<CUfunction> fs(nf);
    if (nf && (r = cuModuleEnumerateFunctions(fs.data(), nf, mod))) return die("cuModuleEnumerateFunctions", r);
    const char* want = in.elem == 8 ? "15calculateKernelIdE" : "15calculateKernelIfE";
    CUfunction fn = nullptr;
    for (CUfunction f : fs) {
        const char* name = nullptr;
        if (!cuFuncGetName(&name, f) && name && std::strstr(name, want)) fn = f;
    }
    if (!fn) return die("calculateKernel instantiation not found in the cubin");
    // __constant__ data (physics.hpp:114-119), with the sizes checked
    struct Sym {
        const char* name;
        const std::vector<unsigned char>* src;
        const void* raw;
        size_t bytes;
    } syms[4] = {
        {"_ZN9cudaprob37physics15mix_data_deviceE", &in.mix, nullptr, 0},
        {"_ZN9cudaprob37physics17A_X_factor_deviceE", &in.axfac, nullptr, 0},
        {"_ZN9cudaprob37physics16mass_data_deviceE", &in.mass, nullptr, 0},
        {"_ZN9cudaprob37physics17mass_order_deviceE", nullptr, in.order, sizeof in.order},
    };
    for (Sym& s : syms) {
        CUdeviceptr p;
        size_t have = 0;
        if ((r = cuModuleGetGlobal(&p, &have, mod, s.name))) return die(s.name, r);
        const void* src = s.src ? (const void*)s.src->data() : s.raw;
        const size_t n = s.src ? s.src->size() : s.bytes;
        if (n > have) return die("constant larger than its symbol");
        if ((r = cuMemcpyHtoD(p, src, n))) return die("cuMemcpyHtoD(constant)", r);
    }
    // device arrays (cudapropagator.cuh:73-79, 132-159, 184-188): density rows
    // allocated 2n+1 and n of them copied, as the reference does
    const size_t e = in.elem;
    const size_t plane = (size_t)in.n_cos * in.n_en;
    CUdeviceptr d_cos, d_en, d_radii, d_rhos, d_maxl, d_out;
    if ((r = cuMemAlloc(&d_cos, e * in.n_cos)) || (r = cuMemAlloc(&d_en, e * in.n_en)) ||
        (r = cuMemAlloc(&d_radii, e * (2 * in.n_rows + 1))) || (r = cuMemAlloc(&d_rhos, e * (2 * in.n_rows + 1))) ||
        (r = cuMemAlloc(&d_maxl, sizeof(int32_t) * in.n_cos)) || (r = cuMemAlloc(&d_out, e * 9 * plane)))
        return die("cuMemAlloc", r);
    if ((r = cuMemsetD8(d_radii, 0, e * (2 * in.n_rows + 1))) || (r = cuMemsetD8(d_rhos, 0, e * (2 * in.n_rows + 1))) ||
        (r = cuMemcpyHtoD(d_cos, in.cos.data(), in.cos.size())) || (r = cuMemcpyHtoD(d_en, in.en.data(), in.en.size())) ||
        (r = cuMemcpyHtoD(d_radii, in.radii.data(), in.radii.size())) ||
        (r = cuMemcpyHtoD(d_rhos, in.rhos.data(), in.rhos.size())) ||
        (r = cuMemcpyHtoD(d_maxl, in.maxl.data(), sizeof(int32_t) * in.n_cos)))
        return die("cuMemcpyHtoD", r);
    // kernel arguments: (NeutrinoType, cos, n_cos, en, n_en, radii, rhos, maxlayers, height, result)
    int32_t type = in.type;
    int32_t nc = in.n_cos, ne = in.n_en;
    double h64 = 0.0;
    float h32 = 0.0f;
    if (e == 8)
        std::memcpy(&h64, in.height.data(), 8);
    else
        std::memcpy(&h32, in.height.data(), 4);
    void* args[10] = {&type, &d_cos, &nc, &d_en, &ne, &d_radii, &d_rhos, &d_maxl,
                      e == 8 ? (void*)&h64 : (void*)&h32, &d_out};
    const unsigned blocks = (unsigned)(((in.n_en + 63) / 64) * (size_t)in.n_cos);
    CUevent a, b;
    if ((r = cuEventCreate(&a, CU_EVENT_DEFAULT)) || (r = cuEventCreate(&b, CU_EVENT_DEFAULT)))
        return die("cuEventCreate", r);
    std::vector<float> ms;
    for (int k = 0; k < reps + 1; k++) {  // the first launch is a warm-up
        if ((r = cuEventRecord(a, 0))) return die("cuEventRecord", r);
        if ((r = cuLaunchKernel(fn, blocks, 1, 1, 64, 1, 1, 0, 0, args, nullptr))) return die("cuLaunchKernel", r);
        if ((r = cuEventRecord(b, 0))) return die("cuEventRecord", r);
        if ((r = cuEventSynchronize(b))) return die("kernel", r);
        float t = 0;
        if ((r = cuEventElapsedTime(&t, a, b))) return die("cuEventElapsedTime", r);
        if (k > 0) ms.push_back(t);
    }
    // strided subset of the planes, as doubles
    std::vector<unsigned char> host(e * 9 * plane);
    if ((r = cuMemcpyDtoH(host.data(), d_out, host.size()))) return die("cuMemcpyDtoH", r);
    const int sc = (in.n_cos + stride - 1) / stride, se = (in.n_en + stride - 1) / stride;
    std::vector<double> sub((size_t)9 * sc * se);
    for (int t = 0; t < 9; t++)
        for (int i = 0; i < sc; i++)
            for (int j = 0; j < se; j++) {
                const size_t at = (size_t)t * plane + (size_t)(i * stride) * in.n_en + (size_t)j * stride;
                double v;
                if (e == 8) {
                    std::memcpy(&v, host.data() + at * 8, 8);
                } else {
                    float f;
                    std::memcpy(&f, host.data() + at * 4, 4);
                    v = f;
                }
                sub[((size_t)t * sc + i) * se + j] = v;
            }
    std::FILE* fo = std::fopen(argv[4], "wb");
    if (!fo || std::fwrite(sub.data(), sizeof(double), sub.size(), fo) != sub.size()) return die("subset file");
    std::fclose(fo);
    int regs = 0, local = 0;
    cuFuncGetAttribute(&regs, CU_FUNC_ATTRIBUTE_NUM_REGS, fn);
    cuFuncGetAttribute(&local, CU_FUNC_ATTRIBUTE_LOCAL_SIZE_BYTES, fn);
    std::vector<float> sorted = ms;
    std::sort(sorted.begin(), sorted.end());
    std::printf("{\"elem\": %d, \"type\": %d, \"n_cos\": %d, \"n_en\": %d, \"blocks\": %u, \"threads\": 64, "
                "\"median_ms\": %.6f, \"min_ms\": %.6f, \"registers\": %d, \"local_bytes\": %d, \"ms\": [",
                in.elem, in.type, in.n_cos, in.n_en, blocks, sorted[sorted.size() / 2], sorted[0], regs, local);
    for (size_t k = 0; k < ms.size(); k++) std::printf("%s%.6f", k ? ", " : "", ms[k]);
    std::printf("], \"subset\": [%d, %d, %d]}\n", 9, sc, se);
    cuMemFree(d_cos);
    cuMemFree(d_en);
    cuMemFree(d_radii);
    cuMemFree(d_rhos);
    cuMemFree(d_maxl);
    cuMemFree(d_out);
    cuModuleUnload(mod);
    cuDevicePrimaryCtxRelease(dev);
    return 0;
}
