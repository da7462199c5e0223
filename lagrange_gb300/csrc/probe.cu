// fwn_probe_fp32_peak: the device's FP32 fused-multiply-add throughput, measured with a short
// throughput kernel. The traversal kernels are bound by FP32 issue, not by HBM or tensor cores,
// so their roofline needs this figure; measuring it in the same process (same clocks, same power
// state) keeps the denominator reproducible instead of a nominal SM-count x clock product.
//
// Every thread of a full-occupancy grid runs independent FMA chains (enough of them to cover the
// pipe latency), with the multiplier and addend passed at run time so nothing folds. Form 0 uses
// scalar fma.rn.f32; form 1 the paired fma.rn.f32x2 (two lanes' worth of FMAs per instruction on
// one 64-bit register pair). Both count an FMA as 2 flops.
#include <algorithm>
#include <string>
#include <vector>

#include "fwn_internal.cuh"

namespace fwn {
namespace {

constexpr int kProbeBlock = 256;
constexpr int kProbeChains = 8;  // independent chains per thread (scalar) / packed pairs (form 1)

__device__ __forceinline__ unsigned long long pack2(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}

__device__ __forceinline__ void unpack2(unsigned long long v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

__global__ void __launch_bounds__(kProbeBlock)
k_fma_scalar(float a, float b, int iters, float* __restrict__ sink) {
    float x[kProbeChains];
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) x[c] = (float)(threadIdx.x + c) * 1e-3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kProbeChains; ++c) x[c] = fmaf(x[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) s += x[c];
    if (s == -1.2345f) *sink = s;  // never true for these inputs; keeps the chains live
}

__global__ void __launch_bounds__(kProbeBlock)
k_fma_paired(float a, float b, int iters, float* __restrict__ sink) {
    unsigned long long x[kProbeChains];
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c)
        x[c] = pack2((float)(threadIdx.x + c) * 1e-3f, (float)(threadIdx.x + 2 * c) * 1e-3f);
    const unsigned long long aa = pack2(a, a), bb = pack2(b, b);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kProbeChains; ++c)
            asm("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[c]) : "l"(aa), "l"(bb));
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) {
        float lo, hi;
        unpack2(x[c], lo, hi);
        s += lo + hi;
    }
    if (s == -1.2345f) *sink = s;
}

}  // namespace
}  // namespace fwn

using namespace fwn;

extern "C" FWN_API fwn_status fwn_probe_fp32_peak(int32_t form, double* flops, double* ms,
                                                  void* stream) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float* sink = nullptr;
    auto release = [&]() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (sink) cudaFree(sink);
    };
    try {
        if (form != 0 && form != 1) throw Error(FWN_INVALID_ARG, "form must be 0 (f32) or 1 (f32x2)");
        if (!flops || !ms) throw Error(FWN_INVALID_ARG, "null output pointer");
        const cudaStream_t st = static_cast<cudaStream_t>(stream);
        int dev = 0, sms = 0, per_sm = 0;
        FWN_CUDA_CHECK(cudaGetDevice(&dev));
        FWN_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        auto kern = form == 0 ? k_fma_scalar : k_fma_paired;
        FWN_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kProbeBlock, 0));
        const unsigned grid = (unsigned)(sms * std::max(per_sm, 1));
        constexpr int kIters = 8192;
        FWN_CUDA_CHECK(cudaMalloc(&sink, sizeof(float)));
        FWN_CUDA_CHECK(cudaEventCreate(&e0));
        FWN_CUDA_CHECK(cudaEventCreate(&e1));
        const float a = 0.9999999f, b = 1e-7f;
        for (int w = 0; w < 2; ++w) kern<<<grid, kProbeBlock, 0, st>>>(a, b, kIters, sink);
        FWN_CUDA_CHECK(cudaGetLastError());
        std::vector<float> t;
        for (int r = 0; r < 5; ++r) {
            FWN_CUDA_CHECK(cudaEventRecord(e0, st));
            kern<<<grid, kProbeBlock, 0, st>>>(a, b, kIters, sink);
            FWN_CUDA_CHECK(cudaEventRecord(e1, st));
            FWN_CUDA_CHECK(cudaEventSynchronize(e1));
            float m = 0.f;
            FWN_CUDA_CHECK(cudaEventElapsedTime(&m, e0, e1));
            t.push_back(m);
        }
        FWN_CUDA_CHECK(cudaGetLastError());
        std::sort(t.begin(), t.end());
        const double fmas_per_thread = (double)kIters * kProbeChains * (form == 0 ? 1 : 2);
        *flops = 2.0 * fmas_per_thread * (double)grid * kProbeBlock;
        *ms = t[t.size() / 2];
        release();
        return FWN_OK;
    } catch (const Error& err) {
        release();
        set_last_error(err.what());
        return err.status;
    } catch (const std::exception& err) {
        release();
        set_last_error(err.what());
        return FWN_INTERNAL;
    }
}
