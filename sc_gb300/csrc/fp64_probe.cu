// fp64_probe.cu -- this GPU's FP64 rates, measured with the library's own kernels.
//
// The move kernel's exact stage is scalar FP64 (add, multiply, divide, square root: the
// reference's operation order, no contraction).  Its roofline denominator is therefore the
// FP64 instruction rate of the GPU it runs on, which this probe measures: a throughput
// kernel (every SM full of warps, eight independent multiply-add chains per thread, as
// separate DMUL and DADD instructions), the same with one active lane per warp (the cost of
// an FP64 warp instruction whatever its active lanes), fused DFMA chains (the FP64 peak as
// usually quoted, 2 FLOP per FMA), and a single dependent chain timed with clock64 (the
// latency of one FP64 operation).

#include <cuda_runtime.h>

#include "../../include/sc_gb300.h"
#include "sc_context.h"

namespace scg {
namespace {

constexpr int kChains = 8;

template <bool ONE_LANE>
__global__ void __launch_bounds__(256) kFp64MulAdd(double* out, int iters, double a, double b) {
    if (ONE_LANE && (threadIdx.x & 31)) return;
    double x[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) x[k] = 1.0 + 1e-3 * k + 1e-9 * threadIdx.x;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) x[k] = __dadd_rn(__dmul_rn(x[k], a), b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) kFp64Fma(double* out, int iters, double a, double b) {
    double x[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) x[k] = 1.0 + 1e-3 * k + 1e-9 * threadIdx.x;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) x[k] = __fma_rn(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void kFp64Latency(double* out, long long* cycles, int iters, double a, double b) {
    double x = 1.0 + 1e-9 * threadIdx.x;
    long long t0 = clock64();
    for (int i = 0; i < iters; ++i) x = __dadd_rn(__dmul_rn(x, a), b);
    long long t1 = clock64();
    out[0] = x;
    cycles[0] = t1 - t0;
}

}  // namespace
}  // namespace scg

using namespace scg;

extern "C" int sc_fp64_rates(int device, double* dmul_dadd_per_s, double* one_lane_per_s, double* fma_flops,
                             double* latency_cycles) {
    DeviceScope dev(device);
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cudaFail(e, "cudaSetDevice");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int threads = 256, blocks = sms * 8, iters = 2048;
    double* out = nullptr;
    long long* cyc = nullptr;
    if ((e = cudaMalloc(&out, sizeof(double) * (size_t)blocks * threads)) != cudaSuccess) return cudaFail(e, "cudaMalloc");
    if ((e = cudaMalloc(&cyc, sizeof(long long))) != cudaSuccess) { cudaFree(out); return cudaFail(e, "cudaMalloc"); }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const double a = 0.9999999, b = 1e-7;
    auto timeIt = [&](auto launch) {
        launch();                                   // warm-up
        float best = 1e30f;
        for (int r = 0; r < 3; ++r) {
            cudaEventRecord(e0);
            launch();
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) best = ms;
        }
        return 1e-3 * best;
    };
    const double ops = (double)blocks * threads * iters * kChains * 2.0;
    double t = timeIt([&] { kFp64MulAdd<false><<<blocks, threads>>>(out, iters, a, b); });
    if (dmul_dadd_per_s) *dmul_dadd_per_s = ops / t;
    t = timeIt([&] { kFp64MulAdd<true><<<blocks, threads>>>(out, iters, a, b); });
    if (one_lane_per_s) *one_lane_per_s = ops / 32.0 / t;
    t = timeIt([&] { kFp64Fma<<<blocks, threads>>>(out, iters, a, b); });
    if (fma_flops) *fma_flops = ops / t;            // kChains FMAs of 2 FLOP per iteration
    kFp64Latency<<<1, 1>>>(out, cyc, 4096, a, b);
    long long c = 0;
    e = cudaMemcpy(&c, cyc, sizeof c, cudaMemcpyDeviceToHost);
    if (latency_cycles) *latency_cycles = (double)c / (2.0 * 4096);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    cudaFree(cyc);
    if (e != cudaSuccess) return cudaFail(e, "FP64 probe");
    e = cudaGetLastError();
    return e == cudaSuccess ? SC_OK : cudaFail(e, "FP64 probe");
}
