// Arithmetic peak of the current GPU, measured: the denominator of the roofline of kernels bound by
// the FP64 (or FP32) pipe rather than by HBM -- the element integration, the FP64 residuals and the
// patch fits.  A register-resident kernel runs 8 independent fused multiply-add chains per thread on
// every SM (8 CTAs of 256 threads per SM), long enough (tens of milliseconds) for the launch to be
// negligible; CUDA events on a private stream time it after one warm-up launch.
#include <algorithm>

#include "amr_internal.h"

namespace {

constexpr int kChains = 8;

// x <- x * a + c on each chain; a < 1 keeps the chains bounded.  The result is stored only if it equals
// a value it never takes, so the work stays and no memory traffic enters the timing.
template <class V>
__global__ void __launch_bounds__(256) k_fma_peak(int iters, V a, V c, V *sink) {
    V x[kChains];
#pragma unroll
    for (int i = 0; i < kChains; i++) x[i] = (V)(threadIdx.x + i);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < kChains; i++) x[i] = fma(x[i], a, c);
    }
    V s = V(0);
#pragma unroll
    for (int i = 0; i < kChains; i++) s += x[i];
    if (s == V(-1)) *sink = s;
}

template <class V>
double measure(int iters) {
    int dev = 0, sms = 0;
    AMR_CUDA(cudaGetDevice(&dev));
    AMR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned grid = (unsigned)sms * 8, threads = 256;
    V *sink = nullptr;
    amr_alloc(&sink, 1);
    cudaStream_t s = nullptr;
    AmrEventPair ev;
    double sec = 0.0;
    try {
        AMR_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        k_fma_peak<V><<<grid, threads, 0, s>>>(iters / 8, (V)0.999999, (V)1e-6, sink);  // warm-up
        AMR_CUDA(cudaEventRecord(ev.t0, s));
        k_fma_peak<V><<<grid, threads, 0, s>>>(iters, (V)0.999999, (V)1e-6, sink);
        AMR_CUDA(cudaEventRecord(ev.t1, s));
        AMR_COUNT(2);
        AMR_CUDA(cudaEventSynchronize(ev.t1));
        float ms = 0.f;
        AMR_CUDA(cudaEventElapsedTime(&ms, ev.t0, ev.t1));
        sec = ms * 1e-3;
    } catch (...) {
        if (s) cudaStreamDestroy(s);
        amr_free(sink);
        throw;
    }
    cudaStreamDestroy(s);
    amr_free(sink);
    const double flops = 2.0 * kChains * (double)iters * grid * threads;
    return flops / sec / 1e12;
}

}  // namespace

extern "C" int amr_measure_peak(int32_t which, double *tflops) {
    if (!tflops) return AMR_EINVAL;
    try {
        if (which == AMR_PEAK_FP64_FMA) *tflops = measure<double>(1 << 12);
        else if (which == AMR_PEAK_FP32_FMA) *tflops = measure<float>(1 << 18);
        else return AMR_EINVAL;
        return AMR_OK;
    } catch (const AmrError &e) {
        return e.code;
    }
}
