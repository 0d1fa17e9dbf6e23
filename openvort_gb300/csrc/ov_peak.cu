// ov_peak.cu - FMA-pipe calibration: the roofline denominator of the
// traversal kernels (FP64 for the bit-faithful path, FP32 for the mixed one).
// Eight independent multiply-add chains per thread, every SM fully occupied;
// 2 flops per FMA.
#include "ov_internal.cuh"

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_chain(T *out, int iters, T a, T b)
{
    T x[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = (T)(threadIdx.x + i);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
    }
    T s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += x[i];
    if (s == (T)1.2345) out[0] = s;   // keeps the chains alive
}

}  // namespace

extern "C" int ov_measure_fma_peak(ov_ctx *c, int precision, double *tflops)
{
    if (!c || !tflops) return OV_ERR_ARG;
    cudaSetDevice(c->device);
    int sms = 0;
    OV_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    int blocks = sms * 8, threads = 256;
    int iters = precision == OV_PREC_FP64 ? 2048 : 32768;
    void *buf = nullptr;
    OV_ALLOC(c, cudaMalloc(&buf, 64));
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        OV_CUDA(c, cudaEventRecord(c->ev0, c->stream));
        if (precision == OV_PREC_FP64)
            k_fma_chain<double><<<blocks, threads, 0, c->stream>>>((double *)buf, iters, 0.999999, 1e-7);
        else
            k_fma_chain<float><<<blocks, threads, 0, c->stream>>>((float *)buf, iters, 0.999999f, 1e-7f);
        c->launches++;
        OV_CUDA(c, cudaEventRecord(c->ev1, c->stream));
        OV_CUDA(c, cudaEventSynchronize(c->ev1));
        float ms = 0;
        OV_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        if (rep > 0) best = ms < best ? ms : best;
    }
    cudaFree(buf);
    double flops = 2.0 * 8.0 * (double)iters * (double)blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return OV_OK;
}
