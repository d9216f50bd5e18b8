// Arithmetic-rate probe of the current GPU: the denominators of the FP64-issue roofline
// that bench.py reports beside the HBM roofline (the FP64 form's gathers in FP64 fused
// multiply-adds are bound by the FP64 pipe, the double-word ones by FP32 issue).
#include <cuda_runtime.h>

#include "mft_ctx.h"

namespace mft {
namespace {

// ILP independent multiply-add chains per thread; the sum is stored so that nothing is
// dead code.
template <int ILP>
__global__ void k_rate_f64(double* out, double a, double b, int iters) {
  double x[ILP];
#pragma unroll
  for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < ILP; ++i) x[i] = fma(x[i], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < ILP; ++i) s += x[i];
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s;
}

template <int ILP>
__global__ void k_rate_f32(double* out, float a, float b, int iters) {
  float x[ILP];
#pragma unroll
  for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 1e-3f + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < ILP; ++i) x[i] = fmaf(x[i], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < ILP; ++i) s += x[i];
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s;
}

}  // namespace
}  // namespace mft

extern "C" mft_status mft_measure_fma_rate(mft_ctx* c, int kind, double* per_second) {
  using namespace mft;
  if (!c || !per_second || (kind != 0 && kind != 1)) return MFT_ERR_ARG;
  try {
    MFT_CUDA(cudaSetDevice(c->device));
    int sms = 0;
    MFT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    const int threads = 256, blocks = sms * 8;
    DBuf<double> out;
    out.alloc((size_t)blocks * threads);
    cudaEvent_t e0, e1;
    MFT_CUDA(cudaEventCreate(&e0));
    MFT_CUDA(cudaEventCreate(&e1));
    constexpr int kIlp64 = 16, kIlp32 = 8;
    const int iters = kind == 0 ? 2048 : 65536;
    const double ops = (double)blocks * threads * iters * (kind == 0 ? kIlp64 : kIlp32);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {  // the first launch is a warm-up
      MFT_CUDA(cudaEventRecord(e0, c->stream));
      if (kind == 0)
        k_rate_f64<kIlp64><<<blocks, threads, 0, c->stream>>>(out.p, 0.999999, 1e-7, iters);
      else
        k_rate_f32<kIlp32><<<blocks, threads, 0, c->stream>>>(out.p, 0.9999f, 1e-7f, iters);
      MFT_CUDA(cudaGetLastError());
      MFT_CUDA(cudaEventRecord(e1, c->stream));
      MFT_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      MFT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *per_second = ops / (best * 1e-3);
    return MFT_OK;
  } catch (const Error& e) {
    c->err = e.what();
    return e.code;
  }
}
