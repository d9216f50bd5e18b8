// Throughput probe for the roofline denominators: FP64 FMA (DFMA), FP32 FMA and
// FP64->FP32 conversion rates of the current GPU, per SM per clock.
#include <cstdio>
#include <cuda_runtime.h>
template <int ILP>
__global__ void dfma_k(double* out, double a, double b, int iters) {
  double x[ILP];
  for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < ILP; ++i) x[i] = fma(x[i], a, b);
  }
  double s = 0; for (int i = 0; i < ILP; ++i) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
template <int ILP>
__global__ void ffma_k(float* out, float a, float b, int iters) {
  float x[ILP];
  for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 1e-3f + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < ILP; ++i) x[i] = fmaf(x[i], a, b);
  }
  float s = 0; for (int i = 0; i < ILP; ++i) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
// F2F.F32.F64: every iteration converts a different value (the last mantissa bit of each
// chain flips by an integer XOR, which no FP64 operation or hoisting can replace).
template <int ILP>
__global__ void cvt_k(float* out, double a, int iters) {
  double x[ILP]; float y[ILP];
  for (int i = 0; i < ILP; ++i) { x[i] = threadIdx.x * 1e-3 + i + a; y[i] = 0.f; }
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < ILP; ++i) {
      y[i] += __double2float_rn(x[i]);
      x[i] = __longlong_as_double(__double_as_longlong(x[i]) ^ 1ll);
    }
  }
  float s = 0; for (int i = 0; i < ILP; ++i) s += y[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
int main() {
  int dev = 0; cudaDeviceProp p; cudaGetDeviceProperties(&p, dev);
  int clk = 0; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, dev);
  printf("gpu %s sms %d clock_khz %d\n", p.name, p.multiProcessorCount, clk);
  const int blocks = p.multiProcessorCount * 8, threads = 256, iters = 4096;
  double* dout; float* fout;
  cudaMalloc(&dout, sizeof(double) * blocks * threads);
  cudaMalloc(&fout, sizeof(float) * blocks * threads);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  float ms;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0); dfma_k<16><<<blocks, threads>>>(dout, 0.999999, 1e-7, iters); cudaEventRecord(e1);
    cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    double ops = double(blocks) * threads * iters * 16;
    printf("DFMA: %.3f ms  %.1f GFMA/s  %.2f TFLOP/s  per-SM-per-clk(at %d MHz) %.2f\n", ms, ops / ms / 1e6, 2 * ops / ms / 1e9,
           clk / 1000, ops / (ms * 1e-3) / p.multiProcessorCount / (clk * 1e3));
    cudaEventRecord(e0); ffma_k<8><<<blocks, threads>>>(fout, 0.9999f, 1e-7f, iters * 8); cudaEventRecord(e1);
    cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    ops = double(blocks) * threads * iters * 8 * 8;
    printf("FFMA: %.3f ms  %.1f GFMA/s  %.2f TFLOP/s  per-SM-per-clk %.2f\n", ms, ops / ms / 1e6, 2 * ops / ms / 1e9,
           ops / (ms * 1e-3) / p.multiProcessorCount / (clk * 1e3));
    cudaEventRecord(e0); cvt_k<8><<<blocks, threads>>>(fout, 1e-9, iters); cudaEventRecord(e1);
    cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    ops = double(blocks) * threads * iters * 8;
    printf("F2F.F32.F64 (+FADD, LOP): %.3f ms  %.1f Gcvt/s per-SM-per-clk %.2f\n", ms, ops / ms / 1e6,
           ops / (ms * 1e-3) / p.multiProcessorCount / (clk * 1e3));
  }
  cudaError_t err = cudaDeviceSynchronize();
  printf("status %s\n", cudaGetErrorString(err));
  return err == cudaSuccess ? 0 : 1;
}
