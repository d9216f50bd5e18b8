// Zhang-Shu positivity limiter on a point cloud (limiter_zhang_shu!,
// src/callbacks_stage/positivity_zhang_shu_point2d.jl:22-82), one variable pass as two
// kernels: the first computes every node's limited state from the unlimited field
// (zero where no limiting is needed), the second writes the non-zero results back, so
// that every node reads its neighbours before any of them changes (as the reference's
// separate local_u array does).
#include "mft_device.cuh"

namespace mft {
namespace {

using namespace dev;

// Base.min on Float64: NaN propagates, -0.0 < 0.0.
static __device__ __forceinline__ double jl_min(double a, double b) {
  if (isnan(a) || isnan(b)) return a + b;
  const bool b_less = b < a || (b == a && signbit(b) && !signbit(a));
  return b_less ? b : a;
}

// Trixi's density(u) / pressure(u) for CompressibleEulerEquations2D, each operation
// rounded separately.
static __device__ __forceinline__ double zs_variable(int variable, double g, const double* uu) {
  if (variable == 0) return uu[0];
  const double q = dmul(0.5, dadd(dmul(uu[1], uu[1]), dmul(uu[2], uu[2])));
  return dmul(dsub(g, 1.0), dsub(uu[3], ddiv(q, uu[0])));
}

__global__ void __launch_bounds__(kBlock) k_zs_limit(int64_t n, EllView ell, const double* u,
                                                    int variable, double threshold, double g,
                                                    double* loc) {
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  if (r >= n) return;
  const int64_t i = ell_node(ell, r);
  const int64_t base = ell.slice_off[r >> 5] + (r & 31);
  const int len = ell.row_len[r];
  double vmin = INFINITY;
  for (int j = 0; j < len; ++j) {
    const int64_t c = __ldg(ell.col + base + ((int64_t)j << 5));
    const double2* p = reinterpret_cast<const double2*>(u) + c * 2;
    const double2 a = __ldg(p), b = __ldg(p + 1);
    const double uu[4] = {a.x, a.y, b.x, b.y};
    vmin = jl_min(vmin, zs_variable(variable, g, uu));
  }
  double o[4] = {0.0, 0.0, 0.0, 0.0};
  if (vmin < threshold) {
    double mean[4] = {0.0, 0.0, 0.0, 0.0};
    for (int j = 0; j < len; ++j) {
      const int64_t c = __ldg(ell.col + base + ((int64_t)j << 5));
#pragma unroll
      for (int v = 0; v < 4; ++v) mean[v] = dadd(mean[v], u[c * 4 + v]);
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) mean[v] = ddiv(mean[v], (double)len);
    const double vmean = zs_variable(variable, g, mean);
    const double theta = ddiv(dsub(vmean, threshold), dsub(vmean, vmin));
#pragma unroll
    for (int v = 0; v < 4; ++v) o[v] = fma(theta, u[i * 4 + v], dmul(dsub(1.0, theta), mean[v]));
  }
  double2* q = reinterpret_cast<double2*>(loc) + i * 2;
  q[0] = make_double2(o[0], o[1]);
  q[1] = make_double2(o[2], o[3]);
}

__global__ void k_zs_apply(int64_t n, const double* loc, double* u, float* u32) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2* p = reinterpret_cast<const double2*>(loc) + i * 2;
  const double2 a = p[0], b = p[1];
  if (a.x == 0.0 && a.y == 0.0 && b.x == 0.0 && b.y == 0.0) return;
  double2* q = reinterpret_cast<double2*>(u) + i * 2;
  q[0] = a;
  q[1] = b;
  if (u32) {
    u32[i * 4 + 0] = (float)a.x;
    u32[i * 4 + 1] = (float)a.y;
    u32[i * 4 + 2] = (float)b.x;
    u32[i * 4 + 3] = (float)b.y;
  }
}

}  // namespace

void launch_zs_limiter(int64_t n, EllView ell, int variable, double threshold, double gamma,
                       double* u, float* u32, double* loc, cudaStream_t s) {
  if (n <= 0) return;
  const unsigned g = (unsigned)((n + kBlock - 1) / kBlock);
  k_zs_limit<<<g, kBlock, 0, s>>>(n, ell, u, variable, threshold, gamma, loc);
  MFT_LAUNCH_CHECK();
  k_zs_apply<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, loc, u, u32);
  MFT_LAUNCH_CHECK();
}

}  // namespace mft
