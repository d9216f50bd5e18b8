// rhs! on 3D point clouds: the plain flux divergence of calc_fluxes!
// (src/solvers/pointcloudsolver/rbfsolver.jl:247-265) over the three gradient operators of
// compute_flux_operator (compute_operators.jl:500-546), FP64, fused with the strong-BC pass
// 2 and the SSP-RK stage combination (finish_node).  CompressibleEulerEquations3D (5
// variables, fluxes formed once per node and gathered) and scalar advection (the flux a_d u
// formed at the neighbour).  The sliced-ELL layout and its row order are those of the 2D
// kernels.
#include <cuda_runtime.h>

#include "mft_device.cuh"
#include "mft_internal.cuh"

namespace mft {

namespace {

using namespace dev;

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

// F[i] = (F_x, F_y, F_z), each the 5 components (rho v_d, rho v v_d + p e_d, (E + p) v_d):
// the textbook flux with one reciprocal of rho for the three velocities.
__global__ void k_flux_euler3d(int64_t n, double g, const double* __restrict__ u,
                               double* __restrict__ F) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* ui = u + i * 5;
  const double rho = ui[0], m1 = ui[1], m2 = ui[2], m3 = ui[3], en = ui[4];
  const double rinv = ddiv(1.0, rho);
  const double v1 = dmul(m1, rinv), v2 = dmul(m2, rinv), v3 = dmul(m3, rinv);
  const double p = dmul(dsub(g, 1.0),
                        dsub(en, dmul(0.5, dadd(dadd(dmul(m1, v1), dmul(m2, v2)), dmul(m3, v3)))));
  const double ep = dadd(en, p);
  const double m[3] = {m1, m2, m3}, v[3] = {v1, v2, v3};
  double* Fi = F + i * 15;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    Fi[d * 5 + 0] = m[d];
    Fi[d * 5 + 1] = d == 0 ? dadd(dmul(m[d], v1), p) : dmul(m[d], v1);
    Fi[d * 5 + 2] = d == 1 ? dadd(dmul(m[d], v2), p) : dmul(m[d], v2);
    Fi[d * 5 + 3] = d == 2 ? dadd(dmul(m[d], v3), p) : dmul(m[d], v3);
    Fi[d * 5 + 4] = dmul(ep, v[d]);
  }
}

// du_i = -sum_j (Dx_ij F_x + Dy_ij F_y + Dz_ij F_z)(node j), one node per thread over the
// sliced ELL (lane r of a warp owns row 32 s + r of slice s), then finish_node.
template <int V>
__global__ void __launch_bounds__(kBlock) k_fwd3_f64(FwdArgs a) {
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  const int32_t* __restrict__ col = a.ell.col;
  const double* __restrict__ wx = a.w[0];
  const double* __restrict__ wy = a.w[1];
  const double* __restrict__ wz = a.w[2];
  double f[V];
#pragma unroll
  for (int v = 0; v < V; ++v) f[v] = 0.0;
#pragma unroll 2
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int64_t c = __ldg(col + p);
    const double x = __ldg(wx + p), y = __ldg(wy + p), z = __ldg(wz + p);
    if constexpr (V == 5) {
      const double* Fc = a.F + c * 15;
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        f[v] = fma(x, __ldg(Fc + v), f[v]);
        f[v] = fma(y, __ldg(Fc + 5 + v), f[v]);
        f[v] = fma(z, __ldg(Fc + 10 + v), f[v]);
      }
    } else {
      const double uc = __ldg(a.u + c);
      f[0] = fma(x, dmul(a.ax, uc), f[0]);
      f[0] = fma(y, dmul(a.ay, uc), f[0]);
      f[0] = fma(z, dmul(a.az, uc), f[0]);
    }
  }
  double du[V];
#pragma unroll
  for (int v = 0; v < V; ++v) du[v] = -f[v];
  finish_node<V>(a.ep, i, du);
}

}  // namespace

void launch_flux_euler3d(int64_t n, double gamma, const double* u, double* F, cudaStream_t s) {
  if (n <= 0) return;
  k_flux_euler3d<<<grid_for(n, 256), 256, 0, s>>>(n, gamma, u, F);
  MFT_LAUNCH_CHECK();
}

void launch_fwd3(const FwdArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  MFT_REQUIRE(a.w[0] && a.w[1] && a.w[2], MFT_ERR_STATE, "3D gradient operators not set");
  MFT_REQUIRE(a.final_epilogue, MFT_ERR_UNSUPPORTED, "3D gather: final epilogue only");
  const unsigned g = grid_for(a.n, kBlock);
  if (a.V == 5) {
    MFT_REQUIRE(a.F, MFT_ERR_STATE, "3D Euler fluxes not formed");
    k_fwd3_f64<5><<<g, kBlock, 0, s>>>(a);
  } else if (a.V == 1) {
    k_fwd3_f64<1><<<g, kBlock, 0, s>>>(a);
  } else {
    throw Error(MFT_ERR_UNSUPPORTED, "3D gather: 5 (Euler) or 1 (advection) variables");
  }
  MFT_LAUNCH_CHECK();
}

}  // namespace mft
