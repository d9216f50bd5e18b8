// rhs! on 3D point clouds: the plain flux divergence of calc_fluxes!
// (src/solvers/pointcloudsolver/rbfsolver.jl:247-265) over the three gradient operators of
// compute_flux_operator (compute_operators.jl:500-546), FP64, fused with the strong-BC pass
// 2 and the SSP-RK stage combination (finish_node).  CompressibleEulerEquations3D (5
// variables, fluxes formed once per node and gathered) and scalar advection (the flux a_d u
// formed at the neighbour).  The sliced-ELL layout and its row order are those of the 2D
// kernels.
#include <cuda_runtime.h>

#include <mutex>
#include <set>

#include "mft_device.cuh"
#include "mft_dw.cuh"
#include "mft_halo.cuh"
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

// Double-word form: the state split into pairs and the flux formed in double-word
// arithmetic (one reciprocal of rho refined by a Newton step).  The momentum flux is
// symmetric, so the 15 flux components hold 12 distinct values, each formed once and
// stored as one pair: F[i] = 6 float4 =
//   (m1, m2), (m3, m1 v1 + p), (m2 v2 + p, m3 v3 + p), (m1 v2, m1 v3), (m2 v3, (E+p) v1),
//   ((E+p) v2, (E+p) v3)
// (96 bytes), and F_x = (m1, m1 v1 + p, m1 v2, m1 v3, (E+p) v1), F_y = (m2, m1 v2,
// m2 v2 + p, m2 v3, (E+p) v2), F_z = (m3, m1 v3, m2 v3, m3 v3 + p, (E+p) v3).  The only
// FP64 operations are the five splits.
__global__ void k_prep_euler3d_dw(int64_t n, float2 gm1, const double* __restrict__ u,
                                  float4* __restrict__ F) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* ui = u + i * 5;
  const float2 rho = dw::split(ui[0]), en = dw::split(ui[4]);
  const float2 m[3] = {dw::split(ui[1]), dw::split(ui[2]), dw::split(ui[3])};
  const float2 r = dw::recip(rho);
  const float2 v[3] = {dw::mul(m[0], r), dw::mul(m[1], r), dw::mul(m[2], r)};
  const float2 mv = dw::add(dw::add(dw::mul(m[0], v[0]), dw::mul(m[1], v[1])), dw::mul(m[2], v[2]));
  const float2 p = dw::mul(gm1, dw::add(en, dw::neg(dw::scale2(mv, 0.5f))));
  const float2 ep = dw::add(en, p);
  const float2 xx = dw::add(dw::mul(m[0], v[0]), p), yy = dw::add(dw::mul(m[1], v[1]), p);
  const float2 zz = dw::add(dw::mul(m[2], v[2]), p);
  const float2 xy = dw::mul(m[0], v[1]), xz = dw::mul(m[0], v[2]), yz = dw::mul(m[1], v[2]);
  const float2 ex = dw::mul(ep, v[0]), ey = dw::mul(ep, v[1]), ez = dw::mul(ep, v[2]);
  float4* Fi = F + i * 6;
  Fi[0] = make_float4(m[0].x, m[0].y, m[1].x, m[1].y);
  Fi[1] = make_float4(m[2].x, m[2].y, xx.x, xx.y);
  Fi[2] = make_float4(yy.x, yy.y, zz.x, zz.y);
  Fi[3] = make_float4(xy.x, xy.y, xz.x, xz.y);
  Fi[4] = make_float4(yz.x, yz.y, ex.x, ex.y);
  Fi[5] = make_float4(ey.x, ey.y, ez.x, ez.y);
}

static __device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
static __device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }

// One stencil entry: the three weight pairs against the record's 15 flux components.
static __device__ __forceinline__ void accum3(dw::Acc* f, const float2* w, const float4* q) {
  const float2 m1 = lo2(q[0]), m2 = hi2(q[0]), m3 = lo2(q[1]), xx = hi2(q[1]);
  const float2 yy = lo2(q[2]), zz = hi2(q[2]), xy = lo2(q[3]), xz = hi2(q[3]);
  const float2 yz = lo2(q[4]), ex = hi2(q[4]), ey = lo2(q[5]), ez = hi2(q[5]);
  const float2 fx[5] = {m1, xx, xy, xz, ex};
  const float2 fy[5] = {m2, xy, yy, yz, ey};
  const float2 fz[5] = {m3, xz, yz, zz, ez};
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    dw::fma_acc(f[v], w[0], fx[v]);
    dw::fma_acc(f[v], w[1], fy[v]);
    dw::fma_acc(f[v], w[2], fz[v]);
  }
}

// du_i = -sum_j (Dx_ij F_x + Dy_ij F_y + Dz_ij F_z)(node j) as compensated sums of
// double-word products (mft_dw.cuh), the stage epilogue in FP64.  Per stencil entry: three
// weight pairs and the neighbour's 96-byte flux record.  HALO: one block per row group
// (ell.halo_rows rows) first stages the group's neighbour records in shared memory (six
// 16-byte chunks each, mft_halo.cuh) and reads them from there; a group without a list
// gathers directly.  Both read the same records in the same order: the same sums.
template <bool HALO>
__global__ void __launch_bounds__(HALO ? kHaloRows : kBlock) k_fwd3_dw(FwdArgs a) {
  const int64_t r = blockIdx.x * (int64_t)(HALO ? (int)blockDim.x : kBlock) + threadIdx.x;
  const float4* __restrict__ F4 = reinterpret_cast<const float4*>(a.Fdw);
  extern __shared__ float4 hsm3[];
  bool staged = false;
  if (HALO) staged = stage_halo<6>(a.ell, hsm3, [&](int k, int64_t c) { return F4 + c * 6 + k; });
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  const int hs = a.ell.halo_stride;
  dw::Acc f[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) f[v] = dw::zero();
  if (HALO && staged) {
    const uint16_t* __restrict__ lcol = a.ell.lcol;
#pragma unroll 2
    for (int j = 0; j < len; ++j) {
      const int64_t p = base + ((int64_t)j << 5);
      const int lc = __ldg(lcol + p);
      const float2 w[3] = {__ldg(a.wdw[0] + p), __ldg(a.wdw[1] + p), __ldg(a.wdw[2] + p)};
      float4 q[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) q[k] = hsm3[k * hs + lc];
      accum3(f, w, q);
    }
  } else {
    const int32_t* __restrict__ col = a.ell.col;
#pragma unroll 2
    for (int j = 0; j < len; ++j) {
      const int64_t p = base + ((int64_t)j << 5);
      const int64_t c = __ldg(col + p);
      const float2 w[3] = {__ldg(a.wdw[0] + p), __ldg(a.wdw[1] + p), __ldg(a.wdw[2] + p)};
      float4 q[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) q[k] = __ldg(F4 + c * 6 + k);
      accum3(f, w, q);
    }
  }
  double du[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) du[v] = -dw::to_double(f[v]);
  finish_node<5>(a.ep, i, du);
}

}  // namespace

void launch_prep_euler3d_dw(int64_t n, double gamma, const double* u, float2* F,
                            cudaStream_t s) {
  if (n <= 0) return;
  const double gm1 = gamma - 1.0;
  const float h = (float)gm1;
  const float2 g2 = make_float2(h, (float)(gm1 - (double)h));
  k_prep_euler3d_dw<<<grid_for(n, 256), 256, 0, s>>>(n, g2, u, reinterpret_cast<float4*>(F));
  MFT_LAUNCH_CHECK();
}

void launch_fwd3_dw(const FwdArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  MFT_REQUIRE(a.V == 5 && a.Fdw && a.wdw[0] && a.wdw[1] && a.wdw[2] && a.final_epilogue,
              MFT_ERR_STATE, "double-word 3D gather: arguments not set");
  if (a.ell.halo_off && a.ell.halo_rows > 0) {
    // one block per row group, six chunks of the longest list in dynamic shared memory
    // (above 48 KB a per-kernel opt-in, made once per device)
    const size_t smem = (size_t)6 * a.ell.halo_stride * sizeof(float4);
    if (smem > 48 * 1024) {
      static std::mutex mu;
      static std::set<int> done;
      int dev = 0;
      MFT_CUDA(cudaGetDevice(&dev));
      std::lock_guard<std::mutex> lock(mu);
      if (done.insert(dev).second)
        MFT_CUDA(cudaFuncSetAttribute(k_fwd3_dw<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(6 * kHaloMax * sizeof(float4))));
    }
    const int rows = a.ell.halo_rows;
    k_fwd3_dw<true><<<grid_for(a.n, rows), rows, smem, s>>>(a);
  } else {
    k_fwd3_dw<false><<<grid_for(a.n, kBlock), kBlock, 0, s>>>(a);
  }
  MFT_LAUNCH_CHECK();
}

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
