// Adjoint of rhs! on the device.
//
// rhs!(u) = M2 [ -sum_d D_d F_d(P u) - gamma H P u ] with P the strong-BC pass
// (Dirichlet values, slip-wall momentum projection; derivative Pi) and M2 the rows
// the second BC pass zeroes.  Its transpose product
//   r = Pi [ -sum_d J_Fd(P u)^T D_d^T (M2 lam) - gamma H^T (M2 lam) ]
// is one transpose-stencil gather over the reverse adjacency (the CSC view of the
// operator stored as a sliced ELL), fused with the flux-Jacobian-transpose product
// at the gathering node and with the SSP-RK3 adjoint stage combination.
#include "mft_device.cuh"
#include "mft_dw.cuh"
#include "mft_halo.cuh"

namespace mft {
namespace {

using namespace dev;

// M2 at node c: Dirichlet rows carry no cotangent, slip walls none in momentum.
template <int V>
static __device__ __forceinline__ void mask_rows(const BcDev& bc, int64_t c, double* l) {
  const int tag = bc.tag[c];
  if (tag == 1) {
#pragma unroll
    for (int v = 0; v < V; ++v) l[v] = 0.0;
  } else if (tag == 2) {
    if constexpr (V == 4) {
      l[1] = 0.0;
      l[2] = 0.0;
    }
  }
}

template <int V>
static __device__ __forceinline__ void load_row(const double* a, int64_t c, double* l) {
  if constexpr (V == 4) {
    const double2* p = reinterpret_cast<const double2*>(a) + c * 2;
    const double2 x = __ldg(p), y = __ldg(p + 1);
    l[0] = x.x; l[1] = x.y; l[2] = y.x; l[3] = y.y;
  } else {
#pragma unroll
    for (int v = 0; v < V; ++v) l[v] = __ldg(a + c * V + v);
  }
}

// Pi at node i on a cotangent row.
template <int V>
static __device__ __forceinline__ void project_row(const BcDev& bc, int64_t i, double* o) {
  const int tag = bc.tag[i];
  if (tag == 1) {
#pragma unroll
    for (int v = 0; v < V; ++v) o[v] = 0.0;
  } else if (tag == 2) {
    if constexpr (V == 4) slip(bc.normal + 2 * (int64_t)bc.slot[i], o);
  }
}

// The node part of the adjoint at node i from the gathered sums gx = Dx^T M2 lam,
// gy = Dy^T M2 lam and gh (the hyperviscosity term): flux-Jacobian-transpose product,
// the SSP-RK3 adjoint stage combination and the BC projection.
// gxp / gyp (double-word path): the gathered sums as pairs, from which the Jacobian product
// is formed in double-word arithmetic (gx / gy unused then).
template <int V, bool EULER, bool BC, int HV>
static __device__ __forceinline__ void adj_finish(const AdjArgs& a, int64_t i, const double* gx,
                                                  const double* gy, const double* gh,
                                                  const float2* gxp = nullptr,
                                                  const float2* gyp = nullptr) {
  double r[V];
  if constexpr (EULER) {
    double uu[4];
    load_row<4>(a.u, i, uu);
    if (BC && a.bc.tag[i] == 2) slip(a.bc.normal + 2 * (int64_t)a.bc.slot[i], uu);
    if (gxp) {
      const double gm1 = a.gamma - 1.0;
      const float2 g2 = dw::split(gm1);
      const float2 up[4] = {dw::split(uu[0]), dw::split(uu[1]), dw::split(uu[2]),
                            dw::split(uu[3])};
      float2 ub[4];
      dw::euler_flux_vjp(g2, up, gxp, gyp, ub);
#pragma unroll
      for (int v = 0; v < V; ++v) r[v] = -dw::value(ub[v]);
    } else {
      double ub[4];
      euler_flux_vjp(a.gamma, uu, gx, gy, ub);
#pragma unroll
      for (int v = 0; v < V; ++v) r[v] = -ub[v];
    }
  } else {
#pragma unroll
    for (int v = 0; v < V; ++v) r[v] = -(a.ax * gx[v] + a.ay * gy[v]);
  }
  if (a.xadd) {
#pragma unroll
    for (int v = 0; v < V; ++v) r[v] = r[v] + a.xadd[i * V + v];
  }
  if constexpr (HV != 0) {
#pragma unroll
    for (int v = 0; v < V; ++v) r[v] = fma(-a.hv_gamma, gh[v], r[v]);
  }
  double o[V];
  if (a.kind == kAdjPlain) {
#pragma unroll
    for (int v = 0; v < V; ++v) o[v] = r[v];
  } else {
    double li[V];
    load_row<V>(a.lam, i, li);
    if (a.kind == kAdjStage3) {
      const double c3 = 2.0 / 3.0, cr = 2.0 * a.dt / 3.0;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        o[v] = c3 * li[v] + cr * r[v];
        a.acc[i * V + v] = div3(li[v]);
      }
    } else if (a.kind == kAdjStage2) {
      const double cr = 0.25 * a.dt;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        o[v] = 0.25 * li[v] + cr * r[v];
        a.acc[i * V + v] = a.acc[i * V + v] + 0.75 * li[v];
      }
    } else {
#pragma unroll
      for (int v = 0; v < V; ++v) o[v] = (a.acc[i * V + v] + li[v]) + a.dt * r[v];
    }
  }
  if (BC) project_row<V>(a.bc, i, o);
#pragma unroll
  for (int v = 0; v < V; ++v) a.out[i * V + v] = o[v];
}

template <int V, bool EULER, bool BC, int HV>
__global__ void __launch_bounds__(kBlock) k_adj_f64(AdjArgs a) {
  const int64_t row = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  if (row >= a.n) return;
  const int64_t i = ell_node(a.ell, row);
  const int64_t base = a.ell.slice_off[row >> 5] + (row & 31);
  const int len = a.ell.row_len[row];
  double gx[V], gy[V], gh[V];
#pragma unroll
  for (int v = 0; v < V; ++v) { gx[v] = 0; gy[v] = 0; gh[v] = 0; }
#pragma unroll 2
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int64_t c = __ldg(a.ell.col + p);
    const double wx = __ldg(a.w[0] + p), wy = __ldg(a.w[1] + p);
    double l[V];
    load_row<V>(a.lam, c, l);
    if (BC) mask_rows<V>(a.bc, c, l);
#pragma unroll
    for (int v = 0; v < V; ++v) {
      gx[v] = fma(wx, l[v], gx[v]);
      gy[v] = fma(wy, l[v], gy[v]);
    }
    if constexpr (HV == 2) {
      const double wh = __ldg(a.wh + p);
#pragma unroll
      for (int v = 0; v < V; ++v) gh[v] = fma(wh, l[v], gh[v]);
    } else if constexpr (HV == 1) {
      const double wh = __ldg(a.wh + p);
      double qq[V];
      load_row<V>(a.q, c, qq);
#pragma unroll
      for (int v = 0; v < V; ++v) gh[v] = fma(wh, qq[v], gh[v]);
    }
  }
  adj_finish<V, EULER, BC, HV>(a, i, gx, gy, gh);
}

// M2 lam as double-word pairs (n x 4 pairs): the cotangent the double-word adjoint
// gather reads, masked once per node instead of once per stencil entry.
template <bool BC>
__global__ void k_lam_pairs(int64_t n, const double* __restrict__ lam, BcDev bc,
                            float4* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double l[4];
  load_row<4>(lam, i, l);
  if (BC) mask_rows<4>(bc, i, l);
  const float2 a = dw::split(l[0]), b = dw::split(l[1]), c = dw::split(l[2]),
               d = dw::split(l[3]);
  out[i * 2] = make_float4(a.x, a.y, b.x, b.y);
  out[i * 2 + 1] = make_float4(c.x, c.y, d.x, d.y);
}

// The adjoint gather of 2D Euler in double-word FP32 arithmetic (as the forward form's
// gathers; the sums over the reverse adjacency in pairs, the node part in FP64).  HV 0
// (no hyperviscosity) or 2 (Flyer, whose term gathers the same M2 lam).
// HALO: blocks of one row group stage the group's neighbour cotangent pairs in shared
// memory first (mft_halo.cuh); same sums, same order.
template <bool BC, int HV, bool HALO>
__global__ void __launch_bounds__(HALO ? kHaloRows : kBlock) k_adj_dw(AdjArgs a) {
  const int64_t row = blockIdx.x * (int64_t)(HALO ? (int)blockDim.x : kBlock) + threadIdx.x;
  const float* __restrict__ L = reinterpret_cast<const float*>(a.lamdw);
  extern __shared__ float4 hsm[];
  bool staged = false;
  if (HALO) {
    const float4* L4 = reinterpret_cast<const float4*>(a.lamdw);
    staged = stage_halo<2>(a.ell, hsm, [&](int k, int64_t c) { return L4 + c * 2 + k; });
  }
  if (row >= a.n) return;
  const int64_t i = ell_node(a.ell, row);
  const int64_t base = a.ell.slice_off[row >> 5] + (row & 31);
  const int len = a.ell.row_len[row];
  const int hs = a.ell.halo_stride;
  dw::Acc gx[4], gy[4], gh[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) { gx[v] = dw::zero(); gy[v] = dw::zero(); gh[v] = dw::zero(); }
#pragma unroll 2
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const float2 wx = __ldg(a.wdw[0] + p), wy = __ldg(a.wdw[1] + p);
    F8 ll;
    if (HALO && staged) {
      const int lc = __ldg(a.ell.lcol + p);
      ll.lo = hsm[lc];
      ll.hi = hsm[hs + lc];
    } else {
      ll = ldg_f8(L + (int64_t)__ldg(a.ell.col + p) * 8);
    }
    const float2 l[4] = {make_float2(ll.lo.x, ll.lo.y), make_float2(ll.lo.z, ll.lo.w),
                         make_float2(ll.hi.x, ll.hi.y), make_float2(ll.hi.z, ll.hi.w)};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      dw::fma_acc(gx[v], wx, l[v]);
      dw::fma_acc(gy[v], wy, l[v]);
    }
    if constexpr (HV == 2) {
      const float2 wh = __ldg(a.whdw + p);
#pragma unroll
      for (int v = 0; v < 4; ++v) dw::fma_acc(gh[v], wh, l[v]);
    }
  }
  // the Jacobian product in double-word arithmetic from the sums as pairs
  float2 gxp[4], gyp[4];
  double ghd[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    gxp[v] = dw::to_pair(gx[v]);
    gyp[v] = dw::to_pair(gy[v]);
    ghd[v] = HV ? dw::to_double(gh[v]) : 0.0;
  }
  adj_finish<4, true, BC, HV>(a, i, nullptr, nullptr, ghd, gxp, gyp);
}

// q_i = sum_j lap[i,j] (M2 lam)_j over the forward sliced ELL.
template <int V, bool BC>
__global__ void __launch_bounds__(kBlock) k_lap_masked(int64_t n, EllView ell, const double* wl,
                                                       const double* lam, BcDev bc, double* q) {
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  if (r >= n) return;
  const int64_t i = ell_node(ell, r);
  const int64_t base = ell.slice_off[r >> 5] + (r & 31);
  const int len = ell.row_len[r];
  double acc[V];
#pragma unroll
  for (int v = 0; v < V; ++v) acc[v] = 0;
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int64_t c = __ldg(ell.col + p);
    const double w = __ldg(wl + p);
    double l[V];
    load_row<V>(lam, c, l);
    if (BC) mask_rows<V>(bc, c, l);
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v] = fma(w, l[v], acc[v]);
  }
#pragma unroll
  for (int v = 0; v < V; ++v) q[i * V + v] = acc[v];
}

template <int V>
__global__ void k_bc_project(int64_t nb, const int32_t* bnode, BcDev bc, double* lam) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const int64_t i = bnode[k];
  double o[V];
#pragma unroll
  for (int v = 0; v < V; ++v) o[v] = lam[i * V + v];
  project_row<V>(bc, i, o);
#pragma unroll
  for (int v = 0; v < V; ++v) lam[i * V + v] = o[v];
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

template <int V, bool EULER, bool BC>
void adj_hv(const AdjArgs& a, cudaStream_t s) {
  const unsigned g = grid_for(a.n, kBlock);
  if (a.hv == 1) k_adj_f64<V, EULER, BC, 1><<<g, kBlock, 0, s>>>(a);
  else if (a.hv == 2) k_adj_f64<V, EULER, BC, 2><<<g, kBlock, 0, s>>>(a);
  else k_adj_f64<V, EULER, BC, 0><<<g, kBlock, 0, s>>>(a);
}

}  // namespace

void launch_adj_f64(const AdjArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  if (a.V == 4) {
    if (a.has_bc) adj_hv<4, true, true>(a, s);
    else adj_hv<4, true, false>(a, s);
  } else {
    if (a.has_bc) adj_hv<1, false, true>(a, s);
    else adj_hv<1, false, false>(a, s);
  }
  MFT_LAUNCH_CHECK();
}

void launch_adj_dw(const AdjArgs& a, float2* lam_pairs, bool staged, cudaStream_t s) {
  if (a.n <= 0) return;
  MFT_REQUIRE(a.V == 4 && a.eq == MFT_EQ_EULER2D && a.hv != 1, MFT_ERR_UNSUPPORTED,
              "double-word adjoint gather: 2D Euler without Tominec hyperviscosity");
  const unsigned gn = grid_for(a.n, 256);
  if (a.has_bc) k_lam_pairs<true><<<gn, 256, 0, s>>>(a.n, a.lam, a.bc, reinterpret_cast<float4*>(lam_pairs));
  else k_lam_pairs<false><<<gn, 256, 0, s>>>(a.n, a.lam, a.bc, reinterpret_cast<float4*>(lam_pairs));
  MFT_LAUNCH_CHECK();
  AdjArgs b = a;
  b.lamdw = lam_pairs;
  if (staged && a.ell.halo_off) {
    const int rows = a.ell.halo_rows;
    const unsigned g = grid_for(a.n, rows);
    const size_t smem = (size_t)2 * a.ell.halo_stride * sizeof(float4);
    if (a.has_bc) {
      if (a.hv == 2) k_adj_dw<true, 2, true><<<g, rows, smem, s>>>(b);
      else k_adj_dw<true, 0, true><<<g, rows, smem, s>>>(b);
    } else {
      if (a.hv == 2) k_adj_dw<false, 2, true><<<g, rows, smem, s>>>(b);
      else k_adj_dw<false, 0, true><<<g, rows, smem, s>>>(b);
    }
  } else {
    const unsigned g = grid_for(a.n, kBlock);
    if (a.has_bc) {
      if (a.hv == 2) k_adj_dw<true, 2, false><<<g, kBlock, 0, s>>>(b);
      else k_adj_dw<true, 0, false><<<g, kBlock, 0, s>>>(b);
    } else {
      if (a.hv == 2) k_adj_dw<false, 2, false><<<g, kBlock, 0, s>>>(b);
      else k_adj_dw<false, 0, false><<<g, kBlock, 0, s>>>(b);
    }
  }
  MFT_LAUNCH_CHECK();
}

void launch_lap_masked(int64_t n, EllView fwd, const double* wl, const double* lam, int V,
                       BcDev bc, int has_bc, double* q, cudaStream_t s) {
  if (n <= 0) return;
  const unsigned g = grid_for(n, kBlock);
  if (V == 4) {
    if (has_bc) k_lap_masked<4, true><<<g, kBlock, 0, s>>>(n, fwd, wl, lam, bc, q);
    else k_lap_masked<4, false><<<g, kBlock, 0, s>>>(n, fwd, wl, lam, bc, q);
  } else {
    if (has_bc) k_lap_masked<1, true><<<g, kBlock, 0, s>>>(n, fwd, wl, lam, bc, q);
    else k_lap_masked<1, false><<<g, kBlock, 0, s>>>(n, fwd, wl, lam, bc, q);
  }
  MFT_LAUNCH_CHECK();
}

void launch_bc_project(int64_t nb, const int32_t* bnode, int V, BcDev bc, double* lam,
                       cudaStream_t s) {
  if (nb <= 0) return;
  if (V == 4) k_bc_project<4><<<grid_for(nb, 256), 256, 0, s>>>(nb, bnode, bc, lam);
  else k_bc_project<1><<<grid_for(nb, 256), 256, 0, s>>>(nb, bnode, bc, lam);
  MFT_LAUNCH_CHECK();
}

}  // namespace mft
