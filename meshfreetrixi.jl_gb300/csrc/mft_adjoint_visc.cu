// Adjoint of the viscosity sources (SourceResidualViscosityTominec, SourceUpwindViscosity-
// Tominec; src/sources/hyperviscosity.jl:246-409) inside the adjoint of rhs!.
//
// The source adds R_v = -sum_d D_d^T (eps o D_d u'_v) to du (u' the BC-corrected state),
// with eps = min(eps_rv, eps_uw) (update_visc!), eps_uw a function of the node's own state
// and eps_rv = K max_v |a_v - P_v| / n_v (update_residual_visc!; a = approx_du, P the
// partial du of the flux divergence, n = ode_maximum(|u' - ode_mean(u')|), K =
// c_rv h^2 / 2).  Its transpose product for the cotangent l = M2 lam, every selection
// (the min, the maximum over variables, the row of ode_maximum, |.|) frozen as the forward
// evaluation took it (the derivative away from ties):
//   linear part         -sum_d D_d^T (eps o D_d l)                (symmetric in u')
//   through eps         ebar_j = -sum_{d,v} (D_d u')_jv (D_d l)_jv, then
//     upwind branch     ebar_j grad eps_uw(u'_j)
//     residual branch   mu_{j v*} = -ebar_j K sign(r) / n_v*  -> -sum_d J_Fd^T D_d^T mu
//                       (the flux divergence's adjoint), and the norm n_v* through
//                       nbar_v = -sum_j ebar_j K |r_j| / n_v^2, added as
//                       nbar_v s_v (e_{j*} - 1/D) (s_v the sign of u'_{j*v} - mean_v,
//                       D the ode_mean denominator, j* the row of ode_maximum)
// approx_du is an input of rhs! (the HistoryCallback's estimate), not differentiated.
#include <cuda_runtime.h>
#include <math.h>

#include <cmath>

#include "mft_ctx.h"
#include "mft_device.cuh"

namespace mft {
namespace {

using namespace dev;

constexpr double kJlEps = 2.220446049250313e-16;

struct ViscAdj {
  int64_t n;
  EllView ell;          // forward layout
  const double* wx;     // D_x, D_y on it
  const double* wy;
  const double* lam;    // n x V cotangent of du
  const double* u;      // n x V BC-corrected state u'
  const double* eps;    // n: the viscosity the forward evaluation used
  const double* du_p;   // n x V partial du the residual viscosity read
  const double* approx; // n x V approx_du
  const double* norms;  // 2V: n_v, 1 / n_v
  const double* mean;   // V
  BcDev bc;
  int has_bc;
  int V, kind, si, mean_mode, max_mode, euler;
  double gamma, uwc, K, uw_adv;
  double* ebar;         // n
  double* sl;           // n x 2V: eps o D_d l
  double* xadd;         // n x V
  double* mu;           // n x V
  double* nbar_node;    // n x V
  int* jstar;           // V
};

template <int V>
__device__ __forceinline__ void load_v(const double* a, int64_t c, double* l) {
#pragma unroll
  for (int v = 0; v < V; ++v) l[v] = a[c * V + v];
}

// ebar and eps o D l per node, over the forward layout.
template <int V, bool BC>
__global__ void __launch_bounds__(kBlock) k_visc_adj_gather(ViscAdj a) {
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  double tx[V], ty[V], lx[V], ly[V];
#pragma unroll
  for (int v = 0; v < V; ++v) { tx[v] = 0; ty[v] = 0; lx[v] = 0; ly[v] = 0; }
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int64_t c = __ldg(a.ell.col + p);
    const double wx = __ldg(a.wx + p), wy = __ldg(a.wy + p);
    double uc[V], lc[V];
    load_v<V>(a.u, c, uc);
    load_v<V>(a.lam, c, lc);
    if (BC) {
      const int tag = a.bc.tag[c];
      if (tag == 1) {
#pragma unroll
        for (int v = 0; v < V; ++v) lc[v] = 0.0;
      } else if (tag == 2 && V == 4) {
        lc[1 % V] = 0.0;
        lc[2 % V] = 0.0;
      }
    }
#pragma unroll
    for (int v = 0; v < V; ++v) {
      tx[v] = fma(wx, uc[v], tx[v]);
      ty[v] = fma(wy, uc[v], ty[v]);
      lx[v] = fma(wx, lc[v], lx[v]);
      ly[v] = fma(wy, lc[v], ly[v]);
    }
  }
  double eb = 0.0;
#pragma unroll
  for (int v = 0; v < V; ++v) eb = eb - (tx[v] * lx[v] + ty[v] * ly[v]);
  a.ebar[i] = eb;
  const double e = a.eps[i];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    a.sl[i * 2 * V + v] = e * lx[v];
    a.sl[i * 2 * V + V + v] = e * ly[v];
  }
}

// Gradient of eps_uw = uwc (|m| / rho + sqrt(gamma p / rho)) at one Euler state (zero
// where a branch of the forward formula is not differentiable: |v| = 0, c = 0).
__device__ __forceinline__ void grad_eps_uw(double g, double uwc, const double* uu, double* gr) {
  const double rho = uu[0], m1 = uu[1], m2 = uu[2], en = uu[3];
  const double v1 = m1 / rho, v2 = m2 / rho;
  const double q2 = v1 * v1 + v2 * v2;
  const double speed = sqrt(q2);
  const double gm1 = g - 1.0;
  const double p = gm1 * (en - 0.5 * (m1 * v1 + m2 * v2));
  double ds[4] = {0, 0, 0, 0}, dc[4] = {0, 0, 0, 0};
  if (speed > 0.0) {
    ds[0] = -speed / rho;
    ds[1] = v1 / (rho * speed);
    ds[2] = v2 / (rho * speed);
  }
  if (!(p < 0.0 || rho < 0.0)) {
    const double c = sqrt(g * p / rho);
    if (c > 0.0) {
      const double k = g / (2.0 * c);
      dc[0] = k * (gm1 * 0.5 * q2 / rho - p / (rho * rho));
      dc[1] = k * (-gm1 * v1) / rho;
      dc[2] = k * (-gm1 * v2) / rho;
      dc[3] = k * gm1 / rho;
    }
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) gr[v] = uwc * (ds[v] + dc[v]);
}

// Branch of eps at each node and the cotangents through it.
template <int V>
__global__ void __launch_bounds__(kBlock) k_visc_adj_node(ViscAdj a) {
  const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  if (i >= a.n) return;
  const double eb = a.ebar[i];
  double xa[V], mu[V], nb[V];
#pragma unroll
  for (int v = 0; v < V; ++v) { xa[v] = 0; mu[v] = 0; nb[v] = 0; }
  double uu[V];
  load_v<V>(a.u, i, uu);
  double eps_uw;
  if (V == 4 && a.euler) {
    const double rho = uu[0], v1 = uu[1 % V] / rho, v2 = uu[2 % V] / rho;
    const double p = (a.gamma - 1.0) * (uu[3 % V] - 0.5 * (uu[1 % V] * v1 + uu[2 % V] * v2));
    const double c = (p < 0.0 || rho < 0.0) ? 0.0 : sqrt(a.gamma * p / rho);
    eps_uw = a.uwc * (sqrt(v1 * v1 + v2 * v2) + c);
  } else {
    eps_uw = a.uw_adv;  // advection: uwc |a|, independent of the state
  }
  const bool uw_finite = isfinite(eps_uw);
  int branch = uw_finite ? 1 : 0;  // 0 none, 1 upwind, 2 residual
  int vs = 0;
  double rs = 0.0;
  if (a.kind == MFT_SRC_RV && a.si != 0) {
    double mr = -1.0;
    for (int v = 0; v < V; ++v) {
      const double r = a.approx[i * V + v] - a.du_p[i * V + v];
      const double q = fabs(r) * a.norms[V + v];
      if (v == 0 || q > mr) { mr = q; vs = v; rs = r; }
    }
    const double eps_rv = a.K * mr;
    if (isfinite(eps_rv)) branch = (uw_finite && eps_uw < eps_rv) ? 1 : 2;
  }
  if (branch == 1 && V == 4 && a.euler) {
    double gr[4];
    grad_eps_uw(a.gamma, a.uwc, uu, gr);
#pragma unroll
    for (int v = 0; v < V; ++v) xa[v] = eb * gr[v % 4];
  } else if (branch == 2) {
    const double ninv = a.norms[V + vs];
    const double sg = rs > 0.0 ? 1.0 : (rs < 0.0 ? -1.0 : 0.0);
    mu[vs] = -eb * a.K * sg * ninv;
    if (a.norms[vs] != kJlEps) nb[vs] = -eb * a.K * fabs(rs) * ninv * ninv;
  }
#pragma unroll
  for (int v = 0; v < V; ++v) {
    a.xadd[i * V + v] = xa[v];
    a.mu[i * V + v] = mu[v];
    a.nbar_node[i * V + v] = nb[v];
  }
}

// The row of ode_maximum: |u' - mean| equal (bit for bit) to the norms; ties take the
// last row, as max(a, b) = isless(b, a) ? a : b does over the nodes in order.
template <int V>
__global__ void k_visc_adj_argmax(ViscAdj a) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  bool all = true;
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const double d = fabs(__dsub_rn(a.u[i * V + v], a.mean[v]));
    const bool eq = __double_as_longlong(d) == __double_as_longlong(a.norms[v]);
    all = all && eq;
    if (a.max_mode != 0 && eq) atomicMax(a.jstar + v, (int)i);
  }
  if (a.max_mode == 0 && all)
    for (int v = 0; v < V; ++v) atomicMax(a.jstar + v, (int)i);
}

// xadd_iv += nbar_v s_v (delta(i, j*_v) - 1 / D)
template <int V>
__global__ void k_visc_adj_norms(ViscAdj a, const double* nbar, double denom) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= a.n) return;
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const int js = a.jstar[v];
    if (js < 0 || a.norms[v] == kJlEps) continue;
    const double d = a.u[(int64_t)js * V + v] - a.mean[v];
    const double s = d > 0.0 ? 1.0 : (d < 0.0 ? -1.0 : 0.0);
    double x = -nbar[v] * s / denom;
    if (i == js) x += nbar[v] * s;
    a.xadd[i * V + v] += x;
  }
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

// The viscosity source's part of (d rhs!/du)^T lam, before the BC projection, added to
// what the flux and hyperviscosity adjoint forms: out (n x V) receives it.  u_bc is the
// BC-corrected state of a forward evaluation just made (its eps, du_p, norms and mean are
// in the context); lam the cotangent of du.  Scratch: t (n x 2V), q, hvf, du_p2 (n x V),
// work_du (n x V), red_partial / red_counter, d_ctr.
void visc_adjoint_terms(mft_ctx* c, const double* u_bc, const double* lam, double* out) {
  cudaStream_t s = c->stream;
  const int V = c->nvars;
  const int64_t n = c->n;
  int iv = -1;
  for (size_t k = 0; k < c->src_kind.size(); ++k)
    if (c->src_kind[k] == MFT_SRC_RV || c->src_kind[k] == MFT_SRC_UPWIND) iv = (int)k;
  if (iv < 0) return;
  const int kind = c->src_kind[iv];
  const double* par = &c->src_par[iv * 4];
  const double c_rv = kind == MFT_SRC_RV ? par[0] : 0.0;
  const double c_uw = kind == MFT_SRC_RV ? par[1] : par[0];
  const double h = kind == MFT_SRC_RV ? par[2] : par[1];
  ViscAdj a{};
  a.n = n;
  a.ell = c->fwd.view();
  a.wx = c->fw[0].p;
  a.wy = c->fw[1].p;
  a.lam = lam;
  a.u = u_bc;
  a.eps = c->eps.p;
  a.du_p = c->du_p.p;
  a.approx = c->approx_du.p;
  a.norms = c->norms.p;
  a.mean = c->mean.p;
  a.bc = BcDev{c->d_tag.p, c->d_slot.p, c->d_normal.p, c->d_dvals.p};
  a.has_bc = c->nb > 0;
  a.V = V;
  a.kind = kind;
  a.si = c->success_iter;
  a.mean_mode = kind == MFT_SRC_RV ? (int)par[3] : 0;
  a.max_mode = a.mean_mode;
  a.euler = c->eq == MFT_EQ_EULER2D;
  a.gamma = c->gamma;
  a.uwc = (c_uw * 0.5) * h;
  a.K = (0.5 * c_rv) * (h * h);
  a.uw_adv = a.uwc * std::sqrt(c->adv[0] * c->adv[0] + c->adv[1] * c->adv[1]);
  // scratch: ebar in hvf (n), eps o D l in t (n x 2V), xadd in work_du, mu in q,
  // nbar per node in du_p2; the argmax row in d_ctr's neighbour word
  a.ebar = c->hvf.p;
  a.sl = c->t.p;
  a.xadd = out;
  a.mu = c->q.p;
  a.nbar_node = c->du_p2.p;
  c->adj_jstar.alloc(8);
  a.jstar = c->adj_jstar.p;
  const unsigned g = grid_for(n, kBlock);
  if (V == 4) {
    if (a.has_bc) k_visc_adj_gather<4, true><<<g, kBlock, 0, s>>>(a);
    else k_visc_adj_gather<4, false><<<g, kBlock, 0, s>>>(a);
    k_visc_adj_node<4><<<g, kBlock, 0, s>>>(a);
  } else {
    if (a.has_bc) k_visc_adj_gather<1, true><<<g, kBlock, 0, s>>>(a);
    else k_visc_adj_gather<1, false><<<g, kBlock, 0, s>>>(a);
    k_visc_adj_node<1><<<g, kBlock, 0, s>>>(a);
  }
  MFT_LAUNCH_CHECK();
  if (kind == MFT_SRC_RV && c->success_iter != 0) {
    // nbar_v = sum_j nbar_node_jv (deterministic block reduction), the ode_maximum row
    c->adj_nbar.alloc(8);
    launch_mean(n, V, c->du_p2.p, 1.0, c->red_partial.p, c->red_counter.p, c->adj_nbar.p,
                c->red_blocks, s);
    MFT_CUDA(cudaMemsetAsync(c->adj_jstar.p, 0xFF, 8 * sizeof(int), s));
    const unsigned g2 = grid_for(n, 256);
    const double denom = a.mean_mode == 0 ? (double)n * V : (double)n;
    if (V == 4) {
      k_visc_adj_argmax<4><<<g2, 256, 0, s>>>(a);
      k_visc_adj_norms<4><<<g2, 256, 0, s>>>(a, c->adj_nbar.p, denom);
    } else {
      k_visc_adj_argmax<1><<<g2, 256, 0, s>>>(a);
      k_visc_adj_norms<1><<<g2, 256, 0, s>>>(a, c->adj_nbar.p, denom);
    }
    MFT_LAUNCH_CHECK();
  }
  // residual branch: the flux divergence's adjoint applied to mu (no M2 mask, no BC
  // projection here), added to out
  AdjArgs b{};
  b.n = n;
  b.ell = c->rev.view();
  b.w[0] = c->rw[0].p;
  b.w[1] = c->rw[1].p;
  b.hv = 0;
  b.lam = c->q.p;
  b.u = u_bc;
  b.eq = c->eq;
  b.V = V;
  b.gamma = c->gamma;
  b.ax = c->adv[0];
  b.ay = c->adv[1];
  b.bc = a.bc;
  b.has_bc = 0;
  b.kind = kAdjPlain;
  b.xadd = out;
  b.out = c->work_du.p;
  launch_adj_f64(b, s);
  // linear part: out = work_du - sum_d D_d^T (eps o D_d l)
  RevArgs r{};
  r.n = n;
  r.ell = c->rev.view();
  r.w[0] = c->rw[0].p;
  r.w[1] = c->rw[1].p;
  r.V = V;
  r.rv = 1;
  r.s = c->t.p;
  r.du_p = c->work_du.p;
  r.final_epilogue = 0;
  r.du_p_out = out;
  launch_rev_f64(r, s);
}

}  // namespace mft
