// Information geometric regularisation source (SourceIGR, src/sources/IGR.jl:17-239) for
// the 2D Euler equations, FP64:
//   b = alpha (tr(Du)^2 + tr(Du^2)), with tr(Du) formed as the reference writes it,
//       Dx rho + Dy v1 (update_igr_rhs!, :143-145), tr(Du^2) = (Dx v1)^2 +
//       2 (Dy v1)(Dx v2) + (Dy v2)^2 (:151-153);
//   sigma from (rho^-1 - alpha (Dx rho^-1 Dx + Dy rho^-1 Dy)) sigma = b by unpreconditioned
//       conjugate gradients from sigma = 0, at most maxiter iterations, relative
//       tolerance sqrt(eps) (the in-place cg! the reference intends at :189);
//   du[rho v1] -= Dx sigma, du[rho v2] -= Dy sigma (:214-237).
// The CG runs as a fixed sequence of kernels (four per iteration) whose scalars live in
// device memory; once converged, the remaining kernels return at entry, so one rhs!
// evaluation is a fixed launch sequence that a CUDA graph can hold.  Reductions are
// block partials finished by the last block in a fixed order (deterministic).
#include <cfloat>

#include "mft_device.cuh"

namespace mft {
namespace {

using namespace dev;

template <int W>
__device__ __forceinline__ void block_sum_igr(double (&v)[W]) {
  __shared__ double sh[W][kBlock / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < W; ++k) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[k][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < W; ++k) {
      double x = sh[k][0];
      for (int w = 1; w < kBlock / 32; ++w) x += sh[k][w];
      v[k] = x;
    }
  }
  __syncthreads();
}

// Block partial of one sum; returns true in thread 0 of the last block to finish, with
// the total in *total (fixed order over the partials).
__device__ bool last_block_total(double x, double* partial, unsigned* counter, double* total) {
  double v[1] = {x};
  block_sum_igr<1>(v);
  __shared__ int last;
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = v[0];
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double a[1] = {0.0};
  for (unsigned b = threadIdx.x; b < gridDim.x; b += kBlock) a[0] += __ldcg(partial + b);
  block_sum_igr<1>(a);
  if (threadIdx.x == 0) {
    *total = a[0];
    *counter = 0u;
  }
  return threadIdx.x == 0;
}

// prim = (rho, v1, v2), rinv = 1 / rho
__global__ void k_igr_prim(int64_t n, const double* __restrict__ u, double* prim, double* rinv) {
  const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  if (i >= n) return;
  const double rho = u[i * 4], m1 = u[i * 4 + 1], m2 = u[i * 4 + 2];
  prim[i * 3] = rho;
  prim[i * 3 + 1] = ddiv(m1, rho);
  prim[i * 3 + 2] = ddiv(m2, rho);
  rinv[i] = ddiv(1.0, rho);
}

// b, x = 0, r = b, u_old = 0 and the initial residual norm.
__global__ void __launch_bounds__(kBlock) k_igr_rhs(IgrArgs a) {
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  double rr = 0.0;
  if (r < a.n) {
    const int64_t i = ell_node(a.ell, r);
    const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
    const int len = a.ell.row_len[r];
    double dxr = 0, dxv1 = 0, dxv2 = 0, dyv1 = 0, dyv2 = 0;
    for (int j = 0; j < len; ++j) {
      const int64_t p = base + ((int64_t)j << 5);
      const int64_t c = __ldg(a.ell.col + p);
      const double wx = __ldg(a.wx + p), wy = __ldg(a.wy + p);
      const double rc = a.prim[c * 3], v1 = a.prim[c * 3 + 1], v2 = a.prim[c * 3 + 2];
      dxr = fma(wx, rc, dxr);
      dxv1 = fma(wx, v1, dxv1);
      dxv2 = fma(wx, v2, dxv2);
      dyv1 = fma(wy, v1, dyv1);
      dyv2 = fma(wy, v2, dyv2);
    }
    const double tr = dadd(dxr, dyv1);
    const double tsq = dadd(dadd(dmul(dxv1, dxv1), dmul(dmul(2.0, dyv1), dxv2)), dmul(dyv2, dyv2));
    const double b = dmul(a.alpha, dadd(dmul(tr, tr), tsq));
    a.x[i] = 0.0;
    a.r[i] = b;
    a.u0[i] = 0.0;
    rr = dmul(b, b);
  }
  double total;
  if (last_block_total(rr, a.partial, a.counter, &total)) {
    IgrScalars* s = a.sc;
    s->res = sqrt(total);
    s->prev = 1.0;
    s->tol = dmul(s->res, sqrt(DBL_EPSILON));
    s->beta = ddiv(dmul(s->res, s->res), 1.0);
    s->iter = 0;
    s->done = (s->res <= s->tol) || a.maxiter <= 0;
  }
}

// u_new = r + beta u_old (elementwise; the gathers below then read u_new directly)
__global__ void k_igr_newdir(IgrArgs a, const double* uo, double* un) {
  if (a.sc->done) return;
  const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  if (i >= a.n) return;
  un[i] = dadd(a.r[i], dmul(a.sc->beta, uo[i]));
}

// t1 = rinv (Dx u_new), t2 = rinv (Dy u_new)
__global__ void __launch_bounds__(kBlock) k_igr_dir(IgrArgs a, const double* un) {
  if (a.sc->done) return;
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  double sx = 0.0, sy = 0.0;
#pragma unroll 4
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int64_t c = __ldg(a.ell.col + p);
    const double uc = un[c];
    sx = fma(__ldg(a.wx + p), uc, sx);
    sy = fma(__ldg(a.wy + p), uc, sy);
  }
  a.t[i * 2] = dmul(a.rinv[i], sx);
  a.t[i * 2 + 1] = dmul(a.rinv[i], sy);
}

// c = rinv u_new - alpha (Dx t1 + Dy t2); alpha_cg = res^2 / (u_new . c)
__global__ void __launch_bounds__(kBlock) k_igr_op(IgrArgs a, const double* un) {
  if (a.sc->done) return;
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  double uc = 0.0;
  if (r < a.n) {
    const int64_t i = ell_node(a.ell, r);
    const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
    const int len = a.ell.row_len[r];
    double sx = 0.0, sy = 0.0;
    const double2* __restrict__ t2 = reinterpret_cast<const double2*>(a.t);
#pragma unroll 4
    for (int j = 0; j < len; ++j) {
      const int64_t p = base + ((int64_t)j << 5);
      const int64_t c = __ldg(a.ell.col + p);
      const double2 tc = t2[c];  // (t1, t2) of the neighbour in one 16-byte load
      sx = fma(__ldg(a.wx + p), tc.x, sx);
      sy = fma(__ldg(a.wy + p), tc.y, sy);
    }
    const double ci = dsub(dmul(a.rinv[i], un[i]), dmul(a.alpha, dadd(sx, sy)));
    a.c[i] = ci;
    uc = dmul(un[i], ci);
  }
  double total;
  if (last_block_total(uc, a.partial, a.counter, &total)) {
    IgrScalars* s = a.sc;
    s->alpha_cg = ddiv(dmul(s->res, s->res), total);
  }
}

// x += alpha_cg u_new; r -= alpha_cg c; new residual, beta, convergence
__global__ void __launch_bounds__(kBlock) k_igr_update(IgrArgs a, const double* un) {
  if (a.sc->done) return;
  const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  double rr = 0.0;
  if (i < a.n) {
    const double al = a.sc->alpha_cg;
    a.x[i] = dadd(a.x[i], dmul(al, un[i]));
    const double r = dsub(a.r[i], dmul(al, a.c[i]));
    a.r[i] = r;
    rr = dmul(r, r);
  }
  double total;
  if (last_block_total(rr, a.partial, a.counter, &total)) {
    IgrScalars* s = a.sc;
    s->prev = s->res;
    s->res = sqrt(total);
    s->iter += 1;
    s->beta = ddiv(dmul(s->res, s->res), dmul(s->prev, s->prev));
    s->done = (s->iter >= a.maxiter) || (s->res <= s->tol);
  }
}

// add = (-(Dx sigma), -(Dy sigma)) for the momentum rows of du
__global__ void __launch_bounds__(kBlock) k_igr_flux(IgrArgs a) {
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  double sx = 0.0, sy = 0.0;
#pragma unroll 4
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int64_t c = __ldg(a.ell.col + p);
    sx = fma(__ldg(a.wx + p), a.x[c], sx);
    sy = fma(__ldg(a.wy + p), a.x[c], sy);
  }
  a.add[i * 2] = -sx;
  a.add[i * 2 + 1] = -sy;
}

}  // namespace

void launch_igr(const IgrArgs& a, const double* u, cudaStream_t s) {
  if (a.n <= 0) return;
  const unsigned g = (unsigned)((a.n + kBlock - 1) / kBlock);
  k_igr_prim<<<g, kBlock, 0, s>>>(a.n, u, a.prim, a.rinv);
  MFT_LAUNCH_CHECK();
  k_igr_rhs<<<g, kBlock, 0, s>>>(a);
  MFT_LAUNCH_CHECK();
  for (int it = 0; it < a.maxiter; ++it) {
    const double* uo = (it & 1) ? a.u1 : a.u0;
    double* un = (it & 1) ? a.u0 : a.u1;
    k_igr_newdir<<<g, kBlock, 0, s>>>(a, uo, un);
    MFT_LAUNCH_CHECK();
    k_igr_dir<<<g, kBlock, 0, s>>>(a, un);
    MFT_LAUNCH_CHECK();
    k_igr_op<<<g, kBlock, 0, s>>>(a, un);
    MFT_LAUNCH_CHECK();
    k_igr_update<<<g, kBlock, 0, s>>>(a, un);
    MFT_LAUNCH_CHECK();
  }
  k_igr_flux<<<g, kBlock, 0, s>>>(a);
  MFT_LAUNCH_CHECK();
}

}  // namespace mft
