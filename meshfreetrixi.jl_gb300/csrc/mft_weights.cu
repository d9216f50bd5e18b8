// K2: batched FP64 polyharmonic-spline + polynomial RBF-FD weights.
//
// Restates the per-node loop of compute_flux_operator
// (src/solvers/pointcloudsolver/compute_operators.jl:409-453 and :549-594):
//   shift_stencil (:225-246)  X^_j = (X_j - X_centre) * s,  s_d = 1/max_j |dX_jd|
//   M = [R P; P' 0] upper (interpolation_block :265-267), R_ij = |X^_i - X^_j|^p,
//   P_im = monomial_m(X^_i)
//   RHS: d^k/dx_d^k of |x - X^_j|^p at the centre (mirror_stencil :248-263 with the
//   centre entry at (eps,...,eps)), monomial derivatives at the origin
//   w = M \ rhs by Bunch-Kaufman (LAPACK dsytf2 + dsytrs, upper), weights s_d^k w.
//
// One warp per system, the system in shared memory, one persistent launch over all
// nodes with a work counter; systems are taken largest first so that uneven stencil
// sizes (interior vs boundary, 2D vs 3D) balance across warps.  Every matrix element
// sees the same sequence of separately rounded operations as in the CPU
// restatement (updates are element-independent and the solve's dot products use a
// fixed 32-way strided partial-sum order), so the weights are bit-identical to it.
#include <cuda_runtime.h>
#include <math.h>

#include <string.h>

#include <algorithm>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "mft_ctx.h"

namespace mft {

namespace {

constexpr int kWarpsPerBlock = 2;  // systems per block with one warp per system
// Buckets of systems larger than kMultiWarpMinN share kSystemWarps warps per system: their
// packed matrices limit an SM to a few systems, and one warp each leaves the FP64 pipe
// idle behind shared-memory and reduction latencies.  Measured on the 1M-stencil batch
// (2D k 35/40-60, 3D k 60-90): one warp everywhere 498 ms; two warps above n = 64
// 482 ms; four warps above n = 64 512 ms (the block barriers of every column step cost
// more than the added warps recover); several warps for the 2D buckets 611-879 ms.
constexpr int kSystemWarps = 2;
constexpr int kMultiWarpMinN = 64;
constexpr unsigned kFull = 0xffffffffu;

// One batch of stencils sharing dimension, basis and derivative order.
constexpr int kMaxMono = 84;  // monomials of total degree <= 6 in 3D
struct WGroup {
  int dim, npoly, rbf_pow, order;
  int periodic;
  double period[3];
  const int64_t* rowptr;
  const int32_t* cols;
  const double* xyz;
  double* w_out;  // nnz x dim (stencil order)
  double* resid;  // optional per node
  int mono[kMaxMono][3];
};

constexpr int kMaxGroups = 2;
// Work item codes: group << kGroupShift | node.
constexpr int kGroupShift = 48;

struct WArgs {
  int nmax, kmax;
  int64_t nsys;
  const int64_t* order_list;  // work item codes, largest stencil first
  int* bad;                   // smallest node index with a zero pivot, or INT_MAX
  unsigned long long* next;
  WGroup g[kMaxGroups];
};

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

__device__ double pow_int(double x, int k) {
  if (k < 0) {
    double r = 1.0;
    for (int i = 0; i < -k; ++i) r = dmul(r, x);
    return ddiv(1.0, r);
  }
  double r = 1.0;
  for (int i = 0; i < k; ++i) r = dmul(r, x);
  return r;
}

__device__ double fact(int k) {
  double r = 1.0;
  for (int i = 2; i <= k; ++i) r = dmul(r, (double)i);
  return r;
}

// d^k/dx_d^k of r^p (Faa di Bruno on s^(p/2), s = |x|^2); same operation order as
// the CPU restatement.
__device__ double phs_deriv(int p, int k, double xd, double r) {
  if (k == 0) return pow_int(r, p);
  double sum = 0.0;
  for (int j = 0; 2 * j <= k; ++j) {
    const int m = k - j;
    double cm = 1.0;
    for (int i = 0; i < m; ++i) cm = dmul(cm, dsub(dmul(0.5, (double)p), (double)i));
    if (cm == 0.0) continue;
    const double cc = ddiv(fact(k), dmul(fact(j), fact(k - 2 * j)));
    const double term =
        dmul(dmul(dmul(cc, pow_int(dmul(2.0, xd), k - 2 * j)), cm), pow_int(r, p - 2 * m));
    sum = dadd(sum, term);
  }
  return sum;
}

__device__ __forceinline__ double min_image(double d, double L) {
  if (d > 0.5 * L) return dsub(d, L);
  if (d < -0.5 * L) return dadd(d, L);
  return d;
}

// first index of the largest |x| among lanes' candidates (value, index).  Lanes
// start from (-1, sentinel); if no candidate compares (all NaN) the result falls
// back to index `lo` so that every later access stays inside the system.
__device__ __forceinline__ void warp_argmax(double& v, int& i, int lo) {
  for (int o = 16; o > 0; o >>= 1) {
    const double v2 = __shfl_xor_sync(kFull, v, o);
    const int i2 = __shfl_xor_sync(kFull, i, o);
    if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
  }
  if (i == (1 << 30)) { i = lo; v = NAN; }
}

__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// Synchronisation of the threads that share one system: the warp (W == 1) or the block.
template <int W>
__device__ __forceinline__ void gsync() {
  if (W == 1) __syncwarp();
  else __syncthreads();
}

// warp_argmax over the W warps of a block (red_v, red_i: W-entry shared scratch); every
// thread of the block must call it.  The warps' candidates combine with the same rule
// (larger value, then smaller index), so the result is the single-warp one.
template <int W>
__device__ __forceinline__ void group_argmax(double& v, int& i, int lo, double* red_v,
                                             int* red_i) {
  for (int o = 16; o > 0; o >>= 1) {
    const double v2 = __shfl_xor_sync(kFull, v, o);
    const int i2 = __shfl_xor_sync(kFull, i, o);
    if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
  }
  if (W > 1) {
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { red_v[w] = v; red_i[w] = i; }
    __syncthreads();
    v = red_v[0];
    i = red_i[0];
    for (int q = 1; q < W; ++q) {
      const double v2 = red_v[q];
      const int i2 = red_i[q];
      if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
    }
    __syncthreads();
  }
  if (i == (1 << 30)) { i = lo; v = NAN; }
}

template <int W>
__device__ __forceinline__ double group_max(double v, double* red_v) {
  v = warp_max(v);
  if (W > 1) {
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) red_v[w] = v;
    __syncthreads();
    v = red_v[0];
    for (int q = 1; q < W; ++q) v = fmax(v, red_v[q]);
    __syncthreads();
  }
  return v;
}

// Advances (i, j), 0 <= i <= j, to the next element a warp stride further along the
// column-major upper triangle (t = j(j+1)/2 + i).
__device__ __forceinline__ void tri_next(int& i, int& j, int step) {
  i += step;
  while (i > j) { i -= j + 1; ++j; }
}

// Doubles of shared memory one warp of k_weights uses: the upper triangle of A packed by
// columns (nmax (nmax + 1) / 2; Bunch-Kaufman in upper storage reads and writes only
// i <= j), B (3 nmax), X (3 kmax), two column-multiplier arrays (2 nmax) and the pivot
// ints (nmax).
__host__ __device__ __forceinline__ size_t weights_smem_doubles(int nmax, int kmax) {
  return (size_t)nmax * (nmax + 1) / 2 + (size_t)nmax * 3 + (size_t)kmax * 3 +
         (size_t)nmax * 2 + nmax;
}

// kOrdered: systems are taken in the order of a.order_list (largest first); otherwise
// in node order.
template <bool kOrdered, int W>
__global__ void __launch_bounds__(W == 1 ? 32 * kWarpsPerBlock : 32 * W) k_weights(WArgs a) {
  extern __shared__ double smem[];
  // W == 1: one warp per system, kWarpsPerBlock systems per block.  W > 1: the W warps
  // of a block share one system (large systems: more warps per SM than the per-system
  // shared memory would otherwise allow); the factorisation's element loops and
  // reductions span the block, the triangular solves run in warp 0.
  constexpr int G = 32 * W;  // threads per system
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int gt = W == 1 ? lane : (int)threadIdx.x;
  const int nmax = a.nmax;
  __shared__ double red_v[W];
  __shared__ int red_i[W];
  __shared__ unsigned long long s_job;
  // per-system shared layout: A[nmax(nmax+1)/2] (upper, packed), B[nmax*3], X[kmax*3],
  // TC[nmax], TC2[nmax],
  // ipiv[nmax] (ints)
  const size_t per = weights_smem_doubles(nmax, a.kmax);
  double* A = smem + per * (W == 1 ? wib : 0);
  double* B = A + (size_t)nmax * (nmax + 1) / 2;
  double* X = B + (size_t)nmax * 3;
  double* TC = X + (size_t)a.kmax * 3;
  double* TC2 = TC + nmax;
  int* ipiv = reinterpret_cast<int*>(TC2 + nmax);
  for (;;) {
    unsigned long long job = 0;
    if (W == 1) {
      if (lane == 0) job = atomicAdd(a.next, 1ull);
      job = __shfl_sync(kFull, job, 0);
    } else {
      __syncthreads();  // every thread is done with the previous system
      if (gt == 0) s_job = atomicAdd(a.next, 1ull);
      __syncthreads();
      job = s_job;
    }
    if (job >= (unsigned long long)a.nsys) break;
    const int64_t code = kOrdered ? a.order_list[job] : (int64_t)job;
    const int grp = (int)(code >> kGroupShift);
    const int64_t e = code & ((1ll << kGroupShift) - 1);
    const int dim = a.g[grp].dim, npoly = a.g[grp].npoly;
    const int rbf_pow = a.g[grp].rbf_pow, order = a.g[grp].order, periodic = a.g[grp].periodic;
    const int64_t* rowptr = a.g[grp].rowptr;
    const int32_t* cols = a.g[grp].cols;
    const double* xyz = a.g[grp].xyz;
    double* w_out = a.g[grp].w_out;
    double* resid = a.g[grp].resid;
    const int64_t rb = rowptr[e];
    if (!kOrdered) {
      // Unordered work comes from caller-owned device arrays that no host code checked
      // (mft_weights_noalloc; one warp per system).  Before any coordinate is read, a
      // stencil is skipped, its weights set to NaN where its row lies inside cols, and a
      // status word set, when its size is outside 1..kmax (word 2 for > kmax, word 3
      // otherwise), its extent leaves [0, rowptr[n]) or a column is not a node (word 3).
      static_assert(kOrdered || W == 1, "unordered systems run one warp per system");
      const int64_t re = rowptr[e + 1], nnz = rowptr[a.nsys];
      const int64_t k64 = re - rb;
      const bool in_cols = rb >= 0 && re <= nnz && k64 >= 0;
      int why = 0;
      if (!in_cols || k64 < 1) why = 3;
      else if (k64 > a.kmax) why = 2;
      if (why == 0) {
        bool badc = false;
        for (int64_t j = gt; j < k64; j += G) {
          const int32_t cj = cols[rb + j];
          badc |= cj < 0 || (int64_t)cj >= a.nsys;
        }
        if (__any_sync(kFull, badc)) why = 3;
      }
      if (why != 0) {
        if (gt == 0) atomicExch(reinterpret_cast<int*>(a.next + why), 1);
        if (in_cols)
          for (int64_t t = rb * dim + gt; t < re * dim; t += G) w_out[t] = __longlong_as_double(0x7FF8000000000000LL);
        continue;
      }
    }
    const int k = (int)(rowptr[e + 1] - rb);
    const int n = k + npoly;
// upper-packed element (i, j), 1 <= i <= j: column j starts at j (j - 1) / 2
#define AM(i, j) A[(((j) * ((j)-1)) >> 1) + ((i)-1)]
#define BM(i, c) B[(size_t)(c) * n + ((i)-1)]
    const int32_t* st = cols + rb;
    const int64_t ce = st[0];
    // shift_stencil
    for (int j = gt; j < k; j += G)
      for (int d = 0; d < dim; ++d) {
        double t = dsub(xyz[(int64_t)st[j] * dim + d], xyz[ce * dim + d]);
        if (periodic) t = min_image(t, a.g[grp].period[d]);
        X[j * 3 + d] = t;
      }
    gsync<W>();
    double s[3] = {1.0, 1.0, 1.0};
    for (int d = 0; d < dim; ++d) {
      double m = 0.0;
      for (int j = gt; j < k; j += G) m = fmax(m, fabs(X[j * 3 + d]));
      m = group_max<W>(m, red_v);
      s[d] = ddiv(1.0, m);
    }
    for (int j = gt; j < k; j += G)
      for (int d = 0; d < dim; ++d) X[j * 3 + d] = dmul(X[j * 3 + d], s[d]);
    gsync<W>();
    // interpolation block (upper triangle, column-major)
    const int T = n * (n + 1) / 2;
    int r = 0, cidx = 0;
    tri_next(r, cidx, gt);
    for (int t = gt; t < T; t += G, tri_next(r, cidx, G)) {
      double v;
      if (cidx < k) {
        double d2 = 0.0;
        for (int d = 0; d < dim; ++d) {
          const double tt = dsub(X[r * 3 + d], X[cidx * 3 + d]);
          d2 = dadd(d2, dmul(tt, tt));
        }
        v = pow_int(sqrt(d2), rbf_pow);
      } else if (r < k) {
        const int* ex = a.g[grp].mono[cidx - k];
        v = 1.0;
        for (int d = 0; d < dim; ++d) v = dmul(v, pow_int(X[r * 3 + d], ex[d]));
      } else {
        v = 0.0;
      }
      A[((cidx * (cidx + 1)) >> 1) + r] = v;
    }
    // right-hand sides
    for (int t = gt; t < n * dim; t += G) {
      const int d = t / n, j = t % n;
      double v;
      if (j < k) {
        double pt[3];
        for (int dd = 0; dd < dim; ++dd)
          pt[dd] = j == 0 ? 2.220446049250313e-16 : -X[j * 3 + dd];
        double d2 = 0.0;
        for (int dd = 0; dd < dim; ++dd) d2 = dadd(d2, dmul(pt[dd], pt[dd]));
        v = phs_deriv(rbf_pow, order, pt[d], sqrt(d2));
      } else {
        const int* ex = a.g[grp].mono[j - k];
        bool ok = true;
        for (int dd = 0; dd < dim; ++dd)
          if (ex[dd] != (dd == d ? order : 0)) ok = false;
        v = ok ? fact(order) : 0.0;
      }
      B[(size_t)d * n + j] = v;
    }
    gsync<W>();

    // ---------------- Bunch-Kaufman factorisation (upper)
    const double alpha = (1.0 + sqrt(17.0)) / 8.0;
    int info = 0;
    int kk = n;
    while (kk >= 1) {
      int kstep = 1, kp;
      const double absakk = fabs(AM(kk, kk));
      double colmax = 0.0;
      int imax = 0;
      if (kk > 1) {
        double v = -1.0;
        int iv = 1 << 30;
        for (int i = 1 + gt; i < kk; i += G) {
          const double x = fabs(AM(i, kk));
          if (x > v) { v = x; iv = i; }
        }
        group_argmax<W>(v, iv, 1, red_v, red_i);
        colmax = v;
        imax = iv;
      }
      if (fmax(absakk, colmax) == 0.0 || isnan(absakk)) {
        if (info == 0) info = kk;
        kp = kk;
      } else {
        if (absakk >= alpha * colmax) {
          kp = kk;
        } else {
          double v = -1.0;
          int iv = 1 << 30;
          for (int j = imax + 1 + gt; j <= kk; j += G) {
            const double x = fabs(AM(imax, j));
            if (x > v) { v = x; iv = j; }
          }
          group_argmax<W>(v, iv, 1, red_v, red_i);
          double rowmax = v;
          if (imax > 1) {
            double v2 = -1.0;
            int iv2 = 1 << 30;
            for (int j = 1 + gt; j < imax; j += G) {
              const double x = fabs(AM(j, imax));
              if (x > v2) { v2 = x; iv2 = j; }
            }
            group_argmax<W>(v2, iv2, 1, red_v, red_i);
            rowmax = fmax(rowmax, v2);
          }
          if (absakk >= alpha * colmax * (colmax / rowmax)) kp = kk;
          else if (fabs(AM(imax, imax)) >= alpha * rowmax) kp = imax;
          else { kp = imax; kstep = 2; }
        }
        // every thread has read the pivot candidates (A(imax, imax) above) before the
        // interchange below overwrites them
        gsync<W>();
        const int kkk = kk - kstep + 1;
        if (kp != kkk) {
          for (int i = 1 + gt; i < kp; i += G) {
            const double t = AM(i, kkk); AM(i, kkk) = AM(i, kp); AM(i, kp) = t;
          }
          for (int j = kp + 1 + gt; j < kkk; j += G) {
            const double t = AM(j, kkk); AM(j, kkk) = AM(kp, j); AM(kp, j) = t;
          }
          if (gt == 0) {
            double t = AM(kkk, kkk); AM(kkk, kkk) = AM(kp, kp); AM(kp, kp) = t;
            if (kstep == 2) { t = AM(kk - 1, kk); AM(kk - 1, kk) = AM(kp, kk); AM(kp, kk) = t; }
          }
          gsync<W>();
        }
        if (kstep == 1) {
          const double r1 = ddiv(1.0, AM(kk, kk));
          // column multipliers temp_j = -r1 x_j (dsyr), then A(i,j) += A(i,kk) temp_j
          // for x_j != 0, one fused multiply-add per element
          for (int j = gt; j < kk - 1; j += G) TC[j] = dmul(-r1, AM(j + 1, kk));
          gsync<W>();
          const int Tu = (kk - 1) * kk / 2;
          int i0 = 0, j0 = 0;
          tri_next(i0, j0, gt);
          for (int t = gt; t < Tu; t += G, tri_next(i0, j0, G)) {
            if (AM(j0 + 1, kk) != 0.0)
              AM(i0 + 1, j0 + 1) = fma(AM(i0 + 1, kk), TC[j0], AM(i0 + 1, j0 + 1));
          }
          gsync<W>();
          for (int i = 1 + gt; i < kk; i += G) AM(i, kk) = dmul(r1, AM(i, kk));
          gsync<W>();
        } else if (kk > 2) {
          const double d12o = AM(kk - 1, kk);
          const double d22 = ddiv(AM(kk - 1, kk - 1), d12o);
          const double d11 = ddiv(AM(kk, kk), d12o);
          const double tt = ddiv(1.0, dsub(dmul(d11, d22), 1.0));
          const double d12 = ddiv(tt, d12o);
          // wkm1, wk of every column j <= kk-2 from the original entries, then
          // A(i,j) -= A(i,kk) wk + A(i,kk-1) wkm1 as two fused multiply-adds, then
          // columns kk-1, kk take wkm1, wk (dsytf2 order: each update reads only
          // rows i <= j, which the column overwrite has not reached)
          for (int j = gt; j < kk - 2; j += G) {
            const double a1 = AM(j + 1, kk - 1), a2 = AM(j + 1, kk);
            TC[j] = dmul(d12, dsub(dmul(d11, a1), a2));
            TC2[j] = dmul(d12, dsub(dmul(d22, a2), a1));
          }
          gsync<W>();
          const int Tu = (kk - 2) * (kk - 1) / 2;
          int i0 = 0, j0 = 0;
          tri_next(i0, j0, gt);
          for (int t = gt; t < Tu; t += G, tri_next(i0, j0, G)) {
            const int j = j0 + 1, i = i0 + 1;
            AM(i, j) = fma(-AM(i, kk - 1), TC[j0], fma(-AM(i, kk), TC2[j0], AM(i, j)));
          }
          gsync<W>();
          for (int j = gt; j < kk - 2; j += G) {
            AM(j + 1, kk) = TC2[j];
            AM(j + 1, kk - 1) = TC[j];
          }
          gsync<W>();
        }
      }
      if (gt == 0) {
        if (kstep == 1) ipiv[kk - 1] = kp;
        else { ipiv[kk - 1] = -kp; ipiv[kk - 2] = -kp; }
      }
      gsync<W>();
      kk -= kstep;
    }

    if (info != 0) {
      if (gt == 0) atomicMin(a.bad, (int)e);
      for (int t = gt; t < k * dim; t += G) w_out[(rb + t / dim) * dim + t % dim] = NAN;
      if (resid && gt == 0) resid[e] = NAN;
      gsync<W>();
      continue;
    }

    gsync<W>();  // factorisation complete and visible to the solving warp
    if (W == 1 || wib == 0) {
    // ---------------- solve (dsytrs, upper), columns independent
    const int nrhs = dim;
    kk = n;
    while (kk >= 1) {
      if (ipiv[kk - 1] > 0) {
        const int kp = ipiv[kk - 1];
        if (kp != kk && lane < nrhs) {
          const double t = BM(kk, lane); BM(kk, lane) = BM(kp, lane); BM(kp, lane) = t;
        }
        __syncwarp();
        for (int c = 0; c < nrhs; ++c) {
          const double bk = BM(kk, c);
          if (bk != 0.0) {
            const double temp = -bk;
            for (int i = 1 + lane; i < kk; i += 32) BM(i, c) = fma(AM(i, kk), temp, BM(i, c));
          }
        }
        __syncwarp();
        const double r = ddiv(1.0, AM(kk, kk));
        if (lane < nrhs) BM(kk, lane) = dmul(r, BM(kk, lane));
        __syncwarp();
        kk -= 1;
      } else {
        const int kp = -ipiv[kk - 1];
        if (kp != kk - 1 && lane < nrhs) {
          const double t = BM(kk - 1, lane); BM(kk - 1, lane) = BM(kp, lane); BM(kp, lane) = t;
        }
        __syncwarp();
        for (int c = 0; c < nrhs; ++c) {
          const double bk = BM(kk, c);
          const double bkm1 = BM(kk - 1, c);
          for (int i = 1 + lane; i <= kk - 2; i += 32) {
            double v = BM(i, c);
            if (bk != 0.0) v = fma(AM(i, kk), -bk, v);
            if (bkm1 != 0.0) v = fma(AM(i, kk - 1), -bkm1, v);
            BM(i, c) = v;
          }
        }
        __syncwarp();
        if (lane < nrhs) {
          const double akm1k = AM(kk - 1, kk);
          const double akm1 = ddiv(AM(kk - 1, kk - 1), akm1k);
          const double ak = ddiv(AM(kk, kk), akm1k);
          const double denom = dsub(dmul(akm1, ak), 1.0);
          const double bkm1 = ddiv(BM(kk - 1, lane), akm1k);
          const double bk = ddiv(BM(kk, lane), akm1k);
          BM(kk - 1, lane) = ddiv(dsub(dmul(ak, bkm1), bk), denom);
          BM(kk, lane) = ddiv(dsub(dmul(akm1, bk), bkm1), denom);
        }
        __syncwarp();
        kk -= 2;
      }
    }
    kk = 1;
    while (kk <= n) {
      const bool one = ipiv[kk - 1] > 0;
      const int ncol = one ? 1 : 2;
      for (int c = 0; c < nrhs; ++c)
        for (int q = 0; q < ncol; ++q) {
          // dot product in a fixed 32-way strided order, then a pairwise tree
          double part = 0.0;
          for (int i = 1 + lane; i < kk; i += 32) part = fma(BM(i, c), AM(i, kk + q), part);
          for (int o = 16; o > 0; o >>= 1) part = dadd(part, __shfl_down_sync(kFull, part, o));
          if (lane == 0) BM(kk + q, c) = dadd(BM(kk + q, c), dmul(-1.0, part));
          __syncwarp();
        }
      const int kp = one ? ipiv[kk - 1] : -ipiv[kk - 1];
      if (kp != kk && lane < nrhs) {
        const double t = BM(kk, lane); BM(kk, lane) = BM(kp, lane); BM(kp, lane) = t;
      }
      __syncwarp();
      kk += ncol;
    }

    // weights: s_d^order * w[1:k, d]
    for (int t = lane; t < k * dim; t += 32) {
      const int j = t / dim, d = t % dim;
      w_out[(rb + j) * dim + d] = dmul(pow_int(s[d], order), BM(j + 1, d));
    }
    if (resid) {
      // ||M w - b||_inf / ||b||_inf per column, M and b re-evaluated from X^
      double worst = 0.0;
      for (int d = 0; d < dim; ++d) {
        double rn = 0.0, bn = 0.0;
        for (int r = lane; r < n; r += 32) {
          double acc = 0.0;
          for (int cidx = 0; cidx < n; ++cidx) {
            const int lo = min(r, cidx), hi = max(r, cidx);
            double v;
            if (hi < k) {
              double d2 = 0.0;
              for (int dd = 0; dd < dim; ++dd) {
                const double tt = dsub(X[lo * 3 + dd], X[hi * 3 + dd]);
                d2 = dadd(d2, dmul(tt, tt));
              }
              v = pow_int(sqrt(d2), rbf_pow);
            } else if (lo < k) {
              const int* ex = a.g[grp].mono[hi - k];
              v = 1.0;
              for (int dd = 0; dd < dim; ++dd) v = dmul(v, pow_int(X[lo * 3 + dd], ex[dd]));
            } else {
              v = 0.0;
            }
            acc += v * BM(cidx + 1, d);
          }
          double bv;
          if (r < k) {
            double pt[3];
            for (int dd = 0; dd < dim; ++dd) pt[dd] = r == 0 ? 2.220446049250313e-16 : -X[r * 3 + dd];
            double d2 = 0.0;
            for (int dd = 0; dd < dim; ++dd) d2 = dadd(d2, dmul(pt[dd], pt[dd]));
            bv = phs_deriv(rbf_pow, order, pt[d], sqrt(d2));
          } else {
            const int* ex = a.g[grp].mono[r - k];
            bool ok = true;
            for (int dd = 0; dd < dim; ++dd)
              if (ex[dd] != (dd == d ? order : 0)) ok = false;
            bv = ok ? fact(order) : 0.0;
          }
          rn = fmax(rn, fabs(acc - bv));
          bn = fmax(bn, fabs(bv));
        }
        rn = warp_max(rn);
        bn = warp_max(bn);
        worst = fmax(worst, bn > 0 ? rn / bn : rn);
      }
      if (lane == 0) resid[e] = worst;
    }
    __syncwarp();
    }
#undef AM
#undef BM
  }
}

int make_monomials(int dim, int deg, int (*ex)[3], int cap) {
  int m = 0;
  for (int q = 0; q <= deg; ++q) {
    if (dim == 1) {
      if (m < cap) { ex[m][0] = q; ex[m][1] = 0; ex[m][2] = 0; }
      m++;
      continue;
    }
    for (int a = q; a >= 0; --a) {
      if (dim == 2) {
        if (m < cap) { ex[m][0] = a; ex[m][1] = q - a; ex[m][2] = 0; }
        m++;
        continue;
      }
      for (int b = q - a; b >= 0; --b) {
        if (m < cap) { ex[m][0] = a; ex[m][1] = b; ex[m][2] = q - a - b; }
        m++;
      }
    }
  }
  return m;
}

}  // namespace

// Host description of one group of a weight batch (host arrays).
struct HostGroup {
  int dim, rbf_pow, polydeg, order;
  const double* period;  // dim lengths or null
  int64_t n;
  const double* d_xyz;   // device coordinates (n x dim)
  const int64_t* rowptr; // host, n + 1
  const int32_t* cols;   // host, rowptr[n]
  double* w_out;         // host, rowptr[n] x dim
};

// All groups' systems, largest first, in persistent launches over size buckets of the
// system order n = k + monomials (one launch per non-empty bucket, each with the shared
// memory and occupancy its largest system allows).
constexpr int kBucketEdges[] = {48, 64, 80, 104};

static void weights_run(cudaStream_t s, const std::vector<HostGroup>& gs, double* max_resid) {
  MFT_REQUIRE(!gs.empty() && gs.size() <= (size_t)kMaxGroups, MFT_ERR_ARG,
              "between 1 and 2 weight groups");
  WArgs a{};
  int kmax = 0, nmax = 0;
  int64_t nsys = 0;
  std::vector<int64_t> order;
  std::vector<int> ks, ns;
  int64_t total = 0;
  for (const HostGroup& h : gs) total += h.n;
  order.reserve(total);
  ks.reserve(total);
  ns.reserve(total);
  for (size_t g = 0; g < gs.size(); ++g) {
    const HostGroup& h = gs[g];
    WGroup& G = a.g[g];
    G.dim = h.dim;
    G.npoly = make_monomials(h.dim, h.polydeg, G.mono, kMaxMono);
    MFT_REQUIRE(G.npoly <= kMaxMono, MFT_ERR_ARG, "polynomial degree too high");
    G.rbf_pow = h.rbf_pow;
    G.order = h.order;
    G.periodic = h.period ? 1 : 0;
    for (int d = 0; d < 3; ++d) G.period[d] = (h.period && d < h.dim) ? h.period[d] : 0.0;
    int km = 0;
    for (int64_t i = 0; i < h.n; ++i) {
      const int k = (int)(h.rowptr[i + 1] - h.rowptr[i]);
      MFT_REQUIRE(k >= 1, MFT_ERR_ARG, "empty stencil");
      km = std::max(km, k);
      order.push_back(((int64_t)g << kGroupShift) | i);
      ks.push_back(k);
      ns.push_back(k + G.npoly);
    }
    kmax = std::max(kmax, km);
    nmax = std::max(nmax, km + G.npoly);
    nsys += h.n;
  }
  // systems by size, largest first, ties in input order: a counting sort on n
  std::vector<int64_t> perm(order.size());
  {
    std::vector<int64_t> start((size_t)nmax + 2, 0);
    for (int v : ns) start[(size_t)(nmax - v) + 1]++;
    for (size_t q = 1; q < start.size(); ++q) start[q] += start[q - 1];
    for (size_t q = 0; q < ns.size(); ++q) perm[start[(size_t)(nmax - ns[q])]++] = (int64_t)q;
  }
  std::vector<int64_t> order_sorted(order.size());
  for (size_t q = 0; q < perm.size(); ++q) order_sorted[q] = order[perm[q]];
  (void)kmax;
  MFT_REQUIRE(weights_smem_doubles(nmax, nmax) * sizeof(double) * kWarpsPerBlock <=
                  227 * 1024 - 256,
              MFT_ERR_ARG, "stencil too large for the weight kernel");
  // buckets: [begin, end) ranges of the sorted list with their largest n and k
  struct Bucket { int64_t begin, end; int nmax, kmax; };
  std::vector<Bucket> buckets;
  auto bucket_of = [](int n) {
    int b = 0;
    for (int edge : kBucketEdges) { if (n <= edge) return b; ++b; }
    return b;
  };
  for (size_t q = 0; q < perm.size(); ++q) {
    const int n = ns[perm[q]], k = ks[perm[q]];
    if (buckets.empty() || bucket_of(n) != bucket_of(buckets.back().nmax))
      buckets.push_back({(int64_t)q, (int64_t)q, n, k});
    Bucket& b = buckets.back();
    b.end = (int64_t)q + 1;
    b.kmax = std::max(b.kmax, k);
  }
  DBuf<int64_t> d_order, d_rp[kMaxGroups];
  DBuf<int32_t> d_ci[kMaxGroups];
  DBuf<double> d_w[kMaxGroups], d_res[kMaxGroups];
  DBuf<int> d_bad;
  DBuf<unsigned long long> d_next;
  d_order.upload(order_sorted, s);
  for (size_t g = 0; g < gs.size(); ++g) {
    const HostGroup& h = gs[g];
    const int64_t nnz = h.rowptr[h.n];
    d_rp[g].upload(h.rowptr, h.n + 1, s);
    d_ci[g].upload(h.cols, nnz, s);
    d_w[g].alloc((size_t)nnz * h.dim);
    if (max_resid) d_res[g].alloc(h.n);
    a.g[g].rowptr = d_rp[g].p;
    a.g[g].cols = d_ci[g].p;
    a.g[g].xyz = h.d_xyz;
    a.g[g].w_out = d_w[g].p;
    a.g[g].resid = max_resid ? d_res[g].p : nullptr;
  }
  d_bad.alloc(1);
  const int big = 0x7fffffff;
  MFT_CUDA(cudaMemcpyAsync(d_bad.p, &big, sizeof(int), cudaMemcpyHostToDevice, s));
  d_next.alloc(buckets.size());
  d_next.zero(s);
  a.bad = d_bad.p;
  int dev = 0, sms = 0;
  MFT_CUDA(cudaGetDevice(&dev));
  MFT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  for (size_t b = 0; b < buckets.size(); ++b) {
    const Bucket& bk = buckets[b];
    WArgs ab = a;
    ab.nmax = bk.nmax;
    ab.kmax = bk.kmax;
    ab.nsys = bk.end - bk.begin;
    ab.order_list = d_order.p + bk.begin;
    ab.next = d_next.p + b;
    const bool multi = bk.nmax > kMultiWarpMinN;
    const int spb = multi ? 1 : kWarpsPerBlock;  // systems per block
    const int threads = multi ? 32 * kSystemWarps : 32 * kWarpsPerBlock;
    const size_t shmem = weights_smem_doubles(bk.nmax, bk.kmax) * sizeof(double) * spb;
    // the opt-in dynamic shared memory this bucket needs (the static part is small)
    int per_sm = 0;
    if (multi) {
      MFT_CUDA(cudaFuncSetAttribute(k_weights<true, kSystemWarps>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem));
      MFT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, k_weights<true, kSystemWarps>, threads, shmem));
    } else {
      MFT_CUDA(cudaFuncSetAttribute(k_weights<true, 1>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem));
      MFT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_weights<true, 1>,
                                                             threads, shmem));
    }
    per_sm = std::max(per_sm, 1);
    const int64_t want = (ab.nsys + spb - 1) / spb;
    const unsigned grid =
        (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * per_sm, want));
    if (multi) k_weights<true, kSystemWarps><<<grid, threads, shmem, s>>>(ab);
    else k_weights<true, 1><<<grid, threads, shmem, s>>>(ab);
    MFT_LAUNCH_CHECK();
  }
  int bad = big;
  std::vector<std::vector<double>> res(gs.size());
  for (size_t g = 0; g < gs.size(); ++g) {
    const HostGroup& h = gs[g];
    MFT_CUDA(cudaMemcpyAsync(h.w_out, d_w[g].p, (size_t)h.rowptr[h.n] * h.dim * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
    if (max_resid) {
      res[g].resize(h.n);
      MFT_CUDA(cudaMemcpyAsync(res[g].data(), d_res[g].p, h.n * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    }
  }
  MFT_CUDA(cudaMemcpyAsync(&bad, d_bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  MFT_CUDA(cudaStreamSynchronize(s));
  MFT_REQUIRE(bad == big, MFT_ERR_SINGULAR,
              "saddle-point system of node " + std::to_string(bad) + " has an exactly zero pivot");
  if (max_resid) {
    double m = 0.0;
    for (auto& r : res)
      for (double x : r) m = std::max(m, x);
    *max_resid = m;
  }
}

void weights_device(mft_ctx* c, int rbf_pow, int polydeg, int deriv_order,
                    std::vector<double>& w_out, double* max_resid) {
  HostGroup h{};
  h.dim = c->dim;
  h.rbf_pow = rbf_pow;
  h.polydeg = polydeg;
  h.order = deriv_order;
  h.period = c->periodic ? c->period : nullptr;
  h.n = c->n;
  h.d_xyz = c->d_xyz.p;
  h.rowptr = c->st_rp.data();
  h.cols = c->st_ci.data();
  w_out.resize((size_t)c->st_ci.size() * c->dim);
  h.w_out = w_out.data();
  weights_run(c->stream, {h}, max_resid);
}

void weights_batch(mft_ctx* c, int ngroups, const mft_weight_group* groups, double* max_resid) {
  MFT_REQUIRE(ngroups >= 1 && ngroups <= kMaxGroups && groups, MFT_ERR_ARG,
              "between 1 and 2 weight groups");
  std::vector<HostGroup> hs(ngroups);
  std::vector<DBuf<double>> xyz(ngroups);
  for (int g = 0; g < ngroups; ++g) {
    const mft_weight_group& q = groups[g];
    MFT_REQUIRE(q.dim >= 1 && q.dim <= 3 && q.n >= 1 && q.xyz && q.rowptr && q.cols && q.w,
                MFT_ERR_ARG, "bad weight group");
    MFT_REQUIRE(q.rbf_pow >= 1 && q.polydeg >= 0 && q.polydeg <= 6 && q.deriv_order >= 1 &&
                    q.deriv_order <= 8, MFT_ERR_ARG, "bad basis or derivative order");
    MFT_REQUIRE(q.rowptr[0] == 0, MFT_ERR_ARG, "rowptr[0] must be 0");
    for (int64_t i = 0; i < q.n; ++i) {
      MFT_REQUIRE(q.rowptr[i + 1] > q.rowptr[i], MFT_ERR_ARG, "empty stencil");
      for (int64_t p = q.rowptr[i]; p < q.rowptr[i + 1]; ++p)
        MFT_REQUIRE(q.cols[p] >= 0 && q.cols[p] < q.n, MFT_ERR_ARG, "stencil index out of range");
    }
    xyz[g].upload(q.xyz, (size_t)q.n * q.dim, c->stream);
    HostGroup& h = hs[g];
    h.dim = q.dim;
    h.rbf_pow = q.rbf_pow;
    h.polydeg = q.polydeg;
    h.order = q.deriv_order;
    h.period = nullptr;
    h.n = q.n;
    h.d_xyz = xyz[g].p;
    h.rowptr = q.rowptr;
    h.cols = q.cols;
    h.w_out = q.w;
  }
  weights_run(c->stream, hs, max_resid);
}

}  // namespace mft

// ---------------------------------------------------------------- allocation-free variant
//
// mft_weights_noalloc is for callers that cannot allocate device memory while they
// compute weights: a solver running inside a stream-ordered memory pool it does not own,
// a host that has handed all device memory to its own allocator, or code that must not
// call cudaMalloc/cudaFree because those calls synchronise the device.  The caller passes
// every input and output as device memory; the only global scratch the solve needs (the
// work counter and two status words) lives in the file-scope array below.

namespace {

// [0] work counter, [1] first node with a zero pivot (low 32 bits, 0x7F7F7F7F = none),
// [2] oversize-stencil flag, [3] invalid-stencil flag (empty or decreasing rowptr, a row
// outside cols, a column that is not a node).  32 bytes on every GPU that loads the
// library, held until the process exits.
constexpr int kNoAllocWords = 4;
static __device__ __align__(256) unsigned long long g_weights_scratch[kNoAllocWords];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_scratch_mu;
unsigned long long* g_scratch_addr[kNoAllocMaxDevices] = {};

void put_err(char* err, int len, const std::string& msg) {
  if (err && len > 0) {
    const size_t m = std::min<size_t>((size_t)len - 1, msg.size());
    memcpy(err, msg.data(), m);
    err[m] = '\0';
  }
}

}  // namespace

extern "C" mft_status mft_weights_noalloc(int dim, int64_t n, const double* xyz,
                                          const double* period, const int64_t* rowptr,
                                          const int32_t* cols, int kmax, int rbf_pow,
                                          int polydeg, int deriv_order, double* w,
                                          void* stream, char* err, int err_len) {
  using namespace mft;
  put_err(err, err_len, "");
  if (dim < 1 || dim > 3 || n < 1 || n > (int64_t)INT32_MAX || !xyz || !rowptr || !cols || !w ||
      kmax < 1 || rbf_pow < 1 || rbf_pow > 15 || polydeg < 0 || polydeg > 6 || deriv_order < 1 ||
      deriv_order > 8) {
    put_err(err, err_len, "mft_weights_noalloc: invalid argument");
    return MFT_ERR_ARG;
  }
  WArgs a{};
  WGroup& G = a.g[0];
  G.dim = dim;
  G.npoly = make_monomials(dim, polydeg, G.mono, kMaxMono);
  G.rbf_pow = rbf_pow;
  G.order = deriv_order;
  G.periodic = period ? 1 : 0;
  for (int d = 0; d < 3; ++d) G.period[d] = (period && d < dim) ? period[d] : 0.0;
  a.kmax = kmax;
  a.nmax = kmax + G.npoly;
  const size_t shmem = weights_smem_doubles(a.nmax, kmax) * sizeof(double) * kWarpsPerBlock;
  const size_t kMaxShmem = 227 * 1024;
  if (G.npoly > kMaxMono || shmem > kMaxShmem) {
    put_err(err, err_len,
            "mft_weights_noalloc: stencil size " + std::to_string(kmax) + " plus " +
                std::to_string(G.npoly) + " monomials needs " + std::to_string(shmem) +
                " bytes of shared memory; the maximum is " + std::to_string(kMaxShmem) +
                " (kmax + monomials <= 161)");
    return MFT_ERR_ARG;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
    put_err(err, err_len, "mft_weights_noalloc: no current CUDA device");
    return MFT_ERR_CUDA;
  }
  unsigned long long* scratch = nullptr;
  {
    // First call on this device (with it current): resolve the device address of the
    // scratch array.  Later calls reuse it.  Make the first call before any capture.  The
    // address is kept for the life of the process: a cudaDeviceReset after the first call
    // on a device is not supported (the kept address would be stale).
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      void* ptr = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&ptr, g_weights_scratch);
      if (e != cudaSuccess || !ptr) {
        put_err(err, err_len, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return MFT_ERR_CUDA;
      }
      g_scratch_addr[dev] = reinterpret_cast<unsigned long long*>(ptr);
    }
    scratch = g_scratch_addr[dev];
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  // the counter and the status words must start from their initial values
  if (cudaMemsetAsync(scratch, 0, sizeof(unsigned long long), s) != cudaSuccess ||
      cudaMemsetAsync(scratch + 1, 0x7F, sizeof(int), s) != cudaSuccess ||
      cudaMemsetAsync(scratch + 2, 0, 2 * sizeof(unsigned long long), s) != cudaSuccess) {
    put_err(err, err_len, "mft_weights_noalloc: cudaMemsetAsync failed");
    return MFT_ERR_CUDA;
  }
  a.nsys = n;
  a.order_list = nullptr;
  G.rowptr = rowptr;
  G.cols = cols;
  G.xyz = xyz;
  G.w_out = w;
  G.resid = nullptr;
  a.bad = reinterpret_cast<int*>(scratch + 1);
  a.next = scratch;
  int sms = 0, per_sm = 0;
  if (cudaFuncSetAttribute(k_weights<false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)shmem) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_weights<false, 1>,
                                                    32 * kWarpsPerBlock, shmem) != cudaSuccess) {
    put_err(err, err_len, "mft_weights_noalloc: kernel configuration failed");
    return MFT_ERR_CUDA;
  }
  per_sm = std::max(per_sm, 1);
  const int64_t want = (n + kWarpsPerBlock - 1) / kWarpsPerBlock;
  const unsigned grid =
      (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * per_sm, want));
  k_weights<false, 1><<<grid, 32 * kWarpsPerBlock, shmem, s>>>(a);
  cudaError_t e = cudaGetLastError();
  int status[3] = {0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status[0], scratch + 1, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status[1], scratch + 2, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status[2], scratch + 3, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    put_err(err, err_len, std::string("mft_weights_noalloc: ") + cudaGetErrorString(e));
    return MFT_ERR_CUDA;
  }
  if (status[2] != 0) {
    put_err(err, err_len,
            "mft_weights_noalloc: a stencil is empty, leaves cols (rowptr not increasing "
            "up to rowptr[n]) or lists a column outside 0..n-1; its weights are NaN");
    return MFT_ERR_ARG;
  }
  if (status[1] != 0) {
    put_err(err, err_len, "mft_weights_noalloc: a stencil is longer than kmax = " +
                              std::to_string(kmax) + "; its weights were not computed (NaN)");
    return MFT_ERR_ARG;
  }
  if (status[0] != 0x7F7F7F7F) {
    put_err(err, err_len, "mft_weights_noalloc: node " + std::to_string(status[0]) +
                              " has an exactly zero pivot");
    return MFT_ERR_SINGULAR;
  }
  return MFT_OK;
}
