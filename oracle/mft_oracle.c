/*
 * mft_oracle.c -- CPU restatement of the MeshfreeTrixi.jl RBF-FD hot path.
 * TEST INFRASTRUCTURE ONLY (the checker); see mft_oracle.h for what is pinned.
 * Every function cites the reference file:line whose behaviour it restates.
 * Build: gcc -O2 -ffp-contract=off -fopenmp -fPIC -shared (no FMA contraction).
 */
#include "mft_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define JL_EPS 2.220446049250313e-16 /* eps(Float64) */

/* ------------------------------------------------------------------------ */
/* Julia Base semantics used by the reference                                */
/* ------------------------------------------------------------------------ */

/* Base.mapreduce_impl(identity, +, A, lo, hi, 1024), inclusive bounds. */
static double pairwise(const double* x, int64_t lo, int64_t hi, int64_t s) {
  if (lo == hi) return x[lo * s];
  if (hi - lo < 1024) {
    double v = x[lo * s] + x[(lo + 1) * s];
    for (int64_t i = lo + 2; i <= hi; ++i) v = v + x[i * s];
    return v;
  }
  int64_t mid = lo + ((hi - lo) >> 1);
  double a = pairwise(x, lo, mid, s);
  double b = pairwise(x, mid + 1, hi, s);
  return a + b;
}

double mfto_pairwise_sum(const double* x, int64_t n, int64_t stride) {
  if (n <= 0) return 0.0;
  if (n == 1) return x[0];
  if (n < 16) { /* Base._mapreduce short-array branch: plain left fold */
    double v = x[0] + x[stride];
    for (int64_t i = 2; i < n; ++i) v = v + x[i * stride];
    return v;
  }
  return pairwise(x, 0, n - 1, stride);
}

/* Base.isless / isequal on Float64 (NaN greatest, -0.0 < 0.0). */
static int jl_isless(double a, double b) {
  if (isnan(a)) return 0;
  if (isnan(b)) return 1;
  if (a < b) return 1;
  if (a > b) return 0;
  return signbit(a) && !signbit(b);
}
static int jl_isequal(double a, double b) {
  if (isnan(a) || isnan(b)) return isnan(a) && isnan(b);
  return a == b && signbit(a) == signbit(b);
}
/* Base.isless(::AbstractVector, ::AbstractVector): lexicographic via cmp. */
static int jl_vec_isless(const double* a, const double* b, int n) {
  for (int i = 0; i < n; ++i)
    if (!jl_isequal(a[i], b[i])) return jl_isless(a[i], b[i]);
  return 0;
}
/* Base.max/min on Float64: NaN propagating, signed zeros ordered. */
static double jl_max(double a, double b) {
  if (isnan(a) || isnan(b)) return a + b;
  return jl_isless(a, b) ? b : a;
}
static double jl_min(double a, double b) {
  if (isnan(a) || isnan(b)) return a + b;
  return jl_isless(b, a) ? b : a;
}

static double pow_int(double x, int k) {
  if (k < 0) return 1.0 / pow_int(x, -k);
  double r = 1.0;
  for (int i = 0; i < k; ++i) r = r * x;
  return r;
}

static int nthreads_or_default(int nt) { return nt > 0 ? nt : 1; }

/* ------------------------------------------------------------------------ */
/* A1  KNN  geometry_primatives.jl:322-339                                   */
/* ------------------------------------------------------------------------ */

typedef struct {
  double d2;
  int32_t j;
} cand_t;

static int cand_cmp(const void* pa, const void* pb) {
  const cand_t* a = (const cand_t*)pa;
  const cand_t* b = (const cand_t*)pb;
  if (a->d2 < b->d2) return -1;
  if (a->d2 > b->d2) return 1;
  return (a->j > b->j) - (a->j < b->j);
}

static double min_image(double d, double L) {
  if (L <= 0.0) return d;
  if (d > 0.5 * L) return d - L;
  if (d < -0.5 * L) return d + L;
  return d;
}

/* Squared distance, summed over dims in order, each square rounded (no FMA). */
static double dist2(int dim, const double* a, const double* b, const double* period) {
  double s = 0.0;
  for (int d = 0; d < dim; ++d) {
    double t = b[d] - a[d];
    if (period) t = min_image(t, period[d]);
    double sq = t * t;
    s = s + sq;
  }
  return s;
}

int mfto_knn(int dim, int64_t n, const double* x, const double* period, int k, int32_t* idx,
             double* dists, double* dx_min, double* dx_avg, int nthreads) {
  if (dim < 1 || dim > 3 || n < 1 || k < 1 || k > n) return -1;
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) {
    lo[d] = hi[d] = x[d];
    for (int64_t i = 1; i < n; ++i) {
      double v = x[i * dim + d];
      if (v < lo[d]) lo[d] = v;
      if (v > hi[d]) hi[d] = v;
    }
  }
  double vol = 1.0;
  for (int d = 0; d < dim; ++d) {
    double ext = period ? period[d] : (hi[d] - lo[d]);
    if (ext <= 0.0) ext = 1.0;
    vol *= ext;
  }
  double cs = pow(vol * 2.0 / (double)n, 1.0 / dim); /* about two nodes per cell */
  int64_t nc[3] = {1, 1, 1};
  double csd[3] = {cs, cs, cs};
  for (int d = 0; d < dim; ++d) {
    double ext = period ? period[d] : (hi[d] - lo[d]);
    int64_t m = (int64_t)floor(ext / cs);
    if (m < 1) m = 1;
    if (m > 4096) m = 4096;
    nc[d] = m;
    csd[d] = period ? period[d] / (double)m : (ext > 0 ? ext / (double)m : 1.0);
    if (!period) csd[d] *= (1.0 + 1e-12);
  }
  int64_t ncell = nc[0] * nc[1] * nc[2];
  int64_t* cstart = (int64_t*)calloc((size_t)ncell + 1, sizeof(int64_t));
  int64_t* cell_of = (int64_t*)malloc((size_t)n * sizeof(int64_t));
  int32_t* cpts = (int32_t*)malloc((size_t)n * sizeof(int32_t));
  if (!cstart || !cell_of || !cpts) {
    free(cstart); free(cell_of); free(cpts);
    return -2;
  }
  for (int64_t i = 0; i < n; ++i) {
    int64_t c = 0, mul = 1;
    for (int d = 0; d < dim; ++d) {
      int64_t ci = (int64_t)floor((x[i * dim + d] - lo[d]) / csd[d]);
      if (ci < 0) ci = 0;
      if (ci >= nc[d]) ci = nc[d] - 1;
      c += ci * mul;
      mul *= nc[d];
    }
    cell_of[i] = c;
    cstart[c + 1]++;
  }
  for (int64_t c = 0; c < ncell; ++c) cstart[c + 1] += cstart[c];
  {
    int64_t* fill = (int64_t*)malloc((size_t)ncell * sizeof(int64_t));
    memcpy(fill, cstart, (size_t)ncell * sizeof(int64_t));
    for (int64_t i = 0; i < n; ++i) cpts[fill[cell_of[i]]++] = (int32_t)i;
    free(fill);
  }

  double* nn = (double*)malloc((size_t)n * sizeof(double));
  int err = 0;
#pragma omp parallel num_threads(nthreads_or_default(nthreads))
  {
    size_t cap = 1024;
    cand_t* cand = (cand_t*)malloc(cap * sizeof(cand_t));
#pragma omp for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
      const double* q = x + i * dim;
      int64_t qc[3] = {0, 0, 0};
      {
        int64_t c = cell_of[i];
        for (int d = 0; d < dim; ++d) { qc[d] = c % nc[d]; c /= nc[d]; }
      }
      for (int r = 1;; ++r) {
        size_t nc_ = 0;
        int full[3] = {1, 1, 1};
        int64_t a0[3] = {0, 0, 0}, a1[3] = {0, 0, 0};
        for (int d = 0; d < 3; ++d) {
          if (d >= dim) { a0[d] = 0; a1[d] = 0; continue; }
          if (period) {
            if (2 * r + 1 >= nc[d]) { a0[d] = 0; a1[d] = nc[d] - 1; full[d] = 1; }
            else { a0[d] = qc[d] - r; a1[d] = qc[d] + r; full[d] = 0; }
          } else {
            a0[d] = qc[d] - r < 0 ? 0 : qc[d] - r;
            a1[d] = qc[d] + r >= nc[d] ? nc[d] - 1 : qc[d] + r;
            full[d] = (a0[d] == 0 && a1[d] == nc[d] - 1);
          }
        }
        for (int64_t c2 = a0[2]; c2 <= a1[2]; ++c2)
          for (int64_t c1 = a0[1]; c1 <= a1[1]; ++c1)
            for (int64_t c0 = a0[0]; c0 <= a1[0]; ++c0) {
              int64_t w0 = c0, w1 = c1, w2 = c2;
              if (period) {
                w0 = ((c0 % nc[0]) + nc[0]) % nc[0];
                w1 = ((c1 % nc[1]) + nc[1]) % nc[1];
                w2 = ((c2 % nc[2]) + nc[2]) % nc[2];
              }
              int64_t c = w0 + nc[0] * (w1 + nc[1] * w2);
              for (int64_t p = cstart[c]; p < cstart[c + 1]; ++p) {
                int32_t j = cpts[p];
                if (nc_ == cap) {
                  cap *= 2;
                  cand = (cand_t*)realloc(cand, cap * sizeof(cand_t));
                }
                cand[nc_].d2 = dist2(dim, q, x + (int64_t)j * dim, period);
                cand[nc_].j = j;
                nc_++;
              }
            }
        int all = 1;
        double bound = INFINITY;
        for (int d = 0; d < dim; ++d) {
          if (full[d]) continue;
          all = 0;
          if (period) {
            double l = q[d] - (lo[d] + (double)(qc[d] - r) * csd[d]);
            double h = (lo[d] + (double)(qc[d] + r + 1) * csd[d]) - q[d];
            bound = fmin(bound, fmin(l, h));
          } else {
            if (a0[d] > 0) bound = fmin(bound, q[d] - (lo[d] + (double)a0[d] * csd[d]));
            if (a1[d] < nc[d] - 1) bound = fmin(bound, (lo[d] + (double)(a1[d] + 1) * csd[d]) - q[d]);
          }
        }
        if ((int64_t)nc_ >= k) {
          qsort(cand, nc_, sizeof(cand_t), cand_cmp);
          double kth = cand[k - 1].d2;
          if (all || (bound > 0 && kth < bound * bound * (1.0 - 1e-9))) {
            for (int m = 0; m < k; ++m) {
              idx[i * k + m] = cand[m].j;
              if (dists) dists[i * k + m] = sqrt(cand[m].d2);
            }
            nn[i] = k >= 2 ? sqrt(cand[1].d2) : NAN;
            break;
          }
        } else if (all) {
#pragma omp atomic write
          err = -3;
          break;
        }
      }
    }
    free(cand);
  }
  if (!err) {
    if (dx_min) {
      double m = INFINITY;
      for (int64_t i = 0; i < n; ++i) m = jl_min(m, nn[i]);
      *dx_min = m;
    }
    if (dx_avg) *dx_avg = mfto_pairwise_sum(nn, n, 1) / (double)n;
  }
  free(nn);
  free(cstart);
  free(cell_of);
  free(cpts);
  return err;
}

/* ------------------------------------------------------------------------ */
/* Bunch-Kaufman LDL^T, upper storage (restating LAPACK dsytf2 + dsytrs,     */
/* the factorisation behind `Symmetric \` at compute_operators.jl:435)       */
/* ------------------------------------------------------------------------ */
/* The rank-1 / rank-2 updates and the solve's axpy and dot products use explicit
 * fused multiply-adds (one rounding per update, as optimised BLAS kernels do); the
 * device solver performs the same operations in the same order. */

#define AM(i, j) a[(size_t)((j)-1) * (size_t)n + (size_t)((i)-1)]
#define BM(i, c) b[(size_t)(c) * (size_t)n + (size_t)((i)-1)]

static int bk_factor(int n, double* a, int* ipiv) {
  const double alpha = (1.0 + sqrt(17.0)) / 8.0;
  int info = 0;
  int k = n;
  while (k >= 1) {
    int kstep = 1, kp;
    double absakk = fabs(AM(k, k));
    int imax = 0;
    double colmax = 0.0;
    if (k > 1) {
      imax = 1;
      colmax = fabs(AM(1, k));
      for (int i = 2; i < k; ++i)
        if (fabs(AM(i, k)) > colmax) { colmax = fabs(AM(i, k)); imax = i; }
    }
    if (fmax(absakk, colmax) == 0.0 || isnan(absakk)) {
      if (info == 0) info = k;
      kp = k;
    } else {
      if (absakk >= alpha * colmax) {
        kp = k;
      } else {
        int jmax = imax + 1;
        double rowmax = fabs(AM(imax, jmax));
        for (int j = imax + 2; j <= k; ++j)
          if (fabs(AM(imax, j)) > rowmax) { rowmax = fabs(AM(imax, j)); jmax = j; }
        if (imax > 1) {
          double v = fabs(AM(1, imax));
          for (int j = 2; j < imax; ++j)
            if (fabs(AM(j, imax)) > v) v = fabs(AM(j, imax));
          rowmax = fmax(rowmax, v);
        }
        if (absakk >= alpha * colmax * (colmax / rowmax)) kp = k;
        else if (fabs(AM(imax, imax)) >= alpha * rowmax) kp = imax;
        else { kp = imax; kstep = 2; }
      }
      int kk = k - kstep + 1;
      if (kp != kk) {
        for (int i = 1; i < kp; ++i) { double t = AM(i, kk); AM(i, kk) = AM(i, kp); AM(i, kp) = t; }
        for (int j = kp + 1; j < kk; ++j) { double t = AM(j, kk); AM(j, kk) = AM(kp, j); AM(kp, j) = t; }
        { double t = AM(kk, kk); AM(kk, kk) = AM(kp, kp); AM(kp, kp) = t; }
        if (kstep == 2) { double t = AM(k - 1, k); AM(k - 1, k) = AM(kp, k); AM(kp, k) = t; }
      }
      if (kstep == 1) {
        double r1 = 1.0 / AM(k, k);
        for (int j = 1; j < k; ++j) {
          double xj = AM(j, k);
          if (xj != 0.0) {
            double temp = -r1 * xj;
            for (int i = 1; i <= j; ++i) AM(i, j) = fma(AM(i, k), temp, AM(i, j));
          }
        }
        for (int i = 1; i < k; ++i) AM(i, k) = r1 * AM(i, k);
      } else if (k > 2) {
        double d12 = AM(k - 1, k);
        double d22 = AM(k - 1, k - 1) / d12;
        double d11 = AM(k, k) / d12;
        double t = 1.0 / (d11 * d22 - 1.0);
        d12 = t / d12;
        for (int j = k - 2; j >= 1; --j) {
          double wkm1 = d12 * (d11 * AM(j, k - 1) - AM(j, k));
          double wk = d12 * (d22 * AM(j, k) - AM(j, k - 1));
          for (int i = j; i >= 1; --i) AM(i, j) = fma(-AM(i, k - 1), wkm1, fma(-AM(i, k), wk, AM(i, j)));
          AM(j, k) = wk;
          AM(j, k - 1) = wkm1;
        }
      }
    }
    if (kstep == 1) ipiv[k - 1] = kp;
    else { ipiv[k - 1] = -kp; ipiv[k - 2] = -kp; }
    k -= kstep;
  }
  return info;
}

/* The dot products of dsytrs (DGEMV 'T') are summed in a fixed order: 32 strided
 * fused multiply-add partial sums (term i goes to partial (i-1) mod 32, ascending i),
 * then combined
 * pairwise (p[L] += p[L+16], then +8, +4, +2, +1).  LAPACK leaves this order to the
 * BLAS build; fixing it here lets the device solve be checked bit for bit. */
static double dot_strided(int m, const double* x, const double* y) {
  double p[32];
  for (int l = 0; l < 32; ++l) p[l] = 0.0;
  for (int i = 0; i < m; ++i) p[i & 31] = fma(x[i], y[i], p[i & 31]);
  for (int o = 16; o > 0; o >>= 1)
    for (int l = 0; l < o; ++l) p[l] = p[l] + p[l + o];
  return p[0];
}

static void bk_solve_factored(int n, const double* a, const int* ipiv, int nrhs, double* b) {
  int k = n;
  while (k >= 1) {
    if (ipiv[k - 1] > 0) {
      int kp = ipiv[k - 1];
      if (kp != k)
        for (int c = 0; c < nrhs; ++c) { double t = BM(k, c); BM(k, c) = BM(kp, c); BM(kp, c) = t; }
      for (int c = 0; c < nrhs; ++c) {
        double bk = BM(k, c);
        if (bk != 0.0) {
          double temp = -bk;
          for (int i = 1; i < k; ++i) BM(i, c) = fma(AM(i, k), temp, BM(i, c));
        }
      }
      double r = 1.0 / AM(k, k);
      for (int c = 0; c < nrhs; ++c) BM(k, c) = r * BM(k, c);
      k -= 1;
    } else {
      int kp = -ipiv[k - 1];
      if (kp != k - 1)
        for (int c = 0; c < nrhs; ++c) { double t = BM(k - 1, c); BM(k - 1, c) = BM(kp, c); BM(kp, c) = t; }
      for (int c = 0; c < nrhs; ++c) {
        double bk = BM(k, c);
        if (bk != 0.0) {
          double temp = -bk;
          for (int i = 1; i <= k - 2; ++i) BM(i, c) = fma(AM(i, k), temp, BM(i, c));
        }
      }
      for (int c = 0; c < nrhs; ++c) {
        double bk = BM(k - 1, c);
        if (bk != 0.0) {
          double temp = -bk;
          for (int i = 1; i <= k - 2; ++i) BM(i, c) = fma(AM(i, k - 1), temp, BM(i, c));
        }
      }
      double akm1k = AM(k - 1, k);
      double akm1 = AM(k - 1, k - 1) / akm1k;
      double ak = AM(k, k) / akm1k;
      double denom = akm1 * ak - 1.0;
      for (int c = 0; c < nrhs; ++c) {
        double bkm1 = BM(k - 1, c) / akm1k;
        double bk = BM(k, c) / akm1k;
        BM(k - 1, c) = (ak * bkm1 - bk) / denom;
        BM(k, c) = (akm1 * bk - bkm1) / denom;
      }
      k -= 2;
    }
  }
  k = 1;
  while (k <= n) {
    if (ipiv[k - 1] > 0) {
      for (int c = 0; c < nrhs; ++c) {
        double temp = dot_strided(k - 1, &BM(1, c), &AM(1, k));
        BM(k, c) = BM(k, c) + (-1.0) * temp;
      }
      int kp = ipiv[k - 1];
      if (kp != k)
        for (int c = 0; c < nrhs; ++c) { double t = BM(k, c); BM(k, c) = BM(kp, c); BM(kp, c) = t; }
      k += 1;
    } else {
      for (int c = 0; c < nrhs; ++c) {
        double temp = dot_strided(k - 1, &BM(1, c), &AM(1, k));
        BM(k, c) = BM(k, c) + (-1.0) * temp;
        temp = dot_strided(k - 1, &BM(1, c), &AM(1, k + 1));
        BM(k + 1, c) = BM(k + 1, c) + (-1.0) * temp;
      }
      int kp = -ipiv[k - 1];
      if (kp != k)
        for (int c = 0; c < nrhs; ++c) { double t = BM(k, c); BM(k, c) = BM(kp, c); BM(kp, c) = t; }
      k += 2;
    }
  }
}

int mfto_bk_solve(int n, double* a, int nrhs, double* b) {
  int* ipiv = (int*)malloc((size_t)n * sizeof(int));
  int info = bk_factor(n, a, ipiv);
  if (info == 0) bk_solve_factored(n, a, ipiv, nrhs, b);
  free(ipiv);
  return info;
}

/* ------------------------------------------------------------------------ */
/* A2-A5  weights  compute_operators.jl:191-453, 549-594                     */
/* ------------------------------------------------------------------------ */

static int binom(int a, int b) {
  long r = 1;
  for (int i = 1; i <= b; ++i) r = r * (a - b + i) / i;
  return (int)r;
}

/* Monomials of total degree <= deg, ascending degree, x-power descending inside
 * a degree.  The RBF weights are invariant to this choice up to rounding. */
static int make_monomials(int dim, int deg, int (*ex)[3]) {
  int m = 0;
  for (int q = 0; q <= deg; ++q) {
    if (dim == 1) { ex[m][0] = q; ex[m][1] = 0; ex[m][2] = 0; m++; continue; }
    for (int a = q; a >= 0; --a) {
      if (dim == 2) { ex[m][0] = a; ex[m][1] = q - a; ex[m][2] = 0; m++; continue; }
      for (int b = q - a; b >= 0; --b) { ex[m][0] = a; ex[m][1] = b; ex[m][2] = q - a - b; m++; }
    }
  }
  return m;
}

static double fact(int k) {
  double r = 1.0;
  for (int i = 2; i <= k; ++i) r *= (double)i;
  return r;
}

/* d^k/dx_d^k of r^p at a point with coordinate xd (along d) and radius r:
 * Faa di Bruno on f(s) = s^(p/2), s = |x|^2:
 *   sum_j k!/(j!(k-2j)!) (2 xd)^(k-2j) f^(k-j)(s),  f^(m)(s) = prod_{i<m}(p/2-i) r^(p-2m).
 * Closed form of the symbolic derivative built at compute_operators.jl:17-82. */
static double phs_deriv(int p, int k, double xd, double r) {
  if (k == 0) return pow_int(r, p);
  double sum = 0.0;
  for (int j = 0; 2 * j <= k; ++j) {
    int m = k - j;
    double cm = 1.0;
    for (int i = 0; i < m; ++i) cm *= (0.5 * p - i);
    if (cm == 0.0) continue;
    double c = fact(k) / (fact(j) * fact(k - 2 * j));
    double term = c * pow_int(2.0 * xd, k - 2 * j) * cm * pow_int(r, p - 2 * m);
    sum = sum + term;
  }
  return sum;
}

static double mono_eval(const int* e, const double* xh, int dim) {
  double v = 1.0;
  for (int d = 0; d < dim; ++d) v = v * pow_int(xh[d], e[d]);
  return v;
}

/* Assembles node e's saddle-point system exactly as mfto_weights does: full
 * symmetric M (n x n, column-major), rhs b (n x dim, column-major), scaling s. */
int mfto_saddle_system(int dim, const double* x, const double* period, const int64_t* rowptr,
                       const int32_t* stencil, int rbf_pow, int polydeg, int deriv_order,
                       int64_t e, double* m_out, double* b_out, double* s_out) {
  int ex[256][3];
  int npoly = make_monomials(dim, polydeg, ex);
  int k = (int)(rowptr[e + 1] - rowptr[e]);
  const int32_t* st = stencil + rowptr[e];
  int nn_ = k + npoly;
  double* xh = (double*)malloc((size_t)k * 3 * sizeof(double));
  double s[3] = {1, 1, 1};
  const double* xc = x + (int64_t)st[0] * dim;
  for (int j = 0; j < k; ++j)
    for (int d = 0; d < dim; ++d) {
      double t = x[(int64_t)st[j] * dim + d] - xc[d];
      if (period) t = min_image(t, period[d]);
      xh[j * 3 + d] = t;
    }
  for (int d = 0; d < dim; ++d) {
    double m = 0.0;
    for (int j = 0; j < k; ++j) m = jl_max(m, fabs(xh[j * 3 + d]));
    s[d] = 1.0 / m;
  }
  for (int j = 0; j < k; ++j)
    for (int d = 0; d < dim; ++d) xh[j * 3 + d] = xh[j * 3 + d] * s[d];
  for (int c = 0; c < nn_; ++c)
    for (int r = 0; r <= c; ++r) {
      double v;
      if (c < k) {
        double d2 = 0.0;
        for (int d = 0; d < dim; ++d) {
          double t = xh[r * 3 + d] - xh[c * 3 + d];
          d2 = d2 + t * t;
        }
        v = pow_int(sqrt(d2), rbf_pow);
      } else if (r < k) {
        v = mono_eval(ex[c - k], xh + r * 3, dim);
      } else {
        v = 0.0;
      }
      m_out[(size_t)c * nn_ + r] = v;
      m_out[(size_t)r * nn_ + c] = v;
    }
  for (int d = 0; d < dim; ++d) {
    for (int j = 0; j < k; ++j) {
      double pt[3];
      for (int dd = 0; dd < dim; ++dd) pt[dd] = j == 0 ? JL_EPS : -xh[j * 3 + dd];
      double d2 = 0.0;
      for (int dd = 0; dd < dim; ++dd) d2 = d2 + pt[dd] * pt[dd];
      b_out[(size_t)d * nn_ + j] = phs_deriv(rbf_pow, deriv_order, pt[d], sqrt(d2));
    }
    for (int m = 0; m < npoly; ++m) {
      int ok = 1;
      for (int dd = 0; dd < dim; ++dd)
        if (ex[m][dd] != (dd == d ? deriv_order : 0)) ok = 0;
      b_out[(size_t)d * nn_ + k + m] = ok ? fact(deriv_order) : 0.0;
    }
  }
  for (int d = 0; d < dim; ++d) s_out[d] = s[d];
  free(xh);
  return nn_;
}

static int weights_impl(int dim, int64_t n, const double* x, const double* period,
                        const int64_t* rowptr, const int32_t* stencil, int rbf_pow, int polydeg,
                        int deriv_order, double* w, double* resid, int nthreads,
                        int64_t nrows, const int64_t* rows);

int mfto_weights(int dim, int64_t n, const double* x, const double* period, const int64_t* rowptr,
                 const int32_t* stencil, int rbf_pow, int polydeg, int deriv_order, double* w,
                 double* resid, int nthreads) {
  return weights_impl(dim, n, x, period, rowptr, stencil, rbf_pow, polydeg, deriv_order, w,
                      resid, nthreads, n, NULL);
}

int mfto_weights_rows(int dim, int64_t n, const double* x, const double* period,
                      const int64_t* rowptr, const int32_t* stencil, int rbf_pow, int polydeg,
                      int deriv_order, double* w, int nthreads, int64_t nrows,
                      const int64_t* rows) {
  return weights_impl(dim, n, x, period, rowptr, stencil, rbf_pow, polydeg, deriv_order, w,
                      NULL, nthreads, nrows, rows);
}

static int weights_impl(int dim, int64_t n, const double* x, const double* period,
                        const int64_t* rowptr, const int32_t* stencil, int rbf_pow, int polydeg,
                        int deriv_order, double* w, double* resid, int nthreads,
                        int64_t nrows, const int64_t* rows) {
  if (dim < 1 || dim > 3 || deriv_order < 1) return -1;
  int ex[256][3];
  int npoly = make_monomials(dim, polydeg, ex);
  if (npoly != binom(polydeg + dim, dim)) return -1;
  int kmax = 0;
  for (int64_t q = 0; q < nrows; ++q) {
    int64_t e = rows ? rows[q] : q;
    int k = (int)(rowptr[e + 1] - rowptr[e]);
    if (k > kmax) kmax = k;
  }
  int64_t first_bad = -1;
#pragma omp parallel num_threads(nthreads_or_default(nthreads))
  {
    int nmax = kmax + npoly;
    double* a = (double*)malloc((size_t)nmax * nmax * sizeof(double));
    double* a0 = resid ? (double*)malloc((size_t)nmax * nmax * sizeof(double)) : NULL;
    double* b = (double*)malloc((size_t)nmax * dim * sizeof(double));
    double* b0 = resid ? (double*)malloc((size_t)nmax * dim * sizeof(double)) : NULL;
    double* xh = (double*)malloc((size_t)kmax * 3 * sizeof(double));
    int* ipiv = (int*)malloc((size_t)nmax * sizeof(int));
#pragma omp for schedule(dynamic, 64)
    for (int64_t q = 0; q < nrows; ++q) {
      const int64_t e = rows ? rows[q] : q;
      int k = (int)(rowptr[e + 1] - rowptr[e]);
      const int32_t* st = stencil + rowptr[e];
      int nn_ = k + npoly;
      /* shift_stencil :225-246 : centre = first stencil node; per-axis scale */
      double s[3] = {1, 1, 1};
      const double* xc = x + (int64_t)st[0] * dim;
      for (int j = 0; j < k; ++j)
        for (int d = 0; d < dim; ++d) {
          double t = x[(int64_t)st[j] * dim + d] - xc[d];
          if (period) t = min_image(t, period[d]);
          xh[j * 3 + d] = t;
        }
      for (int d = 0; d < dim; ++d) {
        double m = 0.0;
        for (int j = 0; j < k; ++j) m = jl_max(m, fabs(xh[j * 3 + d]));
        s[d] = 1.0 / m;
      }
      for (int j = 0; j < k; ++j)
        for (int d = 0; d < dim; ++d) xh[j * 3 + d] = xh[j * 3 + d] * s[d];
      /* interpolation_block :265-267 (upper triangle of [R P; P' 0]) */
      for (int c = 0; c < nn_; ++c)
        for (int r = 0; r <= c; ++r) {
          double v;
          if (c < k) {
            double d2 = 0.0;
            for (int d = 0; d < dim; ++d) {
              double t = xh[r * 3 + d] - xh[c * 3 + d];
              d2 = d2 + t * t;
            }
            v = pow_int(sqrt(d2), rbf_pow); /* rbf_block :191-203 */
          } else if (r < k) {
            v = mono_eval(ex[c - k], xh + r * 3, dim); /* poly_block :211-223 */
          } else {
            v = 0.0;
          }
          a[(size_t)c * nn_ + r] = v;
        }
      /* RHS: rbf_linearoperator at the mirrored stencil (mirror_stencil :248-263,
       * centre replaced by (eps,...,eps)), poly_linearoperator at the centre. */
      for (int d = 0; d < dim; ++d) {
        for (int j = 0; j < k; ++j) {
          double pt[3];
          for (int dd = 0; dd < dim; ++dd) pt[dd] = j == 0 ? JL_EPS : -xh[j * 3 + dd];
          double d2 = 0.0;
          for (int dd = 0; dd < dim; ++dd) d2 = d2 + pt[dd] * pt[dd];
          b[(size_t)d * nn_ + j] = phs_deriv(rbf_pow, deriv_order, pt[d], sqrt(d2));
        }
        for (int m = 0; m < npoly; ++m) {
          int ok = 1;
          for (int dd = 0; dd < dim; ++dd)
            if (ex[m][dd] != (dd == d ? deriv_order : 0)) ok = 0;
          b[(size_t)d * nn_ + k + m] = ok ? fact(deriv_order) : 0.0;
        }
      }
      if (resid) {
        memcpy(a0, a, (size_t)nn_ * nn_ * sizeof(double));
        memcpy(b0, b, (size_t)nn_ * dim * sizeof(double));
      }
      int info = bk_factor(nn_, a, ipiv);
      if (info != 0) {
#pragma omp critical
        {
          if (first_bad < 0 || e < first_bad) first_bad = e;
        }
        for (int j = 0; j < k; ++j)
          for (int d = 0; d < dim; ++d) w[(rowptr[e] + j) * dim + d] = NAN;
        if (resid) resid[e] = NAN;
        continue;
      }
      bk_solve_factored(nn_, a, ipiv, dim, b);
      for (int d = 0; d < dim; ++d) {
        double sc = pow_int(s[d], deriv_order);
        for (int j = 0; j < k; ++j) w[(rowptr[e] + j) * dim + d] = sc * b[(size_t)d * nn_ + j];
      }
      if (resid) {
        double worst = 0.0;
        for (int d = 0; d < dim; ++d) {
          double bn = 0.0, rn = 0.0;
          for (int r = 0; r < nn_; ++r) {
            double acc = 0.0;
            for (int c = 0; c < nn_; ++c) {
              double av = r <= c ? a0[(size_t)c * nn_ + r] : a0[(size_t)r * nn_ + c];
              acc += av * b[(size_t)d * nn_ + c];
            }
            rn = fmax(rn, fabs(acc - b0[(size_t)d * nn_ + r]));
            bn = fmax(bn, fabs(b0[(size_t)d * nn_ + r]));
          }
          worst = fmax(worst, bn > 0 ? rn / bn : rn);
        }
        resid[e] = worst;
      }
    }
    free(a); free(a0); free(b); free(b0); free(xh); free(ipiv);
  }
  return first_bad >= 0 ? (int)(-(first_bad + 1)) : 0;
}

/* ------------------------------------------------------------------------ */
/* SparseArrays products used by rhs! (rbfsolver.jl:10-33)                   */
/* ------------------------------------------------------------------------ */

/* mul!(y, A, x, alpha, 1): column scatter y[row] += val * (x[col]*alpha); per
 * row that is an ascending-column sequence of rounded products and adds. */
void mfto_spmv_accum(const mfto_csr* a, double alpha, const double* x, double* y, int nthreads) {
#pragma omp parallel for num_threads(nthreads_or_default(nthreads)) schedule(static)
  for (int64_t i = 0; i < a->n; ++i) {
    double acc = y[i];
    for (int64_t p = a->rp[i]; p < a->rp[i + 1]; ++p) {
      double ax = x[a->ci[p]] * alpha;
      double term = a->val[p] * ax;
      acc = acc + term;
    }
    y[i] = acc;
  }
}

/* mul!(y, A, x): y = 0, then the same accumulation with alpha = true. */
void mfto_spmv(const mfto_csr* a, const double* x, double* y, int nthreads) {
#pragma omp parallel for num_threads(nthreads_or_default(nthreads)) schedule(static)
  for (int64_t i = 0; i < a->n; ++i) {
    double acc = 0.0;
    for (int64_t p = a->rp[i]; p < a->rp[i + 1]; ++p) {
      double term = a->val[p] * x[a->ci[p]];
      acc = acc + term;
    }
    y[i] = acc;
  }
}

/* mul!(y, A', x, alpha, 1): per column tmp = sum val*x[row] (ascending rows),
 * then y[col] += tmp * alpha. */
void mfto_spmv_t_accum(const mfto_csr* a, double alpha, const double* x, double* y, int nthreads) {
#pragma omp parallel for num_threads(nthreads_or_default(nthreads)) schedule(static)
  for (int64_t i = 0; i < a->n; ++i) {
    double tmp = 0.0;
    for (int64_t p = a->cp[i]; p < a->cp[i + 1]; ++p) {
      double term = a->valt[p] * x[a->ri[p]];
      tmp = tmp + term;
    }
    y[i] = y[i] + tmp * alpha;
  }
}

/* lap' * lap as SparseArrays.spmatmul forms it: H[i,j] = sum over ascending k
 * of lap[k,i]*lap[k,j] (first product assigned, the rest added). */
/* CSC view of a CSR matrix by a counting sort: each column lists its rows ascending. */
void mfto_csr_to_csc(int64_t n, const int64_t* rp, const int32_t* ci, const double* val,
                     int64_t* cp, int32_t* ri, double* valt) {
  for (int64_t j = 0; j <= n; ++j) cp[j] = 0;
  for (int64_t p = 0; p < rp[n]; ++p) cp[ci[p] + 1] += 1;
  for (int64_t j = 0; j < n; ++j) cp[j + 1] += cp[j];
  int64_t* next = (int64_t*)malloc((size_t)n * sizeof(int64_t));
  for (int64_t j = 0; j < n; ++j) next[j] = cp[j];
  for (int64_t i = 0; i < n; ++i)
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p) {
      const int64_t q = next[ci[p]]++;
      ri[q] = (int32_t)i;
      valt[q] = val[p];
    }
  free(next);
}

static int cmp_i32(const void* x, const void* y) {
  const int32_t a = *(const int32_t*)x, b = *(const int32_t*)y;
  return (a > b) - (a < b);
}

/* lap' * lap: row i of the product accumulates lap[k, i] * lap[k, j] over the stored
 * entries k of column i in ascending order, then over row k's entries (SparseArrays'
 * spmatmul order for each entry).  Rows are independent, so they run in parallel; the
 * per-row order and hence every value is the same for any thread count.  hci == NULL:
 * count pass (hrp filled); otherwise fill pass (hrp from the count pass). */
int mfto_ata(const mfto_csr* a, int64_t* hrp, int32_t* hci, double* hval, int nthreads) {
  const int64_t n = a->n;
  int failed = 0;
  if (!hci) hrp[0] = 0;
#pragma omp parallel num_threads(nthreads_or_default(nthreads))
  {
    int64_t* mark = (int64_t*)malloc((size_t)n * sizeof(int64_t));
    double* acc = (double*)malloc((size_t)n * sizeof(double));
    int32_t* cols = (int32_t*)malloc((size_t)n * sizeof(int32_t));
    if (!mark || !acc || !cols) {
#pragma omp atomic write
      failed = 1;
    } else {
      for (int64_t i = 0; i < n; ++i) mark[i] = -1;
#pragma omp for schedule(dynamic, 256)
      for (int64_t i = 0; i < n; ++i) {
        int64_t cnt = 0;
        for (int64_t p = a->cp[i]; p < a->cp[i + 1]; ++p) {
          const int32_t k = a->ri[p];
          const double aki = a->valt[p];
          for (int64_t q = a->rp[k]; q < a->rp[k + 1]; ++q) {
            const int32_t j = a->ci[q];
            const double prod = aki * a->val[q];
            if (mark[j] != i) {
              mark[j] = i;
              cols[cnt++] = j;
              acc[j] = prod;
            } else {
              acc[j] = acc[j] + prod;
            }
          }
        }
        if (!hci) {
          hrp[i + 1] = cnt;
        } else {
          qsort(cols, (size_t)cnt, sizeof(int32_t), cmp_i32);
          for (int64_t m = 0; m < cnt; ++m) {
            hci[hrp[i] + m] = cols[m];
            hval[hrp[i] + m] = acc[cols[m]];
          }
        }
      }
    }
    free(mark);
    free(acc);
    free(cols);
  }
  if (failed) return -2;
  if (!hci)
    for (int64_t i = 0; i < n; ++i) hrp[i + 1] += hrp[i];
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Equations (textbook forms of Trixi's flux and cons2prim)                  */
/* ------------------------------------------------------------------------ */

static void flux_point(const mfto_semi* s, const double* uu, int d, double* f) {
  if (s->eq == MFTO_EQ_EULER3D) {
    /* Trixi's CompressibleEulerEquations3D flux (textbook form) in direction d */
    double rho = uu[0], m1 = uu[1], m2 = uu[2], m3 = uu[3], en = uu[4];
    double v1 = m1 / rho, v2 = m2 / rho, v3 = m3 / rho;
    double p = (s->gamma - 1.0) * (en - 0.5 * (m1 * v1 + m2 * v2 + m3 * v3));
    double m = d == 0 ? m1 : (d == 1 ? m2 : m3);
    double vd = d == 0 ? v1 : (d == 1 ? v2 : v3);
    f[0] = m;
    f[1] = m * v1 + (d == 0 ? p : 0.0);
    f[2] = m * v2 + (d == 1 ? p : 0.0);
    f[3] = m * v3 + (d == 2 ? p : 0.0);
    f[4] = (en + p) * vd;
    return;
  }
  if (s->eq == MFTO_EQ_EULER2D) {
    double rho = uu[0], m1 = uu[1], m2 = uu[2], en = uu[3];
    double v1 = m1 / rho, v2 = m2 / rho;
    double p = (s->gamma - 1.0) * (en - 0.5 * (m1 * v1 + m2 * v2));
    if (d == 0) {
      f[0] = m1;
      f[1] = m1 * v1 + p;
      f[2] = m1 * v2;
      f[3] = (en + p) * v1;
    } else {
      f[0] = m2;
      f[1] = m2 * v1;
      f[2] = m2 * v2 + p;
      f[3] = (en + p) * v2;
    }
  } else {
    for (int v = 0; v < s->nvars; ++v) f[v] = s->adv[d] * uu[v];
  }
}

/* calc_fluxes!  rbfsolver.jl:247-265 */
int mfto_calc_fluxes(const mfto_semi* s, double* const* du, double* const* u, int nthreads) {
  int64_t n = s->n;
  int V = s->nvars;
  double* f = (double*)malloc((size_t)n * V * sizeof(double));
  if (!f) return -2;
  for (int d = 0; d < s->dim; ++d) {
#pragma omp parallel for num_threads(nthreads_or_default(nthreads)) schedule(static)
    for (int64_t e = 0; e < n; ++e) {
      double uu[8], ff[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int v = 0; v < V; ++v) uu[v] = u[v][e];
      flux_point(s, uu, d, ff);
      for (int v = 0; v < V; ++v) f[(size_t)v * n + e] = ff[v];
    }
    for (int v = 0; v < V; ++v) mfto_spmv_accum(&s->dop[d], -1.0, f + (size_t)v * n, du[v], nthreads);
  }
  free(f);
  return 0;
}

/* calc_boundary_flux!  rbfsolver.jl:277-318 with PointCloudBCs.jl:49-115 */
static void bc_pass(const mfto_semi* s, const double* dirichlet, double* const* du, double* const* u) {
  int V = s->nvars;
  for (int b = 0; b < s->n_bc; ++b) {
    int kind = s->bc_kind[b];
    for (int64_t p = s->bc_ptr[b]; p < s->bc_ptr[b + 1]; ++p) {
      int32_t i = s->bc_idx[p];
      if (kind == MFTO_BC_DIRICHLET) {
        for (int v = 0; v < V; ++v) {
          du[v][i] = 0.0;
          u[v][i] = dirichlet[p * V + v];
        }
      } else if (kind == MFTO_BC_SLIP_WALL && s->eq == MFTO_EQ_EULER2D) {
        double n1 = s->bc_normal[p * s->dim + 0], n2 = s->bc_normal[p * s->dim + 1];
        double nrm = sqrt(n1 * n1 + n2 * n2);
        n1 = n1 / nrm;
        n2 = n2 / nrm;
        double vn = u[1][i] * n1 + u[2][i] * n2;
        double s1 = u[1][i] - vn * n1;
        double s2 = u[2][i] - vn * n2;
        du[1][i] = 0.0;
        du[2][i] = 0.0;
        u[1][i] = s1;
        u[2][i] = s2;
      }
    }
  }
}

/* update_upwind_visc! hyperviscosity.jl:246-285 (Euler) and the scalar
 * advection extension eps_uw = c_uw*0.5*h*|a|. */
static void upwind_visc(const mfto_semi* s, double* const* u, double* eps_uw) {
  int64_t n = s->n;
  for (int64_t i = 0; i < n; ++i) {
    if (s->eq == MFTO_EQ_EULER2D) {
      double rho = u[0][i], m1 = u[1][i], m2 = u[2][i], en = u[3][i];
      double v1 = m1 / rho, v2 = m2 / rho;
      double p = (s->gamma - 1.0) * (en - 0.5 * (m1 * v1 + m2 * v2));
      double speed = sqrt(v1 * v1 + v2 * v2);
      double c;
      if (p < 0.0 || rho < 0.0) c = 0.0;
      else c = sqrt(s->gamma * p / rho);
      eps_uw[i] = s->c_uw * 0.5 * s->h * (speed + c);
    } else {
      double a2 = 0.0;
      for (int d = 0; d < s->dim; ++d) a2 = a2 + s->adv[d] * s->adv[d];
      eps_uw[i] = s->c_uw * 0.5 * s->h * sqrt(a2);
    }
  }
}

/* update_residual_visc! hyperviscosity.jl:289-329 with ode_mean/ode_maximum
 * (mpi.jl:40-81). */
static void residual_visc(const mfto_semi* s, double* const* du, double* const* u, double* eps_rv,
                          mfto_rv_diag* diag) {
  int64_t n = s->n;
  int V = s->nvars;
  double mean[8], nrm[8];
  for (int v = 0; v < V; ++v) {
    double sv = mfto_pairwise_sum(u[v], n, 1);
    mean[v] = s->mean_mode == 0 ? sv / (double)(n * V) : sv / (double)n;
  }
  double* loc = (double*)malloc((size_t)n * V * sizeof(double));
  for (int64_t i = 0; i < n; ++i)
    for (int v = 0; v < V; ++v) loc[i * V + v] = fabs(u[v][i] - mean[v]);
  if (s->max_mode == 0) {
    int64_t best = 0;
    for (int64_t i = 1; i < n; ++i)
      if (!jl_vec_isless(loc + i * V, loc + best * V, V)) best = i; /* max(a,b)=isless(b,a)?a:b */
    for (int v = 0; v < V; ++v) nrm[v] = loc[best * V + v];
  } else {
    for (int v = 0; v < V; ++v) {
      double m = loc[v];
      for (int64_t i = 1; i < n; ++i) m = jl_max(m, loc[i * V + v]);
      nrm[v] = m;
    }
  }
  free(loc);
  for (int v = 0; v < V; ++v)
    if (nrm[v] == 0.0) nrm[v] = JL_EPS;
  if (diag) {
    for (int v = 0; v < V; ++v) { diag->mean[v] = mean[v]; diag->norms[v] = nrm[v]; }
  }
  for (int64_t i = 0; i < n; ++i) {
    double mr = 0.0;
    for (int v = 0; v < V; ++v) {
      double r = fabs(s->approx_du[(size_t)v * n + i] - du[v][i]);
      double q = r / nrm[v];
      mr = v == 0 ? q : jl_max(mr, q);
    }
    eps_rv[i] = 0.5 * s->c_rv * (s->h * s->h) * mr;
  }
}

/* update_visc!  hyperviscosity.jl:331-349 */
static void combine_visc(int64_t n, const double* eps_uw, const double* eps_rv, int success_iter,
                         double* eps) {
  for (int64_t i = 0; i < n; ++i) {
    if (isnan(eps_rv[i]) || isinf(eps_rv[i]) || success_iter == 0) {
      if (isnan(eps_uw[i]) || isinf(eps_uw[i])) eps[i] = JL_EPS;
      else eps[i] = eps_uw[i];
    } else {
      eps[i] = jl_min(eps_rv[i], eps_uw[i]);
    }
  }
}

/* (::SourceResidualViscosityTominec) hyperviscosity.jl:382-409 and
 * (::SourceUpwindViscosityTominec) :351-380 */
static int visc_source(const mfto_semi* s, int kind, double* const* du, double* const* u,
                       double* eps_out, mfto_rv_diag* diag, int nthreads) {
  int64_t n = s->n;
  int V = s->nvars;
  double* eps_uw = (double*)malloc((size_t)n * sizeof(double));
  double* eps_rv = (double*)malloc((size_t)n * sizeof(double));
  double* eps = (double*)malloc((size_t)n * sizeof(double));
  double* t = (double*)malloc((size_t)n * sizeof(double));
  if (!eps_uw || !eps_rv || !eps || !t) { free(eps_uw); free(eps_rv); free(eps); free(t); return -2; }
  upwind_visc(s, u, eps_uw);
  if (kind == MFTO_SRC_RV) {
    residual_visc(s, du, u, eps_rv, diag);
    combine_visc(n, eps_uw, eps_rv, s->success_iter, eps);
  } else {
    memcpy(eps, eps_uw, (size_t)n * sizeof(double));
  }
  for (int j = 0; j < s->dim; ++j) {
    for (int v = 0; v < V; ++v) {
      mfto_spmv(&s->dop[j], u[v], t, nthreads);
      for (int64_t i = 0; i < n; ++i) t[i] = eps[i] * t[i];
      mfto_spmv_t_accum(&s->dop[j], -1.0, t, du[v], nthreads);
    }
  }
  if (eps_out) memcpy(eps_out, eps, (size_t)n * sizeof(double));
  free(eps_uw); free(eps_rv); free(eps); free(t);
  return 0;
}

/* Trixi.rhs!  rbfsolver.jl:397-428 */
/* SourceIGR  src/sources/IGR.jl:17-239 (Cao & Schafer 2023): solve
 *   (rho^-1 - alpha (Dx rho^-1 Dx + Dy rho^-1 Dy)) sigma = alpha (tr(Du)^2 + tr(Du^2))
 * by unpreconditioned conjugate gradients from sigma = 0 with at most igr_maxiter
 * iterations and relative tolerance sqrt(eps) (the reference names IterativeSolvers'
 * cg; its call cg(sigma, A, b; maxiter = 20) matches no method of that package, so the
 * in-place cg!(sigma, A, b; maxiter = 20) it intends is restated: Hestenes-Stiefel CG
 * in IterativeSolvers' CGIterable order), then du[rho v1] -= Dx sigma,
 * du[rho v2] -= Dy sigma.  tr(Du) is formed as the reference writes it,
 * Dx(rho) + Dy(v1) (update_igr_rhs!, :143-145), and tr(Du^2) =
 * (Dx v1)^2 + 2 (Dy v1)(Dx v2) + (Dy v2)^2 (:151-153). */
static double dot_seq(int64_t n, const double* a, const double* b) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s = s + a[i] * b[i];
  return s;
}

/* y = (rho^-1 - alpha (Dx rho^-1 Dx + Dy rho^-1 Dy)) v  (IGRCompositeMatrix mul!, :59-73) */
static void igr_apply(const mfto_semi* s, const double* rinv, const double* v, double* y,
                      double* t1, double* t2, double* t3, int nthreads) {
  int64_t n = s->n;
  mfto_spmv(&s->dop[0], v, t1, nthreads);
  mfto_spmv(&s->dop[1], v, t2, nthreads);
  for (int64_t i = 0; i < n; ++i) { t1[i] = rinv[i] * t1[i]; t2[i] = rinv[i] * t2[i]; }
  mfto_spmv(&s->dop[0], t1, t3, nthreads);
  mfto_spmv(&s->dop[1], t2, t1, nthreads);
  for (int64_t i = 0; i < n; ++i) {
    y[i] = rinv[i] * v[i];
    y[i] = y[i] - s->igr_alpha * (t3[i] + t1[i]);
  }
}

static int igr_source(const mfto_semi* s, double* const* du, double* const* u, int nthreads) {
  if (s->eq != MFTO_EQ_EULER2D || s->dim != 2) return -1;
  int64_t n = s->n;
  double* w = (double*)calloc((size_t)n * 16, sizeof(double));
  if (!w) return -2;
  double *rho = w, *v1 = w + n, *v2 = w + 2 * n, *rinv = w + 3 * n, *b = w + 4 * n;
  double *dxr = w + 5 * n, *dxv1 = w + 6 * n, *dxv2 = w + 7 * n, *dyv1 = w + 8 * n,
         *dyv2 = w + 9 * n;
  double *x = w + 10 * n, *r = w + 11 * n, *cu = w + 12 * n, *cc = w + 13 * n;
  double *t1 = dxr, *t2 = dxv1, *t3 = dxv2; /* reused once b is formed */
  for (int64_t i = 0; i < n; ++i) {
    rho[i] = u[0][i];
    v1[i] = u[1][i] / u[0][i];
    v2[i] = u[2][i] / u[0][i];
  }
  mfto_spmv(&s->dop[0], rho, dxr, nthreads);
  mfto_spmv(&s->dop[0], v1, dxv1, nthreads);
  mfto_spmv(&s->dop[0], v2, dxv2, nthreads);
  mfto_spmv(&s->dop[1], v1, dyv1, nthreads);
  mfto_spmv(&s->dop[1], v2, dyv2, nthreads);
  for (int64_t i = 0; i < n; ++i) {
    double tr = 0.0;
    tr = tr + dxr[i];
    tr = tr + dyv1[i];
    double tsq = dxv1[i] * dxv1[i] + 2.0 * dyv1[i] * dxv2[i] + dyv2[i] * dyv2[i];
    b[i] = s->igr_alpha * (tr * tr + tsq);
    rinv[i] = 1.0 / u[0][i];
  }
  /* cg!: x = 0, r = b - A x = b, u = 0 */
  for (int64_t i = 0; i < n; ++i) { x[i] = 0.0; r[i] = b[i]; cu[i] = 0.0; }
  double res = sqrt(dot_seq(n, r, r));
  double prev = 1.0;
  const double tol = res * sqrt(JL_EPS);
  for (int it = 0; it < s->igr_maxiter && !(res <= tol); ++it) {
    double beta = (res * res) / (prev * prev);
    for (int64_t i = 0; i < n; ++i) cu[i] = r[i] + beta * cu[i];
    igr_apply(s, rinv, cu, cc, t1, t2, t3, nthreads);
    double alpha = (res * res) / dot_seq(n, cu, cc);
    for (int64_t i = 0; i < n; ++i) {
      x[i] = x[i] + alpha * cu[i];
      r[i] = r[i] - alpha * cc[i];
    }
    prev = res;
    res = sqrt(dot_seq(n, r, r));
  }
  if (s->igr_sigma) memcpy(s->igr_sigma, x, (size_t)n * sizeof(double));
  mfto_spmv_accum(&s->dop[0], -1.0, x, du[1], nthreads);
  mfto_spmv_accum(&s->dop[1], -1.0, x, du[2], nthreads);
  free(w);
  return 0;
}

int mfto_rhs(const mfto_semi* s, double t, const double* dirichlet, double* const* du,
             double* const* u, double* eps_out, mfto_rv_diag* diag, int nthreads) {
  (void)t;
  int V = s->nvars;
  /* 3D Euler: the plain flux divergence with Dirichlet / do-nothing BCs -- the reference's
   * viscosity sources and slip walls are written for CompressibleEulerEquations2D
   * (hyperviscosity.jl:246-329, PointCloudBCs.jl:15-21) */
  if (s->eq == MFTO_EQ_EULER3D) {
    if (s->n_src > 0) return -1;
    for (int b = 0; b < s->n_bc; ++b)
      if (s->bc_kind[b] == MFTO_BC_SLIP_WALL) return -1;
  }
  for (int v = 0; v < V; ++v) memset(du[v], 0, (size_t)s->n * sizeof(double));
  bc_pass(s, dirichlet, du, u);
  int rc = mfto_calc_fluxes(s, du, u, nthreads);
  if (rc) return rc;
  for (int q = 0; q < s->n_src; ++q) {
    int kind = s->src_kind[q];
    if (kind == MFTO_SRC_RV || kind == MFTO_SRC_UPWIND) {
      rc = visc_source(s, kind, du, u, eps_out, diag, nthreads);
      if (rc) return rc;
    } else if (kind == MFTO_SRC_HV_TOMINEC || kind == MFTO_SRC_HV_FLYER) {
      for (int v = 0; v < V; ++v) mfto_spmv_accum(&s->hv, -s->hv_gamma, u[v], du[v], nthreads);
    } else if (kind == MFTO_SRC_IGR) {
      rc = igr_source(s, du, u, nthreads);
      if (rc) return rc;
    } else {
      return -1;
    }
  }
  bc_pass(s, dirichlet, du, u);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Adjoint of rhs! (extension)                                               */
/* ------------------------------------------------------------------------ */

/* Reverse-mode product of the Euler flux pair (flux_point d = 0, 1) at state uu:
 * ub = (dF/du)^T gx + (dG/du)^T gy, derived from the flux definition
 * F = (m1, m1 v1 + p, m1 v2, (E + p) v1), G = (m2, m2 v1, m2 v2 + p, (E + p) v2),
 * v = m / rho, p = (gamma - 1)(E - (m1 v1 + m2 v2) / 2). */
static void euler_flux_vjp(double gamma, const double* uu, const double* gx, const double* gy,
                           double* ub) {
  double rho = uu[0], m1 = uu[1], m2 = uu[2], en = uu[3];
  double v1 = m1 / rho, v2 = m2 / rho;
  double gm1 = gamma - 1.0;
  double p = gm1 * (en - 0.5 * (m1 * v1 + m2 * v2));
  double ep = en + p;
  double pb = gx[1] + gx[3] * v1 + gy[2] + gy[3] * v2;
  double eb = gx[3] * v1 + gy[3] * v2 + gm1 * pb;
  double v1b = gx[1] * m1 + gx[3] * ep + gy[1] * m2 - 0.5 * gm1 * m1 * pb;
  double v2b = gx[2] * m1 + gy[2] * m2 + gy[3] * ep - 0.5 * gm1 * m2 * pb;
  double m1b = gx[0] + gx[1] * v1 + gx[2] * v2 - 0.5 * gm1 * v1 * pb + v1b / rho;
  double m2b = gy[0] + gy[1] * v1 + gy[2] * v2 - 0.5 * gm1 * v2 * pb + v2b / rho;
  double rhob = -(v1b * v1 + v2b * v2) / rho;
  ub[0] = rhob;
  ub[1] = m1b;
  ub[2] = m2b;
  ub[3] = eb;
}

/* Unit normal of boundary-list entry p. */
static void unit_normal(const mfto_semi* s, int64_t p, double* n1, double* n2) {
  double a = s->bc_normal[p * s->dim + 0], b = s->bc_normal[p * s->dim + 1];
  double nrm = sqrt(a * a + b * b);
  *n1 = a / nrm;
  *n2 = b / nrm;
}

int mfto_rhs_adjoint(const mfto_semi* s, const double* const* u, const double* const* lam,
                     double* const* out, int nthreads) {
  int64_t n = s->n;
  int V = s->nvars, D = s->dim;
  for (int q = 0; q < s->n_src; ++q)
    if (s->src_kind[q] == MFTO_SRC_RV || s->src_kind[q] == MFTO_SRC_UPWIND) return -1;
  /* per-node BC tag (last listing wins, as bc_pass applies them in order) */
  signed char* tag = (signed char*)calloc((size_t)n, 1);
  int64_t* slot = (int64_t*)malloc((size_t)n * sizeof(int64_t));
  double* lt = (double*)malloc((size_t)n * V * sizeof(double));
  double* g = (double*)calloc((size_t)n * V * D, sizeof(double));
  if (!tag || !slot || !lt || !g) { free(tag); free(slot); free(lt); free(g); return -2; }
  for (int b = 0; b < s->n_bc; ++b) {
    for (int64_t p = s->bc_ptr[b]; p < s->bc_ptr[b + 1]; ++p) {
      int32_t i = s->bc_idx[p];
      if (s->bc_kind[b] == MFTO_BC_DIRICHLET) { tag[i] = 1; slot[i] = p; }
      else if (s->bc_kind[b] == MFTO_BC_SLIP_WALL && s->eq == MFTO_EQ_EULER2D) { tag[i] = 2; slot[i] = p; }
    }
  }
  /* lam~ = M2 lam: the rows that bc_pass zeroes in du carry no cotangent */
  for (int v = 0; v < V; ++v)
    for (int64_t i = 0; i < n; ++i) {
      double x = lam[v][i];
      if (tag[i] == 1 || (tag[i] == 2 && (v == 1 || v == 2))) x = 0.0;
      lt[(size_t)v * n + i] = x;
    }
  /* g_d = D_d^T lam~ */
  for (int d = 0; d < D; ++d)
    for (int v = 0; v < V; ++v)
      mfto_spmv_t_accum(&s->dop[d], 1.0, lt + (size_t)v * n, g + ((size_t)d * V + v) * n, nthreads);
  /* flux-Jacobian-transpose products at each node, on the state bc_pass leaves */
#pragma omp parallel for num_threads(nthreads_or_default(nthreads)) schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double uu[8], gx[8], gy[8], ub[8];
    for (int v = 0; v < V; ++v) {
      uu[v] = u[v][i];
      gx[v] = g[(size_t)v * n + i];
      gy[v] = g[((size_t)V + v) * n + i];
    }
    if (s->eq == MFTO_EQ_EULER2D) {
      if (tag[i] == 2) {
        double n1, n2;
        unit_normal(s, slot[i], &n1, &n2);
        double vn = uu[1] * n1 + uu[2] * n2;
        double s1 = uu[1] - vn * n1, s2 = uu[2] - vn * n2;
        uu[1] = s1;
        uu[2] = s2;
      }
      euler_flux_vjp(s->gamma, uu, gx, gy, ub);
    } else {
      for (int v = 0; v < V; ++v) {
        double acc = 0.0;
        for (int d = 0; d < D; ++d) acc = acc + s->adv[d] * g[((size_t)d * V + v) * n + i];
        ub[v] = acc;
      }
    }
    for (int v = 0; v < V; ++v) out[v][i] = -ub[v];
  }
  /* hyperviscosity du -= gamma H u  ->  out -= gamma H^T lam~ */
  for (int q = 0; q < s->n_src; ++q) {
    if (s->src_kind[q] != MFTO_SRC_HV_TOMINEC && s->src_kind[q] != MFTO_SRC_HV_FLYER) continue;
    for (int v = 0; v < V; ++v)
      for (int64_t r = 0; r < n; ++r) {
        double x = lt[(size_t)v * n + r];
        for (int64_t p = s->hv.rp[r]; p < s->hv.rp[r + 1]; ++p)
          out[v][s->hv.ci[p]] -= s->hv_gamma * s->hv.val[p] * x;
      }
  }
  /* Pi: Dirichlet values do not depend on u; slip walls project the momentum */
  for (int64_t i = 0; i < n; ++i) {
    if (tag[i] == 1) {
      for (int v = 0; v < V; ++v) out[v][i] = 0.0;
    } else if (tag[i] == 2) {
      double n1, n2;
      unit_normal(s, slot[i], &n1, &n2);
      double vn = out[1][i] * n1 + out[2][i] * n2;
      double s1 = out[1][i] - vn * n1, s2 = out[2][i] - vn * n2;
      out[1][i] = s1;
      out[2][i] = s2;
    }
  }
  free(tag); free(slot); free(lt); free(g);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Zhang-Shu positivity limiter  positivity_zhang_shu_point2d.jl:22-82       */
/* ------------------------------------------------------------------------ */

/* Trixi's density(u) and pressure(u) for CompressibleEulerEquations2D. */
static double zs_variable(int variable, double gamma, const double* uu) {
  if (variable == 0) return uu[0];
  return (gamma - 1.0) * (uu[3] - 0.5 * (uu[1] * uu[1] + uu[2] * uu[2]) / uu[0]);
}

int64_t mfto_limiter_zhang_shu(int64_t n, int nvars, double gamma, const int64_t* rowptr,
                               const int32_t* cols, int variable, double threshold,
                               double* const* u) {
  double* loc = (double*)calloc((size_t)n * nvars, sizeof(double));
  if (!loc) return -2;
  int64_t limited = 0;
  for (int64_t e = 0; e < n; ++e) {
    double uu[8], mean[8];
    double vmin = INFINITY;
    for (int64_t p = rowptr[e]; p < rowptr[e + 1]; ++p) {
      for (int v = 0; v < nvars; ++v) uu[v] = u[v][cols[p]];
      vmin = jl_min(vmin, zs_variable(variable, gamma, uu));
    }
    if (!(vmin < threshold)) continue;
    for (int v = 0; v < nvars; ++v) mean[v] = 0.0;
    for (int64_t p = rowptr[e]; p < rowptr[e + 1]; ++p)
      for (int v = 0; v < nvars; ++v) mean[v] = mean[v] + u[v][cols[p]];
    const double cnt = (double)(rowptr[e + 1] - rowptr[e]);
    for (int v = 0; v < nvars; ++v) mean[v] = mean[v] / cnt;
    const double vmean = zs_variable(variable, gamma, mean);
    const double theta = (vmean - threshold) / (vmean - vmin);
    for (int v = 0; v < nvars; ++v)
      loc[(size_t)e * nvars + v] = fma(theta, u[v][e], (1.0 - theta) * mean[v]);
  }
  for (int64_t e = 0; e < n; ++e) {
    int nz = 0;
    for (int v = 0; v < nvars; ++v) nz |= loc[(size_t)e * nvars + v] != 0.0;
    if (!nz) continue;
    for (int v = 0; v < nvars; ++v) u[v][e] = loc[(size_t)e * nvars + v];
    limited++;
  }
  free(loc);
  return limited;
}

/* ------------------------------------------------------------------------ */
/* A16  time_deriv_weights!  history.jl:131-152                              */
/* ------------------------------------------------------------------------ */

int mfto_time_deriv_weights(int m, const double* t, double* w) {
  if (m < 1 || m > 16) return -1;
  double a[16][16], b[16], tt[16];
  double tmax = 0.0;
  for (int i = 0; i < m; ++i) tmax = jl_max(tmax, fabs(t[i]));
  double scale = 1.0 / tmax;
  for (int i = 0; i < m; ++i) tt[i] = t[i] * scale;
  double te = tt[0];
  /* A[i][k] = t_i^k ; the solve is with A' : at[k][i] = A[i][k] */
  for (int i = 0; i < m; ++i)
    for (int k = 0; k < m; ++k) a[k][i] = k == 0 ? 1.0 : pow_int(tt[i], k);
  for (int k = 0; k < m; ++k) b[k] = (double)k * (k == 0 ? 1.0 / te : pow_int(te, k - 1));
  /* LU with partial pivoting (Gaussian elimination, first max on ties) */
  int perm[16];
  for (int i = 0; i < m; ++i) perm[i] = i;
  for (int c = 0; c < m; ++c) {
    int p = c;
    double mx = fabs(a[c][c]);
    for (int r = c + 1; r < m; ++r)
      if (fabs(a[r][c]) > mx) { mx = fabs(a[r][c]); p = r; }
    if (p != c) {
      for (int cc = 0; cc < m; ++cc) { double tmp = a[c][cc]; a[c][cc] = a[p][cc]; a[p][cc] = tmp; }
      double tb = b[c]; b[c] = b[p]; b[p] = tb;
      int tp = perm[c]; perm[c] = perm[p]; perm[p] = tp;
    }
    if (a[c][c] == 0.0) return -3;
    double rinv = 1.0 / a[c][c];
    for (int r = c + 1; r < m; ++r) {
      double l = a[r][c] * rinv;
      a[r][c] = l;
      for (int cc = c + 1; cc < m; ++cc) a[r][cc] = a[r][cc] - l * a[c][cc];
    }
  }
  /* triangular solves in the column order of dtrsm (unit lower, then upper) */
  for (int c = 0; c < m; ++c)
    if (b[c] != 0.0)
      for (int r = c + 1; r < m; ++r) b[r] = b[r] - b[c] * a[r][c];
  for (int c = m - 1; c >= 0; --c) {
    if (b[c] != 0.0) {
      b[c] = b[c] / a[c][c];
      for (int r = 0; r < c; ++r) b[r] = b[r] - b[c] * a[r][c];
    }
  }
  for (int i = 0; i < m; ++i) w[i] = scale * b[i];
  return 0;
}
