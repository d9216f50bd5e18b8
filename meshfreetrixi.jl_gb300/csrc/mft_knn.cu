// K1: exact k-nearest-neighbour stencils on a uniform grid of buckets.
//
// Replaces KDTree + knn(tree, points, nv, true) and the dx statistics of PointData
// (src/domains/PointCloudDomain/geometry_primatives.jl:322-339).  The order of a
// stencil is (squared distance, node index): the squared distance is summed over
// axes in order with each square rounded separately (no FMA), as Distances.jl's
// Euclidean reduction does, so ties are resolved by the smaller node index.
//
// One thread per query; queries run in bucket order so that neighbouring threads
// scan the same buckets.  Buckets are visited in growing Chebyshev rings; a ring
// search stops once the k-th best squared distance is below the squared distance
// from the query to the unexplored region (with a 1e-9 relative safety margin).
// The running top-k list lives in shared memory, slot-major across the block's
// threads (conflict-free), as (bits of d2, index) pairs: for non-negative doubles
// the bit pattern orders like the value.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "mft_ctx.h"

namespace mft {

namespace {

constexpr int kKnnBlock = 64;

struct KnnArgs {
  int dim, k;
  int64_t n;
  int64_t nc[3];
  double lo[3], cs[3], period[3];
  int periodic;
  const double* xyz;        // n x dim (caller order)
  const double* cxyz;       // n x dim in bucket order
  const int32_t* cpts;      // bucket order -> node index
  const int64_t* cstart;    // ncell + 1
  const int32_t* qcell;     // bucket of each node (caller order), flattened
  int32_t* out_idx;         // n x k
  double* out_d2;           // n x k squared distances
  int* err;
};

__device__ __forceinline__ double min_image(double d, double L) {
  if (d > 0.5 * L) return __dsub_rn(d, L);
  if (d < -0.5 * L) return __dadd_rn(d, L);
  return d;
}

__device__ __forceinline__ bool key_less(unsigned long long ka, int ja, unsigned long long kb,
                                         int jb) {
  return ka < kb || (ka == kb && ja < jb);
}

__global__ void __launch_bounds__(kKnnBlock) k_knn(KnnArgs a) {
  extern __shared__ unsigned char smem[];
  const int T = kKnnBlock;
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem);
  int* ids = reinterpret_cast<int*>(keys + (size_t)a.k * T);
  const int64_t t = blockIdx.x * (int64_t)T + threadIdx.x;
  if (t >= a.n) return;
  const int k = a.k;
  const int dim = a.dim;
  const int32_t qi = a.cpts[t];  // query node (bucket order)
  double q[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) q[d] = a.xyz[(int64_t)qi * dim + d];
  int64_t qc[3] = {0, 0, 0};
  {
    int64_t c = a.qcell[qi];
    for (int d = 0; d < dim; ++d) {
      qc[d] = c % a.nc[d];
      c /= a.nc[d];
    }
  }
  int cnt = 0;
  // slot m of this thread: keys[m*T + tid]
  auto KEY = [&](int m) -> unsigned long long& { return keys[(size_t)m * T + threadIdx.x]; };
  auto ID = [&](int m) -> int& { return ids[(size_t)m * T + threadIdx.x]; };

  for (int r = 0;; ++r) {
    // index sets per axis at radius r and whether they cover the whole axis
    int64_t lo_i[3] = {0, 0, 0}, hi_i[3] = {0, 0, 0};
    bool full[3] = {true, true, true}, wrapall[3] = {false, false, false};
    for (int d = 0; d < 3; ++d) {
      if (d >= dim) { lo_i[d] = hi_i[d] = 0; full[d] = true; continue; }
      if (a.periodic) {
        if (2 * r + 1 >= a.nc[d]) { lo_i[d] = 0; hi_i[d] = a.nc[d] - 1; full[d] = true; wrapall[d] = true; }
        else { lo_i[d] = qc[d] - r; hi_i[d] = qc[d] + r; full[d] = false; }
      } else {
        lo_i[d] = qc[d] - r < 0 ? 0 : qc[d] - r;
        hi_i[d] = qc[d] + r >= a.nc[d] ? a.nc[d] - 1 : qc[d] + r;
        full[d] = (lo_i[d] == 0 && hi_i[d] == a.nc[d] - 1);
      }
    }
    const int rp = r - 1;  // previous radius (cells already visited)
    for (int64_t c2 = lo_i[2]; c2 <= hi_i[2]; ++c2)
      for (int64_t c1 = lo_i[1]; c1 <= hi_i[1]; ++c1)
        for (int64_t c0 = lo_i[0]; c0 <= hi_i[0]; ++c0) {
          const int64_t cc[3] = {c0, c1, c2};
          // skip buckets already inside the block of radius r-1
          bool inner = rp >= 0;
          int64_t w[3];
          for (int d = 0; d < 3; ++d) {
            int64_t v = cc[d];
            if (d < dim && a.periodic) v = ((v % a.nc[d]) + a.nc[d]) % a.nc[d];
            w[d] = v;
            if (!inner || d >= dim) continue;
            if (a.periodic) {
              if (2 * rp + 1 >= a.nc[d]) continue;
              int64_t off = ((v - qc[d]) % a.nc[d] + a.nc[d]) % a.nc[d];
              if (off > a.nc[d] / 2) off -= a.nc[d];
              if (off < -rp || off > rp) inner = false;
            } else {
              if (v < qc[d] - rp || v > qc[d] + rp) inner = false;
            }
          }
          if (inner) continue;
          (void)wrapall;
          const int64_t cell = w[0] + a.nc[0] * (w[1] + a.nc[1] * w[2]);
          for (int64_t p = a.cstart[cell]; p < a.cstart[cell + 1]; ++p) {
            const int j = a.cpts[p];
            double s = 0.0;
            for (int d = 0; d < dim; ++d) {
              double dd = __dsub_rn(a.cxyz[p * dim + d], q[d]);
              if (a.periodic) dd = min_image(dd, a.period[d]);
              s = __dadd_rn(s, __dmul_rn(dd, dd));
            }
            const unsigned long long key = (unsigned long long)__double_as_longlong(s);
            if (cnt < k) {
              int m = cnt++;
              while (m > 0 && key_less(key, j, KEY(m - 1), ID(m - 1))) {
                KEY(m) = KEY(m - 1);
                ID(m) = ID(m - 1);
                --m;
              }
              KEY(m) = key;
              ID(m) = j;
            } else if (key_less(key, j, KEY(k - 1), ID(k - 1))) {
              int m = k - 1;
              while (m > 0 && key_less(key, j, KEY(m - 1), ID(m - 1))) {
                KEY(m) = KEY(m - 1);
                ID(m) = ID(m - 1);
                --m;
              }
              KEY(m) = key;
              ID(m) = j;
            }
          }
        }
    bool all = true;
    double bound = INFINITY;
    for (int d = 0; d < dim; ++d) {
      if (full[d]) continue;
      all = false;
      if (a.periodic) {
        const double l = q[d] - (a.lo[d] + (double)(qc[d] - r) * a.cs[d]);
        const double h = (a.lo[d] + (double)(qc[d] + r + 1) * a.cs[d]) - q[d];
        bound = fmin(bound, fmin(l, h));
      } else {
        if (lo_i[d] > 0) bound = fmin(bound, q[d] - (a.lo[d] + (double)lo_i[d] * a.cs[d]));
        if (hi_i[d] < a.nc[d] - 1)
          bound = fmin(bound, (a.lo[d] + (double)(hi_i[d] + 1) * a.cs[d]) - q[d]);
      }
    }
    if (cnt >= k) {
      const double kth = __longlong_as_double((long long)KEY(k - 1));
      if (all || (bound > 0 && kth < bound * bound * (1.0 - 1e-9))) break;
    } else if (all) {
      atomicExch(a.err, 1);
      return;
    }
    if (r > 4096) {  // cannot happen for k <= n; keeps the loop bounded
      atomicExch(a.err, 2);
      return;
    }
  }
  for (int m = 0; m < k; ++m) {
    a.out_idx[(int64_t)qi * k + m] = ID(m);
    a.out_d2[(int64_t)qi * k + m] = __longlong_as_double((long long)KEY(m));
  }
}

// Julia's pairwise reduction (Base.mapreduce_impl, block size 1024).
double pairwise(const double* x, int64_t lo, int64_t hi) {
  if (lo == hi) return x[lo];
  if (hi - lo < 1024) {
    double v = x[lo] + x[lo + 1];
    for (int64_t i = lo + 2; i <= hi; ++i) v = v + x[i];
    return v;
  }
  const int64_t mid = lo + ((hi - lo) >> 1);
  const double a = pairwise(x, lo, mid);
  const double b = pairwise(x, mid + 1, hi);
  return a + b;
}

double julia_sum(const std::vector<double>& x) {
  const int64_t n = (int64_t)x.size();
  if (n == 0) return 0.0;
  if (n == 1) return x[0];
  if (n < 16) {
    double v = x[0] + x[1];
    for (int64_t i = 2; i < n; ++i) v = v + x[i];
    return v;
  }
  return pairwise(x.data(), 0, n - 1);
}

}  // namespace

void knn_device(mft_ctx* c, int k, std::vector<int32_t>& idx, std::vector<double>* dist,
                double* dx_min, double* dx_avg) {
  const int dim = c->dim;
  const int64_t n = c->n;
  const double* x = c->xyz.data();
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) {
    lo[d] = hi[d] = x[d];
    for (int64_t i = 1; i < n; ++i) {
      lo[d] = std::min(lo[d], x[i * dim + d]);
      hi[d] = std::max(hi[d], x[i * dim + d]);
    }
  }
  double vol = 1.0;
  for (int d = 0; d < dim; ++d) {
    double ext = c->periodic ? c->period[d] : hi[d] - lo[d];
    if (ext <= 0) ext = 1.0;
    vol *= ext;
  }
  const double cs0 = pow(vol * 2.0 / (double)n, 1.0 / dim);
  int64_t nc[3] = {1, 1, 1};
  double cs[3] = {cs0, cs0, cs0};
  for (int d = 0; d < dim; ++d) {
    const double ext = c->periodic ? c->period[d] : hi[d] - lo[d];
    int64_t m = (int64_t)floor(ext / cs0);
    m = std::max<int64_t>(1, std::min<int64_t>(m, 4096));
    nc[d] = m;
    cs[d] = c->periodic ? c->period[d] / (double)m : (ext > 0 ? ext / (double)m : 1.0);
    if (!c->periodic) cs[d] *= (1.0 + 1e-12);
  }
  const int64_t ncell = nc[0] * nc[1] * nc[2];
  std::vector<int32_t> cell(n);
  std::vector<int64_t> cstart(ncell + 1, 0);
  for (int64_t i = 0; i < n; ++i) {
    int64_t cc = 0, mul = 1;
    for (int d = 0; d < dim; ++d) {
      int64_t ci = (int64_t)floor((x[i * dim + d] - lo[d]) / cs[d]);
      ci = std::max<int64_t>(0, std::min<int64_t>(ci, nc[d] - 1));
      cc += ci * mul;
      mul *= nc[d];
    }
    cell[i] = (int32_t)cc;
    cstart[cc + 1]++;
  }
  for (int64_t q = 0; q < ncell; ++q) cstart[q + 1] += cstart[q];
  std::vector<int32_t> cpts(n);
  std::vector<double> cxyz((size_t)n * dim);
  {
    std::vector<int64_t> fill(cstart.begin(), cstart.end() - 1);
    for (int64_t i = 0; i < n; ++i) {
      const int64_t p = fill[cell[i]]++;
      cpts[p] = (int32_t)i;
      for (int d = 0; d < dim; ++d) cxyz[p * dim + d] = x[i * dim + d];
    }
  }
  cudaStream_t s = c->stream;
  DBuf<double> d_cxyz, d_d2;
  DBuf<int32_t> d_cpts, d_cell, d_idx;
  DBuf<int64_t> d_cstart;
  DBuf<int> d_err;
  d_cxyz.upload(cxyz, s);
  d_cpts.upload(cpts, s);
  d_cell.upload(cell, s);
  d_cstart.upload(cstart, s);
  d_idx.alloc((size_t)n * k);
  d_d2.alloc((size_t)n * k);
  d_err.alloc(1);
  d_err.zero(s);
  KnnArgs a{};
  a.dim = dim;
  a.k = k;
  a.n = n;
  for (int d = 0; d < 3; ++d) {
    a.nc[d] = nc[d];
    a.lo[d] = lo[d];
    a.cs[d] = cs[d];
    a.period[d] = c->period[d];
  }
  a.periodic = c->periodic ? 1 : 0;
  a.xyz = c->d_xyz.p;
  a.cxyz = d_cxyz.p;
  a.cpts = d_cpts.p;
  a.cstart = d_cstart.p;
  a.qcell = d_cell.p;
  a.out_idx = d_idx.p;
  a.out_d2 = d_d2.p;
  a.err = d_err.p;
  const size_t shmem = (size_t)k * kKnnBlock * (sizeof(unsigned long long) + sizeof(int));
  MFT_REQUIRE(shmem <= 200 * 1024, MFT_ERR_ARG, "k too large for the KNN kernel");
  if (shmem > 48 * 1024)
    MFT_CUDA(cudaFuncSetAttribute(k_knn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem));
  k_knn<<<(unsigned)((n + kKnnBlock - 1) / kKnnBlock), kKnnBlock, shmem, s>>>(a);
  MFT_LAUNCH_CHECK();
  int err = 0;
  idx.resize((size_t)n * k);
  MFT_CUDA(cudaMemcpyAsync(&err, d_err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  MFT_CUDA(cudaMemcpyAsync(idx.data(), d_idx.p, idx.size() * sizeof(int32_t),
                           cudaMemcpyDeviceToHost, s));
  // the squared distances: all of them when asked for, else only the nearest other
  // node's (column 1, for dx_min / dx_avg)
  std::vector<double> d2(dist ? (size_t)n * k : (size_t)n);
  if (dist) {
    MFT_CUDA(cudaMemcpyAsync(d2.data(), d_d2.p, d2.size() * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
  } else if (k >= 2) {
    MFT_CUDA(cudaMemcpy2DAsync(d2.data(), sizeof(double), d_d2.p + 1, (size_t)k * sizeof(double),
                               sizeof(double), (size_t)n, cudaMemcpyDeviceToHost, s));
  }
  MFT_CUDA(cudaStreamSynchronize(s));
  MFT_REQUIRE(err == 0, MFT_ERR_ARG, "KNN search could not collect k neighbours");
  if (dist) {
    dist->resize(d2.size());
    for (size_t e = 0; e < d2.size(); ++e) (*dist)[e] = sqrt(d2[e]);
  }
  const int64_t d2_stride = dist ? k : 1, d2_col = dist ? 1 : 0;
  // dx_min = minimum(dists)[2], dx_avg = mean(dists)[2] over the 2-NN query.
  if (k >= 2) {
    std::vector<double> nn(n);
    double m = INFINITY;
    for (int64_t i = 0; i < n; ++i) {
      nn[i] = sqrt(d2[(size_t)i * d2_stride + d2_col]);
      if (nn[i] < m || isnan(nn[i])) m = nn[i];
    }
    if (dx_min) *dx_min = m;
    if (dx_avg) *dx_avg = julia_sum(nn) / (double)n;
  } else {
    if (dx_min) *dx_min = NAN;
    if (dx_avg) *dx_avg = NAN;
  }
}

}  // namespace mft
