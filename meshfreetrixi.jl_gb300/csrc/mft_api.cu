// C ABI of libmeshfree_gb300.so and the host-side orchestration of one rhs!
// evaluation and of the SSP-RK3 integrator with the HistoryCallback.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <numeric>
#include <string>
#include <vector>

#include "mft_ctx.h"

using namespace mft;

#define MFT_VERSION_MAJOR 0
#define MFT_VERSION_MINOR 1
#define MFT_VERSION_PATCH 0

namespace {

template <class F>
mft_status guarded(mft_ctx* c, F&& f) {
  if (!c) return MFT_ERR_ARG;
  try {
    c->err.clear();
    f();
    return MFT_OK;
  } catch (const mft::Error& e) {
    c->err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    c->err = "host allocation failed";
    return MFT_ERR_NOMEM;
  } catch (const std::exception& e) {
    c->err = e.what();
    return MFT_ERR_ARG;
  }
}

void set_device(mft_ctx* c) { MFT_CUDA(cudaSetDevice(c->device)); }

// ---------------------------------------------------------------- ELL layout

// Entry order inside the rows of a staged row group.  A staged gather reads, at each
// slot, one neighbour record per lane from shared memory with 16-byte loads; the 8 lanes
// of a quarter-warp are served together, and records in the same bank group (their
// position in the group's list mod 8) at different positions are served one after
// another.  In ascending-column order the 8 lanes' positions fall into bank groups at
// random (2.1 serialised accesses per quarter-warp load in the forward layout of a
// Morton-ordered jittered cloud, 2.4 in the transpose layout).  A row's sum may run in any
// order that every gather of that layout shares, so the entries of each quarter-warp's
// rows are ordered slot by slot: the rows with the fewest bank groups left choose first,
// each an entry in a bank group no other lane of the quarter takes at this slot -- of the
// free groups the one with the most entries left over the quarter's rows, so that crowded
// groups spread over all slots; a row without a free group takes an entry another lane
// reads at this slot (one address is served once), else one from its fullest group
// (1.09 and 1.21 accesses per load then).  nrows: the quarter's rows (at most 8); lists:
// per row its entries' list positions, in CSR order; out: per row and slot the CSR offset
// (within the row) placed there.
static void spread_quarter(int nrows, const std::vector<int32_t>* lists,
                           std::vector<int32_t>* out) {
  // [row][bank group]: (pos, offset); per host thread, kept between calls (no allocation
  // per quarter once the capacities have grown)
  thread_local std::vector<std::pair<int32_t, int32_t>> bucket[8][8];
  for (auto& row : bucket)
    for (auto& b : row) b.clear();
  int left[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < nrows; ++k) {
    out[k].assign(lists[k].size(), 0);
    left[k] = (int)lists[k].size();
    for (int32_t j = 0; j < (int32_t)lists[k].size(); ++j)
      bucket[k][lists[k][j] & 7].emplace_back(lists[k][j], j);
  }
  for (int slot = 0;; ++slot) {
    int act[8], na = 0, nfree[8];
    int demand[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < nrows; ++k) {
      if (left[k] == 0) continue;
      act[na++] = k;
      nfree[k] = 0;
      for (int g = 0; g < 8; ++g) {
        demand[g] += (int)bucket[k][g].size();
        nfree[k] += bucket[k][g].empty() ? 0 : 1;
      }
    }
    if (na == 0) break;
    for (int a = 1; a < na; ++a)  // fewest choices first (stable)
      for (int b = a; b > 0 && nfree[act[b]] < nfree[act[b - 1]]; --b) std::swap(act[b], act[b - 1]);
    unsigned used = 0;
    int32_t chosen[8];
    int nch = 0;
    for (int a = 0; a < na; ++a) {
      const int k = act[a];
      int g = -1;
      for (int x = 0; x < 8; ++x)
        if (!bucket[k][x].empty() && !(used >> x & 1u) && (g < 0 || demand[x] > demand[g])) g = x;
      size_t at = 0;
      if (g < 0) {
        for (int x = 0; x < 8 && g < 0; ++x)
          for (size_t e = 0; e < bucket[k][x].size() && g < 0; ++e)
            for (int c = 0; c < nch; ++c)
              if (bucket[k][x][e].first == chosen[c]) { g = x; at = e; break; }
        if (g < 0) {
          for (int x = 0; x < 8; ++x)
            if (!bucket[k][x].empty() && (g < 0 || bucket[k][x].size() > bucket[k][g].size())) g = x;
          at = 0;
        }
      }
      const std::pair<int32_t, int32_t> ent = bucket[k][g][at];
      bucket[k][g].erase(bucket[k][g].begin() + (std::ptrdiff_t)at);
      used |= 1u << g;
      chosen[nch++] = ent.first;
      out[k][slot] = ent.second;
      --left[k];
    }
  }
}

// Builds a sliced ELL over rows of a CSR-like structure.  pos[e] receives the
// ELL element of structure entry e.  Layout row r holds node base[r] (base: a spatial
// order of the nodes, see morton_order; null: node r).  With window > 0 the rows are
// then ordered by length, longest first, inside each run of `window` consecutive rows
// (stable, so rows stay near their neighbours): the 32 rows of a slice then have nearly
// equal lengths and the lanes of a warp finish together.
// With halo_rows > 0, the neighbour halos of the row groups are built too (halo_rows rows
// each: distinct columns ascending, and each element's position among them), and with
// spread the rows of the staged groups take their entries in the bank-spreading order of
// spread_quarter (else, and in the other groups, in structure order).
void build_ell(int64_t n, const std::vector<int64_t>& rowptr, const std::vector<int32_t>& cols,
               EllBuf& ell, std::vector<int64_t>& pos, cudaStream_t s, int window = 0,
               const std::vector<int32_t>* base = nullptr, int halo_rows = 0,
               bool spread = false) {
  std::vector<int32_t> order(n);
  if (base) order = *base;
  else std::iota(order.begin(), order.end(), 0);
  if (window > 0) {
#pragma omp parallel for schedule(static)
    for (int64_t w0 = 0; w0 < n; w0 += window) {
      const int64_t w1 = std::min<int64_t>(n, w0 + window);
      std::stable_sort(order.begin() + w0, order.begin() + w1, [&](int32_t x, int32_t y) {
        return rowptr[x + 1] - rowptr[x] > rowptr[y + 1] - rowptr[y];
      });
    }
  }
  const int64_t nsl = (n + kSlice - 1) / kSlice;
  std::vector<int64_t> soff(nsl + 1, 0);
  std::vector<int32_t> rlen(n);
#pragma omp parallel for schedule(static)
  for (int64_t sl = 0; sl < nsl; ++sl) {
    int m = 0;
    for (int64_t r = sl * kSlice; r < std::min<int64_t>(n, (sl + 1) * kSlice); ++r) {
      const int64_t node = order[r];
      const int len = (int)(rowptr[node + 1] - rowptr[node]);
      rlen[r] = len;
      m = std::max(m, len);
    }
    soff[sl + 1] = (int64_t)m * kSlice;
  }
  int maxlen = 0;
  for (int64_t sl = 0; sl < nsl; ++sl) {
    maxlen = std::max<int>(maxlen, (int)(soff[sl + 1] / kSlice));
    soff[sl + 1] += soff[sl];
  }
  const int64_t ne = soff[nsl];
  // neighbour halos: per group the distinct columns its rows gather, ascending
  const bool halos = halo_rows > 0;
  if (halos)
    MFT_REQUIRE(halo_rows % kSlice == 0 && halo_rows <= kHaloRows, MFT_ERR_STATE,
                "halo groups must be whole slices of at most kHaloRows rows");
  const int64_t ng = halos ? (n + halo_rows - 1) / halo_rows : 0;
  std::vector<std::vector<int32_t>> lists(ng);
  // eorder[rowptr[node] + slot]: the CSR offset placed at that slot of the node's row
  std::vector<int32_t> eorder;
  if (halos && spread) eorder.resize(rowptr[n]);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t g = 0; g < ng; ++g) {
    std::vector<int32_t>& h = lists[g];
    const int64_t r0 = g * halo_rows, r1 = std::min<int64_t>(n, r0 + halo_rows);
    for (int64_t r = r0; r < r1; ++r) {
      const int64_t node = order[r];
      h.insert(h.end(), cols.begin() + rowptr[node], cols.begin() + rowptr[node] + rlen[r]);
    }
    std::sort(h.begin(), h.end());
    h.erase(std::unique(h.begin(), h.end()), h.end());
    if ((int64_t)h.size() > kHaloMax) h.clear();
    if (!spread) continue;
    std::vector<int32_t> qlists[8], qout[8];
    for (int64_t r = r0; r < r1; r += 8) {
      const int nr = (int)std::min<int64_t>(8, r1 - r);
      for (int k = 0; k < nr; ++k) {
        const int64_t node = order[r + k];
        const int32_t* rc = cols.data() + rowptr[node];
        qlists[k].resize(rlen[r + k]);
        for (int j = 0; j < rlen[r + k]; ++j)
          qlists[k][j] = h.empty() ? 0
                                   : (int32_t)(std::lower_bound(h.begin(), h.end(), rc[j]) - h.begin());
      }
      if (h.empty()) {  // gathered directly: structure order
        for (int k = 0; k < nr; ++k)
          for (int j = 0; j < rlen[r + k]; ++j) eorder[rowptr[order[r + k]] + j] = j;
        continue;
      }
      spread_quarter(nr, qlists, qout);
      for (int k = 0; k < nr; ++k)
        std::copy(qout[k].begin(), qout[k].end(), eorder.begin() + rowptr[order[r + k]]);
    }
  }
  std::vector<int32_t> col(ne);
  pos.assign(rowptr[n], 0);
  const bool reorder = !eorder.empty();
#pragma omp parallel for schedule(static)
  for (int64_t sl = 0; sl < nsl; ++sl) {
    const int m = (int)((soff[sl + 1] - soff[sl]) / kSlice);
    for (int64_t lane = 0; lane < kSlice; ++lane) {
      const int64_t r = sl * kSlice + lane;
      const int64_t node = r < n ? order[r] : 0;
      for (int j = 0; j < m; ++j) {
        const int64_t e = soff[sl] + (int64_t)j * kSlice + lane;
        if (r < n && j < rlen[r]) {
          const int64_t src = rowptr[node] + (reorder ? eorder[rowptr[node] + j] : j);
          col[e] = cols[src];
          pos[src] = e;
        } else {
          col[e] = (int32_t)(r < n ? node : 0);  // padding: a valid index, never read
        }
      }
    }
  }
  ell.n = n;
  ell.n_elems = ne;
  ell.max_len = maxlen;
  ell.window = window;
  ell.ordered = base != nullptr;
  ell.slice_off.upload(soff, s);
  ell.row_len.upload(rlen, s);
  ell.col.upload(col, s);
  if (window > 0 || base) ell.perm.upload(order, s);
  else ell.perm.release();
  ell.spread = halos && spread;
  ell.bank_milli = 0;
  if (!halos) {
    ell.halo_off.release();
    ell.halo_col.release();
    ell.lcol.release();
    ell.halo_groups = ell.halo_staged = 0;
    ell.halo_stride = 0;
    ell.halo_rows = 0;
    return;
  }
  std::vector<uint16_t> lcol(ne, 0);
  // shared-memory accesses of the staged groups: per quarter-warp load, the largest number
  // of distinct positions in one bank group (summed, and the loads counted)
  std::vector<int64_t> acc_sum(ng, 0), acc_cnt(ng, 0);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t g = 0; g < ng; ++g) {
    const std::vector<int32_t>& h = lists[g];
    if (h.empty()) continue;
    const int64_t r0 = g * halo_rows, r1 = std::min<int64_t>(n, r0 + halo_rows);
    for (int64_t r = r0; r < r1; ++r) {
      const int64_t sl = r / kSlice, lane = r % kSlice;
      for (int j = 0; j < rlen[r]; ++j) {
        const int64_t e = soff[sl] + (int64_t)j * kSlice + lane;
        lcol[e] = (uint16_t)(std::lower_bound(h.begin(), h.end(), col[e]) - h.begin());
      }
    }
    for (int64_t r = r0; r < r1; r += 8) {
      const int64_t sl = r / kSlice;
      const int m = (int)((soff[sl + 1] - soff[sl]) / kSlice);
      for (int j = 0; j < m; ++j) {
        int32_t q[8];
        int nq = 0;
        for (int64_t x = r; x < std::min<int64_t>(r + 8, r1); ++x)
          if (j < rlen[x]) q[nq++] = lcol[soff[sl] + (int64_t)j * kSlice + x % kSlice];
        if (nq == 0) continue;
        std::sort(q, q + nq);
        int per[8] = {0, 0, 0, 0, 0, 0, 0, 0}, worst = 0;
        for (int a = 0; a < nq; ++a)
          if (a == 0 || q[a] != q[a - 1]) worst = std::max(worst, ++per[q[a] & 7]);
        acc_sum[g] += worst;
        acc_cnt[g] += 1;
      }
    }
  }
  std::vector<int32_t> hoff(ng + 1, 0);
  int64_t staged = 0, wsum = 0, wcnt = 0;
  int stride = 0;
  for (int64_t g = 0; g < ng; ++g) {
    hoff[g + 1] = hoff[g] + (int32_t)lists[g].size();
    staged += lists[g].empty() ? 0 : 1;
    stride = std::max(stride, (int)lists[g].size());
    wsum += acc_sum[g];
    wcnt += acc_cnt[g];
  }
  ell.bank_milli = wcnt ? (int)((1000 * wsum + wcnt / 2) / wcnt) : 0;
  std::vector<int32_t> hcol(hoff[ng]);
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < ng; ++g)
    std::copy(lists[g].begin(), lists[g].end(), hcol.begin() + hoff[g]);
  ell.halo_off.upload(hoff, s);
  ell.halo_col.upload(hcol, s);
  ell.lcol.upload(lcol, s);
  ell.halo_groups = ng;
  ell.halo_staged = staged;
  ell.halo_stride = stride;
  ell.halo_rows = halo_rows;
  // the host vectors leave scope before the copies are done
  MFT_CUDA(cudaStreamSynchronize(s));
}

// Layout order of the nodes along a Morton (Z-order) curve of their coordinates: the 32
// rows of a slice are then a compact patch of the cloud instead of a strip of node
// numbers, so the neighbours the slice gathers overlap more and are found in L1 more
// often.  Coordinates are quantised over the cloud's bounding box to 31 bits per axis
// (2D) or 21 (3D) and their bits interleaved; ties keep node order.  Only which thread forms which
// row changes: every row's sum keeps its own order, so the results are unchanged.
// With ensemble members (seg_off, nseg > 0) the curve runs inside each member in turn, so
// that a warp's rows stay in one member (the members of an ensemble may overlap in space).
std::vector<int32_t> morton_order(int dim, int64_t n, const std::vector<double>& xyz,
                                  const std::vector<int64_t>& seg_off = {}) {
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) {
    lo[d] = hi[d] = n ? xyz[d] : 0.0;
    for (int64_t i = 1; i < n; ++i) {
      lo[d] = std::min(lo[d], xyz[i * dim + d]);
      hi[d] = std::max(hi[d], xyz[i * dim + d]);
    }
  }
  const int bits = dim == 1 ? 62 : (dim == 2 ? 31 : 21);
  const double top = (double)((1ull << bits) - 1);
  std::vector<uint64_t> key(n);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    uint64_t k = 0;
    uint64_t q[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      const double span = hi[d] - lo[d];
      double x = span > 0 ? (xyz[i * dim + d] - lo[d]) / span * top : 0.0;
      if (!(x >= 0)) x = 0;
      if (x > top) x = top;
      q[d] = (uint64_t)x;
    }
    for (int b = bits - 1; b >= 0; --b)
      for (int d = 0; d < dim; ++d) k = (k << 1) | ((q[d] >> b) & 1ull);
    key[i] = k;
  }
  std::vector<int32_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  if (seg_off.size() >= 2) {
    for (size_t m = 0; m + 1 < seg_off.size(); ++m)
      std::stable_sort(order.begin() + seg_off[m], order.begin() + seg_off[m + 1],
                       [&](int32_t a, int32_t b) { return key[a] < key[b]; });
  } else {
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t a, int32_t b) { return key[a] < key[b]; });
  }
  return order;
}

}  // namespace

namespace mft {

static cudaEvent_t pool_event(mft_ctx* c) {
  if (!c->ev_pool.empty()) {
    cudaEvent_t e = c->ev_pool.back();
    c->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  MFT_CUDA(cudaEventCreate(&e));
  return e;
}

ProfScope::ProfScope(mft_ctx* ctx, int k) : c(ctx), kind(k) {
  if (!c->prof_on) return;
  e1 = pool_event(c);
  MFT_CUDA(cudaEventRecord(e1, c->stream));
}

ProfScope::~ProfScope() {
  if (!c->prof_on || !e1) return;
  cudaEvent_t e2 = nullptr;
  if (!c->ev_pool.empty()) {
    e2 = c->ev_pool.back();
    c->ev_pool.pop_back();
  } else if (cudaEventCreate(&e2) != cudaSuccess) {
    c->ev_pool.push_back(e1);
    return;
  }
  cudaEventRecord(e2, c->stream);
  c->prof_pending.push_back({kind, {e1, e2}});
}

static void prof_drain(mft_ctx* c) {
  if (c->prof_pending.empty()) return;
  MFT_CUDA(cudaStreamSynchronize(c->stream));
  for (auto& p : c->prof_pending) {
    float ms = 0.f;
    MFT_CUDA(cudaEventElapsedTime(&ms, p.second.first, p.second.second));
    c->prof_ms[p.first] += ms;
    c->prof_n[p.first] += 1;
    c->ev_pool.push_back(p.second.first);
    c->ev_pool.push_back(p.second.second);
  }
  c->prof_pending.clear();
}

void finish_pattern(mft_ctx* c) {
  const int64_t n = c->n;
  const int64_t nnz = c->rp[n];
  // CSC view (rows ascending inside each column) with the map to CSR entries: column
  // counts, a prefix sum, entries placed through per-column cursors by all host
  // threads, then every column put back in ascending row order.
  c->cp.assign(n + 1, 0);
  int64_t* cp = c->cp.data();
  const int32_t* ci = c->ci.data();
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < nnz; ++e) __atomic_fetch_add(&cp[ci[e] + 1], (int64_t)1, __ATOMIC_RELAXED);
  for (int64_t j = 0; j < n; ++j) cp[j + 1] += cp[j];
  c->ri.assign(nnz, 0);
  c->csc2csr.assign(nnz, 0);
  std::vector<int64_t> fill(c->cp.begin(), c->cp.end() - 1);
  int32_t* ri = c->ri.data();
  int64_t* c2r = c->csc2csr.data();
  const int64_t* rp = c->rp.data();
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n; ++r)
    for (int64_t e = rp[r]; e < rp[r + 1]; ++e) {
      const int64_t p = __atomic_fetch_add(&fill[ci[e]], (int64_t)1, __ATOMIC_RELAXED);
      ri[p] = (int32_t)r;
      c2r[p] = e;
    }
#pragma omp parallel
  {
    std::vector<std::pair<int32_t, int64_t>> col;
#pragma omp for schedule(static)
    for (int64_t j = 0; j < n; ++j) {
      const int64_t b = cp[j], e = cp[j + 1];
      col.resize(e - b);
      for (int64_t q = b; q < e; ++q) col[q - b] = {ri[q], c2r[q]};
      std::sort(col.begin(), col.end());
      for (int64_t q = b; q < e; ++q) {
        ri[q] = col[q - b].first;
        c2r[q] = col[q - b].second;
      }
    }
  }
  for (int k = 0; k < kSlots; ++k) {
    c->val[k].clear();
    c->have_val[k] = false;
  }
  c->have_pattern = true;
  c->dev_dirty = true;
  c->fsal_valid = false;
}

void pattern_from_stencils(mft_ctx* c) {
  const int64_t n = c->n;
  c->rp.assign(n + 1, 0);
  c->ci.assign(c->st_ci.size(), 0);
  c->st2csr.assign(c->st_ci.size(), 0);
  // rows sorted by column on all host threads; (column, position) packed in one integer
  // gives one plain sort per row with equal columns in position order (rejected)
  int64_t dup = INT64_MAX;  // smallest row that lists a node twice
#pragma omp parallel
  {
    std::vector<int64_t> key;
    int64_t my_dup = INT64_MAX;
#pragma omp for schedule(static)
    for (int64_t r = 0; r < n; ++r) {
      const int64_t b = c->st_rp[r], e = c->st_rp[r + 1];
      key.resize(e - b);
      for (int64_t q = 0; q < e - b; ++q) key[q] = ((int64_t)c->st_ci[b + q] << 32) | q;
      std::sort(key.begin(), key.end());
      for (int64_t k = 0; k < e - b; ++k) {
        const int64_t src = b + (key[k] & 0xffffffffll);
        if (k > 0 && (key[k] >> 32) == (key[k - 1] >> 32)) my_dup = std::min(my_dup, r);
        c->ci[b + k] = c->st_ci[src];
        c->st2csr[src] = b + k;
      }
      c->rp[r + 1] = e;
    }
#pragma omp critical(mft_pattern_dup)
    dup = std::min(dup, my_dup);
  }
  MFT_REQUIRE(dup == INT64_MAX, MFT_ERR_ARG,
              "stencil of node " + std::to_string(dup) + " lists a node twice");
  finish_pattern(c);
}

void ensure_work(mft_ctx* c) {
  const int64_t n = c->n;
  const int V = c->nvars;
  MFT_REQUIRE(V > 0, MFT_ERR_STATE, "equations not set");
  const size_t nv = (size_t)n * V;
  for (auto* b : {&c->U[0], &c->U[1], &c->U[2], &c->U[3]}) b->alloc(nv);
  c->F.alloc((size_t)n * std::max(c->dim, 2) * V);
  c->du_p.alloc(nv);
  c->du_p2.alloc(nv);
  c->t.alloc((size_t)n * 2 * V);
  c->q.alloc(nv);
  c->hvf.alloc(nv);
  c->eps.alloc(n);
  if (c->approx_du.n != nv) {
    c->approx_du.alloc(nv);
    c->approx_du.zero(c->stream);
  }
  c->soa.alloc(nv);
  c->soa2.alloc(nv);
  c->work_u.alloc(nv);
  c->work_du.alloc(nv);
  if (!c->kerr.p) {
    c->kerr.alloc(1);
    c->kerr.zero(c->stream);
  }
  // the norm reductions: 512 blocks (measured on the 1M cloud: 2048 blocks of four nodes
  // per thread take 37 µs for the mean instead of 25, the per-block combine dominating)
  const int rb = 512;
  if (c->red_blocks != rb) {
    c->red_blocks = rb;
    c->red_partial.alloc((size_t)rb * 8);
  }
  if (!c->red_counter.p) {
    c->red_counter.alloc(2);
    c->red_counter.zero(c->stream);
    c->mean.alloc(8);
    c->norms.alloc(8);
  }
  if (use_dw(c)) {
    c->Fdw.alloc((size_t)n * 2 * V);
    c->udw.alloc(nv);
    c->tdw.alloc((size_t)n * 2 * V);
    c->qdw.alloc(nv);
  }
  if (use_dw3(c)) c->Fdw.alloc((size_t)n * 12);  // the 12 distinct flux pairs of a node
  if (c->precision == MFT_PREC_FP32) {
    for (auto* b : {&c->U32[0], &c->U32[1], &c->U32[2], &c->U32[3]}) b->alloc(nv);
    c->du_p32.alloc(nv);
    c->du_p2_32.alloc(nv);
    c->t32.alloc((size_t)n * 2 * V);
    c->q32.alloc(nv);
    c->work_u32.alloc(nv);
    c->work_du32.alloc(nv);
  }
}

constexpr int kRevWindow = 256;

void ensure_device_ops(mft_ctx* c) {
  MFT_REQUIRE(c->have_pattern, MFT_ERR_STATE, "no operator pattern: call mft_knn, mft_set_stencils or mft_load_csc");
  for (int d = 0; d < c->dim; ++d)
    MFT_REQUIRE(c->have_val[d], MFT_ERR_STATE,
                "gradient operator component " + std::to_string(d) + " not set");
  // The FP64 transpose gathers are FP64-issue-bound, so lanes idling in a slice's
  // longest row cost time: their layout orders rows by length in windows of 256
  // (~99 % lane use instead of ~93 % on jittered clouds).  The latency-bound FP32
  // gathers keep node order, which keeps a warp's neighbours close in L1.
  const int rev_window = c->precision == MFT_PREC_FP64 ? kRevWindow : 0;
  if (c->rev.n == c->n && c->rev.window != rev_window) c->dev_dirty = true;
  const bool spatial = c->layout_order == 1 && !c->xyz.empty();
  if (c->fwd.n == c->n && c->fwd.ordered != spatial) c->dev_dirty = true;
  // double-word operator values are placed only while that form is in use
  const bool dw = use_dw(c) || use_dw3(c);
  if (dw && !c->fwdw[0].p) c->dev_dirty = true;
  // neighbour halos of the row groups, for the staged gathers (double-word 2D and 3D Euler
  // forms, FP32 2D Euler form)
  const bool halo = use_dw(c) || use_dw3(c) ||
                    (c->precision == MFT_PREC_FP32 && c->eq == MFT_EQ_EULER2D);
  if (halo && !c->fwd.halo_off.p) c->dev_dirty = true;
  // 256-row groups when that still gives every SM several blocks, else 128
  int nsm = 0;
  MFT_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
  // 3D clouds: 128-row groups (a 256-row group of a jittered cube gathers ~850 distinct
  // neighbours, beyond kHaloMax; a 128-row group ~520)
  const int halo_rows =
      !halo ? 0
            : (c->halo_rows_opt > 0
                   ? c->halo_rows_opt
                   : (c->dim == 3 || c->n / kHaloRows < 4 * (int64_t)nsm ? kHaloRows / 2
                                                                         : kHaloRows));
  if (halo && c->fwd.halo_rows != halo_rows) c->dev_dirty = true;
  const bool spread = halo && c->entry_order == 1;
  if (halo && c->fwd.spread != spread) c->dev_dirty = true;
  if (!c->dev_dirty) return;
  c->graph_valid = false;
  cudaStream_t s = c->stream;
  std::vector<int64_t> pos;
  std::vector<int32_t> zorder;
  if (spatial)
    zorder = morton_order(c->dim, c->n, c->xyz,
                          c->nseg > 0 ? c->seg_off : std::vector<int64_t>{});
  const std::vector<int32_t>* base = spatial ? &zorder : nullptr;
  build_ell(c->n, c->rp, c->ci, c->fwd, pos, s, 0, base, halo_rows, spread);
  c->fwd_pos.upload(pos, s);
  std::vector<int64_t> rpos_csc;
  build_ell(c->n, c->cp, c->ri, c->rev, rpos_csc, s, rev_window, base, halo_rows, spread);
  std::vector<int64_t> rpos(rpos_csc.size());
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < (int64_t)rpos_csc.size(); ++p) rpos[c->csc2csr[p]] = rpos_csc[p];
  c->rev_pos.upload(rpos, s);
  // values: uploaded once in structure order, placed into both layouts (FP64 and FP32)
  // on the device; padding elements stay zero
  DBuf<double> d_v;
  for (int k = 0; k < kSlots; ++k) {
    if (!c->have_val[k]) {
      c->fw[k].release(); c->rw[k].release(); c->fw32[k].release(); c->rw32[k].release();
      c->fwdw[k].release(); c->rwdw[k].release();
      continue;
    }
    const std::vector<double>& v = c->val[k];
    d_v.upload(v, s);
    c->fw[k].alloc(c->fwd.n_elems);
    c->rw[k].alloc(c->rev.n_elems);
    c->fw32[k].alloc(c->fwd.n_elems);
    c->rw32[k].alloc(c->rev.n_elems);
    for (auto* b : {&c->fw[k], &c->rw[k]}) b->zero(s);
    for (auto* b : {&c->fw32[k], &c->rw32[k]}) b->zero(s);
    if (dw) {
      c->fwdw[k].alloc(c->fwd.n_elems);
      c->rwdw[k].alloc(c->rev.n_elems);
      for (auto* b : {&c->fwdw[k], &c->rwdw[k]}) b->zero(s);
    } else {
      c->fwdw[k].release();
      c->rwdw[k].release();
    }
    launch_scatter_values((int64_t)v.size(), c->fwd_pos.p, d_v.p, c->fw[k].p, c->fw32[k].p,
                          c->fwdw[k].p, s);
    launch_scatter_values((int64_t)v.size(), c->rev_pos.p, d_v.p, c->rw[k].p, c->rw32[k].p,
                          c->rwdw[k].p, s);
  }
  MFT_CUDA(cudaStreamSynchronize(s));
  c->dev_dirty = false;
  for (int &k : c->tuned_fwd) k = -1;
  for (int &k : c->tuned_rev) k = -1;
  for (int &k : c->tuned_fwd_dw) k = -1;
  for (int &k : c->tuned_rev_dw) k = -1;
}

static void ensure_bcs(mft_ctx* c) {
  if (!c->bc_dirty) return;
  c->graph_valid = false;
  cudaStream_t s = c->stream;
  const int64_t n = c->n;
  std::vector<int8_t> tag(n, 0);
  std::vector<int32_t> slot(n, 0);
  std::vector<int32_t> bnode;
  const int64_t total = c->n_bc ? c->bc_ptr[c->n_bc] : 0;
  for (int b = 0; b < c->n_bc; ++b) {
    const int k = c->bc_kind[b];
    for (int64_t p = c->bc_ptr[b]; p < c->bc_ptr[b + 1]; ++p) {
      const int32_t i = c->bc_idx[p];
      if (k == MFT_BC_DO_NOTHING) continue;
      // apply_slip_velocity is written for CompressibleEulerEquations2D
      // (PointCloudBCs.jl:15-21); scalar advection ignores slip walls
      MFT_REQUIRE(!(k == MFT_BC_SLIP_WALL && c->eq == MFT_EQ_EULER3D), MFT_ERR_UNSUPPORTED,
                  "slip walls: 2D Euler only");
      if (k == MFT_BC_SLIP_WALL && c->eq != MFT_EQ_EULER2D) continue;
      MFT_REQUIRE(tag[i] == 0, MFT_ERR_UNSUPPORTED,
                  "node " + std::to_string(i) + " carries two active boundary conditions");
      tag[i] = k == MFT_BC_DIRICHLET ? 1 : 2;
      slot[i] = (int32_t)p;
      bnode.push_back(i);
    }
  }
  c->nb = (int64_t)bnode.size();
  c->d_tag.upload(tag, s);
  c->d_slot.upload(slot, s);
  std::vector<double> nrm((size_t)std::max<int64_t>(total, 1) * 2, 0.0);
  for (int64_t p = 0; p < total && !c->bc_normal.empty(); ++p)
    for (int d = 0; d < 2 && d < c->dim; ++d) nrm[p * 2 + d] = c->bc_normal[p * c->dim + d];
  c->d_normal.upload(nrm, s);
  if (bnode.empty()) bnode.push_back(0);
  c->d_bnode.upload(bnode, s);
  c->d_dvals.alloc((size_t)std::max<int64_t>(total, 1) * std::max(c->nvars, 1));
  if (!c->dir_values.empty())
    MFT_CUDA(cudaMemcpyAsync(c->d_dvals.p, c->dir_values.data(),
                             c->dir_values.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  MFT_CUDA(cudaStreamSynchronize(s));
  c->bc_dirty = false;
}

// Dirichlet values for time t through the registered host callback.
static void refresh_dirichlet(mft_ctx* c, double t) {
  if (!c->dir_fn || c->n_bc == 0) return;
  const int64_t total = c->bc_ptr[c->n_bc];
  c->dir_scratch.assign((size_t)total * c->nvars, 0.0);
  c->dir_fn(t, total, c->nvars, c->dir_scratch.data(), c->dir_user);
  MFT_CUDA(cudaStreamSynchronize(c->stream));
  MFT_CUDA(cudaMemcpyAsync(c->d_dvals.p, c->dir_scratch.data(),
                           c->dir_scratch.size() * sizeof(double), cudaMemcpyHostToDevice,
                           c->stream));
  MFT_CUDA(cudaStreamSynchronize(c->stream));
}

// ---------------------------------------------------------------- gather autotuner
//
// The FP32 Euler gathers have four mappings: one node per thread with direct loads
// (choice 0), one node per thread with each 256-row group's neighbour records staged in
// shared memory (choice 1, mft_halo.cuh), and one warp per 32-row slice with the slice's
// indices/weights staged in shared memory by bulk copies, 4 or 8 slots per copy (choices
// 4, 8).  With
// MFT_GATHER_AUTO the first launch of each kernel configuration times every mapping on
// the live inputs (CUDA events, best of 3 after a warm-up) and keeps the fastest for this
// context until the operators change.

static const int kGatherChoices[4] = {0, 1, 4, 8};

// Times launch(choice) for every choice (a warm-up launch, then the best of 3 CUDA-event
// timed launches) and returns the fastest choice.
template <class Launch>
static int tune_choices(mft_ctx* c, const int* choices, int nchoice, Launch&& launch) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  MFT_CUDA(cudaEventCreate(&e0));
  MFT_CUDA(cudaEventCreate(&e1));
  int best = choices[0];
  float best_ms = 1e30f;
  for (int q = 0; q < nchoice; ++q) {
    const int choice = choices[q];
    launch(choice);
    float t = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      MFT_CUDA(cudaEventRecord(e0, c->stream));
      launch(choice);
      MFT_CUDA(cudaEventRecord(e1, c->stream));
      MFT_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      MFT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      t = std::min(t, ms);
    }
    if (t < best_ms) {
      best_ms = t;
      best = choice;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

template <class Launch>
static int tune_gather(mft_ctx* c, Launch&& launch) {
  return tune_choices(c, kGatherChoices, 4, launch);
}

template <class Launch>
static int tune_variants(mft_ctx* c, int nvariants, Launch&& launch) {
  constexpr int kMax = 16;
  static_assert(kDwVariants <= kMax, "tuner choice table");
  int choices[kMax];
  const int nv = std::min(nvariants, kMax);
  for (int k = 0; k < nv; ++k) choices[k] = k;
  return tune_choices(c, choices, nv, launch);
}

static void launch_fwd_f32_choice(mft_ctx* c, const FwdArgs& a, int ch) {
  if (ch == 1 && launch_fwd_f32_halo(a, c->stream)) return;
  if (ch > 1 && launch_fwd_f32_tma(a, ch, c->kerr.p, c->stream)) return;
  launch_fwd_f32(a, c->stream);
}

static void launch_rev_f32_choice(mft_ctx* c, const RevArgs& a, int ch) {
  if (ch == 1 && launch_rev_f32_halo(a, c->stream)) return;
  if (ch > 1 && launch_rev_f32_tma(a, ch, c->kerr.p, c->stream)) return;
  launch_rev_f32(a, c->stream);
}

static int fwd_choice(mft_ctx* c, const FwdArgs& a) {
  if (a.V != 4) return 0;
  if (c->gather_mode == MFT_GATHER_THREAD) return 0;
  if (c->gather_mode == MFT_GATHER_STAGED) return 8;
  if (c->gather_mode == MFT_GATHER_HALO) return 1;
  const int key = (a.want_t ? 1 : 0) + (a.want_q ? 2 : 0) + 4 * a.flyer;
  if (c->tuned_fwd[key] < 0) {
    FwdArgs probe = a;
    probe.final_epilogue = 0;  // timing launches write only scratch outputs
    c->tuned_fwd[key] = tune_gather(c, [&](int ch) { launch_fwd_f32_choice(c, probe, ch); });
  }
  return c->tuned_fwd[key];
}

static int rev_choice(mft_ctx* c, const RevArgs& a) {
  if (a.V != 4) return 0;
  if (c->gather_mode == MFT_GATHER_THREAD) return 0;
  if (c->gather_mode == MFT_GATHER_STAGED) return 8;
  if (c->gather_mode == MFT_GATHER_HALO) return 1;
  const int key = (a.rv ? 1 : 0) + (a.lap ? 2 : 0);
  if (c->tuned_rev[key] < 0) {
    RevArgs probe = a;
    probe.final_epilogue = 0;
    probe.du_p_out32 = c->du_p2_32.p == a.du_p32 ? c->work_du32.p : c->du_p2_32.p;
    c->tuned_rev[key] = tune_gather(c, [&](int ch) { launch_rev_f32_choice(c, probe, ch); });
  }
  return c->tuned_rev[key];
}

// The double-word gathers have four kernel variants (plain or software-pipelined loop,
// with or without a register cap); with MFT_OPT_DW_VARIANT < 0 (default) the first
// launch of each configuration outside a graph capture times them on the live inputs and
// keeps the fastest until the operators change.
static int dw_fwd_choice(mft_ctx* c, const FwdArgs& a) {
  if (c->dw_variant >= 0) return c->dw_variant;
  const int key = (a.want_t ? 1 : 0) + (a.want_q ? 2 : 0) + 4 * a.flyer;
  if (c->tuned_fwd_dw[key] < 0) {
    if (c->capturing) return 0;
    FwdArgs probe = a;
    probe.final_epilogue = 0;  // timing launches write only scratch outputs
    // with fused staging possible, an unfused variant is timed with the flux kernel it
    // needs (which rewrites the same pairs)
    c->tuned_fwd_dw[key] = tune_variants(c, kDwVariants, [&](int v) {
      if (probe.fuse_flux && !dw_fwd_fuses(v))
        launch_prep_euler_dw(probe.n, c->gamma, probe.ustate, c->Fdw.p, c->udw.p, c->stream);
      launch_fwd_dw(probe, v, c->stream);
    });
  }
  return c->tuned_fwd_dw[key];
}

static int dw_rev_choice(mft_ctx* c, const RevArgs& a) {
  if (c->dw_variant >= 0) return c->dw_variant;
  const int key = (a.rv ? 1 : 0) + (a.lap ? 2 : 0);
  if (c->tuned_rev_dw[key] < 0) {
    if (c->capturing) return 0;
    RevArgs probe = a;
    probe.final_epilogue = 0;
    probe.du_p_out = c->du_p2.p == a.du_p ? c->work_du.p : c->du_p2.p;
    c->tuned_rev_dw[key] = tune_variants(c, kDwVariants, [&](int v) {
      launch_rev_dw(probe, v, c->stream);
    });
  }
  return c->tuned_rev_dw[key];
}

void launch_fwd(mft_ctx* c, const FwdArgs& a) {
  if (c->precision == MFT_PREC_FP32) {
    const int ch = fwd_choice(c, a);
    c->last_fwd_choice = ch;
    launch_fwd_f32_choice(c, a, ch);
  } else if (use_dw(c)) {
    const int v = dw_fwd_choice(c, a);
    c->last_fwd_choice = v;
    launch_fwd_dw(a, v, c->stream);
  } else {
    launch_fwd_f64(a, c->stream);
  }
}
void launch_rev(mft_ctx* c, const RevArgs& a) {
  if (c->precision == MFT_PREC_FP32) {
    const int ch = rev_choice(c, a);
    c->last_rev_choice = ch;
    launch_rev_f32_choice(c, a, ch);
  } else if (use_dw(c)) {
    const int v = dw_rev_choice(c, a);
    c->last_rev_choice = v;
    launch_rev_dw(a, v, c->stream);
  } else {
    launch_rev_f64(a, c->stream);
  }
}

// Device error word set by kernels with bounded waits; read at synchronisation points.
// Synchronises the stream and reads the word: the word's copy into pinned memory is
// queued behind the work, so one synchronisation covers both.
static void check_kernel_errors(mft_ctx* c) {
  if (!c->kerr.p) {
    MFT_CUDA(cudaStreamSynchronize(c->stream));
    return;
  }
  if (!c->h_kerr) MFT_CUDA(cudaMallocHost(reinterpret_cast<void**>(&c->h_kerr), sizeof(int)));
  MFT_CUDA(cudaMemcpyAsync(c->h_kerr, c->kerr.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  MFT_CUDA(cudaStreamSynchronize(c->stream));
  const int e = *c->h_kerr;
  if (e != 0) {
    c->kerr.zero(c->stream);
    MFT_CUDA(cudaStreamSynchronize(c->stream));
    if (e == MFT_ERR_NONFINITE)
      throw mft::Error(e, "the state or du became NaN or infinite (outputs were written)");
    if (e == MFT_ERR_STATE)
      throw mft::Error(e, "a fused staged gather met a row group without a staged list");
    throw mft::Error(e, "a device wait gave up (bulk-copy completion not observed)");
  }
}

// Work buffers of the IGR source.
static void ensure_igr(mft_ctx* c) {
  const size_t n = (size_t)c->n;
  c->igr_prim.alloc(n * 3);
  for (auto* b : {&c->igr_rinv, &c->igr_x, &c->igr_r, &c->igr_u0, &c->igr_u1, &c->igr_c})
    b->alloc(n);
  c->igr_t.alloc(n * 2);
  c->igr_add.alloc(n * 2);
  c->igr_partial.alloc((n + kBlockHost - 1) / kBlockHost + 1);
  if (!c->igr_counter.p) {
    c->igr_counter.alloc(1);
    c->igr_counter.zero(c->stream);
  }
  c->igr_sc.alloc(1);
}

void eval_rhs(mft_ctx* c, double* us, float* us32, double t, const Epilogue& ep_in) {
  NvtxRange rng_rhs("rhs!");
  ensure_device_ops(c);
  ensure_bcs(c);
  refresh_dirichlet(c, t);
  cudaStream_t s = c->stream;
  const int64_t n = c->n;
  const int V = c->nvars;
  const bool f32 = c->precision == MFT_PREC_FP32;
  const bool dw = use_dw(c);
  MFT_REQUIRE(!f32 || us32, MFT_ERR_STATE, "FP32 apply needs the FP32 state shadow");
  MFT_REQUIRE(!dw || (c->Fdw.p && c->udw.p && c->tdw.p && c->qdw.p && c->fwdw[0].p &&
                      c->rwdw[0].p),
              MFT_ERR_STATE, "double-word work buffers not allocated");

  BcDev bc{c->d_tag.p, c->d_slot.p, c->d_normal.p, c->d_dvals.p};
  Epilogue ep = ep_in;
  ep.bc = bc;
  ep.has_bc = c->nb > 0;
  ep.err = c->kerr.p;
  ep.u_s = us;
  ep.fused = f32 ? 1 : 0;
  ep.cdt = ep.kind == kStage2 ? 0.25 * ep.dt : ep.kind == kStage3 ? (2.0 / 3.0) * ep.dt : ep.dt;

  // 1. strong BCs, pass 1 (mutates u)
  if (c->nb > 0) {
    NvtxRange rng("boundary flux");
    ProfScope ps(c, MFT_K_BC);
    launch_bc_pass1(c->nb, c->d_bnode.p, V, c->eq, bc, us, us32, s);
  }

  // sources: at most one viscosity source, one hyperviscosity source and one IGR source
  int iv = -1, ih = -1, ig = -1;
  for (size_t k = 0; k < c->src_kind.size(); ++k) {
    const int kind = c->src_kind[k];
    if (kind == MFT_SRC_RV || kind == MFT_SRC_UPWIND) {
      MFT_REQUIRE(iv < 0, MFT_ERR_UNSUPPORTED, "more than one viscosity source");
      iv = (int)k;
    } else if (kind == MFT_SRC_IGR) {
      MFT_REQUIRE(ig < 0, MFT_ERR_UNSUPPORTED, "more than one IGR source");
      ig = (int)k;
    } else {
      MFT_REQUIRE(ih < 0, MFT_ERR_UNSUPPORTED, "more than one hyperviscosity source");
      ih = (int)k;
    }
  }
  if (c->dim == 3) {
    // 3D clouds: the plain flux divergence (calc_fluxes! over D_x, D_y, D_z) with the
    // strong BCs and the stage epilogue, in FP64 fused multiply-adds
    MFT_REQUIRE(!f32, MFT_ERR_UNSUPPORTED, "3D point clouds: the FP64 form only");
    MFT_REQUIRE(iv < 0 && ih < 0 && ig < 0, MFT_ERR_UNSUPPORTED,
                "3D point clouds: no viscosity, hyperviscosity or IGR source (the "
                "reference writes them for the 2D Euler equations)");
    MFT_REQUIRE(c->have_val[2], MFT_ERR_STATE, "gradient operator component 2 not set");
    FwdArgs fa{};
    fa.n = n;
    fa.ell = c->fwd.view();
    for (int d = 0; d < 3; ++d) fa.w[d] = c->fw[d].p;
    fa.F = c->F.p;
    fa.u = us;
    fa.eq = c->eq;
    fa.V = V;
    fa.gamma = c->gamma;
    fa.ax = c->adv[0];
    fa.ay = c->adv[1];
    fa.az = c->adv[2];
    fa.final_epilogue = 1;
    fa.ep = ep;
    if (use_dw3(c)) {
      // double-word form: flux pairs per node, sums of double-word products
      MFT_REQUIRE(c->Fdw.p && c->fwdw[0].p && c->fwdw[1].p && c->fwdw[2].p, MFT_ERR_STATE,
                  "double-word 3D buffers not allocated");
      for (int d = 0; d < 3; ++d) fa.wdw[d] = c->fwdw[d].p;
      fa.Fdw = c->Fdw.p;
      {
        NvtxRange rng("calc fluxes");
        ProfScope ps(c, MFT_K_FLUX);
        launch_prep_euler3d_dw(n, c->gamma, us, c->Fdw.p, s);
      }
      NvtxRange rng("calc fluxes");
      ProfScope ps(c, MFT_K_FWD);
      launch_fwd3_dw(fa, s);
      return;
    }
    if (c->eq == MFT_EQ_EULER3D) {
      NvtxRange rng("calc fluxes");
      ProfScope ps(c, MFT_K_FLUX);
      launch_flux_euler3d(n, c->gamma, us, c->F.p, s);
    }
    NvtxRange rng("calc fluxes");
    ProfScope ps(c, MFT_K_FWD);
    launch_fwd3(fa, s);
    return;
  }
  const bool tominec = ih >= 0 && c->src_kind[ih] == MFT_SRC_HV_TOMINEC;
  const bool flyer = ih >= 0 && c->src_kind[ih] == MFT_SRC_HV_FLYER;
  const bool hv_first = ih >= 0 && iv >= 0 && ih < iv;
  const double hv_gamma = ih >= 0 ? c->src_par[ih * 4] : 0.0;
  if (tominec) MFT_REQUIRE(c->have_val[kSlotLap], MFT_ERR_STATE, "Tominec HV needs MFT_OP_LAP");
  if (flyer) MFT_REQUIRE(c->have_val[kSlotHv], MFT_ERR_STATE, "Flyer HV needs MFT_OP_HV");

  // Residual-viscosity normalisation (ode_mean, ode_maximum of u): it only reads the
  // BC-corrected state, so outside profiling it runs on a side stream while the flux and
  // forward gather kernels (FP64-bound, they leave memory and issue slots free) run here;
  // the viscosity kernel waits for it.
  auto rv_norms = [&](cudaStream_t st) {
    const int mode = (int)c->src_par[iv * 4 + 3];
    if (c->nseg > 0) {
      {
        ProfScope ps(c, MFT_K_MEAN);
        launch_mean_seg(c->nseg, c->d_seg_off.p, kSegBlocks, V, us, mode, c->seg_partial.p,
                        c->seg_counter.p, c->seg_mean.p, st);
      }
      ProfScope ps(c, MFT_K_LEXMAX);
      launch_lexmax_seg(c->nseg, c->d_seg_off.p, kSegBlocks, V, us, c->seg_mean.p, mode,
                        c->seg_partial.p, c->seg_counter.p + c->nseg, c->seg_norms.p, st,
                        !c->prof_on);
    } else {
      const double denom = mode == 0 ? (double)n * V : (double)n;
      {
        ProfScope ps(c, MFT_K_MEAN);
        launch_mean(n, V, us, denom, c->red_partial.p, c->red_counter.p, c->mean.p,
                    c->red_blocks, st);
      }
      ProfScope ps(c, MFT_K_LEXMAX);
      launch_lexmax(n, V, us, c->mean.p, mode, c->red_partial.p, c->red_counter.p + 1,
                    c->norms.p, c->red_blocks, st, !c->prof_on);
    }
  };
  // With the viscosity formed in the double-word forward gather's epilogue, the norms run
  // on this stream right before that gather, which is launched as their programmatic
  // dependent: its staging and sums overlap the reductions and only its epilogue waits.
  // Otherwise they run on the side stream beside the flux kernel and the forward gather.
  const bool fuse_eps = dw && iv >= 0 && !(tominec && hv_first);
  bool forked = false;
  if (iv >= 0 && c->src_kind[iv] == MFT_SRC_RV && !c->prof_on && !fuse_eps) {
    NvtxRange rng("source terms");
    MFT_CUDA(cudaEventRecord(c->ev_fork, s));
    MFT_CUDA(cudaStreamWaitEvent(c->stream2, c->ev_fork, 0));
    rv_norms(c->stream2);
    MFT_CUDA(cudaEventRecord(c->ev_join, c->stream2));
    forked = true;
  }

  // IGR: sigma from the BC-corrected state, added to the momentum rows in the epilogue
  if (ig >= 0) {
    MFT_REQUIRE(c->eq == MFT_EQ_EULER2D && c->dim == 2, MFT_ERR_UNSUPPORTED,
                "the IGR source needs the 2D Euler equations");
    ensure_igr(c);
    IgrArgs ia{};
    ia.n = n;
    ia.ell = c->fwd.view();
    ia.wx = c->fw[0].p;
    ia.wy = c->fw[1].p;
    ia.alpha = c->src_par[ig * 4];
    ia.maxiter = (int)c->src_par[ig * 4 + 1];
    ia.prim = c->igr_prim.p;
    ia.rinv = c->igr_rinv.p;
    ia.x = c->igr_x.p;
    ia.r = c->igr_r.p;
    ia.u0 = c->igr_u0.p;
    ia.u1 = c->igr_u1.p;
    ia.c = c->igr_c.p;
    ia.t = c->igr_t.p;
    ia.add = c->igr_add.p;
    ia.partial = c->igr_partial.p;
    ia.counter = c->igr_counter.p;
    ia.sc = c->igr_sc.p;
    {
      NvtxRange rng("source terms");
      ProfScope ps(c, MFT_K_IGR);
      launch_igr(ia, us, s);
    }
    ep.xadd = c->igr_add.p;
  }

  // 2. flux per node (FP64 Euler; double-word pairs of the flux and the state for the
  // double-word gathers).  The staged double-word forward variants 7, 11 and 12 can form
  // those records while staging when every row group is staged; once such a variant is
  // the chosen one the flux kernel is skipped (it still runs in the evaluation that tunes,
  // whose unfused variants read its pairs).
  const int fwd_flyer = flyer ? ((iv < 0 || hv_first) ? 1 : 2) : 0;
  const int fwd_key = (iv >= 0 ? 1 : 0) + (tominec ? 2 : 0) + 4 * fwd_flyer;
  const bool fuse_ok = dw && c->fuse_flux && c->fwd.halo_groups > 0 &&
                       c->fwd.halo_staged == c->fwd.halo_groups;
  const int fwd_known = c->dw_variant >= 0 ? c->dw_variant : c->tuned_fwd_dw[fwd_key];
  const bool skip_flux = fuse_ok && fwd_known >= 0 && dw_fwd_fuses(fwd_known);
  c->last_flux_fused = skip_flux ? 1 : 0;
  if (dw) {
    if (!skip_flux) {
      NvtxRange rng("calc fluxes");
      ProfScope ps(c, MFT_K_FLUX);
      launch_prep_euler_dw(n, c->gamma, us, c->Fdw.p, c->udw.p, s);
    }
  } else if (!f32 && c->eq == MFT_EQ_EULER2D) {
    NvtxRange rng("calc fluxes");
    ProfScope ps(c, MFT_K_FLUX);
    launch_flux_f64(n, c->eq, V, c->gamma, us, c->F.p, s);
  }

  // 3. forward gather
  FwdArgs fa{};
  fa.n = n;
  fa.ell = c->fwd.view();
  for (int d = 0; d < 3; ++d) {
    fa.w[d] = d < c->dim ? c->fw[d].p : nullptr;
    fa.w32[d] = d < c->dim ? c->fw32[d].p : nullptr;
  }
  const int wl_slot = tominec ? kSlotLap : (flyer ? kSlotHv : -1);
  fa.wl = wl_slot >= 0 ? c->fw[wl_slot].p : nullptr;
  fa.wl32 = wl_slot >= 0 ? c->fw32[wl_slot].p : nullptr;
  fa.F = c->F.p;
  fa.u = us;
  fa.u32 = us32;
  fa.eq = c->eq;
  fa.V = V;
  fa.gamma = c->gamma;
  fa.ax = c->adv[0];
  fa.ay = c->adv[1];
  fa.hv_gamma = hv_gamma;
  fa.want_t = iv >= 0;
  fa.want_q = tominec;
  fa.flyer = fwd_flyer;
  fa.fuse_flux = fuse_ok ? 1 : 0;
  fa.ustate = us;
  fa.gm1dw = gm1_pair(c->gamma);
  fa.err = c->kerr.p;
  fa.du_p = c->du_p.p;
  fa.t = c->t.p;
  fa.q = c->q.p;
  fa.hvf = c->hvf.p;
  fa.du_p32 = c->du_p32.p;
  fa.t32 = c->t32.p;
  fa.q32 = c->q32.p;
  fa.final_epilogue = (iv < 0 && !tominec);
  fa.ep = ep;
  // viscosity arguments (used by the viscosity kernel, or formed in the double-word
  // forward gather's epilogue when the viscosity's partial du is complete there)
  EpsArgs ea{};
  if (iv >= 0) {
    const int kind = c->src_kind[iv];
    const double* par = &c->src_par[iv * 4];
    ea.n = n;
    ea.eq = c->eq;
    ea.V = V;
    ea.kind = kind;
    ea.gamma = c->gamma;
    ea.ax = c->adv[0];
    ea.ay = c->adv[1];
    ea.c_rv = kind == MFT_SRC_RV ? par[0] : 0.0;
    ea.c_uw = kind == MFT_SRC_RV ? par[1] : par[0];
    ea.h = kind == MFT_SRC_RV ? par[2] : par[1];
    ea.success_iter = c->success_iter;
    ea.u = us;
    ea.u32 = f32 ? us32 : nullptr;
    ea.hvf = nullptr;
    ea.approx_du = c->approx_du.p;
    ea.norms = c->nseg > 0 ? c->seg_norms.p : c->norms.p;
    ea.seg_id = c->nseg > 0 ? c->d_seg_id.p : nullptr;
    ea.seg_h = c->nseg > 0 ? c->d_seg_h.p : nullptr;
    ea.t = (f32 || dw) ? nullptr : c->t.p;
    ea.t32 = f32 ? c->t32.p : nullptr;
    ea.tdw = dw ? c->tdw.p : nullptr;
    ea.eps = c->eps.p;
    ea.tab = c->capturing ? c->d_tab.p : nullptr;
    ea.ctr = c->d_ctr.p;
  }
  if (dw) {
    for (int d = 0; d < 3; ++d) fa.wdw[d] = d < c->dim ? c->fwdw[d].p : nullptr;
    fa.wldw = wl_slot >= 0 ? c->fwdw[wl_slot].p : nullptr;
    fa.Fdw = c->Fdw.p;
    fa.udw = c->udw.p;
    fa.tdw = c->tdw.p;
    fa.qdw = c->qdw.p;
  }
  if (fuse_eps) {
    // the norms of the residual viscosity must be complete before the gather's epilogue
    if (c->src_kind[iv] == MFT_SRC_RV) {
      rv_norms(s);
      // not while profiling (events between the launches) nor when this launch tunes
      // the variant (timing launches would sit between the reductions and the gather)
      fa.pdl = (!c->prof_on && fwd_known >= 0) ? 1 : 0;
    }
    fa.fuse_eps = 1;
    fa.ea = ea;
    fa.ea.du_p = c->du_p.p;
    prepare_eps(fa.ea);
  }
  {
    // the forward gather: the flux divergence (and the fused viscosity when formed here)
    NvtxRange rng("calc fluxes");
    ProfScope ps(c, MFT_K_FWD);
    launch_fwd(c, fa);
  }
  if (fa.final_epilogue) return;

  RevArgs ra{};
  ra.n = n;
  ra.ell = c->rev.view();
  for (int d = 0; d < 3; ++d) {
    ra.w[d] = d < c->dim ? c->rw[d].p : nullptr;
    ra.w32[d] = d < c->dim ? c->rw32[d].p : nullptr;
  }
  ra.wl = tominec ? c->rw[kSlotLap].p : nullptr;
  ra.wl32 = tominec ? c->rw32[kSlotLap].p : nullptr;
  ra.V = V;
  ra.hv_gamma = hv_gamma;
  ra.q = c->q.p;
  ra.q32 = c->q32.p;
  ra.s = c->t.p;
  ra.s32 = c->t32.p;
  if (dw) {
    for (int d = 0; d < 3; ++d) ra.wdw[d] = d < c->dim ? c->rwdw[d].p : nullptr;
    ra.wldw = tominec ? c->rwdw[kSlotLap].p : nullptr;
    ra.sdw = c->tdw.p;
    ra.qdw = c->qdw.p;
  }

  double* dp = c->du_p.p;
  float* dp32 = c->du_p32.p;
  if (tominec && hv_first) {
    // lap' q must be part of the partial du that the residual viscosity reads.
    RevArgs r1 = ra;
    r1.rv = 0;
    r1.lap = 1;
    r1.du_p = dp;
    r1.du_p32 = dp32;
    r1.hvf = nullptr;
    r1.final_epilogue = 0;
    r1.du_p_out = c->du_p2.p;
    r1.du_p_out32 = c->du_p2_32.p;
    r1.ep = ep;
    NvtxRange rng("source terms");
    ProfScope ps(c, MFT_K_REV_LAP);
    launch_rev(c, r1);
    dp = c->du_p2.p;
    dp32 = c->du_p2_32.p;
  }

  if (iv >= 0 && !fuse_eps) {
    if (forked) MFT_CUDA(cudaStreamWaitEvent(s, c->ev_join, 0));
    else if (c->src_kind[iv] == MFT_SRC_RV) rv_norms(s);
    ea.du_p = f32 ? nullptr : dp;
    ea.du_p32 = f32 ? dp32 : nullptr;
    NvtxRange rng("source terms");
    ProfScope ps(c, MFT_K_EPS);
    launch_eps(ea, s);
  }

  RevArgs r2 = ra;
  r2.rv = iv >= 0;
  r2.lap = tominec && !hv_first;
  r2.du_p = dp;
  r2.du_p32 = dp32;
  r2.hvf = (flyer && fa.flyer == 2) ? c->hvf.p : nullptr;
  r2.final_epilogue = 1;
  r2.du_p_out = nullptr;
  r2.ep = ep;
  // the transpose gather applies the viscosity and hyperviscosity sources; its epilogue
  // is pass 2 of the boundary conditions and the stage combination
  NvtxRange rng("source terms");
  ProfScope ps(c, MFT_K_REV);
  launch_rev(c, r2);
}

}  // namespace mft

// ---------------------------------------------------------------- history helpers

namespace {

// time_deriv_weights! (src/callbacks_step/history.jl:131-152): w = scale*(A'\b),
// A[i][k] = (t_i*scale)^k, b[k] = k*(t_0*scale)^(k-1), LU with partial pivoting.
int time_deriv_weights(int m, const double* t, double* w) {
  if (m < 1 || m > 16) return -1;
  double a[16][16], b[16], tt[16];
  double tmax = 0.0;
  for (int i = 0; i < m; ++i) {
    const double v = fabs(t[i]);
    if (isnan(v) || v > tmax) tmax = isnan(tmax) ? tmax : v;
  }
  const double scale = 1.0 / tmax;
  for (int i = 0; i < m; ++i) tt[i] = t[i] * scale;
  const double te = tt[0];
  auto pw = [](double x, int k) {
    if (k < 0) {
      double r = 1.0;
      for (int i = 0; i < -k; ++i) r = r * x;
      return 1.0 / r;
    }
    double r = 1.0;
    for (int i = 0; i < k; ++i) r = r * x;
    return r;
  };
  for (int i = 0; i < m; ++i)
    for (int k = 0; k < m; ++k) a[k][i] = k == 0 ? 1.0 : pw(tt[i], k);
  for (int k = 0; k < m; ++k) b[k] = (double)k * (k == 0 ? 1.0 / te : pw(te, k - 1));
  for (int cc = 0; cc < m; ++cc) {
    int p = cc;
    double mx = fabs(a[cc][cc]);
    for (int r = cc + 1; r < m; ++r)
      if (fabs(a[r][cc]) > mx) { mx = fabs(a[r][cc]); p = r; }
    if (p != cc) {
      for (int k = 0; k < m; ++k) std::swap(a[cc][k], a[p][k]);
      std::swap(b[cc], b[p]);
    }
    if (a[cc][cc] == 0.0) return -3;
    const double rinv = 1.0 / a[cc][cc];
    for (int r = cc + 1; r < m; ++r) {
      const double l = a[r][cc] * rinv;
      a[r][cc] = l;
      for (int k = cc + 1; k < m; ++k) a[r][k] = a[r][k] - l * a[cc][k];
    }
  }
  for (int cc = 0; cc < m; ++cc)
    if (b[cc] != 0.0)
      for (int r = cc + 1; r < m; ++r) b[r] = b[r] - b[cc] * a[r][cc];
  for (int cc = m - 1; cc >= 0; --cc) {
    if (b[cc] != 0.0) {
      b[cc] = b[cc] / a[cc][cc];
      for (int r = 0; r < cc; ++r) b[r] = b[r] - b[cc] * a[r][cc];
    }
  }
  for (int i = 0; i < m; ++i) w[i] = scale * b[i];
  return 0;
}

// modify_cache!(::SourceResidualViscosityTominec) (history.jl:91-103): push (t, u)
// into the ring (newest first) and rebuild approx_du from min(success_iter+1, p+1)
// points.
void history_push(mft_ctx* c, double t, const double* u_aos, int success_iter) {
  if (c->hist_order < 0) return;
  const int slots = c->hist_order + 1;
  const size_t nv = (size_t)c->n * c->nvars;
  cudaStream_t s = c->stream;
  c->success_iter = success_iter;
  for (int k = slots - 1; k > 0; --k) c->hist_t[k] = c->hist_t[k - 1];
  c->hist_t[0] = t;
  c->hist_head = (c->hist_head + slots - 1) % slots;
  const int m = std::min(success_iter + 1, slots);
  // host weights first, so that the timed region holds only the device work
  double w[16];
  if (success_iter > 0)
    MFT_REQUIRE(time_deriv_weights(m, c->hist_t.data(), w) == 0, MFT_ERR_SINGULAR,
                "time_deriv_weights: singular Vandermonde system");
  NvtxRange rng("history");
  ProfScope ps(c, MFT_K_HISTORY);
  if (success_iter <= 0) {
    MFT_CUDA(cudaMemcpyAsync(c->hist[c->hist_head].p, u_aos, nv * sizeof(double),
                             cudaMemcpyDeviceToDevice, s));
    c->approx_du.zero(s);
    return;
  }
  HistW hw{};
  for (int k = 0; k < m; ++k) hw.w[k] = w[k];
  // the kernel reads the new state from u_aos and writes its copy into the ring
  const double* hs[8];
  hs[0] = u_aos;
  for (int k = 1; k < m; ++k) hs[k] = c->hist[(c->hist_head + k) % slots].p;
  launch_history((int64_t)nv, m, hw, hs, c->hist[c->hist_head].p, c->approx_du.p,
                 c->precision == MFT_PREC_FP32, s);
}

void check_state_ready(mft_ctx* c) {
  MFT_REQUIRE(c->n > 0, MFT_ERR_STATE, "no points set");
  MFT_REQUIRE(c->eq >= 0, MFT_ERR_STATE, "equations not set");
}

}  // namespace

// ====================================================================== ABI

extern "C" {

mft_status mft_version(int* major, int* minor, int* patch) {
  if (major) *major = MFT_VERSION_MAJOR;
  if (minor) *minor = MFT_VERSION_MINOR;
  if (patch) *patch = MFT_VERSION_PATCH;
  return MFT_OK;
}

mft_status mft_ctx_create(mft_ctx** out, int device, int flags) {
  if (!out) return MFT_ERR_ARG;
  *out = nullptr;
  (void)flags;
  mft_ctx* c = nullptr;
  try {
    c = new mft_ctx();
  } catch (...) {
    return MFT_ERR_NOMEM;
  }
  c->device = device;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || device < 0 || device >= count) {
    delete c;
    return e != cudaSuccess ? MFT_ERR_CUDA : MFT_ERR_ARG;
  }
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_tab, cudaEventDisableTiming) != cudaSuccess) {
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    delete c;
    return MFT_ERR_CUDA;
  }
  *out = c;
  return MFT_OK;
}

mft_status mft_ctx_destroy(mft_ctx* c) {
  if (!c) return MFT_OK;
  cudaSetDevice(c->device);
  if (c->stream) {
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
  }
  if (c->stream2) {
    cudaStreamSynchronize(c->stream2);
    cudaStreamDestroy(c->stream2);
  }
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->ev_tab) cudaEventDestroy(c->ev_tab);
  if (c->h_tab) cudaFreeHost(c->h_tab);
  if (c->h_kerr) cudaFreeHost(c->h_kerr);
  for (auto& p : c->prof_pending) {
    cudaEventDestroy(p.second.first);
    cudaEventDestroy(p.second.second);
  }
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  for (auto g : c->gexec)
    if (g) cudaGraphExecDestroy(g);
  for (auto e : c->region_ev)
    if (e) cudaEventDestroy(e);
  delete c;
  return MFT_OK;
}

const char* mft_last_error(const mft_ctx* c) { return c ? c->err.c_str() : "null context"; }

mft_status mft_sync(mft_ctx* c) {
  return guarded(c, [&] {
    set_device(c);
    MFT_CUDA(cudaStreamSynchronize(c->stream));
  });
}

mft_status mft_set_points(mft_ctx* c, int dim, int64_t n, const double* xyz, const double* period) {
  return guarded(c, [&] {
    c->graph_valid = false;
    MFT_REQUIRE(dim >= 1 && dim <= 3, MFT_ERR_ARG, "dim must be 1, 2 or 3");
    MFT_REQUIRE(n >= 1 && n < (int64_t)INT32_MAX, MFT_ERR_ARG, "node count out of range");
    MFT_REQUIRE(xyz, MFT_ERR_ARG, "xyz is NULL");
    set_device(c);
    c->dim = dim;
    c->n = n;
    c->xyz.assign(xyz, xyz + (size_t)n * dim);
    c->periodic = period != nullptr;
    for (int d = 0; d < 3; ++d) c->period[d] = (period && d < dim) ? period[d] : 0.0;
    if (period)
      for (int d = 0; d < dim; ++d)
        MFT_REQUIRE(period[d] > 0.0, MFT_ERR_ARG, "period lengths must be positive");
    c->d_xyz.upload(c->xyz, c->stream);
    c->have_stencils = false;
    c->have_pattern = false;
    for (int k = 0; k < kSlots; ++k) c->have_val[k] = false;
    c->dev_dirty = true;
    c->bc_dirty = true;
    c->state_valid = false;
    c->fsal_valid = false;
    MFT_CUDA(cudaStreamSynchronize(c->stream));
  });
}

mft_status mft_set_stencils(mft_ctx* c, const int64_t* rowptr, const int32_t* cols) {
  return guarded(c, [&] {
    MFT_REQUIRE(c->n > 0, MFT_ERR_STATE, "call mft_set_points first");
    MFT_REQUIRE(rowptr && cols, MFT_ERR_ARG, "NULL stencil arrays");
    MFT_REQUIRE(rowptr[0] == 0, MFT_ERR_ARG, "rowptr[0] must be 0");
    for (int64_t i = 0; i < c->n; ++i)
      MFT_REQUIRE(rowptr[i + 1] > rowptr[i], MFT_ERR_ARG, "empty stencil");
    const int64_t nnz = rowptr[c->n];
    for (int64_t e = 0; e < nnz; ++e)
      MFT_REQUIRE(cols[e] >= 0 && cols[e] < c->n, MFT_ERR_ARG, "stencil index out of range");
    c->st_rp.assign(rowptr, rowptr + c->n + 1);
    c->st_ci.assign(cols, cols + nnz);
    c->have_stencils = true;
    pattern_from_stencils(c);
  });
}

mft_status mft_knn(mft_ctx* c, int k, int32_t* out_idx, double* out_dist, double* out_dx_min,
                   double* out_dx_avg) {
  return guarded(c, [&] {
    MFT_REQUIRE(c->n > 0, MFT_ERR_STATE, "call mft_set_points first");
    MFT_REQUIRE(k >= 1 && k <= c->n && k <= 1024, MFT_ERR_ARG, "k out of range");
    set_device(c);
    std::vector<int32_t> idx;
    std::vector<double> dist;
    double dmin = 0, davg = 0;
    knn_device(c, k, idx, out_dist ? &dist : nullptr, &dmin, &davg);
    c->st_rp.resize(c->n + 1);
    for (int64_t i = 0; i <= c->n; ++i) c->st_rp[i] = i * k;
    c->st_ci = idx;
    c->have_stencils = true;
    pattern_from_stencils(c);
    if (out_idx) memcpy(out_idx, idx.data(), idx.size() * sizeof(int32_t));
    if (out_dist) memcpy(out_dist, dist.data(), dist.size() * sizeof(double));
    if (out_dx_min) *out_dx_min = dmin;
    if (out_dx_avg) *out_dx_avg = davg;
  });
}

mft_status mft_weights_batch(mft_ctx* c, int ngroups, const mft_weight_group* groups,
                             double* max_resid) {
  return guarded(c, [&] {
    set_device(c);
    weights_batch(c, ngroups, groups, max_resid);
  });
}

mft_status mft_weights(mft_ctx* c, int op, int rbf_pow, int polydeg, int deriv_order,
                       double* out_w, double* out_max_resid) {
  return guarded(c, [&] {
    MFT_REQUIRE(c->have_stencils, MFT_ERR_STATE, "no stencils: call mft_knn or mft_set_stencils");
    MFT_REQUIRE(op >= MFT_OP_GRAD && op <= MFT_OP_HV, MFT_ERR_ARG, "bad operator slot");
    MFT_REQUIRE(deriv_order >= 1 && deriv_order <= 8, MFT_ERR_ARG, "deriv_order out of range");
    MFT_REQUIRE(polydeg >= 0 && polydeg <= 6, MFT_ERR_ARG, "polydeg out of range");
    MFT_REQUIRE(rbf_pow >= 1 && rbf_pow <= 15, MFT_ERR_ARG, "rbf_pow out of range");
    set_device(c);
    std::vector<double> w;
    weights_device(c, rbf_pow, polydeg, deriv_order, w, out_max_resid);
    const int64_t nnz = (int64_t)c->st_ci.size();
    const int D = c->dim;
    if (out_w) memcpy(out_w, w.data(), (size_t)nnz * D * sizeof(double));
    if (op == MFT_OP_GRAD) {
      for (int d = 0; d < D; ++d) {
        c->val[d].assign(nnz, 0.0);
        double* vd = c->val[d].data();
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < nnz; ++e) vd[c->st2csr[e]] = w[e * D + d];
        c->have_val[d] = true;
      }
    } else {
      const int slot = op == MFT_OP_LAP ? kSlotLap : kSlotHv;
      c->val[slot].assign(nnz, 0.0);
      for (int64_t e = 0; e < nnz; ++e) {
        double acc = w[e * D];
        for (int d = 1; d < D; ++d) acc = acc + w[e * D + d];  // sum(operators)
        c->val[slot][c->st2csr[e]] = acc;
      }
      c->have_val[slot] = true;
    }
    c->dev_dirty = true;
    c->fsal_valid = false;
  });
}

mft_status mft_load_csc(mft_ctx* c, int op, int comp, int64_t n, const int64_t* colptr,
                        const int64_t* rowval, const double* nzval) {
  return guarded(c, [&] {
    MFT_REQUIRE(c->n > 0 && n == c->n, MFT_ERR_ARG, "operator size differs from the point count");
    MFT_REQUIRE(colptr && rowval && nzval, MFT_ERR_ARG, "NULL CSC arrays");
    MFT_REQUIRE(op >= MFT_OP_GRAD && op <= MFT_OP_HV, MFT_ERR_ARG, "bad operator slot");
    MFT_REQUIRE(op != MFT_OP_GRAD || (comp >= 0 && comp < c->dim), MFT_ERR_ARG, "bad component");
    MFT_REQUIRE(colptr[0] == 1, MFT_ERR_ARG, "colptr must be 1-based (colptr[0] == 1)");
    const int64_t nnz = colptr[n] - 1;
    MFT_REQUIRE(nnz >= 0, MFT_ERR_ARG, "bad colptr");
    for (int64_t j = 0; j < n; ++j)
      MFT_REQUIRE(colptr[j + 1] >= colptr[j], MFT_ERR_ARG, "colptr not monotone");
    for (int64_t p = 0; p < nnz; ++p) {
      MFT_REQUIRE(rowval[p] >= 1 && rowval[p] <= n, MFT_ERR_ARG, "rowval out of range");
    }
    // The first load defines the pattern (CSR with ascending columns + CSC view);
    // later loads must repeat it.
    bool same = c->have_pattern && (int64_t)c->ri.size() == nnz;
    if (same) {
      for (int64_t j = 0; j <= n && same; ++j) same = c->cp[j] == colptr[j] - 1;
      for (int64_t p = 0; p < nnz && same; ++p) same = c->ri[p] == rowval[p] - 1;
    }
    if (!same) {
      bool any = false;
      for (int k = 0; k < kSlots; ++k) any = any || (c->have_pattern && c->have_val[k]);
      MFT_REQUIRE(!any, MFT_ERR_ARG, "operator sparsity pattern differs from the loaded operators");
      c->rp.assign(n + 1, 0);
      for (int64_t p = 0; p < nnz; ++p) c->rp[rowval[p]]++;
      for (int64_t i = 0; i < n; ++i) c->rp[i + 1] += c->rp[i];
      c->ci.assign(nnz, 0);
      std::vector<int64_t> fill(c->rp.begin(), c->rp.end() - 1);
      for (int64_t j = 0; j < n; ++j)
        for (int64_t p = colptr[j] - 1; p < colptr[j + 1] - 1; ++p)
          c->ci[fill[rowval[p] - 1]++] = (int32_t)j;
      for (int64_t i = 0; i < n; ++i)
        for (int64_t e = c->rp[i] + 1; e < c->rp[i + 1]; ++e)
          MFT_REQUIRE(c->ci[e] > c->ci[e - 1], MFT_ERR_ARG, "duplicate entries in CSC");
      finish_pattern(c);
      c->st2csr.clear();
      c->have_stencils = false;
    }
    const int slot = op == MFT_OP_GRAD ? comp : (op == MFT_OP_LAP ? kSlotLap : kSlotHv);
    c->val[slot].assign(nnz, 0.0);
    for (int64_t p = 0; p < nnz; ++p) c->val[slot][c->csc2csr[p]] = nzval[p];
    c->have_val[slot] = true;
    c->dev_dirty = true;
    c->fsal_valid = false;
  });
}

mft_status mft_set_equations(mft_ctx* c, int kind, const double* params) {
  return guarded(c, [&] {
    c->graph_valid = false;
    MFT_REQUIRE(params, MFT_ERR_ARG, "params is NULL");
    MFT_REQUIRE(c->dim == 2 || c->dim == 3, MFT_ERR_UNSUPPORTED,
                "the rhs! engine covers 2D and 3D point clouds");
    if (kind == MFT_EQ_EULER2D) {
      MFT_REQUIRE(c->dim == 2, MFT_ERR_ARG, "CompressibleEulerEquations2D needs a 2D cloud");
      c->eq = kind;
      c->nvars = 4;
      c->gamma = params[0];
    } else if (kind == MFT_EQ_EULER3D) {
      MFT_REQUIRE(c->dim == 3, MFT_ERR_ARG, "CompressibleEulerEquations3D needs a 3D cloud");
      c->eq = kind;
      c->nvars = 5;
      c->gamma = params[0];
    } else if (kind == MFT_EQ_ADVECTION) {
      c->eq = kind;
      c->nvars = 1;
      for (int d = 0; d < c->dim; ++d) c->adv[d] = params[d];
    } else {
      throw mft::Error(MFT_ERR_ARG, "unknown equation kind");
    }
    c->bc_dirty = true;
    c->state_valid = false;
    c->fsal_valid = false;
  });
}

mft_status mft_set_bcs(mft_ctx* c, int n_bc, const int* kinds, const int64_t* ptr,
                       const int32_t* idx, const double* normals) {
  return guarded(c, [&] {
    MFT_REQUIRE(n_bc >= 0, MFT_ERR_ARG, "n_bc < 0");
    MFT_REQUIRE(n_bc == 0 || (kinds && ptr), MFT_ERR_ARG, "NULL bc arrays");
    c->n_bc = n_bc;
    c->bc_kind.assign(kinds, kinds + n_bc);
    c->bc_ptr.assign(ptr, ptr + n_bc + 1);
    const int64_t total = n_bc ? ptr[n_bc] : 0;
    MFT_REQUIRE(n_bc == 0 || ptr[0] == 0, MFT_ERR_ARG, "ptr[0] must be 0");
    c->bc_idx.assign(idx, idx + total);
    for (int64_t p = 0; p < total; ++p)
      MFT_REQUIRE(idx[p] >= 0 && idx[p] < c->n, MFT_ERR_ARG, "boundary index out of range");
    for (int b = 0; b < n_bc; ++b)
      MFT_REQUIRE(kinds[b] >= MFT_BC_DIRICHLET && kinds[b] <= MFT_BC_DO_NOTHING, MFT_ERR_ARG,
                  "unknown boundary-condition kind");
    c->bc_normal.assign(normals ? normals : nullptr, normals ? normals + total * c->dim : nullptr);
    c->dir_values.assign((size_t)total * std::max(c->nvars, 1), 0.0);
    c->bc_dirty = true;
    c->fsal_valid = false;
  });
}

mft_status mft_set_dirichlet_values(mft_ctx* c, const double* values) {
  return guarded(c, [&] {
    MFT_REQUIRE(values, MFT_ERR_ARG, "values is NULL");
    MFT_REQUIRE(c->nvars > 0, MFT_ERR_STATE, "equations not set");
    const int64_t total = c->n_bc ? c->bc_ptr[c->n_bc] : 0;
    c->dir_values.assign(values, values + (size_t)total * c->nvars);
    if (!c->bc_dirty && total > 0)
      MFT_CUDA(cudaMemcpyAsync(c->d_dvals.p, c->dir_values.data(),
                               c->dir_values.size() * sizeof(double), cudaMemcpyHostToDevice,
                               c->stream));
    MFT_CUDA(cudaStreamSynchronize(c->stream));
  });
}

mft_status mft_set_dirichlet_callback(mft_ctx* c, mft_dirichlet_fn fn, void* user) {
  return guarded(c, [&] {
    c->dir_fn = fn;
    c->dir_user = user;
  });
}

mft_status mft_set_sources(mft_ctx* c, int n_src, const int* kinds, const double* params) {
  return guarded(c, [&] {
    c->graph_valid = false;
    MFT_REQUIRE(n_src >= 0 && n_src <= 8, MFT_ERR_ARG, "n_src out of range");
    MFT_REQUIRE(n_src == 0 || (kinds && params), MFT_ERR_ARG, "NULL source arrays");
    for (int k = 0; k < n_src; ++k) {
      MFT_REQUIRE(kinds[k] >= MFT_SRC_RV && kinds[k] <= MFT_SRC_IGR, MFT_ERR_ARG,
                  "unknown source kind");
      if (kinds[k] == MFT_SRC_IGR)
        MFT_REQUIRE(params[4 * k + 1] >= 0 && params[4 * k + 1] <= 1000 &&
                        isfinite(params[4 * k]), MFT_ERR_ARG,
                    "IGR parameters: finite alpha and 0..1000 CG iterations");
    }
    c->src_kind.assign(kinds, kinds + n_src);
    c->src_par.assign(params, params + 4 * n_src);
    c->fsal_valid = false;
  });
}

mft_status mft_set_option(mft_ctx* c, int option, int value) {
  return guarded(c, [&] {
    c->graph_valid = false;
    if (option == MFT_OPT_GATHER) {
      MFT_REQUIRE(value >= MFT_GATHER_AUTO && value <= MFT_GATHER_HALO, MFT_ERR_ARG,
                  "unknown gather mapping");
      c->gather_mode = value;
      c->fsal_valid = false;
      for (int& k : c->tuned_fwd) k = -1;
      for (int& k : c->tuned_rev) k = -1;
    } else if (option == MFT_OPT_DW_VARIANT) {
      MFT_REQUIRE(value >= -1 && value < kDwVariants, MFT_ERR_ARG,
                  "double-word gather variant: -1 (tuned) or 0..5");
      c->dw_variant = value;
      c->fsal_valid = false;
    } else if (option == MFT_OPT_HALO_ROWS) {
      MFT_REQUIRE(value == 0 || value == 128 || value == 256, MFT_ERR_ARG,
                  "halo rows: 0 (automatic), 128 or 256");
      c->halo_rows_opt = value;
      c->fsal_valid = false;
    } else if (option == MFT_OPT_FUSE_FLUX) {
      MFT_REQUIRE(value == 0 || value == 1, MFT_ERR_ARG, "fuse flux: 0 or 1");
      c->fuse_flux = value;
      c->fsal_valid = false;
      for (int& k : c->tuned_fwd_dw) k = -1;  // the tuner times the flux kernel by it
    } else if (option == MFT_OPT_ENTRY_ORDER) {
      MFT_REQUIRE(value == 0 || value == 1, MFT_ERR_ARG,
                  "entry order: 0 structure order, 1 bank-spreading");
      c->entry_order = value;
      c->fsal_valid = false;
    } else if (option == MFT_OPT_LAYOUT_ORDER) {
      MFT_REQUIRE(value == 0 || value == 1, MFT_ERR_ARG, "layout order: 0 node order, 1 Morton");
      c->layout_order = value;
      c->fsal_valid = false;
    } else if (option == MFT_OPT_FP64_ARITH) {
      MFT_REQUIRE(value >= MFT_ARITH_AUTO && value <= MFT_ARITH_DW, MFT_ERR_ARG,
                  "unknown FP64 arithmetic");
      c->fp64_arith = value;
      c->fsal_valid = false;
    } else {
      throw mft::Error(MFT_ERR_ARG, "unknown option");
    }
  });
}

mft_status mft_selftest_bounded_wait(mft_ctx* c, int polls) {
  return guarded(c, [&] {
    MFT_REQUIRE(polls >= 1 && polls <= 1000000, MFT_ERR_ARG, "polls must be 1 .. 1000000");
    set_device(c);
    if (!c->kerr.p) {
      c->kerr.alloc(1);
      c->kerr.zero(c->stream);
    }
    launch_wait_selftest(c->kerr.p, (unsigned)polls, c->stream);
    check_kernel_errors(c);
  });
}

mft_status mft_get_option(mft_ctx* c, int option, int* value) {
  return guarded(c, [&] {
    MFT_REQUIRE(value, MFT_ERR_ARG, "value is NULL");
    if (option == MFT_OPT_GATHER) *value = c->gather_mode;
    else if (option == MFT_OPT_TUNED_FWD) *value = c->last_fwd_choice;
    else if (option == MFT_OPT_TUNED_REV) *value = c->last_rev_choice;
    else if (option == MFT_OPT_FP64_ARITH) *value = c->fp64_arith;
    else if (option == MFT_OPT_LAYOUT_ORDER) *value = c->layout_order;
    else if (option == MFT_OPT_DW_VARIANT) *value = c->dw_variant;
    else if (option == MFT_OPT_HALO_STAGED_FWD) *value = (int)c->fwd.halo_staged;
    else if (option == MFT_OPT_HALO_STAGED_REV) *value = (int)c->rev.halo_staged;
    else if (option == MFT_OPT_HALO_GROUPS) *value = (int)c->fwd.halo_groups;
    else if (option == MFT_OPT_ADJ_EVERY) *value = c->adj_every;
    else if (option == MFT_OPT_HALO_ROWS) *value = c->fwd.halo_rows;
    else if (option == MFT_OPT_ENTRY_ORDER) *value = c->entry_order;
    else if (option == MFT_OPT_FUSE_FLUX) *value = c->fuse_flux;
    else if (option == MFT_OPT_FLUX_FUSED) *value = c->last_flux_fused;
    else if (option == MFT_OPT_BANK_FWD) *value = c->fwd.bank_milli;
    else if (option == MFT_OPT_BANK_REV) *value = c->rev.bank_milli;
    else if (option == MFT_OPT_IGR_ITERS) {
      // CG iterations of the last IGR solve (-1: none yet)
      *value = -1;
      if (c->igr_sc.p) {
        set_device(c);
        IgrScalars sc{};
        MFT_CUDA(cudaStreamSynchronize(c->stream));
        MFT_CUDA(cudaMemcpy(&sc, c->igr_sc.p, sizeof(sc), cudaMemcpyDeviceToHost));
        *value = sc.iter;
      }
    }
    else throw mft::Error(MFT_ERR_ARG, "unknown option");
  });
}

mft_status mft_set_segments(mft_ctx* c, int nseg, const int64_t* offsets, const double* h) {
  return guarded(c, [&] {
    c->graph_valid = false;
    MFT_REQUIRE(c->n > 0, MFT_ERR_STATE, "call mft_set_points first");
    MFT_REQUIRE(nseg >= 0 && nseg <= 1 << 20, MFT_ERR_ARG, "nseg out of range");
    set_device(c);
    c->fsal_valid = false;
    // the spatial row order keeps members contiguous, so it follows the segments
    if (c->layout_order == 1 && (nseg > 0 || c->nseg > 0)) c->dev_dirty = true;
    if (nseg == 0) {
      c->nseg = 0;
      return;
    }
    MFT_REQUIRE(offsets && h, MFT_ERR_ARG, "NULL segment arrays");
    MFT_REQUIRE(offsets[0] == 0 && offsets[nseg] == c->n, MFT_ERR_ARG,
                "segment offsets must start at 0 and end at n");
    for (int m = 0; m < nseg; ++m)
      MFT_REQUIRE(offsets[m + 1] > offsets[m], MFT_ERR_ARG, "empty or unordered segment");
    std::vector<int> sid(c->n);
    for (int m = 0; m < nseg; ++m)
      for (int64_t i = offsets[m]; i < offsets[m + 1]; ++i) sid[i] = m;
    if (c->have_pattern)
      for (int64_t i = 0; i < c->n; ++i)
        for (int64_t e = c->rp[i]; e < c->rp[i + 1]; ++e)
          MFT_REQUIRE(sid[c->ci[e]] == sid[i], MFT_ERR_ARG,
                      "the stencil of node " + std::to_string(i) + " leaves its segment");
    c->nseg = nseg;
    c->seg_off.assign(offsets, offsets + nseg + 1);
    cudaStream_t s = c->stream;
    c->d_seg_off.upload(c->seg_off, s);
    c->d_seg_id.upload(sid, s);
    c->d_seg_h.upload(h, nseg, s);
    c->seg_partial.alloc((size_t)nseg * kSegBlocks * 8);
    c->seg_counter.alloc((size_t)2 * nseg);
    c->seg_counter.zero(s);
    c->seg_mean.alloc((size_t)nseg * 8);
    c->seg_norms.alloc((size_t)nseg * 8);
    MFT_CUDA(cudaStreamSynchronize(s));
  });
}

mft_status mft_set_precision(mft_ctx* c, int precision) {
  return guarded(c, [&] {
    c->graph_valid = false;
    MFT_REQUIRE(precision == MFT_PREC_FP64 || precision == MFT_PREC_FP32, MFT_ERR_ARG,
                "unknown precision");
    c->precision = precision;
    c->fsal_valid = false;
  });
}

mft_status mft_rhs_device(mft_ctx* c, double* du, double* u, double t) {
  return guarded(c, [&] {
    check_state_ready(c);
    MFT_REQUIRE(du && u, MFT_ERR_ARG, "NULL device pointers");
    set_device(c);
    ensure_work(c);
    const int64_t n = c->n;
    const int V = c->nvars;
    cudaStream_t s = c->stream;
    launch_aos_from_soa(u, c->work_u.p, n, V, s);
    float* u32 = nullptr;
    if (c->precision == MFT_PREC_FP32) {
      launch_aos_to_f32(c->work_u.p, c->work_u32.p, n * V, s);
      u32 = c->work_u32.p;
    }
    Epilogue ep{};
    ep.kind = kOutDu;
    ep.out = c->work_du.p;
    eval_rhs(c, c->work_u.p, u32, t, ep);
    launch_soa_from_aos(c->work_du.p, du, n, V, s);
    launch_soa_from_aos(c->work_u.p, u, n, V, s);
    check_kernel_errors(c);
  });
}

mft_status mft_rhs(mft_ctx* c, double* const* du, double* const* u, int nvars, double t) {
  return guarded(c, [&] {
    check_state_ready(c);
    MFT_REQUIRE(du && u && nvars == c->nvars, MFT_ERR_ARG, "bad state arrays or nvars");
    set_device(c);
    ensure_work(c);
    const int64_t n = c->n;
    const int V = c->nvars;
    cudaStream_t s = c->stream;
    for (int v = 0; v < V; ++v)
      MFT_CUDA(cudaMemcpyAsync(c->soa.p + (size_t)v * n, u[v], n * sizeof(double),
                               cudaMemcpyHostToDevice, s));
    launch_aos_from_soa(c->soa.p, c->work_u.p, n, V, s);
    float* u32 = nullptr;
    if (c->precision == MFT_PREC_FP32) {
      launch_aos_to_f32(c->work_u.p, c->work_u32.p, n * V, s);
      u32 = c->work_u32.p;
    }
    Epilogue ep{};
    ep.kind = kOutDu;
    ep.out = c->work_du.p;
    eval_rhs(c, c->work_u.p, u32, t, ep);
    launch_soa_from_aos(c->work_du.p, c->soa.p, n, V, s);
    launch_soa_from_aos(c->work_u.p, c->soa2.p, n, V, s);
    for (int v = 0; v < V; ++v) {
      MFT_CUDA(cudaMemcpyAsync(du[v], c->soa.p + (size_t)v * n, n * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
      MFT_CUDA(cudaMemcpyAsync(u[v], c->soa2.p + (size_t)v * n, n * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    }
    check_kernel_errors(c);
  });
}

mft_status mft_set_state(mft_ctx* c, const double* const* u, int nvars, double t) {
  return guarded(c, [&] {
    check_state_ready(c);
    MFT_REQUIRE(u && nvars == c->nvars, MFT_ERR_ARG, "bad state arrays or nvars");
    set_device(c);
    ensure_work(c);
    const int64_t n = c->n;
    cudaStream_t s = c->stream;
    for (int v = 0; v < nvars; ++v)
      MFT_CUDA(cudaMemcpyAsync(c->soa.p + (size_t)v * n, u[v], n * sizeof(double),
                               cudaMemcpyHostToDevice, s));
    launch_aos_from_soa(c->soa.p, c->U[0].p, n, nvars, s);
    MFT_CUDA(cudaStreamSynchronize(s));
    c->t_state = t;
    c->state_valid = true;
    c->fsal_valid = false;
    c->origin_valid = false;
  });
}

mft_status mft_get_state(mft_ctx* c, double* const* u, int nvars, double* t) {
  return guarded(c, [&] {
    MFT_REQUIRE(c->state_valid, MFT_ERR_STATE, "no device state");
    MFT_REQUIRE(u && nvars == c->nvars, MFT_ERR_ARG, "bad state arrays or nvars");
    set_device(c);
    const int64_t n = c->n;
    cudaStream_t s = c->stream;
    launch_soa_from_aos(c->U[0].p, c->soa.p, n, nvars, s);
    for (int v = 0; v < nvars; ++v)
      MFT_CUDA(cudaMemcpyAsync(u[v], c->soa.p + (size_t)v * n, n * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    MFT_CUDA(cudaStreamSynchronize(s));
    if (t) *t = c->t_state;
  });
}

namespace {

// Ring of approx_order + 1 zeroed states (approx_order -1 releases the ring).
void history_setup(mft_ctx* c, int approx_order) {
  c->graph_valid = false;
  c->hist_order = approx_order;
  c->hist_t.assign(approx_order + 1, 0.0);
  const size_t nv = (size_t)c->n * c->nvars;
  for (int k = 0; k < 8; ++k) {
    if (k <= approx_order) {
      c->hist[k].alloc(nv);
      c->hist[k].zero(c->stream);
    } else {
      c->hist[k].release();
    }
  }
  c->hist_w.alloc(16);
  c->hist_head = 0;
  c->success_iter = 0;
  c->fsal_valid = false;
  MFT_CUDA(cudaStreamSynchronize(c->stream));
}

}  // namespace

mft_status mft_history_init(mft_ctx* c, int approx_order) {
  return guarded(c, [&] {
    check_state_ready(c);
    MFT_REQUIRE(approx_order >= 0 && approx_order <= 7, MFT_ERR_ARG, "approx_order out of range");
    set_device(c);
    history_setup(c, approx_order);
  });
}

namespace {

float* shadow(mft_ctx* c, int k) {
  return c->precision == MFT_PREC_FP32 ? c->U32[k].p : nullptr;
}

// Stage limiter: one Zhang-Shu pass per configured variable on stage state u.
void apply_limiter(mft_ctx* c, double* u, float* u32) {
  if (c->lim_n == 0) return;
  MFT_REQUIRE(c->eq == MFT_EQ_EULER2D && c->nvars == 4, MFT_ERR_UNSUPPORTED,
              "the positivity limiter needs the 2D Euler equations");
  c->lim_buf.alloc((size_t)c->n * 4);
  for (int q = 0; q < c->lim_n; ++q) {
    NvtxRange rng("positivity limiter");
    ProfScope ps(c, MFT_K_LIMITER);
    launch_zs_limiter(c->n, c->fwd.view(), c->lim_var[q], c->lim_thr[q], c->gamma, u, u32,
                      c->lim_buf.p, c->stream);
  }
}

// FSAL evaluation at the current state: k0 = f(u_n), stage 1 = u_n + dt*k0.
void fsal_eval(mft_ctx* c, double dt) {
  if (c->fsal_valid && c->fsal_dt == dt) return;
  const int64_t n = c->n;
  const int V = c->nvars;
  if (c->precision == MFT_PREC_FP32) launch_aos_to_f32(c->U[0].p, c->U32[0].p, n * V, c->stream);
  Epilogue ep{};
  ep.kind = kStage1;
  ep.dt = dt;
  ep.out = c->U[1].p;
  ep.out32 = shadow(c, 1);
  eval_rhs(c, c->U[0].p, shadow(c, 0), c->t_state, ep);
  apply_limiter(c, c->U[1].p, shadow(c, 1));
  if (c->hist_order >= 0 && c->success_iter == 0) history_push(c, c->t_state, c->U[0].p, 0);
  c->fsal_valid = true;
  c->fsal_dt = dt;
}

// Stages 2, 3 and the next step's first stage from u_n in buffer `un` (stage-3 state
// into `u3`); `t` is the step start time.
void enqueue_step(mft_ctx* c, double dt, double t, int iu_n, int iu_3) {
  Epilogue e2{};
  e2.kind = kStage2;
  e2.dt = dt;
  e2.u_n = c->U[iu_n].p;
  e2.out = c->U[2].p;
  e2.out32 = shadow(c, 2);
  eval_rhs(c, c->U[1].p, shadow(c, 1), t + dt, e2);
  apply_limiter(c, c->U[2].p, shadow(c, 2));
  Epilogue e3{};
  e3.kind = kStage3;
  e3.dt = dt;
  e3.u_n = c->U[iu_n].p;
  e3.out = c->U[iu_3].p;
  e3.out32 = shadow(c, iu_3);
  eval_rhs(c, c->U[2].p, shadow(c, 2), t + 0.5 * dt, e3);
  apply_limiter(c, c->U[iu_3].p, shadow(c, iu_3));
  Epilogue e1{};
  e1.kind = kStage1;
  e1.dt = dt;
  e1.out = c->U[1].p;
  e1.out32 = shadow(c, 1);
  eval_rhs(c, c->U[iu_3].p, shadow(c, iu_3), t + dt, e1);
  apply_limiter(c, c->U[1].p, shadow(c, 1));
}

// Step times are formed as t_origin + k dt, k counted from the first step of size dt
// after the state was set (or dt changed), as OrdinaryDiffEq's fixed-step loop forms
// them; so a run split over several calls, or resumed from a checkpoint, takes the same
// times bit for bit as one call.
void sync_origin(mft_ctx* c, double dt) {
  if (!c->origin_valid || c->origin_dt != dt ||
      c->t_state != c->t_origin + (double)c->origin_steps * dt) {
    c->origin_valid = true;
    c->t_origin = c->t_state;
    c->origin_dt = dt;
    c->origin_steps = 0;
  }
}

double step_time(const mft_ctx* c, double dt, int64_t k) {
  return c->t_origin + (double)(c->origin_steps + k) * dt;
}

void ssprk33_direct(mft_ctx* c, double dt, int nsteps) {
  sync_origin(c, dt);
  for (int k = 0; k < nsteps; ++k) {
    enqueue_step(c, dt, step_time(c, dt, k), 0, 3);
    const double tn = step_time(c, dt, k + 1);
    std::swap(c->U[0].p, c->U[3].p);
    std::swap(c->U32[0].p, c->U32[3].p);
    c->t_state = tn;
    if (c->hist_order >= 0) history_push(c, tn, c->U[0].p, c->success_iter + 1);
  }
  c->origin_steps += nsteps;
}

// One SSP-RK3 step captured as a CUDA graph, once with u_n in U0 and once with u_n in
// U3 (the buffers swap roles every step).  Per-step values (history weights, the ring
// slot, success_iter) come from the step table at the device step counter.
void capture_step_graphs(mft_ctx* c, double dt) {
  for (int g = 0; g < 2; ++g) {
    if (c->gexec[g]) cudaGraphExecDestroy(c->gexec[g]);
    c->gexec[g] = nullptr;
  }
  c->graph_valid = false;
  const int slots = c->hist_order + 1;
  for (int g = 0; g < 2; ++g) {
    const int iu_n = g == 0 ? 0 : 3, iu_3 = g == 0 ? 3 : 0;
    MFT_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    c->capturing = true;
    try {
      enqueue_step(c, dt, 0.0, iu_n, iu_3);
      if (c->hist_order >= 0) {
        const double* ring[8];
        for (int k = 0; k < slots; ++k) ring[k] = c->hist[k].p;
        launch_history_dev((int64_t)c->n * c->nvars, c->U[iu_3].p, ring, slots, c->d_tab.p,
                           c->d_ctr.p, c->approx_du.p, c->precision == MFT_PREC_FP32,
                           c->stream);
      }
      launch_step_advance(c->d_ctr.p, c->stream);
    } catch (...) {
      c->capturing = false;
      cudaGraph_t junk = nullptr;
      cudaStreamEndCapture(c->stream, &junk);
      if (junk) cudaGraphDestroy(junk);
      throw;
    }
    c->capturing = false;
    cudaGraph_t graph = nullptr;
    MFT_CUDA(cudaStreamEndCapture(c->stream, &graph));
    const cudaError_t e = cudaGraphInstantiate(&c->gexec[g], graph, 0);
    cudaGraphDestroy(graph);
    MFT_CUDA(e);
    c->graph_un[g] = c->U[iu_n].p;
  }
  c->graph_dt = dt;
  c->graph_valid = true;
}

void ssprk33_graph(mft_ctx* c, double dt, int nsteps) {
  const int slots = c->hist_order + 1;
  // host-side bookkeeping of the HistoryCallback for the whole batch
  std::vector<StepParams> tab(nsteps);
  sync_origin(c, dt);
  for (int k = 0; k < nsteps; ++k) {
    StepParams& sp = tab[k];
    memset(&sp, 0, sizeof(sp));
    sp.si_eps = c->success_iter;
    if (c->hist_order >= 0) {
      const double tn = step_time(c, dt, k + 1);
      for (int q = slots - 1; q > 0; --q) c->hist_t[q] = c->hist_t[q - 1];
      c->hist_t[0] = tn;
      c->hist_head = (c->hist_head + slots - 1) % slots;
      sp.head = c->hist_head;
      const int push_si = c->success_iter + 1;
      const int m = std::min(push_si + 1, slots);
      double w[16];
      MFT_REQUIRE(time_deriv_weights(m, c->hist_t.data(), w) == 0, MFT_ERR_SINGULAR,
                  "time_deriv_weights: singular Vandermonde system");
      for (int q = 0; q < m; ++q) sp.w[q] = w[q];
      sp.m = m;
      c->success_iter = push_si;
    }
  }
  if (c->d_tab.n < (size_t)nsteps) {
    c->d_tab.alloc(std::max<size_t>(nsteps, 64));
    c->graph_valid = false;
  }
  if (!c->d_ctr.p) c->d_ctr.alloc(1);
  // stage the table in pinned memory; the previous batch's copy must have left it
  if (c->h_tab_n < (size_t)nsteps) {
    if (c->h_tab) {
      MFT_CUDA(cudaEventSynchronize(c->ev_tab));
      cudaFreeHost(c->h_tab);
      c->h_tab = nullptr;
      c->h_tab_n = 0;
    }
    const size_t cap = std::max<size_t>(nsteps, 64);
    MFT_CUDA(cudaMallocHost(reinterpret_cast<void**>(&c->h_tab), cap * sizeof(StepParams)));
    c->h_tab_n = cap;
  } else {
    MFT_CUDA(cudaEventSynchronize(c->ev_tab));
  }
  memcpy(c->h_tab, tab.data(), nsteps * sizeof(StepParams));
  MFT_CUDA(cudaMemcpyAsync(c->d_tab.p, c->h_tab, nsteps * sizeof(StepParams),
                           cudaMemcpyHostToDevice, c->stream));
  MFT_CUDA(cudaEventRecord(c->ev_tab, c->stream));
  c->d_ctr.zero(c->stream);
  if (!c->graph_valid || c->graph_dt != dt ||
      (c->U[0].p != c->graph_un[0] && c->U[0].p != c->graph_un[1]))
    capture_step_graphs(c, dt);
  const int first = c->U[0].p == c->graph_un[0] ? 0 : 1;
  for (int k = 0; k < nsteps; ++k) MFT_CUDA(cudaGraphLaunch(c->gexec[(first + k) & 1], c->stream));
  if (nsteps & 1) {
    std::swap(c->U[0].p, c->U[3].p);
    std::swap(c->U32[0].p, c->U32[3].p);
  }
  c->t_state = step_time(c, dt, nsteps);
  c->origin_steps += nsteps;
}

void ssprk33_run(mft_ctx* c, double dt, int nsteps, bool use_graph = false) {
  ensure_work(c);
  fsal_eval(c, dt);
  if (use_graph && nsteps > 0 && !c->dir_fn && !c->prof_on) ssprk33_graph(c, dt, nsteps);
  else ssprk33_direct(c, dt, nsteps);
}

}  // namespace

mft_status mft_ssprk33(mft_ctx* c, double dt, int nsteps, int use_graph) {
  return guarded(c, [&] {
    MFT_REQUIRE(c->state_valid, MFT_ERR_STATE, "call mft_set_state first");
    MFT_REQUIRE(nsteps >= 0, MFT_ERR_ARG, "nsteps < 0");
    MFT_REQUIRE(dt > 0 && isfinite(dt), MFT_ERR_ARG, "dt must be positive and finite");
    set_device(c);
    ssprk33_run(c, dt, nsteps, use_graph != 0);
    check_kernel_errors(c);
  });
}

mft_status mft_ssprk33_host(mft_ctx* c, double* const* u, int nvars, double* t, double dt,
                            int nsteps) {
  return guarded(c, [&] {
    check_state_ready(c);
    MFT_REQUIRE(u && t && nvars == c->nvars, MFT_ERR_ARG, "bad state arrays");
    MFT_REQUIRE(dt > 0 && isfinite(dt), MFT_ERR_ARG, "dt must be positive and finite");
    set_device(c);
    ensure_work(c);
    const int64_t n = c->n;
    cudaStream_t s = c->stream;
    // Pinned caller arrays mapped for the device are read and written in place by the
    // layout kernels (one pass over C2C); other host memory goes through staging copies.
    VarPtrs vp{};
    bool direct = nvars <= 8;
    for (int v = 0; v < nvars && direct; ++v) {
      cudaPointerAttributes at{};
      if (cudaPointerGetAttributes(&at, u[v]) != cudaSuccess) {
        cudaGetLastError();
        direct = false;
      } else if (at.type != cudaMemoryTypeHost || !at.devicePointer) {
        direct = false;
      } else {
        vp.p[v] = static_cast<double*>(at.devicePointer);
      }
    }
    if (!direct)
      for (int v = 0; v < nvars; ++v)
        MFT_CUDA(cudaMemcpyAsync(c->soa.p + (size_t)v * n, u[v], n * sizeof(double),
                                 cudaMemcpyHostToDevice, s));
    auto upload_to = [&](double* aos) {
      if (direct) launch_aos_from_vars(vp, aos, n, nvars, s);
      else launch_aos_from_soa(c->soa.p, aos, n, nvars, s);
    };
    // The pending first stage (FSAL) stays valid only if the caller hands back
    // exactly the state this context holds at the same time.
    bool keep = c->state_valid && c->fsal_valid && c->t_state == *t;
    if (keep) {
      upload_to(c->work_u.p);
      c->flag.alloc(1);
      c->flag.zero(s);
      launch_differs(c->work_u.p, c->U[0].p, n * nvars, c->flag.p, s);
      int differs = 1;
      MFT_CUDA(cudaMemcpyAsync(&differs, c->flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      MFT_CUDA(cudaStreamSynchronize(s));
      if (differs) {
        std::swap(c->work_u.p, c->U[0].p);
        keep = false;
      }
    } else {
      upload_to(c->U[0].p);
    }
    c->t_state = *t;
    c->state_valid = true;
    if (!keep) c->fsal_valid = false;
    ssprk33_run(c, dt, nsteps, true);
    if (direct) {
      launch_vars_from_aos(c->U[0].p, vp, n, nvars, s);
    } else {
      launch_soa_from_aos(c->U[0].p, c->soa.p, n, nvars, s);
      for (int v = 0; v < nvars; ++v)
        MFT_CUDA(cudaMemcpyAsync(u[v], c->soa.p + (size_t)v * n, n * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
    }
    check_kernel_errors(c);
    *t = c->t_state;
  });
}

mft_status mft_set_rv_state(mft_ctx* c, const double* const* approx_du, int nvars,
                            int success_iter) {
  return guarded(c, [&] {
    check_state_ready(c);
    MFT_REQUIRE(nvars == c->nvars, MFT_ERR_ARG, "nvars differs from the equations");
    MFT_REQUIRE(success_iter >= 0, MFT_ERR_ARG, "success_iter < 0");
    set_device(c);
    ensure_work(c);
    const int64_t n = c->n;
    cudaStream_t s = c->stream;
    if (approx_du) {
      for (int v = 0; v < nvars; ++v)
        MFT_CUDA(cudaMemcpyAsync(c->soa.p + (size_t)v * n, approx_du[v], n * sizeof(double),
                                 cudaMemcpyHostToDevice, s));
      launch_aos_from_soa(c->soa.p, c->approx_du.p, n, nvars, s);
    }
    c->success_iter = success_iter;
    c->fsal_valid = false;
    MFT_CUDA(cudaStreamSynchronize(s));
  });
}

// ---------------------------------------------------------------- checkpoint / resume

namespace {

// Image layout (host byte order; both supported hosts are little-endian):
//   CkptHeader, u_n (n x nvars node-major FP64), the pending first stage when fsal = 1
//   (u_n + dt f(u_n), same shape), the history ring newest first (hist_order + 1
//   states), approx_du, then the FNV-1a 64-bit hash of everything before it.
struct CkptHeader {
  char magic[8];
  uint32_t version;
  uint32_t header_bytes;
  int64_t n;
  int32_t nvars;
  int32_t hist_order;  // -1: no HistoryCallback
  int32_t success_iter;
  int32_t fsal;
  int32_t form;  // precision * 4 + (double-word gathers): the form the pending stage came from
  int32_t reserved;
  double t;
  double fsal_dt;
  double t_origin, origin_dt;
  int64_t origin_steps;
  int32_t origin_valid;
  int32_t reserved2;
  double hist_t[8];
};
static_assert(sizeof(CkptHeader) == 160, "checkpoint header layout");
constexpr char kCkptMagic[8] = {'M', 'F', 'T', 'C', 'K', 'P', 'T', '\0'};
constexpr uint32_t kCkptVersion = 1;

uint64_t fnv1a64(const unsigned char* p, size_t n) {
  uint64_t h = 14695981039346656037ull;
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

int ckpt_form(const mft_ctx* c) { return c->precision * 4 + (use_dw(c) || use_dw3(c) ? 1 : 0); }

size_t ckpt_bytes(const mft_ctx* c) {
  const size_t nvb = (size_t)c->n * c->nvars * sizeof(double);
  const size_t slots = c->hist_order >= 0 ? (size_t)c->hist_order + 1 : 0;
  return sizeof(CkptHeader) + nvb * (1 + (c->fsal_valid ? 1 : 0) + slots + 1) + 8;
}

}  // namespace

mft_status mft_checkpoint_size(mft_ctx* c, size_t* bytes) {
  return guarded(c, [&] {
    MFT_REQUIRE(bytes, MFT_ERR_ARG, "NULL size pointer");
    MFT_REQUIRE(c->state_valid, MFT_ERR_STATE, "no device state to checkpoint");
    *bytes = ckpt_bytes(c);
  });
}

mft_status mft_checkpoint_save(mft_ctx* c, void* buf, size_t bytes) {
  return guarded(c, [&] {
    MFT_REQUIRE(c->state_valid, MFT_ERR_STATE, "no device state to checkpoint");
    MFT_REQUIRE(buf, MFT_ERR_ARG, "NULL checkpoint buffer");
    const size_t need = ckpt_bytes(c);
    MFT_REQUIRE(bytes >= need, MFT_ERR_ARG,
                "checkpoint buffer too small: " + std::to_string(need) + " bytes needed");
    set_device(c);
    cudaStream_t s = c->stream;
    unsigned char* out = static_cast<unsigned char*>(buf);
    CkptHeader h{};
    memcpy(h.magic, kCkptMagic, 8);
    h.version = kCkptVersion;
    h.header_bytes = sizeof(CkptHeader);
    h.n = c->n;
    h.nvars = c->nvars;
    h.hist_order = c->hist_order;
    h.success_iter = c->success_iter;
    h.fsal = c->fsal_valid ? 1 : 0;
    h.form = ckpt_form(c);
    h.t = c->t_state;
    h.fsal_dt = c->fsal_dt;
    h.t_origin = c->t_origin;
    h.origin_dt = c->origin_dt;
    h.origin_steps = c->origin_steps;
    h.origin_valid = c->origin_valid ? 1 : 0;
    const int slots = c->hist_order + 1;
    for (int k = 0; k < slots && k < 8; ++k) h.hist_t[k] = c->hist_t[k];
    memcpy(out, &h, sizeof(h));
    size_t off = sizeof(h);
    const size_t nvb = (size_t)c->n * c->nvars * sizeof(double);
    auto d2h = [&](const double* src) {
      MFT_CUDA(cudaMemcpyAsync(out + off, src, nvb, cudaMemcpyDeviceToHost, s));
      off += nvb;
    };
    d2h(c->U[0].p);
    if (c->fsal_valid) d2h(c->U[1].p);
    for (int k = 0; k < slots; ++k) d2h(c->hist[(c->hist_head + k) % slots].p);
    d2h(c->approx_du.p);
    MFT_CUDA(cudaStreamSynchronize(s));
    const uint64_t hash = fnv1a64(out, off);
    memcpy(out + off, &hash, 8);
  });
}

mft_status mft_checkpoint_load(mft_ctx* c, const void* buf, size_t bytes) {
  return guarded(c, [&] {
    check_state_ready(c);
    MFT_REQUIRE(buf, MFT_ERR_ARG, "NULL checkpoint buffer");
    MFT_REQUIRE(bytes >= sizeof(CkptHeader) + 8, MFT_ERR_ARG, "checkpoint image truncated");
    const unsigned char* in = static_cast<const unsigned char*>(buf);
    CkptHeader h;
    memcpy(&h, in, sizeof(h));
    MFT_REQUIRE(memcmp(h.magic, kCkptMagic, 8) == 0, MFT_ERR_ARG, "not a checkpoint image");
    MFT_REQUIRE(h.version == kCkptVersion && h.header_bytes == sizeof(CkptHeader), MFT_ERR_ARG,
                "unsupported checkpoint version");
    MFT_REQUIRE(h.n == c->n && h.nvars == c->nvars, MFT_ERR_ARG,
                "checkpoint of another problem size (n " + std::to_string(h.n) + ", nvars " +
                    std::to_string(h.nvars) + ")");
    MFT_REQUIRE(h.hist_order >= -1 && h.hist_order <= 7 && h.success_iter >= 0 &&
                    (h.fsal == 0 || h.fsal == 1),
                MFT_ERR_ARG, "corrupt checkpoint header");
    const size_t nvb = (size_t)c->n * c->nvars * sizeof(double);
    const int slots = h.hist_order + 1;
    const size_t need = sizeof(CkptHeader) + nvb * (1 + h.fsal + slots + 1) + 8;
    MFT_REQUIRE(bytes == need, MFT_ERR_ARG,
                "checkpoint image is " + std::to_string(bytes) + " bytes, expected " +
                    std::to_string(need));
    uint64_t hash = 0;
    memcpy(&hash, in + need - 8, 8);
    MFT_REQUIRE(hash == fnv1a64(in, need - 8), MFT_ERR_ARG, "checkpoint checksum mismatch");
    set_device(c);
    ensure_work(c);
    if (h.hist_order != c->hist_order) history_setup(c, h.hist_order);
    cudaStream_t s = c->stream;
    size_t off = sizeof(h);
    auto h2d = [&](double* dst) {
      MFT_CUDA(cudaMemcpyAsync(dst, in + off, nvb, cudaMemcpyHostToDevice, s));
      off += nvb;
    };
    h2d(c->U[0].p);
    // the pending first stage is kept only for the form that computed it
    const bool fsal = h.fsal == 1 && h.form == ckpt_form(c);
    if (h.fsal == 1) {
      if (fsal) h2d(c->U[1].p);
      else off += nvb;
    }
    for (int k = 0; k < slots; ++k) h2d(c->hist[k].p);
    h2d(c->approx_du.p);
    const int64_t nv = c->n * c->nvars;
    if (c->precision == MFT_PREC_FP32) {
      launch_aos_to_f32(c->U[0].p, c->U32[0].p, nv, s);
      if (fsal) launch_aos_to_f32(c->U[1].p, c->U32[1].p, nv, s);
    }
    MFT_CUDA(cudaStreamSynchronize(s));
    c->hist_head = 0;
    for (int k = 0; k < slots; ++k) c->hist_t[k] = h.hist_t[k];
    c->success_iter = h.success_iter;
    c->t_state = h.t;
    c->state_valid = true;
    c->fsal_valid = fsal;
    c->fsal_dt = h.fsal_dt;
    c->origin_valid = h.origin_valid != 0;
    c->t_origin = h.t_origin;
    c->origin_dt = h.origin_dt;
    c->origin_steps = h.origin_steps;
    c->graph_valid = false;
    if (fsal) {
      // With the pending stage kept, the next step starts without a direct rhs!: one
      // rhs! on a copy of u_n builds the device layouts and times the gather variants
      // now, outside the first step's graph capture (its outputs are scratch).
      MFT_CUDA(cudaMemcpyAsync(c->work_u.p, c->U[0].p, nvb, cudaMemcpyDeviceToDevice, s));
      float* w32 = nullptr;
      if (c->precision == MFT_PREC_FP32) {
        launch_aos_to_f32(c->work_u.p, c->work_u32.p, nv, s);
        w32 = c->work_u32.p;
      }
      Epilogue ep{};
      ep.kind = kStage1;
      ep.dt = c->fsal_dt;
      ep.out = c->U[2].p;
      ep.out32 = shadow(c, 2);
      eval_rhs(c, c->work_u.p, w32, c->t_state, ep);
      MFT_CUDA(cudaStreamSynchronize(s));
      check_kernel_errors(c);
    }
  });
}

mft_status mft_profile(mft_ctx* c, int enable) {
  return guarded(c, [&] {
    set_device(c);
    prof_drain(c);
    for (int k = 0; k < MFT_K_COUNT; ++k) {
      c->prof_ms[k] = 0.0;
      c->prof_n[k] = 0;
    }
    c->prof_on = enable != 0;
  });
}

mft_status mft_profile_get(mft_ctx* c, int kind, double* total_ms, int64_t* launches,
                           const char** name) {
  static const char* names[MFT_K_COUNT] = {"bc_pass1", "flux", "fwd_gather", "mean",
                                           "lexmax", "eps", "rev_gather", "rev_lap",
                                           "history", "layout", "adjoint", "limiter", "igr"};
  return guarded(c, [&] {
    MFT_REQUIRE(kind >= 0 && kind < MFT_K_COUNT, MFT_ERR_ARG, "bad kernel kind");
    set_device(c);
    prof_drain(c);
    if (total_ms) *total_ms = c->prof_ms[kind];
    if (launches) *launches = c->prof_n[kind];
    if (name) *name = names[kind];
  });
}

mft_status mft_region(mft_ctx* c, int begin, double* ms) {
  return guarded(c, [&] {
    set_device(c);
    for (auto& e : c->region_ev)
      if (!e) MFT_CUDA(cudaEventCreate(&e));
    if (begin) {
      MFT_CUDA(cudaEventRecord(c->region_ev[0], c->stream));
    } else {
      MFT_CUDA(cudaEventRecord(c->region_ev[1], c->stream));
      MFT_CUDA(cudaEventSynchronize(c->region_ev[1]));
      float t = 0.f;
      MFT_CUDA(cudaEventElapsedTime(&t, c->region_ev[0], c->region_ev[1]));
      if (ms) *ms = t;
    }
  });
}

mft_status mft_get_viscosity(mft_ctx* c, double* eps) {
  return guarded(c, [&] {
    MFT_REQUIRE(eps, MFT_ERR_ARG, "eps is NULL");
    MFT_REQUIRE(c->eps.p, MFT_ERR_STATE, "no viscosity evaluated yet");
    set_device(c);
    MFT_CUDA(cudaMemcpyAsync(eps, c->eps.p, c->n * sizeof(double), cudaMemcpyDeviceToHost,
                             c->stream));
    MFT_CUDA(cudaStreamSynchronize(c->stream));
  });
}

// ---------------------------------------------------------------- positivity limiter

mft_status mft_set_limiter(mft_ctx* c, int nvar, const int* variables, const double* thresholds) {
  return guarded(c, [&] {
    MFT_REQUIRE(nvar >= 0 && nvar <= 4, MFT_ERR_ARG, "between 0 and 4 limiter variables");
    MFT_REQUIRE(nvar == 0 || (variables && thresholds), MFT_ERR_ARG, "NULL variables/thresholds");
    if (nvar > 0) MFT_REQUIRE(c->eq == MFT_EQ_EULER2D, MFT_ERR_UNSUPPORTED,
                              "the positivity limiter needs the 2D Euler equations");
    for (int q = 0; q < nvar; ++q) {
      MFT_REQUIRE(variables[q] == MFT_LIM_DENSITY || variables[q] == MFT_LIM_PRESSURE,
                  MFT_ERR_ARG, "limiter variable must be MFT_LIM_DENSITY or MFT_LIM_PRESSURE");
      MFT_REQUIRE(isfinite(thresholds[q]), MFT_ERR_ARG, "limiter threshold must be finite");
    }
    c->lim_n = nvar;
    for (int q = 0; q < nvar; ++q) {
      c->lim_var[q] = variables[q];
      c->lim_thr[q] = thresholds[q];
    }
    c->graph_valid = false;
    c->fsal_valid = false;
  });
}

mft_status mft_limit(mft_ctx* c, double* const* u, int nvars) {
  return guarded(c, [&] {
    check_state_ready(c);
    MFT_REQUIRE(u && nvars == c->nvars, MFT_ERR_ARG, "bad state arrays or nvars");
    MFT_REQUIRE(c->lim_n > 0, MFT_ERR_STATE, "no limiter configured (mft_set_limiter)");
    set_device(c);
    ensure_work(c);
    ensure_device_ops(c);
    const int64_t n = c->n;
    cudaStream_t s = c->stream;
    for (int v = 0; v < nvars; ++v)
      MFT_CUDA(cudaMemcpyAsync(c->soa.p + (size_t)v * n, u[v], n * sizeof(double),
                               cudaMemcpyHostToDevice, s));
    launch_aos_from_soa(c->soa.p, c->work_u.p, n, nvars, s);
    apply_limiter(c, c->work_u.p, nullptr);
    launch_soa_from_aos(c->work_u.p, c->soa.p, n, nvars, s);
    for (int v = 0; v < nvars; ++v)
      MFT_CUDA(cudaMemcpyAsync(u[v], c->soa.p + (size_t)v * n, n * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    check_kernel_errors(c);
  });
}

// ---------------------------------------------------------------- adjoint

namespace {

// Hyperviscosity mode of the adjoint (0 none, 1 Tominec, 2 Flyer) and its gamma;
// viscosity sources have no adjoint.
// The hyperviscosity mode of the adjoint (0 none, 1 Tominec, 2 Flyer) and whether a
// residual/upwind viscosity source is present (its selections are differentiated frozen,
// see mft_adjoint_visc.cu).  A viscosity source must come before any hyperviscosity
// source (its partial du is then the flux divergence alone) and needs one problem (no
// ensemble segments).
int adj_hv_mode(mft_ctx* c, double* gamma, bool* visc = nullptr) {
  int mode = 0;
  bool has_visc = false;
  *gamma = 0.0;
  for (size_t k = 0; k < c->src_kind.size(); ++k) {
    const int kind = c->src_kind[k];
    MFT_REQUIRE(kind != MFT_SRC_IGR, MFT_ERR_UNSUPPORTED,
                "adjoint: the IGR source (an iterative solve) has no adjoint");
    if (kind == MFT_SRC_RV || kind == MFT_SRC_UPWIND) {
      MFT_REQUIRE(!has_visc, MFT_ERR_UNSUPPORTED, "more than one viscosity source");
      MFT_REQUIRE(mode == 0, MFT_ERR_UNSUPPORTED,
                  "adjoint: a viscosity source after a hyperviscosity source (the residual "
                  "would include the hyperviscosity term) is not provided");
      MFT_REQUIRE(c->nseg == 0, MFT_ERR_UNSUPPORTED,
                  "adjoint: viscosity sources of ensembles are not provided");
      has_visc = true;
      continue;
    }
    MFT_REQUIRE(mode == 0, MFT_ERR_UNSUPPORTED, "more than one hyperviscosity source");
    mode = kind == MFT_SRC_HV_TOMINEC ? 1 : 2;
    *gamma = c->src_par[k * 4];
  }
  if (visc) *visc = has_visc;
  return mode;
}

void check_adjoint_ready(mft_ctx* c) {
  check_state_ready(c);
  MFT_REQUIRE(c->lim_n == 0, MFT_ERR_UNSUPPORTED,
              "adjoint: the positivity limiter is not differentiable (turn it off)");
  MFT_REQUIRE(c->dim == 2, MFT_ERR_UNSUPPORTED, "adjoint: 2D problems only");
  MFT_REQUIRE(c->precision == MFT_PREC_FP64, MFT_ERR_UNSUPPORTED, "adjoint: FP64 form only");
  double g;
  adj_hv_mode(c, &g);
}

void ensure_adj_work(mft_ctx* c) {
  const size_t nv = (size_t)c->n * c->nvars;
  for (auto& b : c->adj_lam) b.alloc(nv);
  c->adj_acc.alloc(nv);
  c->adj_q.alloc(nv);
}

// out = stage combination `kind` of (d rhs!/du)^T lam at state u (n x V AoS, device) and
// time t (the Dirichlet values of the BC pass, which the viscosity source sees).
void eval_rhs_adjoint(mft_ctx* c, const double* u, const double* lam, int kind, double dt,
                      double* acc, double* out, double t) {
  ensure_device_ops(c);
  ensure_bcs(c);
  double hv_gamma = 0.0;
  bool visc = false;
  const int hv = adj_hv_mode(c, &hv_gamma, &visc);
  const double* xadd = nullptr;
  if (visc) {
    // a forward evaluation at u gives the viscosity, its partial du and norms and the
    // BC-corrected state; then the viscosity source's transpose product
    const size_t nv = (size_t)c->n * c->nvars;
    c->adj_ubc.alloc(nv);
    c->adj_du.alloc(nv);
    c->adj_xadd.alloc(nv);
    MFT_CUDA(cudaMemcpyAsync(c->adj_ubc.p, u, nv * sizeof(double), cudaMemcpyDeviceToDevice,
                             c->stream));
    Epilogue ef{};
    ef.kind = kOutDu;
    ef.out = c->adj_du.p;
    eval_rhs(c, c->adj_ubc.p, nullptr, t, ef);
    ProfScope ps(c, MFT_K_ADJ);
    visc_adjoint_terms(c, c->adj_ubc.p, lam, c->adj_xadd.p);
    xadd = c->adj_xadd.p;
  }
  if (hv == 1) MFT_REQUIRE(c->have_val[kSlotLap], MFT_ERR_STATE, "Tominec HV needs MFT_OP_LAP");
  if (hv == 2) MFT_REQUIRE(c->have_val[kSlotHv], MFT_ERR_STATE, "Flyer HV needs MFT_OP_HV");
  MFT_REQUIRE(out != lam, MFT_ERR_ARG, "adjoint output aliases its input");
  cudaStream_t s = c->stream;
  BcDev bc{c->d_tag.p, c->d_slot.p, c->d_normal.p, c->d_dvals.p};
  const int has_bc = c->nb > 0;
  if (hv == 1) {
    ProfScope ps(c, MFT_K_ADJ);
    launch_lap_masked(c->n, c->fwd.view(), c->fw[kSlotLap].p, lam, c->nvars, bc, has_bc,
                      c->adj_q.p, s);
  }
  AdjArgs a{};
  a.n = c->n;
  a.ell = c->rev.view();
  a.w[0] = c->rw[0].p;
  a.w[1] = c->rw[1].p;
  a.wh = hv == 1 ? c->rw[kSlotLap].p : (hv == 2 ? c->rw[kSlotHv].p : nullptr);
  a.hv = hv;
  a.hv_gamma = hv_gamma;
  a.lam = lam;
  a.q = c->adj_q.p;
  a.u = u;
  a.eq = c->eq;
  a.V = c->nvars;
  a.gamma = c->gamma;
  a.ax = c->adv[0];
  a.ay = c->adv[1];
  a.bc = bc;
  a.has_bc = has_bc;
  a.kind = kind;
  a.dt = dt;
  a.acc = acc;
  a.out = out;
  a.xadd = xadd;
  ProfScope ps(c, MFT_K_ADJ);
  if (use_dw(c) && hv != 1) {
    ensure_device_ops(c);
    a.wdw[0] = c->rwdw[0].p;
    a.wdw[1] = c->rwdw[1].p;
    a.whdw = hv == 2 ? c->rwdw[kSlotHv].p : nullptr;
    c->adj_lamdw.alloc((size_t)c->n * 4);
    // staged unless a fixed direct variant of the double-word gathers is requested
    const bool staged = !(c->dw_variant >= 0 && c->dw_variant < 6);
    a.ell = c->rev.view();
    launch_adj_dw(a, c->adj_lamdw.p, staged, s);
  } else {
    launch_adj_f64(a, s);
  }
}

// Time of the first stage of step k as the FSAL integrator evaluates it.
double stage1_time(double t0, double dt, int k) { return k == 0 ? t0 : (t0 + (k - 1) * dt) + dt; }

// One SSP-RK3 step from x: stage states into s1, s2, the next state into y.  Same
// kernels and epilogues as the FSAL integrator (the first stage fused here).
void record_step(mft_ctx* c, double dt, int k, double* x, double* s1, double* s2, double* y) {
  const double t0 = c->adj_t0;
  const double t = t0 + k * dt;
  Epilogue e1{};
  e1.kind = kStage1;
  e1.dt = dt;
  e1.out = s1;
  eval_rhs(c, x, nullptr, stage1_time(t0, dt, k), e1);
  Epilogue e2{};
  e2.kind = kStage2;
  e2.dt = dt;
  e2.u_n = x;
  e2.out = s2;
  eval_rhs(c, s1, nullptr, t + dt, e2);
  Epilogue e3{};
  e3.kind = kStage3;
  e3.dt = dt;
  e3.u_n = x;
  e3.out = y;
  eval_rhs(c, s2, nullptr, t + 0.5 * dt, e3);
}

void d2d(mft_ctx* c, double* dst, const double* src, size_t count) {
  MFT_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
}

void ssprk33_record(mft_ctx* c, double dt, int nsteps, int every) {
  ensure_work(c);
  ensure_adj_work(c);
  const size_t nv = (size_t)c->n * c->nvars;
  c->adj_valid = false;
  c->adj_t0 = c->t_state;
  c->adj_dt = dt;
  c->adj_nsteps = nsteps;
  c->adj_every = every;
  if (every == 0) {
    c->adj_ckpt.release();
    c->adj_store.alloc((size_t)3 * nsteps * nv);
    double* st = c->adj_store.p;
    d2d(c, st, c->U[0].p, nv);
    for (int k = 0; k < nsteps; ++k) {
      double* x = st + (size_t)3 * k * nv;
      double* y = k + 1 < nsteps ? x + 3 * nv : c->U[0].p;
      record_step(c, dt, k, x, x + nv, x + 2 * nv, y);
    }
  } else {
    const int nck = (nsteps + every - 1) / every;
    c->adj_ckpt.alloc((size_t)nck * nv);
    c->adj_store.alloc((size_t)3 * every * nv);
    for (int k = 0; k < nsteps; ++k) {
      if (k % every == 0) d2d(c, c->adj_ckpt.p + (size_t)(k / every) * nv, c->U[0].p, nv);
      record_step(c, dt, k, c->U[0].p, c->U[1].p, c->U[2].p, c->U[3].p);
      std::swap(c->U[0].p, c->U[3].p);
    }
  }
  c->t_state = c->adj_t0 + nsteps * dt;
  // the pending first stage of the next step, as the FSAL integrator leaves it
  Epilogue e1{};
  e1.kind = kStage1;
  e1.dt = dt;
  e1.out = c->U[1].p;
  eval_rhs(c, c->U[0].p, nullptr, stage1_time(c->adj_t0, dt, nsteps), e1);
  c->fsal_valid = true;
  c->fsal_dt = dt;
  c->adj_valid = true;
}

// Reverse sweep; L holds Pi lam_T on entry (n x V AoS) and dJ/du0 on return.
void ssprk33_adjoint_sweep(mft_ctx* c, double* L) {
  const size_t nv = (size_t)c->n * c->nvars;
  const int N = c->adj_nsteps, E = c->adj_every;
  const double dt = c->adj_dt;
  double* A = c->adj_lam[1].p;
  double* B = c->adj_lam[2].p;
  double* acc = c->adj_acc.p;
  const double t0 = c->adj_t0;
  auto back = [&](int k, const double* x, const double* s1, const double* s2) {
    const double t = t0 + k * dt;
    eval_rhs_adjoint(c, s2, L, kAdjStage3, dt, acc, A, t + 0.5 * dt);
    eval_rhs_adjoint(c, s1, A, kAdjStage2, dt, acc, B, t + dt);
    eval_rhs_adjoint(c, x, B, kAdjStage1, dt, acc, L, stage1_time(t0, dt, k));
  };
  double* st = c->adj_store.p;
  if (E == 0) {
    for (int k = N - 1; k >= 0; --k) {
      const double* x = st + (size_t)3 * k * nv;
      back(k, x, x + nv, x + 2 * nv);
    }
    return;
  }
  const int nck = (N + E - 1) / E;
  for (int seg = nck - 1; seg >= 0; --seg) {
    const int a = seg * E, b = std::min(N, a + E);
    d2d(c, st, c->adj_ckpt.p + (size_t)seg * nv, nv);
    for (int k = a; k < b; ++k) {
      double* x = st + (size_t)3 * (k - a) * nv;
      double* y = k + 1 < b ? x + 3 * nv : c->U[3].p;
      record_step(c, dt, k, x, x + nv, x + 2 * nv, y);
    }
    for (int k = b - 1; k >= a; --k) {
      const double* x = st + (size_t)3 * (k - a) * nv;
      back(k, x, x + nv, x + 2 * nv);
    }
  }
}

void ssprk33_adjoint_soa(mft_ctx* c, double* lam_soa) {
  MFT_REQUIRE(c->adj_valid, MFT_ERR_STATE, "call mft_ssprk33_record first");
  check_adjoint_ready(c);
  ensure_work(c);
  ensure_adj_work(c);
  ensure_bcs(c);
  cudaStream_t s = c->stream;
  const int64_t n = c->n;
  const int V = c->nvars;
  double* L = c->adj_lam[0].p;
  launch_aos_from_soa(lam_soa, L, n, V, s);
  BcDev bc{c->d_tag.p, c->d_slot.p, c->d_normal.p, c->d_dvals.p};
  if (c->nb > 0) launch_bc_project(c->nb, c->d_bnode.p, V, bc, L, s);
  ssprk33_adjoint_sweep(c, L);
  launch_soa_from_aos(L, lam_soa, n, V, s);
}

}  // namespace

mft_status mft_rhs_adjoint(mft_ctx* c, double* const* out, const double* const* lam,
                           const double* const* u, int nvars, double t) {
  return guarded(c, [&] {
    check_adjoint_ready(c);
    MFT_REQUIRE(out && lam && u && nvars == c->nvars, MFT_ERR_ARG, "bad arrays or nvars");
    set_device(c);
    ensure_work(c);
    ensure_adj_work(c);
    const int64_t n = c->n;
    const int V = c->nvars;
    cudaStream_t s = c->stream;
    for (int v = 0; v < V; ++v) {
      MFT_CUDA(cudaMemcpyAsync(c->soa.p + (size_t)v * n, u[v], n * sizeof(double),
                               cudaMemcpyHostToDevice, s));
      MFT_CUDA(cudaMemcpyAsync(c->soa2.p + (size_t)v * n, lam[v], n * sizeof(double),
                               cudaMemcpyHostToDevice, s));
    }
    launch_aos_from_soa(c->soa.p, c->work_u.p, n, V, s);
    launch_aos_from_soa(c->soa2.p, c->adj_lam[0].p, n, V, s);
    eval_rhs_adjoint(c, c->work_u.p, c->adj_lam[0].p, kAdjPlain, 0.0, nullptr, c->adj_lam[1].p,
                     t);
    launch_soa_from_aos(c->adj_lam[1].p, c->soa.p, n, V, s);
    for (int v = 0; v < V; ++v)
      MFT_CUDA(cudaMemcpyAsync(out[v], c->soa.p + (size_t)v * n, n * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    check_kernel_errors(c);
  });
}

mft_status mft_rhs_adjoint_device(mft_ctx* c, double* out, const double* lam, const double* u,
                                  double t) {
  return guarded(c, [&] {
    check_adjoint_ready(c);
    MFT_REQUIRE(out && lam && u, MFT_ERR_ARG, "NULL device array");
    set_device(c);
    ensure_work(c);
    ensure_adj_work(c);
    const int64_t n = c->n;
    const int V = c->nvars;
    cudaStream_t s = c->stream;
    launch_aos_from_soa(u, c->work_u.p, n, V, s);
    launch_aos_from_soa(lam, c->adj_lam[0].p, n, V, s);
    eval_rhs_adjoint(c, c->work_u.p, c->adj_lam[0].p, kAdjPlain, 0.0, nullptr, c->adj_lam[1].p,
                     t);
    launch_soa_from_aos(c->adj_lam[1].p, out, n, V, s);
    check_kernel_errors(c);
  });
}

mft_status mft_ssprk33_record(mft_ctx* c, double dt, int nsteps, int every) {
  return guarded(c, [&] {
    MFT_REQUIRE(c->state_valid, MFT_ERR_STATE, "call mft_set_state first");
    MFT_REQUIRE(nsteps >= 1, MFT_ERR_ARG, "nsteps < 1");
    MFT_REQUIRE(every >= -1, MFT_ERR_ARG, "every < -1");
    MFT_REQUIRE(dt > 0 && isfinite(dt), MFT_ERR_ARG, "dt must be positive and finite");
    check_adjoint_ready(c);
    set_device(c);
    if (every == -1) {
      // every stage state when they fit in half of the device memory free (counting what
      // the previous recording holds), which spares the sweep its recomputation; else
      // checkpoints every ~sqrt(nsteps / 3) steps (the least memory)
      size_t free_b = 0, total_b = 0;
      MFT_CUDA(cudaMemGetInfo(&free_b, &total_b));
      const double avail = (double)free_b + 8.0 * (double)(c->adj_store.n + c->adj_ckpt.n);
      const double need = 3.0 * nsteps * (double)c->n * c->nvars * 8.0;
      every = need <= 0.5 * avail ? 0 : std::max(1, (int)ceil(sqrt(nsteps / 3.0)));
    }
    ssprk33_record(c, dt, nsteps, every);
    check_kernel_errors(c);
  });
}

mft_status mft_ssprk33_adjoint(mft_ctx* c, double* const* lam, int nvars) {
  return guarded(c, [&] {
    MFT_REQUIRE(lam && nvars == c->nvars, MFT_ERR_ARG, "bad arrays or nvars");
    set_device(c);
    ensure_work(c);
    const int64_t n = c->n;
    cudaStream_t s = c->stream;
    for (int v = 0; v < nvars; ++v)
      MFT_CUDA(cudaMemcpyAsync(c->soa2.p + (size_t)v * n, lam[v], n * sizeof(double),
                               cudaMemcpyHostToDevice, s));
    ssprk33_adjoint_soa(c, c->soa2.p);
    for (int v = 0; v < nvars; ++v)
      MFT_CUDA(cudaMemcpyAsync(lam[v], c->soa2.p + (size_t)v * n, n * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    check_kernel_errors(c);
  });
}

mft_status mft_ssprk33_adjoint_device(mft_ctx* c, double* lam) {
  return guarded(c, [&] {
    MFT_REQUIRE(lam, MFT_ERR_ARG, "NULL device array");
    set_device(c);
    ssprk33_adjoint_soa(c, lam);
    check_kernel_errors(c);
  });
}

}  // extern "C"
