// FP32-apply gathers with bulk-copy staging (Euler, V = 4).
//
// The plain FP32 gathers are latency-bound: every stencil entry needs its column index
// before the neighbour state can be loaded.  Here each warp owns one 32-row slice at a
// time (persistent grid) and streams the slice's index and weight arrays into shared
// memory in chunks of kCh slots with cp.async.bulk, two chunks ahead of use and
// completed on an mbarrier.  The warp then issues the kCh neighbour-state gathers of a
// chunk back to back, so only those (L1/L2-resident) loads remain on the critical path.
// Waits are bounded: on a timeout the warp records MFT_ERR_TIMEOUT in *err, waits
// (bounded) for its copies in flight and stops.
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>
#include <vector>

#include "mft_device.cuh"
#include "mft_internal.cuh"
#include "mft_tma.cuh"

namespace mft {

namespace {

using namespace dev;

constexpr int kTmaWarps = 4;    // warps per block
constexpr uint32_t kWaitLimit = 1u << 22;

// Warp-uniform cursor over (slice, chunk) pairs of this warp's slices.
struct Cursor {
  int64_t s;
  int c;
};

__device__ __forceinline__ int slice_slots(const EllView& e, int64_t s) {
  return (int)((e.slice_off[s + 1] - e.slice_off[s]) >> 5);
}

// Row length of this lane's row in slice s (0 past the end); loaded one slice ahead.
__device__ __forceinline__ int row_len_at(const EllView& e, int64_t n, int64_t s, int lane,
                                          int64_t nslices) {
  const int64_t i = (s << 5) + lane;
  return (s < nslices && i < n) ? e.row_len[i] : 0;
}

// The stage epilogue's node records (stage state, step-start state) requested into L2 at
// the start of a slice, so that they arrive while the slice's gathers run.
__device__ __forceinline__ void prefetch_epilogue(const Epilogue& ep, int64_t i) {
  tma::prefetch_l2(ep.u_s + i * 4);
  if (ep.kind == kStage2 || ep.kind == kStage3) tma::prefetch_l2(ep.u_n + i * 4);
}

template <int NARR, int CH>
__device__ __forceinline__ void issue_chunk(unsigned char (*buf)[CH * 128], uint64_t* bar,
                                            const EllView& e, const void* const* arrs,
                                            Cursor cur) {
  const int slots = slice_slots(e, cur.s);
  const int n = min(CH, slots - cur.c * CH);
  const uint32_t bytes = (uint32_t)n * 32u * 4u;
  const int64_t base = e.slice_off[cur.s] + (int64_t)cur.c * CH * 32;
  const uint64_t pol = tma::policy_evict_first();
  tma::fence_proxy_async();
  tma::arrive_expect_tx(bar, bytes * NARR);
#pragma unroll
  for (int k = 0; k < NARR; ++k)
    tma::bulk_g2s_hint(buf[k], static_cast<const unsigned char*>(arrs[k]) + base * 4, bytes,
                       bar, pol);
}

template <int CH>
__device__ __forceinline__ void advance(const EllView& e, Cursor& cur, int64_t stride) {
  const int nch = (slice_slots(e, cur.s) + CH - 1) / CH;
  if (++cur.c >= nch) {
    cur.c = 0;
    cur.s += stride;
  }
}

template <int CH, bool WT, bool WQ, int FLY>
__global__ void __launch_bounds__(32 * kTmaWarps) k_fwd_euler_f32_tma(FwdArgs a, int* err) {
  constexpr int NARR = (WQ || FLY) ? 4 : 3;
  __shared__ __align__(128) unsigned char sbuf[kTmaWarps][2][NARR][CH * 128];
  __shared__ __align__(8) uint64_t bars[kTmaWarps][2];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t nslices = (a.n + 31) >> 5;
  const int64_t stride = (int64_t)gridDim.x * kTmaWarps;
  const int64_t first = (int64_t)blockIdx.x * kTmaWarps + w;
  const void* arrs[4] = {a.ell.col, a.w32[0], a.w32[1], a.wl32};
  if (lane == 0) {
    tma::bar_init(&bars[w][0], 1);
    tma::bar_init(&bars[w][1], 1);
    tma::fence_init();
  }
  __syncwarp();
  const float4* __restrict__ U4 = reinterpret_cast<const float4*>(a.u32);
  const float gm1 = a.gm1_32;
  const float hg = a.hg32;
  uint32_t phase[2] = {0u, 0u};
  bool pending[2] = {false, false};
  Cursor iss{first, 0};
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    if (iss.s < nslices) {
      if (lane == 0) issue_chunk<NARR, CH>(sbuf[w][b], &bars[w][b], a.ell, arrs, iss);
      pending[b] = true;
      advance<CH>(a.ell, iss, stride);
    }
  }
  int buf = 0;
  int len_next = row_len_at(a.ell, a.n, first, lane, nslices);
  for (int64_t s = first; s < nslices; s += stride) {
    const int64_t r = (s << 5) + lane;  // layout row
    const bool valid = r < a.n;
    const int64_t i = valid ? ell_node(a.ell, r) : 0;
    const int len = len_next;
    len_next = row_len_at(a.ell, a.n, s + stride, lane, nslices);
    if (valid && a.final_epilogue) prefetch_epilogue(a.ep, i);
    const int slots = slice_slots(a.ell, s);
    const int nch = (slots + CH - 1) / CH;
    float f[4] = {0, 0, 0, 0}, tx[4] = {0, 0, 0, 0}, ty[4] = {0, 0, 0, 0}, q[4] = {0, 0, 0, 0};
    for (int c = 0; c < nch; ++c) {
      if (!tma::wait_bounded(&bars[w][buf], phase[buf], kWaitLimit)) {
        if (lane == 0) atomicExch(err, MFT_ERR_TIMEOUT);
        for (int b = 0; b < 2; ++b)
          if (pending[b]) tma::wait_bounded(&bars[w][b], phase[b], kWaitLimit);
        return;
      }
      phase[buf] ^= 1u;
      pending[buf] = false;
      const int* scol = reinterpret_cast<const int*>(sbuf[w][buf][0]);
      const float* swx = reinterpret_cast<const float*>(sbuf[w][buf][1]);
      const float* swy = reinterpret_cast<const float*>(sbuf[w][buf][2]);
      const float* swl = reinterpret_cast<const float*>(sbuf[w][buf][NARR - 1]);
      const int j0 = c * CH;
      float4 uc[CH];
#pragma unroll
      for (int k = 0; k < CH; ++k)
        if (j0 + k < len) uc[k] = __ldg(U4 + scol[k * 32 + lane]);
#pragma unroll
      for (int k = 0; k < CH; ++k) {
        if (j0 + k < len) {
          const float wx = swx[k * 32 + lane], wy = swy[k * 32 + lane];
          euler_accum_f32<WT>(gm1, uc[k], wx, wy, f, tx, ty);
          if (WQ || FLY) {
            const float wl = swl[k * 32 + lane];
            q[0] = fmaf(wl, uc[k].x, q[0]); q[1] = fmaf(wl, uc[k].y, q[1]);
            q[2] = fmaf(wl, uc[k].z, q[2]); q[3] = fmaf(wl, uc[k].w, q[3]);
          }
        }
      }
      __syncwarp();
      if (iss.s < nslices) {
        if (lane == 0) issue_chunk<NARR, CH>(sbuf[w][buf], &bars[w][buf], a.ell, arrs, iss);
        pending[buf] = true;
        advance<CH>(a.ell, iss, stride);
      }
      buf ^= 1;
    }
    if (!valid) continue;
    if (WT) f[0] = tx[1] + ty[2];
    float du[4] = {-f[0], -f[1], -f[2], -f[3]};
    if (FLY == 1)
      for (int v = 0; v < 4; ++v) du[v] = fmaf(-hg, q[v], du[v]);
    if (WT) {
      float4* t4 = reinterpret_cast<float4*>(a.t32) + i * 2;
      t4[0] = make_float4(tx[0], tx[1], tx[2], tx[3]);
      t4[1] = make_float4(ty[0], ty[1], ty[2], ty[3]);
    }
    if (WQ) reinterpret_cast<float4*>(a.q32)[i] = make_float4(q[0], q[1], q[2], q[3]);
    if (FLY == 2)
      for (int v = 0; v < 4; ++v) a.hvf[i * 4 + v] = fpconv::f2d(-hg * q[v]);
    if (a.final_epilogue) {
      double d[4] = {fpconv::f2d(du[0]), fpconv::f2d(du[1]), fpconv::f2d(du[2]),
                     fpconv::f2d(du[3])};
      finish_node<4>(a.ep, i, d);
    } else {
      reinterpret_cast<float4*>(a.du_p32)[i] = make_float4(du[0], du[1], du[2], du[3]);
    }
  }
}

template <int CH, bool RV, bool LAP>
__global__ void __launch_bounds__(32 * kTmaWarps) k_rev_f32_tma(RevArgs a, int* err) {
  constexpr int kRevBatch = CH < 4 ? CH : 4;
  constexpr int NARR = 1 + (RV ? 2 : 0) + (LAP ? 1 : 0);
  __shared__ __align__(128) unsigned char sbuf[kTmaWarps][2][NARR][CH * 128];
  __shared__ __align__(8) uint64_t bars[kTmaWarps][2];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t nslices = (a.n + 31) >> 5;
  const int64_t stride = (int64_t)gridDim.x * kTmaWarps;
  const int64_t first = (int64_t)blockIdx.x * kTmaWarps + w;
  const void* arrs[4];
  {
    int k = 0;
    arrs[k++] = a.ell.col;
    if (RV) { arrs[k++] = a.w32[0]; arrs[k++] = a.w32[1]; }
    if (LAP) arrs[k++] = a.wl32;
    for (; k < 4; ++k) arrs[k] = nullptr;
  }
  if (lane == 0) {
    tma::bar_init(&bars[w][0], 1);
    tma::bar_init(&bars[w][1], 1);
    tma::fence_init();
  }
  __syncwarp();
  const float4* __restrict__ Q4 = reinterpret_cast<const float4*>(a.q32);
  const float hg = a.hg32;
  uint32_t phase[2] = {0u, 0u};
  bool pending[2] = {false, false};
  Cursor iss{first, 0};
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    if (iss.s < nslices) {
      if (lane == 0) issue_chunk<NARR, CH>(sbuf[w][b], &bars[w][b], a.ell, arrs, iss);
      pending[b] = true;
      advance<CH>(a.ell, iss, stride);
    }
  }
  int buf = 0;
  int len_next = row_len_at(a.ell, a.n, first, lane, nslices);
  for (int64_t s = first; s < nslices; s += stride) {
    const int64_t r = (s << 5) + lane;  // layout row
    const bool valid = r < a.n;
    const int64_t i = valid ? ell_node(a.ell, r) : 0;
    const int len = len_next;
    len_next = row_len_at(a.ell, a.n, s + stride, lane, nslices);
    if (valid) {
      tma::prefetch_l2(a.du_p32 + i * 4);
      if (a.final_epilogue) prefetch_epilogue(a.ep, i);
    }
    const int slots = slice_slots(a.ell, s);
    const int nch = (slots + CH - 1) / CH;
    float sx[4] = {0, 0, 0, 0}, sy[4] = {0, 0, 0, 0}, sl[4] = {0, 0, 0, 0};
    for (int c = 0; c < nch; ++c) {
      if (!tma::wait_bounded(&bars[w][buf], phase[buf], kWaitLimit)) {
        if (lane == 0) atomicExch(err, MFT_ERR_TIMEOUT);
        for (int b = 0; b < 2; ++b)
          if (pending[b]) tma::wait_bounded(&bars[w][b], phase[b], kWaitLimit);
        return;
      }
      phase[buf] ^= 1u;
      pending[buf] = false;
      const int* scol = reinterpret_cast<const int*>(sbuf[w][buf][0]);
      const float* swx = reinterpret_cast<const float*>(sbuf[w][buf][RV ? 1 : 0]);
      const float* swy = reinterpret_cast<const float*>(sbuf[w][buf][RV ? 2 : 0]);
      const float* swl = reinterpret_cast<const float*>(sbuf[w][buf][NARR - 1]);
      const int j0 = c * CH;
      // batches of kRevBatch slots: both records of every slot of a batch are requested
      // before any is accumulated (one latency per batch, few registers held); each
      // accumulator still takes its slots in order
#pragma unroll
      for (int k0 = 0; k0 < CH; k0 += kRevBatch) {
        F8 st[kRevBatch];
        float4 qs[kRevBatch];
#pragma unroll
        for (int k = 0; k < kRevBatch; ++k) {
          const int kk = k0 + k;
          if (j0 + kk < len) {
            const int64_t cc = scol[kk * 32 + lane];
            if (RV) st[k] = ldg_f8(a.s32 + cc * 8);
            if (LAP) qs[k] = __ldg(Q4 + cc);
          }
        }
#pragma unroll
        for (int k = 0; k < kRevBatch; ++k) {
          const int kk = k0 + k;
          if (j0 + kk >= len) continue;
          if (RV) {
            const float wx = swx[kk * 32 + lane], wy = swy[kk * 32 + lane];
            const float4 xs = st[k].lo, ys = st[k].hi;
            sx[0] = fmaf(wx, xs.x, sx[0]); sx[1] = fmaf(wx, xs.y, sx[1]);
            sx[2] = fmaf(wx, xs.z, sx[2]); sx[3] = fmaf(wx, xs.w, sx[3]);
            sy[0] = fmaf(wy, ys.x, sy[0]); sy[1] = fmaf(wy, ys.y, sy[1]);
            sy[2] = fmaf(wy, ys.z, sy[2]); sy[3] = fmaf(wy, ys.w, sy[3]);
          }
          if (LAP) {
            const float wl = swl[kk * 32 + lane];
            sl[0] = fmaf(wl, qs[k].x, sl[0]); sl[1] = fmaf(wl, qs[k].y, sl[1]);
            sl[2] = fmaf(wl, qs[k].z, sl[2]); sl[3] = fmaf(wl, qs[k].w, sl[3]);
          }
        }
      }
      __syncwarp();
      if (iss.s < nslices) {
        if (lane == 0) issue_chunk<NARR, CH>(sbuf[w][buf], &bars[w][buf], a.ell, arrs, iss);
        pending[buf] = true;
        advance<CH>(a.ell, iss, stride);
      }
      buf ^= 1;
    }
    if (!valid) continue;
    float du[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      float d = a.du_p32[i * 4 + v];
      if (RV) d = (d - sx[v]) - sy[v];
      if (LAP) d = fmaf(-hg, sl[v], d);
      if (a.hvf) d += fpconv::d2f(a.hvf[i * 4 + v]);
      du[v] = d;
    }
    if (a.final_epilogue) {
      double d[4] = {fpconv::f2d(du[0]), fpconv::f2d(du[1]), fpconv::f2d(du[2]),
                     fpconv::f2d(du[3])};
      finish_node<4>(a.ep, i, d);
    } else {
#pragma unroll
      for (int v = 0; v < 4; ++v) a.du_p_out32[i * 4 + v] = du[v];
    }
  }
}

// Resident blocks of one kernel on the current device (SMs x blocks per SM).  The
// instantiations share a function type but not their register or shared-memory use, so
// the figure is cached per (kernel, device): a grid sized for another instantiation
// would run its last blocks as a second partial wave.
int resident_blocks(const void* kernel) {
  struct Entry {
    const void* k;
    int dev, blocks;
  };
  static std::mutex mu;
  static std::vector<Entry> cache;
  int dev = 0;
  MFT_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  for (const Entry& e : cache)
    if (e.k == kernel && e.dev == dev) return e.blocks;
  int sms = 0, per = 0;
  MFT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MFT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 32 * kTmaWarps, 0));
  cache.push_back({kernel, dev, sms * (per > 0 ? per : 1)});
  return cache.back().blocks;
}

// Persistent grid: at most one wave of resident blocks, and no more warps than slices.
// The slices are then spread evenly: with s slices and w warps a warp takes ceil(s / w)
// of them, so w is lowered to the smallest count with the same ceiling.
// Error-path self-test: the barrier is initialised and never arrived on, and no bulk copy
// is issued, so nothing is in flight when the warp gives up.
__global__ void k_wait_selftest(int* err, uint32_t polls) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    tma::bar_init(&bar, 1);
    tma::fence_init();
  }
  __syncwarp();
  const bool done = tma::wait_bounded(&bar, 0u, polls);
  if (!done && threadIdx.x == 0) atomicExch(err, MFT_ERR_TIMEOUT);
}

template <class K>
unsigned persistent_grid(K kernel, int64_t n) {
  const int64_t cap = resident_blocks(reinterpret_cast<const void*>(kernel));
  const int64_t slices = (n + 31) / 32;
  int64_t blocks = (slices + kTmaWarps - 1) / kTmaWarps;
  if (blocks > cap) {
    const int64_t per_warp = (slices + cap * kTmaWarps - 1) / (cap * kTmaWarps);
    const int64_t warps = (slices + per_warp - 1) / per_warp;
    blocks = (warps + kTmaWarps - 1) / kTmaWarps;
  }
  return (unsigned)blocks;
}

}  // namespace

template <int CH>
static void fwd_tma(const FwdArgs& a, int* err, cudaStream_t s) {
  const bool wt = a.want_t != 0, wq = a.want_q != 0;
#define MFT_T(WT, WQ, FLY)                                                              \
  do {                                                                                  \
    const unsigned g = persistent_grid(k_fwd_euler_f32_tma<CH, WT, WQ, FLY>, a.n);      \
    k_fwd_euler_f32_tma<CH, WT, WQ, FLY><<<g, 32 * kTmaWarps, 0, s>>>(a, err);          \
  } while (0)
  if (a.flyer == 0) {
    if (wt && wq) MFT_T(true, true, 0);
    else if (wt) MFT_T(true, false, 0);
    else if (wq) MFT_T(false, true, 0);
    else MFT_T(false, false, 0);
  } else if (a.flyer == 1) {
    if (wt) MFT_T(true, false, 1);
    else MFT_T(false, false, 1);
  } else {
    if (wt) MFT_T(true, false, 2);
    else MFT_T(false, false, 2);
  }
#undef MFT_T
}

template <int CH>
static void rev_tma(const RevArgs& a, int* err, cudaStream_t s) {
  if (a.rv && a.lap)
    k_rev_f32_tma<CH, true, true><<<persistent_grid(k_rev_f32_tma<CH, true, true>, a.n), 32 * kTmaWarps, 0, s>>>(a, err);
  else if (a.rv)
    k_rev_f32_tma<CH, true, false><<<persistent_grid(k_rev_f32_tma<CH, true, false>, a.n), 32 * kTmaWarps, 0, s>>>(a, err);
  else
    k_rev_f32_tma<CH, false, true><<<persistent_grid(k_rev_f32_tma<CH, false, true>, a.n), 32 * kTmaWarps, 0, s>>>(a, err);
}

void launch_wait_selftest(int* err, unsigned polls, cudaStream_t s) {
  k_wait_selftest<<<1, 32, 0, s>>>(err, polls);
  MFT_LAUNCH_CHECK();
}

bool launch_fwd_f32_tma(const FwdArgs& args, int chunk, int* err, cudaStream_t s) {
  if (args.V != 4 || args.n <= 0) return false;
  FwdArgs a = args;
  a.gm1_32 = (float)(a.gamma - 1.0);
  a.hg32 = (float)a.hv_gamma;
  if (chunk <= 4) fwd_tma<4>(a, err, s);
  else fwd_tma<8>(a, err, s);
  MFT_LAUNCH_CHECK();
  return true;
}

bool launch_rev_f32_tma(const RevArgs& args, int chunk, int* err, cudaStream_t s) {
  if (args.V != 4 || args.n <= 0 || (!args.rv && !args.lap)) return false;
  RevArgs a = args;
  a.hg32 = (float)a.hv_gamma;
  if (chunk <= 4) rev_tma<4>(a, err, s);
  else rev_tma<8>(a, err, s);
  MFT_LAUNCH_CHECK();
  return true;
}

}  // namespace mft
