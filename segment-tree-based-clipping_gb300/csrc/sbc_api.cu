// sbc_api.cu -- the C ABI (include/sbclip.h): contexts, host<->device
// staging, the one-to-many driver and diagnostics.
//
// Pipeline::run follows multicore_clipping (src/clip.cpp:1415-2115): one
// segment tree over the base and every overlay, then the per-overlay loop
// (src/clip.cpp:1702-2062).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sbclip.h"
#include "sbc_pipeline.cuh"

namespace sbc {

int Pipeline::run(const double* d_bxy, int nb_, const double* d_cxy, const int* c_sizes, int k_) {
  err_.clear();
  outs_.assign(k_, OverlayOut());
  join_ready_ = 0;
  cover_count_pending_ = false;
  nb = nb_;
  k = k_;
  if (nb < 3) return fail(kEInput, "base polygon needs at least 3 vertices");
  if (k < 1 || k > 9) return fail(kEInput, "1 to 9 overlays are supported");
  for (int i = 0; i < k; ++i)
    if (c_sizes[i] < 3) return fail(kEInput, "overlay polygon needs at least 3 vertices");
  cudaEvent_t ev[8];
  if (timing)
    for (int i = 0; i < 8; ++i) cudaEventCreate(&ev[i]);
  auto mark = [&](int i) {
    if (timing) cudaEventRecord(ev[i], st_);
  };
  mark(0);
  int rc = stage_setup(d_bxy, d_cxy, c_sizes);
  // The grid stage and the first overlay's box join read only the setup's
  // arrays: they run on the side stream, issued by the side worker thread,
  // while this thread issues the tree stages on the main stream.  Each
  // thread's host reads wait for its own stream only.
  bool side_posted = false;
  int side_rc = 0;
  if (!rc) {
    if (!side_stream()) {
      rc = fail(kECuda, "side stream");
    } else {
      cudaEventRecord(ev_setup_, st_);
      side_err_.clear();
      auto side_task = [this]() {
        int r = stage_grid_boxes();
        if (!r) r = stage_grid_count();
        if (!r) r = stage_grid_fill();
        if (!r) r = stage_join(1, st2_);
        if (cudaGetLastError() != cudaSuccess && !r) r = fail(kECuda, "CUDA error in the grid stage");
        return r;
      };
      side_posted = side_.post(dev_, side_task);
      if (!side_posted) {
        // no worker thread: the same steps on this thread, before the tree
        side_rc = side_task();
        if (side_rc) rc = fail(side_rc, side_err_.empty() ? err_ : side_err_);
      } else if (profiling_on()) {
        side_rc = side_.wait();
        side_posted = false;
        if (side_rc) rc = fail(side_rc, side_err_);
      }
      // per-kernel times: while profiling, the side stream's work finishes
      // before the tree stages start, so no two launches share the GPU and
      // each launch's events time it alone
      if (profiling_on()) cudaStreamSynchronize(st2_);
    }
  }
  mark(1);
  if (!rc) rc = stage_elementary();
  mark(2);
  if (!rc) rc = stage_endlists();
  mark(3);
  if (!rc) rc = stage_cover();
  mark(4);
  if (side_posted) {
    side_rc = side_.wait();
    if (side_rc && !rc) rc = fail(side_rc, side_err_);
  }
  // the candidate stage (main stream) reads the grid and the join; on an
  // error, later work on the main stream still waits for the side stream's
  // kernels (they read this context's buffers)
  join_side();
  // a statistic, off the critical path (its kernel reads the leaf ranges)
  if (!rc) launch_cover_count();
  for (int t = 1; t <= k && !rc; ++t) rc = stage_overlay(t, outs_[t - 1]);
  mark(5);
  // the scans' error word lands with the final wait (take_tree_stats)
  unsigned* d_scan_err = scan_error_word();
  const unsigned* r_scan = d_scan_err ? rd_.get(d_scan_err, HostReads::kFlags + 1, st_) : nullptr;
  take_tree_stats();
  finish_counts();
  if (cudaGetLastError() != cudaSuccess && !rc) rc = fail(kECuda, "CUDA error in the pipeline");
  const bool scan_gave_up = r_scan ? (*r_scan != 0u && scan_error_take()) : scan_error_take();
  if (scan_gave_up && !rc) rc = fail(kEInternal, "a scan's bounded wait gave up");
  if (timing) {
    cudaEventSynchronize(ev[5]);
    for (int i = 0; i < 5; ++i) cudaEventElapsedTime(&times.ms[i], ev[i], ev[i + 1]);
    cudaEventElapsedTime(&times.ms[7], ev[0], ev[5]);
    for (int i = 0; i < 8; ++i) cudaEventDestroy(ev[i]);
  }
  return rc;
}

int Pipeline::run_from_hits(const double* d_bxy, int nb_, const double* d_cxy, int nc,
                            const int* rb, const int* rc, const int* rt,
                            const unsigned long long* rkey, long long nhits) {
  err_.clear();
  outs_.assign(1, OverlayOut());
  nb = nb_;
  k = 1;
  if (nb < 3 || nc < 3) return fail(kEInput, "polygons need at least 3 vertices");
  const int sizes[1] = {nc};
  int rc0 = stage_setup(d_bxy, d_cxy, sizes);
  // the setup's non-finite check (run() reads it with the elementary counts)
  if (!rc0 && (read_flags() & kFlagUndef)) rc0 = fail(kEInput, "non-finite vertex coordinate");
  if (!rc0) rc0 = stage_records(1, rb, rc, rt, rkey, nhits, outs_[0], true);
  finish_counts();
  if (cudaGetLastError() != cudaSuccess && !rc0) rc0 = fail(kECuda, "CUDA error in the pipeline");
  if (scan_error_take() && !rc0) rc0 = fail(kEInternal, "a scan's bounded wait gave up");
  return rc0;
}

}  // namespace sbc

using sbc::Pipeline;

struct sbc_ctx {
  int device = 0;
  int flags = 0;
  cudaStream_t own = nullptr;
  Pipeline* pl = nullptr;
  std::string err;
  // host staging (pinned)
  std::vector<int*> h_off;
  std::vector<double*> h_xy;
  std::vector<size_t> h_off_cap, h_xy_cap;
  double* d_in = nullptr;
  size_t d_in_cap = 0;
  long long stats[SBC_STAT_NUM] = {0};
  sbc::BatchRunner* br = nullptr;
  sbc::PairwiseRunner* pw = nullptr;
  // host copies of batched ring results (offsets and coordinates pinned and
  // only grown: nothing is filled before the copies land)
  std::vector<long long> hb_pair_ring;
  long long* hb_ring_off = nullptr;
  size_t hb_ring_off_cap = 0;
  double* hb_xy = nullptr;
  size_t hb_xy_cap = 0;
  std::vector<int> hb_status;
  std::vector<int> hc_off;  // sbc_clip_components: ring offsets as int
  float phase_ms[8] = {0};
};

namespace {

int set_err(sbc_ctx* c, int code, const std::string& m) {
  if (c) c->err = m;
  return code;
}

int cuda_check(sbc_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return SBC_OK;
  return set_err(c, SBC_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
bool ensure_pinned(T*& p, size_t& cap, size_t n) {
  if (cap >= n && p) return true;
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
  size_t want = n + n / 8 + 16;
  if (cudaMallocHost((void**)&p, want * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    p = nullptr;
    return false;
  }
  cap = want;
  return true;
}

void fill_stats(sbc_ctx* c) {
  Pipeline& pl = *c->pl;
  for (auto& s : c->stats) s = 0;
  c->stats[SBC_STAT_EDGES] = pl.stat_edges;
  c->stats[SBC_STAT_ELEMENTARY_POINTS] = pl.stat_epc;
  c->stats[SBC_STAT_TREE_SIZE] = pl.stat_ts;
  c->stats[SBC_STAT_COVER_ENTRIES] = pl.stat_cover;
  c->stats[SBC_STAT_LEAF_END_ENTRIES] = pl.stat_leaf;
  c->stats[SBC_STAT_VERTEX_SORT] = pl.stat_vertex_sort;
  c->stats[SBC_STAT_OUTSIDE_CMBR] = pl.stat_outside_cmbr;
  if (!pl.outputs().empty()) {
    const auto& o = pl.outputs()[0];
    c->stats[SBC_STAT_CANDIDATES_TESTED] = o.tests;
    c->stats[SBC_STAT_RAW_HITS] = o.raw_hits;
    c->stats[SBC_STAT_UNIQUE] = o.unique;
    c->stats[SBC_STAT_SLOTS_B] = o.slots_b;
    c->stats[SBC_STAT_SLOTS_C] = o.slots_c;
    c->stats[SBC_STAT_WORK_UNITS] = o.work;
    c->stats[SBC_STAT_GRID_PAIRS] = o.survivors;
    int slow = 0;
    for (const auto& x : pl.outputs()) slow |= x.slow_path;
    c->stats[SBC_STAT_SERIAL_BACKEND] = slow;
  }
}

int run_device(sbc_ctx* c, const double* d_b, int nb, const double* d_c, const int* sizes, int k,
               cudaStream_t st) {
  Pipeline& pl = *c->pl;
  pl.set_stream(st);
  pl.timing = (c->flags & SBC_FLAG_TIMING) != 0;
  pl.force_serial_backend = (c->flags & SBC_FLAG_SERIAL_BACKEND) ? 1 : 0;
  pl.force_endpoint_sort = (c->flags & SBC_FLAG_ENDPOINT_SORT) ? 1 : 0;
  pl.force_wide_vertex_sort = (c->flags & SBC_FLAG_WIDE_VERTEX_SORT) ? 1 : 0;
  int rc = pl.run(d_b, nb, d_c, sizes, k);
  if (rc) return set_err(c, rc, pl.error());
  fill_stats(c);
  for (int i = 0; i < 8; ++i) c->phase_ms[i] = pl.times.ms[i];
  return SBC_OK;
}

}  // namespace

extern "C" {

int sbc_create(const sbc_options* opt, sbc_ctx** out) {
  if (!out) return SBC_EINPUT;
  *out = nullptr;
  sbc_ctx* c = new (std::nothrow) sbc_ctx();
  if (!c) return SBC_ENOMEM;
  c->device = opt ? opt->device : 0;
  c->flags = opt ? opt->flags : 0;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    int rc = cuda_check(c, e, "sbc_create");
    delete c;
    return rc;
  }
  c->pl = new Pipeline(c->device, c->own);
  c->br = new sbc::BatchRunner(*c->pl);
  c->pw = new sbc::PairwiseRunner(*c->pl);
  c->pl->unite = (c->flags & SBC_FLAG_UNION) != 0;
  c->br->unite = c->pl->unite;
  *out = c;
  return SBC_OK;
}

void sbc_destroy(sbc_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->own) cudaStreamSynchronize(c->own);
  delete c->br;
  delete c->pw;
  delete c->pl;
  for (auto p : c->h_off)
    if (p) cudaFreeHost(p);
  for (auto p : c->h_xy)
    if (p) cudaFreeHost(p);
  if (c->hb_ring_off) cudaFreeHost(c->hb_ring_off);
  if (c->hb_xy) cudaFreeHost(c->hb_xy);
  if (c->d_in) cudaFree(c->d_in);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
}

const char* sbc_last_error(const sbc_ctx* c) { return c ? c->err.c_str() : "null context"; }

int sbc_clip_one_to_many(sbc_ctx* c, const double* b_xy, int nb, const double* c_xy,
                         const int* c_sizes, int k, sbc_rings* out, void* stream) {
  if (!c || !b_xy || !c_xy || !c_sizes || !out) return set_err(c, SBC_EINPUT, "null argument");
  if (k < 1 || k > 9) return set_err(c, SBC_EINPUT, "1 to 9 overlays are supported");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  long long ncv = 0;
  for (int i = 0; i < k; ++i) {
    if (c_sizes[i] < 3) return set_err(c, SBC_EINPUT, "overlay needs at least 3 vertices");
    ncv += c_sizes[i];
  }
  if (nb < 3) return set_err(c, SBC_EINPUT, "base needs at least 3 vertices");
  size_t nin = 2 * ((size_t)nb + (size_t)ncv);
  if (c->d_in_cap < nin) {
    if (c->d_in) cudaFree(c->d_in);
    c->d_in = nullptr;
    c->d_in_cap = 0;
    if (cudaMalloc(&c->d_in, nin * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      return set_err(c, SBC_ENOMEM, "device input staging");
    }
    c->d_in_cap = nin;
  }
  // Copy straight from the caller's buffers: on a Grace host the copy engine
  // reads pageable memory over NVLink-C2C as fast as pinned memory, so a
  // host-side copy into pinned staging would only add a CPU memcpy.
  int rc = cuda_check(c, cudaMemcpyAsync(c->d_in, b_xy, sizeof(double) * 2 * nb,
                                         cudaMemcpyHostToDevice, st),
                      "input copy");
  if (!rc)
    rc = cuda_check(c, cudaMemcpyAsync(c->d_in + 2 * nb, c_xy, sizeof(double) * 2 * ncv,
                                       cudaMemcpyHostToDevice, st),
                    "input copy");
  if (rc) return rc;
  rc = run_device(c, c->d_in, nb, c->d_in + 2 * nb, c_sizes, k, st);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  if (c->flags & SBC_FLAG_TIMING) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
  }
  const auto& outs = c->pl->outputs();
  c->h_off.resize(k, nullptr);
  c->h_xy.resize(k, nullptr);
  c->h_off_cap.resize(k, 0);
  c->h_xy_cap.resize(k, 0);
  for (int i = 0; i < k; ++i) {
    const auto& o = outs[i];
    if (!ensure_pinned(c->h_off[i], c->h_off_cap[i], (size_t)o.nrings + 1) ||
        !ensure_pinned(c->h_xy[i], c->h_xy_cap[i], 2 * (size_t)o.nverts + 2))
      return set_err(c, SBC_ENOMEM, "pinned result buffers");
    c->h_off[i][0] = 0;
    if (o.nrings > 0)
      cudaMemcpyAsync(c->h_off[i], o.d_off, sizeof(int) * (o.nrings + 1), cudaMemcpyDeviceToHost,
                      st);
    if (o.nverts > 0)
      cudaMemcpyAsync(c->h_xy[i], o.d_xy, sizeof(double) * 2 * o.nverts, cudaMemcpyDeviceToHost,
                      st);
  }
  rc = cuda_check(c, cudaStreamSynchronize(st), "result copy");
  if (rc) return rc;
  if (c->flags & SBC_FLAG_TIMING) {
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&c->phase_ms[6], e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  for (int i = 0; i < k; ++i) {
    out[i].nrings = outs[i].nrings;
    out[i].nverts = outs[i].nverts;
    out[i].offsets = c->h_off[i];
    out[i].xy = c->h_xy[i];
  }
  return SBC_OK;
}

int sbc_clip_pair(sbc_ctx* c, const double* b_xy, int nb, const double* c_xy, int nc,
                  sbc_rings* out, void* stream) {
  int sizes[1] = {nc};
  return sbc_clip_one_to_many(c, b_xy, nb, c_xy, sizes, 1, out, stream);
}

int sbc_clip_pair_device(sbc_ctx* c, const double* d_b, int nb, const double* d_c, int nc,
                         sbc_rings* out, void* stream) {
  if (!c || !d_b || !d_c || !out) return set_err(c, SBC_EINPUT, "null argument");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  int sizes[1] = {nc};
  int rc = run_device(c, d_b, nb, d_c, sizes, 1, st);
  if (rc) return rc;
  const auto& o = c->pl->outputs()[0];
  out->nrings = o.nrings;
  out->nverts = o.nverts;
  out->offsets = o.d_off;
  out->xy = o.d_xy;
  return SBC_OK;
}

int sbc_stats(const sbc_ctx* c, long long* out, int n) {
  if (!c || !out) return SBC_EINPUT;
  for (int i = 0; i < n && i < SBC_STAT_NUM; ++i) out[i] = c->stats[i];
  return SBC_OK;
}

int sbc_phase_times(const sbc_ctx* c, float* out, int n) {
  if (!c || !out) return SBC_EINPUT;
  for (int i = 0; i < n && i < 8; ++i) out[i] = c->phase_ms[i];
  return SBC_OK;
}

int sbc_debug_array(sbc_ctx* c, int which, void* dst, long long cap, long long* count) {
  if (!c || !count) return set_err(c, SBC_EINPUT, "null argument");
  Pipeline& p = *c->pl;
  const void* src = nullptr;
  long long n = 0;
  size_t es = sizeof(int);
  switch (which) {
    case SBC_ARR_UNIQ_B: src = p.dbg_ub; n = p.dbg_K; break;
    case SBC_ARR_UNIQ_C: src = p.dbg_uc; n = p.dbg_K; break;
    case SBC_ARR_UNIQ_T: src = p.dbg_ut; n = p.dbg_K; break;
    case SBC_ARR_ISECT_XY: src = p.dbg_isxy; n = 2LL * p.dbg_K; es = sizeof(double); break;
    case SBC_ARR_ISECT_AB: src = p.dbg_aB; n = p.dbg_K; break;
    case SBC_ARR_ISECT_AC: src = p.dbg_aC; n = p.dbg_K; break;
    case SBC_ARR_MERGED_BXY: src = p.dbg_ixB; n = 2LL * p.dbg_nB; es = sizeof(double); break;
    case SBC_ARR_MERGED_CXY: src = p.dbg_ixC; n = 2LL * p.dbg_nQ; es = sizeof(double); break;
    case SBC_ARR_MERGED_BALPHA: src = p.dbg_alB; n = p.dbg_nB; break;
    case SBC_ARR_MERGED_CALPHA: src = p.dbg_alC; n = p.dbg_nQ; break;
    case SBC_ARR_MERGED_BNB: src = p.dbg_nbB; n = p.dbg_nB; break;
    case SBC_ARR_MERGED_CNB: src = p.dbg_nbC; n = p.dbg_nQ; break;
    case SBC_ARR_LABEL_B: src = p.dbg_labB; n = p.dbg_nB; break;
    case SBC_ARR_LABEL_C: src = p.dbg_labC; n = p.dbg_nQ; break;
    case SBC_ARR_ELEMENTARY: src = p.ea; n = p.epc; es = sizeof(double); break;
    case SBC_ARR_LEAF_AFTER: src = p.aft; n = p.E; break;
    case SBC_ARR_LEAF_BEFORE: src = p.bef; n = p.E; break;
    case SBC_ARR_LEAF_RANGE: src = p.lr; n = 2LL * p.E; break;
    default: return set_err(c, SBC_EINPUT, "unknown array");
  }
  if (!src) n = 0;  // not produced by the last call
  *count = n;
  long long m = n < cap ? n : cap;
  if (dst && src && m > 0) {
    cudaStream_t st = c->pl->stream();
    int rc = cuda_check(c, cudaMemcpyAsync(dst, src, es * m, cudaMemcpyDeviceToHost, st), "debug");
    if (rc) return rc;
    return cuda_check(c, cudaStreamSynchronize(st), "debug");
  }
  return SBC_OK;
}

unsigned long long sbc_kernel_launches(void) { return sbc::g_launches; }

int sbc_profile_begin(void) {
  sbc::profile_begin();
  return SBC_OK;
}

int sbc_profile_end(char* names, int names_len, float* ms, int* counts, double* bytes, int cap,
                    int* n_out) {
  std::vector<std::string> nm;
  std::vector<float> t;
  std::vector<int> c;
  std::vector<double> by;
  int n = sbc::profile_end(&nm, &t, &c, &by);
  if (n_out) *n_out = n;
  int w = 0;
  for (int i = 0; i < n && i < cap; ++i) {
    if (ms) ms[i] = t[i];
    if (counts) counts[i] = c[i];
    if (bytes) bytes[i] = by[i];
    if (names) {
      int need = (int)nm[i].size() + 1;
      if (w + need <= names_len) {
        memcpy(names + w, nm[i].c_str(), need);
        w += need;
      }
    }
  }
  return SBC_OK;
}

int sbc_profile_timeline(char* names, int names_len, float* start_ms, float* dur_ms, int* stream,
                         int cap, int* n_out) {
  const auto& tl = sbc::profile_timeline();
  const int n = (int)tl.size();
  if (n_out) *n_out = n;
  int w = 0;
  for (int i = 0; i < n && i < cap; ++i) {
    if (start_ms) start_ms[i] = tl[i].start_ms;
    if (dur_ms) dur_ms[i] = tl[i].dur_ms;
    if (stream) stream[i] = tl[i].stream;
    if (names) {
      const int need = (int)strlen(tl[i].name) + 1;
      if (w + need <= names_len) {
        memcpy(names + w, tl[i].name, need);
        w += need;
      }
    }
  }
  return SBC_OK;
}

const char* sbc_version(void) { return "sbclip-gb300 0.1 (sm_103a)"; }

}  // extern "C"

// ---------------------------------------------------------------- classifier
namespace {
__global__ void k_classify(const double* __restrict__ pairs, int n, int* __restrict__ types,
                           double* __restrict__ alpha, double* __restrict__ beta,
                           int* __restrict__ ai, int* __restrict__ bi) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* p = pairs + 8 * (size_t)i;
  double a = 0.0, b = 0.0;
  int t = sbc::seg_isect(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], &a, &b);
  types[i] = t;
  alpha[i] = a;
  beta[i] = b;
  ai[i] = t ? sbc::alpha_to_int(a) : 0;
  bi[i] = t ? sbc::alpha_to_int(b) : 0;
}
}  // namespace

extern "C" int sbc_classify_pairs(sbc_ctx* c, const double* pairs, int n, int* types,
                                  double* alpha, double* beta, int* alpha_int, int* beta_int) {
  if (!c || (!pairs && n > 0)) return set_err(c, SBC_EINPUT, "null argument");
  if (n <= 0) return SBC_OK;
  cudaSetDevice(c->device);
  cudaStream_t st = c->own;
  sbc::BufferPool& bp = c->pl->pool();
  double* dp = (double*)bp.get("cls_pairs", sizeof(double) * 8 * (size_t)n);
  int* dt = (int*)bp.get("cls_t", sizeof(int) * n);
  double* da = (double*)bp.get("cls_a", sizeof(double) * n);
  double* db = (double*)bp.get("cls_b", sizeof(double) * n);
  int* dai = (int*)bp.get("cls_ai", sizeof(int) * n);
  int* dbi = (int*)bp.get("cls_bi", sizeof(int) * n);
  if (bp.failed) return set_err(c, SBC_ENOMEM, "device allocation failed (classifier)");
  cudaMemcpyAsync(dp, pairs, sizeof(double) * 8 * (size_t)n, cudaMemcpyHostToDevice, st);
  {
    ::sbc::KProbe kp_("k_classify", st);
    k_classify<<<sbc::grid_for(n, 256), 256, 0, st>>>(dp, n, dt, da, db, dai, dbi);
  }
  if (types) cudaMemcpyAsync(types, dt, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
  if (alpha) cudaMemcpyAsync(alpha, da, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
  if (beta) cudaMemcpyAsync(beta, db, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
  if (alpha_int) cudaMemcpyAsync(alpha_int, dai, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
  if (beta_int) cudaMemcpyAsync(beta_int, dbi, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
  return cuda_check(c, cudaStreamSynchronize(st), "classifier");
}

// ------------------------------------------------------------------ batches
namespace {

int batch_check(sbc_ctx* c, const sbc_batch* b) {
  if (!c || !b) return set_err(c, SBC_EINPUT, "null argument");
  if (b->npairs < 0) return set_err(c, SBC_EINPUT, "negative pair count");
  if (b->npairs > 0 && (!b->b_xy || !b->b_off || !b->c_xy || !b->c_off))
    return set_err(c, SBC_EINPUT, "null batch array");
  return SBC_OK;
}

// host batch -> device copies in the context's pool
int batch_to_device(sbc_ctx* c, const sbc_batch* b, cudaStream_t st, sbc_batch* d) {
  const int np = b->npairs;
  *d = *b;
  if (np == 0) return SBC_OK;
  const long long nbv = b->b_off[np], ncv = b->c_off[np];
  if (b->b_off[0] != 0 || b->c_off[0] != 0 || nbv < 0 || ncv < 0)
    return set_err(c, SBC_EINPUT, "batch offsets must start at 0");
  sbc::BufferPool& bp = c->pl->pool();
  auto* dbx = (double*)bp.get("hbt_bxy", sizeof(double) * 2 * (nbv + 1));
  auto* dcx = (double*)bp.get("hbt_cxy", sizeof(double) * 2 * (ncv + 1));
  auto* dbo = (long long*)bp.get("hbt_boff", sizeof(long long) * (np + 1));
  auto* dco = (long long*)bp.get("hbt_coff", sizeof(long long) * (np + 1));
  if (bp.failed) return set_err(c, SBC_ENOMEM, "device allocation failed (batch inputs)");
  cudaMemcpyAsync(dbx, b->b_xy, sizeof(double) * 2 * nbv, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dcx, b->c_xy, sizeof(double) * 2 * ncv, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dbo, b->b_off, sizeof(long long) * (np + 1), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dco, b->c_off, sizeof(long long) * (np + 1), cudaMemcpyHostToDevice, st);
  d->b_xy = dbx;
  d->c_xy = dcx;
  d->b_off = dbo;
  d->c_off = dco;
  return SBC_OK;
}

// dk: the batch's component offsets on the device (null: one ring per
// polygon), nbv / ncv their vertex totals
int batch_run(sbc_ctx* c, const sbc_batch* d, cudaStream_t st,
              const sbc_components* dk = nullptr, long long nbv = 0, long long ncv = 0) {
  c->pl->clear_error();
  c->pl->set_stream(st);
  int rc = c->br->set_components(d->npairs, d->b_off, d->c_off, dk ? dk->b_comp : nullptr,
                                 dk ? dk->nb_comp : 0, dk ? dk->c_comp : nullptr,
                                 dk ? dk->nc_comp : 0, nbv, ncv, st);
  if (!rc) rc = c->br->forward(d->npairs, d->b_xy, d->b_off, d->c_xy, d->c_off, st);
  if (rc) return set_err(c, rc, c->pl->error());
  return SBC_OK;
}

// One side's component offsets (host): 0 = comp[0] < ... < comp[n] = off[np],
// at least 3 vertices per component, every non-empty polygon starting one
// (so no component spans two pairs).
int comps_check(sbc_ctx* c, const long long* comp, long long n, const long long* off, int np) {
  if (!comp) return SBC_OK;
  if (n < 1 || comp[0] != 0 || comp[n] != off[np])
    return set_err(c, SBC_EINPUT, "component offsets must run from 0 to the vertex count");
  for (long long i = 0; i < n; ++i)
    if (comp[i + 1] - comp[i] < 3)
      return set_err(c, SBC_EINPUT, "a component needs at least 3 vertices");
  long long i = 0;
  for (int p = 0; p < np; ++p) {
    if (off[p + 1] <= off[p]) continue;
    while (i < n && comp[i] < off[p]) ++i;
    if (i >= n || comp[i] != off[p])
      return set_err(c, SBC_EINPUT, "every polygon must start a component");
  }
  return SBC_OK;
}

// The components of a batch checked on the host; hb / hk: host copies of the
// batch offsets and the component offsets (read back for _device calls).
// d receives device component offsets.
int comps_prepare(sbc_ctx* c, const sbc_batch* b, const sbc_components* k, bool device,
                  cudaStream_t st, sbc_components* d, long long* nbv, long long* ncv) {
  if (!k) return set_err(c, SBC_EINPUT, "null components");
  const int np = b->npairs;
  *d = *k;
  std::vector<long long> boff(np + 1), coff(np + 1), bc, cc;
  const long long *hbo = b->b_off, *hco = b->c_off, *hbc = k->b_comp, *hcc = k->c_comp;
  if (device) {
    cudaMemcpyAsync(boff.data(), b->b_off, sizeof(long long) * (np + 1), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(coff.data(), b->c_off, sizeof(long long) * (np + 1), cudaMemcpyDeviceToHost, st);
    if (k->b_comp && k->nb_comp >= 0) {
      bc.resize(k->nb_comp + 1);
      cudaMemcpyAsync(bc.data(), k->b_comp, sizeof(long long) * bc.size(), cudaMemcpyDeviceToHost, st);
    }
    if (k->c_comp && k->nc_comp >= 0) {
      cc.resize(k->nc_comp + 1);
      cudaMemcpyAsync(cc.data(), k->c_comp, sizeof(long long) * cc.size(), cudaMemcpyDeviceToHost, st);
    }
    int rc = cuda_check(c, cudaStreamSynchronize(st), "component offsets");
    if (rc) return rc;
    hbo = boff.data();
    hco = coff.data();
    hbc = k->b_comp ? bc.data() : nullptr;
    hcc = k->c_comp ? cc.data() : nullptr;
  }
  int rc = comps_check(c, hbc, k->nb_comp, hbo, np);
  if (!rc) rc = comps_check(c, hcc, k->nc_comp, hco, np);
  if (rc) return rc;
  *nbv = hbo[np];
  *ncv = hco[np];
  if (!device) {
    sbc::BufferPool& bp = c->pl->pool();
    auto* db = k->b_comp ? (long long*)bp.get("hbt_bcomp", sizeof(long long) * (k->nb_comp + 1))
                         : nullptr;
    auto* dc = k->c_comp ? (long long*)bp.get("hbt_ccomp", sizeof(long long) * (k->nc_comp + 1))
                         : nullptr;
    if (bp.failed) return set_err(c, SBC_ENOMEM, "device allocation failed (components)");
    if (db)
      cudaMemcpyAsync(db, k->b_comp, sizeof(long long) * (k->nb_comp + 1), cudaMemcpyHostToDevice, st);
    if (dc)
      cudaMemcpyAsync(dc, k->c_comp, sizeof(long long) * (k->nc_comp + 1), cudaMemcpyHostToDevice, st);
    d->b_comp = db;
    d->c_comp = dc;
  }
  return SBC_OK;
}

}  // namespace

extern "C" int sbc_area_forward_device(sbc_ctx* c, const sbc_batch* b, double* area, int* status,
                                       void* stream) {
  int rc = batch_check(c, b);
  if (rc) return rc;
  if (b->npairs > 0 && !area) return set_err(c, SBC_EINPUT, "null area output");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  rc = batch_run(c, b, st);
  if (rc) return rc;
  const int np = b->npairs;
  if (np > 0) {
    cudaMemcpyAsync(area, c->br->area, sizeof(double) * np, cudaMemcpyDeviceToDevice, st);
    if (status)
      cudaMemcpyAsync(status, c->br->status, sizeof(int) * np, cudaMemcpyDeviceToDevice, st);
  }
  return cuda_check(c, cudaStreamSynchronize(st), "area forward");
}

extern "C" int sbc_area_forward(sbc_ctx* c, const sbc_batch* b, double* area, int* status,
                                void* stream) {
  int rc = batch_check(c, b);
  if (rc) return rc;
  if (b->npairs > 0 && !area) return set_err(c, SBC_EINPUT, "null area output");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  sbc_batch d;
  rc = batch_to_device(c, b, st, &d);
  if (rc) return rc;
  rc = batch_run(c, &d, st);
  if (rc) return rc;
  const int np = b->npairs;
  if (np > 0) {
    cudaMemcpyAsync(area, c->br->area, sizeof(double) * np, cudaMemcpyDeviceToHost, st);
    if (status) cudaMemcpyAsync(status, c->br->status, sizeof(int) * np, cudaMemcpyDeviceToHost, st);
  }
  return cuda_check(c, cudaStreamSynchronize(st), "area forward");
}

extern "C" int sbc_area_backward_device(sbc_ctx* c, const sbc_batch* b, const double* grad_area,
                                        double* grad_b, double* grad_c, void* stream) {
  int rc = batch_check(c, b);
  if (rc) return rc;
  if (b->npairs > 0 && (!grad_area || !grad_b || !grad_c))
    return set_err(c, SBC_EINPUT, "null gradient array");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  if (!(c->br->valid && c->br->np == b->npairs && c->br->key_b == b->b_xy &&
        c->br->key_c == b->c_xy && !c->br->key_bcomp && !c->br->key_ccomp)) {
    rc = batch_run(c, b, st);
    if (rc) return rc;
  }
  c->pl->clear_error();
  rc = c->br->backward(b->b_xy, b->b_off, b->c_xy, b->c_off, grad_area, grad_b, grad_c, st);
  if (rc) return set_err(c, rc, c->pl->error());
  return SBC_OK;
}

extern "C" int sbc_area_backward(sbc_ctx* c, const sbc_batch* b, const double* grad_area,
                                 double* grad_b, double* grad_c, void* stream) {
  int rc = batch_check(c, b);
  if (rc) return rc;
  const int np = b->npairs;
  if (np > 0 && (!grad_area || !grad_b || !grad_c))
    return set_err(c, SBC_EINPUT, "null gradient array");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  sbc_batch d;
  rc = batch_to_device(c, b, st, &d);
  if (rc) return rc;
  rc = batch_run(c, &d, st);
  if (rc) return rc;
  if (np == 0) return SBC_OK;
  const long long nbv = b->b_off[np], ncv = b->c_off[np];
  sbc::BufferPool& bp = c->pl->pool();
  auto* dga = (double*)bp.get("hbt_ga", sizeof(double) * (np + 1));
  auto* dgb = (double*)bp.get("hbt_gb", sizeof(double) * 2 * (nbv + 1));
  auto* dgc = (double*)bp.get("hbt_gc", sizeof(double) * 2 * (ncv + 1));
  if (bp.failed) return set_err(c, SBC_ENOMEM, "device allocation failed (gradients)");
  cudaMemcpyAsync(dga, grad_area, sizeof(double) * np, cudaMemcpyHostToDevice, st);
  c->pl->clear_error();
  rc = c->br->backward(d.b_xy, d.b_off, d.c_xy, d.c_off, dga, dgb, dgc, st);
  if (rc) return set_err(c, rc, c->pl->error());
  cudaMemcpyAsync(grad_b, dgb, sizeof(double) * 2 * nbv, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(grad_c, dgc, sizeof(double) * 2 * ncv, cudaMemcpyDeviceToHost, st);
  return cuda_check(c, cudaStreamSynchronize(st), "area backward");
}

extern "C" int sbc_clip_batch_device(sbc_ctx* c, const sbc_batch* b, sbc_batch_rings* out,
                                     void* stream) {
  int rc = batch_check(c, b);
  if (rc) return rc;
  if (!out) return set_err(c, SBC_EINPUT, "null output");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  rc = batch_run(c, b, st);
  if (rc) return rc;
  long long *pr = nullptr, *ro = nullptr;
  double* xy = nullptr;
  long long nr = 0, nv = 0;
  if (b->npairs > 0) {
    c->pl->clear_error();
    rc = c->br->rings(b->b_xy, b->b_off, b->c_xy, b->c_off, st, &pr, &ro, &xy, &nr, &nv);
    if (rc) return set_err(c, rc, c->pl->error());
  }
  out->npairs = b->npairs;
  out->nrings = nr;
  out->nverts = nv;
  out->pair_ring = pr;
  out->ring_off = ro;
  out->xy = xy;
  out->status = c->br->status;
  return SBC_OK;
}

extern "C" int sbc_clip_batch(sbc_ctx* c, const sbc_batch* b, sbc_batch_rings* out, void* stream) {
  int rc = batch_check(c, b);
  if (rc) return rc;
  if (!out) return set_err(c, SBC_EINPUT, "null output");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  sbc_batch d;
  rc = batch_to_device(c, b, st, &d);
  if (rc) return rc;
  sbc_batch_rings dr;
  rc = sbc_clip_batch_device(c, &d, &dr, st);
  if (rc) return rc;
  const int np = b->npairs;
  c->hb_pair_ring.assign((size_t)np + 1, 0);
  c->hb_status.assign((size_t)np + 1, 0);
  if (!ensure_pinned(c->hb_ring_off, c->hb_ring_off_cap, (size_t)dr.nrings + 1) ||
      !ensure_pinned(c->hb_xy, c->hb_xy_cap, (size_t)2 * dr.nverts + 1))
    return set_err(c, SBC_ENOMEM, "pinned host allocation failed (batch rings)");
  c->hb_ring_off[0] = 0;
  if (np > 0) {
    cudaMemcpyAsync(c->hb_pair_ring.data(), dr.pair_ring, sizeof(long long) * (np + 1),
                    cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(c->hb_ring_off, dr.ring_off, sizeof(long long) * (dr.nrings + 1),
                    cudaMemcpyDeviceToHost, st);
    if (dr.nverts > 0)
      cudaMemcpyAsync(c->hb_xy, dr.xy, sizeof(double) * 2 * dr.nverts, cudaMemcpyDeviceToHost,
                      st);
    cudaMemcpyAsync(c->hb_status.data(), dr.status, sizeof(int) * np, cudaMemcpyDeviceToHost, st);
  }
  rc = cuda_check(c, cudaStreamSynchronize(st), "batch rings");
  if (rc) return rc;
  out->npairs = np;
  out->nrings = dr.nrings;
  out->nverts = dr.nverts;
  out->pair_ring = c->hb_pair_ring.data();
  out->ring_off = c->hb_ring_off;
  out->xy = c->hb_xy;
  out->status = c->hb_status.data();
  return SBC_OK;
}

// ------------------------------------------------------------------ components
extern "C" int sbc_clip_batch_components_device(sbc_ctx* c, const sbc_batch* b,
                                                const sbc_components* k, sbc_batch_rings* out,
                                                void* stream) {
  int rc = batch_check(c, b);
  if (rc) return rc;
  if (!out) return set_err(c, SBC_EINPUT, "null output");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  sbc_components dk;
  long long nbv = 0, ncv = 0;
  rc = comps_prepare(c, b, k, true, st, &dk, &nbv, &ncv);
  if (rc) return rc;
  rc = batch_run(c, b, st, &dk, nbv, ncv);
  if (rc) return rc;
  long long *pr = nullptr, *ro = nullptr;
  double* xy = nullptr;
  long long nr = 0, nv = 0;
  if (b->npairs > 0) {
    c->pl->clear_error();
    rc = c->br->rings(b->b_xy, b->b_off, b->c_xy, b->c_off, st, &pr, &ro, &xy, &nr, &nv);
    if (rc) return set_err(c, rc, c->pl->error());
  }
  out->npairs = b->npairs;
  out->nrings = nr;
  out->nverts = nv;
  out->pair_ring = pr;
  out->ring_off = ro;
  out->xy = xy;
  out->status = c->br->status;
  return SBC_OK;
}

extern "C" int sbc_clip_batch_components(sbc_ctx* c, const sbc_batch* b, const sbc_components* k,
                                         sbc_batch_rings* out, void* stream) {
  int rc = batch_check(c, b);
  if (rc) return rc;
  if (!out) return set_err(c, SBC_EINPUT, "null output");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  sbc_components dk;
  long long nbv = 0, ncv = 0;
  if (b->npairs > 0 && (b->b_off[0] != 0 || b->c_off[0] != 0))
    return set_err(c, SBC_EINPUT, "batch offsets must start at 0");
  rc = comps_prepare(c, b, k, false, st, &dk, &nbv, &ncv);
  if (rc) return rc;
  sbc_batch d;
  rc = batch_to_device(c, b, st, &d);
  if (rc) return rc;
  rc = batch_run(c, &d, st, &dk, nbv, ncv);
  if (rc) return rc;
  const int np = b->npairs;
  long long *pr = nullptr, *ro = nullptr;
  double* xy = nullptr;
  long long nr = 0, nv = 0;
  if (np > 0) {
    c->pl->clear_error();
    rc = c->br->rings(d.b_xy, d.b_off, d.c_xy, d.c_off, st, &pr, &ro, &xy, &nr, &nv);
    if (rc) return set_err(c, rc, c->pl->error());
  }
  c->hb_pair_ring.assign((size_t)np + 1, 0);
  c->hb_status.assign((size_t)np + 1, 0);
  if (!ensure_pinned(c->hb_ring_off, c->hb_ring_off_cap, (size_t)nr + 1) ||
      !ensure_pinned(c->hb_xy, c->hb_xy_cap, (size_t)2 * nv + 1))
    return set_err(c, SBC_ENOMEM, "pinned host allocation failed (batch rings)");
  c->hb_ring_off[0] = 0;
  if (np > 0) {
    cudaMemcpyAsync(c->hb_pair_ring.data(), pr, sizeof(long long) * (np + 1),
                    cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(c->hb_ring_off, ro, sizeof(long long) * (nr + 1), cudaMemcpyDeviceToHost, st);
    if (nv > 0) cudaMemcpyAsync(c->hb_xy, xy, sizeof(double) * 2 * nv, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(c->hb_status.data(), c->br->status, sizeof(int) * np, cudaMemcpyDeviceToHost,
                    st);
  }
  rc = cuda_check(c, cudaStreamSynchronize(st), "batch rings");
  if (rc) return rc;
  out->npairs = np;
  out->nrings = nr;
  out->nverts = nv;
  out->pair_ring = c->hb_pair_ring.data();
  out->ring_off = c->hb_ring_off;
  out->xy = c->hb_xy;
  out->status = c->hb_status.data();
  return SBC_OK;
}

extern "C" int sbc_clip_components(sbc_ctx* c, const double* b_xy, const int* b_comp, int nb_comp,
                                   const double* c_xy, const int* c_comp, int nc_comp,
                                   sbc_rings* out, void* stream) {
  if (!c) return SBC_EINPUT;
  if (!b_xy || !b_comp || !c_xy || !c_comp || !out || nb_comp < 1 || nc_comp < 1)
    return set_err(c, SBC_EINPUT, "null argument or no component");
  std::vector<long long> bk(b_comp, b_comp + nb_comp + 1), ck(c_comp, c_comp + nc_comp + 1);
  const long long boff[2] = {0, bk.back()}, coff[2] = {0, ck.back()};
  const sbc_batch b{1, b_xy, boff, c_xy, coff};
  const sbc_components k{bk.data(), nb_comp, ck.data(), nc_comp};
  sbc_batch_rings r;
  int rc = sbc_clip_batch_components(c, &b, &k, &r, stream);
  if (rc) return rc;
  if (r.status[0] != SBC_OK)
    return set_err(c, r.status[0], r.status[0] == SBC_EUNDEF
                                       ? "reference behaviour undefined for this input"
                                       : "pair failed");
  c->hc_off.resize((size_t)r.nrings + 1);
  for (long long i = 0; i <= r.nrings; ++i) c->hc_off[i] = (int)r.ring_off[i];
  out->nrings = (int)r.nrings;
  out->nverts = r.nverts;
  out->offsets = c->hc_off.data();
  out->xy = r.xy;
  return SBC_OK;
}

extern "C" int sbc_area_forward_components_device(sbc_ctx* c, const sbc_batch* b,
                                                  const sbc_components* k, double* area,
                                                  int* status, void* stream) {
  int rc = batch_check(c, b);
  if (rc) return rc;
  if (b->npairs > 0 && !area) return set_err(c, SBC_EINPUT, "null area output");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  sbc_components dk;
  long long nbv = 0, ncv = 0;
  rc = comps_prepare(c, b, k, true, st, &dk, &nbv, &ncv);
  if (rc) return rc;
  rc = batch_run(c, b, st, &dk, nbv, ncv);
  if (rc) return rc;
  const int np = b->npairs;
  if (np > 0) {
    cudaMemcpyAsync(area, c->br->area, sizeof(double) * np, cudaMemcpyDeviceToDevice, st);
    if (status)
      cudaMemcpyAsync(status, c->br->status, sizeof(int) * np, cudaMemcpyDeviceToDevice, st);
  }
  return cuda_check(c, cudaStreamSynchronize(st), "area forward");
}

extern "C" int sbc_area_backward_components_device(sbc_ctx* c, const sbc_batch* b,
                                                   const sbc_components* k,
                                                   const double* grad_area, double* grad_b,
                                                   double* grad_c, void* stream) {
  int rc = batch_check(c, b);
  if (rc) return rc;
  if (!k) return set_err(c, SBC_EINPUT, "null components");
  if (b->npairs > 0 && (!grad_area || !grad_b || !grad_c))
    return set_err(c, SBC_EINPUT, "null gradient array");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  if (!(c->br->valid && c->br->np == b->npairs && c->br->key_b == b->b_xy &&
        c->br->key_c == b->c_xy && c->br->key_bcomp == k->b_comp &&
        c->br->key_ccomp == k->c_comp)) {
    sbc_components dk;
    long long nbv = 0, ncv = 0;
    rc = comps_prepare(c, b, k, true, st, &dk, &nbv, &ncv);
    if (rc) return rc;
    rc = batch_run(c, b, st, &dk, nbv, ncv);
    if (rc) return rc;
  }
  c->pl->clear_error();
  rc = c->br->backward(b->b_xy, b->b_off, b->c_xy, b->c_off, grad_area, grad_b, grad_c, st);
  if (rc) return set_err(c, rc, c->pl->error());
  return SBC_OK;
}

// ------------------------------------------------------------------ pairwise
namespace {

int pairwise_check(sbc_ctx* c, const sbc_pairwise_job* j) {
  if (!c) return SBC_EINPUT;
  if (!j) return set_err(c, SBC_EINPUT, "null job");
  if (j->nb < 3) return set_err(c, SBC_EINPUT, "base needs at least 3 vertices");
  if (j->noverlays < 0) return set_err(c, SBC_EINPUT, "negative overlay count");
  if (!j->b_xy || (j->noverlays > 0 && (!j->c_xy || !j->c_off)))
    return set_err(c, SBC_EINPUT, "null array");
  return SBC_OK;
}

}  // namespace

extern "C" int sbc_clip_pairwise_device(sbc_ctx* c, const sbc_pairwise_job* j,
                                        sbc_batch_rings* out, void* stream) {
  int rc = pairwise_check(c, j);
  if (rc) return rc;
  if (!out) return set_err(c, SBC_EINPUT, "null output");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  c->pl->set_stream(st);
  c->pl->clear_error();
  rc = c->pw->run(j->b_xy, j->nb, j->noverlays, j->c_xy, j->c_off, st);
  if (rc) return set_err(c, rc, c->pl->error());
  out->npairs = j->noverlays;
  out->nrings = c->pw->total_rings;
  out->nverts = c->pw->total_verts;
  out->pair_ring = c->pw->pair_ring;
  out->ring_off = c->pw->ring_off;
  out->xy = c->pw->xy;
  out->status = c->pw->status;
  return SBC_OK;
}

extern "C" int sbc_clip_pairwise(sbc_ctx* c, const sbc_pairwise_job* j, sbc_batch_rings* out,
                                 void* stream) {
  int rc = pairwise_check(c, j);
  if (rc) return rc;
  if (!out) return set_err(c, SBC_EINPUT, "null output");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  const int nov = j->noverlays;
  if (nov > 0 && j->c_off[0] != 0) return set_err(c, SBC_EINPUT, "c_off[0] must be 0");
  for (int i = 0; i < nov; ++i)
    if (j->c_off[i + 1] < j->c_off[i]) return set_err(c, SBC_EINPUT, "c_off must not decrease");
  const long long ncv = nov > 0 ? j->c_off[nov] : 0;
  sbc::BufferPool& bp = c->pl->pool();
  auto* db = (double*)bp.get("hpw_b", sizeof(double) * 2 * j->nb);
  auto* dc = (double*)bp.get("hpw_c", sizeof(double) * 2 * (ncv + 1));
  auto* dco = (long long*)bp.get("hpw_coff", sizeof(long long) * (nov + 1));
  if (bp.failed) return set_err(c, SBC_ENOMEM, "device allocation failed (pairwise input)");
  // straight from the caller's buffers (pageable copies run at pinned speed on Grace)
  cudaMemcpyAsync(db, j->b_xy, sizeof(double) * 2 * j->nb, cudaMemcpyHostToDevice, st);
  if (ncv > 0) cudaMemcpyAsync(dc, j->c_xy, sizeof(double) * 2 * ncv, cudaMemcpyHostToDevice, st);
  if (nov > 0)
    cudaMemcpyAsync(dco, j->c_off, sizeof(long long) * (nov + 1), cudaMemcpyHostToDevice, st);
  sbc_pairwise_job d{db, j->nb, nov, dc, dco};
  sbc_batch_rings dr;
  rc = sbc_clip_pairwise_device(c, &d, &dr, st);
  if (rc) return rc;
  if (!ensure_pinned(c->hb_ring_off, c->hb_ring_off_cap, (size_t)dr.nrings + 1) ||
      !ensure_pinned(c->hb_xy, c->hb_xy_cap, (size_t)2 * dr.nverts + 1))
    return set_err(c, SBC_ENOMEM, "pinned host allocation failed (pairwise rings)");
  c->hb_ring_off[0] = 0;
  c->hb_pair_ring = c->pw->h_pair_ring;
  c->hb_status = c->pw->h_status;
  c->hb_pair_ring.resize((size_t)nov + 1, 0);
  c->hb_status.resize((size_t)nov + 1, 0);
  if (nov > 0) {
    cudaMemcpyAsync(c->hb_ring_off, dr.ring_off, sizeof(long long) * (dr.nrings + 1),
                    cudaMemcpyDeviceToHost, st);
    if (dr.nverts > 0)
      cudaMemcpyAsync(c->hb_xy, dr.xy, sizeof(double) * 2 * dr.nverts, cudaMemcpyDeviceToHost,
                      st);
  }
  rc = cuda_check(c, cudaStreamSynchronize(st), "pairwise rings");
  if (rc) return rc;
  out->npairs = nov;
  out->nrings = dr.nrings;
  out->nverts = dr.nverts;
  out->pair_ring = c->hb_pair_ring.data();
  out->ring_off = c->hb_ring_off;
  out->xy = c->hb_xy;
  out->status = c->hb_status.data();
  return SBC_OK;
}

extern "C" int sbc_pairwise_info(const sbc_ctx* c, long long* out, int n) {
  if (!c || !out) return SBC_EINPUT;
  const long long v[5] = {c->pw->fallback_pairs, c->pw->hits, c->pw->tested, c->pw->grid_cells,
                          c->pw->big_pairs};
  for (int i = 0; i < n && i < 5; ++i) out[i] = v[i];
  return SBC_OK;
}

extern "C" int sbc_pairwise_set_cell_factor(sbc_ctx* c, double f) {
  if (!c) return SBC_EINPUT;
  if (!(f > 0.0) || f > 1e6) return set_err(c, SBC_EINPUT, "cell factor must be positive");
  c->pw->cell_factor = f;
  return SBC_OK;
}

extern "C" int sbc_pairwise_set_split(sbc_ctx* c, int records) {
  if (!c) return SBC_EINPUT;
  if (records < 1) return set_err(c, SBC_EINPUT, "split must be at least 1 record");
  c->pw->big_k = records;
  return SBC_OK;
}

extern "C" int sbc_pairwise_set_workers(sbc_ctx* c, int workers) {
  if (!c) return SBC_EINPUT;
  if (workers < 1 || workers > 64) return set_err(c, SBC_EINPUT, "workers must be 1 to 64");
  c->pw->big_workers = workers;
  return SBC_OK;
}

extern "C" int sbc_pairwise_get_workers(const sbc_ctx* c) { return c ? c->pw->big_workers : -1; }

extern "C" int sbc_pairwise_autotune(sbc_ctx* c, const sbc_pairwise_job* j, int* split,
                                     double* cell_factor, double* best_ms, void* stream) {
  int rc = pairwise_check(c, j);
  if (rc) return rc;
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  c->pl->set_stream(st);
  c->pl->clear_error();
  rc = c->pw->autotune(j->b_xy, j->nb, j->noverlays, j->c_xy, j->c_off, st, best_ms);
  if (rc) return set_err(c, rc, c->pl->error());
  if (split) *split = c->pw->big_k;
  if (cell_factor) *cell_factor = c->pw->cell_factor;
  return SBC_OK;
}

extern "C" int sbc_batch_set_arena_budget(sbc_ctx* c, long long bytes) {
  if (!c) return SBC_EINPUT;
  if (bytes < 0) return set_err(c, SBC_EINPUT, "negative budget");
  c->br->arena_budget = bytes;
  return SBC_OK;
}

extern "C" int sbc_batch_set_shape(sbc_ctx* c, const int* shape) {
  if (!c || !shape) return SBC_EINPUT;
  for (int i = 0; i < 4; ++i)
    if (shape[i] < 32 || shape[i] > 128 || shape[i] % 32)
      return set_err(c, SBC_EINPUT, "block sizes must be 32, 64, 96 or 128");
  if (shape[4] < 3 || shape[4] > SBC_BATCH_MAX_VERTICES)
    return set_err(c, SBC_EINPUT, "split must be 3 to SBC_BATCH_MAX_VERTICES");
  c->br->shape = sbc::BatchShape{shape[0], shape[1], shape[2], shape[3]};
  c->br->split = shape[4];
  c->br->valid = false;  // later calls re-run the forward pass with these settings
  return SBC_OK;
}

extern "C" int sbc_batch_get_shape(const sbc_ctx* c, int* shape) {
  if (!c || !shape) return SBC_EINPUT;
  const sbc::BatchShape& s = c->br->shape;
  const int v[5] = {s.front, s.cand, s.back, s.bwd, c->br->split};
  for (int i = 0; i < 5; ++i) shape[i] = v[i];
  return SBC_OK;
}

extern "C" int sbc_batch_autotune(sbc_ctx* c, const sbc_batch* b, const double* grad_area,
                                  double* grad_b, double* grad_c, int* shape, double* best_ms,
                                  void* stream) {
  int rc = batch_check(c, b);
  if (rc) return rc;
  if (b->npairs > 0 && (!grad_area || !grad_b || !grad_c))
    return set_err(c, SBC_EINPUT, "null gradient array");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  c->pl->clear_error();
  c->pl->set_stream(st);
  c->br->set_components(b->npairs, b->b_off, b->c_off, nullptr, 0, nullptr, 0, 0, 0, st);
  rc = c->br->autotune(b->npairs, b->b_xy, b->b_off, b->c_xy, b->c_off, grad_area, grad_b, grad_c,
                       st, best_ms);
  if (rc) return set_err(c, rc, c->pl->error());
  if (shape) sbc_batch_get_shape(c, shape);
  return SBC_OK;
}

extern "C" int sbc_batch_info(const sbc_ctx* c, long long* out, int n) {
  if (!c || !out) return SBC_EINPUT;
  const long long v[2] = {c->br->chunks(), c->br->large_pairs()};
  for (int i = 0; i < n && i < 2; ++i) out[i] = v[i];
  return SBC_OK;
}

struct sbc_graph {
  sbc_ctx* ctx = nullptr;
  cudaGraphExec_t exec = nullptr;
  unsigned long long kernels = 0;
  unsigned long long generation = 0;
};

extern "C" int sbc_area_graph_create(sbc_ctx* c, const sbc_batch* b, const double* grad_area,
                                     double* grad_b, double* grad_c, double* area, int* status,
                                     void* stream, sbc_graph** out) {
  if (!out) return set_err(c, SBC_EINPUT, "null output");
  *out = nullptr;
  int rc = batch_check(c, b);
  if (rc) return rc;
  if (!grad_area || !grad_b || !grad_c) return set_err(c, SBC_EINPUT, "null gradient array");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  c->pl->set_stream(st);
  c->pl->clear_error();
  auto* g = new (std::nothrow) sbc_graph();
  if (!g) return set_err(c, SBC_ENOMEM, "graph");
  c->br->set_components(b->npairs, b->b_off, b->c_off, nullptr, 0, nullptr, 0, 0, 0, st);
  rc = c->br->graph_record(b->npairs, b->b_xy, b->b_off, b->c_xy, b->c_off, grad_area, grad_b,
                           grad_c, area, status, st, &g->exec, &g->kernels);
  if (rc) {
    delete g;
    return set_err(c, rc, c->pl->error());
  }
  g->ctx = c;
  g->generation = c->br->generation;
  *out = g;
  return SBC_OK;
}

extern "C" int sbc_area_graph_launch(sbc_graph* g, void* stream) {
  if (!g || !g->exec) return SBC_EINPUT;
  sbc_ctx* c = g->ctx;
  if (c->br->generation != g->generation)
    return set_err(c, SBC_EINPUT, "stale graph: a later batched call replaced its buffers");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  const int rc = cuda_check(c, cudaGraphLaunch(g->exec, st), "graph launch");
  if (!rc) sbc::g_launches += g->kernels;
  return rc;
}

extern "C" void sbc_area_graph_destroy(sbc_graph* g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  delete g;
}

extern "C" int sbc_pairwise_area_device(sbc_ctx* c, const sbc_pairwise_job* j, double* area,
                                        int* status, void* stream) {
  if (c && j && j->noverlays > 0 && !area) return set_err(c, SBC_EINPUT, "null area output");
  sbc_batch_rings dr;
  int rc = sbc_clip_pairwise_device(c, j, &dr, stream);
  if (rc) return rc;
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  rc = c->pw->area(area, st);
  if (rc) return set_err(c, rc, c->pl->error());
  if (status && j->noverlays > 0)
    cudaMemcpyAsync(status, c->pw->status, sizeof(int) * j->noverlays, cudaMemcpyDeviceToDevice, st);
  return cuda_check(c, cudaStreamSynchronize(st), "pairwise area");
}

extern "C" int sbc_pairwise_area_backward_device(sbc_ctx* c, const sbc_pairwise_job* j,
                                                 const double* grad_area, double* grad_b,
                                                 double* grad_c, void* stream) {
  int rc = pairwise_check(c, j);
  if (rc) return rc;
  if (!grad_b || (j->noverlays > 0 && (!grad_area || !grad_c)))
    return set_err(c, SBC_EINPUT, "null gradient array");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->own;
  if (!(c->pw->valid && c->pw->np == j->noverlays && c->pw->key_b == j->b_xy &&
        c->pw->key_c == j->c_xy)) {
    sbc_batch_rings dr;
    rc = sbc_clip_pairwise_device(c, j, &dr, stream);
    if (rc) return rc;
  }
  c->pl->clear_error();
  rc = c->pw->backward(j->b_xy, j->c_xy, j->c_off, grad_area, grad_b, grad_c, st);
  if (rc) return set_err(c, rc, c->pl->error());
  return SBC_OK;
}
