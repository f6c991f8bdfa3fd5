// sbc_front.cu -- polygon setup, elementary intervals, end lists and cover
// lists of the flattened segment tree (reference rows A1, A4-A7).
//
//  A1  gpc_read_multi_polygon            src/clip.cpp:172-311
//  A4  constructElementaryIntervals...   p_seg_tree/oacc_segment_tree.cpp:4513-4692
//  A5  constructTreeIntervalArray...     oacc_segment_tree.cpp:4948-4994 (derived on the fly)
//  A6  insertToLeafLevelEdgeList...      oacc_segment_tree.cpp:1970-2113, merges :1717-1968
//  A7  insertEdgeParallel                oacc_segment_tree.cpp:2496-2607
#include <cstdio>

#include "sbc_pipeline.cuh"

namespace sbc {

// ---------------------------------------------------------------- BufferPool
BufferPool::~BufferPool() { release_all(); }

void* BufferPool::get(const std::string& name, size_t bytes) {
  bytes = ((bytes + 255) / 256) * 256;
  if (bytes == 0) bytes = 256;
  Buf& b = bufs_[name];
  if (b.n >= bytes) return b.p;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.n = 0;
  size_t want = bytes + bytes / 8;  // headroom for slightly larger repeat calls
  if (cudaMalloc(&b.p, want) != cudaSuccess) {
    cudaGetLastError();
    if (cudaMalloc(&b.p, bytes) != cudaSuccess) {
      cudaGetLastError();
      b.p = nullptr;
      failed = 1;
      return nullptr;
    }
    want = bytes;
  }
  b.n = want;
  return b.p;
}

void* BufferPool::get_zeroed(const std::string& name, size_t bytes, cudaStream_t st) {
  void* before = bufs_[name].p;
  void* p = get(name, bytes);
  if (p && p != before) cudaMemsetAsync(p, 0, bufs_[name].n, st);
  return p;
}

size_t BufferPool::bytes_held() const {
  size_t t = 0;
  for (auto& kv : bufs_) t += kv.second.n;
  return t;
}

void BufferPool::release_all() {
  for (auto& kv : bufs_)
    if (kv.second.p) cudaFree(kv.second.p);
  bufs_.clear();
}

namespace {
// set on the side worker's thread: Pipeline::fail records its message apart
thread_local bool t_side_worker = false;
}  // namespace

SideWorker::~SideWorker() {
  if (!started_) return;
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  cv_.notify_all();
  th_.join();
}

bool SideWorker::post(int dev, std::function<int()> f) {
  if (!started_) {
    dev_ = dev;
    try {
      th_ = std::thread(&SideWorker::loop, this);
    } catch (...) {
      return false;
    }
    started_ = true;
  }
  {
    std::lock_guard<std::mutex> lk(mu_);
    task_ = std::move(f);
    has_task_ = true;
    busy_ = true;
  }
  cv_.notify_all();
  return true;
}

int SideWorker::wait() {
  std::unique_lock<std::mutex> lk(mu_);
  cv_.wait(lk, [&] { return !busy_; });
  return result_;
}

void SideWorker::loop() {
  t_side_worker = true;
  cudaSetDevice(dev_);
  std::unique_lock<std::mutex> lk(mu_);
  while (true) {
    cv_.wait(lk, [&] { return has_task_ || stop_; });
    if (stop_) return;
    std::function<int()> f = std::move(task_);
    has_task_ = false;
    lk.unlock();
    const int r = f();
    lk.lock();
    result_ = r;
    busy_ = false;
    cv_.notify_all();
  }
}

int Pipeline::fail(int code, const std::string& msg) {
  std::string& e = t_side_worker ? side_err_ : err_;
  if (e.empty()) e = msg;
  return code;
}

Pipeline::~Pipeline() {
  if (st2_) {
    cudaStreamSynchronize(st2_);
    cudaStreamDestroy(st2_);
  }
  if (ev_setup_) cudaEventDestroy(ev_setup_);
  if (ev_side_) cudaEventDestroy(ev_side_);
  if (ev_lr_) cudaEventDestroy(ev_lr_);
  if (h_side_rd_) cudaFreeHost(h_side_rd_);
}

// the second stream of this pipeline, created on first use with its two
// events and 256 bytes of pinned host memory for reads back
cudaStream_t Pipeline::side_stream() {
  if (st2_) return st2_;
  // the side stream at the highest priority: its grid and join kernels are
  // the large ones, and the main chain's small kernels fill around them
  int lo_pri = 0, hi_pri = 0;
  cudaStream_t s = nullptr;
  if (cudaDeviceGetStreamPriorityRange(&lo_pri, &hi_pri) != cudaSuccess ||
      cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, hi_pri) != cudaSuccess) {
    cudaGetLastError();
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
  }
  if (cudaEventCreateWithFlags(&ev_setup_, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ev_side_, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ev_lr_, cudaEventDisableTiming) != cudaSuccess ||
      cudaMallocHost((void**)&h_side_rd_, 256) != cudaSuccess) {
    cudaStreamDestroy(s);
    return nullptr;
  }
  st2_ = s;
  return st2_;
}

void Pipeline::join_side() {
  if (!st2_) return;
  cudaEventRecord(ev_side_, st2_);
  cudaStreamWaitEvent(st_, ev_side_, 0);
}

void Pipeline::take_tree_stats() {
  // no work of the run outlives the call
  if (st2_) cudaStreamSynchronize(st2_);
  cudaStreamSynchronize(st_);
  if (!tree_stats_pending_) return;
  unsigned long long hc[2];
  memcpy(hc, h_side_rd_ + 32, sizeof(hc));
  stat_leaf = (long long)hc[0];
  stat_cover = (long long)hc[1];
  tree_stats_pending_ = false;
}

unsigned Pipeline::read_flags() {
  const unsigned* f = rd_.get(d_flags, HostReads::kFlags, st_);
  cudaStreamSynchronize(st_);
  return *f;
}

void Pipeline::finish_counts() {
  bool pending = false;
  for (auto& o : outs_) pending |= o.counts != nullptr;
  if (!pending) return;
  cudaStreamSynchronize(st_);
  for (auto& o : outs_)
    if (o.counts) {
      o.nrings = o.counts[0];
      o.nverts = o.counts[1];
      o.counts = nullptr;
    }
}

void Pipeline::clear_flags() { cudaMemsetAsync(d_flags, 0, sizeof(unsigned), st_); }

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ int overlay_of(const int* pref, int k, int g) {
  int i = 0;
  while (i + 1 < k && pref[i + 1] <= g) ++i;
  return i;
}

// interval of tree node v (heap layout, leaves at [L, 2L)): start of its
// leftmost leaf and end of its rightmost leaf; node 0 was never written by the
// reference and reads as [0,0] (zero-filled heap).
__device__ __forceinline__ void node_interval(const double* __restrict__ ea, int logL, int v,
                                              double* s, double* e) {
  if (v <= 0) {
    *s = 0.0;
    *e = 0.0;
    return;
  }
  int d = 31 - __clz(v);
  int h = logL - d;
  int L = 1 << logL;
  int lo = (v << h) - L;
  int hi = ((v + 1) << h) - 1 - L;
  *s = ea[lo];
  *e = ea[hi + 1];
}

// ---------------------------------------------------------------- A1 setup
// the closed base ring, with the order keys of its coordinates (okey) for
// the comparison-only filters
__global__ void k_setup_base(const double* __restrict__ bxy, int nb, double* __restrict__ bP,
                             long long* __restrict__ bK) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > nb) return;
  int s = (i == nb) ? 0 : i;
  const double x = bxy[2 * s], y = bxy[2 * s + 1];
  bP[2 * i] = x;
  bP[2 * i + 1] = y;
  bK[2 * i] = okey(x);
  bK[2 * i + 1] = okey(y);
}

__global__ void k_setup_overlays(const double* __restrict__ cxy, const int* __restrict__ cS,
                                 const int* __restrict__ cc, int k, int total,
                                 double* __restrict__ cP, long long* __restrict__ cK) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  int i = overlay_of(cS, k, g);
  int v = g - cS[i];
  int c = cc[i + 1] - cc[i];
  int src = cc[i] + (v < c ? v : 0);
  const double x = cxy[2 * src], y = cxy[2 * src + 1];
  cP[2 * g] = x;
  cP[2 * g + 1] = y;
  cK[2 * g] = okey(x);
  cK[2 * g + 1] = okey(y);
}

// Edge::getData (edge.h:190-202); ids are offsets into the interleaved arrays
__global__ void k_setup_edges(const double* __restrict__ bP, const double* __restrict__ cP,
                              const int* __restrict__ cS, const int* __restrict__ cc, int nb, int k,
                              int E, int* __restrict__ eid, double* __restrict__ es,
                              double* __restrict__ ee, unsigned long long* __restrict__ minmax,
                              unsigned* __restrict__ flags, unsigned long long* __restrict__ vkey,
                              unsigned* __restrict__ vid, unsigned char* __restrict__ eflip) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long kmin = ~0ull, kmax = 0ull;
  if (e < E) {
    int id;
    double a, b;
    if (e < nb) {
      id = 2 * e;
      a = bP[id];
      b = bP[id + 2];
    } else {
      int g = e - nb;
      int i = overlay_of(cc, k, g);
      id = 2 * (cS[i] + (g - cc[i]));
      a = cP[id];
      b = cP[id + 2];
    }
    eid[e] = id;
    if (a < b) {
      es[e] = a;
      ee[e] = b;
    } else {
      ee[e] = a;
      es[e] = b;
    }
    // the edge's first vertex (vertex e) as a sort key, and whether it is the
    // edge's end point (endpoint 2e+1) rather than its start (2e)
    vkey[e] = dkey(a);
    vid[e] = (unsigned)e;
    eflip[e] = (a < b) ? 0 : 1;
    // every vertex is the first endpoint of exactly one edge: min/max over
    // vertices equals the reference's min/max over non-closing edges
    if (!isfinite(a)) atomicOr(flags, (unsigned)kFlagUndef);
    kmin = kmax = dkey(a);
  }
  for (int s = 16; s > 0; s >>= 1) {
    unsigned long long o1 = __shfl_xor_sync(0xffffffffu, kmin, s);
    unsigned long long o2 = __shfl_xor_sync(0xffffffffu, kmax, s);
    kmin = o1 < kmin ? o1 : kmin;
    kmax = o2 > kmax ? o2 : kmax;
  }
  // one pair of atomics per block: same-address atomics from every warp of
  // the grid serialise at the L2
  __shared__ unsigned long long s_min[32], s_max[32];
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_min[w] = kmin;
    s_max[w] = kmax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < nw; ++i) {
      kmin = s_min[i] < kmin ? s_min[i] : kmin;
      kmax = s_max[i] > kmax ? s_max[i] : kmax;
    }
    atomicMin(&minmax[0], kmin);
    atomicMax(&minmax[1], kmax);
  }
}

static double key_to_double(unsigned long long k) {
  unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  double d;
  memcpy(&d, &u, sizeof d);
  return d;
}

int Pipeline::stage_setup(const double* d_bxy, const double* d_cxy, const int* c_sizes) {
  // tree arrays of an earlier run are not this run's (diagnostics read them)
  ea = nullptr;
  aft = bef = nullptr;
  lr = nullptr;
  hcS.assign(k + 1, 0);
  hcc.assign(k + 1, 0);
  for (int i = 0; i < k; ++i) {
    hcS[i + 1] = hcS[i] + c_sizes[i] + 1;
    hcc[i + 1] = hcc[i] + c_sizes[i];
  }
  clSize = hcc[k];
  E = nb + clSize;
  bP = (double*)pool_.get("bP", sizeof(double) * 2 * (nb + 1));
  cP = (double*)pool_.get("cP", sizeof(double) * 2 * (clSize + k));
  bK = (long long*)pool_.get("bK", sizeof(long long) * 2 * (nb + 1));
  cK = (long long*)pool_.get("cK", sizeof(long long) * 2 * (clSize + k));
  cS = (int*)pool_.get("cS", sizeof(int) * (k + 1));
  cc = (int*)pool_.get("cc", sizeof(int) * (k + 1));
  e_id = (int*)pool_.get("e_id", sizeof(int) * E);
  e_s = (double*)pool_.get("e_s", sizeof(double) * E);
  e_e = (double*)pool_.get("e_e", sizeof(double) * E);
  unsigned long long* mm = (unsigned long long*)pool_.get("minmax", 16);
  d_flags = (unsigned*)pool_.get("flags", 256);
  v_key = (unsigned long long*)pool_.get("v_key", sizeof(unsigned long long) * E);
  v_id = (unsigned*)pool_.get("v_id", sizeof(unsigned) * E);
  e_flip = (unsigned char*)pool_.get("e_flip", E);
  if (pool_.failed) return fail(kENoMem, "device allocation failed (setup)");
  cudaMemcpyAsync(cS, hcS.data(), sizeof(int) * (k + 1), cudaMemcpyHostToDevice, st_);
  cudaMemcpyAsync(cc, hcc.data(), sizeof(int) * (k + 1), cudaMemcpyHostToDevice, st_);
  unsigned long long init[2] = {~0ull, 0ull};
  cudaMemcpyAsync(mm, init, 16, cudaMemcpyHostToDevice, st_);
  clear_flags();
  {
    ::sbc::KProbe kp_("k_setup_base", st_);
    k_setup_base<<<grid_for(nb + 1, 256), 256, 0, st_>>>(d_bxy, nb, bP, bK);
  }
  {
    ::sbc::KProbe kp_("k_setup_overlays", st_);
    k_setup_overlays<<<grid_for(clSize + k, 256), 256, 0, st_>>>(d_cxy, cS, cc, k, clSize + k, cP,
                                                                 cK);
  }
  {
    ::sbc::KProbe kp_("k_setup_edges", st_);
    k_setup_edges<<<grid_for(E, 256), 256, 0, st_>>>(bP, cP, cS, cc, nb, k, E, e_id, e_s, e_e, mm,
                                                   d_flags, v_key, v_id, e_flip);
  }
  // the x range and the non-finite flag are read with the elementary
  // stage's counts (one host round trip for both): nothing before that read
  // needs them on the host, and the kernels in between are index-safe on any
  // coordinate values
  d_minmax = mm;
  return kOk;
}

// ---------------------------------------------------------------- A4 elementary intervals
__global__ void k_ele_keys(const double* __restrict__ es, const double* __restrict__ ee, int E,
                           unsigned long long* __restrict__ keys, unsigned* __restrict__ vals) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= E) return;
  keys[2 * j] = dkey(es[j]);
  keys[2 * j + 1] = dkey(ee[j]);
  vals[2 * j] = 2 * j;
  vals[2 * j + 1] = 2 * j + 1;
}

// The endpoint order from the vertex order.  Every endpoint is a vertex's
// x value, and vertex v is an endpoint of exactly two edges: of edge v (index
// 2v, or 2v+1 when the edge runs right to left and v is its end) and of the
// polygon's previous edge p (v is that edge's second vertex: index 2p+1, or
// 2p when p runs right to left).  When no other vertex shares v's x value,
// its two endpoints are a run of their own in the stable endpoint sort, in
// index order; a shared x value sets kFlagSharedX and the caller sorts the
// endpoints themselves instead.
__global__ void k_ele_expand(const unsigned long long* __restrict__ skey,
                             const unsigned* __restrict__ svid,
                             const unsigned char* __restrict__ flip, const int* __restrict__ cc,
                             int nb, int k, int E, unsigned long long* __restrict__ keys,
                             unsigned* __restrict__ sidx, unsigned* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  const unsigned long long key = skey[i];
  if ((i > 0 && skey[i - 1] == key) || (i + 1 < E && skey[i + 1] == key))
    atomicOr(flags, (unsigned)kFlagSharedX);
  const int v = (int)svid[i];
  int p;
  if (v < nb) {
    p = v ? v - 1 : nb - 1;
  } else {
    const int g = v - nb;
    const int o = overlay_of(cc, k, g);
    p = g == cc[o] ? nb + cc[o + 1] - 1 : v - 1;
  }
  const unsigned a = 2u * (unsigned)v + flip[v];
  const unsigned b = 2u * (unsigned)p + 1u - flip[p];
  keys[2LL * i] = key;
  keys[2LL * i + 1] = key;
  sidx[2LL * i] = a < b ? a : b;
  sidx[2LL * i + 1] = a < b ? b : a;
}

__device__ __forceinline__ double ele_val(const double* es, const double* ee, unsigned idx) {
  return (idx & 1u) ? ee[idx >> 1] : es[idx >> 1];
}

// mark vertical edges reached from the first E sorted endpoints (:4568-4576)
__global__ void k_vl_mark(const unsigned* __restrict__ sidx, const double* __restrict__ es,
                          const double* __restrict__ ee, int E, int* __restrict__ vl) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= E) return;
  int i = sidx[j] >> 1;
  if (es[i] == ee[i]) vl[i] = 1;
}

__global__ void k_vl_loc(const int* __restrict__ vl, int E, int* __restrict__ vloc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  if (vl[i] != vl[i + 1]) vloc[vl[i]] = i;
}

// keep flags (:4603-4636); flag[] has 2E+1 zeroed entries, val[] 2E
__global__ void k_ele_flags(const unsigned* __restrict__ sidx, const double* __restrict__ es,
                            const double* __restrict__ ee, const int* __restrict__ vl,
                            const int* __restrict__ vloc, int E, int* __restrict__ flag,
                            double* __restrict__ val) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long n2 = 2LL * E;
  if (i >= n2 - 1) return;
  double v0 = ele_val(es, ee, sidx[i]);
  double v1 = ele_val(es, ee, sidx[i + 1]);
  int intvi = sidx[i] >> 1;
  int comid = vl[i / 2];
  if (v0 != v1) {
    val[i] = v0;
    flag[i] = 1;
  } else if (es[intvi] == ee[intvi]) {
    bool keep = comid == 0;
    if (!keep) {
      int lookup = vloc[comid - 1];
      keep = es[lookup] != es[intvi] && ee[lookup] != es[intvi];
    }
    if (keep) {
      val[i] = es[intvi];
      flag[i] = 1;
    }
  }
  if (i == n2 - 2) {
    // the last slot repeats the second-to-last sorted value (:4630-4635)
    if (v0 != v1) {
      val[n2 - 1] = v0;
      flag[n2 - 1] = 1;
    }
  }
}

__global__ void k_ele_compact(const int* __restrict__ flag, const double* __restrict__ val,
                              long long n2, double* __restrict__ ea) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n2) return;
  if (flag[i] != flag[i + 1]) ea[flag[i]] = val[i];
}

__global__ void k_ele_pad(double* __restrict__ ea, int count, int round) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + count;
  if (i >= round) return;
  ea[i] = ea[count - 1];
}

static int npow2_host(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

// ---- the vertex order from 32-bit keys.  The key of x is x scaled and
// shifted into [2^19, 2^32 - 2^19]: fma(x, s, c) with s > 0 (one rounding of
// a function increasing in x), then truncation to an unsigned integer; each
// step is monotone, so x < x' gives key <= key'.  The 2^19 margins keep the
// rounding of c and of the fma inside the unsigned range.  Two FP64
// instructions per vertex (the FP64 rate on GB300 is low).  Sorting (key, vertex) takes 4 radix
// passes instead of 8; only vertices with equal keys (x values closer than
// the x range / 2^32) can be out of full order, and those runs are put in
// (full key, vertex) order, the order of the stable sort on full keys.
constexpr int kFixRun = 32;  // longer runs fall back to the 64-bit sort

__global__ void k_vertex_narrow(int E, const unsigned long long* __restrict__ vkey,
                                const unsigned long long* __restrict__ mm,
                                unsigned* __restrict__ g, unsigned* __restrict__ gid) {
  __shared__ double s_scale, s_shift;
  if (threadIdx.x == 0) {
    const double lo = dkey_value(mm[0]), hi = dkey_value(mm[1]);
    const double sc = hi > lo ? (4294967296.0 - 1048576.0) / (hi - lo) : 0.0;
    s_scale = sc;
    s_shift = 524288.0 - lo * sc;
  }
  __syncthreads();
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= E) return;
  g[v] = __double2uint_rz(__fma_rn(dkey_value(vkey[v]), s_scale, s_shift));
  gid[v] = (unsigned)v;
}

// full keys in the narrow order, equal-key runs sorted; the run's first
// thread handles the whole run
__global__ void k_vertex_full(int E, const unsigned* __restrict__ g, unsigned* __restrict__ gid,
                              const unsigned long long* __restrict__ vkey,
                              unsigned long long* __restrict__ skey, unsigned* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  const unsigned gi = g[i];
  const bool prev_eq = i > 0 && g[i - 1] == gi;
  const bool next_eq = i + 1 < E && g[i + 1] == gi;
  if (!prev_eq && !next_eq) {
    skey[i] = vkey[gid[i]];
    return;
  }
  if (prev_eq) return;
  int m = 1;
  while (i + m < E && g[i + m] == gi && m < kFixRun) ++m;
  if (i + m < E && g[i + m] == gi) {
    atomicOr(flags, (unsigned)kFlagLongRun);
    return;
  }
  unsigned long long kk[kFixRun];
  unsigned ii[kFixRun];
  for (int t = 0; t < m; ++t) {
    ii[t] = gid[i + t];
    kk[t] = vkey[ii[t]];
  }
  for (int t = 1; t < m; ++t) {
    const unsigned long long k0 = kk[t];
    const unsigned i0 = ii[t];
    int u = t - 1;
    while (u >= 0 && (kk[u] > k0 || (kk[u] == k0 && ii[u] > i0))) {
      kk[u + 1] = kk[u];
      ii[u + 1] = ii[u];
      --u;
    }
    kk[u + 1] = k0;
    ii[u + 1] = i0;
  }
  for (int t = 0; t < m; ++t) {
    skey[i + t] = kk[t];
    gid[i + t] = ii[t];
  }
}

int Pipeline::stage_elementary() {
  long long n2 = 2LL * E;
  auto* keys = (unsigned long long*)pool_.get("ele_keys", sizeof(unsigned long long) * n2);
  auto* keys2 = (unsigned long long*)pool_.get("ele_keys2", sizeof(unsigned long long) * n2);
  auto* sidx = (unsigned*)pool_.get("ele_sidx", sizeof(unsigned) * n2);
  auto* sidx2 = (unsigned*)pool_.get("ele_sidx2", sizeof(unsigned) * n2);
  void* rscr = pool_.get("radix_scr", radix_scratch_bytes(n2));
  int* vl = (int*)pool_.get("ele_vl", sizeof(int) * (E + 1));
  int* vloc = (int*)pool_.get("ele_vloc", sizeof(int) * (E + 1));
  int* flag = (int*)pool_.get("ele_flag", sizeof(int) * (n2 + 1));
  double* val = (double*)pool_.get("ele_val", sizeof(double) * n2);
  void* sscr = pool_.get_zeroed("scan_scr", scan_scratch_bytes(n2 + 1), st_);
  auto* vkey2 = (unsigned long long*)pool_.get("v_key2", sizeof(unsigned long long) * E);
  auto* vid2 = (unsigned*)pool_.get("v_id2", sizeof(unsigned) * E);
  auto* vg = (unsigned*)pool_.get("v_g", sizeof(unsigned) * E);
  auto* vg2 = (unsigned*)pool_.get("v_g2", sizeof(unsigned) * E);
  auto* vgid = (unsigned*)pool_.get("v_gid", sizeof(unsigned) * E);
  if (pool_.failed) return fail(kENoMem, "device allocation failed (elementary)");
  // every endpoint is a vertex x value: its key lies in the setup's [min, max]
  bool by_vertex = !force_endpoint_sort;
  bool narrow = by_vertex && !force_wide_vertex_sort;
  int count = 0, before_last = 0;
  for (;;) {
  if (by_vertex && narrow) {
    // 32-bit keys (4 passes), then the full keys and the equal-key runs;
    // vkey2 holds the sorted full keys, vgid the vertices
    {
      ::sbc::KProbe kp_("k_vertex_narrow", st_, 16.0 * E);
      k_vertex_narrow<<<grid_for(E, 256), 256, 0, st_>>>(E, v_key, d_minmax, vg, vgid);
    }
    radix_sort_u32(vg, vgid, vg2, vid2, E, 32, rscr, st_);
    {
      ::sbc::KProbe kp_("k_vertex_full", st_, 24.0 * E);
      k_vertex_full<<<grid_for(E, 256), 256, 0, st_>>>(E, vg, vgid, v_key, vkey2, d_flags);
    }
    ::sbc::KProbe kp_("k_ele_expand", st_, 12.0 * E + 9.0 * E + 24.0 * E);
    k_ele_expand<<<grid_for(E, 256), 256, 0, st_>>>(vkey2, vgid, e_flip, cc, nb, k, E, keys, sidx,
                                                    d_flags);
  } else if (by_vertex) {
    // sort the E vertex keys, then expand to the 2E endpoints
    radix_sort_u64(v_key, v_id, vkey2, vid2, E, rscr, st_);
    ::sbc::KProbe kp_("k_ele_expand", st_, 12.0 * E + 9.0 * E + 24.0 * E);
    k_ele_expand<<<grid_for(E, 256), 256, 0, st_>>>(v_key, v_id, e_flip, cc, nb, k, E, keys, sidx,
                                                    d_flags);
  } else {
    {
      ::sbc::KProbe kp_("k_ele_keys", st_);
      k_ele_keys<<<grid_for(E, 256), 256, 0, st_>>>(e_s, e_e, E, keys, sidx);
    }
    radix_sort_u64(keys, sidx, keys2, sidx2, n2, rscr, st_);
  }
  cudaMemsetAsync(vl, 0, sizeof(int) * (E + 1), st_);
  {
    ::sbc::KProbe kp_("k_vl_mark", st_);
    k_vl_mark<<<grid_for(E, 256), 256, 0, st_>>>(sidx, e_s, e_e, E, vl);
  }
  exclusive_scan_i32(vl, E + 1, sscr, st_, true);
  {
    ::sbc::KProbe kp_("k_vl_loc", st_);
    k_vl_loc<<<grid_for(E, 256), 256, 0, st_>>>(vl, E, vloc);
  }
  cudaMemsetAsync(flag, 0, sizeof(int) * (n2 + 1), st_);
  {
    ::sbc::KProbe kp_("k_ele_flags", st_);
    k_ele_flags<<<grid_for(n2, 256), 256, 0, st_>>>(sidx, e_s, e_e, vl, vloc, E, flag, val);
  }
  exclusive_scan_i32(flag, n2 + 1, sscr, st_, true);
  const int* r_cnt = rd_.get(flag + n2 - 1, HostReads::kFront, st_, 2);  // before_last, count
  const unsigned* r_fl = rd_.get(d_flags, HostReads::kFront + 1, st_);
  const unsigned long long* r_mm = rd_.get(d_minmax, HostReads::kFront + 2, st_, 2);
  cudaStreamSynchronize(st_);
  before_last = r_cnt[0];
  count = r_cnt[1];
  const unsigned fl = *r_fl;
  const unsigned long long hm[2] = {r_mm[0], r_mm[1]};
  if (fl & kFlagUndef) return fail(kEInput, "non-finite vertex coordinate");
  key_lo = hm[0];
  key_hi = hm[1];
  minI = key_to_double(hm[0]);
  maxI = key_to_double(hm[1]);
  if (narrow && (fl & kFlagLongRun)) {
    // nearly equal x values in a long run: the 64-bit vertex sort
    narrow = false;
    clear_flags();
    continue;
  }
  if (by_vertex && (fl & kFlagSharedX)) {
    // a shared x value: the endpoints' own stable sort decides their order
    by_vertex = false;
    clear_flags();
    continue;
  }
  break;
  }
  stat_vertex_sort = by_vertex ? (narrow ? 2 : 1) : 0;
  if (count < 1) return fail(kEUndef, "no elementary interval (all endpoints equal)");
  int round = npow2_host(count) + 1;
  epc = round;
  numLeaves = round - 1;
  ts = 2 * numLeaves;
  logL = 0;
  while ((1 << logL) < numLeaves) ++logL;
  ea = (double*)pool_.get("ea", sizeof(double) * (round + 1));
  if (pool_.failed) return fail(kENoMem, "device allocation failed (ea)");
  {
    ::sbc::KProbe kp_("k_ele_compact", st_);
    k_ele_compact<<<grid_for(n2, 256), 256, 0, st_>>>(flag, val, n2, ea);
  }
  if (round > count) {
    {
      ::sbc::KProbe kp_("k_ele_pad", st_);
      k_ele_pad<<<grid_for(round - count, 256), 256, 0, st_>>>(ea, count, round);
    }
  }
  ele_count = count;
  ele_tail = count != before_last;  // the last slot repeats the second-to-last value
  stat_edges = E;
  stat_epc = epc;
  stat_ts = ts;
  return kOk;
}

// ---------------------------------------------------------------- A6 end lists
// Border sequence S(m) = boaders[sortedIndex[m]] (:1970-2008, :2016-2020):
// boaders[i-1] = ea[i] for i in [1, epc); the never-written slot epc-1 reads
// 0.0 and its digit key 0 sorts after the z leading zero keys.
struct Borders {
  const double* ea;
  int epc, z;
  __device__ __forceinline__ double S(int m) const {
    if (m < 0 || m >= epc) return __longlong_as_double(0x7ff8000000000000ll);  // past the arrays
    if (m < z) return ea[m + 1];
    if (m == z) return 0.0;
    return ea[m];
  }
  // boundary index j = sortedIndex[m]
  __device__ __forceinline__ int J(int m) const { return m < z ? m : (m == z ? epc - 1 : m - 1); }
};

// findBoarder, oacc_segment_tree.cpp:420-460
__device__ __forceinline__ int find_border(const Borders& B, double q) {
  int l = 0, h = B.epc;
  while (l < h) {
    int m = l + (h - l) / 2;
    double sm = B.S(m);
    if (sm == q) {
      if (B.S(m - 1) != q) {
        h = m;
        l = h;
      } else {
        h = m - 1;
      }
    } else if (sm < q) {
      l = m + 1;
    } else {
      h = m - 1;
    }
  }
  if (!(B.S(h) == q)) return -1;
  return h;
}

// integer border keys must be non-decreasing and non-negative for the
// shortcut ordering above (they are, by construction, unless rounding pushes
// a key to 1e11)
__global__ void k_border_check(const double* __restrict__ ea, int epc, double scale, double absMin,
                               int shift, int* __restrict__ zcount, unsigned* __restrict__ flags) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1;  // boundary i in [1, epc)
  if (i >= epc) return;
  auto key = [&](int t) -> long long {
    double v = shift ? dmul(scale, dadd(ea[t], absMin)) : dmul(scale, ea[t]);
    return (long long)v;
  };
  long long ki = key(i);
  if (ki < 0 || ki >= 100000000000LL) atomicOr(flags, (unsigned)kFlagUndef);
  if (i + 1 < epc && key(i + 1) < ki) atomicOr(flags, (unsigned)kFlagUndef);
  if (ki == 0) atomicAdd(zcount, 1);
}

// The two end-list leaves of each edge (insertToLeafLevelEdgeListMulticore,
// oacc_segment_tree.cpp:2010-2113): the leaf right of its end's border and
// the leaf left of its start's border; -1 where the reference drops the
// entry.  An internal node's end list is the set of edges with a leaf below
// it (buildInternalEndListsMulticore, :1717-1968), so these two leaves are
// all the end lists hold.  cnt[0] counts the entries.
__global__ void k_find_leaves(const double* __restrict__ es, const double* __restrict__ ee, int E,
                              Borders B, int logL, int* __restrict__ aft, int* __restrict__ bef,
                              unsigned long long* __restrict__ cnt) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned n = 0;
  if (e < E) {
  const int L = 1 << logL;
  const double* ea = B.ea;
  int a = -1, b = -1;
  int en = find_border(B, ee[e]);
  int st = find_border(B, es[e]);
  if (en >= 0) {
    int j = B.J(en);  // right[j]
    int node = 0;
    if (j <= B.epc - 2) {
      int i = j + 1;
      node = L + i;
      if (i != 1 && i + 1 < B.epc && ea[i] == ea[i + 1]) node = L + i + 1;
    }
    // node 0 ([0,0]) and node 2L (past the tree) are dropped
    if (node >= L && node < 2 * L && ea[node - L] != ea[node - L + 1]) a = node;
  }
  if (st >= 0) {
    int j = B.J(st);  // left[j]
    int node = 0;
    if (j <= B.epc - 2) node = L + j;
    if (node >= L && node < 2 * L && ea[node - L] != ea[node - L + 1]) b = node;
  }
  aft[e] = a;
  bef[e] = b;
  n = (a >= 0) + (b >= 0);
  }
  n = __reduce_add_sync(0xffffffffu, n);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(cnt, (unsigned long long)n);
}

// ---- end leaves and leaf ranges from the endpoint sort.  The endpoints of
// one value form a run of the sorted order; with ea sorted, the entries of
// ea equal to the value are [F[run start], F[run end + 1]) (F: the keep
// flags' exclusive prefix), the padding added when the value is ea's last.
// findBoarder then runs on positions (border_by_position) and the leaf range
// needs no search.
__global__ void k_ea_sorted(int epc, const double* __restrict__ ea, unsigned* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i + 1 < epc && !(ea[i] <= ea[i + 1])) atomicOr(flags, (unsigned)kFlagUnsorted);
}

__global__ void k_run_start(long long n2, const unsigned long long* __restrict__ keys,
                            int* __restrict__ chg) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n2) return;
  chg[i] = (i < n2 && (i == 0 || keys[i] != keys[i - 1])) ? 1 : 0;
}

// after the exclusive scan of the run starts: first and last position of each run
__global__ void k_run_bounds(long long n2, const unsigned long long* __restrict__ keys,
                             const int* __restrict__ rpre, int* __restrict__ rs,
                             int* __restrict__ re) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n2) return;
  const bool first = i == 0 || keys[i] != keys[i - 1];
  const bool last = i == n2 - 1 || keys[i + 1] != keys[i];
  const int r = rpre[i] + (first ? 0 : -1);
  if (first) rs[r] = (int)i;
  if (last) re[r] = (int)i;
}

// the positions [lo, hi) of ea holding the value of run r (sorted endpoint
// keys; run r spans [rs[r], re[r]])
__device__ __forceinline__ int2 run_range(int r, unsigned long long key,
                                          const int* __restrict__ rs, const int* __restrict__ re,
                                          const int* __restrict__ F, unsigned long long kl,
                                          int epc) {
  int lo = F[rs[r]], hi = F[re[r] + 1];
  if (key == kl) hi = epc;             // and the padding
  else if (key > kl) lo = hi = epc;    // above every entry, padding included
  return make_int2(lo, hi);
}

// per endpoint: its value's positions [lo, hi) in ea and its run
__global__ void k_endpoint_range(long long n2, const unsigned long long* __restrict__ keys,
                                 const unsigned* __restrict__ sidx, const int* __restrict__ rpre,
                                 const int* __restrict__ rs, const int* __restrict__ re,
                                 const int* __restrict__ F, int count, int epc,
                                 const double* __restrict__ ea, int2* __restrict__ erange,
                                 int* __restrict__ erun) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n2) return;
  const bool first = i == 0 || keys[i] != keys[i - 1];
  const int r = rpre[i] + (first ? 0 : -1);
  const unsigned x = sidx[i];
  erange[x] = run_range(r, keys[i], rs, re, F, dkey(ea[count - 1]), epc);
  erun[x] = r;
}

// per run of equal endpoint values: findBoarder's search (followed on
// positions, border_by_position), the same for every endpoint of the run;
// one thread per run (runs = rpre[n2])
__global__ void k_run_border(long long n2, const unsigned long long* __restrict__ keys,
                             const unsigned* __restrict__ sidx, const int* __restrict__ rpre,
                             const int* __restrict__ rs, const int* __restrict__ re,
                             const int* __restrict__ F, int count, int epc, int z,
                             const double* __restrict__ ea, const double* __restrict__ es,
                             const double* __restrict__ ee, int* __restrict__ rbord) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rpre[n2]) return;
  const int i = rs[r];
  const unsigned x = sidx[i];
  const double q = (x & 1u) ? ee[x >> 1] : es[x >> 1];
  const int2 lh = run_range((int)r, keys[i], rs, re, F, dkey(ea[count - 1]), epc);
  rbord[r] = border_by_position(epc, z, lh.x, lh.y, q);
}

__global__ void k_edge_tree(int E, const int2* __restrict__ erange, const int* __restrict__ erun,
                            const int* __restrict__ rbord,
                            const double* __restrict__ ea, int epc, int z, int logL,
                            int* __restrict__ aft, int* __restrict__ bef, int2* __restrict__ lr,
                            unsigned long long* __restrict__ cnt) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned n_leaf = 0;
  if (e < E) {
    const int L = 1 << logL;
    const int2 rS = erange[2 * e], rE = erange[2 * e + 1];
    auto J = [&](int m) { return m < z ? m : (m == z ? epc - 1 : m - 1); };
    int a = -1, b = -1;
    const int en = rbord[erun[2 * e + 1]];
    if (en >= 0) {
      const int j = J(en);  // right[j]
      int node = 0;
      if (j <= epc - 2) {
        const int i = j + 1;
        node = L + i;
        if (i != 1 && i + 1 < epc && ea[i] == ea[i + 1]) node = L + i + 1;
      }
      if (node >= L && node < 2 * L && ea[node - L] != ea[node - L + 1]) a = node;
    }
    const int st = rbord[erun[2 * e]];
    if (st >= 0) {
      const int j = J(st);  // left[j]
      int node = 0;
      if (j <= epc - 2) node = L + j;
      if (node >= L && node < 2 * L && ea[node - L] != ea[node - L + 1]) b = node;
    }
    aft[e] = a;
    bef[e] = b;
    n_leaf = (a >= 0) + (b >= 0);
    // leaves inside [start, end]: from the first entry >= start to before
    // the first entry > end
    const int l = rS.x < L ? rS.x : L;
    int r1 = rE.y - 1;
    r1 = r1 < 0 ? 0 : (r1 > L ? L : r1);
    lr[e] = make_int2(l, r1 > l ? r1 : l);
  }
  const unsigned long long t_leaf = block_sum((unsigned long long)n_leaf);
  if (threadIdx.x == 0 && t_leaf) atomicAdd(cnt, t_leaf);
}

// The number of cover-list entries (a statistic: the nodes of every edge's
// canonical decomposition of its leaf range), counted off the critical path
// on the side stream.  cnt[1] accumulates it.
__global__ void k_cover_count(int E, const int2* __restrict__ lr, int logL,
                              unsigned long long* __restrict__ cnt) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned n_cover = 0;
  if (e < E) {
    const int L = 1 << logL;
    const int2 r = lr[e];
    for (int x = r.x + L, y = r.y + L; x < y; x >>= 1, y >>= 1) {
      if (x & 1) {
        ++n_cover;
        ++x;
      }
      if (y & 1) {
        ++n_cover;
        --y;
      }
    }
  }
  const unsigned long long t = block_sum((unsigned long long)n_cover);
  if (threadIdx.x == 0 && t) atomicAdd(cnt + 1, t);
}

static int digit_count_host(double val) {
  int d = 1;
  int iv = (int)trunc(val);
  while (iv / 10 > 0) {
    iv /= 10;
    d++;
  }
  return d;
}

int Pipeline::stage_endlists() {
  double absMin = fabs(minI);
  double dv = maxI + absMin;
  if (!(dv < 2147483647.0)) return fail(kEUndef, "coordinate range too large for realToInt");
  int d = digit_count_host(dv);
  double scale = pow(10.0, 11 - d);
  int* zc = (int*)pool_.get("zcount", 256);
  aft = (int*)pool_.get("aft", sizeof(int) * E);
  bef = (int*)pool_.get("bef", sizeof(int) * E);
  d_treecnt = (unsigned long long*)pool_.get("tree_counts", 256);
  if (pool_.failed) return fail(kENoMem, "device allocation failed (end lists)");
  cudaMemsetAsync(zc, 0, sizeof(int), st_);
  cudaMemsetAsync(d_treecnt, 0, 2 * sizeof(unsigned long long), st_);
  clear_flags();
  {
    ::sbc::KProbe kp_("k_border_check", st_);
    k_border_check<<<grid_for(epc, 256), 256, 0, st_>>>(ea, epc, scale, absMin, minI < 0 ? 1 : 0, zc,
                                                     d_flags);
  }
  {
    ::sbc::KProbe kp_("k_ea_sorted", st_, 8.0 * epc);
    k_ea_sorted<<<grid_for(epc, 256), 256, 0, st_>>>(epc, ea, d_flags);
  }
  const int* r_z = rd_.get(zc, HostReads::kFront, st_);
  const unsigned* r_fl = rd_.get(d_flags, HostReads::kFront + 1, st_);
  cudaStreamSynchronize(st_);
  const int z = *r_z;
  const unsigned fl = *r_fl;
  if (fl & kFlagUndef) return fail(kEUndef, "border keys not monotone (realToInt)");
  z_garbage = z;
  lr_ready = false;
  if (!(fl & kFlagUnsorted) && !ele_tail) {
    // positions from the endpoint sort (see k_endpoint_range)
    const long long n2 = 2LL * E;
    auto* keys = (unsigned long long*)pool_.get("ele_keys", sizeof(unsigned long long) * n2);
    auto* sidx = (unsigned*)pool_.get("ele_sidx", sizeof(unsigned) * n2);
    int* F = (int*)pool_.get("ele_flag", sizeof(int) * (n2 + 1));
    int* rpre = (int*)pool_.get("run_pre", sizeof(int) * (n2 + 1));
    int* rs = (int*)pool_.get("run_s", sizeof(int) * n2);
    int* re = (int*)pool_.get("run_e", sizeof(int) * n2);
    int2* erange = (int2*)pool_.get("endpoint_range", sizeof(int2) * n2);
    int* erun = (int*)pool_.get("endpoint_run", sizeof(int) * n2);
    int* rbord = (int*)pool_.get("run_border", sizeof(int) * n2);
    void* sscr = pool_.get_zeroed("scan_scr", scan_scratch_bytes(n2 + 1), st_);
    lr = (int2*)pool_.get("edge_leaf_range", sizeof(int2) * (E + 1));
    if (pool_.failed) return fail(kENoMem, "device allocation failed (end lists)");
    {
      ::sbc::KProbe kp_("k_run_start", st_, 12.0 * n2);
      k_run_start<<<grid_for(n2 + 1, 256), 256, 0, st_>>>(n2, keys, rpre);
    }
    exclusive_scan_i32(rpre, n2 + 1, sscr, st_, true);
    {
      ::sbc::KProbe kp_("k_run_bounds", st_, 20.0 * n2);
      k_run_bounds<<<grid_for(n2, 256), 256, 0, st_>>>(n2, keys, rpre, rs, re);
    }
    {
      ::sbc::KProbe kp_("k_endpoint_range", st_, 36.0 * n2);
      k_endpoint_range<<<grid_for(n2, 256), 256, 0, st_>>>(n2, keys, sidx, rpre, rs, re, F,
                                                           ele_count, epc, ea, erange, erun);
    }
    {
      ::sbc::KProbe kp_("k_run_border", st_);
      k_run_border<<<grid_for(n2, 256), 256, 0, st_>>>(n2, keys, sidx, rpre, rs, re, F, ele_count,
                                                       epc, z, ea, e_s, e_e, rbord);
    }
    {
      // es, ee and two endpoint ranges in; aft, bef, leaf range out
      ::sbc::KProbe kp_("k_edge_tree", st_, 48.0 * E);
      k_edge_tree<<<grid_for(E, 256), 256, 0, st_>>>(E, erange, erun, rbord, ea, epc, z, logL,
                                                     aft, bef, lr, d_treecnt);
    }
    lr_ready = true;
    return kOk;
  }
  // ea[0] < 0 decides the shift; ea[0] equals minI
  Borders B{ea, epc, z};
  {
    ::sbc::KProbe kp_("k_find_leaves", st_, 24.0 * E);  // es, ee in; aft, bef out
    k_find_leaves<<<grid_for(E, 256), 256, 0, st_>>>(e_s, e_e, E, B, logL, aft, bef, d_treecnt);
  }
  return kOk;
}

// ---------------------------------------------------------------- A7 cover lists
// insertEdgeParallel (oacc_segment_tree.cpp:2496-2564) adds an edge to node v
// when v's interval lies inside the edge's [start, end] and recurses into the
// children whose interval touches it.  A leaf q = [ea[q], ea[q+1]] lies inside
// iff ea[q] >= start and ea[q+1] <= end; ea is sorted, so those leaves form
// one range [l, r1), every ancestor of a contained node touches the edge, and
// the nodes the recursion adds are exactly the canonical decomposition of
// [l, r1) (maximal nodes inside it).  The range is all the candidate stage
// needs; the lists themselves are never built.  cnt[1] counts their entries.
__global__ void k_edge_range(const double* __restrict__ es, const double* __restrict__ ee, int E,
                             const double* __restrict__ ea, int logL, int2* __restrict__ lr,
                             unsigned long long* __restrict__ cnt) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned n = 0;
  if (e < E) {
    const int L = 1 << logL;
    double s = es[e], x = ee[e];
    int lo = 0, hi = L;  // l = first leaf with ea[q] >= s
    while (lo < hi) {
      int m = (lo + hi) >> 1;
      if (ea[m] < s) lo = m + 1;
      else hi = m;
    }
    const int l = lo;
    lo = 0;
    hi = L;  // r1 = first leaf with ea[q+1] > x
    while (lo < hi) {
      int m = (lo + hi) >> 1;
      if (ea[m + 1] <= x) lo = m + 1;
      else hi = m;
    }
    const int r1 = lo;
    lr[e] = make_int2(l, r1 > l ? r1 : l);
    for (int a = l + L, b = r1 + L; a < b; a >>= 1, b >>= 1) {
      if (a & 1) {
        ++n;
        ++a;
      }
      if (b & 1) {
        ++n;
        --b;
      }
    }
  }
  n = __reduce_add_sync(0xffffffffu, n);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(cnt + 1, (unsigned long long)n);
}

int Pipeline::stage_cover() {
  lr = (int2*)pool_.get("edge_leaf_range", sizeof(int2) * (E + 1));
  if (pool_.failed) return fail(kENoMem, "device allocation failed (leaf ranges)");
  if (!lr_ready) {
    ::sbc::KProbe kp_("k_edge_range", st_, 24.0 * E);  // es, ee in; leaf range out
    k_edge_range<<<grid_for(E, 256), 256, 0, st_>>>(e_s, e_e, E, ea, logL, lr, d_treecnt);
  }
  // the two counts are statistics only, read at the end of run().  With the
  // leaf ranges from the sort, the cover entries are counted by
  // k_cover_count on the side stream (launch_cover_count)
  if (!side_stream()) return fail(kECuda, "side stream");
  if (lr_ready) {
    cudaEventRecord(ev_lr_, st_);
    cover_count_pending_ = true;
  } else {
    cudaMemcpyAsync(h_side_rd_ + 32, d_treecnt, 2 * sizeof(unsigned long long),
                    cudaMemcpyDeviceToHost, st_);
  }
  tree_stats_pending_ = true;
  return kOk;
}

void Pipeline::launch_cover_count() {
  if (!cover_count_pending_) return;
  cover_count_pending_ = false;
  cudaStreamWaitEvent(st2_, ev_lr_, 0);
  {
    ::sbc::KProbe kp_("k_cover_count", st2_);
    k_cover_count<<<grid_for(E, 256), 256, 0, st2_>>>(E, lr, logL, d_treecnt);
  }
  cudaMemcpyAsync(h_side_rd_ + 32, d_treecnt, 2 * sizeof(unsigned long long),
                  cudaMemcpyDeviceToHost, st2_);
}

}  // namespace sbc
