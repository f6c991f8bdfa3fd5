// sbc_pipeline.cuh -- state of one clipping run (base polygon + k overlays)
// and the stage entry points implemented in sbc_front.cu / sbc_cand.cu /
// sbc_mid.cu / sbc_back.cu.  One Pipeline per sbc_ctx; every buffer is grow-only so
// repeated calls of the same size allocate nothing.
#pragma once

#include <array>
#include <condition_variable>
#include <functional>
#include <map>
#include <mutex>
#include <thread>
#include <string>
#include <memory>
#include <vector>

#include "../../include/sbclip.h"
#include "sbc_internal.cuh"

namespace sbc {

// grow-only device buffers keyed by name
class BufferPool {
 public:
  ~BufferPool();
  // returns a device pointer of at least `bytes` (256-byte aligned)
  void* get(const std::string& name, size_t bytes);
  // the same, with newly allocated memory cleared on stream st (for scan
  // scratch, which every scan leaves zero)
  void* get_zeroed(const std::string& name, size_t bytes, cudaStream_t st);
  size_t bytes_held() const;
  void release_all();
  int failed = 0;

 private:
  struct Buf {
    void* p = nullptr;
    size_t n = 0;
  };
  std::map<std::string, Buf> bufs_;
};

// per-overlay results kept on the device
struct OverlayOut {
  int nrings = 0;
  long long nverts = 0;
  int* d_off = nullptr;     // nrings+1 vertex offsets
  double* d_xy = nullptr;   // 2*nverts
  // diagnostics
  long long raw_hits = 0, tests = 0, unique = 0, slots_b = 0, slots_c = 0, work = 0, survivors = 0;
  int slow_path = 0;
  // nrings and nverts still on their way to this host word pair (set by
  // the back end, filled by Pipeline::finish_counts)
  const int* counts = nullptr;
};

// Small host reads of device values.  A copy into pageable memory waits for
// the stream by itself, so every pageable read is a round trip; these copies
// go to pinned memory instead and all land at the stream's next
// synchronisation: a stage pays one round trip for all its reads.  The area
// is kWords 8-byte words; each stage reads through its own words
// (HostReads::k*), valid after the synchronisation that follows the copy.
class HostReads {
 public:
  static constexpr int kWords = 256;
  static constexpr int kFlags = 0;       // read_flags
  static constexpr int kFront = 8;       // elementary and end-list stages
  static constexpr int kCand = 24;       // candidate and exact stages
  static constexpr int kMid = 40;        // record and merge stages
  static constexpr int kBack = 64;       // back end
  static constexpr int kCounts = 128;    // per overlay (1..9): ring and vertex counts
  HostReads() = default;
  HostReads(const HostReads&) = delete;
  HostReads& operator=(const HostReads&) = delete;
  ~HostReads() {
    if (pinned_) cudaFreeHost(p_);
  }
  // queue a copy of n values at word w; returns where they will be
  template <typename T>
  T* get(const T* d, int w, cudaStream_t st, int n = 1) {
    T* h = (T*)word(w);
    cudaMemcpyAsync(h, d, sizeof(T) * n, cudaMemcpyDeviceToHost, st);
    return h;
  }
  void* word(int w) {
    if (!p_) {
      if (cudaMallocHost((void**)&p_, 8 * kWords) == cudaSuccess) {
        pinned_ = true;
      } else {
        cudaGetLastError();
        fallback_.assign(8 * kWords, 0);  // pageable: correct, one round trip per read
        p_ = fallback_.data();
      }
    }
    return p_ + 8 * w;
  }

 private:
  unsigned char* p_ = nullptr;
  bool pinned_ = false;
  std::vector<unsigned char> fallback_;
};

// One host thread that issues a pipeline's side-stream work (the grid stage
// and the first overlay's box join), so the host reads of that work wait for
// the side stream only, and the main thread's reads for the main stream only:
// neither stream idles behind the other's round trips.
class SideWorker {
 public:
  SideWorker() = default;
  SideWorker(const SideWorker&) = delete;
  SideWorker& operator=(const SideWorker&) = delete;
  ~SideWorker();
  // run f on the worker thread (started on first use, current device dev);
  // false if no thread could be started (the caller runs f itself)
  bool post(int dev, std::function<int()> f);
  // the posted task's result
  int wait();

 private:
  void loop();
  std::thread th_;
  std::mutex mu_;
  std::condition_variable cv_;
  std::function<int()> task_;
  bool has_task_ = false, busy_ = false, stop_ = false, started_ = false;
  int result_ = 0, dev_ = 0;
};

struct Timing {
  // milliseconds per phase (CUDA events), accumulated over one run
  float ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

class Pipeline {
 public:
  Pipeline(int device, cudaStream_t st) : dev_(device), st_(st) {}
  ~Pipeline();
  // polygons already on the device (no closing vertex), sizes on the host
  int run(const double* d_bxy, int nb, const double* d_cxy, const int* c_sizes, int k);
  const std::vector<OverlayOut>& outputs() const { return outs_; }
  const char* error() const { return err_.c_str(); }
  BufferPool& pool() { return pool_; }
  cudaStream_t stream() const { return st_; }
  void set_stream(cudaStream_t s) { st_ = s; }
  bool timing = false;
  Timing times;
  // tree statistics of the last run
  long long stat_edges = 0, stat_epc = 0, stat_ts = 0, stat_cover = 0, stat_leaf = 0;
  long long stat_outside_cmbr = 0;     // edges left out of the candidate grid (common MBR)
  // force the serial emulation of the back end (test hook)
  int force_serial_backend = 0;
  // union instead of intersection (the Foster back end's UNION switch)
  bool unite = false;

  // ---- shared state (public for the stage kernels' launchers) ----
  int nb = 0, k = 0, clSize = 0, E = 0;
  std::vector<int> hcS, hcc;           // prefix of (c_i + 1) and of c_i
  double* bP = nullptr;                // (nb+1)*2
  double* cP = nullptr;                // (clSize+k)*2
  long long* bK = nullptr;             // order keys (okey) of bP's coordinates
  long long* cK = nullptr;             // order keys of cP's coordinates
  int* cS = nullptr;                   // device copy of hcS (k+1)
  int* cc = nullptr;                   // device copy of hcc (k+1)
  int* e_id = nullptr;
  double* e_s = nullptr;
  double* e_e = nullptr;
  unsigned long long* v_key = nullptr;  // per vertex (= its edge): order key of its x value
  unsigned* v_id = nullptr;            // vertex index (the sort's payload)
  unsigned char* e_flip = nullptr;     // edge runs right to left (its first vertex is its end)
  int force_endpoint_sort = 0;         // test hook: sort the 2E endpoints, not the E vertices
  int force_wide_vertex_sort = 0;      // test hook: the vertex sort on 64-bit keys only
  int stat_vertex_sort = 0;            // the last run's endpoint order: 0 endpoint sort, 1 vertex
                                       // sort on 64-bit keys, 2 on 32-bit keys
  double minI = 0, maxI = 0;
  unsigned long long key_lo = 0, key_hi = 0;  // order keys of minI and maxI
  unsigned long long* d_minmax = nullptr;     // device copy of (key_lo, key_hi) from the setup
  // tree
  double* ea = nullptr;
  int epc = 0, numLeaves = 0, ts = 0, logL = 0;
  int z_garbage = 0;                   // position of the zero border entry
  int ele_count = 0;                   // elementary points before padding
  bool ele_tail = false;               // the last slot repeats the second-to-last value
  bool lr_ready = false;               // end leaves and leaf ranges came from the sort
  int* aft = nullptr;                  // leaf node from the edge's end (or -1)
  int* bef = nullptr;                  // leaf node from the edge's start (or -1)
  int2* lr = nullptr;                  // per edge: leaves [l, r1) its interval contains
  unsigned long long* d_treecnt = nullptr;  // [0] end-list leaf entries, [1] cover entries
  // uniform grid over float edge boxes (candidate pairs, sbc_cand.cu)
  struct GridParams {
    float x0 = 0.f, y0 = 0.f, inv = 1.f;
    int gx = 1, gy = 1;
  } grid_;
  int* g_tstart = nullptr;             // edge-index start of each polygon class (k+2)
  float4* fbox = nullptr;              // float edge boxes, bounds rounded outwards
  float4* vfB = nullptr;               // base vertices as float hi/lo pairs
  float4* vfC = nullptr;               // overlay vertices as float hi/lo pairs
  unsigned char* g_islong = nullptr;   // edge spans too many cells for the grid
  int* g_long = nullptr;               // those edges
  unsigned* g_long_count = nullptr;
  int* g_bstart = nullptr;             // first entry of each (cell, class) bucket (+ end)
  unsigned* g_vals = nullptr;          // edge of each grid entry, grouped by bucket
  long long g_n = 0;
  int g_nCells = 0;                    // gx * gy
  long long pair_cap_ = 0;             // candidate-pair buffer size that sufficed last time
  unsigned* d_flags = nullptr;         // device error flags (DevFlag bits)
  unsigned* g_bnd = nullptr;           // grid bounds (order keys), extent sum, outside count
  int* g_fill = nullptr;               // per-bucket fill counters of the grid scatter
  int join_ready_ = 0;                 // overlay whose box join below is ready (0: none)
  const int2* join_pairs_ = nullptr;
  unsigned long long* join_counters_ = nullptr;
  const double2* raw_ab_ = nullptr;    // (alpha, beta) of each candidate hit (stage_candidates)
  long long join_npairs_ = 0, join_work_ = 0;
  // intermediate arrays of the last overlay processed (device, diagnostics)
  int *dbg_ub = nullptr, *dbg_uc = nullptr, *dbg_ut = nullptr;
  int dbg_K = 0;
  double* dbg_isxy = nullptr;
  int *dbg_aB = nullptr, *dbg_aC = nullptr;
  double *dbg_ixB = nullptr, *dbg_ixC = nullptr;
  int *dbg_alB = nullptr, *dbg_alC = nullptr, *dbg_nbB = nullptr, *dbg_nbC = nullptr;
  int *dbg_labB = nullptr, *dbg_labC = nullptr;
  int dbg_nB = 0, dbg_nQ = 0;

  // stage entry points (return Status)
  int stage_setup(const double* d_bxy, const double* d_cxy, const int* c_sizes);
  int stage_elementary();
  int stage_endlists();
  int stage_cover();
  // the grid in three steps on the side stream: boxes and bounds; cell
  // counts (reads the bounds); entries (reads the count, then the main
  // stream waits for the side stream)
  int stage_grid_boxes();
  int stage_grid_count();
  int stage_grid_fill();
  // the box join of overlay cType on stream st (results kept for the
  // candidate stage of that overlay)
  int stage_join(int cType, cudaStream_t st);
  cudaStream_t side_stream();     // created on first use; nullptr if that fails
  void join_side();               // later work on the main stream waits for the side stream
  void take_tree_stats();         // the cover stage's statistics, once their copy landed
  void launch_cover_count();      // the cover-entry statistic on the side stream
  int stage_candidates(int cType, int** rb, int** rc, int** rt, unsigned long long** rkey,
                       long long* nhits, OverlayOut& out);
  int stage_overlay(int cType, OverlayOut& out);
  int stage_records(int cType, const int* rb, const int* rc, const int* rt,
                    const unsigned long long* rkey, long long nraw, OverlayOut& out,
                    bool unique_sorted = false);
  // one pair's rows A10-A18 from its unique candidate hits in A9's order
  // (base id, then first-emission key; no tree): the same rings as run() on
  // that pair when the hits are the pair's own
  int run_from_hits(const double* d_bxy, int nb, const double* d_cxy, int nc, const int* rb,
                    const int* rc, const int* rt, const unsigned long long* rkey, long long nhits);

  // records the first error message (the side worker's own, on its thread)
  int fail(int code, const std::string& msg);
  void clear_error() { err_.clear(); }
  unsigned read_flags();
  void clear_flags();
  HostReads& reads() { return rd_; }
  // ring and vertex counts of the overlays whose back end queued them
  // (OverlayOut::counts): waits for the main stream once if any is pending
  void finish_counts();

 private:
  int dev_;
  cudaStream_t st_;
  cudaStream_t st2_ = nullptr;         // side stream (grid stage)
  cudaEvent_t ev_setup_ = nullptr, ev_side_ = nullptr, ev_lr_ = nullptr;
  bool cover_count_pending_ = false;
  unsigned* h_side_rd_ = nullptr;      // 256 B pinned: the grid stage's reads ([0..9]),
                                       // the cover stage's two counts ([32..35])
  bool tree_stats_pending_ = false;
  std::vector<int> h_tstart_;
  BufferPool pool_;
  HostReads rd_;
  // the side worker's buffers, host reads and first error (its stages run
  // concurrently with the main thread's)
  BufferPool side_pool_;
  HostReads side_rd_;
  std::string side_err_;
  SideWorker side_;
  std::vector<OverlayOut> outs_;
  std::string err_;
};

// back end entry (sbc_back.cu): from the merged arrays to rings
struct Merged {
  int nB = 0, nQ = 0, K = 0, bSize = 0, cSize = 0, cStart = 0;
  const double* ixB;   // 2*nB
  const double* ixC;   // 2*nQ
  const int* alB;      // nB
  const int* nbB;      // nB
  const int* nbC;      // nQ
  const int* labB;     // nB
  const int* labC;     // nQ
  const int* bND;      // bSize+1 exclusive prefix of non-degenerate counts
  const int* cND;      // cSize+1
  const double* bP;    // base with closing vertex
  const double* cP;    // overlays with closing vertices
};
int run_backend(Pipeline& pl, const Merged& m, OverlayOut& out);

// Many independent pairs (sbc_batch.cu): pairs whose polygons have at most
// SBC_BATCH_MAX_VERTICES vertices one device thread each, in chunks whose
// arenas fit a memory budget; larger pairs through the Pipeline with a
// provenance tape.  The forward pass keeps the last chunk's rings and tapes
// resident for rings() and backward(); other chunks are recomputed there.
// block sizes of the batch engine's kernels (tuning knobs: results do not
// depend on them); each a multiple of 32, at most 128
struct BatchShape {
  int front = 128, cand = 128, back = 128, bwd = 128;
};

class BatchRunner {
 public:
  explicit BatchRunner(Pipeline& pl) : pl_(pl) {}
  BatchShape shape;
  int split = SBC_BATCH_MAX_VERTICES;  // polygons above it go to the pair pipeline (<= the max)
  // components of the current call (device, pair-relative successor of each
  // vertex within its component; null: one ring per polygon).  A batch with
  // components clips every pair here: the pair pipeline takes one ring.
  const int* bnx = nullptr;
  const int* cnx = nullptr;
  const void* key_bcomp = nullptr;  // the component offsets they came from
  const void* key_ccomp = nullptr;
  int split_now() const { return (bnx || cnx) ? 0x7fffffff : split; }
  // components for the calls that follow (device offsets, each side's
  // component starts ending with its vertex count; null: one ring per
  // polygon): builds bnx / cnx
  int set_components(int np, const long long* d_boff, const long long* d_coff,
                     const long long* d_bcomp, long long nbc, const long long* d_ccomp,
                     long long ncc, long long nbv, long long ncv, cudaStream_t st);
  // times forward + backward of the batch under each knob's candidates in
  // turn (the better of two runs), keeps the fastest; the forward results of
  // the last run are left as forward() leaves them
  int autotune(int np, const double* d_bxy, const long long* d_boff, const double* d_cxy,
               const long long* d_coff, const double* d_gA, double* d_gb, double* d_gc,
               cudaStream_t st, double* best_ms);
  int forward(int np, const double* d_bxy, const long long* d_boff, const double* d_cxy,
              const long long* d_coff, cudaStream_t st);
  int rings(const double* d_bxy, const long long* d_boff, const double* d_cxy,
            const long long* d_coff, cudaStream_t st, long long** pair_ring, long long** ring_off,
            double** xy, long long* total_rings, long long* total_verts);
  int backward(const double* d_bxy, const long long* d_boff, const double* d_cxy,
               const long long* d_coff, const double* d_gA, double* d_gb, double* d_gc,
               cudaStream_t st);
  // per pair (device): status, rings, vertices, area
  int np = 0;
  int *status = nullptr, *nrings = nullptr, *nverts = nullptr;
  double* area = nullptr;
  double in_verts = 0.0;         // input vertices of the batch (profiling)
  const void* key_b = nullptr;  // the forward's inputs (for reuse by backward)
  const void* key_c = nullptr;
  bool valid = false;
  long long arena_budget = 0;   // bytes per chunk of arenas; 0: min(96 GiB, half of free)
  bool unite = false;           // union instead of intersection
  // the area forward + backward of this batch as one CUDA graph (needs one
  // arena chunk and no large pair); kernels: launches per replay
  int graph_record(int np, const double* d_bxy, const long long* d_boff, const double* d_cxy,
                   const long long* d_coff, const double* d_gA, double* d_gb, double* d_gc,
                   double* out_area, int* out_status, cudaStream_t st, cudaGraphExec_t* exec,
                   unsigned long long* kernels);
  unsigned long long generation = 0;  // bumped by every forward pass
  int chunks() const { return (int)chunks_.size(); }
  int large_pairs() const { return (int)big_.size(); }

 private:
  struct BigOut {
    int p = 0, nrings = 0, nverts = 0;
    bool ok = false;
    int* off = nullptr;
    double* xy = nullptr;
    int4* tape = nullptr;
  };
  int plan(int np, const long long* d_boff, const long long* d_coff, cudaStream_t st);
  int run_chunk(int c, const double* d_bxy, const long long* d_boff, const double* d_cxy,
                const long long* d_coff, cudaStream_t st);
  int run_big(const double* d_bxy, const double* d_cxy, cudaStream_t st);
  Pipeline& pl_;
  unsigned char* arena[2] = {nullptr, nullptr};
  long long* aoff[2] = {nullptr, nullptr};
  long long abase_[2] = {0, 0};
  int* pass = nullptr;
  int* need_ = nullptr;          // per pair: hits found by a first pass that ran out of room
  void* sscr_ = nullptr;
  std::vector<long long> h_boff_, h_coff_, h_aoff0_;
  std::vector<std::pair<int, int>> chunks_;
  std::vector<BigOut> big_;
  int resident_ = -1;
};

// One base polygon against many overlays with pairwise results: overlay i's
// rings are those of `seg base overlay_i` (sbc_pairwise.cu).  Pairs outside
// the rank shortcut's conditions run through the Pipeline.
class PairwiseRunner {
 public:
  explicit PairwiseRunner(Pipeline& pl);
  ~PairwiseRunner();
  int run(const double* d_bxy, int nb, int nov, const double* d_cxy, const long long* d_coff,
          cudaStream_t st);
  int autotune(const double* d_bxy, int nb, int nov, const double* d_cxy, const long long* d_coff,
               cudaStream_t st, double* best_ms);
  // area of every overlay's result (device, np doubles) from the last run
  int area(double* d_area, cudaStream_t st);
  // d(sum grad_area * area)/d(base, overlays) from the last run's rings
  int backward(const double* d_bxy, const double* d_cxy, const long long* d_coff,
               const double* d_gA, double* d_gb, double* d_gc, cudaStream_t st);
  const void* key_b = nullptr;   // the last run's inputs (for reuse by backward)
  const void* key_c = nullptr;
  bool valid = false;
  int np = 0;
  int* status = nullptr;            // device, per overlay: SBC_* code
  long long* pair_ring = nullptr;   // device, np+1
  long long* ring_off = nullptr;    // device, total_rings+1
  double* xy = nullptr;             // device, 2*total_verts
  long long total_rings = 0, total_verts = 0;
  std::vector<int> h_status;
  std::vector<long long> h_pair_ring;
  // diagnostics of the last run
  int fallback_pairs = 0;           // pairs clipped by the whole pair pipeline
  int big_pairs = 0;                // pairs whose records went to its rows A9-A18
  int big_k = 8192;                 // records from which a pair counts as big
  int big_workers = 8;              // host threads, each with a pipeline and a stream, for big pairs
  int pair_reserve = 1;             // block slots per SM the per-pair kernel leaves to big pairs
  long long hits = 0, tested = 0, grid_cells = 0;
  double cell_factor = 1.0;         // grid cell width in units of sqrt(area / n_b)

 private:
  struct BigWorker;
  std::vector<std::unique_ptr<BigWorker>> workers_;
  Pipeline& pl_;
  unsigned long long hit_cap_ = 0;
  cudaStream_t st2_ = nullptr;      // the per-pair kernel's stream
  cudaEvent_t ev_[2] = {nullptr, nullptr};
  std::vector<int> order_h;
  unsigned pair_blocks_ = 0;
  unsigned pair_grid(int nov, bool reserve);
  // the last run, for area and backward
  int last_nb_ = 0;
  long long last_totalC_ = 0, last_nh_ = 0;
  std::vector<long long> h_coff_;
  std::vector<std::array<int, 4>> fb_rec_;  // records of pipeline-clipped pairs: pair, b, c, type
  std::vector<double> fb_xy_;
};

}  // namespace sbc
