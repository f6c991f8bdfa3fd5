// sbc_prims.cu -- device-wide exclusive scan and stable LSD radix sort.
//
// These replace the reference's Thrust calls (p_seg_tree/thrust_func.cu:19-42:
// stable_sort_by_key on double / int / long keys, exclusive_scan on int /
// long).  HBM-bound: each radix pass reads and writes every (key, value)
// once; one histogram kernel counts all digit positions up front, and passes
// whose digit is constant over all keys are skipped on the device.
#include "sbc_internal.cuh"

#include <cstdint>
#include <cstdio>
#include <mutex>

namespace sbc {

std::atomic<unsigned long long> g_launches{0};

// ============================================================== launch probes
namespace {
struct ProbeRec {
  const char* name;
  cudaEvent_t a, b;
  double bytes;
  cudaStream_t st;
};
// the last profiled window, launch by launch: start relative to the first
// launch's start, duration, stream (numbered in order of first use)
std::vector<TimelineRec> g_timeline;
// probes may come from several host threads (the pairwise engine's big-pair
// workers): the record list is guarded
std::atomic<bool> g_prof_on{false};
std::mutex g_prof_mu;
std::vector<ProbeRec> g_recs;
std::vector<cudaEvent_t> g_event_pool;
size_t g_event_next = 0;

cudaEvent_t next_event() {
  if (g_event_next == g_event_pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    g_event_pool.push_back(e);
  }
  return g_event_pool[g_event_next++];
}
}  // namespace

KProbe::KProbe(const char* name, cudaStream_t st, double bytes) : name_(name), st_(st), slot_(-1) {
  ++g_launches;
  if (!g_prof_on) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  ProbeRec r{name, next_event(), next_event(), bytes, st};
  cudaEventRecord(r.a, st);
  slot_ = (int)g_recs.size();
  g_recs.push_back(r);
}

KProbe::~KProbe() {
  if (slot_ < 0) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  cudaEventRecord(g_recs[slot_].b, st_);
}

bool profiling_on() { return g_prof_on; }

bool profiling_suspend() {
  const bool on = g_prof_on;
  g_prof_on = false;
  return on;
}

void profiling_restore(bool on) { g_prof_on = on; }

const std::vector<TimelineRec>& profile_timeline() { return g_timeline; }

void profile_begin() {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_recs.clear();
  g_event_next = 0;
  g_prof_on = true;
}

int profile_end(std::vector<std::string>* names, std::vector<float>* ms, std::vector<int>* counts,
                std::vector<double>* bytes) {
  g_prof_on = false;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  names->clear();
  ms->clear();
  counts->clear();
  if (bytes) bytes->clear();
  g_timeline.clear();
  std::vector<cudaStream_t> streams;
  for (auto& r : g_recs) {
    cudaEventSynchronize(r.b);
    float t = 0.f, t0 = 0.f;
    cudaEventElapsedTime(&t, r.a, r.b);
    cudaEventElapsedTime(&t0, g_recs[0].a, r.a);
    int sid = 0;
    while (sid < (int)streams.size() && streams[sid] != r.st) ++sid;
    if (sid == (int)streams.size()) streams.push_back(r.st);
    g_timeline.push_back(TimelineRec{r.name, t0, t, sid});
    size_t i = 0;
    while (i < names->size() && (*names)[i] != r.name) ++i;
    if (i == names->size()) {
      names->push_back(r.name);
      ms->push_back(0.f);
      counts->push_back(0);
      if (bytes) bytes->push_back(0.0);
    }
    (*ms)[i] += t;
    (*counts)[i] += 1;
    if (bytes) (*bytes)[i] += r.bytes;
  }
  g_recs.clear();
  g_event_next = 0;
  return (int)names->size();
}

// ============================================================== scan
namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // 4096

// a thread's kScanItems consecutive elements as 16-byte loads and stores
// (the array 16-byte aligned, all items in range); else one by one
template <typename T>
__device__ __forceinline__ void scan_load(const T* d, long long base, long long n, bool vec,
                                          T (&v)[kScanItems]) {
  constexpr int nv = (int)(sizeof(T) * kScanItems / 16);
  if (vec && base + kScanItems <= n) {
    union {
      uint4 u[nv];
      T t[kScanItems];
    } x;
    const uint4* q = reinterpret_cast<const uint4*>(d + base);
#pragma unroll
    for (int k = 0; k < nv; ++k) x.u[k] = q[k];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) v[i] = x.t[i];
    return;
  }
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) v[i] = (base + i < n) ? d[base + i] : T(0);
}

template <typename T>
__device__ __forceinline__ void scan_store(T* d, long long base, long long n, bool vec,
                                           const T (&v)[kScanItems]) {
  constexpr int nv = (int)(sizeof(T) * kScanItems / 16);
  if (vec && base + kScanItems <= n) {
    union {
      uint4 u[nv];
      T t[kScanItems];
    } x;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) x.t[i] = v[i];
    uint4* q = reinterpret_cast<uint4*>(d + base);
#pragma unroll
    for (int k = 0; k < nv; ++k) q[k] = x.u[k];
    return;
  }
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) d[base + i] = v[i];
}

template <typename T>
__device__ T block_exclusive_scan(T v, T* smem_warp, T* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    T w = lane < nw ? smem_warp[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) smem_warp[lane] = w;
  }
  __syncthreads();
  T warp_off = warp > 0 ? smem_warp[warp - 1] : T(0);
  if (total) *total = smem_warp[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_off + x - v;
}

template <typename T>
__global__ void k_scan_reduce(const T* __restrict__ d, long long n, T* __restrict__ sums) {
  __shared__ T sw[32];
  long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  T s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += d[base + i];
  T tot;
  block_exclusive_scan<T>(s, sw, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <typename T>
__global__ void k_scan_apply(T* __restrict__ d, long long n, const T* __restrict__ offs, bool vec) {
  __shared__ T sw[32];
  long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  T v[kScanItems];
  scan_load(d, base, n, vec, v);
  T s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) s += v[i];
  T ex = block_exclusive_scan<T>(s, sw, nullptr);
  T run = ex + (offs ? offs[blockIdx.x] : T(0));
  T o[kScanItems];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    o[i] = run;
    run += v[i];
  }
  scan_store(d, base, n, vec, o);
}

template <typename T>
void scan_multi(T* d, long long n, T* scratch, cudaStream_t st);

// Single-pass scan with decoupled look-back.  Each block takes the next
// tile index from a counter (so every earlier tile is already resident),
// publishes its tile total, then warp 0 walks back over the predecessors 32
// at a time, summing totals until it meets a tile that has published its
// inclusive prefix, and publishes its own.  Status words: bits 63..62 =
// 0 not ready / 1 total / 2 inclusive prefix, bits 61..0 = value (scanned
// values are non-negative counts).  Every wait is bounded; a wait that gives
// up sets g_scan_error (checked by the caller's pipeline) and carries on.
constexpr unsigned long long kLbTotal = 1ull << 62, kLbPrefix = 2ull << 62;
constexpr unsigned long long kLbMask = (1ull << 62) - 1;
constexpr unsigned kLbSpin = 1u << 20;
// Two-level look-back: tiles also add their totals into a word per group of
// kScanGroup tiles (count in bits 56-61, sum below), and a group's last tile
// marks the word with the group's inclusive prefix (bit 63).  A tile reads its
// own group's tile words, then whole groups, 32 per round trip: when every
// tile starts at once, the walk to tile 0 takes tiles / 1024 round trips
// instead of tiles / 32.
constexpr int kScanGroup = 32;
constexpr unsigned long long kGrpInc = 1ull << 63, kGrpOne = 1ull << 56;
constexpr unsigned long long kGrpMask = (1ull << 56) - 1;
__host__ __device__ constexpr unsigned scan_groups(unsigned tiles) {
  return (tiles + kScanGroup - 1) / kScanGroup;
}
// look-back words of one scan over `tiles` tiles: ticket, tiles, groups, done counter
__host__ __device__ constexpr size_t scan_words(unsigned tiles) {
  return (size_t)tiles + scan_groups(tiles) + 2;
}
__device__ unsigned g_scan_error = 0;

// Up to kScanMulti independent arrays in one launch: blockIdx.y picks the
// array; each has its own look-back words, gridDim.x + 2 of them, and blocks
// past an array's own tile count only count themselves done.
constexpr int kScanMulti = 4;
template <typename T>
struct ScanSet {
  T* d[kScanMulti];
  long long n[kScanMulti];
  bool vec[kScanMulti];
};

// One tile of a decoupled look-back scan over n values: load(base, v)
// fetches the kScanItems values from position base (zero past n), store(base,
// o) writes their exclusive prefix.  `state` holds scan_words(gridDim.x)
// look-back words; T_ = gridDim.x tiles are launched.
template <typename T, typename Load, typename Store>
__device__ __forceinline__ void scan_tile_lb(Load load, Store store, long long n,
                                             unsigned long long* __restrict__ state) {
  __shared__ T sw[32];
  __shared__ unsigned s_tile;
  __shared__ T s_prefix;
  const unsigned T_ = gridDim.x, G_ = scan_groups(gridDim.x);
  if (threadIdx.x == 0) s_tile = atomicAdd((unsigned*)state, 1u);
  __syncthreads();
  const unsigned tile = s_tile;
  unsigned long long* ts = state + 1;         // tile words
  unsigned long long* gs = state + 1 + T_;    // group words
  const long long ntiles = (n + kScanTile - 1) / kScanTile;
  if ((long long)tile < ntiles) {
    const long long base = (long long)tile * kScanTile + (long long)threadIdx.x * kScanItems;
    T v[kScanItems];
    load(base, v);
    T s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) s += v[i];
    T tot;
    const T ex = block_exclusive_scan<T>(s, sw, &tot);
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      const long long g = tile / kScanGroup, g0 = g * kScanGroup;
      // the group's aggregate first, then the tile's own word: whoever sees
      // the tile word also sees its share of the group word
      if (lane == 0) {
        atomicAdd(&gs[g], kGrpOne | ((unsigned long long)tot & kGrpMask));
        __threadfence();
        atomicExch(&ts[tile], (tile == 0 ? kLbPrefix : kLbTotal) |
                                  ((unsigned long long)tot & kLbMask));
      }
      T prefix = 0;
      if (tile > 0) {
        // 1. the tiles of the own group before this one (one round trip)
        const long long j = (long long)tile - 1 - lane;
        unsigned long long w = 0;
        if (j >= g0) {
          unsigned spins = 0;
          do {
            w = *(volatile unsigned long long*)&ts[j];
          } while ((w >> 62) == 0 && ++spins < kLbSpin);
          if ((w >> 62) == 0) {
            atomicOr(&g_scan_error, 1u);
            w = kLbPrefix;
          }
        }
        unsigned pm = __ballot_sync(0xffffffffu, j >= g0 && (w >> 62) == 2);
        int firstP = pm ? __ffs(pm) - 1 : 32;
        T val = (j >= g0 && lane <= firstP) ? (T)(w & kLbMask) : T(0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
        prefix += val;
        // 2. earlier groups, 32 per round trip, nearest first, until a
        // group's inclusive prefix (or group 0)
        bool done = pm != 0;
        for (long long gt = g - 1; !done && gt >= 0; gt -= 32) {
          const long long q = gt - lane;
          unsigned long long x = 0;
          if (q >= 0) {
            unsigned spins = 0;
            do {
              x = *(volatile unsigned long long*)&gs[q];
            } while (!(x & kGrpInc) && (x >> 56) != (unsigned long long)kScanGroup &&
                     ++spins < kLbSpin);
            if (!(x & kGrpInc) && (x >> 56) != (unsigned long long)kScanGroup) {
              atomicOr(&g_scan_error, 1u);
              x = kGrpInc;
            }
          }
          pm = __ballot_sync(0xffffffffu, q >= 0 && (x & kGrpInc));
          firstP = pm ? __ffs(pm) - 1 : 32;
          val = (q >= 0 && lane <= firstP) ? (T)(x & kGrpMask) : T(0);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
          prefix += val;
          done = pm != 0;
        }
        if (lane == 0) atomicExch(&ts[tile], kLbPrefix | ((unsigned long long)(prefix + tot) & kLbMask));
      }
      // the group's last tile publishes the group's inclusive prefix (every
      // tile of the group has added to the group word: step 1 saw their words)
      if (lane == 0 && ((long long)tile == g0 + kScanGroup - 1 || (long long)tile == ntiles - 1))
        atomicExch(&gs[g], kGrpInc | ((unsigned long long)(prefix + tot) & kGrpMask));
      if (lane == 0) s_prefix = prefix;
    }
    __syncthreads();
    T run = ex + s_prefix;
    T o[kScanItems];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
      o[i] = run;
      run += v[i];
    }
    store(base, o);
  }
  // The last block to finish clears the look-back words (ticket, tile and
  // group words, this counter) so the next scan on the same scratch needs no
  // memset: a block counts itself done only after its own look-back reads, so
  // when the count reaches the number of blocks nobody reads the words any more.
  __shared__ bool s_last;
  const unsigned last_word = T_ + G_ + 1;
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&state[last_word], 1ull) == (unsigned long long)gridDim.x - 1;
  }
  __syncthreads();
  if (s_last)
    for (unsigned i = threadIdx.x; i <= last_word; i += blockDim.x) state[i] = 0ull;
}

template <typename T>
__global__ void __launch_bounds__(kScanThreads)
k_scan_lb(ScanSet<T> set, unsigned long long* __restrict__ state_all) {
  // the array of this blockIdx.y (selects, not an indexed parameter: that
  // would copy the set to local memory)
  const unsigned y = blockIdx.y;
  T* __restrict__ d = y == 0 ? set.d[0] : y == 1 ? set.d[1] : y == 2 ? set.d[2] : set.d[3];
  const long long n = y == 0 ? set.n[0] : y == 1 ? set.n[1] : y == 2 ? set.n[2] : set.n[3];
  const bool vec = y == 0 ? set.vec[0] : y == 1 ? set.vec[1] : y == 2 ? set.vec[2] : set.vec[3];
  scan_tile_lb<T>([&](long long base, T(&v)[kScanItems]) { scan_load(d, base, n, vec, v); },
                  [&](long long base, const T(&o)[kScanItems]) { scan_store(d, base, n, vec, o); },
                  n, state_all + (size_t)y * scan_words(gridDim.x));
}

template <typename T>
void scan_rec(T* d, long long n, T* scratch, cudaStream_t st, bool state_zero = false) {
  if (n <= 0) return;
  const long long tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles > 1) {
    auto* state = (unsigned long long*)scratch;
    // the scan leaves its words zero; a scratch not known to start zero is cleared first
    if (!state_zero)
      cudaMemsetAsync(state, 0, sizeof(unsigned long long) * scan_words((unsigned)tiles), st);
    ScanSet<T> set{};
    set.d[0] = d;
    set.n[0] = n;
    set.vec[0] = ((uintptr_t)d & 15) == 0;
    ::sbc::KProbe kp_("k_scan_lb", st, 2.0 * sizeof(T) * (double)n);
    k_scan_lb<T><<<dim3((unsigned)tiles, 1), kScanThreads, 0, st>>>(set, state);
    return;
  }
  scan_multi(d, n, scratch, st);
}

// count arrays scanned in one launch (see k_scan_lb)
template <typename T>
void scan_set(T* const* d, const long long* n, int count, T* scratch, cudaStream_t st,
              bool state_zero) {
  long long tiles = 1;
  double bytes = 0.0;
  ScanSet<T> set{};
  int c = 0;
  for (int i = 0; i < count; ++i) {
    if (n[i] <= 0) continue;
    set.d[c] = d[i];
    set.n[c] = n[i];
    set.vec[c] = ((uintptr_t)d[i] & 15) == 0;
    const long long t = (n[i] + kScanTile - 1) / kScanTile;
    tiles = t > tiles ? t : tiles;
    bytes += 2.0 * sizeof(T) * (double)n[i];
    ++c;
  }
  if (c == 0) return;
  auto* state = (unsigned long long*)scratch;
  if (!state_zero)
    cudaMemsetAsync(state, 0, sizeof(unsigned long long) * scan_words((unsigned)tiles) * c, st);
  ::sbc::KProbe kp_("k_scan_lb", st, bytes);
  k_scan_lb<T><<<dim3((unsigned)tiles, (unsigned)c), kScanThreads, 0, st>>>(set, state);
}

template <typename T>
void scan_multi(T* d, long long n, T* scratch, cudaStream_t st) {
  if (n <= 0) return;
  long long nb = (n + kScanTile - 1) / kScanTile;
  if (nb == 1) {
    {
      ::sbc::KProbe kp_("k_scan_apply", st);
      k_scan_apply<T><<<1, kScanThreads, 0, st>>>(d, n, nullptr, ((uintptr_t)d & 15) == 0);
    }
    return;
  }
  T* sums = scratch;
  {
    ::sbc::KProbe kp_("k_scan_reduce", st);
    k_scan_reduce<T><<<(unsigned)nb, kScanThreads, 0, st>>>(d, n, sums);
  }
  scan_multi<T>(sums, nb, scratch + ((nb + 63) / 64) * 64, st);
  {
    ::sbc::KProbe kp_("k_scan_apply", st);
    k_scan_apply<T><<<(unsigned)nb, kScanThreads, 0, st>>>(d, n, sums, ((uintptr_t)d & 15) == 0);
  }
}

}  // namespace

size_t scan_scratch_bytes(long long n) {
  const unsigned tiles = (unsigned)((n + kScanTile - 1) / kScanTile);
  const size_t lb = scan_words(tiles > 0 ? tiles : 1) * sizeof(unsigned long long);
  size_t tot = 0;
  while (n > kScanTile) {
    long long nb = (n + kScanTile - 1) / kScanTile;
    tot += (size_t)((nb + 63) / 64) * 64 * sizeof(long long);
    n = nb;
  }
  return (tot > lb ? tot : lb) + 256;
}

unsigned* scan_error_word() {
  static std::mutex mu;
  static unsigned* addr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scan_error) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    addr[dev] = (unsigned*)p;
  }
  return addr[dev];
}

bool scan_error_take() {
  unsigned h = 0;
  cudaMemcpyFromSymbol(&h, g_scan_error, sizeof(h));
  if (h) {
    const unsigned z = 0;
    cudaMemcpyToSymbol(g_scan_error, &z, sizeof(z));
  }
  return h != 0;
}

size_t scan_set_scratch_bytes(long long n_max, int count) {
  const unsigned tiles = (unsigned)((n_max + kScanTile - 1) / kScanTile);
  return (size_t)count * scan_words(tiles > 0 ? tiles : 1) * sizeof(unsigned long long) + 256;
}

void exclusive_scan_i32_set(int* const* d, const long long* n, int count, void* scratch,
                            cudaStream_t st, bool state_zero) {
  scan_set<int>(d, n, count, (int*)scratch, st, state_zero);
}

void exclusive_scan_i32(int* d, long long n, void* scratch, cudaStream_t st, bool state_zero) {
  scan_rec<int>(d, n, (int*)scratch, st, state_zero);
}
void exclusive_scan_i64(long long* d, long long n, void* scratch, cudaStream_t st,
                        bool state_zero) {
  scan_rec<long long>(d, n, (long long*)scratch, st, state_zero);
}

// ============================================================== radix sort
// Stable LSD radix sort with 8-bit digits in the onesweep arrangement
// (Adinets and Merrill, "Onesweep: a faster least significant digit radix
// sort for GPUs", 2022).  One histogram kernel counts every digit position in
// a single read of the keys.  Each pass is then one scatter kernel: a tile
// ranks its keys per digit with warp match/popc, publishes its per-digit
// counts, and takes its bucket offsets from a decoupled look-back over the
// tiles before it (a tile takes its index from a counter, so every earlier
// tile is already running; waits are bounded).  Keys are staged in shared
// memory in tile order so each digit's run is written out contiguously.
// A pass whose digit is the same for every key (one bucket holds all n) is
// skipped on the device, and which buffer a pass reads is worked out on the
// device from the passes before it, so the sort never waits on the host.
namespace {

constexpr int kOsThreads = 256;
constexpr int kOsWarps = kOsThreads / 32;
constexpr int kOsItems = 16;                    // keys per thread
constexpr int kOsTile = kOsThreads * kOsItems;  // 4096 keys per tile
constexpr int kOsMaxPasses = 8;
constexpr int kOsHistItems = 4;                 // keys per thread per round of the histogram
constexpr unsigned long long kOsAgg = 1ull << 62, kOsInc = 2ull << 62;
constexpr unsigned long long kOsMask = (1ull << 62) - 1;
constexpr size_t kOsHistBytes = sizeof(unsigned long long) * kOsMaxPasses * 256;
constexpr size_t kOsCtrBytes = 256;

// the digit positions (bytes) the host launches passes for, in order
struct OsPlan {
  int npass;
  int pos[kOsMaxPasses];
};

template <typename K>
__device__ __forceinline__ unsigned os_digit(K k, int pos) {
  return (unsigned)((k >> (8 * pos)) & 0xffu);
}

// The lanes of the warp holding the same 9-bit value d (a digit, or 256 for
// "no key"): the AND over its bits of the bit's ballot or its complement.
// Nine votes; every lane of the warp must take part.
__device__ __forceinline__ unsigned os_peers(unsigned d) {
  unsigned m = 0xffffffffu;
#pragma unroll
  for (int b = 0; b < 9; ++b) {
    const bool bit = (d >> b) & 1u;
    const unsigned v = __ballot_sync(0xffffffffu, bit);
    m &= bit ? v : ~v;
  }
  return m;
}

// Counts of every planned digit position in one read of the keys: a warp
// whose keys share the digit adds 32 with one atomic (the high, nearly
// constant digits), otherwise every lane adds its own.  Also zeroes the
// look-back words of the first pass.
template <typename K>
__global__ void __launch_bounds__(kOsThreads)
k_os_hist(const K* __restrict__ keys, long long n, OsPlan plan,
          unsigned long long* __restrict__ hist, unsigned long long* __restrict__ look0,
          long long look_words) {
  __shared__ unsigned h[kOsMaxPasses][256];
  for (int i = threadIdx.x; i < kOsMaxPasses * 256; i += kOsThreads) (&h[0][0])[i] = 0u;
  const long long gstride = (long long)gridDim.x * kOsThreads;
  for (long long i = (long long)blockIdx.x * kOsThreads + threadIdx.x; i < look_words; i += gstride)
    look0[i] = 0ull;
  __syncthreads();
  const unsigned lt = (1u << (threadIdx.x & 31)) - 1u;
  const long long step = gstride * kOsHistItems;
  // the loop bound is the same for every thread of the block, so whole warps
  // reach the match instructions
  for (long long base = (long long)blockIdx.x * kOsThreads * kOsHistItems; base < n; base += step) {
    K k[kOsHistItems];
    bool ok[kOsHistItems];
#pragma unroll
    for (int r = 0; r < kOsHistItems; ++r) {
      const long long j = base + (long long)r * kOsThreads + threadIdx.x;
      ok[r] = j < n;
      k[r] = ok[r] ? keys[j] : K(0);
    }
#pragma unroll
    for (int r = 0; r < kOsHistItems; ++r) {
      for (int q = 0; q < plan.npass; ++q) {
        const unsigned d = ok[r] ? os_digit(k[r], plan.pos[q]) : 256u;
        const unsigned d0 = __shfl_sync(0xffffffffu, d, 0);
        if (__all_sync(0xffffffffu, d == d0 && d0 < 256u)) {
          if (lt == 0u) atomicAdd(&h[q][d0], 32u);
        } else if (ok[r]) {
          atomicAdd(&h[q][d], 1u);
        }
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < plan.npass * 256; i += kOsThreads) {
    const unsigned v = (&h[0][0])[i];
    if (v) atomicAdd(&hist[i], (unsigned long long)v);
  }
}

// whether planned pass q sorts nothing: its histogram has one bucket of n
// (warp-wide: every lane of the calling warp must take part)
__device__ __forceinline__ bool os_constant(const unsigned long long* __restrict__ hist, int q,
                                            long long n) {
  bool full = false;
  for (int d = threadIdx.x & 31; d < 256; d += 32) full |= hist[q * 256 + d] == (unsigned long long)n;
  return __any_sync(0xffffffffu, full);
}

// exclusive scan of one value per thread over a 256-thread block
template <typename T>
__device__ __forceinline__ T os_block_scan(T v, T* s_warp) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[w] = x;
  __syncthreads();
  T off = 0;
  for (int i = 0; i < w; ++i) off += s_warp[i];
  __syncthreads();
  return off + x - v;
}

// One pass: planned pass `q` (digit position plan.pos[q]).  (ka, va) hold the
// input of the first pass; each pass that runs moves the keys to the other
// buffer pair.  Dynamic shared memory: kOsTile keys then kOsTile values.
constexpr int kOsLook = 32;  // earlier tiles read per look-back round trip
template <typename K>
constexpr size_t os_dyn_smem() { return (sizeof(K) + sizeof(unsigned)) * kOsTile; }

template <typename K>
__global__ void __launch_bounds__(kOsThreads, 2)
k_os_scatter(K* __restrict__ ka, unsigned* __restrict__ va, K* __restrict__ kb,
             unsigned* __restrict__ vb, long long n, int q, OsPlan plan,
             const unsigned long long* __restrict__ hist, unsigned* __restrict__ ctr,
             unsigned long long* __restrict__ look, long long tiles) {
  extern __shared__ __align__(16) unsigned char os_smem[];
  K* s_k = reinterpret_cast<K*>(os_smem);                                   // tile order
  unsigned* s_v = reinterpret_cast<unsigned*>(os_smem + sizeof(K) * kOsTile);
  __shared__ unsigned s_wcnt[kOsWarps][256];         // per-warp digit counts, then offsets
  __shared__ unsigned s_dstart[256];                 // tile-local start of each digit
  __shared__ unsigned long long s_gbase[256];        // output position of each digit's first key
  __shared__ unsigned long long s_wscan[kOsWarps];
  __shared__ unsigned s_tile;
  __shared__ int s_skip, s_odd;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int pos = plan.pos[q];
  // per pass parity: tile words (tiles x 256), then group words (groups x 256)
  const long long groups = (tiles + kScanGroup - 1) / kScanGroup;
  unsigned long long* cur = look + (size_t)(q & 1) * (tiles + groups) * 256;
  unsigned long long* nxt = look + (size_t)((q + 1) & 1) * (tiles + groups) * 256;
  unsigned long long* gcur = cur + (size_t)tiles * 256;
  // the next pass's look-back words (not read by this pass)
  if (q + 1 < plan.npass) {
    nxt[(size_t)blockIdx.x * 256 + t] = 0ull;
    if (blockIdx.x < groups) nxt[(size_t)(tiles + blockIdx.x) * 256 + t] = 0ull;
  }
  if (w == 0) {
    int ran = 0;
    for (int p = 0; p < q; ++p) ran += os_constant(hist, p, n) ? 0 : 1;
    const bool skip = os_constant(hist, q, n);
    if (lane == 0) {
      s_skip = skip;
      s_odd = ran & 1;
      if (!skip) s_tile = atomicAdd(&ctr[q], 1u);
    }
  }
  for (int i = t; i < kOsWarps * 256; i += kOsThreads) (&s_wcnt[0][0])[i] = 0u;
  __syncthreads();
  if (s_skip) return;
  const K* __restrict__ sk = s_odd ? kb : ka;
  const unsigned* __restrict__ sv = s_odd ? vb : va;
  K* __restrict__ dk = s_odd ? ka : kb;
  unsigned* __restrict__ dv = s_odd ? va : vb;
  const long long tile = s_tile;
  const long long base = tile * kOsTile;
  const long long wbase = base + (long long)w * 32 * kOsItems;
  const unsigned lt = (1u << lane) - 1u;

  // load (warp w owns keys [wbase, wbase + 32*kOsItems), lane order within a round)
  K k[kOsItems];
  unsigned v[kOsItems], rank[kOsItems];
#pragma unroll
  for (int r = 0; r < kOsItems; ++r) {
    const long long j = wbase + r * 32 + lane;
    k[r] = j < n ? sk[j] : K(0);
    v[r] = j < n ? sv[j] : 0u;
  }
  // stable ranks within the warp, per digit
#pragma unroll
  for (int r = 0; r < kOsItems; ++r) {
    const bool ok = wbase + r * 32 + lane < n;
    const unsigned d = ok ? os_digit(k[r], pos) : 256u;
    const unsigned peers = os_peers(d);
    rank[r] = ok ? s_wcnt[w][d] + __popc(peers & lt) : 0u;
    __syncwarp();
    if (ok && (peers & lt) == 0u) s_wcnt[w][d] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit t: warp offsets and the tile's count; publish it at once so
  // later tiles can move on
  unsigned cnt = 0;
  for (int i = 0; i < kOsWarps; ++i) {
    const unsigned c = s_wcnt[i][t];
    s_wcnt[i][t] = cnt;
    cnt += c;
  }
  unsigned long long* row = cur + (size_t)tile * 256;
  const long long grp = tile / kScanGroup, g0 = grp * kScanGroup;
  // the group's count first, then the tile's own word (see k_scan_lb)
  atomicAdd(&gcur[(size_t)grp * 256 + t], kGrpOne | (unsigned long long)cnt);
  __threadfence();
  atomicExch(&row[t], (tile == 0 ? kOsInc : kOsAgg) | (unsigned long long)cnt);
  // the digit's global start, and its start inside the tile
  const unsigned long long gstart = os_block_scan<unsigned long long>(hist[q * 256 + t], s_wscan);
  const unsigned long long lstart = os_block_scan<unsigned long long>(cnt, s_wscan);
  s_dstart[t] = (unsigned)lstart;
  __syncthreads();
  // keys and values into tile order (the registers are free before the wait)
#pragma unroll
  for (int r = 0; r < kOsItems; ++r) {
    if (wbase + r * 32 + lane < n) {
      const unsigned d = os_digit(k[r], pos);
      const unsigned lp = rank[r] + s_dstart[d] + s_wcnt[w][d];
      s_k[lp] = k[r];
      s_v[lp] = v[r];
    }
  }
  // decoupled look-back for digit t in two levels (see k_scan_lb): the
  // tiles of the own group before this one, nearest first, until a tile's
  // inclusive prefix; then whole groups, kOsLook per round trip, until a
  // group's inclusive prefix or group 0.  Every wait is bounded.
  unsigned long long excl = 0;
  if (tile > 0) {
    bool done = false;
    {
      unsigned long long wv[kScanGroup];
#pragma unroll
      for (int u = 0; u < kScanGroup; ++u)
        wv[u] = (tile - 1 - u >= g0) ? __ldcg(&cur[(size_t)(tile - 1 - u) * 256 + t]) : 0ull;
#pragma unroll
      for (int u = 0; u < kScanGroup; ++u) {
        if (!done && tile - 1 - u >= g0) {
          unsigned long long x = wv[u];
          if ((x >> 62) == 0) {
            unsigned spins = 0;
            do {
              x = *(volatile unsigned long long*)&cur[(size_t)(tile - 1 - u) * 256 + t];
            } while ((x >> 62) == 0 && ++spins < kLbSpin);
            if ((x >> 62) == 0) {
              atomicOr(&g_scan_error, 2u);
              x = kOsInc;
            }
          }
          excl += x & kOsMask;
          if ((x >> 62) == 2) done = true;
        }
      }
    }
    for (long long gt = grp - 1; !done && gt >= 0; gt -= kOsLook) {
      unsigned long long wv[kOsLook];
#pragma unroll
      for (int u = 0; u < kOsLook; ++u)
        wv[u] = (gt - u >= 0) ? __ldcg(&gcur[(size_t)(gt - u) * 256 + t]) : kGrpInc;
#pragma unroll
      for (int u = 0; u < kOsLook; ++u) {
        if (!done) {
          unsigned long long x = wv[u];
          auto ready = [](unsigned long long y) {
            return (y & kGrpInc) || (y >> 56) == (unsigned long long)kScanGroup;
          };
          if (!ready(x)) {
            unsigned spins = 0;
            do {
              x = *(volatile unsigned long long*)&gcur[(size_t)(gt - u) * 256 + t];
            } while (!ready(x) && ++spins < kLbSpin);
            if (!ready(x)) {
              atomicOr(&g_scan_error, 2u);
              x = kGrpInc;
            }
          }
          excl += x & kGrpMask;
          if (x & kGrpInc) done = true;
        }
      }
    }
    atomicExch(&row[t], kOsInc | ((excl + cnt) & kOsMask));
  }
  // the group's last tile: the group's inclusive prefix for digit t
  if (tile == g0 + kScanGroup - 1 || tile == tiles - 1)
    atomicExch(&gcur[(size_t)grp * 256 + t], kGrpInc | ((excl + cnt) & kGrpMask));
  s_gbase[t] = gstart + excl;
  __syncthreads();
  // out: each digit's keys to consecutive positions
  const int tn = (int)((n - base) < kOsTile ? (n - base) : kOsTile);
  for (int i = t; i < tn; i += kOsThreads) {
    const K kk = s_k[i];
    const unsigned d = os_digit(kk, pos);
    const unsigned long long o = s_gbase[d] + (unsigned long long)(i - (int)s_dstart[d]);
    dk[o] = kk;
    dv[o] = s_v[i];
  }
}

// after the passes: if an odd number of them ran, the result is in (kb, vb)
template <typename K>
__global__ void k_os_final(K* __restrict__ ka, unsigned* __restrict__ va, const K* __restrict__ kb,
                           const unsigned* __restrict__ vb, long long n, OsPlan plan,
                           const unsigned long long* __restrict__ hist) {
  __shared__ int s_odd;
  if (threadIdx.x < 32) {
    int ran = 0;
    for (int p = 0; p < plan.npass; ++p) ran += os_constant(hist, p, n) ? 0 : 1;
    if (threadIdx.x == 0) s_odd = ran & 1;
  }
  __syncthreads();
  if (!s_odd) return;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    ka[i] = kb[i];
    va[i] = vb[i];
  }
}

long long os_tiles(long long n) { return (n + kOsTile - 1) / kOsTile; }
long long os_groups(long long tiles) { return (tiles + kScanGroup - 1) / kScanGroup; }

// the scatter's dynamic shared memory (with its static part above 48 KB)
// needs an opt-in, once per device
template <typename K>
void os_smem_optin() {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return;
  std::lock_guard<std::mutex> lk(mu);
  if (done[dev]) return;
  cudaFuncSetAttribute((const void*)k_os_scatter<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)os_dyn_smem<K>());
  done[dev] = true;
}

template <typename K>
void onesweep(K* keys, unsigned* vals, K* keys_tmp, unsigned* vals_tmp, long long n,
              unsigned pos_mask, void* scratch, cudaStream_t st) {
  if (n <= 1) return;
  OsPlan plan{};
  for (int p = 0; p < (int)sizeof(K) && p < kOsMaxPasses; ++p)
    if ((pos_mask >> p) & 1u) plan.pos[plan.npass++] = p;
  if (plan.npass == 0) return;
  const long long tiles = os_tiles(n);
  auto* hist = (unsigned long long*)scratch;
  auto* ctr = (unsigned*)((char*)scratch + kOsHistBytes);
  auto* look = (unsigned long long*)((char*)scratch + kOsHistBytes + kOsCtrBytes);
  cudaMemsetAsync(scratch, 0, kOsHistBytes + kOsCtrBytes, st);
  {
    long long g = (n + (long long)kOsThreads * kOsHistItems - 1) / ((long long)kOsThreads * kOsHistItems);
    if (g > 152 * 8) g = 152 * 8;
    ::sbc::KProbe kp_(sizeof(K) == 8 ? "k_os_hist_u64" : "k_os_hist_u32", st, (double)sizeof(K) * n);
    k_os_hist<K><<<(unsigned)g, kOsThreads, 0, st>>>(keys, n, plan, hist, look,
                                                     (tiles + os_groups(tiles)) * 256);
  }
  os_smem_optin<K>();
  for (int q = 0; q < plan.npass; ++q) {
    ::sbc::KProbe kp_(sizeof(K) == 8 ? "k_os_scatter_u64" : "k_os_scatter_u32", st,
                      2.0 * (sizeof(K) + sizeof(unsigned)) * n);
    k_os_scatter<K><<<(unsigned)tiles, kOsThreads, os_dyn_smem<K>(), st>>>(
        keys, vals, keys_tmp, vals_tmp, n, q, plan, hist, ctr, look, tiles);
  }
  {
    long long g = (n + 1023) / 1024;
    if (g > 152 * 4) g = 152 * 4;
    ::sbc::KProbe kp_("k_os_final", st);
    k_os_final<K><<<(unsigned)g, 256, 0, st>>>(keys, vals, keys_tmp, vals_tmp, n, plan, hist);
  }
}

}  // namespace

size_t radix_scratch_bytes(long long n) {
  const long long tiles = os_tiles(n > 1 ? n : 1);
  return kOsHistBytes + kOsCtrBytes +
         (size_t)2 * (tiles + os_groups(tiles)) * 256 * sizeof(unsigned long long) + 256;
}

void radix_sort_u32(unsigned* keys, unsigned* vals, unsigned* keys_tmp, unsigned* vals_tmp,
                    long long n, int key_bits, void* scratch, cudaStream_t st) {
  unsigned mask = 0;
  for (int p = 0; p < 4 && 8 * p < key_bits; ++p) mask |= 1u << p;
  onesweep<unsigned>(keys, vals, keys_tmp, vals_tmp, n, mask, scratch, st);
}

void radix_sort_u64(unsigned long long* keys, unsigned* vals, unsigned long long* keys_tmp,
                    unsigned* vals_tmp, long long n, void* scratch, cudaStream_t st) {
  onesweep<unsigned long long>(keys, vals, keys_tmp, vals_tmp, n, 0xffu, scratch, st);
}

void radix_sort_u64_within(unsigned long long* keys, unsigned* vals, unsigned long long* keys_tmp,
                           unsigned* vals_tmp, long long n, unsigned long long lo,
                           unsigned long long hi, void* scratch, cudaStream_t st) {
  // keys in [lo, hi] share every bit above the highest bit where lo and hi
  // differ: only the bytes at or below it can vary
  const unsigned long long d = lo ^ hi;
  unsigned mask = 0;
  if (d) {
    const int top = 63 - __builtin_clzll(d);
    for (int p = 0; p <= top / 8; ++p) mask |= 1u << p;
  }
  onesweep<unsigned long long>(keys, vals, keys_tmp, vals_tmp, n, mask, scratch, st);
}

}  // namespace sbc
