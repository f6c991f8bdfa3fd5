// sbc_prims.cu -- device-wide exclusive scan and stable LSD radix sort.
//
// These replace the reference's Thrust calls (p_seg_tree/thrust_func.cu:19-42:
// stable_sort_by_key on double / int / long keys, exclusive_scan on int /
// long).  HBM-bound: each radix pass reads and writes every (key, value) once
// plus a per-tile digit histogram; passes whose digit is constant over all
// keys are skipped (one OR/AND reduction decides).
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
};
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
  ProbeRec r{name, next_event(), next_event(), bytes};
  cudaEventRecord(r.a, st);
  slot_ = (int)g_recs.size();
  g_recs.push_back(r);
}

KProbe::~KProbe() {
  if (slot_ < 0) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  cudaEventRecord(g_recs[slot_].b, st_);
}

bool profiling_suspend() {
  const bool on = g_prof_on;
  g_prof_on = false;
  return on;
}

void profiling_restore(bool on) { g_prof_on = on; }

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
  for (auto& r : g_recs) {
    cudaEventSynchronize(r.b);
    float t = 0.f;
    cudaEventElapsedTime(&t, r.a, r.b);
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
__device__ unsigned g_scan_error = 0;

template <typename T>
__global__ void __launch_bounds__(kScanThreads)
k_scan_lb(T* __restrict__ d, long long n, unsigned long long* __restrict__ state, bool vec) {
  __shared__ T sw[32];
  __shared__ unsigned s_tile;
  __shared__ T s_prefix;
  if (threadIdx.x == 0) s_tile = atomicAdd((unsigned*)state, 1u);
  __syncthreads();
  const unsigned tile = s_tile;
  unsigned long long* ts = state + 1;
  const long long base = (long long)tile * kScanTile + (long long)threadIdx.x * kScanItems;
  T v[kScanItems];
  scan_load(d, base, n, vec, v);
  T s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) s += v[i];
  T tot;
  const T ex = block_exclusive_scan<T>(s, sw, &tot);
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    T prefix = 0;
    if (tile == 0) {
      if (lane == 0) atomicExch(&ts[0], kLbPrefix | ((unsigned long long)tot & kLbMask));
    } else {
      if (lane == 0) atomicExch(&ts[tile], kLbTotal | ((unsigned long long)tot & kLbMask));
      long long top = (long long)tile - 1;
      bool done = false;
      while (!done) {
        const long long j = top - lane;
        unsigned long long w = kLbPrefix;  // before tile 0: nothing to add
        if (j >= 0) {
          unsigned spins = 0;
          do {
            w = *(volatile unsigned long long*)&ts[j];
          } while ((w >> 62) == 0 && ++spins < kLbSpin);
          if ((w >> 62) == 0) {
            atomicOr(&g_scan_error, 1u);
            w = kLbPrefix;
          }
        }
        const unsigned pm = __ballot_sync(0xffffffffu, (w >> 62) == 2);
        const int firstP = pm ? __ffs(pm) - 1 : 32;
        T val = (lane <= firstP && j >= 0) ? (T)(w & kLbMask) : T(0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
        prefix += val;
        done = pm != 0;
        top -= 32;
      }
      if (lane == 0) atomicExch(&ts[tile], kLbPrefix | ((unsigned long long)(prefix + tot) & kLbMask));
    }
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
  scan_store(d, base, n, vec, o);
}

template <typename T>
void scan_rec(T* d, long long n, T* scratch, cudaStream_t st) {
  if (n <= 0) return;
  const long long tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles > 1) {
    auto* state = (unsigned long long*)scratch;
    cudaMemsetAsync(state, 0, sizeof(unsigned long long) * (tiles + 1), st);
    ::sbc::KProbe kp_("k_scan_lb", st, 2.0 * sizeof(T) * (double)n);
    k_scan_lb<T><<<(unsigned)tiles, kScanThreads, 0, st>>>(d, n, state,
                                                       ((uintptr_t)d & 15) == 0);
    return;
  }
  scan_multi(d, n, scratch, st);
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
  const size_t lb = (size_t)((n + kScanTile - 1) / kScanTile + 1) * sizeof(unsigned long long);
  size_t tot = 0;
  while (n > kScanTile) {
    long long nb = (n + kScanTile - 1) / kScanTile;
    tot += (size_t)((nb + 63) / 64) * 64 * sizeof(long long);
    n = nb;
  }
  return (tot > lb ? tot : lb) + 256;
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

void exclusive_scan_i32(int* d, long long n, void* scratch, cudaStream_t st) {
  scan_rec<int>(d, n, (int*)scratch, st);
}
void exclusive_scan_i64(long long* d, long long n, void* scratch, cudaStream_t st) {
  scan_rec<long long>(d, n, (long long*)scratch, st);
}

// ============================================================== radix sort
namespace {

constexpr int kRadThreads = 256;
constexpr int kRadWarps = kRadThreads / 32;
// 32-key rounds per warp: 4, 8 or 16 (tiles of 1024, 2048 or 4096 keys),
// chosen per sort so that the grid has about four CTAs per SM
constexpr int kRadMinTile = kRadThreads * 4;

template <typename K>
__global__ void k_bits_reduce(const K* __restrict__ keys, long long n, K* __restrict__ out_or,
                              K* __restrict__ out_and) {
  K o = 0, a = ~K(0);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    K k = keys[i];
    o |= k;
    a &= k;
  }
  for (int s = 16; s > 0; s >>= 1) {
    o |= __shfl_xor_sync(0xffffffffu, o, s);
    a &= __shfl_xor_sync(0xffffffffu, a, s);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicOr(out_or, o);
    atomicAnd(out_and, a);
  }
}

template <typename K>
__device__ __forceinline__ unsigned digit_of(K k, int shift) {
  return (unsigned)((k >> shift) & 0xffu);
}

// per-block digit histogram, digit-major layout hist[d * nblocks + b]
template <typename K, int kRadRounds>
__global__ void k_rad_hist(const K* __restrict__ keys, long long n, int shift,
                           unsigned* __restrict__ hist, unsigned nblocks) {
  constexpr int kRadTile = kRadThreads * kRadRounds;
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  long long base = (long long)blockIdx.x * kRadTile;
  for (int i = threadIdx.x; i < kRadTile; i += kRadThreads) {
    long long j = base + i;
    if (j < n) atomicAdd(&h[digit_of(keys[j], shift)], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// stable scatter: warp w owns keys [base + w*32*R, base + (w+1)*32*R) in order
template <typename K, int kRadRounds>
__global__ void k_rad_scatter(const K* __restrict__ keys, const unsigned* __restrict__ vals,
                              K* __restrict__ okeys, unsigned* __restrict__ ovals, long long n,
                              int shift, const unsigned* __restrict__ offs, unsigned nblocks) {
  constexpr int kRadTile = kRadThreads * kRadRounds;
  __shared__ unsigned wcnt[kRadWarps][256];
  __shared__ unsigned boff[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kRadWarps * 256; i += kRadThreads) (&wcnt[0][0])[i] = 0;
  boff[threadIdx.x] = offs[(size_t)threadIdx.x * nblocks + blockIdx.x];
  __syncthreads();
  const long long wbase = (long long)blockIdx.x * kRadTile + (long long)warp * (32 * kRadRounds);
  const unsigned lt = (1u << lane) - 1u;
  // pass A: per-warp digit counts
  for (int r = 0; r < kRadRounds; ++r) {
    long long j = wbase + r * 32 + lane;
    unsigned d = j < n ? digit_of(keys[j], shift) : 256u;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    if (d < 256u && (peers & lt) == 0) wcnt[warp][d] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // exclusive scan over warps per digit
  {
    unsigned d = threadIdx.x, run = 0;
    for (int w = 0; w < kRadWarps; ++w) {
      unsigned c = wcnt[w][d];
      wcnt[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
  // pass B: ranks and scatter
  for (int r = 0; r < kRadRounds; ++r) {
    long long j = wbase + r * 32 + lane;
    bool ok = j < n;
    K k = ok ? keys[j] : K(0);
    unsigned d = ok ? digit_of(k, shift) : 256u;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    unsigned pos = 0;
    if (ok) pos = boff[d] + wcnt[warp][d] + __popc(peers & lt);
    __syncwarp();
    if (ok && (peers & lt) == 0) wcnt[warp][d] += __popc(peers);
    __syncwarp();
    if (ok) {
      okeys[pos] = k;
      ovals[pos] = vals[j];
    }
  }
}

template <typename K, int kRadRounds>
void radix_pass(const K* sk, const unsigned* sv, K* dk, unsigned* dv, long long n, int shift,
                unsigned* hist, unsigned nblocks, void* sscr, cudaStream_t st) {
  {
    ::sbc::KProbe kp_(sizeof(K) == 8 ? "k_rad_hist_u64" : "k_rad_hist_u32", st,
                      (double)sizeof(K) * n);
    k_rad_hist<K, kRadRounds><<<nblocks, kRadThreads, 0, st>>>(sk, n, shift, hist, nblocks);
  }
  // exclusive scan of the digit-major histogram gives each (digit, block) its base
  scan_rec<int>((int*)hist, (long long)256 * nblocks, (int*)sscr, st);
  {
    ::sbc::KProbe kp_(sizeof(K) == 8 ? "k_rad_scatter_u64" : "k_rad_scatter_u32", st,
                      2.0 * (sizeof(K) + sizeof(unsigned)) * n);
    k_rad_scatter<K, kRadRounds><<<nblocks, kRadThreads, 0, st>>>(sk, sv, dk, dv, n, shift, hist,
                                                                nblocks);
  }
}

template <typename K>
void radix_sort_impl(K* keys, unsigned* vals, K* keys_tmp, unsigned* vals_tmp, long long n,
                     int key_bits, void* scratch, cudaStream_t st, const K* known_vary = nullptr) {
  if (n <= 1) return;
  // tile size: the largest of 4096 / 2048 / 1024 keys that still gives about
  // four CTAs per SM (152 SMs)
  const int rounds = n >= 4LL * 152 * kRadThreads * 16 ? 16 : (n >= 4LL * 152 * kRadThreads * 8 ? 8 : 4);
  const int tile = kRadThreads * rounds;
  unsigned nblocks = (unsigned)((n + tile - 1) / tile);
  // scratch: [or, and] then hist (256*nblocks u32) then scan scratch
  K* d_or = (K*)scratch;
  K* d_and = d_or + 1;
  unsigned* hist = (unsigned*)((char*)scratch + 64);
  void* sscr = (char*)scratch + 64 + (((size_t)256 * nblocks * sizeof(unsigned) + 255) / 256) * 256;
  // 64-bit keys (doubles) often have constant high digits: one OR/AND
  // reduction (and a host round trip) finds the digits worth sorting.  For
  // 32-bit keys the caller's key_bits already bounds the passes.
  K vary = ~K(0);
  if (known_vary) {
    vary = *known_vary;
  } else if (sizeof(K) == 8) {
    K h_or = 0, h_and = ~K(0);
    cudaMemcpyAsync(d_or, &h_or, sizeof(K), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_and, &h_and, sizeof(K), cudaMemcpyHostToDevice, st);
    unsigned g = (unsigned)((n + 1023) / 1024);
    if (g > 2048) g = 2048;
    {
      ::sbc::KProbe kp_("k_bits_reduce", st);
      k_bits_reduce<K><<<g, 1024, 0, st>>>(keys, n, d_or, d_and);
    }
    K o, a;
    cudaMemcpyAsync(&o, d_or, sizeof(K), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&a, d_and, sizeof(K), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    vary = o ^ a;
  }
  K* src_k = keys;
  unsigned* src_v = vals;
  K* dst_k = keys_tmp;
  unsigned* dst_v = vals_tmp;
  for (int shift = 0; shift < key_bits; shift += 8) {
    if (((vary >> shift) & K(0xff)) == 0) continue;
    if (rounds == 16)
      radix_pass<K, 16>(src_k, src_v, dst_k, dst_v, n, shift, hist, nblocks, sscr, st);
    else if (rounds == 8)
      radix_pass<K, 8>(src_k, src_v, dst_k, dst_v, n, shift, hist, nblocks, sscr, st);
    else
      radix_pass<K, 4>(src_k, src_v, dst_k, dst_v, n, shift, hist, nblocks, sscr, st);
    K* tk = src_k; src_k = dst_k; dst_k = tk;
    unsigned* tv = src_v; src_v = dst_v; dst_v = tv;
  }
  if (src_k != keys) {
    cudaMemcpyAsync(keys, src_k, sizeof(K) * n, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(vals, src_v, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, st);
  }
}

}  // namespace

size_t radix_scratch_bytes(long long n) {
  long long nblocks = (n + kRadMinTile - 1) / kRadMinTile;
  size_t h = (((size_t)256 * nblocks * sizeof(unsigned) + 255) / 256) * 256;
  return 64 + h + scan_scratch_bytes(256 * nblocks) * 2 + 256;
}

void radix_sort_u32(unsigned* keys, unsigned* vals, unsigned* keys_tmp, unsigned* vals_tmp,
                    long long n, int key_bits, void* scratch, cudaStream_t st) {
  radix_sort_impl<unsigned>(keys, vals, keys_tmp, vals_tmp, n, key_bits, scratch, st);
}

void radix_sort_u64(unsigned long long* keys, unsigned* vals, unsigned long long* keys_tmp,
                    unsigned* vals_tmp, long long n, void* scratch, cudaStream_t st) {
  radix_sort_impl<unsigned long long>(keys, vals, keys_tmp, vals_tmp, n, 64, scratch, st);
}

void radix_sort_u64_within(unsigned long long* keys, unsigned* vals, unsigned long long* keys_tmp,
                           unsigned* vals_tmp, long long n, unsigned long long lo,
                           unsigned long long hi, void* scratch, cudaStream_t st) {
  // keys in [lo, hi] share every bit above the highest bit where lo and hi differ
  const unsigned long long d = lo ^ hi;
  const unsigned long long vary = d ? (~0ull >> __builtin_clzll(d)) : 0ull;
  radix_sort_impl<unsigned long long>(keys, vals, keys_tmp, vals_tmp, n, 64, scratch, st, &vary);
}

}  // namespace sbc
