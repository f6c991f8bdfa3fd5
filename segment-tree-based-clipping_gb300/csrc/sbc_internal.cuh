// sbc_internal.cuh -- shared device helpers and declarations of the sm_103a
// segment-tree clipping pipeline.
//
// Data layout in HBM (structure of arrays, 256-byte aligned buffers):
//   polygons     bP[(nb+1)*2], cP[(sum c_i + k)*2]   interleaved x,y with the
//                closing vertex repeated (the reference's bPoly / cPoly)
//   edges        e_id[E], e_start[E], e_end[E] (+ e_type derived from index)
//   tree         ea[epc] elementary points; node intervals are derived from
//                ea on the fly (node v covers leaves [lo(v), hi(v)])
//   cover lists  cov_node[P], cov_edge[P] sorted by (node, edge index)
//   end lists    leaf entries sorted by (polygon class, leaf)
//   candidates   raw hits (bId, cId, type, emission key) -> unique records
//   merged       ring slot arrays ixB / ixC (x,y), alpha, neighbour, label
#pragma once

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace sbc {

constexpr double kEps = 0.000000001;  // EPSILON, p_seg_tree/util/constants.h:13

// ---------------------------------------------------------------- status codes
enum Status : int {
  kOk = 0,
  kEInput = 1,     // malformed input
  kEUndef = 2,     // input on which the reference's behaviour is undefined
  kENoMem = 3,
  kECuda = 4,
  kEInternal = 5,
};

// device-side error flags (bit mask written by kernels, read by the host)
enum DevFlag : unsigned {
  kFlagUndef = 1u,          // reference behaviour undefined (e.g. negative radix digit)
  kFlagOverflow = 2u,       // an output buffer was too small; host grows and retries
  kFlagSlowPath = 4u,       // back end needs the serial emulation path
  kFlagSpin = 8u,           // a bounded wait gave up
  kFlagUnsorted = 16u,      // the elementary array is not in order
  kFlagSharedX = 32u,       // two vertices share an x value (endpoint order needs the full sort)
  kFlagLongRun = 64u,       // a run of equal 32-bit vertex keys too long to fix up in place
};

// ---------------------------------------------------------------- FP64 geometry
// Every FP64 operation is an explicit round-to-nearest intrinsic so no FMA
// contraction can occur (the reference's x86-64 -O2 build has none).
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// A(P,Q,R) = (Q.x-P.x)*(R.y-P.y) - (Q.y-P.y)*(R.x-P.x)
// (p_seg_tree/oacc_segment_tree.cpp:5334-5337, foster/point2D.h:73-75)
__device__ __forceinline__ double area3(double px, double py, double qx, double qy, double rx,
                                        double ry) {
  return dsub(dmul(dsub(qx, px), dsub(ry, py)), dmul(dsub(qy, py), dsub(rx, px)));
}

// Edge-pair classification, lineSegmentIntersection(2)
// (p_seg_tree/oacc_segment_tree.cpp:5426-5611).  Returns the type 0..8 and
// the parameters alpha (on P) and beta (on Q).
__device__ __forceinline__ int seg_isect(double p1x, double p1y, double p2x, double p2y,
                                         double q1x, double q1y, double q2x, double q2y,
                                         double* alpha, double* beta) {
  double AP1 = area3(p1x, p1y, q1x, q1y, q2x, q2y);
  double AP2 = area3(p2x, p2y, q1x, q1y, q2x, q2y);
  double d = dsub(AP1, AP2);
  if (fabs(d) > kEps) {
    double AQ1 = area3(q1x, q1y, p1x, p1y, p2x, p2y);
    double AQ2 = area3(q2x, q2y, p1x, p1y, p2x, p2y);
    double a = ddiv(AP1, d);
    double b = ddiv(AQ1, dsub(AQ1, AQ2));
    *alpha = a;
    *beta = b;
    bool a01 = false, a0 = false, b01 = false, b0 = false;
    if (a > kEps && a < 1.0 - kEps) a01 = true;
    else if (fabs(a) <= kEps) a0 = true;
    if (b > kEps && b < 1.0 - kEps) b01 = true;
    else if (fabs(b) <= kEps) b0 = true;
    if (a01 && b01) return 1;
    if (a0 && b01) return 2;
    if (b0 && a01) return 3;
    if (a0 && b0) return 4;
  } else if (fabs(AP1) < kEps) {
    double dPx = dsub(p2x, p1x), dPy = dsub(p2y, p1y);
    double dQx = dsub(q2x, q1x), dQy = dsub(q2y, q1y);
    double PQx = dsub(q1x, p1x), PQy = dsub(q1y, p1y);
    double a = ddiv(dadd(dmul(PQx, dPx), dmul(PQy, dPy)), dadd(dmul(dPx, dPx), dmul(dPy, dPy)));
    double b = ddiv(-dadd(dmul(PQx, dQx), dmul(PQy, dQy)), dadd(dmul(dQx, dQx), dmul(dQy, dQy)));
    *alpha = a;
    *beta = b;
    bool a01 = false, a0 = false, an = false, b01 = false, b0 = false, bn = false;
    if (a > kEps && a < 1.0 - kEps) a01 = true;
    else if (fabs(a) <= kEps) a0 = true;
    else an = true;
    // the reference classifies beta's zero case with fabs(alpha) (:5595)
    if (b > kEps && b < 1.0 - kEps) b01 = true;
    else if (fabs(a) <= kEps) b0 = true;
    else bn = true;
    if (a01 && b01) return 5;
    if (an && b01) return 6;
    if (bn && a01) return 7;
    if (a0 && b0) return 8;
  }
  return 0;
}

// alphaToInt (oacc_segment_tree.cpp:7247-7252) with the x86-64 truncating
// conversion: values outside int range become INT_MIN.
__device__ __forceinline__ int alpha_to_int(double a) {
  if (a < kEps) return 0;
  double v = dmul(1000000000.0, a);
  if (!(v > -2147483649.0 && v < 2147483648.0)) return (int)0x80000000;
  return __double2int_rz(v);
}

// Order-preserving 64-bit key of a double (-0.0 folded onto +0.0 so the two
// compare equal, as the reference's `<` / `==` do).
__device__ __forceinline__ unsigned long long dkey(double x) {
  unsigned long long u = (unsigned long long)__double_as_longlong(x == 0.0 ? 0.0 : x);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
// A signed order key of a finite double by integer operations alone:
// x < y  <=>  okey(x) < okey(y), and -0.0, +0.0 share the key 0.  On GB300 an
// FP64 compare issues at the FP64 rate (a small fraction of the integer
// rate), so comparison-only work runs on these keys.
__device__ __forceinline__ long long okey(double x) {
  const long long u = __double_as_longlong(x);
  return u >= 0 ? u : -(u & 0x7fffffffffffffffll);
}

// LSMF, the reference's bounding-box filter of an edge pair
// (oacc_segment_tree.cpp:5282-5316: the min/max swaps and the four
// separation tests), on order keys: the same decisions as on the doubles
__device__ __forceinline__ bool lsmf_keys(long long p1x, long long p1y, long long p2x,
                                          long long p2y, long long q1x, long long q1y,
                                          long long q2x, long long q2y) {
  const long long minPX = p1x > p2x ? p2x : p1x, maxPX = p1x > p2x ? p1x : p2x;
  const long long minPY = p1y > p2y ? p2y : p1y, maxPY = p1y > p2y ? p1y : p2y;
  const long long minQX = q1x > q2x ? q2x : q1x, maxQX = q1x > q2x ? q1x : q2x;
  const long long minQY = q1y > q2y ? q2y : q1y, maxQY = q1y > q2y ? q1y : q2y;
  if (minPX > maxQX || maxPX < minQX) return false;
  if (minPY > maxQY || maxPY < minQY) return false;
  return true;
}

// the value of an order key
__device__ __forceinline__ double dkey_value(unsigned long long k) {
  const unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}

// ---------------------------------------------------------------- block reductions
// Sum (or min) over the block, then one atomic per block: same-address
// atomics from every warp of a large grid serialise at the L2.  Every
// thread of the block must call these (blockDim a multiple of 32, <= 1024).
template <typename T>
__device__ __forceinline__ T block_sum(T v) {
  __shared__ T part[32];
  for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) part[w] = v;
  __syncthreads();
  T t = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < nw; ++i) t += part[i];
  return t;  // valid in thread 0
}

__device__ __forceinline__ unsigned block_min(unsigned v) {
  __shared__ unsigned part[32];
  v = __reduce_min_sync(0xffffffffu, v);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) part[w] = v;
  __syncthreads();
  unsigned t = 0xffffffffu;
  if (threadIdx.x == 0)
    for (int i = 0; i < nw; ++i) t = part[i] < t ? part[i] : t;
  return t;  // valid in thread 0
}

// ---------------------------------------------------------------- findBoarder on positions
// The border sequence S(m) of preparePointsToNodeMapMulticore
// (oacc_segment_tree.cpp:1970-2008) is the sorted elementary array ea with
// the never-written slot read as 0.0 moved to position z: S(m) = ea[m+1] for
// m < z, 0.0 at z, ea[m] above, past the arrays NaN.  When ea is sorted and
// the entries equal to q sit at positions [lo, hi) of ea, comparing S(m)
// with q needs no memory access.  Returns -1 smaller, 0 equal, 1 greater,
// 2 past the arrays.
// cz: the comparison at the zero slot, (0.0 == q) ? 0 : (0.0 < q ? -1 : 1),
// taken once per search
__device__ __forceinline__ int border_cmp(int epc, int z, int m, int lo, int hi, int cz) {
  if (m < 0 || m >= epc) return 2;
  if (m == z) return cz;
  const int t = m < z ? m + 1 : m;
  return t < lo ? -1 : (t < hi ? 0 : 1);
}

// findBoarder (oacc_segment_tree.cpp:420-460), its search path followed on
// positions (including the misses the zero slot causes)
__device__ __forceinline__ int border_by_position(int epc, int z, int lo, int hi, double q) {
  const int cz = (0.0 == q) ? 0 : (0.0 < q ? -1 : 1);
  int l = 0, h = epc;
  while (l < h) {
    const int m = l + (h - l) / 2;
    const int c = border_cmp(epc, z, m, lo, hi, cz);
    if (c == 0) {
      if (border_cmp(epc, z, m - 1, lo, hi, cz) != 0) {
        h = m;
        l = h;
      } else {
        h = m - 1;
      }
    } else if (c == -1) {
      l = m + 1;
    } else {
      h = m - 1;
    }
  }
  return border_cmp(epc, z, h, lo, hi, cz) == 0 ? h : -1;
}

// ---------------------------------------------------------------- primitives
// (sbc_prims.cu)  All run on `st`; scratch comes from the caller.
size_t scan_scratch_bytes(long long n);
// exclusive scan in place over n int32 (or int64) values.  The scan leaves
// the look-back words of its scratch zero; state_zero says the scratch is
// known to start zero (allocated zeroed and only used by scans), which saves
// a memset per scan.
void exclusive_scan_i32(int* d, long long n, void* scratch, cudaStream_t st,
                        bool state_zero = false);
void exclusive_scan_i64(long long* d, long long n, void* scratch, cudaStream_t st,
                        bool state_zero = false);
// up to 4 independent exclusive scans in one launch (arrays d[i] of n[i]
// int32 values); the scratch holds scan_set_scratch_bytes(max n, count)
// bytes, left zero as the single scans leave theirs
size_t scan_set_scratch_bytes(long long n_max, int count);
void exclusive_scan_i32_set(int* const* d, const long long* n, int count, void* scratch,
                            cudaStream_t st, bool state_zero = false);
// true (and cleared) if a scan's bounded look-back wait gave up since the last call
bool scan_error_take();
// the device address of the scans' error word (for a read queued on a
// stream); nullptr if it cannot be had
unsigned* scan_error_word();

// Stable LSD radix sort of (key, value) pairs, 8-bit digits, only the digit
// positions that vary are sorted.  keys/vals are sorted in place; tmp buffers
// of the same sizes plus `radix_scratch_bytes(n)` bytes are needed; n < 2^32.
// No host synchronisation.
size_t radix_scratch_bytes(long long n);
void radix_sort_u32(unsigned* keys, unsigned* vals, unsigned* keys_tmp, unsigned* vals_tmp,
                    long long n, int key_bits, void* scratch, cudaStream_t st);
void radix_sort_u64(unsigned long long* keys, unsigned* vals, unsigned long long* keys_tmp,
                    unsigned* vals_tmp, long long n, void* scratch, cudaStream_t st);
// the same for keys known to lie in [lo, hi]: the digits above the highest bit
// where lo and hi differ are constant, so no reduction (and no host round
// trip) is needed to skip them
void radix_sort_u64_within(unsigned long long* keys, unsigned* vals, unsigned long long* keys_tmp,
                           unsigned* vals_tmp, long long n, unsigned long long lo,
                           unsigned long long hi, void* scratch, cudaStream_t st);

// number of this library's kernels launched by the process (any host thread)
extern std::atomic<unsigned long long> g_launches;

// Scoped launch probe: counts the launch and, while profiling is on, brackets
// it with a pair of CUDA events on its stream (per-kernel device time).
// `bytes` is the launch's algorithmic traffic (its inputs read and outputs
// written once; 0 where none is stated), summed per kernel for rooflines.
struct KProbe {
  KProbe(const char* name, cudaStream_t st, double bytes = 0.0);
  ~KProbe();
  const char* name_;
  cudaStream_t st_;
  int slot_;
};
void profile_begin();
// per-launch events stay out of a graph being captured
bool profiling_on();
bool profiling_suspend();
void profiling_restore(bool on);
// aggregated per kernel name: returns the number of distinct kernels
struct TimelineRec {
  const char* name;
  float start_ms, dur_ms;
  int stream;
};
int profile_end(std::vector<std::string>* names, std::vector<float>* ms, std::vector<int>* counts,
                std::vector<double>* bytes = nullptr);
// the launches of the window profile_end closed, in launch order
const std::vector<TimelineRec>& profile_timeline();

inline unsigned grid_for(long long n, int per_block) {
  long long g = (n + per_block - 1) / per_block;
  return (unsigned)(g > 0 ? g : 1);
}

}  // namespace sbc

