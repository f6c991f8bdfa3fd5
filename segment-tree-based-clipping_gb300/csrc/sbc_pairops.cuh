// sbc_pairops.cuh -- per-pair device helpers shared by the engines that clip
// one pair per device thread: the batched small-pair engine (sbc_batch.cu)
// and the one-base-many-overlays engine (sbc_pairwise.cu).
#pragma once

#include "sbc_internal.cuh"

namespace sbc {
namespace {

// Arrays of one pair, carved in a fixed order from a base pointer (a null
// base gives the byte count).
struct Carver {
  unsigned char* base;
  size_t off;
  template <class T>
  __host__ __device__ T* take(long long n) {
    off = (off + 15) & ~(size_t)15;
    T* r = (T*)(base + off);
    off += sizeof(T) * (size_t)(n > 0 ? n : 0);
    return r;
  }
};

__host__ __device__ __forceinline__ int npow2_dev(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

// ------------------------------------------------------------------ small helpers
__device__ __forceinline__ double bvx(const double* p, int n, int i) { return p[2 * (i % n)]; }
__device__ __forceinline__ double bvy(const double* p, int n, int i) { return p[2 * (i % n) + 1]; }

__device__ __forceinline__ bool lsmf_d(double p1x, double p1y, double p2x, double p2y, double q1x,
                                       double q1y, double q2x, double q2y) {
  // on order keys: integer compares instead of FP64 ones, same decisions
  return lsmf_keys(okey(p1x), okey(p1y), okey(p2x), okey(p2y), okey(q1x), okey(q1y), okey(q2x),
                   okey(q2y));
}

// stable bottom-up merge sort of idx[0..n) by less(a, b)
template <class Less>
__device__ void merge_sort(int* idx, int* tmp, int n, Less less) {
  for (int w = 1; w < n; w <<= 1) {
    for (int lo = 0; lo < n; lo += 2 * w) {
      const int mid = min(lo + w, n), hi = min(lo + 2 * w, n);
      int i = lo, j = mid, o = lo;
      while (i < mid && j < hi) tmp[o++] = less(idx[j], idx[i]) ? idx[j++] : idx[i++];
      while (i < mid) tmp[o++] = idx[i++];
      while (j < hi) tmp[o++] = idx[j++];
    }
    for (int i = 0; i < n; ++i) idx[i] = tmp[i];
  }
}

__device__ __forceinline__ bool canonical_s(int v, int logL, int l, int r1) {
  const int L = 1 << logL;
  const int d = 31 - __clz(v), h = logL - d;
  const int lo = (v << h) - L, hi = ((v + 1) << h) - L;
  if (lo < l || hi > r1) return false;
  if (v == 1) return true;
  const int p = v >> 1;
  const int plo = (p << (h + 1)) - L, phi = ((p + 1) << (h + 1)) - L;
  return !(plo >= l && phi <= r1);
}

__device__ __forceinline__ bool below_s(int x, int v, int logL) {
  if (x < 0) return false;
  const int h = logL - (31 - __clz(v));
  return (x >> h) == v;
}

// Emission count and first-emission key of base edge b with overlay edge c
// (the candidate loops of saveIntersectionsIdsMulticore,
// oacc_segment_tree.cpp:6010-6244, as a rule over the two edges): rb, rc are
// the edges' covered leaf ranges [l, r1), eb0/eb1 and ec0/ec1 their end-list
// leaves (aft, bef; -1 when dropped); c is the overlay edge's index in the
// pair's edge numbering and cId its id.  Kind 0 (v in both cover lists) and
// kind 1 (v covers b, c ends below v) carry cId; kind 2 (v covers c, b ends
// below v) carries c.
__device__ unsigned emission_q(int2 rb, int2 rc, int eb0, int eb1, int ec0, int ec1, int c,
                               int cId, int logL, unsigned long long* key) {
  const int L = 1 << logL;
  unsigned n = 0;
  unsigned long long best = ~0ull;
  for (int a = rb.x + L, z = rb.y + L; a < z; a >>= 1, z >>= 1) {
    for (int side = 0; side < 2; ++side) {
      int v = -1;
      if (side == 0 && (a & 1)) v = a++;
      if (side == 1 && (z & 1)) v = --z;
      if (v < 0) continue;
      if (canonical_s(v, logL, rc.x, rc.y)) {
        n += 2;
        best = min(best, ((unsigned long long)v << 33) | (unsigned)cId);
      }
      if (below_s(ec0, v, logL) || below_s(ec1, v, logL)) {
        n += 1;
        best = min(best, ((unsigned long long)v << 33) | (1ull << 31) | (unsigned)cId);
      }
    }
  }
  for (int a = rc.x + L, z = rc.y + L; a < z; a >>= 1, z >>= 1) {
    for (int side = 0; side < 2; ++side) {
      int v = -1;
      if (side == 0 && (a & 1)) v = a++;
      if (side == 1 && (z & 1)) v = --z;
      if (v < 0) continue;
      if (below_s(eb0, v, logL) || below_s(eb1, v, logL)) {
        n += 1;
        best = min(best, ((unsigned long long)v << 33) | (1ull << 32) | (unsigned)c);
      }
    }
  }
  *key = best;
  return n;
}

__device__ __forceinline__ bool nd_b(int t) { return t == 1 || t == 3 || t == 5 || t == 7; }
__device__ __forceinline__ bool nd_c(int t) { return t == 1 || t == 2 || t == 6; }

// status codes of one pair
enum { PS_OK = 0, PS_UNDEF = 2, PS_CAP = 3 };

}  // namespace
}  // namespace sbc
