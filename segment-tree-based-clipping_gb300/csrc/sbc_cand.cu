// sbc_cand.cu -- candidate edge pairs (reference row A8) without the node
// enumeration.
//
// The reference (saveIntersectionsIdsMulticore, p_seg_tree/oacc_segment_tree.cpp:
// 6108-6244) walks every tree node with a cover list and tests every ordered
// pair in cover x cover and cover x end list.  A pair (b, c) of a base and an
// overlay edge is emitted at node v exactly when
//   kind 0: v is in the cover lists of both (emitted twice, once per order),
//   kind 1: v is in b's cover list and c has an end-list leaf below v,
//   kind 2: v is in c's cover list and b has an end-list leaf below v,
// and the emission is kept when LSMF passes and the classification is not 0.
// Only box-overlapping pairs can pass LSMF, so this file finds those with a
// uniform grid over float edge boxes, and derives from each pair's two
// cover decompositions and end leaves (a) how many times the reference emits
// it and (b) its first emission in the reference's order: smallest node,
// then the cover entry b before c, then cover x cover before cover x end,
// then the partner's id.  That key orders the unique pairs of one base edge
// exactly as the reference's stable sort + first-occurrence dedup does
// (src/clip.cpp:441-493).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "sbc_pipeline.cuh"

namespace sbc {

namespace {

constexpr int kLongCells = 1024;  // edges spanning more cells are joined by brute force
constexpr int kGBlock = 256;
constexpr int kGSmallMax = 64;    // cell products up to this size: one thread each
constexpr int kGStage = 512;      // survivors staged per warp in shared memory

__device__ __forceinline__ int class_of_edge(const int* tstart, int k, int e) {
  int c = 0;
  while (c < k && tstart[c + 1] <= e) ++c;
  return c;
}

__device__ __forceinline__ unsigned fkey(float f) {
  unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// ------------------------------------------------------------------ grid
struct Grid {
  float x0, y0, inv;
  int gx, gy;
  __device__ __forceinline__ int cx(float x) const {
    int c = (int)floorf(__fmul_rn(__fsub_rn(x, x0), inv));
    return min(max(c, 0), gx - 1);
  }
  __device__ __forceinline__ int cy(float y) const {
    int c = (int)floorf(__fmul_rn(__fsub_rn(y, y0), inv));
    return min(max(c, 0), gy - 1);
  }
};

// Float edge boxes (bounds rounded outwards), the bounding box of the base's
// edges and of the overlays' edges, and the summed extent.  bnd holds order
// keys: [0..3] base box, [4..7] overlay box (min x, min y, max x, max y).
__global__ void k_edge_fbox(int E, const int* __restrict__ e_id, const int* __restrict__ tstart,
                            int k, const double* __restrict__ bP, const double* __restrict__ cP,
                            float4* __restrict__ fbox, unsigned* __restrict__ bnd,
                            double* __restrict__ sum_ext) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  // per class (0 base, 1 overlays): min x, min y, max x, max y as order keys
  unsigned kb[2][4] = {{0xffffffffu, 0xffffffffu, 0u, 0u}, {0xffffffffu, 0xffffffffu, 0u, 0u}};
  float ext = 0.f;
  if (e < E) {
    const int cl = class_of_edge(tstart, k, e) == 0 ? 0 : 1;
    const double* p = (cl == 0 ? bP : cP) + e_id[e];
    const float4 f = make_float4(__double2float_rd(fmin(p[0], p[2])), __double2float_rd(fmin(p[1], p[3])),
                                 __double2float_ru(fmax(p[0], p[2])), __double2float_ru(fmax(p[1], p[3])));
    fbox[e] = f;
    kb[cl][0] = fkey(f.x);
    kb[cl][1] = fkey(f.y);
    kb[cl][2] = fkey(f.z);
    kb[cl][3] = fkey(f.w);
    ext = fmaxf(f.z - f.x, f.w - f.y);
  }
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      kb[c][0] = min(kb[c][0], __shfl_xor_sync(0xffffffffu, kb[c][0], o));
      kb[c][1] = min(kb[c][1], __shfl_xor_sync(0xffffffffu, kb[c][1], o));
      kb[c][2] = max(kb[c][2], __shfl_xor_sync(0xffffffffu, kb[c][2], o));
      kb[c][3] = max(kb[c][3], __shfl_xor_sync(0xffffffffu, kb[c][3], o));
    }
    ext += __shfl_xor_sync(0xffffffffu, ext, o);
  }
  // one set of atomics per block (same-address atomics serialise)
  __shared__ unsigned sk[8][8];
  __shared__ float se[8];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    for (int j = 0; j < 8; ++j) sk[j][w] = kb[j >> 2][j & 3];
    se[w] = ext;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    const int j = threadIdx.x, nw = blockDim.x >> 5;
    unsigned v = sk[j][0];
    for (int i = 1; i < nw; ++i) v = (j & 3) < 2 ? min(v, sk[j][i]) : max(v, sk[j][i]);
    if ((j & 3) < 2) atomicMin(&bnd[j], v);
    else atomicMax(&bnd[j], v);
  }
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    double es = 0.0;
    for (int i = 0; i < nw; ++i) es += se[i];
    atomicAdd(sum_ext, es);
  }
}

// Grid entries are grouped by bucket = cell * (k + 1) + polygon class (a
// counting sort: the order inside a bucket does not matter, each pair is a
// set element and its emission key fixes its final order).  Edges spanning
// more than kLongCells cells go to long_list instead.
// Common-MBR filter (the reference's getCMBR, src/clip.cpp:743-777): an edge
// whose box misses the intersection of the base's and the overlays' boxes
// overlaps no edge of the other polygon, so it never forms a candidate pair.
// Such an edge gets islong = 2 and enters neither the grid nor the long list
// (the tree build keeps every edge: the elementary points do not change).
__global__ void k_grid_count(int E, const float4* __restrict__ fbox, Grid g,
                             const int* __restrict__ tstart, int k, int* __restrict__ bcnt,
                             unsigned char* __restrict__ islong, int* __restrict__ long_list,
                             unsigned* __restrict__ long_count, float4 cmbr,
                             unsigned* __restrict__ outside) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const float4 f = fbox[e];
  if (f.x > cmbr.z || f.z < cmbr.x || f.y > cmbr.w || f.w < cmbr.y) {
    islong[e] = 2;
    atomicAdd(outside, 1u);
    return;
  }
  const int x0 = g.cx(f.x), x1 = g.cx(f.z), y0 = g.cy(f.y), y1 = g.cy(f.w);
  const long long n = (long long)(x1 - x0 + 1) * (y1 - y0 + 1);
  const bool lg = n > kLongCells;
  islong[e] = lg ? 1 : 0;
  if (lg) {
    long_list[atomicAdd(long_count, 1u)] = e;
    return;
  }
  const int cls = class_of_edge(tstart, k, e);
  for (int y = y0; y <= y1; ++y)
    for (int x = x0; x <= x1; ++x) atomicAdd(&bcnt[((long long)y * g.gx + x) * (k + 1) + cls], 1);
}

__global__ void k_grid_scatter(int E, const float4* __restrict__ fbox, Grid g,
                               const int* __restrict__ tstart, int k, const int* __restrict__ bstart,
                               int* __restrict__ fill, const unsigned char* __restrict__ islong,
                               unsigned* __restrict__ vals) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E || islong[e]) return;
  const float4 f = fbox[e];
  const int x0 = g.cx(f.x), x1 = g.cx(f.z), y0 = g.cy(f.y), y1 = g.cy(f.w);
  const int cls = class_of_edge(tstart, k, e);
  for (int y = y0; y <= y1; ++y)
    for (int x = x0; x <= x1; ++x) {
      const long long bkt = ((long long)y * g.gx + x) * (k + 1) + cls;
      vals[bstart[bkt] + atomicAdd(&fill[bkt], 1)] = (unsigned)e;
    }
}

// per cell: {first base entry, base entries, first cType entry, cType
// entries}; whether it is a small product (one thread) and its warp tiles
// otherwise
__global__ void k_cell_items(int nCells, const int* __restrict__ bstart, int k, int cType,
                             int4* __restrict__ cdesc, int* __restrict__ smalls,
                             int* __restrict__ tiles, long long* __restrict__ work) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c > nCells) return;
  if (c == nCells) {
    smalls[c] = 0;
    tiles[c] = 0;
    work[c] = 0;
    return;
  }
  const long long b0 = (long long)c * (k + 1);
  const int a = bstart[b0], nB = bstart[b0 + 1] - a;
  const int cs = bstart[b0 + cType], nC = bstart[b0 + cType + 1] - cs;
  const long long prod = (long long)nB * nC;
  cdesc[c] = make_int4(a, nB, cs, nC);
  smalls[c] = (prod > 0 && prod <= kGSmallMax) ? 1 : 0;
  tiles[c] = prod > kGSmallMax ? (nC + 31) / 32 : 0;
  work[c] = prod;
}

__global__ void k_cell_expand(int nCells, const int* __restrict__ smalls,
                              const int* __restrict__ tiles, int* __restrict__ srec,
                              int2* __restrict__ wrec) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nCells) return;
  if (smalls[c + 1] != smalls[c]) srec[smalls[c]] = c;
  for (int t = 0, w = tiles[c]; w < tiles[c + 1]; ++t, ++w) wrec[w] = make_int2(c, t);
}

// ---- survivor staging (per warp, shared memory; one atomic per flush)
struct Stage {
  int2* buf;
  int n;
};

__device__ __forceinline__ void st_flush(Stage& s, int lane, unsigned long long* counter,
                                         long long cap, int2* out) {
  __syncwarp();
  if (s.n == 0) return;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(counter, (unsigned long long)s.n);
  base = __shfl_sync(0xffffffffu, base, 0);
  for (int k = lane; k < s.n; k += 32) {
    const long long w = (long long)base + k;
    if (w < cap) out[w] = s.buf[k];
  }
  __syncwarp();
  s.n = 0;
}

__device__ __forceinline__ void st_push(Stage& s, int lane, bool hit, int2 v,
                                        unsigned long long* counter, long long cap, int2* out) {
  const unsigned b = __ballot_sync(0xffffffffu, hit);
  if (b == 0) return;
  if (hit) s.buf[s.n + __popc(b & ((1u << lane) - 1u))] = v;
  s.n += __popc(b);
  if (s.n > kGStage - 32) st_flush(s, lane, counter, cap, out);
}

// boxes overlap, and the lower corner of their overlap lies in cell (gxc,
// gyc): each overlapping pair is reported by exactly one of the cells both
// boxes touch
__device__ __forceinline__ bool pair_here(const float4& a, const float4& b, const Grid& g, int gxc,
                                          int gyc) {
  if (a.x > b.z || a.z < b.x || a.y > b.w || a.w < b.y) return false;
  return g.cx(fmaxf(a.x, b.x)) == gxc && g.cy(fmaxf(a.y, b.y)) == gyc;
}

// small cell products: one thread per cell, the warp's threads in lockstep
__global__ void __launch_bounds__(kGBlock)
k_grid_small(const int* __restrict__ srec, int nS, const int4* __restrict__ cdesc,
             const unsigned* __restrict__ vals,
             const float4* __restrict__ fbox, Grid g, unsigned long long* __restrict__ counter,
             long long cap, int2* __restrict__ out) {
  __shared__ int2 stage[kGBlock / 32][kGStage];
  const int lane = threadIdx.x & 31;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i - lane >= nS) return;  // warp-uniform; no block-wide barrier follows
  Stage st{stage[threadIdx.x >> 5], 0};
  int4 d = make_int4(0, 0, 0, 1);
  int gxc = 0, gyc = 0, prod = 0;
  if (i < nS) {
    const int cell = srec[i];
    d = cdesc[cell];
    gxc = cell % g.gx;
    gyc = cell / g.gx;
    prod = d.y * d.w;
  }
  const int maxp = __reduce_max_sync(0xffffffffu, prod);
  int ib = 0, ic = 0, be = 0;
  float4 bb = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int k2 = 0; k2 < maxp; ++k2) {
    bool hit = false;
    int ce = 0;
    if (k2 < prod) {
      if (ic == 0) {
        be = (int)vals[d.x + ib];
        bb = fbox[be];
      }
      ce = (int)vals[d.z + ic];
      hit = pair_here(bb, fbox[ce], g, gxc, gyc);
      if (++ic == d.w) {
        ic = 0;
        ++ib;
      }
    }
    st_push(st, lane, hit, make_int2(be, ce), counter, cap, out);
  }
  st_flush(st, lane, counter, cap, out);
}

// larger cell products: one warp per 32 overlay entries of a cell, base
// entries broadcast 32 at a time
__global__ void __launch_bounds__(kGBlock)
k_grid_warp(const int2* __restrict__ wrec, int nW, const int4* __restrict__ cdesc,
            const unsigned* __restrict__ vals,
            const float4* __restrict__ fbox, Grid g, unsigned long long* __restrict__ counter,
            long long cap, int2* __restrict__ out) {
  __shared__ int2 stage[kGBlock / 32][kGStage];
  const int lane = threadIdx.x & 31;
  const long long it = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (it >= nW) return;  // warp-uniform; no block-wide barrier follows
  Stage st{stage[threadIdx.x >> 5], 0};
  const int2 r = wrec[it];
  const int4 d = cdesc[r.x];
  const int gxc = r.x % g.gx, gyc = r.x / g.gx;
  const int j = r.y * 32 + lane;
  const bool cvalid = j < d.w;
  const int ce = cvalid ? (int)vals[d.z + j] : 0;
  const float4 cb = cvalid ? fbox[ce] : make_float4(0.f, 0.f, 0.f, 0.f);
  for (int b0 = 0; b0 < d.y; b0 += 32) {
    const int nthis = min(32, d.y - b0);
    int mye = 0;
    float4 myb = make_float4(0.f, 0.f, 0.f, 0.f);
    if (lane < nthis) {
      mye = (int)vals[d.x + b0 + lane];
      myb = fbox[mye];
    }
    for (int k2 = 0; k2 < nthis; ++k2) {
      float4 bb;
      bb.x = __shfl_sync(0xffffffffu, myb.x, k2);
      bb.y = __shfl_sync(0xffffffffu, myb.y, k2);
      bb.z = __shfl_sync(0xffffffffu, myb.z, k2);
      bb.w = __shfl_sync(0xffffffffu, myb.w, k2);
      const int be = __shfl_sync(0xffffffffu, mye, k2);
      const bool hit = cvalid && pair_here(bb, cb, g, gxc, gyc);
      st_push(st, lane, hit, make_int2(be, ce), counter, cap, out);
    }
  }
  st_flush(st, lane, counter, cap, out);
}

// edges too long for the grid: one warp per long edge against every edge of
// the other polygon (long x long pairs once, from the base side)
__global__ void __launch_bounds__(kGBlock)
k_grid_long(const int* __restrict__ long_list, const unsigned* __restrict__ long_count,
            const int* __restrict__ tstart, int cType, const unsigned char* __restrict__ islong,
            const float4* __restrict__ fbox, unsigned long long* __restrict__ counter, long long cap,
            int2* __restrict__ out) {
  __shared__ int2 stage[kGBlock / 32][kGStage];
  const int lane = threadIdx.x & 31;
  Stage st{stage[threadIdx.x >> 5], 0};
  const unsigned nl = *long_count;
  const long long nw = (long long)gridDim.x * (kGBlock / 32);
  for (long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nl; w += nw) {
    const int e = long_list[w];
    const bool isBase = e < tstart[1];
    if (!isBase && (e < tstart[cType] || e >= tstart[cType + 1])) continue;  // other overlay
    const int o0 = isBase ? tstart[cType] : 0, o1 = isBase ? tstart[cType + 1] : tstart[1];
    const float4 fe = fbox[e];
    for (int ob = o0; ob < o1; ob += 32) {
      const int o = ob + lane;
      bool hit = false;
      if (o < o1 && (isBase || !islong[o])) {
        const float4 fo = fbox[o];
        hit = !(fe.x > fo.z || fe.z < fo.x || fe.y > fo.w || fe.w < fo.y);
      }
      st_push(st, lane, hit, isBase ? make_int2(e, o) : make_int2(o, e), counter, cap, out);
    }
  }
  st_flush(st, lane, counter, cap, out);
}

// ------------------------------------------------------------------ emission
// Node v's leaf range is [lo, hi) (leaf indices); canonical for [l, r1) when
// contained in it and its parent is not.
__device__ __forceinline__ bool canonical(int v, int logL, int l, int r1) {
  const int L = 1 << logL;
  const int d = 31 - __clz(v), h = logL - d;
  const int lo = (v << h) - L, hi = ((v + 1) << h) - L;
  if (lo < l || hi > r1) return false;
  if (v == 1) return true;
  const int p = v >> 1;
  const int plo = (p << (h + 1)) - L, phi = ((p + 1) << (h + 1)) - L;
  return !(plo >= l && phi <= r1);
}

// leaf node x (or -1) lies below node v
__device__ __forceinline__ bool below(int x, int v, int logL) {
  if (x < 0) return false;
  const int h = logL - (31 - __clz(v));
  return (x >> h) == v;
}

// How many times the reference emits base edge b with overlay edge c, and
// the key of the first emission: node << 33 | (cover entry is c) << 32 |
// payload, payload = phase << 31 | cId for cover entry b (phase 0 cover x
// cover, 1 cover x end) and c's edge index for cover entry c.
__device__ __forceinline__ unsigned emission(int b, int c, int cId, const int2* __restrict__ lr,
                                             const int* __restrict__ aft,
                                             const int* __restrict__ bef, int logL,
                                             unsigned long long* key) {
  const int L = 1 << logL;
  const int2 rb = lr[b], rc = lr[c];
  const int eb0 = aft[b], eb1 = bef[b], ec0 = aft[c], ec1 = bef[c];
  unsigned n = 0;
  unsigned long long best = ~0ull;
  int a = rb.x + L, z = rb.y + L;
  while (a < z) {
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      int v = -1;
      if (side == 0 && (a & 1)) v = a++;
      if (side == 1 && (z & 1)) v = --z;
      if (v < 0) continue;
      if (canonical(v, logL, rc.x, rc.y)) {
        n += 2;
        best = min(best, ((unsigned long long)v << 33) | (unsigned)cId);
      }
      if (below(ec0, v, logL) || below(ec1, v, logL)) {
        n += 1;
        best = min(best, ((unsigned long long)v << 33) | (1ull << 31) | (unsigned)cId);
      }
    }
    a >>= 1;
    z >>= 1;
  }
  a = rc.x + L;
  z = rc.y + L;
  while (a < z) {
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      int v = -1;
      if (side == 0 && (a & 1)) v = a++;
      if (side == 1 && (z & 1)) v = --z;
      if (v < 0) continue;
      if (below(eb0, v, logL) || below(eb1, v, logL)) {
        n += 1;
        best = min(best, ((unsigned long long)v << 33) | (1ull << 32) | (unsigned)c);
      }
    }
    a >>= 1;
    z >>= 1;
  }
  *key = best;
  return n;
}

// ------------------------------------------------------------------ exact stage
__device__ __forceinline__ float vdx(const float4& a, const float4& b) {
  return __fadd_rn(__fsub_rn(a.x, b.x), __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ float vdy(const float4& a, const float4& b) {
  return __fadd_rn(__fsub_rn(a.y, b.y), __fsub_rn(a.w, b.w));
}
__device__ __forceinline__ float fcross(float ax, float ay, float bx, float by) {
  return __fsub_rn(__fmul_rn(ax, by), __fmul_rn(ay, bx));
}

// True only when lineSegmentIntersection2 (seg_isect) certainly returns 0
// for P = (p1, p2), Q = (q1, q2), decided in float from vertex hi/lo pairs.
//
// With a = q1 - p1, b = q2 - p1, w = p2 - p1 the four areas seg_isect uses
// are AP1 = a x b, AQ1 = w x a, AQ2 = w x b and AP2 = AP1 + AQ1 - AQ2.
//  * If AP1 and AP2 have the same strict sign, |AP1| > 2e-9 and
//    |AP1| > 2e-9 |AP2|, then alpha = AP1 / (AP1 - AP2) is > 1 or
//    < -EPSILON, and the collinear branch (|AP1| < EPSILON) is excluded:
//    the type is 0.
//  * If AQ1 and AQ2 have the same strict sign, |AQ1| > 2e-9 |AQ2| and
//    |AP1| > 2e-9, then beta is > 1 or < -EPSILON in the general branch and
//    the collinear branch is excluded again: the type is 0.
// Segments that do not meet satisfy one of the two unless they are within
// the float error of touching.  Each float area carries the bound
// 32 u m^2 + 64 u^2 m M (u = 2^-24, m = largest difference component,
// M = coordinate magnitude), at least 2.6 times the worst case of the
// difference and product rounding; the FP64 areas of seg_isect differ from
// the exact ones by about 1e-15 m^2, far inside it.
__device__ __forceinline__ bool certainly_disjoint(const float4& p1, const float4& p2,
                                                   const float4& q1, const float4& q2) {
  const float ax = vdx(q1, p1), ay = vdy(q1, p1);
  const float bx = vdx(q2, p1), by = vdy(q2, p1);
  const float wx = vdx(p2, p1), wy = vdy(p2, p1);
  const float AP1 = fcross(ax, ay, bx, by);
  const float AQ1 = fcross(wx, wy, ax, ay);
  const float AQ2 = fcross(wx, wy, bx, by);
  const float AP2 = __fsub_rn(__fadd_rn(AP1, AQ1), AQ2);
  const float m = fmaxf(fmaxf(fmaxf(fabsf(ax), fabsf(ay)), fmaxf(fabsf(bx), fabsf(by))),
                        fmaxf(fabsf(wx), fabsf(wy)));
  const float M = __fadd_rn(fmaxf(fabsf(p1.x), fabsf(p1.y)), __fmul_rn(2.f, m));
  const float u = 5.9604645e-8f;  // 2^-24
  const float Bx = __fadd_rn(__fmul_rn(__fmul_rn(32.f * u, m), m),
                             __fadd_rn(__fmul_rn(__fmul_rn(64.f * u * u, m), M), 1e-30f));
  const float B2 = __fadd_rn(__fmul_rn(3.f, Bx),
                             __fmul_rn(4.f * u, __fadd_rn(__fadd_rn(fabsf(AP1), fabsf(AQ1)), fabsf(AQ2))));
  const float L1 = __fsub_rn(fabsf(AP1), Bx);
  if (!(L1 > 2e-9f)) return false;  // also keeps the collinear branch out
  const bool sameP = (AP1 > Bx && AP2 > B2) || (AP1 < -Bx && AP2 < -B2);
  if (sameP && L1 > __fmul_rn(2e-9f, __fadd_rn(fabsf(AP2), B2))) return true;
  const bool sameQ = (AQ1 > Bx && AQ2 > Bx) || (AQ1 < -Bx && AQ2 < -Bx);
  const float LQ1 = __fsub_rn(fabsf(AQ1), Bx);
  return sameQ && LQ1 > __fmul_rn(2e-9f, __fadd_rn(fabsf(AQ2), Bx));
}

// Vertex coordinates as float pairs: hi = x rounded to float, lo = (x - hi)
// rounded to float, so hi + lo is within 2^-48 |x| of the double.
__global__ void k_vertex_f4(long long nv, const double* __restrict__ xy, float4* __restrict__ out) {
  long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const double x = xy[2 * v], y = xy[2 * v + 1];
  const float hx = __double2float_rn(x), hy = __double2float_rn(y);
  out[v] = make_float4(hx, hy, __double2float_rn(dsub(x, (double)hx)),
                       __double2float_rn(dsub(y, (double)hy)));
}

// Exact stage per candidate pair.  Phase 1 (one pair per thread): FP64 LSMF,
// then the float pre-test; pairs it cannot rule out are queued in shared
// memory.  Phase 2: the queue runs seg_isect in full warps (divergent FP64
// lanes would cost a full warp each); pairs with a non-zero type get their
// emission count and first key (a pair the reference never emits is
// dropped there).
// counters: [0] unique hits, [1] pairs passing LSMF, [3] emissions with a
// non-zero type (the reference's raw hit count).
constexpr int kExBlock = 256;
constexpr int kExPer = 4;
constexpr int kExChunk = kExBlock * kExPer;

__global__ void __launch_bounds__(kExBlock)
k_pair_exact(long long n, const int2* __restrict__ pairs, const int* __restrict__ e_id,
             const double* __restrict__ bP, const double* __restrict__ cP,
             const long long* __restrict__ bK, const long long* __restrict__ cK,
             const float4* __restrict__ vfB, const float4* __restrict__ vfC,
             const int2* __restrict__ lr, const int* __restrict__ aft, const int* __restrict__ bef,
             int logL, unsigned long long* __restrict__ counters, long long cap,
             int* __restrict__ rb, int* __restrict__ rc, int* __restrict__ rt,
             unsigned long long* __restrict__ rkey, double2* __restrict__ rab) {
  __shared__ int4 q[kExChunk];
  __shared__ int qn;
  __shared__ unsigned long long ntested;
  const int tid = threadIdx.x, lane = tid & 31;
  const unsigned lt = (1u << lane) - 1u;
  const long long base = (long long)blockIdx.x * kExChunk;
  if (tid == 0) {
    qn = 0;
    ntested = 0;
  }
  __syncthreads();
  unsigned long long my_tested = 0;
  for (int r = 0; r < kExPer; ++r) {
    const long long i = base + (long long)r * kExBlock + tid;
    bool keep = false;
    int4 e = make_int4(0, 0, 0, 0);
    if (i < n) {
      const int2 pr = pairs[i];
      const int bId = e_id[pr.x], cId = e_id[pr.y];
      const long long* kb = bK + bId;
      const long long* kc = cK + cId;
      if (lsmf_keys(kb[0], kb[1], kb[2], kb[3], kc[0], kc[1], kc[2], kc[3])) {
        ++my_tested;
        if (!certainly_disjoint(vfB[bId >> 1], vfB[(bId >> 1) + 1], vfC[cId >> 1],
                                vfC[(cId >> 1) + 1])) {
          keep = true;
          e = make_int4(bId, cId, pr.x, pr.y);
        }
      }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (bal) {
      int w0 = 0;
      if (lane == 0) w0 = atomicAdd(&qn, __popc(bal));
      w0 = __shfl_sync(0xffffffffu, w0, 0);
      if (keep) q[w0 + __popc(bal & lt)] = e;
    }
  }
  for (int o = 16; o > 0; o >>= 1) my_tested += __shfl_xor_sync(0xffffffffu, my_tested, o);
  if (lane == 0 && my_tested) atomicAdd(&ntested, my_tested);
  __syncthreads();
  if (tid == 0 && ntested) atomicAdd(&counters[1], ntested);
  const int nq = qn;
  const int nq32 = (nq + 31) & ~31;  // warp-uniform loop bound
  unsigned long long my_raw = 0;
  for (int j = tid; j < nq32; j += kExBlock) {
    bool hit = false;
    int ty = 0;
    int4 e = make_int4(0, 0, 0, 0);
    unsigned long long key = 0;
    double al = 0.0, be = 0.0;
    if (j < nq) {
      e = q[j];
      const double* pb = bP + e.x;
      const double* pc = cP + e.y;
      ty = seg_isect(pb[0], pb[1], pb[2], pb[3], pc[0], pc[1], pc[2], pc[3], &al, &be);
      if (ty != 0) {
        const unsigned cnt = emission(e.z, e.w, e.y, lr, aft, bef, logL, &key);
        hit = cnt > 0;
        my_raw += cnt;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (m) {
      const int leader = __ffs(m) - 1;
      unsigned long long hb = 0;
      if (lane == leader) hb = atomicAdd(&counters[0], (unsigned long long)__popc(m));
      hb = __shfl_sync(0xffffffffu, hb, leader);
      if (hit) {
        const long long idx = (long long)hb + __popc(m & lt);
        if (idx < cap) {
          rb[idx] = e.x;
          rc[idx] = e.y;
          rt[idx] = ty;
          rkey[idx] = key;
          rab[idx] = make_double2(al, be);  // the record stage reuses them
        }
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) my_raw += __shfl_xor_sync(0xffffffffu, my_raw, o);
  if (lane == 0 && my_raw) atomicAdd(&counters[3], my_raw);
}

}  // namespace

// ------------------------------------------------------------------ host
// The grid stage does not depend on the tree: it runs on the pipeline's
// second stream (side_stream()), issued in three steps that run() interleaves
// with the tree stages, so its kernels overlap the tree build and its two
// host reads mostly find the work already done.  The last step makes the
// main stream wait for the grid before the candidate stage.
int Pipeline::stage_grid_boxes() {
  cudaStream_t st = side_stream();
  if (!st) return fail(kECuda, "side stream");
  h_tstart_.assign(k + 2, 0);
  for (int t = 0; t <= k; ++t) h_tstart_[t + 1] = nb + hcc[t];
  g_tstart = (int*)side_pool_.get("grid_tstart", sizeof(int) * (k + 2));
  fbox = (float4*)side_pool_.get("grid_fbox", sizeof(float4) * (E + 1));
  g_bnd = (unsigned*)side_pool_.get("grid_bnd", 256);
  vfB = (float4*)side_pool_.get("grid_vfB", sizeof(float4) * (nb + 1));
  vfC = (float4*)side_pool_.get("grid_vfC", sizeof(float4) * ((long long)clSize + k));
  g_islong = (unsigned char*)side_pool_.get("grid_islong", (size_t)E + 1);
  g_long = (int*)side_pool_.get("grid_long", sizeof(int) * (E + 1));
  g_long_count = (unsigned*)side_pool_.get("grid_long_count", 256);
  if (side_pool_.failed) return fail(kENoMem, "device allocation failed (grid)");
  auto* sum_ext = (double*)((char*)g_bnd + 64);
  // the setup's arrays are written on the main stream (run() records
  // ev_setup_ after the setup)
  cudaStreamWaitEvent(st, ev_setup_, 0);
  cudaMemcpyAsync(g_tstart, h_tstart_.data(), sizeof(int) * (k + 2), cudaMemcpyHostToDevice, st);
  static const unsigned init[8] = {0xffffffffu, 0xffffffffu, 0u, 0u,
                                   0xffffffffu, 0xffffffffu, 0u, 0u};
  cudaMemcpyAsync(g_bnd, init, sizeof(init), cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(sum_ext, 0, sizeof(double), st);
  cudaMemsetAsync(g_long_count, 0, sizeof(unsigned), st);
  {
    ::sbc::KProbe kp_("k_edge_fbox", st);
    k_edge_fbox<<<grid_for(E, 256), 256, 0, st>>>(E, e_id, g_tstart, k, bP, cP, fbox, g_bnd,
                                                  sum_ext);
  }
  {
    ::sbc::KProbe kp_("k_vertex_f4", st);
    k_vertex_f4<<<grid_for(nb + 1, 256), 256, 0, st>>>(nb + 1, bP, vfB);
  }
  {
    ::sbc::KProbe kp_("k_vertex_f4", st);
    k_vertex_f4<<<grid_for((long long)clSize + k, 256), 256, 0, st>>>((long long)clSize + k, cP, vfC);
  }
  side_rd_.get(g_bnd, 0, st, 8);
  side_rd_.get(sum_ext, 4, st);
  return kOk;
}

int Pipeline::stage_grid_count() {
  cudaStream_t st = side_stream();
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(kECuda, "grid bounds");
  unsigned hb[8];
  double hsum = 0.0;
  memcpy(hb, side_rd_.word(0), sizeof(hb));
  memcpy(&hsum, side_rd_.word(4), sizeof(double));
  auto unkey = [](unsigned kk) {
    unsigned u = (kk & 0x80000000u) ? (kk & 0x7fffffffu) : ~kk;
    float f;
    memcpy(&f, &u, sizeof f);
    return f;
  };
  // the grid covers the common MBR: the base's box cut with the overlays'
  // box (an empty cut leaves a one-cell grid that every edge misses)
  float x0 = std::max(unkey(hb[0]), unkey(hb[4])), y0 = std::max(unkey(hb[1]), unkey(hb[5]));
  float x1 = std::min(unkey(hb[2]), unkey(hb[6])), y1 = std::min(unkey(hb[3]), unkey(hb[7]));
  const float4 cmbr = make_float4(x0, y0, x1, y1);
  if (!(x1 >= x0)) x1 = x0;
  if (!(y1 >= y0)) y1 = y0;
  const double spanx = (double)x1 - x0, spany = (double)y1 - y0;
  // cell size: 1.5 x the mean edge extent, with at most max(2^21, 4E)
  // (cell, class) buckets in all
  const double maxBuckets = std::max(2097152.0, 4.0 * E);
  double s = 1.5 * hsum / (E > 0 ? E : 1);
  s = std::max(s, std::max(spanx, spany) / 8192.0);
  s = std::max(s, std::sqrt(spanx * spany * (k + 1) / maxBuckets));
  if (!(s > 0.0)) s = 1.0;
  grid_.x0 = x0;
  grid_.y0 = y0;
  grid_.inv = (float)(1.0 / s);
  grid_.gx = (int)std::min(8192.0, std::floor(spanx / s) + 1.0);
  grid_.gy = (int)std::min(8192.0, std::floor(spany / s) + 1.0);
  const Grid g{grid_.x0, grid_.y0, grid_.inv, grid_.gx, grid_.gy};
  g_nCells = grid_.gx * grid_.gy;
  const long long nBk = (long long)g_nCells * (k + 1);
  g_bstart = (int*)side_pool_.get("grid_bstart", sizeof(int) * (nBk + 1));
  g_fill = (int*)side_pool_.get("grid_fill", sizeof(int) * (nBk + 1));
  void* sscr2 = side_pool_.get_zeroed("scan_scr_grid2", scan_scratch_bytes(nBk + 1), st);
  if (side_pool_.failed) return fail(kENoMem, "device allocation failed (grid buckets)");
  cudaMemsetAsync(g_bstart, 0, sizeof(int) * (nBk + 1), st);
  cudaMemsetAsync(g_fill, 0, sizeof(int) * (nBk + 1), st);
  unsigned* outside = (unsigned*)((char*)g_bnd + 128);
  cudaMemsetAsync(outside, 0, sizeof(unsigned), st);
  {
    ::sbc::KProbe kp_("k_grid_count", st);
    k_grid_count<<<grid_for(E, 256), 256, 0, st>>>(E, fbox, g, g_tstart, k, g_bstart, g_islong,
                                                 g_long, g_long_count, cmbr, outside);
  }
  exclusive_scan_i32(g_bstart, nBk + 1, sscr2, st, true);
  side_rd_.get(g_bstart + nBk, 0, st);
  side_rd_.get(outside, 1, st);
  return kOk;
}

int Pipeline::stage_grid_fill() {
  cudaStream_t st = side_stream();
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(kECuda, "grid count");
  int total = 0;
  unsigned n_out = 0;
  memcpy(&total, side_rd_.word(0), sizeof(int));
  memcpy(&n_out, side_rd_.word(1), sizeof(unsigned));
  stat_outside_cmbr = n_out;
  if (total < 0) return fail(kEInput, "grid too large");
  g_n = total;
  g_vals = (unsigned*)side_pool_.get("grid_vals", sizeof(unsigned) * ((long long)total + 1));
  if (side_pool_.failed) return fail(kENoMem, "device allocation failed (grid entries)");
  const Grid g{grid_.x0, grid_.y0, grid_.inv, grid_.gx, grid_.gy};
  if (total > 0) {
    ::sbc::KProbe kp_("k_grid_scatter", st);
    k_grid_scatter<<<grid_for(E, 256), 256, 0, st>>>(E, fbox, g, g_tstart, k, g_bstart, g_fill,
                                                   g_islong, g_vals);
  }
  return kOk;
}

// The box join of overlay cType on stream `st`: every box-overlapping
// (base edge, overlay edge) pair, reported once (in the cell of the low
// corner of the boxes' overlap).  It reads only the grid, so run() issues the
// first overlay's join on the side stream, next to the tree build.
int Pipeline::stage_join(int cType, cudaStream_t st) {
  // on the side stream it runs on the side worker: its buffers and reads
  BufferPool& pool = st == st2_ ? side_pool_ : pool_;
  HostReads& rd = st == st2_ ? side_rd_ : rd_;
  join_ready_ = 0;
  const Grid g{grid_.x0, grid_.y0, grid_.inv, grid_.gx, grid_.gy};
  const int nCells = g_nCells;
  auto* cdesc = (int4*)pool.get("cg_desc", sizeof(int4) * ((long long)nCells + 1));
  int* smalls = (int*)pool.get("cg_small", sizeof(int) * ((long long)nCells + 1));
  int* tiles = (int*)pool.get("cg_tiles", sizeof(int) * ((long long)nCells + 1));
  long long* work = (long long*)pool.get("cg_work", sizeof(long long) * ((long long)nCells + 1));
  auto* counters = (unsigned long long*)pool.get("cg_counters", 64);
  void* sscr = pool.get_zeroed("scan_scr_cg", scan_scratch_bytes((long long)nCells + 1), st);
  if (pool.failed) return fail(kENoMem, "device allocation failed (grid items)");
  {
    ::sbc::KProbe kp_("k_cell_items", st);
    k_cell_items<<<grid_for((long long)nCells + 1, 256), 256, 0, st>>>(nCells, g_bstart, k, cType,
                                                                       cdesc, smalls, tiles, work);
  }
  exclusive_scan_i32(smalls, (long long)nCells + 1, sscr, st, true);
  exclusive_scan_i32(tiles, (long long)nCells + 1, sscr, st, true);
  exclusive_scan_i64(work, (long long)nCells + 1, sscr, st, true);
  const int* r_nS = rd.get(smalls + nCells, HostReads::kCand, st);
  const int* r_nW = rd.get(tiles + nCells, HostReads::kCand + 1, st);
  const long long* r_W = rd.get(work + nCells, HostReads::kCand + 2, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(kECuda, "grid items");
  const int nS = *r_nS, nW = *r_nW;
  const long long W = *r_W;
  int* srec = (int*)pool.get("cg_srec", sizeof(int) * ((long long)nS + 1));
  auto* wrec = (int2*)pool.get("cg_wrec", sizeof(int2) * ((long long)nW + 1));
  if (pool.failed) return fail(kENoMem, "device allocation failed (grid items)");
  if (nCells > 0) {
    ::sbc::KProbe kp_("k_cell_expand", st);
    k_cell_expand<<<grid_for(nCells, 256), 256, 0, st>>>(nCells, smalls, tiles, srec, wrec);
  }
  // box-overlapping pairs (grow and retry on overflow)
  long long cap = pair_cap_ > 0 ? pair_cap_ : 4LL * E + (1 << 20);
  long long npairs = 0;
  int2* pairs = nullptr;
  for (int attempt = 0; attempt < 2; ++attempt) {
    pairs = (int2*)pool.get("cg_pairs", sizeof(int2) * (cap + 1));
    if (pool.failed) return fail(kENoMem, "device allocation failed (candidate pairs)");
    cudaMemsetAsync(counters, 0, 64, st);
    if (nS > 0) {
      ::sbc::KProbe kp_("k_grid_small", st);
      k_grid_small<<<grid_for(nS, kGBlock), kGBlock, 0, st>>>(srec, nS, cdesc, g_vals, fbox, g,
                                                            &counters[2], cap, pairs);
    }
    if (nW > 0) {
      ::sbc::KProbe kp_("k_grid_warp", st);
      k_grid_warp<<<grid_for((long long)nW * 32, kGBlock), kGBlock, 0, st>>>(
          wrec, nW, cdesc, g_vals, fbox, g, &counters[2], cap, pairs);
    }
    {
      ::sbc::KProbe kp_("k_grid_long", st);
      k_grid_long<<<64, kGBlock, 0, st>>>(g_long, g_long_count, g_tstart, cType, g_islong, fbox,
                                          &counters[2], cap, pairs);
    }
    const unsigned long long* r_hp = rd.get(counters + 2, HostReads::kCand + 3, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail(kECuda, "candidate pairs");
    npairs = (long long)*r_hp;
    if (npairs <= cap) break;
    cap = npairs + (1 << 20);
  }
  pair_cap_ = cap;
  join_counters_ = counters;
  join_pairs_ = pairs;
  join_npairs_ = npairs;
  join_work_ = W;
  join_ready_ = cType;
  return kOk;
}

int Pipeline::stage_candidates(int cType, int** rb_out, int** rc_out, int** rt_out,
                               unsigned long long** rkey_out, long long* nhits, OverlayOut& out) {
  cudaStream_t st = st_;
  if (join_ready_ != cType) {
    const int rj = stage_join(cType, st);
    if (rj) return rj;
  }
  join_ready_ = 0;
  const long long npairs = join_npairs_;
  const int2* pairs = join_pairs_;
  // the join's counters: [2] holds its pair count, the others start at zero
  auto* counters = join_counters_;
  // exact stage: one record per unique hit
  long long hcap = npairs + 1;
  int* rb = (int*)pool_.get("raw_b", sizeof(int) * hcap);
  int* rc = (int*)pool_.get("raw_c", sizeof(int) * hcap);
  int* rt = (int*)pool_.get("raw_t", sizeof(int) * hcap);
  auto* rkey = (unsigned long long*)pool_.get("raw_key", sizeof(unsigned long long) * hcap);
  auto* rab = (double2*)pool_.get("raw_ab", sizeof(double2) * hcap);
  if (pool_.failed) return fail(kENoMem, "device allocation failed (hits)");
  raw_ab_ = rab;
  if (npairs > 0) {
    ::sbc::KProbe kp_("k_pair_exact", st, 72.0 * npairs);  // pair + both edges' coordinates
    k_pair_exact<<<grid_for(npairs, kExChunk), kExBlock, 0, st>>>(
        npairs, pairs, e_id, bP, cP, bK, cK, vfB, vfC, lr, aft, bef, logL, counters, hcap, rb, rc,
        rt, rkey, rab);
  }
  const unsigned long long* hc = rd_.get(counters, HostReads::kCand + 8, st, 4);
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(kECuda, "exact stage");
  if ((long long)hc[0] > hcap) return fail(kEInternal, "hit buffer overflow");
  if (hc[0] >= (1ULL << 31)) return fail(kEInput, "too many intersections");
  *rb_out = rb;
  *rc_out = rc;
  *rt_out = rt;
  *rkey_out = rkey;
  *nhits = (long long)hc[0];
  out.survivors = npairs;
  out.tests = (long long)hc[1];
  out.raw_hits = (long long)hc[3];
  out.work = join_work_;
  return kOk;
}

}  // namespace sbc
