// sbc_mid.cu -- per-overlay stages between the tree and the back end
// (reference rows A8-A14):
//
//  A8   saveIntersectionsIdsMulticore      p_seg_tree/oacc_segment_tree.cpp:6108-6244
//  A9   radixsort + removeDuplicatesAtEdge src/clip.cpp:368-493, :1731-1742
//  A10  countEdgeIntersections + scans     src/clip.cpp:522-601, :1805-1861
//  A11  saveIntersectionsParallel          oacc_segment_tree.cpp:7247-7341
//  A12  sortIntersectionsAtEdgesParallel   oacc_segment_tree.cpp:7436-7473
//  A13  copyIntersectionsParallel          oacc_segment_tree.cpp:7508-7664
//  A14  calculateInitLabelParallel         oacc_segment_tree.cpp:7826-7988
//
// Emission order.  The reference emits candidates node by node, and inside a
// node by cover entry, then cover x cover before cover x end, then partner
// order.  Each hit here carries the key (cover position P, phase, partner id)
// which orders hits exactly like that; duplicates keep the smallest key, and
// hits of one base edge stay in key order, which is the reference's
// first-occurrence order after its stable radix sort by base id.
#include <cstdio>

#include "sbc_pipeline.cuh"

namespace sbc {

namespace {

__device__ __forceinline__ int lower_bound_u32(const unsigned* a, int lo, int hi, unsigned x) {
  while (lo < hi) {
    int m = (lo + hi) >> 1;
    if (a[m] < x) lo = m + 1;
    else hi = m;
  }
  return lo;
}

__device__ __forceinline__ int class_of(const int* tstart, int k, int e) {
  int c = 0;
  while (c < k && tstart[c + 1] <= e) ++c;
  return c;
}

__device__ __forceinline__ void leaf_range(int v, int logL, int* lo, int* hi) {
  int d = 31 - __clz(v);
  int h = logL - d;
  int L = 1 << logL;
  *lo = (v << h) - L;
  *hi = ((v + 1) << h) - 1 - L;
}

// ---------------------------------------------------------------- A8 candidates
// LSMF bounding-box filter, oacc_segment_tree.cpp:5282-5316
__device__ __forceinline__ bool lsmf(double p1x, double p1y, double p2x, double p2y, double q1x,
                                     double q1y, double q2x, double q2y) {
  double minPX = p1x, minPY = p1y, maxPX = p2x, maxPY = p2y;
  double minQX = q1x, minQY = q1y, maxQX = q2x, maxQY = q2y;
  if (minPX > p2x) { minPX = p2x; maxPX = p1x; }
  if (minPY > p2y) { minPY = p2y; maxPY = p1y; }
  if (minQX > q2x) { minQX = q2x; maxQX = q1x; }
  if (minQY > q2y) { minQY = q2y; maxQY = q1y; }
  if (minPX > maxQX || maxPX < minQX) return false;
  if (minPY > maxQY || maxPY < minQY) return false;
  return true;
}

constexpr int kCandBlock = 256;

// conservative float bounds of an edge's y extent (rounded outwards), one
// record per leaf entry: {edge, leaf, ymin rounded down, ymax rounded up}
__global__ void k_pack_leaf(long long n, const int* __restrict__ le_edge,
                            const int* __restrict__ le_leaf, const int* __restrict__ e_id,
                            const int* __restrict__ tstart, int k, const double* __restrict__ bP,
                            const double* __restrict__ cP, int4* __restrict__ pack) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int e = le_edge[i];
  const double* p = (class_of(tstart, k, e) == 0 ? bP : cP) + e_id[e];
  double y0 = fmin(p[1], p[3]), y1 = fmax(p[1], p[3]);
  pack[i] = make_int4(e, le_leaf[i], __float_as_int(__double2float_rd(y0)),
                      __float_as_int(__double2float_ru(y1)));
}

__global__ void k_edge_ybox(int E, const int* __restrict__ e_id, const int* __restrict__ tstart,
                            int k, const double* __restrict__ bP, const double* __restrict__ cP,
                            float2* __restrict__ ybox, int2* __restrict__ ab,
                            const int* __restrict__ aft, const int* __restrict__ bef) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const double* p = (class_of(tstart, k, e) == 0 ? bP : cP) + e_id[e];
  double y0 = fmin(p[1], p[3]), y1 = fmax(p[1], p[3]);
  ybox[e] = make_float2(__double2float_rd(y0), __double2float_ru(y1));
  ab[e] = make_int2(aft[e], bef[e]);
}

// per node with cover entries: the candidate products of its three kinds
//   kind 0: base cover entries x overlay cover entries of the same node
//   kind 1: base cover entries x overlay end-list entries (class cType leaves)
//   kind 2: overlay cover entries x base end-list entries (class 0 leaves)
// In every kind the "covers" are swept and the "partners" held in registers.
struct NodeTiles {
  int s, e;        // cover entries [s, e) of the node
  int nb;          // base cover entries [s, s+nb)
  int bsT, ncT;    // overlay cover entries [bsT, bsT+ncT)
  long long lbT, nT, lb0, n0;  // leaf-entry ranges of class cType and of class 0
  int lo, hi;      // leaf range of the node
};

constexpr int kTile = 256;     // partners per warp tile (8 per lane)
constexpr int kCTile = 1024;   // cover entries per warp tile
constexpr int kSmallMax = 64;  // products of at most this many pairs: one thread each
constexpr int kStage = 512;    // survivors staged per warp in shared memory

__device__ __forceinline__ NodeTiles node_tiles(int v, const int* node_start, const int* node_end,
                                                const unsigned* cov_edge, const int* tstart,
                                                int cType, int logL, int numLeaves,
                                                const int* le_off) {
  NodeTiles t;
  t.s = node_start[v];
  t.e = node_end[v];
  t.nb = lower_bound_u32(cov_edge, t.s, t.e, (unsigned)tstart[1]) - t.s;
  t.bsT = lower_bound_u32(cov_edge, t.s, t.e, (unsigned)tstart[cType]);
  t.ncT = lower_bound_u32(cov_edge, t.s, t.e, (unsigned)tstart[cType + 1]) - t.bsT;
  int d = 31 - __clz(v), h = logL - d, L = 1 << logL;
  t.lo = (v << h) - L;
  t.hi = ((v + 1) << h) - 1 - L;
  size_t cT = (size_t)cType * numLeaves;
  t.lbT = le_off[cT + t.lo];
  t.nT = le_off[cT + t.hi + 1] - t.lbT;
  t.lb0 = le_off[t.lo];
  t.n0 = le_off[t.hi + 1] - t.lb0;
  return t;
}

// node descriptor: three int4 per node, written by k_node_items
__device__ __forceinline__ NodeTiles load_desc(const int4* __restrict__ desc, int i) {
  const int4 d0 = desc[3 * i], d1 = desc[3 * i + 1], d2 = desc[3 * i + 2];
  NodeTiles t;
  t.s = d0.x;
  t.e = 0;
  t.nb = d0.y;
  t.bsT = d0.z;
  t.ncT = d0.w;
  t.lo = d1.x;
  t.hi = d1.y;
  t.lbT = d1.z;
  t.nT = d1.w;
  t.lb0 = d2.x;
  t.n0 = d2.y;
  return t;
}

__device__ __forceinline__ void kind_sizes(const NodeTiles& t, int kind, long long* p,
                                           long long* cv) {
  *p = kind == 0 ? t.ncT : (kind == 1 ? t.nT : t.n0);
  *cv = kind == 2 ? t.ncT : t.nb;
}

__device__ __forceinline__ int cover_start(const NodeTiles& t, int kind) {
  return kind == 2 ? t.bsT : t.s;
}

__device__ __forceinline__ long long tiles_of(long long n) { return (n + kTile - 1) / kTile; }
__device__ __forceinline__ long long ctiles_of(long long n) { return (n + kCTile - 1) / kCTile; }

// Partner j of `kind` in node t: its edge index and float y box, or -1 (and
// an empty box) when it is the second leaf entry of an edge whose first entry
// lies in the same subtree (an end list holds each edge once).
__device__ __forceinline__ int load_partner(const NodeTiles& t, int kind, long long j, int L,
                                            const unsigned* __restrict__ cov_edge,
                                            const int4* __restrict__ pack,
                                            const float2* __restrict__ ybox,
                                            const int2* __restrict__ ab, float* y0, float* y1) {
  if (kind == 0) {
    int e = (int)cov_edge[t.bsT + j];
    float2 bx = ybox[e];
    *y0 = bx.x;
    *y1 = bx.y;
    return e;
  }
  int4 r = pack[(kind == 1 ? t.lbT : t.lb0) + j];
  int2 o = ab[r.x];
  int leaf = r.y + L;
  int other = (o.x == leaf) ? o.y : o.x;
  if (other >= 0 && other >= t.lo + L && other <= t.hi + L && other < leaf) {
    *y0 = __int_as_float(0x7f800000);  // +inf
    *y1 = __int_as_float(0xff800000);  // -inf: overlaps no finite box
    return -1;
  }
  *y0 = __int_as_float(r.z);
  *y1 = __int_as_float(r.w);
  return r.x;
}

__global__ void k_node_list(long long nCover, const unsigned* __restrict__ cov_node,
                            const int* __restrict__ hpre, int* __restrict__ nodes) {
  long long P = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (P >= nCover) return;
  if (P == 0 || cov_node[P] != cov_node[P - 1]) nodes[hpre[P]] = (int)cov_node[P];
}

__global__ void k_node_heads(long long nCover, const unsigned* __restrict__ cov_node,
                             int* __restrict__ h) {
  long long P = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (P > nCover) return;
  h[P] = (P < nCover && (P == 0 || cov_node[P] != cov_node[P - 1])) ? 1 : 0;
}

// per node: its descriptor, its warp tiles (items), its small products
// (smalls) and its pair count (work units)
__global__ void k_node_items(int nNodes, const int* __restrict__ nodes,
                             const int* __restrict__ node_start, const int* __restrict__ node_end,
                             const unsigned* __restrict__ cov_edge, const int* __restrict__ tstart,
                             int cType, int logL, int numLeaves, const int* __restrict__ le_off,
                             long long* __restrict__ items, long long* __restrict__ smalls,
                             long long* __restrict__ wunits, int4* __restrict__ desc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > nNodes) return;
  if (i == nNodes) {
    items[i] = 0;
    smalls[i] = 0;
    wunits[i] = 0;
    return;
  }
  NodeTiles t = node_tiles(nodes[i], node_start, node_end, cov_edge, tstart, cType, logL,
                           numLeaves, le_off);
  desc[3 * i + 0] = make_int4(t.s, t.nb, t.bsT, t.ncT);
  desc[3 * i + 1] = make_int4(t.lo, t.hi, (int)t.lbT, (int)t.nT);
  desc[3 * i + 2] = make_int4((int)t.lb0, (int)t.n0, 0, 0);
  long long n = 0, ns = 0, w = 0;
  for (int kind = 0; kind < 3; ++kind) {
    long long p, cv;
    kind_sizes(t, kind, &p, &cv);
    if (p <= 0 || cv <= 0) continue;
    w += p * cv;
    if (p * cv <= kSmallMax) ++ns;
    else n += tiles_of(p) * ctiles_of(cv);
  }
  items[i] = n;
  smalls[i] = ns;
  wunits[i] = w;
}

// warp tiles {node index, kind, partner tile, cover tile} and small
// products {node index, kind}, in node order
__global__ void k_expand_items(int nNodes, const long long* __restrict__ items,
                               const long long* __restrict__ smalls,
                               const int4* __restrict__ desc, int4* __restrict__ rec,
                               int2* __restrict__ srec) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nNodes) return;
  const NodeTiles t = load_desc(desc, i);
  long long w = items[i], sw = smalls[i];
  for (int kind = 0; kind < 3; ++kind) {
    long long p, cv;
    kind_sizes(t, kind, &p, &cv);
    if (p <= 0 || cv <= 0) continue;
    if (p * cv <= kSmallMax) {
      srec[sw++] = make_int2(i, kind);
      continue;
    }
    const long long np = tiles_of(p), nc = ctiles_of(cv);
    for (long long c = 0; c < nc; ++c)
      for (long long q = 0; q < np; ++q) rec[w++] = make_int4(i, kind, (int)q, (int)c);
  }
}

// Survivors of the float filter are staged per warp in shared memory and
// reserved in the global list with one atomic per flush.
struct WarpStage {
  int2* buf;
  int n;  // warp-uniform fill
};

__device__ __forceinline__ void stage_flush(WarpStage& s, int lane,
                                            unsigned long long* __restrict__ counter,
                                            long long scap, int2* __restrict__ surv) {
  __syncwarp();
  if (s.n == 0) return;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(counter, (unsigned long long)s.n);
  base = __shfl_sync(0xffffffffu, base, 0);
  for (int k = lane; k < s.n; k += 32) {
    long long w = (long long)base + k;
    if (w < scap) surv[w] = s.buf[k];
  }
  __syncwarp();
  s.n = 0;
}

// at most one survivor per lane
__device__ __forceinline__ void stage_push1(WarpStage& s, int lane, bool hit, int2 v,
                                            unsigned long long* __restrict__ counter,
                                            long long scap, int2* __restrict__ surv) {
  const unsigned b = __ballot_sync(0xffffffffu, hit);
  if (b == 0) return;
  if (hit) s.buf[s.n + __popc(b & ((1u << lane) - 1u))] = v;
  s.n += __popc(b);
  if (s.n > kStage - 32) stage_flush(s, lane, counter, scap, surv);
}

// Candidate filter by node tiles (saveIntersectionsIdsMulticore,
// oacc_segment_tree.cpp:6118-6241, reordered).  A warp holds up to 256
// partners of one node in registers and sweeps the node's cover entries of
// the other polygon over them, so an end list is read once per node instead
// of once per cover entry.  Every partner in the same cover list or the end
// list of the node overlaps the cover edge in x (both span or touch the
// node's interval), so the LSMF box test reduces to the y test; a
// conservative float y test (bounds rounded outwards) rejects most pairs from
// registers.  The rest are compacted into a survivor list for k_cand_exact
// (FP64 work in full warps: the FP64 pipe costs the same per warp
// instruction however few lanes are active).
//
// Tile shapes: more than 32 partners -> Q = 2, 4 or 8 partners per lane, one
// cover per step for the whole warp; at most 32 partners -> lanes form
// 32 / P2 groups of P2 = next power of two >= partners, each group testing
// a different cover per step.
template <int Q>
__device__ __forceinline__ void sweep_wide(const NodeTiles& t, int kind, long long pbase, int pt,
                                           int cs, int cn, int L, int lane,
                                           const unsigned* __restrict__ cov_edge,
                                           const int4* __restrict__ pack,
                                           const float2* __restrict__ ybox,
                                           const int2* __restrict__ ab, WarpStage& st,
                                           unsigned long long* __restrict__ counter,
                                           long long scap, int2* __restrict__ surv) {
  int pe[Q];
  float py0[Q], py1[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int jj = q * 32 + lane;
    pe[q] = -1;
    py0[q] = __int_as_float(0x7f800000);
    py1[q] = __int_as_float(0xff800000);
    if (jj < pt) pe[q] = load_partner(t, kind, pbase + jj, L, cov_edge, pack, ybox, ab, &py0[q], &py1[q]);
  }
  for (int cb = 0; cb < cn; cb += 32) {
    float2 mybox = make_float2(0.f, 0.f);
    if (cb + lane < cn) mybox = ybox[cov_edge[cs + cb + lane]];
    const int nthis = min(32, cn - cb);
    for (int k2 = 0; k2 < nthis; ++k2) {
      const float sx = __shfl_sync(0xffffffffu, mybox.x, k2);
      const float sy = __shfl_sync(0xffffffffu, mybox.y, k2);
      unsigned m = 0;
#pragma unroll
      for (int q = 0; q < Q; ++q)
        if (!(sx > py1[q] || sy < py0[q])) m |= 1u << q;
      if (!__any_sync(0xffffffffu, m != 0)) continue;
      const int P = cs + cb + k2;
      const int cnt = __popc(m);
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      int w = st.n + incl - cnt;
      while (m) {
        int q = __ffs(m) - 1;
        m &= m - 1;
        st.buf[w++] = make_int2(P, pe[q] | (kind << 30));
      }
      st.n += total;
      if (st.n > kStage - 32 * Q) stage_flush(st, lane, counter, scap, surv);
    }
  }
}

__device__ __forceinline__ void sweep_grouped(const NodeTiles& t, int kind, long long pbase,
                                              int pt, int cs, int cn, int L, int lane,
                                              const unsigned* __restrict__ cov_edge,
                                              const int4* __restrict__ pack,
                                              const float2* __restrict__ ybox,
                                              const int2* __restrict__ ab, WarpStage& st,
                                              unsigned long long* __restrict__ counter,
                                              long long scap, int2* __restrict__ surv) {
  const int lg = pt <= 1 ? 0 : 32 - __clz(pt - 1);  // P2 = 1 << lg >= pt
  const int G = 32 >> lg;                            // cover groups
  const int slot = lane & ((1 << lg) - 1);
  const int g = lane >> lg;
  float py0 = __int_as_float(0x7f800000), py1 = __int_as_float(0xff800000);
  int pe = -1;
  if (slot < pt) pe = load_partner(t, kind, pbase + slot, L, cov_edge, pack, ybox, ab, &py0, &py1);
  for (int cb = 0; cb < cn; cb += 32) {
    float2 mybox = make_float2(0.f, 0.f);
    if (cb + lane < cn) mybox = ybox[cov_edge[cs + cb + lane]];
    const int nthis = min(32, cn - cb);
    const int steps = (nthis + G - 1) / G;  // steps * G <= 32 (G divides 32)
    for (int k2 = 0; k2 < steps; ++k2) {
      const int ci = k2 * G + g;
      const float sx = __shfl_sync(0xffffffffu, mybox.x, ci);
      const float sy = __shfl_sync(0xffffffffu, mybox.y, ci);
      const bool hit = ci < nthis && pe >= 0 && !(sx > py1 || sy < py0);
      stage_push1(st, lane, hit, make_int2(cs + cb + ci, pe | (kind << 30)), counter, scap, surv);
    }
  }
}

__global__ void __launch_bounds__(kCandBlock)
k_cand_test(const int4* __restrict__ rec, const int4* __restrict__ desc, long long nItems,
            const unsigned* __restrict__ cov_edge, int logL, const int4* __restrict__ pack,
            const float2* __restrict__ ybox, const int2* __restrict__ ab,
            unsigned long long* __restrict__ counters, long long scap, int2* __restrict__ surv) {
  __shared__ int2 stage_all[kCandBlock / 32][kStage];
  const int lane = threadIdx.x & 31;
  const long long it = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (it >= nItems) return;  // warp-uniform; no block-wide barrier follows
  WarpStage st{stage_all[threadIdx.x >> 5], 0};
  const int4 rc4 = rec[it];
  const NodeTiles t = load_desc(desc, rc4.x);
  const int kind = rc4.y;
  const long long tile = rc4.z;
  const int ctile = rc4.w;
  const int L = 1 << logL;
  long long p, cv;
  kind_sizes(t, kind, &p, &cv);
  const long long pbase = tile * kTile;
  const int pt = (int)min((long long)kTile, p - pbase);
  const int cs = cover_start(t, kind) + ctile * kCTile;
  const int cn = (int)min((long long)kCTile, cv - (long long)ctile * kCTile);
  unsigned long long* counter = &counters[2];
  if (pt > 128)
    sweep_wide<8>(t, kind, pbase, pt, cs, cn, L, lane, cov_edge, pack, ybox, ab, st, counter, scap, surv);
  else if (pt > 64)
    sweep_wide<4>(t, kind, pbase, pt, cs, cn, L, lane, cov_edge, pack, ybox, ab, st, counter, scap, surv);
  else if (pt > 32)
    sweep_wide<2>(t, kind, pbase, pt, cs, cn, L, lane, cov_edge, pack, ybox, ab, st, counter, scap, surv);
  else
    sweep_grouped(t, kind, pbase, pt, cs, cn, L, lane, cov_edge, pack, ybox, ab, st, counter, scap, surv);
  stage_flush(st, lane, counter, scap, surv);
}

// Small products (at most kSmallMax pairs): one thread each, the warp's
// threads stepping through their own products in lockstep (partner-major).
__global__ void __launch_bounds__(kCandBlock)
k_cand_small(const int2* __restrict__ srec, long long nS, const int4* __restrict__ desc,
             const unsigned* __restrict__ cov_edge, int logL, const int4* __restrict__ pack,
             const float2* __restrict__ ybox, const int2* __restrict__ ab,
             unsigned long long* __restrict__ counters, long long scap, int2* __restrict__ surv) {
  __shared__ int2 stage_all[kCandBlock / 32][kStage];
  const int lane = threadIdx.x & 31;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i - lane >= nS) return;  // warp-uniform; no block-wide barrier follows
  WarpStage st{stage_all[threadIdx.x >> 5], 0};
  const int L = 1 << logL;
  NodeTiles t{};
  int kind = 0, prod = 0, cvn = 1, cs = 0;
  if (i < nS) {
    const int2 r = srec[i];
    t = load_desc(desc, r.x);
    kind = r.y;
    long long p, cv;
    kind_sizes(t, kind, &p, &cv);
    prod = (int)(p * cv);
    cvn = (int)cv;
    cs = cover_start(t, kind);
  }
  const int maxp = __reduce_max_sync(0xffffffffu, prod);
  unsigned long long* counter = &counters[2];
  int pj = 0, ck = 0, pe = -1;
  float py0 = 0.f, py1 = 0.f;
  for (int k = 0; k < maxp; ++k) {
    bool hit = false;
    int P = 0, e = -1;
    if (k < prod) {
      if (ck == 0) pe = load_partner(t, kind, pj, L, cov_edge, pack, ybox, ab, &py0, &py1);
      P = cs + ck;
      e = pe;
      if (pe >= 0) {
        const float2 bx = ybox[cov_edge[P]];
        hit = !(bx.x > py1 || bx.y < py0);
      }
      if (++ck == cvn) {
        ck = 0;
        ++pj;
      }
    }
    stage_push1(st, lane, hit, make_int2(P, e | (kind << 30)), counter, scap, surv);
  }
  stage_flush(st, lane, counter, scap, surv);
}

// Vertex coordinates as float pairs: hi = x rounded to float, lo = (x - hi)
// rounded to float, so hi + lo is within 2^-48 |x| of the double.  The
// difference of two nearby vertices, (hiA - hiB) + (loA - loB), is then
// accurate to about 2^-23 of itself plus 2^-46 of the coordinates.
__global__ void k_vertex_f4(long long nv, const double* __restrict__ xy, float4* __restrict__ out) {
  long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const double x = xy[2 * v], y = xy[2 * v + 1];
  const float hx = __double2float_rn(x), hy = __double2float_rn(y);
  out[v] = make_float4(hx, hy, __double2float_rn(dsub(x, (double)hx)),
                       __double2float_rn(dsub(y, (double)hy)));
}

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
// for P = (p1, p2), Q = (q1, q2), decided in float.
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

// Exact LSMF and classification of the filtered pairs.  Phase 1 (one
// survivor per thread, kExPer rounds): FP64 LSMF, then the float pre-test;
// pairs it cannot rule out are queued in shared memory.  Phase 2: the queue
// runs seg_isect in full warps, so the FP64 pipe serves only the pairs that
// need it.
constexpr int kExBlock = 256;
constexpr int kExPer = 4;
constexpr int kExChunk = kExBlock * kExPer;

__global__ void __launch_bounds__(kExBlock)
k_cand_exact(long long n, const int2* __restrict__ surv, const unsigned* __restrict__ cov_edge,
             const int* __restrict__ e_id, const double* __restrict__ bP,
             const double* __restrict__ cP, const float4* __restrict__ vfB,
             const float4* __restrict__ vfC, unsigned long long* __restrict__ counters,
             long long cap, int* __restrict__ rb, int* __restrict__ rc, int* __restrict__ rt,
             unsigned long long* __restrict__ rkey) {
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
  unsigned my_tested = 0;
  for (int r = 0; r < kExPer; ++r) {
    const long long i = base + (long long)r * kExBlock + tid;
    bool keep = false;
    int4 e = make_int4(0, 0, 0, 0);
    if (i < n) {
      const int2 sv = surv[i];
      const int P = sv.x;
      const int partner = sv.y & 0x3fffffff;
      const int kind = (unsigned)sv.y >> 30;
      const bool selfBase = kind != 2;
      const int sid = e_id[cov_edge[P]];
      const int pid = e_id[partner];
      const int bId = selfBase ? sid : pid;
      const int cId = selfBase ? pid : sid;
      const double* pb = bP + bId;
      const double* pc = cP + cId;
      if (lsmf(pb[0], pb[1], pb[2], pb[3], pc[0], pc[1], pc[2], pc[3])) {
        ++my_tested;
        if (!certainly_disjoint(vfB[bId >> 1], vfB[(bId >> 1) + 1], vfC[cId >> 1],
                                vfC[(cId >> 1) + 1])) {
          keep = true;
          e = make_int4(bId, cId, P, ((kind == 0 ? 0 : 1) << 30) | (pid >> 1));
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
  my_tested = __reduce_add_sync(0xffffffffu, my_tested);
  if (lane == 0 && my_tested) atomicAdd(&ntested, (unsigned long long)my_tested);
  __syncthreads();
  if (tid == 0 && ntested) atomicAdd(&counters[1], ntested);
  const int nq = qn;
  const int nq32 = (nq + 31) & ~31;  // warp-uniform loop bound
  for (int j = tid; j < nq32; j += kExBlock) {
    bool hit = false;
    int ty = 0;
    int4 e = make_int4(0, 0, 0, 0);
    if (j < nq) {
      e = q[j];
      const double* pb = bP + e.x;
      const double* pc = cP + e.y;
      double al, be;
      ty = seg_isect(pb[0], pb[1], pb[2], pb[3], pc[0], pc[1], pc[2], pc[3], &al, &be);
      hit = ty != 0;
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
          rkey[idx] = ((unsigned long long)e.z << 36) |
                      ((unsigned long long)((unsigned)e.w >> 30) << 35) |
                      (unsigned long long)(e.w & 0x3fffffff);
        }
      }
    }
  }
}

// ---------------------------------------------------------------- A9 dedup
__global__ void k_iota_keys(const int* __restrict__ rb, long long n, unsigned* __restrict__ keys,
                            unsigned* __restrict__ vals) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keys[i] = (unsigned)rb[i];
  vals[i] = (unsigned)i;
}

__global__ void k_seg_heads(const unsigned* __restrict__ keys, long long n, int* __restrict__ h) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  h[i] = (i < n && (i == 0 || keys[i] != keys[i - 1])) ? 1 : 0;
}

__global__ void k_seg_starts(const int* __restrict__ hs, long long n, int* __restrict__ start) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  if (i == n) {
    start[hs[n]] = (int)n;
    return;
  }
  if (hs[i + 1] != hs[i]) start[hs[i]] = (int)i;
}

// per base edge: order hits by emission key, keep the first hit of each
// overlay edge (removeDuplicatesAtEdge); ord[] receives raw indices in key
// order, keep[] the flags
__global__ void k_dedup(const int* __restrict__ start, int nseg, const unsigned* __restrict__ svals,
                        const unsigned long long* __restrict__ rkey, const int* __restrict__ rc,
                        unsigned* __restrict__ ord, int* __restrict__ keep) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  int a = start[s], b = start[s + 1];
  int m = b - a;
  // insertion sort of raw indices by key, in place in ord[a..b)
  for (int i = 0; i < m; ++i) {
    unsigned r = svals[a + i];
    unsigned long long kr = rkey[r];
    int j = i;
    while (j > 0 && rkey[ord[a + j - 1]] > kr) {
      ord[a + j] = ord[a + j - 1];
      --j;
    }
    ord[a + j] = r;
  }
  for (int i = 0; i < m; ++i) {
    int ci = rc[ord[a + i]];
    int k2 = 1;
    for (int j = 0; j < i; ++j)
      if (rc[ord[a + j]] == ci) {
        k2 = 0;
        break;
      }
    keep[a + i] = k2;
  }
}

__global__ void k_dedup_write(const unsigned* __restrict__ ord, const int* __restrict__ pos,
                              long long n, const int* __restrict__ rb, const int* __restrict__ rc,
                              const int* __restrict__ rt, int* __restrict__ ub, int* __restrict__ uc,
                              int* __restrict__ ut) {
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  if (pos[p + 1] == pos[p]) return;
  int j = pos[p];
  unsigned r = ord[p];
  ub[j] = rb[r];
  uc[j] = rc[r];
  ut[j] = rt[r];
}

// ---------------------------------------------------------------- A10 counts
// isNonDegenerateCase, src/clip.cpp:508-517
__device__ __forceinline__ bool nondeg_b(int t) { return t == 1 || t == 3 || t == 5 || t == 7; }
__device__ __forceinline__ bool nondeg_c(int t) { return t == 1 || t == 2 || t == 6; }

__global__ void k_counts(const int* __restrict__ ub, const int* __restrict__ uc,
                         const int* __restrict__ ut, int K, int cStart, int* __restrict__ bAll,
                         int* __restrict__ bND, int* __restrict__ cAll, int* __restrict__ cND) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= K) return;
  int t = ut[j];
  int eb = ub[j] >> 1;
  int ec = (uc[j] >> 1) - cStart;
  atomicAdd(&bAll[eb], 1);
  if (nondeg_b(t)) atomicAdd(&bND[eb], 1);
  atomicAdd(&cAll[ec], 1);
  if (nondeg_c(t)) atomicAdd(&cND[ec], 1);
}

// ---------------------------------------------------------------- A11 records
__global__ void k_records(const int* __restrict__ ub, const int* __restrict__ uc,
                          int* __restrict__ ut, int K, const double* __restrict__ bP,
                          const double* __restrict__ cP, double* __restrict__ isxy,
                          int* __restrict__ aB, int* __restrict__ aC) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= K) return;
  const double* b = bP + ub[j];
  const double* c = cP + uc[j];
  double al = 0.0, be = 0.0;
  int ty = seg_isect(b[0], b[1], b[2], b[3], c[0], c[1], c[2], c[3], &al, &be);
  double x = 0.0, y = 0.0;
  if (ty == 1) {
    // (1-alpha)*b1 + alpha*b2, mulScalar/add (:5349-5363)
    double oma = dsub(1.0, al);
    x = dadd(dmul(oma, b[0]), dmul(al, b[2]));
    y = dadd(dmul(oma, b[1]), dmul(al, b[3]));
  } else if (ty == 3 || ty == 4 || ty == 5 || ty == 7 || ty == 8) {
    x = c[0];
    y = c[1];
  } else if (ty == 2 || ty == 6) {
    x = b[0];
    y = b[1];
  }
  isxy[2 * j] = x;
  isxy[2 * j + 1] = y;
  if (ty) {
    ut[j] = ty;
    aB[j] = alpha_to_int(al);
    aC[j] = alpha_to_int(be);
  } else {
    aB[j] = 0;
    aC[j] = 0;
  }
}

// ---------------------------------------------------------------- A12 alpha sort
// stable sort of positions [s,e) of one edge by alpha mod 1e9 (9 decimal
// LSD passes), only for edges with more than one non-degenerate intersection
__global__ void k_alpha_sort(int n, const int* __restrict__ allPS, const int* __restrict__ ndPS,
                             const int* __restrict__ alpha, const int* __restrict__ order,
                             int* __restrict__ sorted, unsigned* __restrict__ flags) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int s = allPS[e], t = allPS[e + 1];
  for (int i = s; i < t; ++i) sorted[i] = i;
  if (ndPS[e + 1] - ndPS[e] <= 1) return;
  for (int i = s; i < t; ++i) {
    int a = alpha[order ? order[i] : i];
    if (a < 0) {
      atomicOr(flags, (unsigned)kFlagUndef);
      return;
    }
  }
  for (int i = s + 1; i < t; ++i) {
    int p = sorted[i];
    int kp = alpha[order ? order[p] : p] % 1000000000;
    int j = i;
    while (j > s) {
      int q = sorted[j - 1];
      int kq = alpha[order ? order[q] : q] % 1000000000;
      if (kq <= kp) break;
      sorted[j] = q;
      --j;
    }
    sorted[j] = p;
  }
}

// ---------------------------------------------------------------- A13 merged arrays
__global__ void k_copy_src(const double* __restrict__ P, int n, int off, const int* __restrict__ ndPS,
                           double* __restrict__ ix, int* __restrict__ al, int* __restrict__ nbr) {
  int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= n) return;
  int p = id + ndPS[id];
  ix[2 * p] = P[2 * (off + id)];
  ix[2 * p + 1] = P[2 * (off + id) + 1];
  al[p] = -100;
  nbr[p] = -100;
}

// one edge run of the reference's copy loop (:7556-7656).  entry(pos) maps a
// position of the alpha-sorted order to a unique-record index.
template <bool BASE>
__global__ void k_copy_runs(int n, int K, const int* __restrict__ allPS,
                            const int* __restrict__ ndPS, const int* __restrict__ sorted,
                            const int* __restrict__ order, const int* __restrict__ ids, int idShift,
                            const int* __restrict__ ut, const double* __restrict__ isxy,
                            const int* __restrict__ avals, double* __restrict__ ix,
                            int* __restrict__ al, int* __restrict__ NI) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int s = allPS[e];
  if (allPS[e + 1] == s) return;
  auto entry = [&](int pos) { return order ? order[sorted[pos]] : sorted[pos]; };
  int bid = s;
  int lid = entry(bid);
  int t = ut[lid];
  bool deg = BASE ? (t == 2 || t == 4 || t == 6 || t == 8)
                  : (t == 3 || t == 4 || t == 5 || t == 7 || t == 8);
  if (deg) {
    int slot = e + ndPS[e];
    al[slot] = avals[lid];
    NI[lid] = slot;
    if (bid < K - 1) lid = entry(++bid);
  }
  int edge = (ids[lid] >> 1) - idShift;
  // a run holding only its degenerate entry hands the loop to the next
  // edge's entries; the reference rewrites those slots when it reaches that
  // edge, so nothing is written here
  if (edge != e) return;
  int ns = ndPS[e], ne = ndPS[e + 1];
  for (int q = 0; q < ne - ns; ++q) {
    int slot = ns + e + 1 + q;
    ix[2 * slot] = isxy[2 * lid];
    ix[2 * slot + 1] = isxy[2 * lid + 1];
    al[slot] = avals[lid];
    NI[lid] = slot;
    if (bid < K - 1) lid = entry(++bid);
  }
}

__global__ void k_winner(const int* __restrict__ tgt, int K, int* __restrict__ win) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K) return;
  atomicMax(&win[tgt[i]], i);
}

__global__ void k_nbr_apply(const int* __restrict__ win, int n, const int* __restrict__ otherNI,
                            int* __restrict__ nbr) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int w = win[p];
  if (w >= 0) nbr[p] = otherNI[w] + 1;
}

// ---------------------------------------------------------------- A14 labels
__global__ void k_labels(int nB, int nQ, const double* __restrict__ ixB,
                         const double* __restrict__ ixC, const int* __restrict__ alB,
                         const int* __restrict__ nbB, int* __restrict__ labB,
                         int* __restrict__ cWin, unsigned* __restrict__ flags) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nB) return;
  labB[i] = 0;
  if (alB[i] == -100) return;
  double cx = ixB[2 * i], cy = ixB[2 * i + 1];
  int tm = (i - 1 == -1) ? nB - 1 : i - 1;  // getCircularId
  double pmx = ixB[2 * tm], pmy = ixB[2 * tm + 1];
  int pMN = alB[tm] != -100 ? nbB[tm] - 1 : -100;
  int tp = (i + 1 == nB) ? 0 : i + 1;
  double ppx = ixB[2 * tp], ppy = ixB[2 * tp + 1];
  int pPN = alB[tp] != -100 ? nbB[tp] - 1 : -100;
  int nId = nbB[i] - 1;
  int qt[2];
  for (int side = 0; side < 2; ++side) {
    int q = side == 0 ? nId - 1 : nId + 1;
    if (q == nQ) q = 0;
    else if (q == -1) q = nQ - 1;
    if (q < 0 || q >= nQ) {
      atomicOr(flags, (unsigned)kFlagUndef);
      return;
    }
    double qx = ixC[2 * q], qy = ixC[2 * q + 1];
    int r;
    if (pMN != -100 && pMN == q) r = 2;
    else if (pPN != -100 && pPN == q) r = 3;
    else {
      double s1 = area3(qx, qy, pmx, pmy, cx, cy);
      double s2 = area3(qx, qy, cx, cy, ppx, ppy);
      double s3 = area3(pmx, pmy, cx, cy, ppx, ppy);
      if (s3 > 0) r = (s1 > 0 && s2 > 0) ? 0 : 1;
      else r = (s1 < 0 && s2 < 0) ? 1 : 0;
    }
    qt[side] = r;
  }
  int qm = qt[0], qp = qt[1], lab;
  if ((qm == 0 && qp == 1) || (qm == 1 && qp == 0)) lab = 1;
  else if ((qm == 0 && qp == 0) || (qm == 1 && qp == 1)) lab = 2;
  else if ((qp == 3 && qm == 1) || (qm == 3 && qp == 1)) lab = 3;
  else if ((qp == 3 && qm == 0) || (qm == 3 && qp == 0)) lab = 4;
  else if ((qp == 3 && qm == 2) || (qm == 3 && qp == 2)) lab = 5;
  else if ((qm == 2 && qp == 1) || (qp == 2 && qm == 1)) lab = 6;
  else if ((qm == 2 && qp == 0) || (qp == 2 && qm == 0)) lab = 7;
  else lab = -102;
  labB[i] = lab;
  if (nId < 0 || nId >= nQ) {
    atomicOr(flags, (unsigned)kFlagUndef);
    return;
  }
  atomicMax(&cWin[nId], i);
}

__global__ void k_labels_c(int nQ, const int* __restrict__ cWin, const int* __restrict__ labB,
                           int* __restrict__ labC) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nQ) return;
  int w = cWin[q];
  labC[q] = w >= 0 ? labB[w] : 0;
}

}  // namespace

// ============================================================== stage_overlay
int Pipeline::stage_overlay(int cType, OverlayOut& out) {
  cudaStream_t st = st_;
  const int cListId = cType - 1;
  const int bSize = nb;
  const int cStart = hcS[cListId];
  const int cSize = hcS[cType] - hcS[cListId] - 1;
  std::vector<int> hstart(k + 2);
  hstart[0] = 0;
  for (int t = 0; t <= k; ++t) hstart[t + 1] = nb + hcc[t];
  int* tstart = (int*)pool_.get("type_start", sizeof(int) * (k + 2));
  cudaMemcpyAsync(tstart, hstart.data(), sizeof(int) * (k + 2), cudaMemcpyHostToDevice, st);

  // ---- A8 candidate tests
  void* sscr = pool_.get("scan_scr4", scan_scratch_bytes(nCover + 2));
  auto* counters = (unsigned long long*)pool_.get("cand_counters", 64);
  if (pool_.failed) return fail(kENoMem, "device allocation failed (candidates)");
  long long W = 0;
  // packed leaf entries, edge y boxes and the node tiles of the test kernel
  int4* pack = (int4*)pool_.get("cand_pack", sizeof(int4) * (nLeafEnt + 1));
  float2* ybox = (float2*)pool_.get("cand_ybox", sizeof(float2) * (E + 1));
  int2* abx = (int2*)pool_.get("cand_ab", sizeof(int2) * (E + 1));
  int* nheads = (int*)pool_.get("cand_nheads", sizeof(int) * (nCover + 2));
  if (pool_.failed) return fail(kENoMem, "device allocation failed (candidate tables)");
  if (cType == 1) {
    if (nLeafEnt > 0) {
      ::sbc::KProbe kp_("k_pack_leaf", st);
      k_pack_leaf<<<grid_for(nLeafEnt, 256), 256, 0, st>>>(nLeafEnt, le_edge, le_leaf, e_id, tstart, k,
                                                        bP, cP, pack);
    }
    ::sbc::KProbe kp_("k_edge_ybox", st);
    k_edge_ybox<<<grid_for(E, 256), 256, 0, st>>>(E, e_id, tstart, k, bP, cP, ybox, abx, aft, bef);
  }
  float4* vfB = (float4*)pool_.get("cand_vfB", sizeof(float4) * (nb + 1));
  float4* vfC = (float4*)pool_.get("cand_vfC", sizeof(float4) * ((long long)clSize + k));
  if (pool_.failed) return fail(kENoMem, "device allocation failed (vertex tables)");
  if (cType == 1) {
    {
      ::sbc::KProbe kp_("k_vertex_f4", st);
      k_vertex_f4<<<grid_for(nb + 1, 256), 256, 0, st>>>(nb + 1, bP, vfB);
    }
    ::sbc::KProbe kp_("k_vertex_f4", st);
    k_vertex_f4<<<grid_for((long long)clSize + k, 256), 256, 0, st>>>((long long)clSize + k, cP, vfC);
  }
  {
    ::sbc::KProbe kp_("k_node_heads", st);
    k_node_heads<<<grid_for(nCover + 1, 256), 256, 0, st>>>(nCover, cov_node, nheads);
  }
  exclusive_scan_i32(nheads, nCover + 1, sscr, st);
  int nNodes = 0;
  cudaMemcpyAsync(&nNodes, nheads + nCover, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  int* nodes = (int*)pool_.get("cand_nodes", sizeof(int) * (nNodes + 1));
  long long* items = (long long*)pool_.get("cand_items", sizeof(long long) * (nNodes + 1));
  long long* wun = (long long*)pool_.get("cand_wunits", sizeof(long long) * (nNodes + 1));
  long long* smalls = (long long*)pool_.get("cand_smalls", sizeof(long long) * (nNodes + 1));
  int4* desc = (int4*)pool_.get("cand_desc", sizeof(int4) * 3 * (nNodes + 1));
  if (pool_.failed) return fail(kENoMem, "device allocation failed (candidate nodes)");
  if (nCover > 0) {
    ::sbc::KProbe kp_("k_node_list", st);
    k_node_list<<<grid_for(nCover, 256), 256, 0, st>>>(nCover, cov_node, nheads, nodes);
  }
  {
    ::sbc::KProbe kp_("k_node_items", st);
    k_node_items<<<grid_for(nNodes + 1, 256), 256, 0, st>>>(nNodes, nodes, node_start, node_end,
                                                          cov_edge, tstart, cType, logL, numLeaves,
                                                          le_off, items, smalls, wun, desc);
  }
  exclusive_scan_i64(items, nNodes + 1, sscr, st);
  exclusive_scan_i64(smalls, nNodes + 1, sscr, st);
  exclusive_scan_i64(wun, nNodes + 1, sscr, st);
  long long nItems = 0, nSmall = 0;
  cudaMemcpyAsync(&nItems, items + nNodes, sizeof(long long), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&nSmall, smalls + nNodes, sizeof(long long), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&W, wun + nNodes, sizeof(long long), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  int4* rec = (int4*)pool_.get("cand_rec", sizeof(int4) * (nItems + 1));
  int2* srec = (int2*)pool_.get("cand_srec", sizeof(int2) * (nSmall + 1));
  if (pool_.failed) return fail(kENoMem, "device allocation failed (candidate tiles)");
  if (nNodes > 0) {
    ::sbc::KProbe kp_("k_expand_items", st);
    k_expand_items<<<grid_for(nNodes, 256), 256, 0, st>>>(nNodes, items, smalls, desc, rec, srec);
  }

  // filter: node tiles -> survivor pairs (grow and retry on overflow)
  long long scap = sv_cap_ > 0 ? sv_cap_ : 8LL * E + (1 << 20);
  long long nsurv = 0;
  int2* surv = nullptr;
  auto* counters3 = counters;
  for (int attempt = 0; attempt < 2; ++attempt) {
    surv = (int2*)pool_.get("cand_surv", sizeof(int2) * (scap + 1));
    if (pool_.failed) return fail(kENoMem, "device allocation failed (candidate survivors)");
    cudaMemsetAsync(counters3, 0, 24, st);
    if (nItems > 0) {
      ::sbc::KProbe kp_("k_cand_test", st);
      k_cand_test<<<grid_for(nItems * 32, kCandBlock), kCandBlock, 0, st>>>(
          rec, desc, nItems, cov_edge, logL, pack, ybox, abx, counters3, scap, surv);
    }
    if (nSmall > 0) {
      ::sbc::KProbe kp_("k_cand_small", st);
      k_cand_small<<<grid_for(nSmall, kCandBlock), kCandBlock, 0, st>>>(
          srec, nSmall, desc, cov_edge, logL, pack, ybox, abx, counters3, scap, surv);
    }
    unsigned long long hs = 0;
    cudaMemcpyAsync(&hs, counters3 + 2, sizeof(hs), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    nsurv = (long long)hs;
    if (nsurv <= scap) break;
    scap = nsurv + (1 << 20);
  }
  sv_cap_ = scap;
  // exact LSMF + classification of the survivors
  long long cap = 4LL * E + (1 << 20);
  if (cap > nsurv + 1) cap = nsurv + 1;
  int *rb = nullptr, *rc = nullptr, *rt = nullptr;
  unsigned long long* rkey = nullptr;
  rb = (int*)pool_.get("raw_b", sizeof(int) * cap);
  rc = (int*)pool_.get("raw_c", sizeof(int) * cap);
  rt = (int*)pool_.get("raw_t", sizeof(int) * cap);
  rkey = (unsigned long long*)pool_.get("raw_key", sizeof(unsigned long long) * cap);
  if (pool_.failed) return fail(kENoMem, "device allocation failed (raw candidates)");
  if (nsurv > 0) {
    ::sbc::KProbe kp_("k_cand_exact", st);
    k_cand_exact<<<grid_for(nsurv, kExChunk), kExBlock, 0, st>>>(nsurv, surv, cov_edge, e_id, bP,
                                                                 cP, vfB, vfC, counters3, cap, rb,
                                                                 rc, rt, rkey);
  }
  unsigned long long hcnt[2];
  cudaMemcpyAsync(hcnt, counters3, 16, cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  long long nraw = (long long)hcnt[0];
  long long ntested = (long long)hcnt[1];
  if (nraw > cap) return fail(kEInternal, "candidate hit buffer overflow");
  out.survivors = nsurv;
  if (nraw >= (1LL << 31)) return fail(kEInput, "too many candidate hits");
  out.raw_hits = nraw;
  out.tests = ntested;
  out.work = W;

  // ---- A9 dedup: stable sort by base id, per-edge key order, first per overlay edge
  long long R = nraw;
  auto* sk = (unsigned*)pool_.get("dd_keys", sizeof(unsigned) * (R + 1));
  auto* sv = (unsigned*)pool_.get("dd_vals", sizeof(unsigned) * (R + 1));
  auto* sk2 = (unsigned*)pool_.get("dd_keys2", sizeof(unsigned) * (R + 1));
  auto* sv2 = (unsigned*)pool_.get("dd_vals2", sizeof(unsigned) * (R + 1));
  int* heads = (int*)pool_.get("dd_heads", sizeof(int) * (R + 2));
  int* segstart = (int*)pool_.get("dd_segstart", sizeof(int) * (R + 2));
  auto* ord = (unsigned*)pool_.get("dd_ord", sizeof(unsigned) * (R + 1));
  int* keep = (int*)pool_.get("dd_keep", sizeof(int) * (R + 2));
  void* rscr = pool_.get("radix_scr_dd", radix_scratch_bytes(R + 1));
  void* sscr2 = pool_.get("scan_scr5", scan_scratch_bytes(R + 2));
  if (pool_.failed) return fail(kENoMem, "device allocation failed (dedup)");
  int K = 0;
  int nseg = 0;
  if (R > 0) {
    {
      ::sbc::KProbe kp_("k_iota_keys", st);
      k_iota_keys<<<grid_for(R, 256), 256, 0, st>>>(rb, R, sk, sv);
    }
    int bits = 1;
    while ((1LL << bits) < 2LL * bSize) ++bits;
    radix_sort_u32(sk, sv, sk2, sv2, R, bits, rscr, st);
    {
      ::sbc::KProbe kp_("k_seg_heads", st);
      k_seg_heads<<<grid_for(R + 1, 256), 256, 0, st>>>(sk, R, heads);
    }
    exclusive_scan_i32(heads, R + 1, sscr2, st);
    cudaMemcpyAsync(&nseg, heads + R, sizeof(int), cudaMemcpyDeviceToHost, st);
    {
      ::sbc::KProbe kp_("k_seg_starts", st);
      k_seg_starts<<<grid_for(R + 1, 256), 256, 0, st>>>(heads, R, segstart);
    }
    cudaStreamSynchronize(st);
    {
      ::sbc::KProbe kp_("k_dedup", st);
      k_dedup<<<grid_for(nseg, 128), 128, 0, st>>>(segstart, nseg, sv, rkey, rc, ord, keep);
    }
    cudaMemsetAsync(keep + R, 0, sizeof(int), st);
    exclusive_scan_i32(keep, R + 1, sscr2, st);
    cudaMemcpyAsync(&K, keep + R, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
  }
  out.unique = K;
  int* ub = (int*)pool_.get("u_b", sizeof(int) * (K + 1));
  int* uc = (int*)pool_.get("u_c", sizeof(int) * (K + 1));
  int* ut = (int*)pool_.get("u_t", sizeof(int) * (K + 1));
  if (pool_.failed) return fail(kENoMem, "device allocation failed (unique)");
  if (K > 0) {
    {
      ::sbc::KProbe kp_("k_dedup_write", st);
      k_dedup_write<<<grid_for(R, 256), 256, 0, st>>>(ord, keep, R, rb, rc, rt, ub, uc, ut);
    }
  }

  // ---- A10 counts (radixsort of overlay ids by value mod 10^d must be complete)
  {
    long long m = 1;
    long long v = 2LL * clSize;
    while (v > 0) {
      v /= 10;
      m *= 10;
    }
    long long maxCid = 2LL * (hcS[k] - 2);
    if (maxCid >= m) return fail(kEUndef, "overlay ids exceed the reference's radix digit count");
  }
  int* bAll = (int*)pool_.get("bAll", sizeof(int) * (bSize + 2));
  int* bND = (int*)pool_.get("bND", sizeof(int) * (bSize + 2));
  int* cAll = (int*)pool_.get("cAll", sizeof(int) * (cSize + 2));
  int* cND = (int*)pool_.get("cND", sizeof(int) * (cSize + 2));
  auto* csk = (unsigned*)pool_.get("cs_keys", sizeof(unsigned) * (K + 1));
  auto* csv = (unsigned*)pool_.get("cs_vals", sizeof(unsigned) * (K + 1));
  auto* csk2 = (unsigned*)pool_.get("cs_keys2", sizeof(unsigned) * (K + 1));
  auto* csv2 = (unsigned*)pool_.get("cs_vals2", sizeof(unsigned) * (K + 1));
  void* rscr2 = pool_.get("radix_scr_cs", radix_scratch_bytes(K + 1));
  void* sscr3 = pool_.get("scan_scr6", scan_scratch_bytes(bSize + cSize + 4));
  if (pool_.failed) return fail(kENoMem, "device allocation failed (counts)");
  cudaMemsetAsync(bAll, 0, sizeof(int) * (bSize + 1), st);
  cudaMemsetAsync(bND, 0, sizeof(int) * (bSize + 1), st);
  cudaMemsetAsync(cAll, 0, sizeof(int) * (cSize + 1), st);
  cudaMemsetAsync(cND, 0, sizeof(int) * (cSize + 1), st);
  if (K > 0) {
    {
      ::sbc::KProbe kp_("k_counts", st);
      k_counts<<<grid_for(K, 256), 256, 0, st>>>(ub, uc, ut, K, cStart, bAll, bND, cAll, cND);
    }
    {
      ::sbc::KProbe kp_("k_iota_keys", st);
      k_iota_keys<<<grid_for(K, 256), 256, 0, st>>>(uc, K, csk, csv);
    }
    int bits = 1;
    while ((1LL << bits) < 2LL * (clSize + k)) ++bits;
    radix_sort_u32(csk, csv, csk2, csv2, K, bits, rscr2, st);
  }
  exclusive_scan_i32(bAll, bSize + 1, sscr3, st);
  exclusive_scan_i32(bND, bSize + 1, sscr3, st);
  exclusive_scan_i32(cAll, cSize + 1, sscr3, st);
  exclusive_scan_i32(cND, cSize + 1, sscr3, st);
  int hb = 0, hc = 0;
  cudaMemcpyAsync(&hb, bND + bSize, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&hc, cND + cSize, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  const int nB = bSize + hb, nQ = cSize + hc;
  out.slots_b = nB;
  out.slots_c = nQ;
  const int* csorted = (const int*)csv;

  // ---- A11 records
  double* isxy = (double*)pool_.get("isxy", sizeof(double) * 2 * (K + 1));
  int* aB = (int*)pool_.get("aB", sizeof(int) * (K + 1));
  int* aC = (int*)pool_.get("aC", sizeof(int) * (K + 1));
  int* sB = (int*)pool_.get("sB", sizeof(int) * (K + 1));
  int* sC = (int*)pool_.get("sC", sizeof(int) * (K + 1));
  if (pool_.failed) return fail(kENoMem, "device allocation failed (records)");
  clear_flags();
  if (K > 0) {
    {
      ::sbc::KProbe kp_("k_records", st);
      k_records<<<grid_for(K, 256), 256, 0, st>>>(ub, uc, ut, K, bP, cP, isxy, aB, aC);
    }
    // ---- A12 per-edge alpha sorts
    {
      ::sbc::KProbe kp_("k_alpha_sort", st);
      k_alpha_sort<<<grid_for(bSize, 128), 128, 0, st>>>(bSize, bAll, bND, aB, nullptr, sB, d_flags);
    }
    {
      ::sbc::KProbe kp_("k_alpha_sort", st);
      k_alpha_sort<<<grid_for(cSize, 128), 128, 0, st>>>(cSize, cAll, cND, aC, csorted, sC, d_flags);
    }
  }

  // ---- A13 merged arrays
  double* ixB = (double*)pool_.get("ixB", sizeof(double) * 2 * nB);
  double* ixC = (double*)pool_.get("ixC", sizeof(double) * 2 * nQ);
  int* alB = (int*)pool_.get("alB", sizeof(int) * nB);
  int* alC = (int*)pool_.get("alC", sizeof(int) * nQ);
  int* nbB = (int*)pool_.get("nbB", sizeof(int) * nB);
  int* nbC = (int*)pool_.get("nbC", sizeof(int) * nQ);
  int* bNI = (int*)pool_.get("bNI", sizeof(int) * (K + 1));
  int* cNI = (int*)pool_.get("cNI", sizeof(int) * (K + 1));
  int* winB = (int*)pool_.get("winB", sizeof(int) * nB);
  int* winC = (int*)pool_.get("winC", sizeof(int) * nQ);
  int* labB = (int*)pool_.get("labB", sizeof(int) * nB);
  int* labC = (int*)pool_.get("labC", sizeof(int) * nQ);
  if (pool_.failed) return fail(kENoMem, "device allocation failed (merged)");
  // the reference's arrays come from a zero-filled heap: slots no loop writes read 0
  cudaMemsetAsync(ixB, 0, sizeof(double) * 2 * nB, st);
  cudaMemsetAsync(ixC, 0, sizeof(double) * 2 * nQ, st);
  cudaMemsetAsync(alB, 0, sizeof(int) * nB, st);
  cudaMemsetAsync(alC, 0, sizeof(int) * nQ, st);
  cudaMemsetAsync(nbB, 0, sizeof(int) * nB, st);
  cudaMemsetAsync(nbC, 0, sizeof(int) * nQ, st);
  {
    ::sbc::KProbe kp_("k_copy_src", st);
    k_copy_src<<<grid_for(bSize, 256), 256, 0, st>>>(bP, bSize, 0, bND, ixB, alB, nbB);
  }
  {
    ::sbc::KProbe kp_("k_copy_src", st);
    k_copy_src<<<grid_for(cSize, 256), 256, 0, st>>>(cP, cSize, cStart, cND, ixC, alC, nbC);
  }
  cudaMemsetAsync(bNI, 0, sizeof(int) * (K + 1), st);
  cudaMemsetAsync(cNI, 0, sizeof(int) * (K + 1), st);
  if (K > 0) {
    {
      ::sbc::KProbe kp_("k_copy_runs", st);
      k_copy_runs<true><<<grid_for(bSize, 128), 128, 0, st>>>(bSize, K, bAll, bND, sB, nullptr, ub, 0,
                                                           ut, isxy, aB, ixB, alB, bNI);
    }
    {
      ::sbc::KProbe kp_("k_copy_runs", st);
      k_copy_runs<false><<<grid_for(cSize, 128), 128, 0, st>>>(cSize, K, cAll, cND, sC, csorted, uc,
                                                            cStart, ut, isxy, aC, ixC, alC, cNI);
    }
    cudaMemsetAsync(winB, 0xff, sizeof(int) * nB, st);
    cudaMemsetAsync(winC, 0xff, sizeof(int) * nQ, st);
    {
      ::sbc::KProbe kp_("k_winner", st);
      k_winner<<<grid_for(K, 256), 256, 0, st>>>(bNI, K, winB);
    }
    {
      ::sbc::KProbe kp_("k_winner", st);
      k_winner<<<grid_for(K, 256), 256, 0, st>>>(cNI, K, winC);
    }
    {
      ::sbc::KProbe kp_("k_nbr_apply", st);
      k_nbr_apply<<<grid_for(nB, 256), 256, 0, st>>>(winB, nB, cNI, nbB);
    }
    {
      ::sbc::KProbe kp_("k_nbr_apply", st);
      k_nbr_apply<<<grid_for(nQ, 256), 256, 0, st>>>(winC, nQ, bNI, nbC);
    }
  }

  // ---- A14 initial labels
  cudaMemsetAsync(winC, 0xff, sizeof(int) * nQ, st);
  {
    ::sbc::KProbe kp_("k_labels", st);
    k_labels<<<grid_for(nB, 256), 256, 0, st>>>(nB, nQ, ixB, ixC, alB, nbB, labB, winC, d_flags);
  }
  {
    ::sbc::KProbe kp_("k_labels_c", st);
    k_labels_c<<<grid_for(nQ, 256), 256, 0, st>>>(nQ, winC, labB, labC);
  }
  if (read_flags() & kFlagUndef)
    return fail(kEUndef, "reference behaviour undefined (negative alpha key or bad neighbour)");

  // ---- A15-A19 back end
  Merged m;
  m.nB = nB;
  m.nQ = nQ;
  m.K = K;
  m.bSize = bSize;
  m.cSize = cSize;
  m.cStart = cStart;
  m.ixB = ixB;
  m.ixC = ixC;
  m.alB = alB;
  m.nbB = nbB;
  m.nbC = nbC;
  m.labB = labB;
  m.labC = labC;
  m.bND = bND;
  m.cND = cND;
  m.bP = bP;
  m.cP = cP;
  // keep the intermediate arrays reachable for diagnostics
  dbg_ub = ub; dbg_uc = uc; dbg_ut = ut; dbg_K = K;
  dbg_isxy = isxy; dbg_aB = aB; dbg_aC = aC;
  dbg_ixB = ixB; dbg_ixC = ixC; dbg_alB = alB; dbg_alC = alC; dbg_nbB = nbB; dbg_nbC = nbC;
  dbg_labB = labB; dbg_labC = labC; dbg_nB = nB; dbg_nQ = nQ;
  return run_backend(*this, m, out);
}

}  // namespace sbc
