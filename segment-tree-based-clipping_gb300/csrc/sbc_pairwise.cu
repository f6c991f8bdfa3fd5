// sbc_pairwise.cu -- one base polygon against many overlays, pairwise.
//
// The result for overlay i is the reference's `seg base overlay_i` (the same
// rings as sbc_clip_pair on that pair).  Every pair would build its own
// segment tree over the base's edges and the overlay's; here no pair builds
// one.  The base is prepared once: its sorted distinct x values, the rank of
// each vertex among them, and a uniform grid over its edge boxes.  A pair's
// tree quantities then follow from ranks alone:
//
//  * With no vertical edge (equal x at both ends) in either polygon and no x
//    value shared between them, the elementary points of the pair
//    (constructElementaryIntervalsArrayMulticore, oacc_segment_tree.cpp:
//    4513-4692) are the distinct x values of both polygons in order, without
//    the largest, padded with the second largest up to 2^k + 1 entries.
//    Position t of a value is its rank among the base's values plus its rank
//    among the overlay's.
//  * findBoarder (:420-460) runs over those positions with the zero border
//    slot at z (preparePointsToNodeMapMulticore, :1970-2008): its comparisons
//    become integer comparisons of positions, so its search path, including
//    the misses the zero slot causes, is followed exactly.
//  * The end-list leaves and the covered leaf range of an edge
//    (insertToLeafLevelEdgeListMulticore :2010-2113, insertEdgeParallel
//    :2496-2564) and the emission rule of the candidate loops (:6010-6244)
//    follow from those positions as in the pair pipeline.
//
// A pair that breaks one of these conditions, or whose arrays take a path
// the sparse back end does not follow (see below), is clipped by the pair
// pipeline instead, so every pair's result is the pair pipeline's.
//
// Candidates: one thread per overlay edge visits the base grid cells its box
// covers; a base edge is tested in the cell holding the low corner of the two
// boxes' overlap only, so every box-overlapping pair is tested once.
//
// Back end: one warp per pair runs rows A9-A18 (src/clip.cpp:368-695,
// foster/polyclip.h:337-787), its lanes sharing the per-record, per-run and
// per-slot steps, with the overlay's merged arrays in full and the
// base's only where intersections are: the base's merged list holds ~n_b
// plain vertices per pair, so its linked list is built with run nodes (a
// stretch of plain vertices as one node, sbc_serial.cuh) and pointInPoly
// against it adds the winding steps of the run-internal base edges from one
// row of the grid.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/sbclip.h"
#include "sbc_pipeline.cuh"
#include "sbc_pairops.cuh"
#include "sbc_serial.cuh"

namespace sbc {

namespace {

constexpr unsigned kFullMask = 0xffffffffu;
constexpr int kPwMaxOverlay = 16384;  // larger overlays go to the pair pipeline
constexpr int kPwMaxCells = 1 << 14;  // an overlay edge box over more cells: pair pipeline
constexpr int kPwLongCells = 64;      // base edges over more cells per axis skip the grid
constexpr int kPwPrepThreads = 256;
constexpr int kPwPairBlock = 64;

enum { PW_FAST = 0, PW_FALLBACK = 1, PW_INPUT = 2 };
enum { PS_FALLBACK = 4 };

// base statistics (device)
struct PwBaseStats {
  unsigned long long mnx, mxx, mny, mxy;  // dkey of min/max x and y
  double ext;                             // sum of max(|dx|, |dy|) over edges
  unsigned flags;                         // 1: non-finite, 2: vertical edge
};

struct PwGrid {
  float x0, y0, inv;
  int gx, gy;
};

__device__ __forceinline__ int pw_cellx(const PwGrid& g, float x) {
  const float t = floorf(__fmul_rn(__fsub_rn(x, g.x0), g.inv));
  return t < 0.f ? 0 : (t >= (float)g.gx ? g.gx - 1 : (int)t);
}
__device__ __forceinline__ int pw_celly(const PwGrid& g, float y) {
  const float t = floorf(__fmul_rn(__fsub_rn(y, g.y0), g.inv));
  return t < 0.f ? 0 : (t >= (float)g.gy ? g.gy - 1 : (int)t);
}

// per overlay: how it is clipped and its tree parameters
struct PwPair {
  int mode;   // PW_FAST / PW_FALLBACK / PW_INPUT
  int nuc;    // distinct overlay x values
  int count;  // elementary points before padding
  int epc;    // 2^k + 1
  int logL;
  int z;      // zero border slot
};

struct PwHit {
  int pair, b, j, type;
  unsigned long long key;  // first emission
  double al, bt;           // lineSegmentIntersection's alpha and beta
};

__device__ __forceinline__ int lower_bound_d(const double* a, int n, double x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (a[m] < x) lo = m + 1;
    else hi = m;
  }
  return lo;
}

// ------------------------------------------------------------------ tree by rank
struct PwTree {
  int count, epc, z, L, logL;
};

// positions [lo, hi) of the elementary entries equal to the value of
// combined rank r (entries before lo are smaller)
__device__ __forceinline__ void pw_lohi(const PwTree& T, int r, int* lo, int* hi) {
  if (r < T.count - 1) {
    *lo = r;
    *hi = r + 1;
  } else if (r == T.count - 1) {
    *lo = r;
    *hi = T.epc;
  } else {
    *lo = *hi = T.epc;
  }
}

// end-list leaves and covered leaf range of an edge whose start (smaller x)
// s has combined rank rs and whose end e has rank re
__device__ void pw_edge_tree(const PwTree& T, int rs, double s, int re, double e, int* aft,
                             int* bef, int2* lr) {
  const int L = T.L, epc = T.epc;
  auto J = [&](int m) { return m < T.z ? m : (m == T.z ? epc - 1 : m - 1); };
  auto eqnext = [&](int i) { return i >= T.count - 1; };  // ea[i] == ea[i+1]
  int lo, hi;
  pw_lohi(T, re, &lo, &hi);
  const int hiE = hi;
  int a = -1, b = -1;
  const int en = border_by_position(T.epc, T.z, lo, hi, e);
  if (en >= 0) {
    const int j = J(en);
    int node = 0;
    if (j <= epc - 2) {
      const int i = j + 1;
      node = L + i;
      if (i != 1 && i + 1 < epc && eqnext(i)) node = L + i + 1;
    }
    if (node >= L && node < 2 * L && !eqnext(node - L)) a = node;
  }
  pw_lohi(T, rs, &lo, &hi);
  const int st = border_by_position(T.epc, T.z, lo, hi, s);
  if (st >= 0) {
    const int j = J(st);
    int node = 0;
    if (j <= epc - 2) node = L + j;
    if (node >= L && node < 2 * L && !eqnext(node - L)) b = node;
  }
  *aft = a;
  *bef = b;
  const int l = lo < L ? lo : L;
  int r1 = hiE - 1;
  r1 = r1 < 0 ? 0 : (r1 > L ? L : r1);
  *lr = make_int2(l, r1 > l ? r1 : l);
}

// ------------------------------------------------------------------ base preparation
__global__ void k_pw_base_edges(int nb, const double* __restrict__ b,
                                unsigned long long* __restrict__ keys, unsigned* __restrict__ vals,
                                float4* __restrict__ fbox, PwBaseStats* st) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nb) return;
  const int w = v + 1 == nb ? 0 : v + 1;
  const double x0 = b[2 * v], y0 = b[2 * v + 1], x1 = b[2 * w], y1 = b[2 * w + 1];
  keys[v] = dkey(x0);
  vals[v] = v;
  fbox[v] = make_float4(__double2float_rd(fmin(x0, x1)), __double2float_rd(fmin(y0, y1)),
                        __double2float_ru(fmax(x0, x1)), __double2float_ru(fmax(y0, y1)));
  unsigned f = 0;
  if (!isfinite(x0) || !isfinite(y0)) f |= 1u;
  if (x0 == x1) f |= 2u;
  if (f) atomicOr(&st->flags, f);
  atomicMin(&st->mnx, dkey(x0));
  atomicMax(&st->mxx, dkey(x0));
  atomicMin(&st->mny, dkey(y0));
  atomicMax(&st->mxy, dkey(y0));
  atomicAdd(&st->ext, fmax(fabs(x1 - x0), fabs(y1 - y0)));
}

__global__ void k_pw_uflag(int n, const unsigned long long* __restrict__ keys, int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  flag[i] = (i < n && (i == 0 || keys[i] != keys[i - 1])) ? 1 : 0;
}

// after the exclusive scan of the flags: distinct values and vertex ranks
__global__ void k_pw_uscatter(int n, const unsigned long long* __restrict__ keys,
                              const unsigned* __restrict__ vals, const int* __restrict__ pre,
                              const double* __restrict__ b, double* __restrict__ ub,
                              int* __restrict__ rank) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool first = i == 0 || keys[i] != keys[i - 1];
  const int u = pre[i] + (first ? 0 : -1);
  const int v = (int)vals[i];
  if (first) ub[u] = b[2 * v];
  rank[v] = u;
}

__global__ void k_pw_grid_count(int nb, const float4* __restrict__ fbox, PwGrid g,
                                int* __restrict__ cnt, int* __restrict__ lng,
                                unsigned* __restrict__ nlong) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nb) return;
  const float4 f = fbox[e];
  const int cx0 = pw_cellx(g, f.x), cx1 = pw_cellx(g, f.z);
  const int cy0 = pw_celly(g, f.y), cy1 = pw_celly(g, f.w);
  if (cx1 - cx0 >= kPwLongCells || cy1 - cy0 >= kPwLongCells) {
    lng[atomicAdd(nlong, 1u)] = e;
    return;
  }
  for (int cy = cy0; cy <= cy1; ++cy)
    for (int cx = cx0; cx <= cx1; ++cx) atomicAdd(&cnt[cy * g.gx + cx], 1);
}

__global__ void k_pw_grid_fill(int nb, const float4* __restrict__ fbox, PwGrid g,
                               const int* __restrict__ start, int* __restrict__ cur,
                               int* __restrict__ ent) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nb) return;
  const float4 f = fbox[e];
  const int cx0 = pw_cellx(g, f.x), cx1 = pw_cellx(g, f.z);
  const int cy0 = pw_celly(g, f.y), cy1 = pw_celly(g, f.w);
  if (cx1 - cx0 >= kPwLongCells || cy1 - cy0 >= kPwLongCells) return;
  for (int cy = cy0; cy <= cy1; ++cy)
    for (int cx = cx0; cx <= cx1; ++cx) {
      const int c = cy * g.gx + cx;
      ent[start[c] + atomicAdd(&cur[c], 1)] = e;
    }
}

// ------------------------------------------------------------------ overlay preparation
// One CTA per overlay of the size class (lo, hi]: sort its x values in shared
// memory, rank them, check the conditions of the rank shortcut and work out
// the pair's tree parameters.
__global__ void __launch_bounds__(kPwPrepThreads)
k_pw_overlay_prep(int nov, const long long* __restrict__ coff, const double* __restrict__ cxy,
                  int lo_n, int hi_n, const double* __restrict__ ub, int nub, int base_flags,
                  PwPair* __restrict__ pp, int* __restrict__ rankC, int* __restrict__ rankCB,
                  double* __restrict__ uval) {
  extern __shared__ unsigned long long sk[];
  const int i = blockIdx.x;
  if (i >= nov) return;
  const long long o = coff[i];
  const int n = (int)(coff[i + 1] - o);
  if (n <= lo_n || n > hi_n) return;
  const int tid = threadIdx.x;
  int P2 = 1;
  while (P2 < n) P2 <<= 1;
  int* sidx = (int*)(sk + P2);
  __shared__ int s_bad, s_cnt[kPwPrepThreads];
  if (tid == 0) s_bad = 0;
  const double* c = cxy + 2 * o;
  for (int t = tid; t < P2; t += blockDim.x) {
    if (t < n) {
      const double x = c[2 * t];
      sk[t] = dkey(x);
      sidx[t] = t;
      const double xn = c[2 * (t + 1 == n ? 0 : t + 1)];
      if (!isfinite(x) || !isfinite(c[2 * t + 1]) || x == xn) atomicOr(&s_bad, 1);
    } else {
      sk[t] = ~0ull;
      sidx[t] = -1;
    }
  }
  __syncthreads();
  for (int k = 2; k <= P2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = tid; t < P2; t += blockDim.x) {
        const int u = t ^ j;
        if (u > t) {
          const bool up = (t & k) == 0;
          const unsigned long long a = sk[t], bk = sk[u];
          if ((a > bk) == up) {
            sk[t] = bk;
            sk[u] = a;
            const int ti = sidx[t];
            sidx[t] = sidx[u];
            sidx[u] = ti;
          }
        }
      }
      __syncthreads();
    }
  }
  // distinct ranks: each thread a contiguous chunk
  const int chunk = (n + blockDim.x - 1) / blockDim.x;
  const int t0 = tid * chunk, t1 = min(n, t0 + chunk);
  int local = 0;
  for (int t = t0; t < t1; ++t) local += (t == 0 || sk[t] != sk[t - 1]) ? 1 : 0;
  s_cnt[tid] = local;
  __syncthreads();
  if (tid == 0) {
    int run = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      const int x = s_cnt[t];
      s_cnt[t] = run;
      run += x;
    }
    pp[i].nuc = run;
  }
  __syncthreads();
  {
    int u = s_cnt[tid] - 1;
    for (int t = t0; t < t1; ++t) {
      const bool first = t == 0 || sk[t] != sk[t - 1];
      if (first) {
        ++u;
        uval[o + u] = c[2 * sidx[t]];
      }
      rankC[o + sidx[t]] = u;
    }
  }
  // rank among the base's values; a shared x value breaks the shortcut
  for (int t = tid; t < n; t += blockDim.x) {
    const double x = c[2 * t];
    const int r = lower_bound_d(ub, nub, x);
    rankCB[o + t] = r;
    if (r < nub && ub[r] == x) atomicOr(&s_bad, 2);
  }
  __syncthreads();
  if (tid != 0) return;
  PwPair q = pp[i];
  q.mode = PW_FAST;
  if (n < 3) {
    q.mode = PW_INPUT;
    pp[i] = q;
    return;
  }
  if (s_bad || (base_flags & 3)) {
    q.mode = PW_FALLBACK;
    pp[i] = q;
    return;
  }
  const int nuc = q.nuc;
  const double* uc = uval + o;
  const int count = nub + nuc - 1;
  const double minI = fmin(ub[0], uc[0]), maxI = fmax(ub[nub - 1], uc[nuc - 1]);
  const double absMin = fabs(minI);
  const double dv = dadd(maxI, absMin);
  bool ok = count >= 1 && dv < 2147483647.0;
  int epc = 0, logL = 0, z = 0;
  if (ok) {
    epc = npow2_dev(count) + 1;
    while ((1 << logL) < epc - 1) ++logL;
    int digits = 1;
    for (int iv = (int)trunc(dv); iv / 10 > 0; iv /= 10) ++digits;
    double scale = 1.0;
    for (int t = 0; t < 11 - digits; ++t) scale = dmul(scale, 10.0);
    const bool shift = minI < 0;
    auto key = [&](double v) -> long long {
      return (long long)(shift ? dmul(scale, dadd(v, absMin)) : dmul(scale, v));
    };
    // the smallest elementary points in order: merge the two sorted sets
    int ib = 0, ic = 0;
    auto next_val = [&]() -> double {
      if (ic >= nuc || (ib < nub && ub[ib] < uc[ic])) return ub[ib++];
      return uc[ic++];
    };
    (void)next_val();  // ea[0]
    for (int t = 1; t < epc && ok; ++t) {
      const double v = t < count ? next_val() : (count >= 2 ? 0.0 : 0.0);
      if (t >= count) {
        ok = false;  // all points key to zero: leave it to the pair pipeline
        break;
      }
      if (key(v) != 0) break;
      if (++z > 64) ok = false;
    }
    // the last border (padding: the second largest distinct value) must key below 1e11
    if (ok) {
      int jb = nub - 1, jc = nuc - 1;
      // drop the largest, then take the next
      if (jc < 0 || (jb >= 0 && ub[jb] > uc[jc])) --jb;
      else --jc;
      const double v2 = (jc < 0 || (jb >= 0 && ub[jb] > uc[jc])) ? ub[jb] : uc[jc];
      const long long k2 = key(v2);
      if (k2 < 0 || k2 >= 100000000000LL) ok = false;
    }
  }
  if (!ok) {
    q.mode = PW_FALLBACK;
  } else {
    q.count = count;
    q.epc = epc;
    q.logL = logL;
    q.z = z;
  }
  pp[i] = q;
}

// ------------------------------------------------------------------ candidates
struct PwCandArgs {
  int nov;
  const long long* coff;
  long long totalC;
  const double* cxy;
  const double* b;
  int nb;
  PwGrid g;
  const int* gstart;
  const int* gent;
  const int* lng;
  const unsigned* nlong;
  const float4* fbox;
  PwPair* pp;
  const int* rankB;
  const int* rankC;
  const int* rankCB;
  const double* uval;
  int* tpair;                  // per overlay edge: its pair, or -1 (not on the fast path)
  long long* coffs;            // per overlay edge: its candidates' offset (count before the scan)
  int2* cand;                  // (overlay edge, base edge) of every candidate
  long long ncand;
  PwHit* raw;                  // intersecting candidates (key not yet known)
  unsigned long long rawcap;
  unsigned long long* nraw;
  PwHit* hits;
  unsigned long long cap;
  unsigned long long* nhits;
  int* pairK;
  unsigned long long* tested;  // box-overlapping pairs passing LSMF
};

// Candidates in three converged steps (one thread per overlay edge walking
// a varying number of grid entries, with the FP64 test inside the walk,
// leaves most lanes of a warp idle on the FP64 pipe):
//   1. per overlay edge, the base edges whose float boxes overlap its own,
//      each in the cell of the overlap's low corner (counted, then written);
//   2. one thread per candidate: LSMF and lineSegmentIntersection in FP64;
//   3. one thread per intersection: tree quantities and emission key.
// The overlay edge's cells; false when it is not on the fast path.
struct PwEdge {
  int i, n, j, j2;
  double q1x, q1y, q2x, q2y;
  float4 fc;
  int cx0, cx1, cy0, cy1;
};

__device__ bool pw_edge_of(const PwCandArgs& A, long long t, PwEdge& E, bool fast_only = true) {
  int lo = 0, hi = A.nov;  // pair: last i with coff[i] <= t
  while (hi - lo > 1) {
    const int m = (lo + hi) >> 1;
    if (A.coff[m] <= t) lo = m;
    else hi = m;
  }
  E.i = lo;
  if (fast_only && A.pp[E.i].mode != PW_FAST) return false;
  const long long o = A.coff[E.i];
  E.n = (int)(A.coff[E.i + 1] - o);
  E.j = (int)(t - o);
  E.j2 = E.j + 1 == E.n ? 0 : E.j + 1;
  const double* c = A.cxy + 2 * o;
  E.q1x = c[2 * E.j];
  E.q1y = c[2 * E.j + 1];
  E.q2x = c[2 * E.j2];
  E.q2y = c[2 * E.j2 + 1];
  E.fc = make_float4(__double2float_rd(fmin(E.q1x, E.q2x)), __double2float_rd(fmin(E.q1y, E.q2y)),
                     __double2float_ru(fmax(E.q1x, E.q2x)), __double2float_ru(fmax(E.q1y, E.q2y)));
  E.cx0 = pw_cellx(A.g, E.fc.x);
  E.cx1 = pw_cellx(A.g, E.fc.z);
  E.cy0 = pw_celly(A.g, E.fc.y);
  E.cy1 = pw_celly(A.g, E.fc.w);
  return true;
}

// every base edge whose box overlaps the overlay edge's, once: in the cell of
// the overlap's low corner, or from the list of long base edges
template <class F>
__device__ void pw_edge_walk(const PwCandArgs& A, const PwEdge& E, F f) {
  const float4 fc = E.fc;
  for (int cy = E.cy0; cy <= E.cy1; ++cy) {
    for (int cx = E.cx0; cx <= E.cx1; ++cx) {
      const int cell = cy * A.g.gx + cx;
      const int e0 = A.gstart[cell], e1 = A.gstart[cell + 1];
      for (int k = e0; k < e1; ++k) {
        const int be = A.gent[k];
        const float4 fb = A.fbox[be];
        if (fb.x > fc.z || fb.z < fc.x || fb.y > fc.w || fb.w < fc.y) continue;
        if (pw_cellx(A.g, fmaxf(fb.x, fc.x)) != cx || pw_celly(A.g, fmaxf(fb.y, fc.y)) != cy)
          continue;
        f(be);
      }
    }
  }
  const int nl = (int)*A.nlong;
  for (int k = 0; k < nl; ++k) {
    const int be = A.lng[k];
    const float4 fb = A.fbox[be];
    if (fb.x > fc.z || fb.z < fc.x || fb.y > fc.w || fb.w < fc.y) continue;
    f(be);
  }
}

__global__ void k_pw_cand_count(PwCandArgs A) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t > A.totalC) return;
  long long cnt = 0;
  int pair = -1;
  PwEdge E;
  if (t < A.totalC && pw_edge_of(A, t, E)) {
    if ((long long)(E.cx1 - E.cx0 + 1) * (E.cy1 - E.cy0 + 1) > kPwMaxCells) {
      atomicExch(&A.pp[E.i].mode, PW_FALLBACK);
    } else {
      pair = E.i;
      pw_edge_walk(A, E, [&](int) { ++cnt; });
    }
  }
  A.coffs[t] = cnt;
  if (t < A.totalC) A.tpair[t] = pair;
}

__global__ void k_pw_cand_fill(PwCandArgs A) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.totalC || A.tpair[t] < 0) return;
  PwEdge E;
  pw_edge_of(A, t, E, false);  // counted: fill every slot even if the pair left the fast path
  long long k = A.coffs[t];
  pw_edge_walk(A, E, [&](int be) { A.cand[k++] = make_int2((int)t, be); });
}

// appends to a counter-indexed buffer, one atomic per warp: all 32 lanes
// call it; lanes with `take` get consecutive slots
__device__ __forceinline__ unsigned long long warp_append(bool take, unsigned long long* counter) {
  const int lane = threadIdx.x & 31;
  const unsigned m = __ballot_sync(kFullMask, take);
  if (!m) return 0;
  const int leader = __ffs(m) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(m));
  base = __shfl_sync(kFullMask, base, leader);
  return base + __popc(m & ((1u << lane) - 1u));
}

__global__ void k_pw_cand_test(PwCandArgs A) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool ok = c < A.ncand;
  int ty = 0, t = 0, be = 0, i = 0, j = 0;
  double al = 0.0, bt = 0.0;
  bool lsmf = false;
  if (ok) {
    const int2 cb = A.cand[c];
    t = cb.x;
    be = cb.y;
    i = A.tpair[t];
    const long long o = A.coff[i];
    const int n = (int)(A.coff[i + 1] - o);
    j = (int)(t - o);
    const int j2 = j + 1 == n ? 0 : j + 1;
    const double* cc = A.cxy + 2 * o;
    const double q1x = cc[2 * j], q1y = cc[2 * j + 1], q2x = cc[2 * j2], q2y = cc[2 * j2 + 1];
    const int be2 = be + 1 == A.nb ? 0 : be + 1;
    const double p1x = A.b[2 * be], p1y = A.b[2 * be + 1];
    const double p2x = A.b[2 * be2], p2y = A.b[2 * be2 + 1];
    lsmf = lsmf_d(p1x, p1y, p2x, p2y, q1x, q1y, q2x, q2y);
    if (lsmf) ty = seg_isect(p1x, p1y, p2x, p2y, q1x, q1y, q2x, q2y, &al, &bt);
  }
  const unsigned tm = __ballot_sync(kFullMask, lsmf);
  if ((threadIdx.x & 31) == 0 && tm) atomicAdd(A.tested, (unsigned long long)__popc(tm));
  const unsigned long long h = warp_append(ty != 0, A.nraw);
  if (ty != 0 && h < A.rawcap) A.raw[h] = PwHit{i, be, j, ty, 0ull, al, bt};
}

__global__ void k_pw_hit_tree(PwCandArgs A, long long nraw) {
  const long long h = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool emit = false;
  PwHit x{};
  if (h < nraw) {
    x = A.raw[h];
    const PwPair q = A.pp[x.pair];
    const long long o = A.coff[x.pair];
    const int n = (int)(A.coff[x.pair + 1] - o);
    const int j = x.j, j2 = j + 1 == n ? 0 : j + 1;
    const double* c = A.cxy + 2 * o;
    const double q1x = c[2 * j], q2x = c[2 * j2];
    const PwTree T{q.count, q.epc, q.z, q.epc - 1, q.logL};
    int aftC, befC, aftB, befB;
    int2 lrC, lrB;
    const int c1 = A.rankC[o + j] + A.rankCB[o + j], c2 = A.rankC[o + j2] + A.rankCB[o + j2];
    if (q1x < q2x) pw_edge_tree(T, c1, q1x, c2, q2x, &aftC, &befC, &lrC);
    else pw_edge_tree(T, c2, q2x, c1, q1x, &aftC, &befC, &lrC);
    const int be = x.b, be2 = be + 1 == A.nb ? 0 : be + 1;
    const double p1x = A.b[2 * be], p2x = A.b[2 * be2];
    const double* uc = A.uval + o;
    const int r1 = A.rankB[be] + lower_bound_d(uc, q.nuc, p1x);
    const int r2 = A.rankB[be2] + lower_bound_d(uc, q.nuc, p2x);
    if (p1x < p2x) pw_edge_tree(T, r1, p1x, r2, p2x, &aftB, &befB, &lrB);
    else pw_edge_tree(T, r2, p2x, r1, p1x, &aftB, &befB, &lrB);
    emit = emission_q(lrB, lrC, aftB, befB, aftC, befC, A.nb + j, 2 * j, T.logL, &x.key) != 0;
  }
  const unsigned long long slot = warp_append(emit, A.nhits);
  if (emit && slot < A.cap) A.hits[slot] = x;
  // per pair counts: one atomic per group of lanes with the same pair
  const unsigned em = __ballot_sync(kFullMask, emit);
  if (emit) {
    const unsigned same = __match_any_sync(em, x.pair);
    if ((threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&A.pairK[x.pair], __popc(same));
  }
}

// The hits of every pair in the reference's record order (base id, then
// first emission; removeDuplicatesAtEdge after radixsort, src/clip.cpp:368-
// 493): a stable sort by the emission key, then a stable sort by (pair, base
// edge), then a gather.
__global__ void k_pw_hit_keys(long long nh, const PwHit* __restrict__ hits,
                              unsigned long long* __restrict__ keys, unsigned* __restrict__ vals) {
  const long long h = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= nh) return;
  keys[h] = hits[h].key;
  vals[h] = (unsigned)h;
}

__global__ void k_pw_hit_keys2(long long nh, const PwHit* __restrict__ hits,
                               const unsigned* __restrict__ vals,
                               unsigned long long* __restrict__ keys) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nh) return;
  const PwHit& x = hits[vals[t]];
  keys[t] = ((unsigned long long)(unsigned)x.pair << 32) | (unsigned)x.b;
}

__global__ void k_pw_gather(long long nh, const PwHit* __restrict__ hits,
                            const unsigned* __restrict__ vals, PwHit* __restrict__ out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nh) return;
  out[t] = hits[vals[t]];
}

// one pair's records as the pair pipeline's candidate hits
__global__ void k_pw_split(int n, const PwHit* __restrict__ h, int* __restrict__ rb,
                           int* __restrict__ rc, int* __restrict__ rt,
                           unsigned long long* __restrict__ key) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  rb[i] = 2 * h[i].b;
  rc[i] = 2 * h[i].j;
  rt[i] = h[i].type;
  key[i] = h[i].key;
}

// ------------------------------------------------------------------ one pair
struct PwCaps {
  int nc, K, nQmax, sp, capP, capQ, capR, rcap;
};

__host__ __device__ __forceinline__ PwCaps pw_caps(int nb, int nc, int K, int pass) {
  PwCaps c;
  c.nc = nc;
  c.K = K;
  c.nQmax = nc + K;
  c.sp = 2 * K + 1;
  c.capP = 7 * K + 16;
  c.capQ = c.nQmax + 2 * K + 8;
  c.capR = pass == 0 ? 2 * c.nQmax + 8 * K + 64 : nb + K + c.nQmax + 2 * (2 * K + 8) + 16;
  c.rcap = 2 * K + 16;
  return c;
}

struct PwWork {
  int *hord, *htmp, *ub, *uc, *ut;
  unsigned long long* sscr;  // warp sorts of long runs; ring lengths at output
  int *re_e, *re_s, *re_nd, *re_pre, *re_si;
  int *cAll, *cND, *cfill, *csorted;
  double* isxy;
  int *aB, *aC, *sB, *sC, *bNI, *cNI, *bSI;
  double *spx, *spy;
  int *spal, *spnb, *splab, *spnode;
  double* ixC;
  int *alC, *nbC, *labC, *cWin, *cWinSI, *nbCsi;
  Pool P, Q, R;
  int* runIds;
  int* rroot;
  int* counts;
  unsigned char *splitP, *splitQ, *crossP, *crossQ;
  int* roff;
  double* rxy;
};

__host__ __device__ __forceinline__ void pw_pool(Carver& cv, int cap, Pool& p, bool runs) {
  p.x = cv.take<double>(cap);
  p.y = cv.take<double>(cap);
  p.next = cv.take<int>(cap);
  p.prev = cv.take<int>(cap);
  p.nb = cv.take<int>(cap);
  p.label = cv.take<int>(cap);
  p.enex = cv.take<int>(cap);
  p.source = cv.take<unsigned char>(cap);
  p.isect = cv.take<unsigned char>(cap);
  p.src = nullptr;
  p.run = runs ? cv.take<int>(cap) : nullptr;
  p.rv0 = runs ? cv.take<int>(cap) : nullptr;
  p.rxy = nullptr;
  p.n = 0;
  p.cap = cap;
}

__host__ __device__ __forceinline__ PwWork pw_carve(Carver& cv, const PwCaps& c) {
  PwWork w;
  const int K = c.K;
  w.hord = cv.take<int>(K);
  w.htmp = cv.take<int>(K);
  w.sscr = cv.take<unsigned long long>(2 * K + 16);  // also one per ring (rcap)
  w.ub = cv.take<int>(K);
  w.uc = cv.take<int>(K);
  w.ut = cv.take<int>(K);
  w.re_e = cv.take<int>(K + 1);
  w.re_s = cv.take<int>(K + 1);
  w.re_nd = cv.take<int>(K + 1);
  w.re_pre = cv.take<int>(K + 1);
  w.re_si = cv.take<int>(K + 1);
  w.cAll = cv.take<int>(c.nc + 1);
  w.cND = cv.take<int>(c.nc + 1);
  w.cfill = cv.take<int>(c.nc + 1);
  w.csorted = cv.take<int>(K);
  w.isxy = cv.take<double>(2 * K);
  w.aB = cv.take<int>(K);
  w.aC = cv.take<int>(K);
  w.sB = cv.take<int>(K);
  w.sC = cv.take<int>(K);
  w.bNI = cv.take<int>(K);
  w.cNI = cv.take<int>(K);
  w.bSI = cv.take<int>(K);
  w.spx = cv.take<double>(c.sp);
  w.spy = cv.take<double>(c.sp);
  w.spal = cv.take<int>(c.sp);
  w.spnb = cv.take<int>(c.sp);
  w.splab = cv.take<int>(c.sp);
  w.spnode = cv.take<int>(c.sp);
  w.ixC = cv.take<double>(2 * c.nQmax);
  w.alC = cv.take<int>(c.nQmax);
  w.nbC = cv.take<int>(c.nQmax);
  w.labC = cv.take<int>(c.nQmax);
  w.cWin = cv.take<int>(c.nQmax);
  w.cWinSI = cv.take<int>(c.nQmax);
  w.nbCsi = cv.take<int>(c.nQmax);
  pw_pool(cv, c.capP, w.P, true);
  pw_pool(cv, c.capQ, w.Q, false);
  pw_pool(cv, c.capR, w.R, false);
  w.runIds = cv.take<int>(c.capP);
  w.rroot = cv.take<int>(c.rcap);
  w.counts = cv.take<int>(4);
  w.splitP = cv.take<unsigned char>(c.capP);
  w.crossP = cv.take<unsigned char>(c.capP);
  w.splitQ = cv.take<unsigned char>(c.capQ);
  w.crossQ = cv.take<unsigned char>(c.capQ);
  w.roff = cv.take<int>(c.rcap + 1);
  w.rxy = cv.take<double>(2 * (long long)c.capR);
  return w;
}

__host__ __device__ __forceinline__ size_t pw_arena_bytes(int nb, int nc, int K, int pass) {
  Carver cv{nullptr, 0};
  pw_carve(cv, pw_caps(nb, nc, K, pass));
  return (cv.off + 255) & ~(size_t)255;
}

// pointInPoly against the base side of a pair whose list has run nodes: the
// steps of the edges between nodes, plus those of the base edges inside run
// nodes, which come from the grid row holding ry (each edge counted in the
// first cell of its box in that row).  Called by all 32 lanes of a warp with
// the same arguments: the row's cells and the long edges are split over the
// lanes and the steps summed (the winding number is order-free).
struct PwPip {
  const double* b;
  int nb;
  PwGrid g;
  const int* gstart;
  const int* gent;
  const int* lng;
  int nlong;
  const float4* fbox;
  const int* runIds;
  int nruns;
  __device__ bool internal(const Pool& P, int u) const {
    int lo = 0, hi = nruns;  // runs with rv0 <= u
    while (lo < hi) {
      const int m = (lo + hi) >> 1;
      if (P.rv0[runIds[m]] <= u) lo = m + 1;
      else hi = m;
    }
    if (lo == 0) return false;
    const int v = runIds[lo - 1];
    return u + 1 <= P.rv0[v] + P.run[v];
  }
  __device__ int operator()(SerialArgs& a, int root, double rx, double ry) const {
    const Pool& P = a.P;
    const int lane = threadIdx.x & 31;
    // the edges between list nodes: every pool node is on the list
    int part = 0;
    for (int v = lane; v < P.n; v += 32) {
      const int nx = P.next[v];
      part += pip_step(last_x(P, v), last_y(P, v), P.x[nx], P.y[nx], rx, ry);
    }
    const int cy = pw_celly(g, __double2float_rd(ry));
    // the step first: most edges of the row do not cross the ray, and only
    // those that do need the cell and run-membership tests
    for (int cx = lane; cx < g.gx; cx += 32) {
      const int cell = cy * g.gx + cx;
      for (int k = gstart[cell]; k < gstart[cell + 1]; ++k) {
        const int u = gent[k];
        const int st = pip_step(b[2 * u], b[2 * u + 1], b[2 * u + 2], b[2 * u + 3], rx, ry);
        if (st && pw_cellx(g, fbox[u].x) == cx && internal(P, u)) part += st;
      }
    }
    for (int k = lane; k < nlong; k += 32) {
      const int u = lng[k];
      const int st = pip_step(b[2 * u], b[2 * u + 1], b[2 * u + 2], b[2 * u + 3], rx, ry);
      if (st && internal(P, u)) part += st;
    }
    return (__reduce_add_sync(kFullMask, part) % 2) != 0;
  }
};

// ---------------------------------------------------------------- warp helpers
// first i in [0, n) with pred(i), or -1; called by all 32 lanes
template <class Pred>
__device__ int warp_first(int n, Pred pred) {
  const int lane = threadIdx.x & 31;
  for (int i0 = 0; i0 < n; i0 += 32) {
    const int i = i0 + lane;
    const unsigned m = __ballot_sync(kFullMask, i < n && pred(i));
    if (m) return i0 + __ffs(m) - 1;
  }
  return -1;
}

// pointInPoly against a pool every node of which is on its one list (the
// pairwise back end never unlinks a list node): the winding steps of the
// edges v -> next[v], summed over the lanes
__device__ int warp_ppip(const Pool& p, double rx, double ry) {
  const int lane = threadIdx.x & 31;
  int part = 0;
  for (int v = lane; v < p.n; v += 32) {
    const int nx = p.next[v];
    part += pip_step(last_x(p, v), last_y(p, v), p.x[nx], p.y[nx], rx, ry);
  }
  return __reduce_add_sync(kFullMask, part);
}

// rcopy of a plain pool whose list is its nodes in index order: ring node
// base + i is list node i
__device__ int warp_rcopy_plain(SerialArgs& a, const Pool& p) {
  const int lane = threadIdx.x & 31;
  const int r = rnew(a);
  if (r < 0) return -1;
  Pool& R = a.R;
  const int n = p.n, base = R.n;
  if (n == 0) return 0;
  if (base + n > R.cap) {
    a.rfull = 1;
    return -1;
  }
  for (int i = lane; i < n; i += 32) {
    const int v = base + i;
    R.x[v] = p.x[i];
    R.y[v] = p.y[i];
    R.next[v] = i + 1 == n ? base : v + 1;
    R.prev[v] = i == 0 ? base + n - 1 : v - 1;
    R.nb[v] = -1;
    R.label[v] = L_NONE;
    R.enex[v] = EX_NEITHER;
    R.source[v] = 0;
    R.isect[v] = 0;
  }
  R.n = base + n;
  a.rroot[r] = base;
  __syncwarp();
  return 0;
}

// transition of the entry/exit walk (polyclip.h:337-709 step 4) at a node
// with label `lab`, on state x = (status is entry) | (first << 1)
__device__ __forceinline__ int walk_step(int lab, int x) {
  const int sb = x & 1, f = x >> 1;
  if (lab == L_CROSSING) return (sb ^ 1) | (f << 1);
  if (lab == L_DCROSS) return f ? sb : ((sb ^ 1) | 2);
  if (lab == L_DBOUNCE) return (sb ^ 1) | ((f ^ 1) << 1);
  return x;
}
// the transition as a table: 2 bits per state
__device__ __forceinline__ unsigned walk_table(int lab) {
  unsigned t = 0;
  for (int x = 0; x < 4; ++x) t |= (unsigned)walk_step(lab, x) << (2 * x);
  return t;
}
// g after f
__device__ __forceinline__ unsigned walk_compose(unsigned g, unsigned f) {
  unsigned h = 0;
  for (int x = 0; x < 4; ++x) h |= ((g >> (2 * ((f >> (2 * x)) & 3))) & 3) << (2 * x);
  return h;
}

// labelIntersections2 + createResult2 (polyclip.h:337-759) of one pair, run
// by all 32 lanes: the serial restatement (sbc_serial.cuh) with the searches,
// point-in-polygon sums, list copies and the entry/exit walk spread over the
// lanes.  On entry both lists are their pools in index order; a list node is
// never unlinked, so every pool node is on its list throughout.
__device__ int pw_label_trace(SerialArgs& a, const PwPip& pipP) {
  const int lane = threadIdx.x & 31;
  Pool& P = a.P;
  Pool& Q = a.Q;
  // (2) chains: rare (overlapping edges), so the serial pass runs only when
  // a chain start exists
  if (warp_first(P.n, [&](int v) {
        return P.isect[v] && (P.label[v] == L_LEFT_ON || P.label[v] == L_RIGHT_ON);
      }) >= 0) {
    int V = 0;
    do {
      if (P.isect[V] && (P.label[V] == L_LEFT_ON || P.label[V] == L_RIGHT_ON)) {
        int x = P.label[V] == L_LEFT_ON ? 0 : 1;
        int X = V, I = V;
        int guard = P.n + 1;
        do {
          P.label[I] = L_NONE;
          if (P.nb[I] < 0) return 2;
          Q.label[P.nb[I]] = L_NONE;
          I = P.next[I];
          if (--guard < 0) return 2;
        } while (P.label[I] == L_ON_ON);
        int y = P.label[I] == L_ON_LEFT ? 0 : 1;
        int chain = (x != y) ? L_DCROSS : L_DBOUNCE;
        P.label[X] = chain;
        P.label[I] = chain;
        if (P.nb[X] < 0 || P.nb[I] < 0) return 2;
        Q.label[P.nb[X]] = chain;
        Q.label[P.nb[I]] = chain;
      }
      V = P.next[V];
    } while (V != 0);
    __syncwarp();
  }
  auto pip_of = [&](int s, double rx, double ry) -> int {
    if (s == 0) return pipP(a, 0, rx, ry);
    return (warp_ppip(Q, rx, ry) % 2) != 0;
  };
  // (3.5) sides without crossings
  int noIsect[2] = {0, 0}, ident[2] = {0, 0};
  for (int s = 0; s < 2; ++s) {
    Pool& p = side(a, s);
    Pool& o = side(a, 1 - s);
    const int n = p.n;
    const bool cross = warp_first(n, [&](int v) {
                         if (!p.isect[v]) return false;
                         const int l = p.label[v];
                         // noCrossingVertex(UNION), foster/polygon.h:465-475
                         return l == L_CROSSING || l == L_DCROSS ||
                                (a.unite && (l == L_BOUNCING || l == L_DBOUNCE));
                       }) >= 0;
    if (cross) continue;
    noIsect[s] = 1;
    if (warp_first(n, [&](int v) { return p.label[v] != L_ON_ON; }) < 0) {
      ident[s] = 1;
      continue;
    }
    double px, py;
    const int f = warp_first(n, [&](int v) { return !p.isect[v]; });
    if (f >= 0) {
      px = p.x[f];
      py = p.y[f];
    } else {
      const int V = warp_first(n, [&](int v) {
        const int nbV = p.nb[v], nbN = p.nb[p.next[v]];
        return nbV < 0 || (nbN != o.prev[nbV] && nbN != o.next[nbV]);
      });
      if (V < 0 || p.nb[V] < 0) return 2;
      px = dmul(0.5, dadd(p.x[V], p.x[p.next[V]]));
      py = dmul(0.5, dadd(p.y[V], p.y[p.next[V]]));
    }
    if (pip_of(1 - s, px, py) ^ a.unite) {
      const int rc = s == 1 ? warp_rcopy_plain(a, p) : rcopy(a, p, 0);
      if (rc) return 3;
    }
  }
  if (ident[0] && ident[1]) {
    const int target = P.nb[0];
    if (warp_first(Q.n, [&](int v) { return v == target; }) >= 0 && rcopy(a, P, 0)) return 3;
  }
  __syncwarp();
  // (4) entry/exit walk from a non-intersection vertex of each side
  for (int s = 0; s < 2; ++s) {
    if (noIsect[s]) continue;
    Pool& p = side(a, s);
    Pool& o = side(a, 1 - s);
    unsigned char* split = s == 0 ? a.splitP : a.splitQ;
    unsigned char* cross = s == 0 ? a.crossP : a.crossQ;
    const int n0 = p.n;  // this side's list is still its pool in index order
    int V = warp_first(n0, [&](int v) { return !p.isect[v]; });
    int start = V;
    if (V < 0) {
      const int U = warp_first(n0, [&](int v) {
        const int nbV = p.nb[v], nbN = p.nb[p.next[v]];
        return nbV < 0 || (nbN != o.prev[nbV] && nbN != o.next[nbV]);
      });
      if (U < 0 || p.nb[U] < 0) return 2;
      const double mx = dmul(0.5, dadd(p.x[U], p.x[p.next[U]]));
      const double my = dmul(0.5, dadd(p.y[U], p.y[p.next[U]]));
      V = pnew(p, mx, my);
      if (V < 0) return 3;
      pinsert_after(p, V, U);
      start = U + 1 == n0 ? 0 : U + 1;  // the midpoint itself is no intersection
      __syncwarp();
    }
    int x0 = 1 | 2;  // entry, first
    if (pip_of(1 - s, p.x[V], p.y[V])) x0 ^= 1;
    // the walk over the list from V: its original nodes in cyclic index
    // order from `start`; transitions composed by a warp scan per chunk
    for (int j0 = 0; j0 < n0; j0 += 32) {
      const int j = j0 + lane;
      int I = start + j;
      if (I >= n0) I -= n0;
      const bool ok = j < n0;
      const int lab = ok && p.isect[I] ? p.label[I] : L_NONE;
      unsigned t = walk_table(lab);
      for (int d = 1; d < 32; d <<= 1) {
        const unsigned u = __shfl_up_sync(kFullMask, t, d);
        if (lane >= d) t = walk_compose(t, u);
      }
      const int after = (t >> (2 * x0)) & 3;
      int before = __shfl_up_sync(kFullMask, after, 1);
      if (lane == 0) before = x0;
      x0 = __shfl_sync(kFullMask, after, 31);
      if (!ok || !p.isect[I]) continue;
      const int status = (before & 1) ? EX_ENTRY : EX_EXIT;
      const int first = before >> 1;
      if (lab == L_CROSSING) p.enex[I] = status;
      if (lab == L_BOUNCING && ((status == EX_EXIT) ^ a.unite)) split[I] = 1;
      if (lab == L_DCROSS) {
        p.enex[I] = status;
        if (first ? ((status == EX_EXIT) ^ a.unite) : ((status == EX_ENTRY) ^ a.unite))
          p.label[I] = L_CROSSING;
      }
      if (lab == L_DBOUNCE) {
        p.enex[I] = status;
        if (first ? ((status == EX_EXIT) ^ a.unite) : ((status == EX_ENTRY) ^ a.unite))
          cross[I] = 1;
      }
    }
    __syncwarp();
  }
  // (5) split pairs: rare (bouncing vertices), serial when present
  const int nP0 = P.n;
  if (warp_first(nP0, [&](int v) { return a.splitP[v] != 0; }) >= 0) {
    for (int IP = 0; IP < nP0; ++IP) {
      if (!a.splitP[IP]) continue;
      int IQ = P.nb[IP];
      if (IQ < 0 || !a.splitQ[IQ]) continue;
      int VP = pnew(P, P.x[IP], P.y[IP]);
      int VQ = pnew(Q, Q.x[IQ], Q.y[IQ]);
      if (VP < 0 || VQ < 0) return 3;
      double sP = area3(last_x(P, P.prev[IP]), last_y(P, P.prev[IP]), P.x[IP], P.y[IP],
                        P.x[P.next[IP]], P.y[P.next[IP]]);
      double sQ = area3(Q.x[Q.prev[IQ]], Q.y[Q.prev[IQ]], Q.x[IQ], Q.y[IQ], Q.x[Q.next[IQ]],
                        Q.y[Q.next[IQ]]);
      if (dmul(sP, sQ) > 0) {
        P.nb[IP] = VQ; Q.nb[VQ] = IP; P.isect[IP] = 1; Q.isect[VQ] = 1;
        Q.nb[IQ] = VP; P.nb[VP] = IQ; Q.isect[IQ] = 1; P.isect[VP] = 1;
      } else {
        P.nb[VP] = VQ; Q.nb[VQ] = VP; P.isect[VP] = 1; Q.isect[VQ] = 1;
      }
      pinsert_after(P, VP, IP);
      pinsert_after(Q, VQ, IQ);
      if (!a.unite) {
        P.enex[IP] = EX_EXIT; P.enex[VP] = EX_ENTRY;
        Q.enex[IQ] = EX_EXIT; Q.enex[VQ] = EX_ENTRY;
      } else {
        P.enex[IP] = EX_ENTRY; P.enex[VP] = EX_EXIT;
        Q.enex[IQ] = EX_ENTRY; Q.enex[VQ] = EX_EXIT;
      }
      P.label[IP] = P.label[VP] = L_CROSSING;
      Q.label[IQ] = Q.label[VQ] = L_CROSSING;
    }
    __syncwarp();
  }
  // (6) each P node and its neighbour, independently
  for (int IP = lane; IP < P.n; IP += 32) {
    if (!a.crossP[IP]) continue;
    const int IQ = P.nb[IP];
    if (IQ >= 0 && a.crossQ[IQ]) {
      P.label[IP] = L_CROSSING;
      Q.label[IQ] = L_CROSSING;
    }
  }
  __syncwarp();
  // createResult2 (serial, on every lane).  Rings grow at their end only, so
  // a traced vertex is appended to the ring pool (coordinates alone: nothing
  // reads the other fields of ring nodes) and the ring is linked in pool
  // order once it is closed.  A run node's vertices are copied by all lanes.
  {
    Pool& R = a.R;
    auto emit = [&](const Pool& p, int v, bool forward) -> bool {
      if (!is_run(p, v)) {
        if (R.n >= R.cap) {
          a.rfull = 1;
          return false;
        }
        R.x[R.n] = p.x[v];
        R.y[R.n] = p.y[v];
        ++R.n;
        return true;
      }
      const int n = p.run[v] + 1, room = R.cap - R.n, m = n < room ? n : room;
      for (int t = lane; t < m; t += 32) {
        const int u = p.rv0[v] + (forward ? t : n - 1 - t);
        R.x[R.n + t] = p.rxy[2 * u];
        R.y[R.n + t] = p.rxy[2 * u + 1];
      }
      R.n += m;
      if (m < n) {
        a.rfull = 1;
        return false;
      }
      return true;
    };
    int It = 0;
    long long guard = 4LL * (P.n + Q.n) + 16;
    do {
      if (P.isect[It] && P.label[It] == L_CROSSING) {
        const int r = rnew(a);
        if (r < 0) return 3;
        const int rs = R.n;
        int sI = 0, I = It, sV = 0, V = I;
        P.isect[I] = 0;
        int enV = P.enex[V];
        do {
          int status = enV;
          tog(&status);
          const bool fwd = (status == EX_EXIT) ^ a.unite;
          Pool* pv = &side(a, sV);
          // a node's fields, its successor among them, are all read before
          // anything is stored (a byte store may alias them), so the next
          // node's reads need not wait for this node's stores
          int nx = fwd ? pv->next[V] : pv->prev[V];
          int en, nbV;
          do {
            V = nx;
            en = pv->enex[V];
            nbV = pv->nb[V];
            nx = fwd ? pv->next[V] : pv->prev[V];
            const bool run = is_run(*pv, V);
            const double x = pv->x[V], y = pv->y[V];
            pv->isect[V] = 0;
            if (!run) {
              if (R.n >= R.cap) {
                a.rfull = 1;
                return 2;
              }
              R.x[R.n] = x;
              R.y[R.n] = y;
              ++R.n;
            } else if (!emit(*pv, V, fwd)) {
              return 2;
            }
            if (--guard < 0) return 2;
          } while (!(en == status) && !(sV == sI && V == I));
          if (!(sV == sI && V == I)) {
            if (nbV < 0) return 2;
            sV = 1 - sV;
            V = nbV;
            side(a, sV).isect[V] = 0;
            enV = side(a, sV).enex[V];
          }
        } while (!(sV == sI && V == I));
        for (int v = rs + lane; v < R.n; v += 32) {
          R.next[v] = v + 1 == R.n ? rs : v + 1;
          R.prev[v] = v == rs ? R.n - 1 : v - 1;
        }
        a.rroot[r] = rs;
      }
      It = P.next[It];
    } while (It != 0);
    __syncwarp();
  }
  return 0;
}

struct PwPairArgs {
  int nov;
  const long long* coff;
  const double* cxy;
  const double* b;
  int nb;
  const PwPair* pp;
  const int* hstart;
  const PwHit* hits;
  const int* pass_of;  // null: every fast pair, pass 0
  const int* order;    // pairs by decreasing expected work (warp w takes order[w])
  unsigned char* arena;
  const long long* aoff;
  int* status;  // per pair: PS_* code
  int unite;    // union instead of intersection
  int* nrings;
  int* nverts;
  PwPip pip;
};

// global slot s of the base's merged list: its sparse index, or -1 for a
// plain vertex slot (then *vtx is the vertex)
// (hint: a run index near the answer; the search is narrowed to runs
// hint-1 .. hint+1 when they bracket s, and covers every run otherwise)
__device__ __forceinline__ int pw_slot(const PwWork& w, int nr, int s, int* vtx, int hint = -1) {
  auto start = [&](int k) { return w.re_e[k] + w.re_pre[k]; };
  int lo = 0, hi = nr;  // the count of runs starting at or before s lies in [lo, hi]
  if (hint >= 0) {
    const int a = max(0, min(nr, hint - 1)), bnd = min(nr, hint + 2);
    if ((a == 0 || start(a - 1) <= s) && (bnd == nr || start(bnd) > s)) {
      lo = a;
      hi = bnd;
    }
  }
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (w.re_e[m] + w.re_pre[m] <= s) lo = m + 1;
    else hi = m;
  }
  const int r = lo - 1;
  if (r >= 0) {
    const int st = w.re_e[r] + w.re_pre[r];
    if (s <= st + w.re_nd[r]) return w.re_si[r] + (s - st);
    *vtx = s - (w.re_pre[r] + w.re_nd[r]);
  } else {
    *vtx = s;
  }
  return -1;
}

// exclusive prefix sums of a[0..n) in place by the calling warp (all 32 lanes);
// returns the total.  Element i is read and written by lane i % 32.
__device__ int warp_excl_scan(int* a, int n) {
  const int lane = threadIdx.x & 31;
  int carry = 0;
  for (int i0 = 0; i0 < n; i0 += 32) {
    const int i = i0 + lane;
    const int x = i < n ? a[i] : 0;
    int s = x;
    for (int d = 1; d < 32; d <<= 1) {
      const int t = __shfl_up_sync(kFullMask, s, d);
      if (lane >= d) s += t;
    }
    if (i < n) a[i] = carry + s - x;
    carry += __shfl_sync(kFullMask, s, 31);
  }
  return carry;
}

// closes a lane-parallel step: orders its stores before the next step's
// loads and tells every lane whether any lane failed
__device__ __forceinline__ bool warp_fail(bool bad) {
  __syncwarp();
  return __any_sync(kFullMask, bad);
}

constexpr int kWarpSortMin = 32;  // runs longer than this are sorted by the whole warp

// sorts scr[0..n) -- distinct 64-bit values, key(m) for m < n -- ascending,
// by the whole warp: a bitonic network over the next power of two (padding
// sorts last)
template <class Key>
__device__ void warp_bitonic(int n, unsigned long long* scr, Key key) {
  const int lane = threadIdx.x & 31;
  const int np = npow2_dev(n);
  for (int m = lane; m < np; m += 32) scr[m] = m < n ? key(m) : ~0ull;
  __syncwarp();
  for (int k = 2; k <= np; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int m = lane; m < np; m += 32) {
        const int l = m ^ j;
        if (l > m) {
          const unsigned long long x = scr[m], y = scr[l];
          if ((x > y) == ((m & k) == 0)) {
            scr[m] = y;
            scr[l] = x;
          }
        }
      }
      __syncwarp();
    }
}

// stable order of sorted[s..t) (holding s..t) by alpha mod 1e9, by the whole
// warp: ties keep position order because the position is the key's low half.
// False (on every lane) when an alpha is negative.
__device__ bool warp_alpha_sort(int s, int t, const int* alpha, const int* order, int* sorted,
                                unsigned long long* scr) {
  const int lane = threadIdx.x & 31;
  bool neg = false;
  for (int x = s + lane; x < t; x += 32)
    if (alpha[order ? order[x] : x] < 0) neg = true;
  if (warp_fail(neg)) return false;
  warp_bitonic(t - s, scr, [&](int m) {
    const int x = s + m;
    return ((unsigned long long)(alpha[order ? order[x] : x] % 1000000000) << 32) | (unsigned)x;
  });
  for (int m = lane; m < t - s; m += 32) sorted[s + m] = (int)(unsigned)scr[m];
  __syncwarp();
  return true;
}

// A13 for base run r (copyIntersectionsParallel for one edge): its slots,
// then its records' positions in the merged list, walking the run's records
// in α order (they never run past the run's own records)
__device__ __forceinline__ void pw_fill_run(PwWork& w, const double* b, const int* ub,
                                            const int* ut, int K, int r) {
  const int e = w.re_e[r], s = w.re_s[r], pre = w.re_pre[r], si = w.re_si[r], nd = w.re_nd[r];
  w.spx[si] = b[2 * e];
  w.spy[si] = b[2 * e + 1];
  w.spal[si] = -100;
  w.spnb[si] = -100;
  w.splab[si] = 0;
  w.spnode[si] = -1;
  for (int q = 1; q <= nd; ++q) {
    w.spx[si + q] = w.spy[si + q] = 0.0;
    w.spal[si + q] = w.spnb[si + q] = 0;
    w.splab[si + q] = 0;
    w.spnode[si + q] = -1;
  }
  int bid = s;
  int lid = w.sB[bid];
  const int t = ut[lid];
  if (t == 2 || t == 4 || t == 6 || t == 8) {
    w.spal[si] = w.aB[lid];
    w.bNI[lid] = e + pre;
    w.bSI[lid] = si;
    if (bid < K - 1) lid = w.sB[++bid];
  }
  if ((ub[lid] >> 1) != e) return;
  for (int q = 0; q < nd; ++q) {
    w.spx[si + 1 + q] = w.isxy[2 * lid];
    w.spy[si + 1 + q] = w.isxy[2 * lid + 1];
    w.spal[si + 1 + q] = w.aB[lid];
    w.bNI[lid] = pre + e + 1 + q;
    w.bSI[lid] = si + 1 + q;
    if (bid < K - 1) lid = w.sB[++bid];
  }
}

// A13 for overlay edge e: its vertex slot, then its intersection slots
__device__ __forceinline__ void pw_fill_edge(PwWork& w, const double* c, const int* uc,
                                             const int* ut, int K, int e) {
  const int vs = e + w.cND[e];
  w.ixC[2 * vs] = c[2 * e];
  w.ixC[2 * vs + 1] = c[2 * e + 1];
  w.alC[vs] = -100;
  w.nbC[vs] = -100;
  const int s = w.cAll[e];
  if (w.cAll[e + 1] == s) return;
  auto entry = [&](int pos) { return w.csorted[w.sC[pos]]; };
  int bid = s;
  int lid = entry(bid);
  const int t = ut[lid];
  if (t == 3 || t == 4 || t == 5 || t == 7 || t == 8) {
    w.alC[vs] = w.aC[lid];
    w.cNI[lid] = vs;
    if (bid < K - 1) lid = entry(++bid);
  }
  if ((uc[lid] >> 1) != e) return;
  const int ns = w.cND[e], ne = w.cND[e + 1];
  for (int q = 0; q < ne - ns; ++q) {
    const int slot = ns + e + 1 + q;
    w.ixC[2 * slot] = w.isxy[2 * lid];
    w.ixC[2 * slot + 1] = w.isxy[2 * lid + 1];
    w.alC[slot] = w.aC[lid];
    w.cNI[lid] = slot;
    if (bid < K - 1) lid = entry(++bid);
  }
}

// Rows A9-A18 of one pair, run by all 32 lanes of a warp.  The serial steps
// (the linked-list build of the base, labelling, tracing, clean-up) run on
// every lane alike: the lanes read the same values, take the same branches
// and store the same values, so the warp never diverges there.  The steps
// that are independent per record, per run, per overlay edge or per slot
// split their loops over the lanes and end with __syncwarp; where the serial
// loop lets the last of several writes to one slot win, the lanes keep the
// largest writer index with atomicMax and that writer stores.  Every return
// is taken by all lanes together.
__device__ int pw_clip_pair(const PwPairArgs& A, int p, const PwCaps& cp, PwWork& w, int* nrings_out,
                            int* nverts_out) {
  const int lane = threadIdx.x & 31;
  const double* b = A.b;
  const int nb = A.nb;
  const long long o = A.coff[p];
  const int nc = (int)(A.coff[p + 1] - o);
  const double* c = A.cxy + 2 * o;
  const PwHit* H = A.hits + A.hstart[p];
  const int K = cp.K;
  // ---- A9: records arrive in the reference's order (base id, then first
  // emission), sorted for all pairs at once
  for (int i = lane; i < K; i += 32) {
    const PwHit& h = H[i];
    w.ub[i] = 2 * h.b;
    w.uc[i] = 2 * h.j;
    w.ut[i] = h.type;
  }
  for (int r = lane; r <= K; r += 32) w.re_nd[r] = 0;
  for (int i = lane; i <= nc; i += 32) w.cAll[i] = w.cND[i] = w.cfill[i] = 0;
  __syncwarp();
  const int* ub = w.ub;
  const int* uc = w.uc;
  const int* ut = w.ut;
  // ---- A10: base edges with records (runs), overlay counts
  int nr = 0, knd = 0;
  for (int i0 = 0; i0 < K; i0 += 32) {
    const int i = i0 + lane;
    const bool ok = i < K;
    const int e = ok ? ub[i] >> 1 : 0;
    const bool start = ok && (i == 0 || e != (ub[i - 1] >> 1));
    const bool nd = ok && nd_b(ut[i]);
    const unsigned sm = __ballot_sync(kFullMask, start);
    const int ri = nr + __popc(sm & ((2u << lane) - 1u)) - 1;  // the run holding record i
    if (start) {
      w.re_e[ri] = e;
      w.re_s[ri] = i;
    }
    if (nd) atomicAdd(&w.re_nd[ri], 1);
    if (ok) {
      const int ec = uc[i] >> 1;
      atomicAdd(&w.cAll[ec], 1);
      if (nd_c(ut[i])) atomicAdd(&w.cND[ec], 1);
    }
    nr += __popc(sm);
    knd += __popc(__ballot_sync(kFullMask, nd));
  }
  w.re_s[nr] = K;
  __syncwarp();
  for (int r = lane; r <= nr; r += 32) w.re_pre[r] = w.re_nd[r];  // re_nd[nr] is 0
  warp_excl_scan(w.re_pre, nr + 1);
  for (int r = lane; r <= nr; r += 32) w.re_si[r] = r + w.re_pre[r];
  warp_excl_scan(w.cAll, nc + 1);
  warp_excl_scan(w.cND, nc + 1);
  __syncwarp();
  // records of each overlay edge, in record order
  for (int i = lane; i < K; i += 32) {
    const int ec = uc[i] >> 1;
    w.csorted[w.cAll[ec] + atomicAdd(&w.cfill[ec], 1)] = i;
  }
  __syncwarp();
  for (int e0 = 0; e0 < nc; e0 += 32) {
    const int e = e0 + lane;
    const int s = e < nc ? w.cAll[e] : 0, t = e < nc ? w.cAll[e + 1] : 0;
    if (t - s > 1 && t - s <= kWarpSortMin) {
      int* v = w.csorted + s;
      for (int i = 1; i < t - s; ++i) {
        const int x = v[i];
        int j = i;
        while (j > 0 && v[j - 1] > x) {
          v[j] = v[j - 1];
          --j;
        }
        v[j] = x;
      }
    }
    for (unsigned m = __ballot_sync(kFullMask, t - s > kWarpSortMin); m; m &= m - 1) {
      const int ee = e0 + __ffs(m) - 1;
      const int s2 = w.cAll[ee], t2 = w.cAll[ee + 1];
      warp_bitonic(t2 - s2, w.sscr, [&](int k) { return (unsigned long long)w.csorted[s2 + k]; });
      for (int k = lane; k < t2 - s2; k += 32) w.csorted[s2 + k] = (int)w.sscr[k];
      __syncwarp();
    }
  }
  const int nB = nb + knd, nQ = nc + w.cND[nc];
  // ---- A11 records
  for (int i = lane; i < K; i += 32) {
    const int bi = ub[i] >> 1, ci = uc[i] >> 1;
    const int bi2 = bi + 1 == nb ? 0 : bi + 1, ci2 = ci + 1 == nc ? 0 : ci + 1;
    const double p1x = b[2 * bi], p1y = b[2 * bi + 1], p2x = b[2 * bi2], p2y = b[2 * bi2 + 1];
    const double q1x = c[2 * ci], q1y = c[2 * ci + 1];
    const double al = H[i].al, bt = H[i].bt;  // lineSegmentIntersection of the candidate test
    const int ty = ut[i];
    double x = 0.0, y = 0.0;
    if (ty == 1) {
      const double oma = dsub(1.0, al);
      x = dadd(dmul(oma, p1x), dmul(al, p2x));
      y = dadd(dmul(oma, p1y), dmul(al, p2y));
    } else if (ty == 3 || ty == 4 || ty == 5 || ty == 7 || ty == 8) {
      x = q1x;
      y = q1y;
    } else if (ty == 2 || ty == 6) {
      x = p1x;
      y = p1y;
    }
    w.isxy[2 * i] = x;
    w.isxy[2 * i + 1] = y;
    w.aB[i] = ty ? alpha_to_int(al) : 0;
    w.aC[i] = ty ? alpha_to_int(bt) : 0;
    w.sB[i] = w.sC[i] = i;
  }
  __syncwarp();
  // ---- A12 per-edge alpha order (stable by alpha mod 1e9), one run or one
  // overlay edge per lane
  // (stable insertion for short runs on one lane; a long run -- an overlay
  // edge across a jagged base can hold hundreds of crossings -- is sorted by
  // the whole warp)
  // (the run, at most kWarpSortMin long, holds positions s..t-1; its keys
  // are copied to the lane's own array first)
  auto isort = [&](int s, int t, const int* alpha, const int* order, int* sorted) -> bool {
    int key[kWarpSortMin], val[kWarpSortMin];
    const int m = t - s;
    for (int i = 0; i < m; ++i) {
      const int a = alpha[order ? order[s + i] : s + i];
      if (a < 0) return false;
      key[i] = a % 1000000000;
      val[i] = s + i;
    }
    for (int i = 1; i < m; ++i) {
      const int kp = key[i], pv = val[i];
      int j = i;
      while (j > 0 && key[j - 1] > kp) {
        key[j] = key[j - 1];
        val[j] = val[j - 1];
        --j;
      }
      key[j] = kp;
      val[j] = pv;
    }
    for (int i = 0; i < m; ++i) sorted[s + i] = val[i];
    return true;
  };
  bool bad = false;
  for (int r0 = 0; r0 < nr; r0 += 32) {
    const int r = r0 + lane;
    bool lng = false;
    if (r < nr && w.re_nd[r] > 1) {
      if (w.re_s[r + 1] - w.re_s[r] > kWarpSortMin) lng = true;
      else if (!isort(w.re_s[r], w.re_s[r + 1], w.aB, nullptr, w.sB)) bad = true;
    }
    for (unsigned m = __ballot_sync(kFullMask, lng); m; m &= m - 1) {
      const int rr = r0 + __ffs(m) - 1;
      if (!warp_alpha_sort(w.re_s[rr], w.re_s[rr + 1], w.aB, nullptr, w.sB, w.sscr)) bad = true;
    }
  }
  for (int e0 = 0; e0 < nc; e0 += 32) {
    const int e = e0 + lane;
    bool lng = false;
    if (e < nc && w.cND[e + 1] - w.cND[e] > 1) {
      if (w.cAll[e + 1] - w.cAll[e] > kWarpSortMin) lng = true;
      else if (!isort(w.cAll[e], w.cAll[e + 1], w.aC, w.csorted, w.sC)) bad = true;
    }
    for (unsigned m = __ballot_sync(kFullMask, lng); m; m &= m - 1) {
      const int ee = e0 + __ffs(m) - 1;
      if (!warp_alpha_sort(w.cAll[ee], w.cAll[ee + 1], w.aC, w.csorted, w.sC, w.sscr)) bad = true;
    }
  }
  if (warp_fail(bad)) return PS_FALLBACK;
  // ---- A13 merged arrays: the base's where it has records, the overlay's in
  // full.  A run (overlay edge) writes only its own slots and the neighbour
  // indices of its own records, so runs (edges) go one per lane.
  for (int i = lane; i < nQ; i += 32) {
    w.ixC[2 * i] = w.ixC[2 * i + 1] = 0.0;
    w.alC[i] = w.nbC[i] = 0;
    w.nbCsi[i] = -1;
    w.cWin[i] = -1;
  }
  for (int i = lane; i < K; i += 32) {
    w.bNI[i] = w.cNI[i] = 0;
    w.bSI[i] = -1;  // the sparse index of bNI[i] once a slot is written
  }
  __syncwarp();
  // base runs (copyIntersectionsParallel per edge), in chunks of 32 runs
  for (int r0 = 0; r0 < nr; r0 += 32) {
    const int r = r0 + lane;
    if (r < nr) pw_fill_run(w, b, ub, ut, K, r);
    __syncwarp();
  }
  // overlay edges: the vertex slot, then the edge's intersection slots
  for (int e0 = 0; e0 < nc; e0 += 32) {
    const int e = e0 + lane;
    if (e < nc) pw_fill_edge(w, c, uc, ut, K, e);
    __syncwarp();
  }
  // neighbours: the last record written to a slot wins (spnode and cWin hold
  // the winning record until the winners have stored)
  int si0;  // sparse index of slot 0, where records never written point
  {
    int vtx;
    si0 = pw_slot(w, nr, 0, &vtx);
  }
  for (int i = lane; i < K; i += 32) {
    const int si = w.bSI[i] < 0 ? si0 : w.bSI[i];
    if (si < 0) {
      bad = true;  // a plain slot would change
      continue;
    }
    atomicMax(&w.spnode[si], i);
    atomicMax(&w.cWin[w.cNI[i]], i);
  }
  if (warp_fail(bad)) return PS_FALLBACK;
  for (int i = lane; i < K; i += 32) {
    const int si = w.bSI[i] < 0 ? si0 : w.bSI[i];
    const int cq = w.cNI[i];
    if (w.spnode[si] == i) w.spnb[si] = cq + 1;
    if (w.cWin[cq] == i) {
      w.nbC[cq] = w.bNI[i] + 1;
      w.nbCsi[cq] = si;
    }
  }
  __syncwarp();
  const int nsp = w.re_si[nr];
  for (int s = lane; s < nsp; s += 32) w.spnode[s] = -1;
  for (int q = lane; q < nQ; q += 32) w.cWin[q] = -1;
  __syncwarp();
  // slot contents of the base's merged list
  auto info = [&](int s, int hint, double* x, double* y, int* al, int* nbv) {
    int vtx = 0;
    const int si = pw_slot(w, nr, s, &vtx, hint);
    if (si >= 0) {
      *x = w.spx[si];
      *y = w.spy[si];
      *al = w.spal[si];
      *nbv = w.spnb[si];
    } else {
      *x = b[2 * vtx];
      *y = b[2 * vtx + 1];
      *al = -100;
      *nbv = -100;
    }
  };
  // ---- A14 initial labels, one sparse slot per lane (spnode holds each
  // slot's run meanwhile); the overlay slot takes the label of the last base
  // slot naming it.  Loops over lanes run in chunks closed by __syncwarp, so
  // that lanes that branch apart join again every chunk.
  for (int r0 = 0; r0 < nr; r0 += 32) {
    const int r = r0 + lane;
    if (r < nr) {
      const int si0 = w.re_si[r], nd = w.re_nd[r];
      for (int q = 0; q <= nd; ++q) w.spnode[si0 + q] = r;
    }
    __syncwarp();
  }
  for (int s0 = 0; s0 < nsp; s0 += 32) {
    const int si = s0 + lane;
    if (si < nsp && !bad && w.spal[si] != -100) {
      const int r = w.spnode[si];
      const int e = w.re_e[r], nd = w.re_nd[r], q = si - w.re_si[r];
      const int i = e + w.re_pre[r] + q;
      const double cx = w.spx[si], cy = w.spy[si];
      // the slots before and after: the next sparse ones inside a run or
      // across adjacent runs, else plain base vertices (wrapping at the ends)
      double pmx, pmy, ppx, ppy;
      int alm, nbm, alp, nbp;
      auto sparse = [&](int s2, double* x, double* y, int* al, int* nbv) {
        *x = w.spx[s2];
        *y = w.spy[s2];
        *al = w.spal[s2];
        *nbv = w.spnb[s2];
      };
      auto plainv = [&](int vtx, double* x, double* y, int* al, int* nbv) {
        *x = b[2 * vtx];
        *y = b[2 * vtx + 1];
        *al = -100;
        *nbv = -100;
      };
      if (q > 0 || (e > 0 && r > 0 && w.re_e[r - 1] == e - 1)) sparse(si - 1, &pmx, &pmy, &alm, &nbm);
      else if (e > 0) plainv(e - 1, &pmx, &pmy, &alm, &nbm);
      else if (w.re_e[nr - 1] == nb - 1) sparse(nsp - 1, &pmx, &pmy, &alm, &nbm);
      else plainv(nb - 1, &pmx, &pmy, &alm, &nbm);
      if (q < nd || (e + 1 < nb && r + 1 < nr && w.re_e[r + 1] == e + 1))
        sparse(si + 1, &ppx, &ppy, &alp, &nbp);
      else if (e + 1 < nb) plainv(e + 1, &ppx, &ppy, &alp, &nbp);
      else if (w.re_e[0] == 0) sparse(0, &ppx, &ppy, &alp, &nbp);
      else plainv(0, &ppx, &ppy, &alp, &nbp);
      const int pMN = alm != -100 ? nbm - 1 : -100;
      const int pPN = alp != -100 ? nbp - 1 : -100;
      const int nId = w.spnb[si] - 1;
      // the overlay slots before and after nId: left (0), right (1), or the
      // base neighbours' own slots (2, 3)
      auto side_of = [&](int qq) -> int {
        if (pMN != -100 && pMN == qq) return 2;
        if (pPN != -100 && pPN == qq) return 3;
        const double qx = w.ixC[2 * qq], qy = w.ixC[2 * qq + 1];
        const double s1 = area3(qx, qy, pmx, pmy, cx, cy);
        const double s2 = area3(qx, qy, cx, cy, ppx, ppy);
        const double s3 = area3(pmx, pmy, cx, cy, ppx, ppy);
        if (s3 > 0) return (s1 > 0 && s2 > 0) ? 0 : 1;
        return (s1 < 0 && s2 < 0) ? 1 : 0;
      };
      int qq0 = nId - 1, qq1 = nId + 1;
      if (qq0 == nQ) qq0 = 0;
      else if (qq0 == -1) qq0 = nQ - 1;
      if (qq1 == nQ) qq1 = 0;
      else if (qq1 == -1) qq1 = nQ - 1;
      if (qq0 < 0 || qq0 >= nQ || qq1 < 0 || qq1 >= nQ) {
        bad = true;
      } else {
        const int qm = side_of(qq0), qp = side_of(qq1);
        int lab;
        if ((qm == 0 && qp == 1) || (qm == 1 && qp == 0)) lab = 1;
        else if ((qm == 0 && qp == 0) || (qm == 1 && qp == 1)) lab = 2;
        else if ((qp == 3 && qm == 1) || (qm == 3 && qp == 1)) lab = 3;
        else if ((qp == 3 && qm == 0) || (qm == 3 && qp == 0)) lab = 4;
        else if ((qp == 3 && qm == 2) || (qm == 3 && qp == 2)) lab = 5;
        else if ((qm == 2 && qp == 1) || (qp == 2 && qm == 1)) lab = 6;
        else if ((qm == 2 && qp == 0) || (qp == 2 && qm == 0)) lab = 7;
        else lab = -102;
        w.splab[si] = lab;
        if (nId < 0 || nId >= nQ) bad = true;
        else atomicMax(&w.cWin[nId], i);  // slots come in increasing order: the last one wins
      }
    }
    __syncwarp();
  }
  if (warp_fail(bad)) return PS_FALLBACK;
  for (int s0 = 0; s0 < nsp; s0 += 32) {
    const int si = s0 + lane;
    if (si < nsp && w.spal[si] != -100) {
      const int r = w.spnode[si];
      const int nId = w.spnb[si] - 1;
      if (w.cWin[nId] == w.re_e[r] + w.re_pre[r] + (si - w.re_si[r])) w.cWinSI[nId] = si;
    }
    __syncwarp();
  }
  for (int s = lane; s < nsp; s += 32) w.spnode[s] = -1;
  for (int q = lane; q < nQ; q += 32) w.labC[q] = w.cWin[q] >= 0 ? w.splab[w.cWinSI[q]] : 0;
  __syncwarp();
  // ---- A15 linked lists (copyToLinkedList, src/clip.cpp:606-695): the base's
  // with run nodes for its stretches of plain vertices.  Its walk visits, per
  // run r, the stretch of plain vertices since the previous run (one run
  // node), the vertex of edge e_r and its intersections, and a last stretch
  // to the end -- unless a coordinate stops the walk early: a slot of edge
  // e_r repeating vertex e_r + 1, or a NaN.  Those lists take the serial walk.
  Pool& P = w.P;
  Pool& Q = w.Q;
  P.n = Q.n = w.R.n = 0;
  P.rxy = b;
  int nruns = 0, lastPlain = -1;
  bool oddP = false;
  for (int r = lane; r < nr && !oddP; r += 32) {
    const int e = w.re_e[r], si = w.re_si[r], nd = w.re_nd[r];
    if (!(w.spx[si] == b[2 * e] && w.spy[si] == b[2 * e + 1])) oddP = true;
    if (nd == 0) continue;
    const int nx = e + 1 == nb ? 0 : e + 1;
    const double vx = b[2 * nx], vy = b[2 * nx + 1];
    if (!(vx == vx && vy == vy)) oddP = true;
    for (int q = 1; q <= nd; ++q)
      if (w.spx[si + q] == vx && w.spy[si + q] == vy) oddP = true;
  }
  if (!__any_sync(kFullMask, oddP)) {
    // nodes per run (stretch, vertex, intersections), offsets by a scan in re_s
    for (int r = lane; r < nr; r += 32) {
      const int e = w.re_e[r], pe = r == 0 ? 0 : w.re_e[r - 1] + 1;
      w.re_s[r] = (e > pe ? 1 : 0) + 1 + w.re_nd[r];
    }
    if (lane == (nr & 31)) w.re_s[nr] = 0;
    __syncwarp();
    const int tot0 = warp_excl_scan(w.re_s, nr + 1);
    const int pe_last = nr == 0 ? 0 : w.re_e[nr - 1] + 1;
    const int tail = pe_last < nb ? 1 : 0;
    if (tot0 + tail > P.cap) return PS_CAP;
    auto put = [&](int v, double x, double y, int src1, int lab, int isect) {
      P.x[v] = x;
      P.y[v] = y;
      P.nb[v] = -1;
      P.label[v] = lab;
      P.enex[v] = EX_NEITHER;
      P.source[v] = (unsigned char)src1;
      P.isect[v] = (unsigned char)isect;
      P.run[v] = 0;
      P.rv0[v] = 0;
    };
    __syncwarp();
    for (int r0 = 0; r0 < nr; r0 += 32) {
      const int r = r0 + lane;
      if (r < nr) {
        const int e = w.re_e[r], pe = r == 0 ? 0 : w.re_e[r - 1] + 1, si = w.re_si[r];
        int v = w.re_s[r];
        if (e > pe) {  // the stretch pe .. e-1; it is stretch number v - r - re_pre[r]
          put(v, b[2 * pe], b[2 * pe + 1], 1, L_NONE, 0);
          P.run[v] = e - pe - 1;
          P.rv0[v] = pe;
          w.runIds[v - r - w.re_pre[r]] = v;
          ++v;
        }
        put(v, b[2 * e], b[2 * e + 1], 1, w.splab[si], w.spal[si] != -100);
        w.spnode[si] = v++;
        for (int q = 1; q <= w.re_nd[r]; ++q) {
          put(v, w.spx[si + q], w.spy[si + q], 0, w.splab[si + q], 1);
          w.spnode[si + q] = v++;
        }
      }
      __syncwarp();
    }
    if (tail && lane == 0) {
      put(tot0, b[2 * pe_last], b[2 * pe_last + 1], 1, L_NONE, 0);
      P.run[tot0] = nb - pe_last - 1;
      P.rv0[tot0] = pe_last;
      w.runIds[tot0 - nr - knd] = tot0;
    }
    nruns = tot0 - nr - knd + tail;
    P.n = tot0 + tail;
  } else {
  auto plain = [&](int v0, int len) -> int {
    if (lastPlain >= 0 && lastPlain == P.n - 1 && P.rv0[lastPlain] + P.run[lastPlain] == v0 - 1) {
      P.run[lastPlain] += len;
      return 0;
    }
    const int v = pnew(P, b[2 * v0], b[2 * v0 + 1]);
    if (v < 0) return PS_CAP;
    P.source[v] = 1;
    P.rv0[v] = v0;
    P.run[v] = len - 1;
    w.runIds[nruns++] = v;
    lastPlain = v;
    return 0;
  };
  {
    int vn = 0, i = 0, r = 0;
    for (int ii = 0; ii <= nb;) {
      while (r < nr && w.re_e[r] < ii) ++r;
      if (ii < nb) {
        const int slot = ii + w.re_pre[r];
        const bool hasRec = r < nr && w.re_e[r] == ii;
        if (!hasRec && i == slot) {
          const int stop = r < nr ? w.re_e[r] : nb;
          const int st = plain(ii, stop - ii);
          if (st) return st;
          vn += stop - ii;
          i += stop - ii;
          ii = stop;
          continue;
        }
      }
      const int sv = ii < nb ? ii : 0;
      const double vx = b[2 * sv], vy = b[2 * sv + 1];
      for (;;) {
        const int s = i % nB;
        double sx, sy;
        int sal, snb;
        info(s, r, &sx, &sy, &sal, &snb);
        if (sx == vx && sy == vy) break;
        if (i >= nB) return PS_UNDEF;
        int vtx;
        const int si = pw_slot(w, nr, s, &vtx, r);
        if (si < 0) return PS_FALLBACK;
        const int v = pnew(P, sx, sy);
        if (v < 0) return PS_CAP;
        P.label[v] = w.splab[si];
        P.isect[v] = 1;
        w.spnode[si] = v;
        lastPlain = -1;
        ++vn;
        ++i;
      }
      if (ii < nb) {
        if (vn != i) return PS_UNDEF;
        if (i != ii + w.re_pre[r]) return PS_FALLBACK;  // stopped at another slot
        int vtx;
        const int si = pw_slot(w, nr, i, &vtx, r);
        if (si >= 0) {
          const int v = pnew(P, vx, vy);
          if (v < 0) return PS_CAP;
          P.source[v] = 1;
          P.label[v] = w.splab[si];
          if (w.spal[si] != -100) P.isect[v] = 1;
          w.spnode[si] = v;
          lastPlain = -1;
        } else {
          const int st = plain(ii, 1);
          if (st) return st;
        }
        ++vn;
      }
      ++i;
      ++ii;
    }
    if (vn != nB) return PS_UNDEF;
  }
  }
  __syncwarp();
  for (int v = lane; v < P.n; v += 32) {
    P.next[v] = v + 1 == P.n ? 0 : v + 1;
    P.prev[v] = v == 0 ? P.n - 1 : v - 1;
  }
  // The overlay's list is its merged array in order (node i is slot i) unless
  // a slot's coordinates stop the reference's walk early: an overlay vertex
  // whose slot does not hold its own coordinates (NaN), or an intersection
  // slot of edge e that repeats vertex e + 1.  The walk then takes the serial
  // path below, which follows the reference in every case.
  bool odd = false;
  for (int e = lane; e < nc && !odd; e += 32) {
    const int vs = e + w.cND[e], ne = w.cND[e + 1] - w.cND[e];
    const int nx = e + 1 == nc ? 0 : e + 1;
    const double vx = c[2 * nx], vy = c[2 * nx + 1];
    if (!(w.ixC[2 * vs] == c[2 * e] && w.ixC[2 * vs + 1] == c[2 * e + 1])) odd = true;
    for (int q = 1; q <= ne; ++q)
      if (w.ixC[2 * (vs + q)] == vx && w.ixC[2 * (vs + q) + 1] == vy) odd = true;
  }
  if (!__any_sync(kFullMask, odd)) {
    // node v = slot v; the first failing slot decides the status
    int first = INT_MAX;  // 4 * slot + 1 (undefined) or + 2 (pair pipeline)
    for (int e0 = 0; e0 < nc; e0 += 32) {
      const int e = e0 + lane;
      const int vs = e < nc ? e + w.cND[e] : 0, ne = e < nc ? w.cND[e + 1] - w.cND[e] : -1;
      for (int q = 0; q <= ne; ++q) {
        const int v = vs + q;
        Q.x[v] = w.ixC[2 * v];
        Q.y[v] = w.ixC[2 * v + 1];
        Q.nb[v] = -1;
        Q.label[v] = w.labC[v];
        Q.enex[v] = EX_NEITHER;
        Q.source[v] = q == 0;
        Q.isect[v] = 0;
        Q.next[v] = v + 1 == nQ ? 0 : v + 1;
        Q.prev[v] = v == 0 ? nQ - 1 : v - 1;
        if (q == 0 && w.nbC[v] == -100) continue;  // a plain overlay vertex
        const int t = w.nbC[v] - 1;
        if (t < 0 || t >= nB) {
          first = min(first, 4 * v + 1);
          continue;
        }
        const int si = w.nbCsi[v];
        if (si < 0 || w.spnode[si] < 0) {
          first = min(first, 4 * v + 2);
          continue;
        }
        Q.isect[v] = 1;
        Q.nb[v] = w.spnode[si];
        atomicMax(&P.nb[w.spnode[si]], v);  // the last overlay node naming it wins
      }
      __syncwarp();
    }
    first = __reduce_min_sync(kFullMask, first);
    __syncwarp();
    if (first != INT_MAX) return (first & 3) == 1 ? PS_UNDEF : PS_FALLBACK;
    Q.n = nQ;
  } else {
    int i = 0;
    for (int ii = 0; ii <= nc; ++ii) {
      const int sv = ii < nc ? ii : 0;
      const double vx = c[2 * sv], vy = c[2 * sv + 1];
      while (w.ixC[(2 * i) % (2 * nQ)] != vx || w.ixC[(2 * i + 1) % (2 * nQ)] != vy) {
        if (i >= nQ) return PS_UNDEF;
        const int v = pnew(Q, w.ixC[2 * i], w.ixC[2 * i + 1]);
        if (v < 0) return PS_CAP;
        Q.label[v] = w.labC[i];
        Q.isect[v] = 1;
        const int t = w.nbC[i] - 1;
        if (t < 0 || t >= nB) return PS_UNDEF;
        const int si = w.nbCsi[i];
        if (si < 0 || w.spnode[si] < 0) return PS_FALLBACK;
        Q.nb[v] = w.spnode[si];
        P.nb[w.spnode[si]] = v;
        i++;
      }
      if (ii < nc) {
        const int v = pnew(Q, vx, vy);
        if (v != i) return PS_UNDEF;
        Q.source[v] = 1;
        Q.label[v] = w.labC[i];
        if (w.nbC[i] != -100) {
          const int t = w.nbC[i] - 1;
          if (t < 0 || t >= nB) return PS_UNDEF;
          const int si = w.nbCsi[i];
          if (si < 0 || w.spnode[si] < 0) return PS_FALLBACK;
          Q.isect[v] = 1;
          Q.nb[v] = w.spnode[si];
          P.nb[w.spnode[si]] = v;
        }
      }
      i++;
    }
    if (Q.n != nQ) return PS_UNDEF;
    for (int v = 0; v < nQ; ++v) {
      Q.next[v] = (v + 1) % nQ;
      Q.prev[v] = (v + nQ - 1) % nQ;
    }
  }
  for (int i = lane; i < cp.capP; i += 32) w.splitP[i] = w.crossP[i] = 0;
  for (int i = lane; i < cp.capQ; i += 32) w.splitQ[i] = w.crossQ[i] = 0;
  __syncwarp();
  // ---- A16-A18 (serial, on every lane; pointInPoly against the base splits
  // its grid row over the lanes)
  SerialArgs a;
  a.P = P;
  a.Q = Q;
  a.R = w.R;
  a.rroot = w.rroot;
  a.rcap = cp.rcap;
  a.nrings = &w.counts[0];
  a.status = &w.counts[1];
  a.splitP = w.splitP;
  a.splitQ = w.splitQ;
  a.crossP = w.crossP;
  a.crossQ = w.crossQ;
  a.bSize = nb;
  a.cSize = nc;
  a.cStart = 0;
  a.nB = nB;
  a.nQ = nQ;
  a.bP = b;
  a.cP = c;
  a.ixB = nullptr;
  a.ixC = w.ixC;
  a.alB = nullptr;
  a.nbC = w.nbC;
  a.labB = nullptr;
  a.labC = w.labC;
  a.unite = A.unite;
  *a.nrings = 0;
  PwPip pip = A.pip;
  pip.runIds = w.runIds;
  pip.nruns = nruns;
  int st = pw_label_trace(a, pip);
  if (a.rfull) return PS_CAP;
  if (st) return st == 2 ? PS_UNDEF : PS_CAP;
  // cleanUpResult2 (ser_cleanup).  Rings are built one after another and
  // grow at their end, so ring r is the pool nodes rroot[r] .. rroot[r+1]-1
  // in order.  A vertex with |area3| < eps marks its ring; with no ring
  // marked nothing is removed and the output is the pool itself.
  const int nring = *a.nrings;
  for (int r = lane; r < nring; r += 32) w.sscr[r] = 0;
  __syncwarp();
  {
    const Pool& R = a.R;
    for (int v = lane; v < R.n; v += 32) {
      const double ar = fabs(area3(R.x[R.prev[v]], R.y[R.prev[v]], R.x[v], R.y[v],
                                   R.x[R.next[v]], R.y[R.next[v]]));
      if (!(ar < kEps)) continue;
      int lo = 0, hi = nring;  // rings with rroot <= v
      while (lo < hi) {
        const int m = (lo + hi) >> 1;
        if (a.rroot[m] <= v) lo = m + 1;
        else hi = m;
      }
      if (lo > 0) w.sscr[lo - 1] = 1;
    }
  }
  __syncwarp();
  if (warp_first(nring, [&](int r) {
        return w.sscr[r] != 0 || (r > 0 && a.rroot[r] <= a.rroot[r - 1]);
      }) < 0 &&
      (nring == 0 || a.rroot[0] == 0)) {
    const Pool& R = a.R;
    for (int v = lane; v < R.n; v += 32) {
      w.rxy[2 * v] = R.x[v];
      w.rxy[2 * v + 1] = R.y[v];
    }
    for (int r = lane; r < nring; r += 32) w.roff[r] = a.rroot[r];
    if (lane == 0) w.roff[nring] = R.n;
    __syncwarp();
    *nrings_out = nring;
    *nverts_out = R.n;
    return PS_OK;
  }
  // some ring loses vertices: ring by ring, one ring per lane (rings share no
  // nodes), then each ring's length: ring r's vertex count in the low half of
  // sscr[r], 1 << 32 in the high half when it is not empty
  {
    Pool& R = a.R;
    for (int r = lane; r < nring; r += 32) {
      auto A3 = [&](int v) {
        return fabs(area3(R.x[R.prev[v]], R.y[R.prev[v]], R.x[v], R.y[v], R.x[R.next[v]],
                          R.y[R.next[v]]));
      };
      int root = a.rroot[r];
      auto remove = [&](int V) {
        if (root == V) {
          root = R.next[V];
          if (R.next[root] == root) root = -1;
        }
        R.next[R.prev[V]] = R.next[V];
        R.prev[R.next[V]] = R.prev[V];
      };
      while (root >= 0 && A3(root) < kEps) remove(root);
      unsigned long long len = 0;
      if (root >= 0) {
        const int start = root;
        int V = start;
        do {
          const int nx = R.next[V];
          if (A3(V) < kEps) remove(V);
          V = nx;
        } while (V != start);
      }
      if (root >= 0) {
        int V = root;
        do {
          ++len;
          V = R.next[V];
        } while (V != root);
        len |= 1ull << 32;
      }
      a.rroot[r] = root;
      w.sscr[r] = len;
    }
  }
  __syncwarp();
  // output offsets (one scan of both halves), then the rings' coordinates
  {
    unsigned long long carry = 0;
    for (int r0 = 0; r0 < nring; r0 += 32) {
      const int r = r0 + lane;
      const unsigned long long x = r < nring ? w.sscr[r] : 0;
      unsigned long long sc = x;
      for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long t = __shfl_up_sync(kFullMask, sc, d);
        if (lane >= d) sc += t;
      }
      if (r < nring) w.sscr[r] = carry + sc - x;
      carry += __shfl_sync(kFullMask, sc, 31);
    }
    __syncwarp();
    w.roff[0] = 0;
    for (int r = lane; r < nring; r += 32) {
      const int root = a.rroot[r];
      if (root < 0) continue;
      const unsigned long long off = w.sscr[r];
      int nv = (int)(unsigned)off;
      const int k = (int)(off >> 32);
      int v = root;
      do {
        w.rxy[2 * nv] = a.R.x[v];
        w.rxy[2 * nv + 1] = a.R.y[v];
        ++nv;
        v = a.R.next[v];
      } while (v != root);
      w.roff[k + 1] = nv;
    }
    __syncwarp();
    *nrings_out = (int)(carry >> 32);
    *nverts_out = (int)(unsigned)carry;
  }
  return PS_OK;
}

__global__ void k_pw_sizes(int nov, const long long* __restrict__ coff, int nb,
                           const PwPair* __restrict__ pp, const int* __restrict__ pairK,
                           const int* __restrict__ pass_of, long long* __restrict__ bytes) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > nov) return;
  if (p == nov) {
    bytes[p] = 0;
    return;
  }
  const int pass = pass_of ? pass_of[p] : 0;
  const bool run = pp[p].mode == PW_FAST && pass >= 0;
  bytes[p] = run ? (long long)pw_arena_bytes(nb, (int)(coff[p + 1] - coff[p]), pairK[p], pass) : 0;
}

// Persistent work queue, one pair per warp at a time (32 pairs sharing a warp
// would take turns through diverging paths; one warp shares a pair's
// data-parallel steps among its lanes instead).  The queue hands out pairs by
// decreasing expected work; a warp takes the next one until the queue is
// empty.
__global__ void __launch_bounds__(kPwPairBlock)
k_pw_pairs(PwPairArgs A, const int* __restrict__ pairK, int* __restrict__ queue) {
  for (;;) {
    int wi = 0;
    if ((threadIdx.x & 31) == 0) wi = atomicAdd(queue, 1);
    wi = __shfl_sync(kFullMask, wi, 0);
    if (wi >= A.nov) return;
    const int p = A.order[wi];
    const int pass = A.pass_of ? A.pass_of[p] : 0;
    if (pass < 0) continue;
    if (A.pp[p].mode != PW_FAST) {
      A.status[p] = A.pp[p].mode == PW_INPUT ? PS_UNDEF + 100 : PS_FALLBACK;
      A.nrings[p] = A.nverts[p] = 0;
      continue;
    }
    const int nc = (int)(A.coff[p + 1] - A.coff[p]);
    const PwCaps cp = pw_caps(A.nb, nc, pairK[p], pass);
    Carver cv{A.arena + A.aoff[p], 0};
    PwWork w = pw_carve(cv, cp);
    int nr = 0, nv = 0;
    const int st = pw_clip_pair(A, p, cp, w, &nr, &nv);
    A.status[p] = st;
    A.nrings[p] = st == PS_OK ? nr : 0;
    A.nverts[p] = st == PS_OK ? nv : 0;
  }
}

// where a pair's rings live: pass 0 arena, or the retry arena
struct PwArenas {
  const unsigned char* a0;
  const long long* off0;
  const unsigned char* a1;
  const long long* off1;
  const int* pass;
  __device__ const unsigned char* at(int p) const {
    return pass[p] == 1 ? a1 + off1[p] : a0 + off0[p];
  }
};

__global__ void k_pw_pack(int nov, const long long* __restrict__ coff, int nb,
                          const int* __restrict__ pairK, PwArenas ar, const int* __restrict__ fast,
                          const long long* __restrict__ rpre, const long long* __restrict__ vpre,
                          long long* __restrict__ ring_off, double* __restrict__ xy) {
  // one warp per pair, its lanes over the ring offsets and coordinates
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int p = (int)(t >> 5), lane = threadIdx.x & 31;
  if (p >= nov || !fast[p]) return;
  const long long r0 = rpre[p], v0 = vpre[p];
  const int nr = (int)(rpre[p + 1] - r0);
  if (nr == 0) return;
  const PwCaps cp = pw_caps(nb, (int)(coff[p + 1] - coff[p]), pairK[p], ar.pass[p]);
  Carver cv{const_cast<unsigned char*>(ar.at(p)), 0};
  const PwWork w = pw_carve(cv, cp);
  for (int r = lane; r < nr; r += 32) ring_off[r0 + r] = v0 + w.roff[r];
  const int nv = w.roff[nr];
  for (int i = lane; i < 2 * nv; i += 32) xy[2 * v0 + i] = w.rxy[i];
}

}  // namespace

// ------------------------------------------------------------------ host
// one pipeline, stream and host thread taking big pairs
struct PairwiseRunner::BigWorker {
  cudaStream_t st = nullptr;
  std::unique_ptr<Pipeline> pl;
  int rc = 0;
  std::string msg;
  ~BigWorker() {
    if (!st) return;
    cudaStreamSynchronize(st);
    pl.reset();
    cudaStreamDestroy(st);
  }
};

// persistent grid of the per-pair kernel: every block slot of every SM, less
// `pair_reserve` slots per SM while big pairs run beside it (their pipeline
// kernels need room on the SMs)
unsigned PairwiseRunner::pair_grid(int nov, bool reserve) {
  static_assert(kPwPairBlock % 32 == 0, "whole warps");
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pw_pairs, kPwPairBlock, 0);
  const int slots = std::max(1, reserve ? per_sm - pair_reserve : per_sm);
  pair_blocks_ = (unsigned)std::max(1, sms * slots);
  const unsigned need = grid_for(32LL * nov, kPwPairBlock);
  return need < pair_blocks_ ? need : pair_blocks_;
}

// Time the job under a few settings and keep the fastest (results depend on
// none of them), one setting at a time at the best so far: the big-pair
// split, the block slots left to big pairs, the big-pair worker count, the
// grid cell width.
int PairwiseRunner::autotune(const double* d_bxy, int nb, int nov, const double* d_cxy,
                             const long long* d_coff, cudaStream_t st, double* best_ms) {
  // the better of two runs: one run's time varies by several percent
  auto timed = [&](double* ms) -> int {
    *ms = 1e300;
    for (int k = 0; k < 2; ++k) {
      const auto t0 = std::chrono::steady_clock::now();
      const int rc = run(d_bxy, nb, nov, d_cxy, d_coff, st);
      if (rc) return rc;
      if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise autotune");
      const double t =
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      *ms = std::min(*ms, t);
    }
    return kOk;
  };
  double ms = 0;
  int rc = timed(&ms);  // warm-up: buffers grow to size
  if (rc) return rc;
  int best_split = big_k;
  double best_cell = cell_factor, best = 1e300;
  for (int split : {2048, 4096, 6144, 8192, 10240, 12288, 14336, 16384, 32768}) {
    big_k = split;
    rc = timed(&ms);
    if (rc) return rc;
    if (ms < best) {
      best = ms;
      best_split = split;
    }
  }
  big_k = best_split;
  int best_reserve = pair_reserve;
  for (int r : {0, 1, 2}) {
    if (r == best_reserve) continue;
    pair_reserve = r;
    rc = timed(&ms);
    if (rc) return rc;
    if (ms < best) {
      best = ms;
      best_reserve = r;
    }
  }
  pair_reserve = best_reserve;
  int best_workers = big_workers;
  for (int nw : {4, 16}) {
    big_workers = nw;
    rc = timed(&ms);
    if (rc) return rc;
    if (ms < best) {
      best = ms;
      best_workers = nw;
    }
  }
  big_workers = best_workers;
  for (double f : {0.5, 2.0}) {
    cell_factor = f;
    rc = timed(&ms);
    if (rc) return rc;
    if (ms < best) {
      best = ms;
      best_cell = f;
    }
  }
  cell_factor = best_cell;
  if (best_ms) *best_ms = best;
  return kOk;
}

PairwiseRunner::PairwiseRunner(Pipeline& pl) : pl_(pl) {}

PairwiseRunner::~PairwiseRunner() {
  if (st2_) {
    cudaStreamSynchronize(st2_);
    cudaStreamDestroy(st2_);
  }
  for (auto e : ev_)
    if (e) cudaEventDestroy(e);
}

int PairwiseRunner::run(const double* d_bxy, int nb, int nov, const double* d_cxy,
                        const long long* d_coff, cudaStream_t st) {
  BufferPool& pool = pl_.pool();
  np = nov;
  fallback_pairs = 0;
  big_pairs = 0;
  fb_rec_.clear();
  fb_xy_.clear();
  valid = false;
  hits = 0;
  tested = 0;
  if (nb < 3) return pl_.fail(kEInput, "base needs at least 3 vertices");
  if (nov < 0) return pl_.fail(kEInput, "negative overlay count");
  status = (int*)pool.get("pw_status", sizeof(int) * (nov + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise)");
  h_status.assign(nov, SBC_OK);
  h_pair_ring.assign(nov + 1, 0);
  total_rings = total_verts = 0;
  if (nov == 0) return kOk;
  long long totalC = 0;
  std::vector<long long> hoff(nov + 1);
  cudaMemcpyAsync(hoff.data(), d_coff, sizeof(long long) * (nov + 1), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise offsets");
  totalC = hoff[nov];
  for (int i = 0; i < nov; ++i)
    if (hoff[i + 1] < hoff[i]) return pl_.fail(kEInput, "overlay offsets must not decrease");
  // ---- base
  auto* keys = (unsigned long long*)pool.get("pw_bkeys", sizeof(unsigned long long) * nb);
  auto* keys2 = (unsigned long long*)pool.get("pw_bkeys2", sizeof(unsigned long long) * nb);
  auto* vals = (unsigned*)pool.get("pw_bvals", sizeof(unsigned) * nb);
  auto* vals2 = (unsigned*)pool.get("pw_bvals2", sizeof(unsigned) * nb);
  void* rscr = pool.get("pw_rscr", radix_scratch_bytes(nb));
  auto* fbox = (float4*)pool.get("pw_fbox", sizeof(float4) * nb);
  auto* stats = (PwBaseStats*)pool.get("pw_bstats", sizeof(PwBaseStats));
  int* flag = (int*)pool.get("pw_uflag", sizeof(int) * (nb + 1));
  void* sscr = pool.get("pw_scan", scan_scratch_bytes((long long)nb + nov + 2) * 2);
  double* ub = (double*)pool.get("pw_ub", sizeof(double) * nb);
  int* rankB = (int*)pool.get("pw_rankb", sizeof(int) * nb);
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise base)");
  PwBaseStats hs0{~0ull, 0ull, ~0ull, 0ull, 0.0, 0u};
  cudaMemcpyAsync(stats, &hs0, sizeof(hs0), cudaMemcpyHostToDevice, st);
  {
    ::sbc::KProbe kp_("k_pw_base_edges", st, 16.0 * nb + 28.0 * nb);
    k_pw_base_edges<<<grid_for(nb, 256), 256, 0, st>>>(nb, d_bxy, keys, vals, fbox, stats);
  }
  radix_sort_u64(keys, vals, keys2, vals2, nb, rscr, st);
  {
    ::sbc::KProbe kp_("k_pw_uflag", st);
    k_pw_uflag<<<grid_for(nb + 1, 256), 256, 0, st>>>(nb, keys, flag);
  }
  exclusive_scan_i32(flag, nb + 1, sscr, st);
  {
    ::sbc::KProbe kp_("k_pw_uscatter", st);
    k_pw_uscatter<<<grid_for(nb, 256), 256, 0, st>>>(nb, keys, vals, flag, d_bxy, ub, rankB);
  }
  PwBaseStats hs;
  int nub = 0;
  cudaMemcpyAsync(&hs, stats, sizeof(hs), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&nub, flag + nb, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise base");
  auto unkey = [](unsigned long long k) {
    unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    double d;
    std::memcpy(&d, &u, sizeof d);
    return d;
  };
  // grid: cells the larger of sqrt(area / n_b) and 1.5 mean edge extents
  // wide, times the tuned factor, at most 2^22 cells
  const double bx0 = unkey(hs.mnx), bx1 = unkey(hs.mxx), by0 = unkey(hs.mny), by1 = unkey(hs.mxy);
  const double W = std::max(bx1 - bx0, 1e-300), Hh = std::max(by1 - by0, 1e-300);
  double h = cell_factor * std::max(std::sqrt(W * Hh / nb), 1.5 * hs.ext / nb);
  if (!(h > 0) || !std::isfinite(h)) h = std::max(W, Hh);
  while ((W / h + 1) * (Hh / h + 1) > (double)(1 << 22)) h *= 1.25;
  PwGrid g;
  g.x0 = (float)bx0;
  g.y0 = (float)by0;
  g.inv = (float)(1.0 / h);
  g.gx = std::max(1, (int)std::ceil(W / h) + 1);
  g.gy = std::max(1, (int)std::ceil(Hh / h) + 1);
  grid_cells = (long long)g.gx * g.gy;
  const int ncell = g.gx * g.gy;
  int* gstart = (int*)pool.get("pw_gstart", sizeof(int) * (ncell + 1));
  int* gcur = (int*)pool.get("pw_gcur", sizeof(int) * (ncell + 1));
  int* lng = (int*)pool.get("pw_long", sizeof(int) * nb);
  unsigned* nlong = (unsigned*)pool.get("pw_nlong", 256);
  void* gscr = pool.get("pw_gscan", scan_scratch_bytes(ncell + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise grid)");
  cudaMemsetAsync(gstart, 0, sizeof(int) * (ncell + 1), st);
  cudaMemsetAsync(gcur, 0, sizeof(int) * (ncell + 1), st);
  cudaMemsetAsync(nlong, 0, sizeof(unsigned), st);
  {
    ::sbc::KProbe kp_("k_pw_grid_count", st);
    k_pw_grid_count<<<grid_for(nb, 256), 256, 0, st>>>(nb, fbox, g, gstart, lng, nlong);
  }
  exclusive_scan_i32(gstart, ncell + 1, gscr, st);
  int gtotal = 0;
  cudaMemcpyAsync(&gtotal, gstart + ncell, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise grid");
  int* gent = (int*)pool.get("pw_gent", sizeof(int) * (gtotal + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise grid)");
  {
    ::sbc::KProbe kp_("k_pw_grid_fill", st);
    k_pw_grid_fill<<<grid_for(nb, 256), 256, 0, st>>>(nb, fbox, g, gstart, gcur, gent);
  }
  // ---- overlays
  PwPair* pp = (PwPair*)pool.get("pw_pairs", sizeof(PwPair) * nov);
  int* rankC = (int*)pool.get("pw_rankc", sizeof(int) * (totalC + 1));
  int* rankCB = (int*)pool.get("pw_rankcb", sizeof(int) * (totalC + 1));
  double* uval = (double*)pool.get("pw_uval", sizeof(double) * (totalC + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise overlays)");
  cudaMemsetAsync(pp, 0, sizeof(PwPair) * nov, st);
  const int base_flags = (int)hs.flags;
  int maxn = 0;
  for (int i = 0; i < nov; ++i) maxn = std::max<long long>(maxn, hoff[i + 1] - hoff[i]);
  const int classes[4] = {-1, 1024, 4096, kPwMaxOverlay};
  for (int k = 0; k < 3; ++k) {
    if (maxn <= classes[k]) break;
    const int P2 = classes[k + 1];
    const size_t smem = (size_t)P2 * (sizeof(unsigned long long) + sizeof(int));
    cudaFuncSetAttribute(k_pw_overlay_prep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    ::sbc::KProbe kp_("k_pw_overlay_prep", st);
    k_pw_overlay_prep<<<nov, kPwPrepThreads, smem, st>>>(nov, d_coff, d_cxy, classes[k], P2, ub, nub,
                                                         base_flags, pp, rankC, rankCB, uval);
  }
  // overlays above the largest class
  if (maxn > kPwMaxOverlay) {
    std::vector<PwPair> hp(nov);
    cudaMemcpyAsync(hp.data(), pp, sizeof(PwPair) * nov, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise prep");
    for (int i = 0; i < nov; ++i)
      if (hoff[i + 1] - hoff[i] > kPwMaxOverlay) hp[i].mode = PW_FALLBACK;
    cudaMemcpyAsync(pp, hp.data(), sizeof(PwPair) * nov, cudaMemcpyHostToDevice, st);
  }
  // ---- candidates
  int* pairK = (int*)pool.get("pw_pairk", sizeof(int) * (nov + 1));
  int* hstart = (int*)pool.get("pw_hstart", sizeof(int) * (nov + 1));
  auto* cnt = (unsigned long long*)pool.get("pw_counters", 256);
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise)");
  int* tpair = (int*)pool.get("pw_tpair", sizeof(int) * (totalC + 1));
  long long* coffs = (long long*)pool.get("pw_coffs", sizeof(long long) * (totalC + 1));
  void* cscr = pool.get("pw_cscan", scan_scratch_bytes(totalC + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise candidates)");
  cudaMemsetAsync(pairK, 0, sizeof(int) * (nov + 1), st);
  cudaMemsetAsync(cnt, 0, 3 * sizeof(unsigned long long), st);
  PwCandArgs ca{};
  ca.nov = nov;
  ca.coff = d_coff;
  ca.totalC = totalC;
  ca.cxy = d_cxy;
  ca.b = d_bxy;
  ca.nb = nb;
  ca.g = g;
  ca.gstart = gstart;
  ca.gent = gent;
  ca.lng = lng;
  ca.nlong = nlong;
  ca.fbox = fbox;
  ca.pp = pp;
  ca.rankB = rankB;
  ca.rankC = rankC;
  ca.rankCB = rankCB;
  ca.uval = uval;
  ca.tpair = tpair;
  ca.coffs = coffs;
  ca.nhits = &cnt[0];
  ca.tested = &cnt[1];
  ca.nraw = &cnt[2];
  ca.pairK = pairK;
  // 1. box-overlapping (overlay edge, base edge) pairs
  long long ncand = 0;
  if (totalC > 0) {
    {
      ::sbc::KProbe kp_("k_pw_cand_count", st, 40.0 * totalC);
      k_pw_cand_count<<<grid_for(totalC + 1, 128), 128, 0, st>>>(ca);
    }
    exclusive_scan_i64(coffs, totalC + 1, cscr, st);
    cudaMemcpyAsync(&ncand, coffs + totalC, sizeof(long long), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise candidates");
  }
  int2* cand = (int2*)pool.get("pw_cand", sizeof(int2) * (ncand + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise candidates)");
  ca.cand = cand;
  ca.ncand = ncand;
  if (ncand > 0) {
    ::sbc::KProbe kp_("k_pw_cand_fill", st, 40.0 * totalC + 8.0 * ncand);
    k_pw_cand_fill<<<grid_for(totalC, 128), 128, 0, st>>>(ca);
  }
  // 2. the FP64 test of each
  unsigned long long rawcap = std::max<unsigned long long>(hit_cap_, 1ull << 16);
  unsigned long long nraw = 0;
  for (int attempt = 0; attempt < 2; ++attempt) {
    ca.raw = (PwHit*)pool.get("pw_raw", sizeof(PwHit) * rawcap);
    ca.rawcap = rawcap;
    if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise hits)");
    cudaMemsetAsync(&cnt[1], 0, 2 * sizeof(unsigned long long), st);
    if (ncand > 0) {
      ::sbc::KProbe kp_("k_pw_cand_test", st, 72.0 * ncand);
      k_pw_cand_test<<<grid_for(ncand, 256), 256, 0, st>>>(ca);
    }
    unsigned long long hc[2];
    cudaMemcpyAsync(hc, &cnt[1], sizeof(hc), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise candidates");
    tested = (long long)hc[0];
    nraw = hc[1];
    if (nraw <= rawcap) break;
    rawcap = nraw + nraw / 4 + 1024;
  }
  if (nraw > rawcap) return pl_.fail(kEInternal, "pairwise hit count changed between passes");
  hit_cap_ = std::max(hit_cap_, nraw);
  // 3. tree quantities and emission keys of the intersections
  PwHit* hbuf = (PwHit*)pool.get("pw_hits", sizeof(PwHit) * (nraw + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise hits)");
  ca.hits = hbuf;
  ca.cap = nraw + 1;
  unsigned long long nh = 0;
  if (nraw > 0) {
    {
      ::sbc::KProbe kp_("k_pw_hit_tree", st, 120.0 * (double)nraw);
      k_pw_hit_tree<<<grid_for((long long)nraw, 256), 256, 0, st>>>(ca, (long long)nraw);
    }
    cudaMemcpyAsync(&nh, &cnt[0], sizeof(nh), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise candidates");
  }
  hits = (long long)nh;
  cudaMemcpyAsync(hstart, pairK, sizeof(int) * (nov + 1), cudaMemcpyDeviceToDevice, st);
  exclusive_scan_i32(hstart, nov + 1, sscr, st);
  PwHit* grouped = (PwHit*)pool.get("pw_hits_grouped", sizeof(PwHit) * (nh + 1));
  auto* hk = (unsigned long long*)pool.get("pw_hk", sizeof(unsigned long long) * (nh + 1));
  auto* hk2 = (unsigned long long*)pool.get("pw_hk2", sizeof(unsigned long long) * (nh + 1));
  auto* hv = (unsigned*)pool.get("pw_hv", sizeof(unsigned) * (nh + 1));
  auto* hv2 = (unsigned*)pool.get("pw_hv2", sizeof(unsigned) * (nh + 1));
  void* hscr = pool.get("pw_hscr", radix_scratch_bytes((long long)nh + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise hits)");
  if (nh) {
    {
      ::sbc::KProbe kp_("k_pw_hit_keys", st, 52.0 * (double)nh);
      k_pw_hit_keys<<<grid_for((long long)nh, 256), 256, 0, st>>>((long long)nh, hbuf, hk, hv);
    }
    radix_sort_u64(hk, hv, hk2, hv2, (long long)nh, hscr, st);
    {
      ::sbc::KProbe kp_("k_pw_hit_keys2", st, 20.0 * (double)nh);
      k_pw_hit_keys2<<<grid_for((long long)nh, 256), 256, 0, st>>>((long long)nh, hbuf, hv, hk);
    }
    radix_sort_u64(hk, hv, hk2, hv2, (long long)nh, hscr, st);
    {
      ::sbc::KProbe kp_("k_pw_gather", st, 84.0 * (double)nh);
      k_pw_gather<<<grid_for((long long)nh, 256), 256, 0, st>>>((long long)nh, hbuf, hv, grouped);
    }
  }
  // ---- pairs with many intersections take the pair pipeline's data-parallel
  // rows A9-A18 on these records (no tree), on worker streams; the rest run
  // one warp per pair on a second stream at the same time.  Then pairs that
  // ran out of ring room run again with full room.
  long long* aoff0 = (long long*)pool.get("pw_aoff0", sizeof(long long) * (nov + 1));
  long long* aoff1 = (long long*)pool.get("pw_aoff1", sizeof(long long) * (nov + 1));
  int* pass = (int*)pool.get("pw_pass", sizeof(int) * (nov + 1));
  int* nrings = (int*)pool.get("pw_nrings", sizeof(int) * (nov + 1));
  int* nverts = (int*)pool.get("pw_nverts", sizeof(int) * (nov + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise)");
  std::vector<int> hK(nov + 1);
  std::vector<PwPair> hpp(nov);
  unsigned hlong = 0;
  cudaMemcpyAsync(hK.data(), pairK, sizeof(int) * nov, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hpp.data(), pp, sizeof(PwPair) * nov, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&hlong, nlong, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise counts");
  std::vector<int> hpass(nov, 0), is_big(nov, 0);
  std::vector<long long> hstart_h(nov + 1, 0);
  int maxBig = 0;
  big_pairs = 0;
  for (int p = 0; p < nov; ++p) {
    hstart_h[p + 1] = hstart_h[p] + hK[p];
    if (hpp[p].mode == PW_FAST && hK[p] >= big_k) {
      is_big[p] = 1;
      hpass[p] = -1;
      maxBig = std::max(maxBig, hK[p]);
      ++big_pairs;
    }
  }
  cudaMemcpyAsync(pass, hpass.data(), sizeof(int) * nov, cudaMemcpyHostToDevice, st);
  // longest first: the warps that start first take the pairs with the most
  // records and vertices
  {
    std::vector<long long> cost(nov);
    order_h.resize(nov);
    for (int p = 0; p < nov; ++p) {
      order_h[p] = p;
      cost[p] = 8LL * hK[p] + (hoff[p + 1] - hoff[p]);
    }
    std::stable_sort(order_h.begin(), order_h.end(),
                     [&](int a, int b) { return cost[a] > cost[b]; });
  }
  int* order = (int*)pool.get("pw_order", sizeof(int) * (nov + 1));
  int* queue = (int*)pool.get("pw_queue", 256);
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise)");
  cudaMemcpyAsync(order, order_h.data(), sizeof(int) * nov, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(queue, 0, 2 * sizeof(int), st);
  PwPip pip{d_bxy, nb, g, gstart, gent, lng, (int)hlong, fbox, nullptr, 0};
  {
    ::sbc::KProbe kp_("k_pw_sizes", st);
    k_pw_sizes<<<grid_for(nov + 1, 256), 256, 0, st>>>(nov, d_coff, nb, pp, pairK, pass, aoff0);
  }
  exclusive_scan_i64(aoff0, nov + 1, sscr, st);
  long long total = 0;
  cudaMemcpyAsync(&total, aoff0 + nov, sizeof(long long), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise sizes");
  unsigned char* arena0 = (unsigned char*)pool.get("pw_arena0", (size_t)total + 256);
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise arena)");
  if (!st2_ && cudaStreamCreateWithFlags(&st2_, cudaStreamNonBlocking) != cudaSuccess)
    return pl_.fail(kECuda, "pairwise stream");
  if (!ev_[0] && (cudaEventCreateWithFlags(&ev_[0], cudaEventDisableTiming) != cudaSuccess ||
                  cudaEventCreateWithFlags(&ev_[1], cudaEventDisableTiming) != cudaSuccess))
    return pl_.fail(kECuda, "pairwise events");
  PwPairArgs pa{nov, d_coff, d_cxy, d_bxy, nb, pp, hstart, grouped, pass, order, arena0, aoff0,
                status, pl_.unite ? 1 : 0, nrings, nverts, pip};
  cudaEventRecord(ev_[0], st);
  cudaStreamWaitEvent(st2_, ev_[0], 0);
  {
    // coordinates and records in; rings out
    ::sbc::KProbe kp_("k_pw_pairs", st2_, 16.0 * totalC + 40.0 * (double)nh);
    k_pw_pairs<<<pair_grid(nov, big_pairs > 0), kPwPairBlock, 0, st2_>>>(pa, pairK, queue);
  }
  cudaEventRecord(ev_[1], st2_);
  struct Stash {
    std::vector<int> off;
    std::vector<double> xy;
  };
  std::vector<Stash> stash(nov);
  std::vector<int> stash_of(nov, -1), hnr(nov, 0), hnv(nov, 0), fast(nov, 0);
  auto keep = [&](int p) -> int {
    const auto& out = pl_.outputs()[0];
    Stash& sh = stash[p];
    sh.off.assign(out.nrings + 1, 0);
    sh.xy.resize(2 * out.nverts);
    if (out.nrings > 0)
      cudaMemcpyAsync(sh.off.data(), out.d_off, sizeof(int) * (out.nrings + 1),
                      cudaMemcpyDeviceToHost, st);
    if (out.nverts > 0)
      cudaMemcpyAsync(sh.xy.data(), out.d_xy, sizeof(double) * 2 * out.nverts,
                      cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise pipeline");
    hnr[p] = out.nrings;
    hnv[p] = (int)out.nverts;
    stash_of[p] = p;
    return kOk;
  };
  // big pairs: worker host threads, each with its own pipeline and stream,
  // take them one at a time (a pair's pipeline waits on the host between its
  // stages; several pairs in flight keep the GPU busy meanwhile)
  std::vector<int> bigs;
  for (int p = 0; p < nov; ++p)
    if (is_big[p]) bigs.push_back(p);
  if (!bigs.empty()) {
    const int nw = std::max(1, std::min<int>(big_workers, (int)bigs.size()));
    int dev = 0;
    cudaGetDevice(&dev);
    while ((int)workers_.size() < nw) {
      auto wk = std::make_unique<BigWorker>();
      if (cudaStreamCreateWithFlags(&wk->st, cudaStreamNonBlocking) != cudaSuccess)
        return pl_.fail(kECuda, "pairwise worker stream");
      wk->pl = std::make_unique<Pipeline>(dev, wk->st);
      workers_.push_back(std::move(wk));
    }
    std::atomic<int> next{0};
    std::atomic<bool> stop{false};
    auto work = [&](BigWorker& W) {
      cudaSetDevice(dev);
      Pipeline& wp = *W.pl;
      wp.unite = pl_.unite;
      wp.force_serial_backend = pl_.force_serial_backend;
      W.rc = 0;
      W.msg.clear();
      BufferPool& wpool = wp.pool();
      int* brb = (int*)wpool.get("pw_big_rb", sizeof(int) * (maxBig + 1));
      int* brc = (int*)wpool.get("pw_big_rc", sizeof(int) * (maxBig + 1));
      int* brt = (int*)wpool.get("pw_big_rt", sizeof(int) * (maxBig + 1));
      auto* bkey =
          (unsigned long long*)wpool.get("pw_big_key", sizeof(unsigned long long) * (maxBig + 1));
      if (wpool.failed) {
        W.rc = kENoMem;
        W.msg = "device allocation failed (pairwise big pairs)";
        stop = true;
        return;
      }
      cudaStreamWaitEvent(W.st, ev_[0], 0);  // the grouped records
      for (;;) {
        const int i = stop ? (int)bigs.size() : next++;
        if (i >= (int)bigs.size()) break;
        const int p = bigs[i];
        const int K = hK[p];
        {
          ::sbc::KProbe kp_("k_pw_split", W.st, 72.0 * K);
          k_pw_split<<<grid_for(K, 256), 256, 0, W.st>>>(K, grouped + hstart_h[p], brb, brc, brt,
                                                         bkey);
        }
        wp.clear_error();
        const int rc = wp.run_from_hits(d_bxy, nb, d_cxy + 2 * hoff[p],
                                        (int)(hoff[p + 1] - hoff[p]), brb, brc, brt, bkey, K);
        if (rc == kEInput || rc == kEUndef) {
          h_status[p] = rc == kEInput ? SBC_EINPUT : SBC_EUNDEF;
          continue;
        }
        if (rc) {
          W.rc = rc;
          W.msg = wp.error();
          stop = true;
          break;
        }
        const auto& out = wp.outputs()[0];
        Stash& sh = stash[p];
        sh.off.assign(out.nrings + 1, 0);
        sh.xy.resize(2 * out.nverts);
        if (out.nrings > 0)
          cudaMemcpyAsync(sh.off.data(), out.d_off, sizeof(int) * (out.nrings + 1),
                          cudaMemcpyDeviceToHost, W.st);
        if (out.nverts > 0)
          cudaMemcpyAsync(sh.xy.data(), out.d_xy, sizeof(double) * 2 * out.nverts,
                          cudaMemcpyDeviceToHost, W.st);
        if (cudaStreamSynchronize(W.st) != cudaSuccess) {
          W.rc = kECuda;
          W.msg = "pairwise pipeline";
          stop = true;
          break;
        }
        hnr[p] = out.nrings;
        hnv[p] = (int)out.nverts;
        stash_of[p] = p;
      }
      cudaStreamSynchronize(W.st);
    };
    for (int w = 0; w < nw; ++w) {
      workers_[w]->rc = 0;
      workers_[w]->msg.clear();
    }
    std::vector<std::thread> th;
    for (int w = 1; w < nw; ++w) {
      // a thread that cannot be started leaves its share to the others (the
      // queue is shared)
      try {
        th.emplace_back(work, std::ref(*workers_[w]));
      } catch (...) {
        break;
      }
    }
    work(*workers_[0]);
    for (auto& t : th) t.join();
    for (int w = 0; w < nw; ++w)
      if (workers_[w]->rc) return pl_.fail(workers_[w]->rc, workers_[w]->msg);
  }
  cudaStreamWaitEvent(st, ev_[1], 0);
  std::vector<int> hst(nov);
  cudaMemcpyAsync(hst.data(), status, sizeof(int) * nov, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise clip");
  int retry = 0;
  for (int p = 0; p < nov; ++p) {
    hpass[p] = -1;
    if (!is_big[p] && hst[p] == PS_CAP) {
      hpass[p] = 1;
      ++retry;
    }
  }
  unsigned char* arena1 = arena0;
  if (retry) {
    cudaMemcpyAsync(pass, hpass.data(), sizeof(int) * nov, cudaMemcpyHostToDevice, st);
    {
      ::sbc::KProbe kp_("k_pw_sizes", st);
      k_pw_sizes<<<grid_for(nov + 1, 256), 256, 0, st>>>(nov, d_coff, nb, pp, pairK, pass, aoff1);
    }
    exclusive_scan_i64(aoff1, nov + 1, sscr, st);
    cudaMemcpyAsync(&total, aoff1 + nov, sizeof(long long), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise sizes");
    arena1 = (unsigned char*)pool.get("pw_arena1", (size_t)total + 256);
    if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise arena)");
    pa.arena = arena1;
    pa.aoff = aoff1;
    {
      ::sbc::KProbe kp_("k_pw_pairs", st);
      k_pw_pairs<<<pair_grid(nov, false), kPwPairBlock, 0, st>>>(pa, pairK, queue + 1);
    }
    cudaMemcpyAsync(hst.data(), status, sizeof(int) * nov, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise clip");
  }
  for (int p = 0; p < nov; ++p) hpass[p] = hpass[p] == 1 ? 1 : 0;
  cudaMemcpyAsync(pass, hpass.data(), sizeof(int) * nov, cudaMemcpyHostToDevice, st);
  // ---- per pair: fast result, input error, or the whole pair pipeline
  std::vector<int> fnr(nov), fnv(nov);
  cudaMemcpyAsync(fnr.data(), nrings, sizeof(int) * nov, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(fnv.data(), nverts, sizeof(int) * nov, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise clip");
  for (int p = 0; p < nov; ++p) {
    if (is_big[p]) continue;
    if (hst[p] == PS_OK) {
      fast[p] = 1;
      hnr[p] = fnr[p];
      hnv[p] = fnv[p];
      continue;
    }
    const long long n = hoff[p + 1] - hoff[p];
    if (hst[p] == PS_UNDEF + 100 || n < 3) {
      h_status[p] = SBC_EINPUT;
      continue;
    }
    // the pair pipeline, exactly as sbc_clip_pair would run it
    ++fallback_pairs;
    const int sizes[1] = {(int)n};
    pl_.clear_error();
    const int rc = pl_.run(d_bxy, nb, d_cxy + 2 * hoff[p], sizes, 1);
    if (rc == kEInput || rc == kEUndef) {
      h_status[p] = rc == kEInput ? SBC_EINPUT : SBC_EUNDEF;
      continue;
    }
    if (rc) return rc;
    // its records too (the gradient's provenance of crossings)
    const int K = pl_.dbg_K;
    if (K > 0) {
      std::vector<int> rb(K), rc2(K), rt(K);
      std::vector<double> rxy(2 * (size_t)K);
      cudaMemcpyAsync(rb.data(), pl_.dbg_ub, sizeof(int) * K, cudaMemcpyDeviceToHost, st);
      cudaMemcpyAsync(rc2.data(), pl_.dbg_uc, sizeof(int) * K, cudaMemcpyDeviceToHost, st);
      cudaMemcpyAsync(rt.data(), pl_.dbg_ut, sizeof(int) * K, cudaMemcpyDeviceToHost, st);
      cudaMemcpyAsync(rxy.data(), pl_.dbg_isxy, sizeof(double) * 2 * K, cudaMemcpyDeviceToHost, st);
      if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise records");
      for (int r = 0; r < K; ++r) {
        if (rt[r] != 1) continue;
        fb_rec_.push_back({{p, rb[r] >> 1, rc2[r] >> 1, 1}});
        fb_xy_.push_back(rxy[2 * r]);
        fb_xy_.push_back(rxy[2 * r + 1]);
      }
    }
    const int k2 = keep(p);
    if (k2) return k2;
  }
  pl_.clear_error();
  // ---- packed output
  std::vector<long long> rpre(nov + 1, 0), vpre(nov + 1, 0);
  for (int p = 0; p < nov; ++p) {
    rpre[p + 1] = rpre[p] + hnr[p];
    vpre[p + 1] = vpre[p] + hnv[p];
  }
  total_rings = rpre[nov];
  total_verts = vpre[nov];
  h_pair_ring = rpre;
  long long* d_rpre = (long long*)pool.get("pw_rpre", sizeof(long long) * (nov + 1));
  long long* d_vpre = (long long*)pool.get("pw_vpre", sizeof(long long) * (nov + 1));
  int* d_fast = (int*)pool.get("pw_fast", sizeof(int) * (nov + 1));
  ring_off = (long long*)pool.get("pw_ring_off", sizeof(long long) * (total_rings + 1));
  xy = (double*)pool.get("pw_xy", sizeof(double) * 2 * (total_verts + 1));
  pair_ring = d_rpre;
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise output)");
  cudaMemcpyAsync(d_rpre, rpre.data(), sizeof(long long) * (nov + 1), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d_vpre, vpre.data(), sizeof(long long) * (nov + 1), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d_fast, fast.data(), sizeof(int) * nov, cudaMemcpyHostToDevice, st);
  {
    const PwArenas ar{arena0, aoff0, arena1, aoff1, pass};
    ::sbc::KProbe kp_("k_pw_pack", st);
    k_pw_pack<<<grid_for(32LL * nov, 128), 128, 0, st>>>(nov, d_coff, nb, pairK, ar, d_fast, d_rpre,
                                                  d_vpre, ring_off, xy);
  }
  std::vector<long long> roff_h;
  for (int p = 0; p < nov; ++p) {
    if (stash_of[p] < 0 || hnr[p] == 0) continue;
    const Stash& s = stash[p];
    roff_h.resize(hnr[p]);
    for (int r = 0; r < hnr[p]; ++r) roff_h[r] = vpre[p] + s.off[r];
    cudaMemcpyAsync(ring_off + rpre[p], roff_h.data(), sizeof(long long) * hnr[p],
                    cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(xy + 2 * vpre[p], s.xy.data(), sizeof(double) * 2 * hnv[p],
                    cudaMemcpyHostToDevice, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise output");
  }
  cudaMemcpyAsync(ring_off + total_rings, &total_verts, sizeof(long long), cudaMemcpyHostToDevice,
                  st);
  cudaMemcpyAsync(status, h_status.data(), sizeof(int) * nov, cudaMemcpyHostToDevice, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise output");
  // kept for the area gradient
  last_nb_ = nb;
  last_totalC_ = totalC;
  last_nh_ = (long long)nh;
  h_coff_ = hoff;
  key_b = d_bxy;
  key_c = d_cxy;
  valid = true;
  return kOk;
}

}  // namespace sbc

// ------------------------------------------------------------------ area and gradient
// Area of overlay i's result: the signed shoelace sum of its rings.  Its
// gradient with the combinatorial structure held fixed chains through where
// each ring vertex comes from, found by exact coordinates in the order a base
// vertex, an overlay vertex, a proper crossing I = (1 - a) b1 + a b2 (a
// type-1 record) -- candidates sorted by (pair, x, y), ties in that order.
namespace sbc {
namespace {

__global__ void k_pwa_area(int nov, const long long* __restrict__ pair_ring,
                           const long long* __restrict__ ring_off, const double* __restrict__ xy,
                           const int* __restrict__ status, double* __restrict__ area) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nov) return;
  double a = 0.0;
  if (status[p] == SBC_OK) {
    for (long long r = pair_ring[p]; r < pair_ring[p + 1]; ++r) {
      const long long s = ring_off[r], e = ring_off[r + 1];
      double s2 = 0.0;
      for (long long i = s; i < e; ++i) {
        const long long j = (i + 1 == e) ? s : i + 1;
        s2 = dadd(s2, dsub(dmul(xy[2 * i], xy[2 * j + 1]), dmul(xy[2 * j], xy[2 * i + 1])));
      }
      a = dadd(a, dmul(0.5, s2));
    }
  }
  area[p] = a;
}

__global__ void k_pwa_base_keys(int nb, const double* __restrict__ b,
                                unsigned long long* __restrict__ kx,
                                unsigned long long* __restrict__ ky, unsigned* __restrict__ val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  kx[i] = dkey(b[2 * i]);
  ky[i] = dkey(b[2 * i + 1]);
  val[i] = (unsigned)i;
}

// per-pair candidates: overlay vertices, then the type-1 records of the
// batched pairs (hits), then those of pairs the pair pipeline clipped
struct PwaCand {
  int nov;
  const long long* coff;
  long long totalC;
  const double* cxy;
  long long nh;
  const PwHit* hits;
  int nb;
  const double* b;
  long long nfb;
  const int4* fb_rec;   // pair, base edge, overlay edge, type
  const double* fb_xy;  // crossing coordinates
};

__device__ __forceinline__ void pwa_decode(const PwaCand& C, long long i, int* pair, int4* t) {
  if (i < C.totalC) {
    int lo = 0, hi = C.nov;
    while (hi - lo > 1) {
      const int m = (lo + hi) >> 1;
      if (C.coff[m] <= i) lo = m;
      else hi = m;
    }
    *pair = lo;
    *t = make_int4(1, (int)(i - C.coff[lo]), 0, 0);
  } else if (i < C.totalC + C.nh) {
    const PwHit& h = C.hits[i - C.totalC];
    *pair = h.pair;
    *t = make_int4(2, h.b, h.j, h.type);
  } else {
    const int4 r = C.fb_rec[i - C.totalC - C.nh];
    *pair = r.x;
    *t = make_int4(2, r.y, r.z, r.w);
  }
}

__global__ void k_pwa_cand(PwaCand C, long long n, unsigned long long* __restrict__ kx,
                           unsigned long long* __restrict__ ky, unsigned long long* __restrict__ kp,
                           unsigned* __restrict__ val) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int pair;
  int4 t;
  pwa_decode(C, i, &pair, &t);
  double x = 0.0, y = 0.0;
  bool use = true;
  if (t.x == 1) {
    x = C.cxy[2 * (C.coff[pair] + t.y)];
    y = C.cxy[2 * (C.coff[pair] + t.y) + 1];
  } else if (i < C.totalC + C.nh) {
    use = t.w == 1;
    if (use) {  // I = (1 - a) b1 + a b2, as the record stage computed it
      const double al = C.hits[i - C.totalC].al;
      const int i2 = t.y + 1 == C.nb ? 0 : t.y + 1;
      const double oma = dsub(1.0, al);
      x = dadd(dmul(oma, C.b[2 * t.y]), dmul(al, C.b[2 * i2]));
      y = dadd(dmul(oma, C.b[2 * t.y + 1]), dmul(al, C.b[2 * i2 + 1]));
    }
  } else {
    const long long r = i - C.totalC - C.nh;
    x = C.fb_xy[2 * r];
    y = C.fb_xy[2 * r + 1];
  }
  kx[i] = use ? dkey(x) : ~0ull;
  ky[i] = use ? dkey(y) : ~0ull;
  kp[i] = use ? (unsigned long long)pair : ~0ull;
  val[i] = (unsigned)i;
}

__global__ void k_pwa_gather(long long n, const unsigned long long* __restrict__ src,
                             const unsigned* __restrict__ val, unsigned long long* __restrict__ dst) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dst[t] = src[val[t]];
}

struct PwaLook {
  int nov;
  const long long* pair_ring;
  long long nrings;
  const long long* ring_off;
  const double* xy;
  int nb;
  const unsigned long long* bkx;  // base vertices sorted by (x, y)
  const unsigned long long* bky;
  const unsigned* bval;
  long long nc;                   // candidates sorted by (pair, x, y)
  const unsigned long long* ckp;
  const unsigned long long* ckx;
  const unsigned long long* cky;
  const unsigned* cval;
  PwaCand C;
};

// the ring and pair that own output vertex v
__device__ __forceinline__ void pwa_owner(const PwaLook& L, long long v, long long* ring, int* pair) {
  long long lo = 0, hi = L.nrings;
  while (hi - lo > 1) {
    const long long m = (lo + hi) >> 1;
    if (L.ring_off[m] <= v) lo = m;
    else hi = m;
  }
  *ring = lo;
  int a = 0, b = L.nov;  // last pair with pair_ring <= ring (and rings to own)
  while (b - a > 1) {
    const int m = (a + b) >> 1;
    if (L.pair_ring[m] <= lo) a = m;
    else b = m;
  }
  while (a + 1 < L.nov && L.pair_ring[a + 1] <= lo) ++a;
  *pair = a;
}

__global__ void k_pwa_tape(PwaLook L, long long nv, int4* __restrict__ tape) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  long long ring;
  int pair;
  pwa_owner(L, v, &ring, &pair);
  const unsigned long long qx = dkey(L.xy[2 * v]), qy = dkey(L.xy[2 * v + 1]);
  int4 t = make_int4(-1, 0, 0, 0);
  {
    int lo = 0, hi = L.nb;
    while (lo < hi) {
      const int m = (lo + hi) >> 1;
      if (L.bkx[m] < qx || (L.bkx[m] == qx && L.bky[m] < qy)) lo = m + 1;
      else hi = m;
    }
    if (lo < L.nb && L.bkx[lo] == qx && L.bky[lo] == qy) t = make_int4(0, (int)L.bval[lo], 0, 0);
  }
  if (t.x < 0) {
    const unsigned long long qp = (unsigned long long)pair;
    long long lo = 0, hi = L.nc;
    while (lo < hi) {
      const long long m = (lo + hi) >> 1;
      const bool less = L.ckp[m] < qp || (L.ckp[m] == qp && (L.ckx[m] < qx ||
                                                            (L.ckx[m] == qx && L.cky[m] < qy)));
      if (less) lo = m + 1;
      else hi = m;
    }
    if (lo < L.nc && L.ckp[lo] == qp && L.ckx[lo] == qx && L.cky[lo] == qy) {
      int pr;
      int4 d;
      pwa_decode(L.C, (long long)L.cval[lo], &pr, &d);
      t = d.x == 1 ? make_int4(1, d.y, 0, 0) : make_int4(2, d.y, d.z, 0);
    }
  }
  tape[v] = t;
}

__global__ void k_pwa_backward(PwaLook L, long long nv, const int4* __restrict__ tape,
                               const double* __restrict__ gA, const double* __restrict__ b,
                               const double* __restrict__ cxy, const long long* __restrict__ coff,
                               double* __restrict__ gb, double* __restrict__ gc) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  long long ring;
  int pair;
  pwa_owner(L, v, &ring, &pair);
  const long long s = L.ring_off[ring], e = L.ring_off[ring + 1];
  const long long ip = (v + 1 == e) ? s : v + 1, im = (v == s) ? e - 1 : v - 1;
  const double g = gA[pair];
  const double gx = 0.5 * g * (L.xy[2 * ip + 1] - L.xy[2 * im + 1]);
  const double gy = 0.5 * g * (L.xy[2 * im] - L.xy[2 * ip]);
  const int4 t = tape[v];
  const int nb = L.nb;
  const long long c0 = coff[pair];
  const int nc = (int)(coff[pair + 1] - c0);
  const double* c = cxy + 2 * c0;
  double* gcp = gc + 2 * c0;
  if (t.x == 0) {
    atomicAdd(&gb[2 * t.y], gx);
    atomicAdd(&gb[2 * t.y + 1], gy);
  } else if (t.x == 1) {
    atomicAdd(&gcp[2 * t.y], gx);
    atomicAdd(&gcp[2 * t.y + 1], gy);
  } else if (t.x == 2) {
    const int i1 = t.y, i2 = (t.y + 1) % nb, j1 = t.z, j2 = (t.z + 1) % nc;
    const double b1x = b[2 * i1], b1y = b[2 * i1 + 1], b2x = b[2 * i2], b2y = b[2 * i2 + 1];
    const double c1x = c[2 * j1], c1y = c[2 * j1 + 1], c2x = c[2 * j2], c2y = c[2 * j2 + 1];
    const double A1 = (c1x - b1x) * (c2y - b1y) - (c1y - b1y) * (c2x - b1x);
    const double A2 = (c1x - b2x) * (c2y - b2y) - (c1y - b2y) * (c2x - b2x);
    const double d = A1 - A2;
    const double al = A1 / d;
    const double ga = gx * (b2x - b1x) + gy * (b2y - b1y);
    const double k1 = -A2 / (d * d) * ga, k2 = A1 / (d * d) * ga;
    atomicAdd(&gb[2 * i1], (1.0 - al) * gx + k1 * (c1y - c2y));
    atomicAdd(&gb[2 * i1 + 1], (1.0 - al) * gy + k1 * (c2x - c1x));
    atomicAdd(&gb[2 * i2], al * gx + k2 * (c1y - c2y));
    atomicAdd(&gb[2 * i2 + 1], al * gy + k2 * (c2x - c1x));
    atomicAdd(&gcp[2 * j1], k1 * (c2y - b1y) + k2 * (c2y - b2y));
    atomicAdd(&gcp[2 * j1 + 1], k1 * (b1x - c2x) + k2 * (b2x - c2x));
    atomicAdd(&gcp[2 * j2], k1 * (b1y - c1y) + k2 * (b2y - c1y));
    atomicAdd(&gcp[2 * j2 + 1], k1 * (c1x - b1x) + k2 * (c1x - b2x));
  }
}

}  // namespace

int PairwiseRunner::area(double* d_area, cudaStream_t st) {
  if (!valid) return pl_.fail(kEInput, "no pairwise result to take the area of");
  if (np <= 0) return kOk;
  ::sbc::KProbe kp_("k_pwa_area", st, 16.0 * (double)total_verts);
  k_pwa_area<<<grid_for(np, 128), 128, 0, st>>>(np, pair_ring, ring_off, xy, status, d_area);
  return kOk;
}

int PairwiseRunner::backward(const double* d_bxy, const double* d_cxy, const long long* d_coff,
                             const double* d_gA, double* d_gb, double* d_gc, cudaStream_t st) {
  if (!valid) return pl_.fail(kEInput, "no pairwise result to differentiate");
  BufferPool& pool = pl_.pool();
  const int nb = last_nb_;
  const long long totalC = last_totalC_, nh = last_nh_, nfb = (long long)fb_rec_.size();
  cudaMemsetAsync(d_gb, 0, sizeof(double) * 2 * nb, st);
  if (totalC > 0) cudaMemsetAsync(d_gc, 0, sizeof(double) * 2 * totalC, st);
  if (np <= 0 || total_verts == 0) {
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise backward");
    return kOk;
  }
  // base vertices sorted by (x, y): by y, then stably by x
  auto* bkx = (unsigned long long*)pool.get("pwa_bkx", sizeof(unsigned long long) * (nb + 1));
  auto* bky = (unsigned long long*)pool.get("pwa_bky", sizeof(unsigned long long) * (nb + 1));
  auto* bk2 = (unsigned long long*)pool.get("pwa_bk2", sizeof(unsigned long long) * (nb + 1));
  auto* bk3 = (unsigned long long*)pool.get("pwa_bk3", sizeof(unsigned long long) * (nb + 1));
  auto* bval = (unsigned*)pool.get("pwa_bval", sizeof(unsigned) * (nb + 1));
  auto* bval2 = (unsigned*)pool.get("pwa_bval2", sizeof(unsigned) * (nb + 1));
  const long long nc = totalC + nh + nfb;
  auto* ckx = (unsigned long long*)pool.get("pwa_ckx", sizeof(unsigned long long) * (nc + 1));
  auto* cky = (unsigned long long*)pool.get("pwa_cky", sizeof(unsigned long long) * (nc + 1));
  auto* ckp = (unsigned long long*)pool.get("pwa_ckp", sizeof(unsigned long long) * (nc + 1));
  auto* ck2 = (unsigned long long*)pool.get("pwa_ck2", sizeof(unsigned long long) * (nc + 1));
  auto* ck3 = (unsigned long long*)pool.get("pwa_ck3", sizeof(unsigned long long) * (nc + 1));
  auto* cval = (unsigned*)pool.get("pwa_cval", sizeof(unsigned) * (nc + 1));
  auto* cval2 = (unsigned*)pool.get("pwa_cval2", sizeof(unsigned) * (nc + 1));
  void* rscr = pool.get("pwa_rscr", radix_scratch_bytes((nc > nb ? nc : nb) + 1));
  int4* fbr = (int4*)pool.get("pwa_fbrec", sizeof(int4) * (nfb + 1));
  double* fbxy = (double*)pool.get("pwa_fbxy", sizeof(double) * 2 * (nfb + 1));
  int4* tape = (int4*)pool.get("pwa_tape", sizeof(int4) * (total_verts + 1));
  const PwHit* hits = (const PwHit*)pool.get("pw_hits_grouped", sizeof(PwHit) * (nh + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (pairwise backward)");
  if (nfb) {
    std::vector<int4> h(nfb);
    for (long long r = 0; r < nfb; ++r)
      h[r] = make_int4(fb_rec_[r][0], fb_rec_[r][1], fb_rec_[r][2], fb_rec_[r][3]);
    cudaMemcpyAsync(fbr, h.data(), sizeof(int4) * nfb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(fbxy, fb_xy_.data(), sizeof(double) * 2 * nfb, cudaMemcpyHostToDevice, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise backward");
  }
  {
    ::sbc::KProbe kp_("k_pwa_base_keys", st, 36.0 * nb);
    k_pwa_base_keys<<<grid_for(nb, 256), 256, 0, st>>>(nb, d_bxy, bkx, bky, bval);
  }
  cudaMemcpyAsync(bk2, bky, sizeof(unsigned long long) * nb, cudaMemcpyDeviceToDevice, st);
  radix_sort_u64(bk2, bval, bk3, bval2, nb, rscr, st);
  k_pwa_gather<<<grid_for(nb, 256), 256, 0, st>>>(nb, bkx, bval, bk2);
  radix_sort_u64(bk2, bval, bk3, bval2, nb, rscr, st);
  // bk2: x keys in (x, y) order; bk3: the y keys in that order
  k_pwa_gather<<<grid_for(nb, 256), 256, 0, st>>>(nb, bky, bval, bk3);
  PwaCand C{np, d_coff, totalC, d_cxy, nh, hits, nb, d_bxy, nfb, fbr, fbxy};
  {
    ::sbc::KProbe kp_("k_pwa_cand", st, 40.0 * (double)nc);
    k_pwa_cand<<<grid_for(nc, 256), 256, 0, st>>>(C, nc, ckx, cky, ckp, cval);
  }
  // by y, by x, by pair (stable): sorted by (pair, x, y), ties in candidate order
  cudaMemcpyAsync(ck2, cky, sizeof(unsigned long long) * nc, cudaMemcpyDeviceToDevice, st);
  radix_sort_u64(ck2, cval, ck3, cval2, nc, rscr, st);
  k_pwa_gather<<<grid_for(nc, 256), 256, 0, st>>>(nc, ckx, cval, ck2);
  radix_sort_u64(ck2, cval, ck3, cval2, nc, rscr, st);
  k_pwa_gather<<<grid_for(nc, 256), 256, 0, st>>>(nc, ckp, cval, ck2);
  radix_sort_u64(ck2, cval, ck3, cval2, nc, rscr, st);
  // ck2 now holds pair keys in order; gather x and y keys in the same order
  k_pwa_gather<<<grid_for(nc, 256), 256, 0, st>>>(nc, ckx, cval, ck3);
  k_pwa_gather<<<grid_for(nc, 256), 256, 0, st>>>(nc, cky, cval, ckx);
  // (ckx reused for sorted y keys: the unsorted x keys are no longer needed)
  const PwaLook L{np, pair_ring, total_rings, ring_off, xy, nb, bk2, bk3, bval, nc, ck2, ck3, ckx,
                  cval, C};
  {
    ::sbc::KProbe kp_("k_pwa_tape", st, 48.0 * (double)total_verts);
    k_pwa_tape<<<grid_for(total_verts, 256), 256, 0, st>>>(L, total_verts, tape);
  }
  {
    ::sbc::KProbe kp_("k_pwa_backward", st, 64.0 * (double)total_verts);
    k_pwa_backward<<<grid_for(total_verts, 256), 256, 0, st>>>(L, total_verts, tape, d_gA, d_bxy,
                                                               d_cxy, d_coff, d_gb, d_gc);
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "pairwise backward");
  return kOk;
}

}  // namespace sbc
