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
#include "sbc_pwpair.cuh"
#include "sbc_serial.cuh"

namespace sbc {

namespace {

constexpr int kPwMaxOverlay = 16384;  // larger overlays go to the pair pipeline
constexpr int kPwMaxCells = 1 << 14;  // an overlay edge box over more cells: pair pipeline
constexpr int kPwLongCells = 64;      // base edges over more cells per axis skip the grid
constexpr int kPwPrepThreads = 256;
constexpr int kPwPairBlock = 64;

enum { PW_FAST = 0, PW_FALLBACK = 1, PW_INPUT = 2 };

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

__device__ int pw_clip_pair(const PwPairArgs& A, int p, const PwCaps& cp, PwWork& w, int* nrings_out,
                            int* nverts_out) {
  const long long o = A.coff[p];
  const int nc = (int)(A.coff[p + 1] - o);
  return pw_clip_core(A.b, A.nb, A.cxy + 2 * o, nc, A.hits + A.hstart[p], cp, w, A.pip, A.unite,
                      nrings_out, nverts_out);
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

// one warp per pair: each ring's shoelace terms summed lane by lane, the
// lanes' sums combined in a fixed order (the area does not depend on the
// launch shape)
__global__ void k_pwa_area(int nov, const long long* __restrict__ pair_ring,
                           const long long* __restrict__ ring_off, const double* __restrict__ xy,
                           const int* __restrict__ status, double* __restrict__ area) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if ((t >> 5) >= nov) return;
  const int p = (int)(t >> 5);
  double a = 0.0;
  if (status[p] == SBC_OK) {
    for (long long r = pair_ring[p]; r < pair_ring[p + 1]; ++r) {
      const long long s = ring_off[r], e = ring_off[r + 1];
      double s2 = 0.0;
      for (long long i = s + lane; i < e; i += 32) {
        const long long j = (i + 1 == e) ? s : i + 1;
        s2 = dadd(s2, dsub(dmul(xy[2 * i], xy[2 * j + 1]), dmul(xy[2 * j], xy[2 * i + 1])));
      }
      for (int o = 16; o > 0; o >>= 1) s2 = dadd(s2, __shfl_xor_sync(0xffffffffu, s2, o));
      a = dadd(a, dmul(0.5, s2));
    }
  }
  if (lane == 0) area[p] = a;
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
  k_pwa_area<<<grid_for(32LL * np, 128), 128, 0, st>>>(np, pair_ring, ring_off, xy, status, d_area);
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
