// sbc_pwpair.cuh -- one pair's rows A9-A18 (src/clip.cpp:368-695,
// foster/polyclip.h:337-787) by one warp, its lanes sharing the per-record,
// per-run and per-slot steps: the overlay's merged arrays in full, the base's
// only where intersections are (a stretch of plain base vertices is one run
// node of the linked list, sbc_serial.cuh).  Used by the one-base-many-
// overlays engine (sbc_pairwise.cu) and by the batched small-pair engine
// (sbc_batch.cu); each supplies the pointInPoly functor of the base side.
#pragma once

#include <climits>

#include "sbc_pairops.cuh"
#include "sbc_serial.cuh"

namespace sbc {
namespace {

constexpr unsigned kFullMask = 0xffffffffu;
enum { PS_FALLBACK = 4 };

// one unique hit of a pair: base edge b, overlay edge j, the classifier's
// type, the first-emission key and lineSegmentIntersection's alpha and beta
struct PwHit {
  int pair, b, j, type;
  unsigned long long key;  // first emission
  double al, bt;           // lineSegmentIntersection's alpha and beta
};

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
  int* mid;  // PwMid between the steps when they run as separate kernels
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
  w.mid = cv.take<int>(8);
  return w;
}

__host__ __device__ __forceinline__ size_t pw_arena_bytes(int nb, int nc, int K, int pass) {
  Carver cv{nullptr, 0};
  pw_carve(cv, pw_caps(nb, nc, K, pass));
  return (cv.off + 255) & ~(size_t)255;
}

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
template <class Pip>
__device__ int pw_label_trace(SerialArgs& a, const Pip& pipP) {
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
  // each lane takes compare-exchange pairs (m, m + j): every lane works in
  // every round
  for (int k = 2; k <= np; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int q = lane; q < (np >> 1); q += 32) {
        const int m = ((q & ~(j - 1)) << 1) | (q & (j - 1)), l = m | j;
        const unsigned long long x = scr[m], y = scr[l];
        if ((x > y) == ((m & k) == 0)) {
          scr[m] = y;
          scr[l] = x;
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
// The scalars the two halves of the warp back end share.
struct PwMid {
  int nr, knd, nB, nQ;  // base runs, non-degenerate base records, slot counts
  int pn, qn, nruns;    // after the lists: node counts of P and Q, P's run nodes
};

__device__ __forceinline__ void pw_mid_store(const PwMid& m, int* d) {
  d[0] = m.nr;
  d[1] = m.knd;
  d[2] = m.nB;
  d[3] = m.nQ;
  d[4] = m.pn;
  d[5] = m.qn;
  d[6] = m.nruns;
}

__device__ __forceinline__ PwMid pw_mid_load(const int* d) {
  return PwMid{d[0], d[1], d[2], d[3], d[4], d[5], d[6]};
}

// Rows A9-A14: records, counts, alpha order, merged arrays, initial labels.
__device__ int pw_clip_head(const double* b, int nb, const double* c, int nc, const PwHit* H,
                            const PwCaps& cp, PwWork& w, PwMid* mid) {
  const int lane = threadIdx.x & 31;
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
    const int bi2 = bi + 1 == nb ? 0 : bi + 1;
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
  *mid = PwMid{nr, knd, nB, nQ, 0, 0, 0};
  return PS_OK;
}

// Row A15 from the head's arrays: the linked lists (mid receives their node
// counts and P's run nodes).
__device__ int pw_clip_lists(const double* b, int nb, const double* c, int nc, const PwCaps& cp,
                             PwWork& w, PwMid* mid) {
  const int lane = threadIdx.x & 31;
  const int nr = mid->nr, knd = mid->knd, nB = mid->nB, nQ = mid->nQ;
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
  mid->pn = P.n;
  mid->qn = Q.n;
  mid->nruns = nruns;
  return PS_OK;
}

// Rows A16-A18 from the lists: labelling, tracing, clean-up and the rings out.
template <class Pip>
__device__ int pw_clip_trace(const double* b, int nb, const double* c, int nc, const PwCaps& cp,
                             PwWork& w, const PwMid& mid, Pip pip, int unite, int* nrings_out,
                             int* nverts_out) {
  const int lane = threadIdx.x & 31;
  const int nB = mid.nB, nQ = mid.nQ;
  Pool& P = w.P;
  Pool& Q = w.Q;
  P.n = mid.pn;
  Q.n = mid.qn;
  P.rxy = b;
  w.R.n = 0;
  const int nruns = mid.nruns;
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
  a.unite = unite;
  *a.nrings = 0;
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

// One pair, rows A9-A18, by the calling warp (all 32 lanes): base b (nb
// vertices), overlay c (nc), its K unique hits H in the reference's order
// (base id, then first emission), a pointInPoly functor for the base side
// (pip: its runIds / nruns are set by the tail), union or intersection.
// Returns PS_OK with the rings in w.roff / w.rxy, PS_FALLBACK where the
// sparse back end does not follow the arrays (the caller clips the pair
// another way), PS_UNDEF or PS_CAP.  The head, the lists and the trace may
// also run as separate kernels, PwMid carried between them.
template <class Pip>
__device__ int pw_clip_core(const double* b, int nb, const double* c, int nc, const PwHit* H,
                            const PwCaps& cp, PwWork& w, Pip pip, int unite, int* nrings_out,
                            int* nverts_out) {
  PwMid mid;
  int st = pw_clip_head(b, nb, c, nc, H, cp, w, &mid);
  if (st == PS_OK) st = pw_clip_lists(b, nb, c, nc, cp, w, &mid);
  if (st != PS_OK) return st;
  return pw_clip_trace(b, nb, c, nc, cp, w, mid, pip, unite, nrings_out, nverts_out);
}

}  // namespace
}  // namespace sbc
