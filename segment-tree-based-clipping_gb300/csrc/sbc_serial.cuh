// sbc_serial.cuh -- the exact single-thread linked-list back end
// (copyToLinkedList src/clip.cpp:606-695, labelIntersections2
// foster/polyclip.h:337-709, createResult2 :717-759, cleanUpResult2
// :767-787) over index-linked node pools.  Device functions only; the pools
// may live in global or shared memory.  Used by the pair pipeline when its
// data-parallel back end cannot follow an input (sbc_back.cu) and by the
// batched small-pair engine (sbc_batch.cu).
#pragma once

#include "sbc_internal.cuh"

namespace sbc {
namespace {

enum { L_NONE = 0, L_CROSSING, L_BOUNCING, L_LEFT_ON, L_RIGHT_ON, L_ON_ON, L_ON_LEFT, L_ON_RIGHT,
       L_DCROSS, L_DBOUNCE };
enum { EX_EXIT = 0, EX_ENTRY = 1, EX_NEITHER = 2 };

// ================================================================ serial emulation
// A literal restatement of copyToLinkedList + labelIntersections2 +
// createResult2 + cleanUpResult2 over index-linked pools (one thread).
struct Pool {
  double *x, *y;
  int *next, *prev, *nb, *label, *enex;
  unsigned char *source, *isect;
  int n, cap;
  // optional: where each node's coordinates come from (ring nodes: side << 30
  // | merged slot, list nodes: their merged slot; -1 unknown).  Null when the
  // caller does not track it.
  int* src = nullptr;
  // optional run nodes: a node v with run[v] > 0 stands for run[v] + 1
  // consecutive plain vertices rv0[v] .. rv0[v] + run[v] of the interleaved
  // coordinate array rxy (no labels, not intersections); x/y hold the first.
  // Null when every node is one vertex.
  int* run = nullptr;
  int* rv0 = nullptr;
  const double* rxy = nullptr;
};

__device__ __forceinline__ bool is_run(const Pool& p, int v) { return p.run && p.run[v] > 0; }
// coordinates of the last vertex of node v (the one next to its successor)
__device__ __forceinline__ double last_x(const Pool& p, int v) {
  return is_run(p, v) ? p.rxy[2 * (p.rv0[v] + p.run[v])] : p.x[v];
}
__device__ __forceinline__ double last_y(const Pool& p, int v) {
  return is_run(p, v) ? p.rxy[2 * (p.rv0[v] + p.run[v]) + 1] : p.y[v];
}

struct SerialArgs {
  Pool P, Q, R;
  int* rroot;
  int rcap;
  int* nrings;
  unsigned char *splitP, *splitQ, *crossP, *crossQ;
  int bSize, cSize, cStart, nB, nQ;
  const double *bP, *cP, *ixB, *ixC;
  const int *alB, *nbC, *labB, *labC;
  int* status;   // 0 ok, 2 undefined, 3 capacity
  int rfull = 0;  // set when the ring pool ran out of nodes
  int unite = 0;  // union instead of intersection (foster/polyclip.h:39 UNION)
  // components (Foster's multi-component polygons): the successor of each
  // source vertex within its component (null: one ring), and the list node of
  // each component's first vertex, ending with the node count (the caller's;
  // null with one ring: root 0)
  const int* bnx = nullptr;
  const int* cnx = nullptr;
  int* rootsP = nullptr;
  int* rootsQ = nullptr;
  int nrP = 1, nrQ = 1;
};

__device__ __forceinline__ int sroot(const SerialArgs& a, int s, int k) {
  const int* r = s == 0 ? a.rootsP : a.rootsQ;
  return r ? r[k] : 0;
}

__device__ int pnew(Pool& p, double x, double y) {
  if (p.n >= p.cap) return -1;
  int v = p.n++;
  if (p.src) p.src[v] = -1;
  if (p.run) p.run[v] = 0;
  p.x[v] = x;
  p.y[v] = y;
  p.next[v] = p.prev[v] = v;
  p.nb[v] = -1;
  p.label[v] = L_NONE;
  p.enex[v] = EX_NEITHER;
  p.source[v] = 0;
  p.isect[v] = 0;
  return v;
}

__device__ void pinsert_after(Pool& p, int V, int curr) {
  curr = p.next[curr];
  p.next[p.prev[curr]] = V;
  p.prev[V] = p.prev[curr];
  p.next[V] = curr;
  p.prev[curr] = V;
}

// winding-number step of pointInPoly (foster/polygon.h:427-448) for the edge
// (x0,y0)-(x1,y1); the winding number is the (order-free) sum of the steps
// one edge's step of pointInPoly (foster/polygon.h:427-448); the compares
// run on integer order keys (okey: the same decisions as on the doubles, at
// the integer rate), the orientation test in FP64
__device__ __forceinline__ int pip_step(double x0, double y0, double x1, double y1, double rx,
                                        double ry) {
  const long long ky0 = okey(y0), ky1 = okey(y1), kry = okey(ry);
  if ((ky0 < kry) != (ky1 < kry)) {
    const long long kx0 = okey(x0), kx1 = okey(x1), krx = okey(rx);
    const int d = 2 * (ky1 > ky0) - 1;
    if (kx0 >= krx) {
      if (kx1 > krx) return d;
      if ((area3(x0, y0, x1, y1, rx, ry) > 0) == (ky1 > ky0)) return d;
    } else if (kx1 > krx) {
      if ((area3(x0, y0, x1, y1, rx, ry) > 0) == (ky1 > ky0)) return d;
    }
  }
  return 0;
}

__device__ int ppip(const Pool& p, int root, double rx, double ry) {
  int w = 0, one = root;
  do {
    int two = p.next[one];
    w += pip_step(p.x[one], p.y[one], p.x[two], p.y[two], rx, ry);
    one = two;
  } while (one != root);
  return (w % 2) != 0;
}

__device__ int rnew(SerialArgs& a) {
  if (*a.nrings >= a.rcap) return -1;
  int r = (*a.nrings)++;
  a.rroot[r] = -1;
  return r;
}

__device__ int radd(SerialArgs& a, int r, double x, double y, int prov = -1) {
  int v = pnew(a.R, x, y);
  if (v < 0) {
    a.rfull = 1;
    return -1;
  }
  if (a.R.src) a.R.src[v] = prov;
  int root = a.rroot[r];
  if (root < 0) {
    a.rroot[r] = v;
  } else {
    a.R.prev[v] = a.R.prev[root];
    a.R.next[v] = root;
    a.R.next[a.R.prev[root]] = v;
    a.R.prev[root] = v;
  }
  return 0;
}

// every vertex of node v of p to ring r, in walking order (a run node's
// vertices backwards when walking backwards)
__device__ int radd_node(SerialArgs& a, int r, const Pool& p, int v, bool forward, int prov) {
  if (!is_run(p, v)) return radd(a, r, p.x[v], p.y[v], prov);
  const int n = p.run[v];
  for (int t = 0; t <= n; ++t) {
    const int u = p.rv0[v] + (forward ? t : n - t);
    if (radd(a, r, p.rxy[2 * u], p.rxy[2 * u + 1])) return -1;
  }
  return 0;
}

__device__ int rcopy(SerialArgs& a, const Pool& p, int root) {
  int r = rnew(a);
  if (r < 0) return -1;
  int v = root;
  do {
    const int prov = (p.src && p.src[v] >= 0) ? (((&p == &a.Q) ? 1 : 0) << 30) | p.src[v] : -1;
    if (radd_node(a, r, p, v, true, prov)) return -1;
    v = p.next[v];
  } while (v != root);
  return 0;
}

__device__ void tog(int* s) {
  if (*s == EX_ENTRY) *s = EX_EXIT;
  else if (*s == EX_EXIT) *s = EX_ENTRY;
}

// copyToLinkedList (src/clip.cpp:606-695) for one side, one component after
// another: each walked from its first vertex and closed on it as the
// reference's single ring is; the lists wrap within their component.  O:
// the base's pool when building the overlay's (neighbour links), else null.
__device__ int ser_build_side(Pool& P, Pool* O, const double* poly, int n, const int* nx,
                              int* roots, int nr, const double* ix, int nS, const int* alpha,
                              const int* nbr, const int* lab) {
  int vs = 0;
  for (int k = 0; k < nr; ++k) {
    int ve = vs + 1;
    while (ve < n && (nx ? nx[ve - 1] : ve) == ve) ++ve;
    const int lo = roots ? roots[k] : 0, hi = roots ? roots[k + 1] : nS;
    int i = lo;
    for (int ii = vs; ii <= ve; ++ii) {
      const bool last = ii == ve;
      const int sv = last ? vs : ii;
      const double vx = poly[2 * sv], vy = poly[2 * sv + 1];
      const long long kvx = okey(vx), kvy = okey(vy);  // compares on order keys
      for (;;) {
        const int sl = i == hi ? lo : i;
        if (i > hi || (okey(ix[2 * sl]) == kvx && okey(ix[2 * sl + 1]) == kvy)) break;
        if (i >= hi) return 2;
        const int v = pnew(P, ix[2 * i], ix[2 * i + 1]);
        if (v < 0) return 3;
        P.label[v] = lab[i];
        P.isect[v] = 1;
        if (O) {
          const int t = nbr[i] - 1;
          if (t < 0 || t >= O->n) return 2;
          P.nb[v] = t;
          O->nb[t] = v;
        }
        i++;
      }
      if (i > hi || (!last && i >= hi)) return 2;  // more vertices than the component's slots
      if (!last) {
        const int v = pnew(P, vx, vy);
        if (v != i) return 2;
        P.source[v] = 1;
        P.label[v] = lab[i];
        if (!O) {
          if (alpha[i] != -100) P.isect[v] = 1;
        } else if (nbr[i] != -100) {
          const int t = nbr[i] - 1;
          if (t < 0 || t >= O->n) return 2;
          P.isect[v] = 1;
          P.nb[v] = t;
          O->nb[t] = v;
        }
      }
      i++;
    }
    for (int v = lo; v < hi; ++v) {
      P.next[v] = v + 1 == hi ? lo : v + 1;
      P.prev[v] = v == lo ? hi - 1 : v - 1;
    }
    vs = ve;
  }
  return P.n == nS ? 0 : 2;
}

__device__ int ser_build(SerialArgs& a) {
  const int r = ser_build_side(a.P, nullptr, a.bP, a.bSize, a.bnx, a.rootsP, a.nrP, a.ixB, a.nB,
                               a.alB, nullptr, a.labB);
  if (r) return r;
  return ser_build_side(a.Q, &a.P, a.cP + 2 * a.cStart, a.cSize, a.cnx, a.rootsQ, a.nrQ, a.ixC,
                        a.nQ, nullptr, a.nbC, a.labC);
}

__device__ Pool& side(SerialArgs& a, int s) { return s == 0 ? a.P : a.Q; }

__device__ int ser_non_isect_vertex(SerialArgs& a, int s, int root) {
  Pool& p = side(a, s);
  Pool& o = side(a, 1 - s);
  int V = root;
  do {
    if (!p.isect[V]) return V;
    V = p.next[V];
  } while (V != root);
  V = root;
  do {
    int nbV = p.nb[V], nbN = p.nb[p.next[V]];
    if (nbV < 0) return -2;
    if (nbN != o.prev[nbV] && nbN != o.next[nbV]) {
      double mx = 0.5 * (p.x[V] + p.x[p.next[V]]);
      double my = 0.5 * (p.y[V] + p.y[p.next[V]]);
      mx = dmul(0.5, dadd(p.x[V], p.x[p.next[V]]));
      my = dmul(0.5, dadd(p.y[V], p.y[p.next[V]]));
      int T = pnew(p, mx, my);
      if (T < 0) return -3;
      pinsert_after(p, T, V);
      return T;
    }
    V = p.next[V];
  } while (V != root);
  return -2;
}

// pointInPoly against side s: the pool's own edges, or, for a pool with run
// nodes, the caller's run-aware test
struct NoRunPip {
  __device__ int operator()(SerialArgs& a, int root, double rx, double ry) const {
    return ppip(a.P, root, rx, ry);
  }
};

template <class PipP>
__device__ int pip_side(SerialArgs& a, int s, int root, double rx, double ry, const PipP& pp) {
  Pool& p = side(a, s);
  if (p.run) return pp(a, root, rx, ry);
  return ppip(p, root, rx, ry);
}

// pointInPoly against every component of side s: each one containing the
// point toggles the answer (lib/optimizedFostersAlgorithm/polyclip.cpp:
// 503-507, :593-595); one component is the reference's test
template <class PipP>
__device__ int pip_all(SerialArgs& a, int s, double rx, double ry, const PipP& pp) {
  const int nr = s == 0 ? a.nrP : a.nrQ;
  int in = 0;
  for (int k = 0; k < nr; ++k) in ^= pip_side(a, s, sroot(a, s, k), rx, ry, pp);
  return in;
}

// noCrossingVertex(UNION) (foster/polygon.h:465-475) of the component at root
__device__ bool no_cross(SerialArgs& a, const Pool& p, int root) {
  int V = root;
  do {
    if (p.isect[V] && (p.label[V] == L_CROSSING || p.label[V] == L_DCROSS)) return false;
    if (a.unite && p.isect[V] && (p.label[V] == L_BOUNCING || p.label[V] == L_DBOUNCE))
      return false;
    V = p.next[V];
  } while (V != root);
  return true;
}

__device__ bool all_on_on(const Pool& p, int root) {
  int V = root;
  do {
    if (p.label[V] != L_ON_ON) return false;
    V = p.next[V];
  } while (V != root);
  return true;
}

// labelIntersections2 (foster/polyclip.h:337-709) over every component of
// both sides, in the order of Foster's multi-component code (lib/
// optimizedFostersAlgorithm/polyclip.cpp:335-780): chains, interior and
// identical components, entry/exit flags per component; then createResult2
// (:717-759) from P's components in order.  A component's "no crossing"
// and "all ON_ON" tests are repeated where needed: no label they read
// changes between the steps.
template <class PipP>
__device__ int ser_label_trace_t(SerialArgs& a, const PipP& pipP) {
  Pool& P = a.P;
  Pool& Q = a.Q;
  // (2) chains
  for (int k = 0; k < a.nrP; ++k) {
    const int root = sroot(a, 0, k);
    int V = root;
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
    } while (V != root);
  }
  // (3.5) components without crossings: inside the other side (or outside,
  // for the union), copied whole
  for (int s = 0; s < 2; ++s)
    for (int k = 0; k < (s == 0 ? a.nrP : a.nrQ); ++k) {
      Pool& p = side(a, s);
      const int root = sroot(a, s, k);
      if (!no_cross(a, p, root) || all_on_on(p, root)) continue;
      double px = 0, py = 0;
      int found = 0, V = root;
      do {
        if (!p.isect[V]) {
          px = p.x[V];
          py = p.y[V];
          found = 1;
          break;
        }
        V = p.next[V];
      } while (V != root);
      if (!found) {
        Pool& o = side(a, 1 - s);
        V = root;
        do {
          int nbV = p.nb[V], nbN = p.nb[p.next[V]];
          if (nbV < 0) return 2;
          if (nbN != o.prev[nbV] && nbN != o.next[nbV]) {
            px = dmul(0.5, dadd(p.x[V], p.x[p.next[V]]));
            py = dmul(0.5, dadd(p.y[V], p.y[p.next[V]]));
            found = 1;
            break;
          }
          V = p.next[V];
        } while (V != root);
        if (!found) return 2;
      }
      if (pip_all(a, 1 - s, px, py, pipP) ^ a.unite)
        if (rcopy(a, p, root)) return 3;
    }
  // identical components (polyclip.cpp:516-538): P's component k is added
  // when the identical component of Q holding its root's neighbour is a hole
  // exactly when k is (inside an odd number of its side's other components)
  for (int k = 0; k < a.nrP; ++k) {
    const int rk = sroot(a, 0, k);
    if (!no_cross(a, P, rk) || !all_on_on(P, rk)) continue;
    int holeP = 0;
    for (int j = 0; j < a.nrP; ++j)
      if (j != k) holeP ^= pip_side(a, 0, sroot(a, 0, j), P.x[rk], P.y[rk], pipP);
    const int target = P.nb[rk];
    for (int m = 0; m < a.nrQ; ++m) {
      const int rm = sroot(a, 1, m);
      if (!no_cross(a, Q, rm) || !all_on_on(Q, rm)) continue;
      int V = rm, found = 0;
      do {
        if (V == target) found = 1;
        V = Q.next[V];
      } while (V != rm);
      if (!found) continue;
      int holeQ = 0;
      for (int j = 0; j < a.nrQ; ++j)
        if (j != m) holeQ ^= pip_side(a, 1, sroot(a, 1, j), Q.x[rm], Q.y[rm], pipP);
      if (holeP == holeQ && rcopy(a, P, rk)) return 3;
      break;
    }
  }
  // (4)
  for (int s = 0; s < 2; ++s)
    for (int k = 0; k < (s == 0 ? a.nrP : a.nrQ); ++k) {
      Pool& p = side(a, s);
      if (no_cross(a, p, sroot(a, s, k))) continue;
      unsigned char* split = s == 0 ? a.splitP : a.splitQ;
      unsigned char* cross = s == 0 ? a.crossP : a.crossQ;
      int V = ser_non_isect_vertex(a, s, sroot(a, s, k));
      if (V == -3) return 3;
      if (V < 0) return 2;
      int status = EX_ENTRY;
      if (pip_all(a, 1 - s, p.x[V], p.y[V], pipP)) tog(&status);
      int first = 1, I = V;
      do {
        if (p.isect[I]) {
          if (p.label[I] == L_CROSSING) {
            p.enex[I] = status;
            tog(&status);
          }
          if (p.label[I] == L_BOUNCING && ((status == EX_EXIT) ^ a.unite)) split[I] = 1;
          if (p.label[I] == L_DCROSS) {
            p.enex[I] = status;
            if (first) {
              if ((status == EX_EXIT) ^ a.unite) p.label[I] = L_CROSSING;
              first = 0;
            } else {
              if ((status == EX_ENTRY) ^ a.unite) p.label[I] = L_CROSSING;
              first = 1;
              tog(&status);
            }
          }
          if (p.label[I] == L_DBOUNCE) {
            p.enex[I] = status;
            if (first) {
              if ((status == EX_EXIT) ^ a.unite) cross[I] = 1;
              first = 0;
            } else {
              if ((status == EX_ENTRY) ^ a.unite) cross[I] = 1;
              first = 1;
            }
            tog(&status);
          }
        }
        I = p.next[I];
      } while (I != V);
    }
  // (5) split pairs
  {
    int nP0 = P.n;
    for (int IP = 0; IP < nP0; ++IP) {
      if (!a.splitP[IP]) continue;
      int IQ = P.nb[IP];
      if (IQ < 0 || !a.splitQ[IQ]) continue;
      int VP = pnew(P, P.x[IP], P.y[IP]);
      int VQ = pnew(Q, Q.x[IQ], Q.y[IQ]);
      if (VP < 0 || VQ < 0) return 3;
      if (P.src) P.src[VP] = P.src[IP];
      if (Q.src) Q.src[VQ] = Q.src[IQ];
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
  }
  // (6)
  for (int IP = 0; IP < P.n; ++IP) {
    if (!a.crossP[IP]) continue;
    int IQ = P.nb[IP];
    if (IQ >= 0 && a.crossQ[IQ]) {
      P.label[IP] = L_CROSSING;
      Q.label[IQ] = L_CROSSING;
    }
  }
  // createResult2
  long long guard = 4LL * (P.n + Q.n) + 16;
  for (int k = 0; k < a.nrP; ++k) {
    int root = sroot(a, 0, k), It = root;
    do {
      if (P.isect[It] && P.label[It] == L_CROSSING) {
        int r = rnew(a);
        if (r < 0) return 3;
        int sI = 0, I = It, sV = 0, V = I;
        P.isect[I] = 0;
        do {
          int status = side(a, sV).enex[V];
          tog(&status);
          Pool* pv;
          do {
            pv = &side(a, sV);
            V = ((status == EX_EXIT) ^ a.unite) ? pv->next[V] : pv->prev[V];
            pv->isect[V] = 0;
            const int prov = (pv->src && pv->src[V] >= 0) ? (sV << 30) | pv->src[V] : -1;
            if (radd_node(a, r, *pv, V, (status == EX_EXIT) ^ a.unite, prov)) return 2;
            if (--guard < 0) return 2;
          } while (!(pv->enex[V] == status) && !(sV == sI && V == I));
          if (!(sV == sI && V == I)) {
            int nbv = side(a, sV).nb[V];
            if (nbv < 0) return 2;
            sV = 1 - sV;
            V = nbv;
            side(a, sV).isect[V] = 0;
          }
        } while (!(sV == sI && V == I));
      }
      It = P.next[It];
    } while (It != root);
  }
  return 0;
}

__device__ int ser_label_trace(SerialArgs& a) { return ser_label_trace_t(a, NoRunPip{}); }

__device__ void ser_cleanup(SerialArgs& a) {
  Pool& p = a.R;
  for (int r = 0; r < *a.nrings; ++r) {
    auto A = [&](int v) {
      return fabs(area3(p.x[p.prev[v]], p.y[p.prev[v]], p.x[v], p.y[v], p.x[p.next[v]],
                        p.y[p.next[v]]));
    };
    auto remove = [&](int V) {
      if (a.rroot[r] == V) {
        a.rroot[r] = p.next[V];
        if (p.next[a.rroot[r]] == a.rroot[r]) a.rroot[r] = -1;
      }
      p.next[p.prev[V]] = p.next[V];
      p.prev[p.next[V]] = p.prev[V];
    };
    while (a.rroot[r] >= 0 && A(a.rroot[r]) < kEps) remove(a.rroot[r]);
    if (a.rroot[r] < 0) continue;
    int start = a.rroot[r], V = start;
    do {
      int nx = p.next[V];
      if (A(V) < kEps) remove(V);
      V = nx;
    } while (V != start);
  }
}


}  // namespace
}  // namespace sbc
