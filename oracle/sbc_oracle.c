/*
 * sbc_oracle.c -- CPU restatement of the reference's segment-tree polygon
 * clipping path.  TEST INFRASTRUCTURE ONLY (the checker; the product is the
 * CUDA library).  Plain C, one thread, no dependency on the product code.
 *
 * It follows multicore_clipping (reference src/clip.cpp:1415-2115) with the
 * semantics of the 1-thread CPU build under the harness patches (64-bit
 * realToInt, zero-filled malloc).  Each function cites the reference lines it
 * restates.  Reads the reference performs past the end of an array are given
 * one fixed meaning here (documented at each site).
 *
 * Build: cc -O2 -ffp-contract=off -fPIC -shared sbc_oracle.c -lm
 * (-ffp-contract=off is required: every FP64 expression must round exactly as
 * the reference's unfused x86-64 build does.)
 */
#include "sbc_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define EPS 0.000000001 /* p_seg_tree/util/constants.h:13 EPSILON */

/* ------------------------------------------------------------------------- */
/* small helpers                                                              */
/* ------------------------------------------------------------------------- */

typedef struct {
  int *a;
  long n, cap;
} ivec;

static int iv_push(ivec *v, int x) {
  if (v->n == v->cap) {
    long nc = v->cap ? v->cap * 2 : 64;
    int *na = (int *)realloc(v->a, (size_t)nc * sizeof(int));
    if (!na) return -1;
    v->a = na;
    v->cap = nc;
  }
  v->a[v->n++] = x;
  return 0;
}

/* Util::getNPowOf2 (p_seg_tree/util.cpp:18-28): smallest power of two >= n
 * (0 and 1 both give 1). */
static int npow2(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

/* number of decimal digits of m, i.e. how many passes `for (exp=1; m/exp>0;
 * exp*=10)` makes (src/clip.cpp:428, oacc_segment_tree.cpp:918). */
static int dec_passes(long m) {
  int d = 0;
  while (m > 0) {
    m /= 10;
    d++;
  }
  return d;
}

static long ipow10(int d) {
  long p = 1;
  while (d-- > 0) p *= 10;
  return p;
}

/* Stable argsort of int64 keys (bottom-up merge sort). Restates every stable
 * LSD decimal radix sort of the reference, whose result is a stable sort by
 * key mod 10^passes. */
static int stable_argsort_l(const long *key, int *idx, long n) {
  int *tmp = (int *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
  if (!tmp) return -1;
  for (long w = 1; w < n; w <<= 1) {
    for (long lo = 0; lo < n; lo += 2 * w) {
      long mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
      long i = lo, j = mid, o = lo;
      while (i < mid && j < hi) tmp[o++] = (key[idx[j]] < key[idx[i]]) ? idx[j++] : idx[i++];
      while (i < mid) tmp[o++] = idx[i++];
      while (j < hi) tmp[o++] = idx[j++];
    }
    memcpy(idx, tmp, (size_t)n * sizeof(int));
  }
  free(tmp);
  return 0;
}

/* Stable argsort of doubles with `<` (thrust::stable_sort_by_key,
 * oacc_segment_tree.cpp:4556). */
static int stable_argsort_d(const double *key, int *idx, long n) {
  int *tmp = (int *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
  if (!tmp) return -1;
  for (long w = 1; w < n; w <<= 1) {
    for (long lo = 0; lo < n; lo += 2 * w) {
      long mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
      long i = lo, j = mid, o = lo;
      while (i < mid && j < hi) tmp[o++] = (key[idx[j]] < key[idx[i]]) ? idx[j++] : idx[i++];
      while (i < mid) tmp[o++] = idx[i++];
      while (j < hi) tmp[o++] = idx[j++];
    }
    memcpy(idx, tmp, (size_t)n * sizeof(int));
  }
  free(tmp);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* geometry: oacc_segment_tree.cpp:5282-5611, 7247-7252                        */
/* ------------------------------------------------------------------------- */

/* A(P,Q,R), oacc_segment_tree.cpp:5334-5337 / foster/point2D.h:73-75 */
static double A3(double px, double py, double qx, double qy, double rx, double ry) {
  return (qx - px) * (ry - py) - (qy - py) * (rx - px);
}

/* LSMF bounding-box filter, oacc_segment_tree.cpp:5282-5316 */
static int lsmf(double l1p1x, double l1p1y, double l1p2x, double l1p2y, double l2p1x,
                double l2p1y, double l2p2x, double l2p2y) {
  double minPX = l1p1x, minPY = l1p1y, maxPX = l1p2x, maxPY = l1p2y;
  double minQX = l2p1x, minQY = l2p1y, maxQX = l2p2x, maxQY = l2p2y;
  if (minPX > l1p2x) { minPX = l1p2x; maxPX = l1p1x; }
  if (minPY > l1p2y) { minPY = l1p2y; maxPY = l1p1y; }
  if (minQX > l2p2x) { minQX = l2p2x; maxQX = l2p1x; }
  if (minQY > l2p2y) { minQY = l2p2y; maxQY = l2p1y; }
  if (minPX > maxQX || maxPX < minQX) return 0;
  if (minPY > maxQY || maxPY < minQY) return 0;
  return 1;
}

/* lineSegmentIntersection, oacc_segment_tree.cpp:5426-5517 (the candidate
 * search uses the identical lineSegmentIntersection2, :5520-5611). */
static int seg_isect(double p1x, double p1y, double p2x, double p2y, double q1x, double q1y,
                     double q2x, double q2y, double *alpha, double *beta) {
  double AP1 = A3(p1x, p1y, q1x, q1y, q2x, q2y);
  double AP2 = A3(p2x, p2y, q1x, q1y, q2x, q2y);
  if (fabs(AP1 - AP2) > EPS) {
    double AQ1 = A3(q1x, q1y, p1x, p1y, p2x, p2y);
    double AQ2 = A3(q2x, q2y, p1x, p1y, p2x, p2y);
    double a = AP1 / (AP1 - AP2), b = AQ1 / (AQ1 - AQ2);
    *alpha = a;
    *beta = b;
    int a01 = 0, a0 = 0, b01 = 0, b0 = 0;
    if ((a > EPS) && (a < 1.0 - EPS)) a01 = 1;
    else if (fabs(a) <= EPS) a0 = 1;
    if ((b > EPS) && (b < 1.0 - EPS)) b01 = 1;
    else if (fabs(b) <= EPS) b0 = 1;
    if (a01 && b01) return 1;
    if (a0 && b01) return 2;
    if (b0 && a01) return 3;
    if (a0 && b0) return 4;
  } else if (fabs(AP1) < EPS) {
    double dPx = p2x - p1x, dPy = p2y - p1y;
    double dQx = q2x - q1x, dQy = q2y - q1y;
    double PQx = q1x - p1x, PQy = q1y - p1y;
    double a = (PQx * dPx + PQy * dPy) / (dPx * dPx + dPy * dPy);
    double b = -(PQx * dQx + PQy * dQy) / (dQx * dQx + dQy * dQy);
    *alpha = a;
    *beta = b;
    int a01 = 0, a0 = 0, an = 0, b01 = 0, b0 = 0, bn = 0;
    if ((a > EPS) && (a < 1.0 - EPS)) a01 = 1;
    else if (fabs(a) <= EPS) a0 = 1;
    else an = 1;
    /* the reference tests fabs(alpha) here, not fabs(beta) (:5595) */
    if ((b > EPS) && (b < 1.0 - EPS)) b01 = 1;
    else if (fabs(a) <= EPS) b0 = 1;
    else bn = 1;
    if (a01 && b01) return 5;
    if (an && b01) return 6;
    if (bn && a01) return 7;
    if (a0 && b0) return 8;
  }
  return 0;
}

int sbco_segment_intersection(const double *p1, const double *p2, const double *q1,
                              const double *q2, double *alpha, double *beta) {
  double a = 0, b = 0;
  int t = seg_isect(p1[0], p1[1], p2[0], p2[1], q1[0], q1[1], q2[0], q2[1], &a, &b);
  if (alpha) *alpha = a;
  if (beta) *beta = b;
  return t;
}

/* alphaToInt, oacc_segment_tree.cpp:7247-7252: (int)(1e9*alpha) with x86-64
 * cvttsd2si semantics (out of range -> INT_MIN). */
static int alpha_to_int(double a) {
  if (a < EPS) return 0;
  double v = (double)1000000000 * a;
  if (!(v > -2147483649.0 && v < 2147483648.0)) return INT_MIN;
  return (int)v;
}

/* ------------------------------------------------------------------------- */
/* run state                                                                  */
/* ------------------------------------------------------------------------- */

struct ov_out {
  void *arr[SBCO_NUM_ARRAYS];
  long len[SBCO_NUM_ARRAYS];
};

struct sbco_run {
  int status;
  char msg[256];
  int k;
  struct ov_out *ov;
  long stats[SBCO_STAT_NUM];
  void *tree[SBCO_TREE_NUM];
  long tree_len[SBCO_TREE_NUM];
};

static void set_err(sbco_run *r, int st, const char *m) {
  if (r->status == SBCO_OK) {
    r->status = st;
    snprintf(r->msg, sizeof r->msg, "%s", m);
  }
}

static int put_ints(struct ov_out *o, int which, const int *a, long n) {
  int *c = (int *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
  if (!c) return -1;
  if (n) memcpy(c, a, (size_t)n * sizeof(int));
  o->arr[which] = c;
  o->len[which] = n;
  return 0;
}

static int put_reals(struct ov_out *o, int which, const double *a, long n) {
  double *c = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
  if (!c) return -1;
  if (n) memcpy(c, a, (size_t)n * sizeof(double));
  o->arr[which] = c;
  o->len[which] = n;
  return 0;
}

/* ------------------------------------------------------------------------- */
/* tree (overlay independent)                                                 */
/* ------------------------------------------------------------------------- */

typedef struct {
  /* polygons with closing vertex (src/clip.cpp:233-237, :285-288) */
  double *bP;  /* (nb+1)*2 */
  double *cP;  /* (clSize+k)*2 */
  int nb, k, clSize;
  int *cS;     /* k+1 prefix of (c_i+1) */
  /* end vertex of the edge that starts at each vertex: bnx[v] indexes bP
   * (v+1 for a single ring, whose last edge ends at the closing copy), cnx
   * indexes cP's slots; with several components an edge from a component's
   * last vertex ends at that component's first vertex */
  int *bnx, *cnx;
  /* edges (intervals), src/clip.cpp:207-298 */
  int E;
  int *eid, *etype;
  double *es, *ee;
  double minI, maxI;
  /* elementary intervals / tree */
  double *ea;  /* epc */
  int epc, numLeaves, ts;
  double *nia; /* 2*ts */
  /* cover lists CSR by node: cov_off[ts+1], cov_edge[...] (edge index order) */
  int *cov_off, *cov_edge;
  /* leaf end-list entries CSR by leaf (leaf - ts/2): leaf_off[numLeaves+1], leaf_edge */
  int *leaf_off, *leaf_edge;
} tree_t;

static void tree_free(tree_t *t) {
  free(t->bP); free(t->cP); free(t->cS); free(t->bnx); free(t->cnx);
  free(t->eid); free(t->etype); free(t->es); free(t->ee);
  free(t->ea); free(t->nia);
  free(t->cov_off); free(t->cov_edge);
  free(t->leaf_off); free(t->leaf_edge);
}

/* getData, p_seg_tree/segment_tree/edge.h:190-202 */
static void put_edge(tree_t *t, int e, int id, int type, double a, double b) {
  t->eid[e] = id;
  t->etype[e] = type;
  if (a < b) { t->es[e] = a; t->ee[e] = b; }
  else { t->ee[e] = a; t->es[e] = b; }
}

/* gpc_read_multi_polygon, src/clip.cpp:172-311 (from arrays, not files).
 * bcomp/ccomp (NULL: one ring each) split the base and the single overlay
 * into components (Foster's .poly format, lib/optimizedFostersAlgorithm/
 * README.md:43-62): component i is vertices [comp[i], comp[i+1]).  Edges keep
 * the reference's order, one per vertex in vertex order; every component
 * closes on its own first vertex, and closing edges leave the interval
 * bounds alone as the reference's closing edges do (:233-237). */
static int read_input(tree_t *t, const double *bxy, int nb, const double *cxy, const int *csz,
                      int k, const int *bcomp, int nbc, const int *ccomp, int ncc) {
  t->nb = nb;
  t->k = k;
  t->clSize = 0;
  for (int i = 0; i < k; ++i) t->clSize += csz[i];
  t->cS = (int *)calloc((size_t)k + 1, sizeof(int));
  t->bP = (double *)malloc(sizeof(double) * 2 * ((size_t)nb + 1));
  t->cP = (double *)malloc(sizeof(double) * 2 * ((size_t)t->clSize + k));
  t->E = nb + t->clSize;
  t->eid = (int *)malloc(sizeof(int) * (size_t)t->E);
  t->etype = (int *)malloc(sizeof(int) * (size_t)t->E);
  t->es = (double *)malloc(sizeof(double) * (size_t)t->E);
  t->ee = (double *)malloc(sizeof(double) * (size_t)t->E);
  t->bnx = (int *)malloc(sizeof(int) * (size_t)nb);
  t->cnx = (int *)malloc(sizeof(int) * ((size_t)t->clSize + k));
  if (!t->cS || !t->bP || !t->cP || !t->eid || !t->etype || !t->es || !t->ee || !t->bnx ||
      !t->cnx)
    return -1;
  for (int i = 0; i < k; ++i) t->cS[i + 1] = t->cS[i] + csz[i] + 1;
  memcpy(t->bP, bxy, sizeof(double) * 2 * (size_t)nb);
  t->bP[2 * nb] = t->bP[0];
  t->bP[2 * nb + 1] = t->bP[1];
  for (int v = 0; v < nb; ++v) t->bnx[v] = v + 1;
  for (int i = 0; bcomp && i < nbc; ++i) t->bnx[bcomp[i + 1] - 1] = bcomp[i];
  int id = 0, first = 1;
  for (int v = 0; v < nb; ++v) {
    const int w = t->bnx[v];
    put_edge(t, id, 2 * v, 0, t->bP[2 * v], t->bP[2 * w]);
    if (w == v + 1 && v + 1 < nb) {
      if (first) { t->minI = t->es[id]; t->maxI = t->ee[id]; first = 0; }
      if (t->minI > t->es[id]) t->minI = t->es[id];
      if (t->maxI < t->ee[id]) t->maxI = t->ee[id];
    }
    id++;
  }
  long off = 0;
  for (int i = 0; i < k; ++i) {
    int c = csz[i];
    int v0 = t->cS[i];
    memcpy(t->cP + 2 * v0, cxy + off, sizeof(double) * 2 * (size_t)c);
    off += 2L * c;
    t->cP[2 * (v0 + c)] = t->cP[2 * v0];
    t->cP[2 * (v0 + c) + 1] = t->cP[2 * v0 + 1];
    for (int v = 0; v <= c; ++v) t->cnx[v0 + v] = v0 + v + 1;
    for (int j = 0; ccomp && j < ncc; ++j) t->cnx[v0 + ccomp[j + 1] - 1] = v0 + ccomp[j];
    for (int v = 0; v < c; ++v) {
      const int w = t->cnx[v0 + v];
      put_edge(t, id, 2 * (v0 + v), i + 1, t->cP[2 * (v0 + v)], t->cP[2 * w]);
      if (w == v0 + v + 1 && v + 1 < c) {
        if (t->minI > t->es[id]) t->minI = t->es[id];
        if (t->maxI < t->ee[id]) t->maxI = t->ee[id];
      }
      id++;
    }
  }
  return 0;
}

/* constructElementaryIntervalsArrayMulticore, oacc_segment_tree.cpp:4513-4692 */
static int elementary(tree_t *t) {
  int ic = t->E;
  long n2 = 2L * ic;
  double *ele = (double *)malloc(sizeof(double) * (size_t)n2);
  int *sidx = (int *)malloc(sizeof(int) * (size_t)n2);
  int *vl = (int *)calloc((size_t)n2 + 1, sizeof(int));
  int *flag = (int *)calloc((size_t)n2 + 1, sizeof(int));
  double *arr3 = (double *)calloc((size_t)n2, sizeof(double));
  int *vloc = NULL;
  int rc = -1;
  if (!ele || !sidx || !vl || !flag || !arr3) goto out;
  for (int j = 0; j < ic; ++j) {
    ele[2 * j] = t->es[j];
    ele[2 * j + 1] = t->ee[j];
  }
  for (long i = 0; i < n2; ++i) sidx[i] = (int)i;
  if (stable_argsort_d(ele, sidx, n2)) goto out;
  /* mark vertical edges: only the edges of the first ic sorted endpoints are
   * visited (:4568-4576); the rest stay zero (zero-filled heap). */
  for (int j = 0; j < ic; ++j) {
    int i = sidx[j] / 2;
    vl[i] = 0;
    if (i == ic - 1) vl[i + 1] = 0;
    if (t->es[i] == t->ee[i]) vl[i] = 1;
  }
  {
    int s = 0;
    for (long i = 0; i <= n2; ++i) { int x = vl[i]; vl[i] = s; s += x; }
  }
  int numV = vl[n2];
  vloc = (int *)malloc(sizeof(int) * (size_t)(numV > 0 ? numV : 1));
  if (!vloc) goto out;
  for (int i = 0; i < ic; ++i)
    if (vl[i] != vl[i + 1]) vloc[vl[i]] = i;
  /* keep a value when it differs from the next sorted value, or when it is a
   * vertical edge not matching the last vertical edge before index i/2
   * (:4603-4636; note `verticalLines[i/2]`, and the last element handling
   * that stores the second-to-last value). */
  for (long i = 0; i < n2 - 1; ++i) {
    int intvi = sidx[i] / 2;
    int comid = vl[i / 2];
    int lookup = comid > 0 ? vloc[comid - 1] : 0;
    if (ele[sidx[i]] != ele[sidx[i + 1]]) {
      arr3[i] = ele[sidx[i]];
      flag[i] = 1;
    } else if (t->es[intvi] == t->ee[intvi] &&
               (comid == 0 || (t->es[lookup] != t->es[intvi] && t->ee[lookup] != t->es[intvi]))) {
      arr3[i] = t->es[intvi];
      flag[i] = 1;
    }
    if (i == n2 - 2) {
      if (ele[sidx[n2 - 2]] != ele[sidx[n2 - 1]]) {
        arr3[n2 - 1] = ele[sidx[n2 - 2]];
        flag[n2 - 1] = 1;
      }
    }
  }
  {
    int s = 0;
    for (long i = 0; i <= n2; ++i) { int x = flag[i]; flag[i] = s; s += x; }
  }
  int eleCount = flag[n2];
  if (eleCount < 1) { rc = -2; goto out; }
  int round = npow2(eleCount) + 1;
  t->ea = (double *)malloc(sizeof(double) * (size_t)round);
  if (!t->ea) goto out;
  for (long i = 0; i < n2; ++i)
    if (flag[i] != flag[i + 1]) t->ea[flag[i]] = arr3[i];
  for (int q = 0; q < round - eleCount; ++q) t->ea[eleCount + q] = t->ea[eleCount - 1];
  t->epc = round;
  t->numLeaves = round - 1;
  t->ts = 2 * t->numLeaves;
  rc = 0;
out:
  free(ele); free(sidx); free(vl); free(flag); free(arr3); free(vloc);
  return rc;
}

/* constructTreeIntervalArrayMulticore, oacc_segment_tree.cpp:4948-4994.
 * node 0 is never written by the reference; zero-filled heap gives [0,0]. */
static int tree_intervals(tree_t *t) {
  int ts = t->ts;
  t->nia = (double *)calloc((size_t)2 * ts, sizeof(double));
  if (!t->nia) return -1;
  for (int q = 0; q < t->numLeaves; ++q) {
    t->nia[ts + 2 * q] = t->ea[q];
    t->nia[ts + 2 * q + 1] = t->ea[q + 1];
  }
  for (int nid = ts / 2 - 1; nid >= 1; --nid) {
    t->nia[2 * nid] = t->nia[2 * (2 * nid)];
    t->nia[2 * nid + 1] = t->nia[2 * (2 * nid + 1) + 1];
  }
  return 0;
}

/* getDigitCount, oacc_segment_tree.cpp:250-262 */
static int digit_count(double val) {
  int d = 1;
  int iv = (int)trunc(val);
  while (iv / 10 > 0) { iv /= 10; d++; }
  return d;
}

/* findBoarder, oacc_segment_tree.cpp:420-460, over S(m) = boaders[sortedIndex[m]].
 * Reads at m = -1 or m = epc (past the arrays in the reference) compare
 * unequal to every query. */
static int find_border(const double *bo, const int *sidx, int epc, double q) {
#define SB(m) (((m) >= 0 && (m) < epc) ? bo[sidx[(m)]] : NAN)
  int l = 0, h = epc;
  while (l < h) {
    int m = l + (h - l) / 2;
    if (SB(m) == q) {
      if (SB(m - 1) != q) { h = m; l = h; }
      else h = m - 1;
    } else if (SB(m) < q) {
      l = m + 1;
    } else {
      h = m - 1;
    }
  }
  if (!(SB(h) == q)) return -1;
  return h;
#undef SB
}

/* End-list leaf insertion, insertToLeafLevelEdgeListMulticore and
 * preparePointsToNodeMapMulticore, oacc_segment_tree.cpp:1970-2113.
 * Produces, per leaf, the list of edge indices (unsorted). */
static int leaf_end_lists(tree_t *t) {
  int epc = t->epc, ts = t->ts, L = ts / 2;
  double *bo = (double *)calloc((size_t)epc, sizeof(double));
  long *ib = (long *)calloc((size_t)epc, sizeof(long));
  int *left = (int *)calloc((size_t)epc, sizeof(int));
  int *right = (int *)calloc((size_t)epc, sizeof(int));
  int *sidx = (int *)malloc(sizeof(int) * (size_t)epc);
  int *cnt = (int *)calloc((size_t)t->numLeaves + 1, sizeof(int));
  int *after = (int *)malloc(sizeof(int) * (size_t)t->E);
  int *before = (int *)malloc(sizeof(int) * (size_t)t->E);
  int rc = -1;
  if (!bo || !ib || !left || !right || !sidx || !cnt || !after || !before) goto out;
  {
    double absMin = fabs(t->minI);
    int d = digit_count(t->maxI + absMin);
    double scale = pow(10, 11 - d);
    for (int i = 1; i < epc; ++i) {
      left[i - 1] = L + i - 1;
      right[i - 1] = L + i;
      /* elementaryArray[epc] (i = epc-1) lies past the array: taken unequal */
      if (i != 1 && i + 1 < epc && t->ea[i] == t->ea[i + 1]) right[i - 1] = L + i + 1;
      bo[i - 1] = t->ea[i];
      if (t->ea[0] < 0) ib[i - 1] = (long)(scale * (t->ea[i] + absMin));
      else ib[i - 1] = (long)(scale * t->ea[i]);
      if (ib[i - 1] < 0) { rc = -2; goto out; } /* the reference's digit sort crashes */
    }
    /* radixsort(intBoaders, .., MAX_INTERVAL_DIGIT_COUNT=11): stable by value
     * mod 1e11, over all epc entries including the zero garbage entry epc-1 */
    long mod = ipow10(11);
    for (int i = 0; i < epc; ++i) { ib[i] %= mod; sidx[i] = i; }
    if (stable_argsort_l(ib, sidx, epc)) goto out;
  }
  for (int e = 0; e < t->E; ++e) {
    after[e] = before[e] = -1;
    int en = find_border(bo, sidx, epc, t->ee[e]);
    int st = find_border(bo, sidx, epc, t->es[e]);
    if (en >= 0) {
      int a = right[sidx[en]];
      /* node ts lies past the tree (reference reads past nodeIntervalArray):
       * the entry is dropped; node 0 is [0,0] and is dropped by the test */
      if (a >= L && a < ts && t->nia[2 * a] != t->nia[2 * a + 1]) after[e] = a;
    }
    if (st >= 0) {
      int b = left[sidx[st]];
      if (b >= L && b < ts && t->nia[2 * b] != t->nia[2 * b + 1]) before[e] = b;
    }
    if (after[e] >= 0) cnt[after[e] - L]++;
    if (before[e] >= 0) cnt[before[e] - L]++;
  }
  t->leaf_off = (int *)malloc(sizeof(int) * ((size_t)t->numLeaves + 1));
  if (!t->leaf_off) goto out;
  {
    int s = 0;
    for (int q = 0; q < t->numLeaves; ++q) { t->leaf_off[q] = s; s += cnt[q]; cnt[q] = 0; }
    t->leaf_off[t->numLeaves] = s;
    t->leaf_edge = (int *)malloc(sizeof(int) * (size_t)(s > 0 ? s : 1));
    if (!t->leaf_edge) goto out;
  }
  for (int e = 0; e < t->E; ++e) {
    if (after[e] >= 0) { int q = after[e] - L; t->leaf_edge[t->leaf_off[q] + cnt[q]++] = e; }
    if (before[e] >= 0) { int q = before[e] - L; t->leaf_edge[t->leaf_off[q] + cnt[q]++] = e; }
  }
  rc = 0;
out:
  free(bo); free(ib); free(left); free(right); free(sidx); free(cnt); free(after); free(before);
  return rc;
}

/* insertEdgeParallel, oacc_segment_tree.cpp:2496-2564 (Edge::contains /
 * Edge::intersects, edge.h:160-188). Appends (node, edge) pairs in visit
 * order. */
static int cover_insert(const tree_t *t, int e, int v, ivec *nodes, ivec *edges) {
  double s = t->es[e], x = t->ee[e];
  if (s <= t->nia[2 * v] && x >= t->nia[2 * v + 1]) {
    if (iv_push(nodes, v) || iv_push(edges, e)) return -1;
    return 0;
  }
  for (int c = 2 * v; c <= 2 * v + 1; ++c) {
    if (c >= t->ts) continue;
    double cs = t->nia[2 * c], ce = t->nia[2 * c + 1];
    int inter = (s <= cs && x >= ce) || (cs <= s && ce >= x) || (s <= cs && x >= cs) ||
                (ce <= x && ce >= s);
    if (inter && cover_insert(t, e, c, nodes, edges)) return -1;
  }
  return 0;
}

/* insertAllParallel at one thread, oacc_segment_tree.cpp:2571-2607: cover
 * lists in edge index order. */
static int cover_lists(tree_t *t) {
  ivec nodes = {0}, edges = {0};
  int rc = -1;
  for (int e = 0; e < t->E; ++e)
    if (cover_insert(t, e, 1, &nodes, &edges)) goto out;
  t->cov_off = (int *)calloc((size_t)t->ts + 1, sizeof(int));
  t->cov_edge = (int *)malloc(sizeof(int) * (size_t)(edges.n > 0 ? edges.n : 1));
  if (!t->cov_off || !t->cov_edge) goto out;
  for (long i = 0; i < nodes.n; ++i) t->cov_off[nodes.a[i] + 1]++;
  for (int v = 0; v < t->ts; ++v) t->cov_off[v + 1] += t->cov_off[v];
  {
    int *fill = (int *)calloc((size_t)t->ts, sizeof(int));
    if (!fill) goto out;
    for (long i = 0; i < nodes.n; ++i) {
      int v = nodes.a[i];
      t->cov_edge[t->cov_off[v] + fill[v]++] = edges.a[i];
    }
    free(fill);
  }
  rc = 0;
out:
  free(nodes.a);
  free(edges.a);
  return rc;
}

/* end list of node v: union of the leaf lists below v, unique by (id, type),
 * ordered by (id, type): the merged lists of buildInternalEndListsMulticore
 * (oacc_segment_tree.cpp:1717-1968, leaf sort edgeRadixsort :909-922). */
static long key_id_type(const tree_t *t, int e) { return (long)t->eid[e] * 16 + t->etype[e]; }

static int end_list(const tree_t *t, int v, ivec *out) {
  int L = t->ts / 2;
  int lo = v, hi = v + 1;
  while (lo < L) { lo *= 2; hi *= 2; }
  out->n = 0;
  for (int q = t->leaf_off[lo - L]; q < t->leaf_off[hi - L]; ++q)
    if (iv_push(out, t->leaf_edge[q])) return -1;
  long n = out->n;
  if (n == 0) return 0;
  long *key = (long *)malloc(sizeof(long) * (size_t)n);
  int *idx = (int *)malloc(sizeof(int) * (size_t)n);
  int *tmp = (int *)malloc(sizeof(int) * (size_t)n);
  if (!key || !idx || !tmp) { free(key); free(idx); free(tmp); return -1; }
  for (long i = 0; i < n; ++i) { key[i] = key_id_type(t, out->a[i]); idx[i] = (int)i; }
  stable_argsort_l(key, idx, n);
  long m = 0;
  for (long i = 0; i < n; ++i) {
    if (m > 0 && key[idx[i]] == key_id_type(t, tmp[m - 1])) continue;
    tmp[m++] = out->a[idx[i]];
  }
  memcpy(out->a, tmp, sizeof(int) * (size_t)m);
  out->n = m;
  free(key); free(idx); free(tmp);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* per-overlay clipping                                                       */
/* ------------------------------------------------------------------------- */

/* saveIntersectionsIdsMulticore at one thread, oacc_segment_tree.cpp:6108-6244 */
static int candidates(const tree_t *t, int cType, ivec *rb, ivec *rc, ivec *rt) {
  ivec el = {0};
  const double *bP = t->bP, *cP = t->cP;
  for (int nid = 1; nid < t->ts; ++nid) {
    int cs = t->cov_off[nid], ce = t->cov_off[nid + 1];
    if (cs == ce) continue; /* treeNode never created: skipped (:6121) */
    if (end_list(t, nid, &el)) goto fail;
    for (int a = cs; a < ce; ++a) {
      int it = t->cov_edge[a];
      for (int b2 = cs; b2 < ce; ++b2) {
        int in = t->cov_edge[b2];
        int bId, cId, go = 0;
        if (t->etype[it] == 0 && t->etype[in] == cType) { bId = t->eid[it]; cId = t->eid[in]; go = 1; }
        else if (t->etype[it] == cType && t->etype[in] == 0) { bId = t->eid[in]; cId = t->eid[it]; go = 1; }
        if (!go) continue;
        const double *bq = bP + 2 * t->bnx[bId / 2], *cq = cP + 2 * t->cnx[cId / 2];
        if (lsmf(bP[bId], bP[bId + 1], bq[0], bq[1], cP[cId], cP[cId + 1], cq[0], cq[1])) {
          double al, be;
          int ty = seg_isect(bP[bId], bP[bId + 1], bq[0], bq[1], cP[cId], cP[cId + 1], cq[0],
                             cq[1], &al, &be);
          if (ty && (iv_push(rb, bId) || iv_push(rc, cId) || iv_push(rt, ty))) goto fail;
        }
      }
      for (long q = 0; q < el.n; ++q) {
        int en = el.a[q];
        int bId, cId, go = 0;
        if (t->etype[it] == 0 && t->etype[en] == cType) { bId = t->eid[it]; cId = t->eid[en]; go = 1; }
        else if (t->etype[it] == cType && t->etype[en] == 0) { cId = t->eid[it]; bId = t->eid[en]; go = 1; }
        if (!go) continue;
        const double *bq = bP + 2 * t->bnx[bId / 2], *cq = cP + 2 * t->cnx[cId / 2];
        if (lsmf(bP[bId], bP[bId + 1], bq[0], bq[1], cP[cId], cP[cId + 1], cq[0], cq[1])) {
          double al, be;
          int ty = seg_isect(bP[bId], bP[bId + 1], bq[0], bq[1], cP[cId], cP[cId + 1], cq[0],
                             cq[1], &al, &be);
          if (ty && (iv_push(rb, bId) || iv_push(rc, cId) || iv_push(rt, ty))) goto fail;
        }
      }
    }
  }
  free(el.a);
  return 0;
fail:
  free(el.a);
  return -1;
}

/* isNonDegenerateCase, src/clip.cpp:508-517 */
static int nondegen(char poly, int type) {
  if (poly == 'b') return type == 1 || type == 3 || type == 5 || type == 7;
  return type == 1 || type == 2 || type == 6;
}

/* countEdgeIntersections, src/clip.cpp:522-601 (K = 0: all counts zero; the
 * reference reads an empty vector there). */
static void count_edges(const int *edges, const int *sidx, int cStart, const int *types, int K,
                        char poly, int *all, int *nd, int *uids, int polysize, int *nuniq) {
  if (K <= 0) {
    for (int i = 0; i < polysize; ++i) all[i] = nd[i] = 0;
    *nuniq = 0;
    return;
  }
  int *ec = (int *)malloc(sizeof(int) * (size_t)K);
  int *nc = (int *)malloc(sizeof(int) * (size_t)K);
  int j = 0, edgeCount = 1, ndc = 0;
  int cur = edges[sidx[0]];
  ec[0] = edgeCount;
  uids[0] = cur;
  if (nondegen(poly, types[sidx[0]])) ndc = 1;
  nc[0] = ndc;
  for (int i = 1; i < K; ++i) {
    if (edges[sidx[i]] == cur) {
      edgeCount++;
      if (nondegen(poly, types[sidx[i]])) ndc++;
    } else {
      ec[j] = edgeCount;
      nc[j] = ndc;
      uids[j + 1] = edges[sidx[i]];
      cur = edges[sidx[i]];
      j++;
      edgeCount = 1;
      ndc = nondegen(poly, types[sidx[i]]) ? 1 : 0;
    }
    if (i == K - 1) { ec[j] = edgeCount; nc[j] = ndc; }
  }
  /* uids past the last run are zero in the reference (zero-filled heap) and
   * never match an edge i >= 1; only the runs found are consulted here */
  int nfound = j + 1;
  j = 0;
  for (int i = 0; i < polysize; ++i) {
    if (j < nfound && (i + cStart) == uids[j] / 2) {
      all[i] = ec[j];
      nd[i] = nc[j];
      j++;
    } else {
      all[i] = nd[i] = 0;
    }
  }
  *nuniq = j;
  free(ec);
  free(nc);
}

static void excl_scan(int *a, int n) { /* thrust::exclusive_scan in place over n */
  int s = 0;
  for (int i = 0; i < n; ++i) { int x = a[i]; a[i] = s; s += x; }
}

/* sortIntersectionsAtEdgesParallel, oacc_segment_tree.cpp:7436-7473: per edge
 * with more than one non-degenerate intersection, stable 9-digit decimal sort
 * (value mod 1e9) of its slice. */
static int sort_at_edges(const int *alpha, const int *sidx, int cStart, const int *allPS,
                         const int *ndPS, const int *uids, int nuniq, int K, int *out) {
  long *cp = (long *)malloc(sizeof(long) * (size_t)(K > 0 ? K : 1));
  if (!cp) return -1;
  for (int i = 0; i < K; ++i) { out[i] = i; cp[i] = alpha[sidx[i]]; }
  for (int id = 0; id < nuniq; ++id) {
    int eid = uids[id] / 2 - cStart;
    int s = allPS[eid], e = allPS[eid + 1];
    int ns = ndPS[eid], ne = ndPS[eid + 1];
    if (ne - ns > 1) {
      for (int i = s; i < e; ++i)
        if (cp[i] < 0) { free(cp); return -2; } /* negative digit: reference crashes */
      long *key = (long *)malloc(sizeof(long) * (size_t)K);
      if (!key) { free(cp); return -1; }
      for (int i = s; i < e; ++i) key[i] = cp[i] % 1000000000L;
      /* stable argsort of positions s..e-1 by key; out[s..e) holds positions */
      stable_argsort_l(key, out + s, e - s);
      free(key);
    }
  }
  free(cp);
  return 0;
}

/* ---- linked lists (foster/polygon.h) as index arrays ---------------------- */

enum { L_NONE = 0, L_CROSSING, L_BOUNCING, L_LEFT_ON, L_RIGHT_ON, L_ON_ON, L_ON_LEFT,
       L_ON_RIGHT, L_DELAYED_CROSSING, L_DELAYED_BOUNCING };
enum { EX_EXIT = 0, EX_ENTRY = 1, EX_NEITHER = 2 };

typedef struct {
  double *x, *y;
  int *next, *prev, *nb;
  unsigned char *source, *isect;
  int *label, *enex;
  int n, cap;
} pool_t;

static int pool_init(pool_t *p, int cap) {
  memset(p, 0, sizeof *p);
  p->cap = cap;
  p->x = (double *)malloc(sizeof(double) * (size_t)cap);
  p->y = (double *)malloc(sizeof(double) * (size_t)cap);
  p->next = (int *)malloc(sizeof(int) * (size_t)cap);
  p->prev = (int *)malloc(sizeof(int) * (size_t)cap);
  p->nb = (int *)malloc(sizeof(int) * (size_t)cap);
  p->source = (unsigned char *)calloc((size_t)cap, 1);
  p->isect = (unsigned char *)calloc((size_t)cap, 1);
  p->label = (int *)calloc((size_t)cap, sizeof(int));
  p->enex = (int *)malloc(sizeof(int) * (size_t)cap);
  if (!p->x || !p->y || !p->next || !p->prev || !p->nb || !p->source || !p->isect || !p->label ||
      !p->enex)
    return -1;
  return 0;
}

static void pool_free(pool_t *p) {
  free(p->x); free(p->y); free(p->next); free(p->prev); free(p->nb);
  free(p->source); free(p->isect); free(p->label); free(p->enex);
}

/* vertex(point2D&) constructor: label NONE, enex NEITHER, no neighbour */
static int pool_new(pool_t *p, double x, double y) {
  if (p->n >= p->cap) return -1;
  int v = p->n++;
  p->x[v] = x; p->y[v] = y;
  p->next[v] = p->prev[v] = v;
  p->nb[v] = -1;
  p->source[v] = 0; p->isect[v] = 0;
  p->label[v] = L_NONE; p->enex[v] = EX_NEITHER;
  return v;
}

/* insertVertex(V, curr) with alpha = -1: V goes between curr and curr->next
 * (polygon.h:101-113). */
static void insert_after(pool_t *p, int V, int curr) {
  curr = p->next[curr];
  p->next[p->prev[curr]] = V;
  p->prev[V] = p->prev[curr];
  p->next[V] = curr;
  p->prev[curr] = V;
}

/* pointInPoly, polygon.h:427-448, over the current list from root */
static int point_in_poly(const pool_t *p, int root, double rx, double ry) {
  int w = 0;
  int one = root;
  do {
    int two = p->next[one];
    double x0 = p->x[one], y0 = p->y[one], x1 = p->x[two], y1 = p->y[two];
    if ((y0 < ry) != (y1 < ry)) {
      if (x0 >= rx) {
        if (x1 > rx) w = w + 2 * (y1 > y0) - 1;
        else if ((A3(x0, y0, x1, y1, rx, ry) > 0) == (y1 > y0)) w = w + 2 * (y1 > y0) - 1;
      } else if (x1 > rx) {
        if ((A3(x0, y0, x1, y1, rx, ry) > 0) == (y1 > y0)) w = w + 2 * (y1 > y0) - 1;
      }
    }
    one = two;
  } while (one != root);
  return (w % 2) != 0;
}

/* result rings: each ring is a vertex list in `rp` */
typedef struct {
  pool_t rp;
  int *root;
  int nr, rcap;
} rings_t;

static int ring_new(rings_t *R) {
  if (R->nr == R->rcap) {
    int nc = R->rcap ? R->rcap * 2 : 16;
    int *na = (int *)realloc(R->root, sizeof(int) * (size_t)nc);
    if (!na) return -1;
    R->root = na;
    R->rcap = nc;
  }
  R->root[R->nr] = -1;
  return R->nr++;
}

/* polygon::newVertex appended to ring r (polygon.h:388-407) */
static int ring_add(rings_t *R, int r, double x, double y) {
  int v = pool_new(&R->rp, x, y);
  if (v < 0) return -1;
  int root = R->root[r];
  if (root < 0) {
    R->root[r] = v;
  } else {
    R->rp.prev[v] = R->rp.prev[root];
    R->rp.next[v] = root;
    R->rp.next[R->rp.prev[root]] = v;
    R->rp.prev[root] = v;
  }
  return 0;
}

/* rPolyList.push_back(P) of a whole input list (labelIntersections2 step 3.5) */
static int ring_copy_list(rings_t *R, const pool_t *p, int root) {
  int r = ring_new(R);
  if (r < 0) return -1;
  int v = root;
  do {
    if (ring_add(R, r, p->x[v], p->y[v])) return -1;
    v = p->next[v];
  } while (v != root);
  return 0;
}

/* removeVertex, polygon.h:412-421, for ring r */
static void ring_remove(rings_t *R, int r, int V) {
  pool_t *p = &R->rp;
  if (R->root[r] == V) {
    R->root[r] = p->next[V];
    if (p->next[R->root[r]] == R->root[r]) R->root[r] = -1;
  }
  p->next[p->prev[V]] = p->next[V];
  p->prev[p->next[V]] = p->prev[V];
}

/* cleanUpResult2, foster/polyclip.h:767-787.  The reference keeps iterating
 * from a deleted vertex; its (freed but intact) next pointer is followed,
 * which is what this loop does. */
static void cleanup(rings_t *R) {
  pool_t *p = &R->rp;
  for (int r = 0; r < R->nr; ++r) {
    while (R->root[r] >= 0) {
      int v = R->root[r];
      if (!(fabs(A3(p->x[p->prev[v]], p->y[p->prev[v]], p->x[v], p->y[v], p->x[p->next[v]],
                    p->y[p->next[v]])) < EPS))
        break;
      ring_remove(R, r, v);
    }
    if (R->root[r] < 0) continue;
    int start = R->root[r];
    int V = start;
    do {
      int nx = p->next[V];
      if (fabs(A3(p->x[p->prev[V]], p->y[p->prev[V]], p->x[V], p->y[V], p->x[nx], p->y[nx])) <
          EPS)
        ring_remove(R, r, V);
      V = nx;
    } while (V != start);
  }
}

/* roots[s][k]: the list node of side s's component k's first vertex (its
 * merged slot); roots[s][nr[s]] = the side's slot count.  One component per
 * side reproduces the reference (root 0). */
typedef struct {
  pool_t P, Q;
  int *roots[2];
  int nr[2];
} lists_t;

/* copyToLinkedList, src/clip.cpp:606-695, restated over slot arrays, one
 * component after another (each walked from its first vertex and closed on
 * it, as the reference's single ring is).  The list order equals the slot
 * order; a source vertex matched early by an intersection vertex with
 * identical coordinates makes the reference's bookkeeping undefined
 * (rejected here).  vs[k] .. vs[k+1] are component k's source vertices. */
static int build_side(pool_t *P, pool_t *O, int is_q, const double *poly, int start,
                      const int *vs, int nr, const int *roots, const double *ix, int n,
                      const int *alpha, const int *nb, const int *lab) {
  for (int k = 0; k < nr; ++k) {
    const int lo = roots[k], hi = roots[k + 1];
    int i = lo;
    for (int ii = vs[k]; ii <= vs[k + 1]; ++ii) {
      const int last = ii == vs[k + 1];
      const int srcv = last ? vs[k] : ii;
      const double vx = poly[2 * (start + srcv)], vy = poly[2 * (start + srcv) + 1];
      for (;;) {
        const int sl = i == hi ? lo : i;
        if (i > hi || (ix[2 * sl] == vx && ix[2 * sl + 1] == vy)) break;
        if (i >= hi) return -2;
        int v = pool_new(P, ix[2 * i], ix[2 * i + 1]);
        P->label[v] = lab[i];
        P->isect[v] = 1;
        if (is_q) {
          int t = nb[i] - 1;
          if (t < 0 || t >= O->n) return -2;
          P->nb[v] = t;
          O->nb[t] = v;
        }
        i++;
      }
      if (i > hi || (!last && i >= hi)) return -2; /* more vertices than the component's slots */
      if (!last) {
        int v = pool_new(P, vx, vy);
        if (v != i) return -2;
        P->source[v] = 1;
        P->label[v] = lab[i];
        if (!is_q) {
          if (alpha[i] != -100) P->isect[v] = 1;
        } else if (nb[i] != -100) {
          int t = nb[i] - 1;
          if (t < 0 || t >= O->n) return -2;
          P->isect[v] = 1;
          P->nb[v] = t;
          O->nb[t] = v;
        }
      }
      i++;
    }
    for (int v = lo; v < hi; ++v) {
      P->next[v] = v + 1 == hi ? lo : v + 1;
      P->prev[v] = v == lo ? hi - 1 : v - 1;
    }
  }
  return P->n == n ? 0 : -2;
}

static int build_lists(lists_t *Ls, const double *bPoly, const double *cPoly, int cStart,
                       const int *vsB, const int *vsC, const double *ixB, const double *ixC,
                       const int *alphaB, const int *nbC, int nB, int nQ, const int *labB,
                       const int *labC, int extra) {
  pool_t *P = &Ls->P, *Q = &Ls->Q;
  if (pool_init(P, nB + extra) || pool_init(Q, nQ + extra)) return -1;
  int r = build_side(P, Q, 0, bPoly, 0, vsB, Ls->nr[0], Ls->roots[0], ixB, nB, alphaB, NULL,
                     labB);
  if (r) return r;
  /* the base's node count is its slot count: a neighbour id past it is
   * undefined, as the reference's (t >= nB) check */
  return build_side(Q, P, 1, cPoly, cStart, vsC, Ls->nr[1], Ls->roots[1], ixC, nQ, NULL, nbC,
                    labC);
}

/* neighbour of vertex v of polygon `side` lives in the other polygon */
#define OTHER(s) (1 - (s))

static pool_t *side_pool(lists_t *Ls, int s) { return s == 0 ? &Ls->P : &Ls->Q; }

/* oracle(): relative position of Q w.r.t. chain (P1,P2,P3), polyclip.h:299-328 */

/* getNonIntersectionVertex, polygon.h:497-513 (may insert a temporary vertex) */
static int non_isect_vertex(lists_t *Ls, int s, int root, int *err) {
  pool_t *p = side_pool(Ls, s), *o = side_pool(Ls, OTHER(s));
  int V = root;
  do {
    if (!p->isect[V]) return V;
    V = p->next[V];
  } while (V != root);
  V = root;
  do {
    int nbV = p->nb[V], nbN = p->nb[p->next[V]];
    if (nbV < 0) { *err = 1; return -1; }
    if (nbN != o->prev[nbV] && nbN != o->next[nbV]) {
      double mx = 0.5 * (p->x[V] + p->x[p->next[V]]);
      double my = 0.5 * (p->y[V] + p->y[p->next[V]]);
      int T = pool_new(p, mx, my);
      if (T < 0) { *err = 1; return -1; }
      insert_after(p, T, V);
      return T;
    }
    V = p->next[V];
  } while (V != root);
  *err = 1;
  return -1;
}

/* getNonIntersectionPoint, polygon.h:480-492 */
static int non_isect_point(lists_t *Ls, int s, int root, double *x, double *y) {
  pool_t *p = side_pool(Ls, s), *o = side_pool(Ls, OTHER(s));
  int V = root;
  do {
    if (!p->isect[V]) { *x = p->x[V]; *y = p->y[V]; return 0; }
    V = p->next[V];
  } while (V != root);
  V = root;
  do {
    int nbV = p->nb[V], nbN = p->nb[p->next[V]];
    if (nbV < 0) return -1;
    if (nbN != o->prev[nbV] && nbN != o->next[nbV]) {
      *x = 0.5 * (p->x[V] + p->x[p->next[V]]);
      *y = 0.5 * (p->y[V] + p->y[p->next[V]]);
      return 0;
    }
    V = p->next[V];
  } while (V != root);
  return -1;
}

static void toggle(int *st) {
  if (*st == EX_ENTRY) *st = EX_EXIT;
  else if (*st == EX_EXIT) *st = EX_ENTRY;
}

/* The back end's UNION switch (foster/polyclip.h:39): the reference's seg
 * driver leaves it off; its Foster back end supports it (:451-470, :571-618,
 * :669-680, :740). */
static int g_union = 0;
void sbco_set_union(int on) { g_union = on ? 1 : 0; }

/* pointInPoly against every component of side s: a component toggles the
 * answer when it contains the point (lib/optimizedFostersAlgorithm/
 * polyclip.cpp:503-507, :593-595); one component is the reference's test */
static int point_in_side(lists_t *Ls, int s, double x, double y) {
  int in = 0;
  for (int k = 0; k < Ls->nr[s]; ++k) in ^= point_in_poly(side_pool(Ls, s), Ls->roots[s][k], x, y);
  return in;
}

/* labelIntersections2 + createResult2, foster/polyclip.h:337-759, over every
 * component of both sides in the order of Foster's multi-component code
 * (lib/optimizedFostersAlgorithm/polyclip.cpp:335-780): chains, interior and
 * identical components, entry/exit flags per component, and the result
 * traced from P's components in order. */
static int label_and_trace(lists_t *Ls, rings_t *R) {
  pool_t *P = &Ls->P, *Q = &Ls->Q;
  /* (2) intersection chains on P */
  for (int k = 0; k < Ls->nr[0]; ++k) {
    const int root = Ls->roots[0][k];
    int V = root;
    do {
      if (P->isect[V] && (P->label[V] == L_LEFT_ON || P->label[V] == L_RIGHT_ON)) {
        int x = P->label[V] == L_LEFT_ON ? 0 : 1; /* LEFT=0 RIGHT=1 */
        int X = V, I = V;
        long guard = 0;
        do {
          P->label[I] = L_NONE;
          if (P->nb[I] < 0) return -2;
          Q->label[P->nb[I]] = L_NONE;
          I = P->next[I];
          if (++guard > P->n + 1) return -2;
        } while (P->label[I] == L_ON_ON);
        int y = P->label[I] == L_ON_LEFT ? 0 : 1;
        int chain = (x != y) ? L_DELAYED_CROSSING : L_DELAYED_BOUNCING;
        P->label[X] = chain;
        P->label[I] = chain;
        if (P->nb[X] < 0 || P->nb[I] < 0) return -2;
        Q->label[P->nb[X]] = chain;
        Q->label[P->nb[I]] = chain;
      }
      V = P->next[V];
    } while (V != root);
  }
  /* (3.5) special cases, per component */
  unsigned char *noIsect[2], *ident[2];
  noIsect[0] = (unsigned char *)calloc((size_t)Ls->nr[0] + 1, 1);
  noIsect[1] = (unsigned char *)calloc((size_t)Ls->nr[1] + 1, 1);
  ident[0] = (unsigned char *)calloc((size_t)Ls->nr[0] + 1, 1);
  ident[1] = (unsigned char *)calloc((size_t)Ls->nr[1] + 1, 1);
  unsigned char *split[2] = {NULL, NULL}, *cross[2] = {NULL, NULL};
  int rc = -1;
  if (!noIsect[0] || !noIsect[1] || !ident[0] || !ident[1]) goto done;
  for (int s = 0; s < 2; ++s)
  for (int k = 0; k < Ls->nr[s]; ++k) {
    pool_t *p = side_pool(Ls, s);
    int nocross = 1, root = Ls->roots[s][k];
    int V = root;
    do {
      if (p->isect[V] && (p->label[V] == L_CROSSING || p->label[V] == L_DELAYED_CROSSING)) nocross = 0;
      /* noCrossingVertex(UNION), foster/polygon.h:465-475 */
      if (g_union && p->isect[V] &&
          (p->label[V] == L_BOUNCING || p->label[V] == L_DELAYED_BOUNCING))
        nocross = 0;
      V = p->next[V];
    } while (V != root);
    if (!nocross) continue;
    noIsect[s][k] = 1;
    int allon = 1;
    V = root;
    do {
      if (p->label[V] != L_ON_ON) allon = 0;
      V = p->next[V];
    } while (V != root);
    if (allon) {
      ident[s][k] = 1;
    } else {
      double px, py;
      if (non_isect_point(Ls, s, root, &px, &py)) { rc = -2; goto done; }
      if (point_in_side(Ls, OTHER(s), px, py) ^ g_union)
        if (ring_copy_list(R, p, root)) goto done;
    }
  }
  /* identical components (polyclip.cpp:516-538): P's component k is added
   * when the identical component of Q holding its root's neighbour is a hole
   * exactly when k is (inside an odd number of its side's other components) */
  for (int k = 0; k < Ls->nr[0]; ++k) {
    if (!ident[0][k]) continue;
    const int rk = Ls->roots[0][k];
    int holeP = 0;
    for (int j = 0; j < Ls->nr[0]; ++j)
      if (j != k) holeP ^= point_in_poly(P, Ls->roots[0][j], P->x[rk], P->y[rk]);
    const int target = P->nb[rk];
    for (int m = 0; m < Ls->nr[1]; ++m) {
      if (!ident[1][m]) continue;
      const int rm = Ls->roots[1][m];
      int V = rm, found = 0;
      do {
        if (V == target) found = 1;
        V = Q->next[V];
      } while (V != rm);
      if (!found) continue;
      int holeQ = 0;
      for (int j = 0; j < Ls->nr[1]; ++j)
        if (j != m) holeQ ^= point_in_poly(Q, Ls->roots[1][j], Q->x[rm], Q->y[rm]);
      if (holeP == holeQ && ring_copy_list(R, P, rk)) goto done;
      break;
    }
  }
  /* (4) entry/exit flags, split and crossing candidates */
  split[0] = (unsigned char *)calloc((size_t)P->cap, 1);
  split[1] = (unsigned char *)calloc((size_t)Q->cap, 1);
  cross[0] = (unsigned char *)calloc((size_t)P->cap, 1);
  cross[1] = (unsigned char *)calloc((size_t)Q->cap, 1);
  if (!split[0] || !split[1] || !cross[0] || !cross[1]) goto done;
  for (int s = 0; s < 2; ++s)
  for (int k = 0; k < Ls->nr[s]; ++k) {
    if (noIsect[s][k]) continue;
    pool_t *p = side_pool(Ls, s);
    int err = 0;
    int V = non_isect_vertex(Ls, s, Ls->roots[s][k], &err);
    if (err) { rc = -2; goto done; }
    int status = EX_ENTRY;
    if (point_in_side(Ls, OTHER(s), p->x[V], p->y[V])) toggle(&status);
    int first = 1;
    int I = V;
    do {
      if (p->isect[I]) {
        if (p->label[I] == L_CROSSING) { p->enex[I] = status; toggle(&status); }
        if (p->label[I] == L_BOUNCING && ((status == EX_EXIT) ^ g_union)) split[s][I] = 1;
        if (p->label[I] == L_DELAYED_CROSSING) {
          p->enex[I] = status;
          if (first) {
            if ((status == EX_EXIT) ^ g_union) p->label[I] = L_CROSSING;
            first = 0;
          } else {
            if ((status == EX_ENTRY) ^ g_union) p->label[I] = L_CROSSING;
            first = 1;
            toggle(&status);
          }
        }
        if (p->label[I] == L_DELAYED_BOUNCING) {
          p->enex[I] = status;
          if (first) {
            if ((status == EX_EXIT) ^ g_union) cross[s][I] = 1;
            first = 0;
          } else {
            if ((status == EX_ENTRY) ^ g_union) cross[s][I] = 1;
            first = 1;
          }
          toggle(&status);
        }
      }
      I = p->next[I];
    } while (I != V);
  }
  /* (5) split vertex pairs (order independent) */
  {
    int nP0 = P->n;
    for (int IP = 0; IP < nP0; ++IP) {
      if (!split[0][IP]) continue;
      int IQ = P->nb[IP];
      if (IQ < 0 || !split[1][IQ]) continue;
      int VP = pool_new(P, P->x[IP], P->y[IP]);
      int VQ = pool_new(Q, Q->x[IQ], Q->y[IQ]);
      if (VP < 0 || VQ < 0) { rc = -2; goto done; }
      double sP = A3(P->x[P->prev[IP]], P->y[P->prev[IP]], P->x[IP], P->y[IP], P->x[P->next[IP]],
                     P->y[P->next[IP]]);
      double sQ = A3(Q->x[Q->prev[IQ]], Q->y[Q->prev[IQ]], Q->x[IQ], Q->y[IQ], Q->x[Q->next[IQ]],
                     Q->y[Q->next[IQ]]);
      if (sP * sQ > 0) {
        P->nb[IP] = VQ; Q->nb[VQ] = IP; P->isect[IP] = 1; Q->isect[VQ] = 1;
        Q->nb[IQ] = VP; P->nb[VP] = IQ; Q->isect[IQ] = 1; P->isect[VP] = 1;
      } else {
        P->nb[VP] = VQ; Q->nb[VQ] = VP; P->isect[VP] = 1; Q->isect[VQ] = 1;
      }
      insert_after(P, VP, IP);
      insert_after(Q, VQ, IQ);
      if (!g_union) {
        P->enex[IP] = EX_EXIT; P->enex[VP] = EX_ENTRY;
        Q->enex[IQ] = EX_EXIT; Q->enex[VQ] = EX_ENTRY;
      } else {
        P->enex[IP] = EX_ENTRY; P->enex[VP] = EX_EXIT;
        Q->enex[IQ] = EX_ENTRY; Q->enex[VQ] = EX_EXIT;
      }
      P->label[IP] = P->label[VP] = L_CROSSING;
      Q->label[IQ] = Q->label[VQ] = L_CROSSING;
    }
  }
  /* (6) crossing candidates */
  for (int IP = 0; IP < P->n; ++IP) {
    if (!cross[0][IP]) continue;
    int IQ = P->nb[IP];
    if (IQ >= 0 && cross[1][IQ]) { P->label[IP] = L_CROSSING; Q->label[IQ] = L_CROSSING; }
  }
  /* createResult2, polyclip.h:717-759 */
  long guard_total = 0, guard_max = 4L * (P->n + Q->n) + 16;
  for (int k = 0; k < Ls->nr[0]; ++k) {
    int root = Ls->roots[0][k];
    int It = root;
    do {
      if (P->isect[It] && P->label[It] == L_CROSSING) {
        int r = ring_new(R);
        if (r < 0) goto done;
        int sI = 0, I = It; /* (side, vertex) */
        int sV = 0, V = I;
        P->isect[I] = 0;
        do {
          pool_t *pv = side_pool(Ls, sV);
          int status = pv->enex[V];
          toggle(&status);
          do {
            pv = side_pool(Ls, sV);
            V = ((status == EX_EXIT) ^ g_union) ? pv->next[V] : pv->prev[V];
            pv->isect[V] = 0;
            /* the pool holds every vertex once plus slack: running out means
             * the trace never returns to its start (the reference loops) */
            if (ring_add(R, r, pv->x[V], pv->y[V])) { rc = -2; goto done; }
            if (++guard_total > guard_max) { rc = -2; goto done; }
          } while (!(pv->enex[V] == status) && !(sV == sI && V == I));
          if (!(sV == sI && V == I)) {
            int nbv = side_pool(Ls, sV)->nb[V];
            if (nbv < 0) { rc = -2; goto done; }
            sV = OTHER(sV);
            V = nbv;
            side_pool(Ls, sV)->isect[V] = 0;
          }
        } while (!(sV == sI && V == I));
      }
      It = P->next[It];
    } while (It != root);
  }
  rc = 0;
done:
  free(split[0]); free(split[1]); free(cross[0]); free(cross[1]);
  free(noIsect[0]); free(noIsect[1]); free(ident[0]); free(ident[1]);
  return rc;
}

/* one overlay: src/clip.cpp:1702-2062 */
static int clip_overlay(sbco_run *run, const tree_t *t, int cType) {
  struct ov_out *o = &run->ov[cType - 1];
  int bSize = t->nb, cListId = cType - 1;
  int cStart = t->cS[cListId];
  int cSize = t->cS[cType] - t->cS[cListId] - 1;
  ivec rb = {0}, rcv = {0}, rt = {0};
  int st = -1;
  int *sidxDup = NULL, *ub = NULL, *uc = NULL, *ut = NULL, *csorted = NULL;
  int *bAll = NULL, *cAll = NULL, *bND = NULL, *cND = NULL, *bU = NULL, *cU = NULL;
  double *isxy = NULL, *ixB = NULL, *ixC = NULL;
  int *aB = NULL, *aC = NULL, *sB = NULL, *sC = NULL, *alB = NULL, *alC = NULL, *nbB = NULL,
      *nbC = NULL, *bNI = NULL, *cNI = NULL, *labB = NULL, *labC = NULL;
  int *vsB = NULL, *vsC = NULL, *qlo = NULL, *qhi = NULL;
  lists_t Ls;
  memset(&Ls, 0, sizeof Ls);
  rings_t R;
  memset(&R, 0, sizeof R);

  if (candidates(t, cType, &rb, &rcv, &rt)) goto out;
  put_ints(o, SBCO_RAW_B, rb.a, rb.n);
  put_ints(o, SBCO_RAW_C, rcv.a, rcv.n);
  put_ints(o, SBCO_RAW_T, rt.a, rt.n);
  int Kd = (int)rb.n;

  /* radixsort(bIds, m = bSize*2), src/clip.cpp:1731 + removeDuplicatesAtEdge :441-493 */
  sidxDup = (int *)malloc(sizeof(int) * (size_t)(Kd > 0 ? Kd : 1));
  ub = (int *)malloc(sizeof(int) * (size_t)(Kd > 0 ? Kd : 1));
  uc = (int *)malloc(sizeof(int) * (size_t)(Kd > 0 ? Kd : 1));
  ut = (int *)malloc(sizeof(int) * (size_t)(Kd > 0 ? Kd : 1));
  if (!sidxDup || !ub || !uc || !ut) goto out;
  {
    long *key = (long *)malloc(sizeof(long) * (size_t)(Kd > 0 ? Kd : 1));
    if (!key) goto out;
    long mod = ipow10(dec_passes(2L * bSize));
    for (int i = 0; i < Kd; ++i) { key[i] = rb.a[i] % mod; sidxDup[i] = i; }
    stable_argsort_l(key, sidxDup, Kd);
    free(key);
  }
  int K = 0;
  {
    unsigned char *dup = (unsigned char *)calloc((size_t)(Kd > 0 ? Kd : 1), 1);
    if (!dup) goto out;
    for (int id = 0; id < Kd;) {
      int sid = sidxDup[id];
      if (!dup[sid]) {
        for (int id2 = id + 1; id2 < Kd; ++id2) {
          int sid2 = sidxDup[id2];
          if (rb.a[sid] == rb.a[sid2] && rcv.a[sid] == rcv.a[sid2]) dup[sid2] = 1;
          if (rb.a[sid] != rb.a[sid2]) break;
        }
        id = id + 1;
        ub[K] = rb.a[sid];
        uc[K] = rcv.a[sid];
        ut[K] = rt.a[sid];
        K++;
      } else {
        ++id;
      }
    }
    free(dup);
  }
  put_ints(o, SBCO_UNIQ_B, ub, K);
  put_ints(o, SBCO_UNIQ_C, uc, K);
  put_ints(o, SBCO_UNIQ_T, ut, K);

  /* radixsort(cPolLineIds, m = clSize*2), src/clip.cpp:1805 */
  csorted = (int *)malloc(sizeof(int) * (size_t)(K > 0 ? K : 1));
  int *bsorted = (int *)malloc(sizeof(int) * (size_t)(K > 0 ? K : 1));
  if (!csorted || !bsorted) { free(bsorted); goto out; }
  {
    long *key = (long *)malloc(sizeof(long) * (size_t)(K > 0 ? K : 1));
    if (!key) { free(bsorted); goto out; }
    long mod = ipow10(dec_passes(2L * t->clSize));
    for (int i = 0; i < K; ++i) { key[i] = uc[i] % mod; csorted[i] = i; bsorted[i] = i; }
    stable_argsort_l(key, csorted, K);
    free(key);
  }
  bAll = (int *)calloc((size_t)bSize + 1, sizeof(int));
  cAll = (int *)calloc((size_t)cSize + 1, sizeof(int));
  bND = (int *)calloc((size_t)bSize + 1, sizeof(int));
  cND = (int *)calloc((size_t)cSize + 1, sizeof(int));
  bU = (int *)malloc(sizeof(int) * (size_t)(K > 0 ? K : 1));
  cU = (int *)malloc(sizeof(int) * (size_t)(K > 0 ? K : 1));
  if (!bAll || !cAll || !bND || !cND || !bU || !cU) { free(bsorted); goto out; }
  int nUB = 0, nUC = 0;
  count_edges(ub, bsorted, 0, ut, K, 'b', bAll, bND, bU, bSize, &nUB);
  count_edges(uc, csorted, cStart, ut, K, 'c', cAll, cND, cU, cSize, &nUC);
  excl_scan(bAll, bSize + 1);
  excl_scan(cAll, cSize + 1);
  excl_scan(bND, bSize + 1);
  excl_scan(cND, cSize + 1);
  int nB = bSize + bND[bSize], nQ = cSize + cND[cSize];

  /* saveIntersectionsParallel, oacc_segment_tree.cpp:7257-7341 */
  isxy = (double *)calloc((size_t)2 * (K > 0 ? K : 1), sizeof(double));
  aB = (int *)calloc((size_t)(K > 0 ? K : 1), sizeof(int));
  aC = (int *)calloc((size_t)(K > 0 ? K : 1), sizeof(int));
  if (!isxy || !aB || !aC) { free(bsorted); goto out; }
  for (int id = 0; id < K; ++id) {
    const double *bp = t->bP + ub[id], *cp = t->cP + uc[id];
    const double *bq = t->bP + 2 * t->bnx[ub[id] / 2], *cq = t->cP + 2 * t->cnx[uc[id] / 2];
    double al = 0, be = 0;
    int ty = seg_isect(bp[0], bp[1], bq[0], bq[1], cp[0], cp[1], cq[0], cq[1], &al, &be);
    if (ty) {
      switch (ty) {
        case 1:
          isxy[2 * id] = (1.0 - al) * bp[0] + al * bq[0];
          isxy[2 * id + 1] = (1.0 - al) * bp[1] + al * bq[1];
          break;
        case 3: case 4: case 5: case 7: case 8:
          isxy[2 * id] = cp[0];
          isxy[2 * id + 1] = cp[1];
          break;
        case 2: case 6:
          isxy[2 * id] = bp[0];
          isxy[2 * id + 1] = bp[1];
          break;
      }
      ut[id] = ty;
      aB[id] = alpha_to_int(al);
      aC[id] = alpha_to_int(be);
    }
  }
  put_reals(o, SBCO_ISECT_XY, isxy, 2L * K);
  put_ints(o, SBCO_ISECT_AB, aB, K);
  put_ints(o, SBCO_ISECT_AC, aC, K);

  sB = (int *)malloc(sizeof(int) * (size_t)(K > 0 ? K : 1));
  sC = (int *)malloc(sizeof(int) * (size_t)(K > 0 ? K : 1));
  if (!sB || !sC) { free(bsorted); goto out; }
  {
    int r1 = sort_at_edges(aB, bsorted, 0, bAll, bND, bU, nUB, K, sB);
    int r2 = sort_at_edges(aC, csorted, cStart, cAll, cND, cU, nUC, K, sC);
    if (r1 || r2) {
      free(bsorted);
      st = (r1 == -2 || r2 == -2) ? -2 : -1;
      goto out;
    }
  }

  /* copyIntersectionsParallel, oacc_segment_tree.cpp:7508-7664 (C source
   * vertices are all copied; the reference copies only the first bSize) */
  ixB = (double *)malloc(sizeof(double) * 2 * (size_t)nB);
  ixC = (double *)malloc(sizeof(double) * 2 * (size_t)nQ);
  alB = (int *)malloc(sizeof(int) * (size_t)nB);
  alC = (int *)malloc(sizeof(int) * (size_t)nQ);
  nbB = (int *)malloc(sizeof(int) * (size_t)nB);
  nbC = (int *)malloc(sizeof(int) * (size_t)nQ);
  bNI = (int *)calloc((size_t)(K > 0 ? K : 1), sizeof(int));
  cNI = (int *)calloc((size_t)(K > 0 ? K : 1), sizeof(int));
  if (!ixB || !ixC || !alB || !alC || !nbB || !nbC || !bNI || !cNI) { free(bsorted); goto out; }
  for (int id = 0; id < bSize; ++id) {
    int pId = id + bND[id];
    ixB[2 * pId] = t->bP[2 * id];
    ixB[2 * pId + 1] = t->bP[2 * id + 1];
    alB[pId] = -100;
    nbB[pId] = -100;
  }
  for (int id = 0; id < cSize; ++id) {
    int pId = id + cND[id];
    ixC[2 * pId] = t->cP[2 * id + 2 * cStart];
    ixC[2 * pId + 1] = t->cP[2 * id + 2 * cStart + 1];
    alC[pId] = -100;
    nbC[pId] = -100;
  }
  for (int id = 0; id < K; ++id) {
    int blid = bsorted[sB[id]], clid = csorted[sC[id]];
    int bid = id, cid = id, prevblid = 0, prevclid = 0;
    if (id > 0) { prevblid = bsorted[sB[id - 1]]; prevclid = csorted[sC[id - 1]]; }
    if (id <= 0 || ub[prevblid] != ub[blid]) {
      int ty = ut[blid];
      if (ty == 2 || ty == 4 || ty == 6 || ty == 8) {
        int bId = ub[blid] / 2;
        bId += bND[bId];
        alB[bId] = aB[blid];
        bNI[blid] = bId;
        if (bid < K - 1) blid = bsorted[sB[++bid]];
      }
      int bId = ub[blid] / 2;
      int s = bND[bId], e = bND[bId + 1];
      for (int q = 0, nBId = s + bId + 1; q < e - s; ++q, ++nBId) {
        ixB[2 * nBId] = isxy[2 * blid];
        ixB[2 * nBId + 1] = isxy[2 * blid + 1];
        alB[nBId] = aB[blid];
        bNI[blid] = nBId;
        if (bid < K - 1) blid = bsorted[sB[++bid]];
      }
    }
    if (id <= 0 || uc[prevclid] != uc[clid]) {
      int ty = ut[clid];
      if (ty == 3 || ty == 4 || ty == 5 || ty == 7 || ty == 8) {
        int cId = uc[clid] / 2 - cStart;
        cId += cND[cId];
        alC[cId] = aC[clid];
        cNI[clid] = cId;
        if (cid < K - 1) clid = csorted[sC[++cid]];
      }
      int cId = uc[clid] / 2 - cStart;
      int s = cND[cId], e = cND[cId + 1];
      for (int q = 0, nCId = s + cId + 1; q < e - s; ++q, ++nCId) {
        ixC[2 * nCId] = isxy[2 * clid];
        ixC[2 * nCId + 1] = isxy[2 * clid + 1];
        alC[nCId] = aC[clid];
        cNI[clid] = nCId;
        if (cid < K - 1) clid = csorted[sC[++cid]];
      }
    }
  }
  for (int i = 0; i < K; ++i) {
    nbB[bNI[i]] = cNI[i] + 1;
    nbC[cNI[i]] = bNI[i] + 1;
  }
  free(bsorted);
  put_reals(o, SBCO_MERGED_BXY, ixB, 2L * nB);
  put_reals(o, SBCO_MERGED_CXY, ixC, 2L * nQ);
  put_ints(o, SBCO_MERGED_BALPHA, alB, nB);
  put_ints(o, SBCO_MERGED_CALPHA, alC, nQ);
  put_ints(o, SBCO_MERGED_BNB, nbB, nB);
  put_ints(o, SBCO_MERGED_CNB, nbC, nQ);

  /* components: their first source vertices (vs, ending with the vertex
   * count) and first merged slots (roots, ending with the slot count) */
  vsB = (int *)malloc(sizeof(int) * ((size_t)bSize + 1));
  vsC = (int *)malloc(sizeof(int) * ((size_t)cSize + 1));
  Ls.roots[0] = (int *)malloc(sizeof(int) * ((size_t)bSize + 1));
  Ls.roots[1] = (int *)malloc(sizeof(int) * ((size_t)cSize + 1));
  qlo = (int *)malloc(sizeof(int) * (size_t)(nQ > 0 ? nQ : 1));
  qhi = (int *)malloc(sizeof(int) * (size_t)(nQ > 0 ? nQ : 1));
  if (!vsB || !vsC || !Ls.roots[0] || !Ls.roots[1] || !qlo || !qhi) goto out;
  for (int v = 0; v < bSize; ++v)
    if (v == 0 || t->bnx[v - 1] != v) vsB[Ls.nr[0]++] = v;
  vsB[Ls.nr[0]] = bSize;
  for (int v = 0; v < cSize; ++v)
    if (v == 0 || t->cnx[cStart + v - 1] != cStart + v) vsC[Ls.nr[1]++] = v;
  vsC[Ls.nr[1]] = cSize;
  for (int k = 0; k <= Ls.nr[0]; ++k) Ls.roots[0][k] = vsB[k] + bND[vsB[k]];
  for (int k = 0; k <= Ls.nr[1]; ++k) Ls.roots[1][k] = vsC[k] + cND[vsC[k]];
  for (int k = 0; k < Ls.nr[1]; ++k)
    for (int q = Ls.roots[1][k]; q < Ls.roots[1][k + 1]; ++q) {
      qlo[q] = Ls.roots[1][k];
      qhi[q] = Ls.roots[1][k + 1];
    }

  /* calculateInitLabelParallel, oacc_segment_tree.cpp:7925-7988; the
   * circular neighbours (getCircularId :7826-7834) wrap within the slot's
   * component */
  labB = (int *)calloc((size_t)nB, sizeof(int));
  labC = (int *)calloc((size_t)nQ, sizeof(int));
  if (!labB || !labC) goto out;
  for (int bid = 0, kb = 0; bid < bSize; ++bid) {
    if (bid == vsB[kb + 1]) ++kb;
    const int lo = Ls.roots[0][kb], hi = Ls.roots[0][kb + 1];
    int s = bid + bND[bid], e = bid + bND[bid + 1] + 1;
    for (int i = s; i < e; ++i) {
      labB[i] = 0;
      if (alB[i] == -100) continue;
      double cx = ixB[2 * i], cy = ixB[2 * i + 1];
      int tm = (i - 1 < lo) ? hi - 1 : i - 1;
      double pmx = ixB[2 * tm], pmy = ixB[2 * tm + 1];
      int pMN = alB[tm] != -100 ? nbB[tm] - 1 : -100;
      int tp = (i + 1 == hi) ? lo : i + 1;
      double ppx = ixB[2 * tp], ppy = ixB[2 * tp + 1];
      int pPN = alB[tp] != -100 ? nbB[tp] - 1 : -100;
      int nId = nbB[i] - 1;
      int qt[2];
      /* a neighbour outside the overlay's slots: undefined (the reference
       * indexes past its arrays) */
      if (nId < 0 || nId >= nQ) { st = -2; goto out; }
      for (int side = 0; side < 2; ++side) {
        int q = side == 0 ? nId - 1 : nId + 1;
        if (q == qhi[nId]) q = qlo[nId];
        else if (q == qlo[nId] - 1) q = qhi[nId] - 1;
        double qx = ixC[2 * q], qy = ixC[2 * q + 1];
        int r;
        /* oracle(), :7847-7875 */
        if (pMN != -100 && pMN == q) r = 2;
        else if (pPN != -100 && pPN == q) r = 3;
        else {
          double s1 = A3(qx, qy, pmx, pmy, cx, cy);
          double s2 = A3(qx, qy, cx, cy, ppx, ppy);
          double s3 = A3(pmx, pmy, cx, cy, ppx, ppy);
          if (s3 > 0) r = (s1 > 0 && s2 > 0) ? 0 : 1;
          else r = (s1 < 0 && s2 < 0) ? 1 : 0;
        }
        qt[side] = r;
      }
      /* getInitialLabel, :7896-7920 */
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
      labC[nId] = lab;
    }
  }
  put_ints(o, SBCO_LABEL_B, labB, nB);
  put_ints(o, SBCO_LABEL_C, labC, nQ);

  /* copyToLinkedList + labelIntersections2 + createResult2 + cleanUpResult2 */
  {
    int extra = 2 * K + 8;
    int r = build_lists(&Ls, t->bP, t->cP, cStart, vsB, vsC, ixB, ixC, alB, nbC, nB, nQ, labB,
                        labC, extra);
    if (r) { st = r; goto out; }
    if (pool_init(&R.rp, nB + nQ + 2 * extra + 16)) goto out;
    r = label_and_trace(&Ls, &R);
    if (r) { st = r; goto out; }
    cleanup(&R);
  }
  /* ring output, polygon.h:576-585 (rings whose root vanished print nothing) */
  {
    int *off = (int *)malloc(sizeof(int) * ((size_t)R.nr + 1));
    long tot = 0;
    if (!off) goto out;
    int nr = 0;
    for (int r = 0; r < R.nr; ++r) {
      if (R.root[r] < 0) continue;
      int v = R.root[r];
      do { tot++; v = R.rp.next[v]; } while (v != R.root[r]);
    }
    double *xy = (double *)malloc(sizeof(double) * 2 * (size_t)(tot > 0 ? tot : 1));
    if (!xy) { free(off); goto out; }
    long w = 0;
    off[0] = 0;
    for (int r = 0; r < R.nr; ++r) {
      if (R.root[r] < 0) continue;
      int v = R.root[r];
      do {
        xy[2 * w] = R.rp.x[v];
        xy[2 * w + 1] = R.rp.y[v];
        w++;
        v = R.rp.next[v];
      } while (v != R.root[r]);
      off[++nr] = (int)w;
    }
    o->arr[SBCO_RING_OFFSETS] = off;
    o->len[SBCO_RING_OFFSETS] = nr + 1;
    o->arr[SBCO_RING_XY] = xy;
    o->len[SBCO_RING_XY] = 2 * w;
  }
  st = 0;
out:
  free(rb.a); free(rcv.a); free(rt.a);
  free(sidxDup); free(ub); free(uc); free(ut); free(csorted);
  free(bAll); free(cAll); free(bND); free(cND); free(bU); free(cU);
  free(isxy); free(ixB); free(ixC); free(aB); free(aC); free(sB); free(sC);
  free(alB); free(alC); free(nbB); free(nbC); free(bNI); free(cNI); free(labB); free(labC);
  pool_free(&Ls.P); pool_free(&Ls.Q); pool_free(&R.rp); free(R.root);
  free(Ls.roots[0]); free(Ls.roots[1]); free(vsB); free(vsC); free(qlo); free(qhi);
  if (st == -2) set_err(run, SBCO_EUNDEF, "reference behaviour undefined for this input");
  else if (st) set_err(run, SBCO_ENOMEM, "out of memory");
  return st;
}

/* component offsets: 0 = comp[0] < comp[1] < ... < comp[nc] = n, every
 * component with at least 3 vertices (NULL: one ring) */
static int comps_ok(const int *comp, int nc, int n) {
  if (!comp) return 1;
  if (nc < 1 || comp[0] != 0 || comp[nc] != n) return 0;
  for (int i = 0; i < nc; ++i)
    if (comp[i + 1] - comp[i] < 3) return 0;
  return 1;
}

static sbco_run *clip_run(const double *b_xy, int nb, const int *bcomp, int nbc,
                          const double *c_xy, const int *c_sizes, int k, const int *ccomp,
                          int ncc) {
  sbco_run *run = (sbco_run *)calloc(1, sizeof(sbco_run));
  if (!run) return NULL;
  tree_t t;
  memset(&t, 0, sizeof t);
  if (k < 1 || k > 9 || nb < 3) {
    set_err(run, SBCO_EINPUT, "need nb >= 3 and 1..9 overlays");
    return run;
  }
  if (!comps_ok(bcomp, nbc, nb) || (ccomp && (k != 1 || !comps_ok(ccomp, ncc, c_sizes[0])))) {
    set_err(run, SBCO_EINPUT, "bad component offsets");
    return run;
  }
  for (int i = 0; i < k; ++i)
    if (c_sizes[i] < 3) {
      set_err(run, SBCO_EINPUT, "overlay with fewer than 3 vertices");
      return run;
    }
  run->k = k;
  run->ov = (struct ov_out *)calloc((size_t)k, sizeof(struct ov_out));
  if (!run->ov) { set_err(run, SBCO_ENOMEM, "out of memory"); return run; }
  int r;
  if (read_input(&t, b_xy, nb, c_xy, c_sizes, k, bcomp, nbc, ccomp, ncc)) {
    set_err(run, SBCO_ENOMEM, "out of memory");
    goto done;
  }
  r = elementary(&t);
  if (r) { set_err(run, r == -2 ? SBCO_EUNDEF : SBCO_ENOMEM, "elementary intervals"); goto done; }
  if (tree_intervals(&t)) { set_err(run, SBCO_ENOMEM, "out of memory"); goto done; }
  r = leaf_end_lists(&t);
  if (r) { set_err(run, r == -2 ? SBCO_EUNDEF : SBCO_ENOMEM, "end lists"); goto done; }
  if (cover_lists(&t)) { set_err(run, SBCO_ENOMEM, "out of memory"); goto done; }
  run->stats[SBCO_STAT_EDGES] = t.E;
  run->stats[SBCO_STAT_ELEM_COUNT] = t.epc;
  run->stats[SBCO_STAT_TREE_SIZE] = t.ts;
  run->stats[SBCO_STAT_COVER_TOTAL] = t.cov_off[t.ts];
  run->stats[SBCO_STAT_LEAF_END_TOTAL] = t.leaf_off[t.numLeaves];
  /* the run keeps the tree's arrays for sbco_tree_data (the tree itself is
   * freed at the end of the run) */
  {
    const void *src[SBCO_TREE_NUM] = {t.ea, t.leaf_off, t.leaf_edge, t.cov_off, t.cov_edge};
    const long n[SBCO_TREE_NUM] = {t.epc, (long)t.numLeaves + 1, t.leaf_off[t.numLeaves],
                                   (long)t.ts + 1, t.cov_off[t.ts]};
    for (int w = 0; w < SBCO_TREE_NUM; ++w) {
      const size_t es = w == SBCO_TREE_EA ? sizeof(double) : sizeof(int);
      run->tree[w] = malloc(es * (size_t)(n[w] > 0 ? n[w] : 1));
      if (!run->tree[w]) { set_err(run, SBCO_ENOMEM, "out of memory"); goto done; }
      if (n[w]) memcpy(run->tree[w], src[w], es * (size_t)n[w]);
      run->tree_len[w] = n[w];
    }
  }
  for (int c = 1; c <= k; ++c)
    if (clip_overlay(run, &t, c)) break;
done:
  tree_free(&t);
  return run;
}

sbco_run *sbco_clip(const double *b_xy, int nb, const double *c_xy, const int *c_sizes, int k) {
  return clip_run(b_xy, nb, NULL, 0, c_xy, c_sizes, k, NULL, 0);
}

sbco_run *sbco_clip_components(const double *b_xy, int nb, const int *bcomp, int nbc,
                               const double *c_xy, int nc, const int *ccomp, int ncc) {
  return clip_run(b_xy, nb, bcomp, nbc, c_xy, &nc, 1, ccomp, ncc);
}

int sbco_status(const sbco_run *r) { return r ? r->status : SBCO_ENOMEM; }
const char *sbco_message(const sbco_run *r) { return r ? r->msg : "null run"; }

long sbco_len(const sbco_run *r, int ov, int which) {
  if (!r || !r->ov || ov < 1 || ov > r->k || which < 0 || which >= SBCO_NUM_ARRAYS) return -1;
  return r->ov[ov - 1].len[which];
}

const void *sbco_data(const sbco_run *r, int ov, int which) {
  if (!r || !r->ov || ov < 1 || ov > r->k || which < 0 || which >= SBCO_NUM_ARRAYS) return NULL;
  return r->ov[ov - 1].arr[which];
}

long sbco_stat(const sbco_run *r, int which) {
  if (!r || which < 0 || which >= SBCO_STAT_NUM) return -1;
  return r->stats[which];
}

long sbco_tree_len(const sbco_run *r, int which) {
  if (!r || which < 0 || which >= SBCO_TREE_NUM || !r->tree[which]) return -1;
  return r->tree_len[which];
}

const void *sbco_tree_data(const sbco_run *r, int which) {
  if (!r || which < 0 || which >= SBCO_TREE_NUM) return NULL;
  return r->tree[which];
}

void sbco_free(sbco_run *r) {
  if (!r) return;
  for (int w = 0; w < SBCO_TREE_NUM; ++w) free(r->tree[w]);
  if (r->ov)
    for (int i = 0; i < r->k; ++i)
      for (int w = 0; w < SBCO_NUM_ARRAYS; ++w) free(r->ov[i].arr[w]);
  free(r->ov);
  free(r);
}
