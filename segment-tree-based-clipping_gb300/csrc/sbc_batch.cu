// sbc_batch.cu -- many small independent base/overlay pairs in one launch,
// and the area of their intersections with its gradient.
//
// One device thread clips one pair with the same rules as the pair pipeline
// (rows A1-A18 of the reference, multicore_clipping src/clip.cpp:1415-2115),
// in order, over a private scratch arena: the elementary intervals and their
// quirks, the border search, each edge's leaf range and end leaves, the
// candidate pairs with their first-emission keys (all base x overlay edge
// pairs are tested: small pairs need no grid), the unique records, per-edge
// counts, alpha order, merged arrays, initial labels, and the exact
// linked-list back end (sbc_serial.cuh).  Results are those of
// sbc_clip_pair for every pair.
//
// Area and gradient.  The area of a pair is the sum of the shoelace areas of
// its rings.  Every ring vertex is a copy of a merged slot (base slots are
// searched first), so it is a base vertex, an overlay vertex or a proper
// crossing I = (1 - alpha) b1 + alpha b2, alpha = A(b1,c1,c2) / (A(b1,c1,c2)
// - A(b2,c1,c2)).  The forward pass stores that provenance ("tape"); the
// backward pass chains d(area)/d(vertex) through it with the combinatorial
// structure held fixed.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/sbclip.h"
#include "sbc_pipeline.cuh"
#include "sbc_pairops.cuh"
#include "sbc_pwpair.cuh"
#include "sbc_serial.cuh"

namespace sbc {

namespace {

constexpr int kBatchBlock = 128;

// ------------------------------------------------------------------ arena
// capacities of one pair
struct Caps {
  int nb, nc, E, K;        // K = capacity for unique hits
  int epcMax, nBmax, nQmax, capP, capQ, capR, rcap;
};

__host__ __device__ __forceinline__ Caps caps_of(int nb, int nc, int K) {
  Caps c;
  c.nb = nb;
  c.nc = nc;
  c.E = nb + nc;
  c.K = K;
  c.epcMax = npow2_dev(2 * c.E) + 2;
  c.nBmax = nb + K;
  c.nQmax = nc + K;
  c.capP = c.nBmax + 2 * K + 8;
  c.capQ = c.nQmax + 2 * K + 8;
  c.capR = c.nBmax + c.nQmax + 2 * (2 * K + 8) + 16;
  // ring count: the serial back end's bound, or the warp back end's
  c.rcap = (c.nBmax > 2 * K ? c.nBmax : 2 * K) + 16;
  return c;
}

// The arrays of one pair.  Carved in a fixed order from a base pointer, so a
// null base gives the byte count.
struct PairWork {
  // edges, and the order keys (okey) of their ends for comparison-only work
  double *es, *ee;
  long long *kes, *kee;
  float4* fbox;
  // elementary intervals
  int *sidx, *stmp, *vl, *vloc;
  double* ea;
  long long* kea;  // order keys of ea
  // end leaves, leaf ranges
  int *aft, *bef;
  int2* lr;
  // hits
  int *hb, *hc, *ht, *hord, *htmp;
  unsigned long long* hkey;
  double *hal, *hbt;  // lineSegmentIntersection's alpha and beta of each hit
  // counts, order, records
  int *bAll, *bND, *cAll, *cND, *cfill, *csorted;
  double* isxy;
  int *aB, *aC, *sB, *sC, *skey;
  // merged arrays
  double *ixB, *ixC;
  int *alB, *alC, *nbB, *nbC, *bNI, *cNI, *labB, *labC, *cWin, *srcB, *srcC, *recB, *recC;
  // back end
  Pool P, Q, R;
  int *rroot, *counts;
  // between the three kernels of a pair: [0] front status, [1] logL, [2] hits
  int* state;
  unsigned char *splitP, *splitQ, *crossP, *crossQ;
  // output: ring offsets, ring xy, provenance
  int* roff;
  double* rxy;
  int4* tape;
  // the warp back end (sbc_pwpair.cuh): its hits in record order, its
  // arrays, and the coordinate table of the provenance lookup (ptab
  // entries: a candidate's index, and the best provenance of its point)
  PwHit* phit;
  PwWork pw;
  int *ptab, *pbest;
  int ptabn;
  // the warp front's endpoint sort: (key, endpoint) pairs padded to a power of two
  long long* fkey;
  int* fval;
  int* eflag;  // per sorted endpoint: entries it adds to the elementary array
  unsigned long long* csort;  // the candidate sweep's overlay edges by box min x
  float4* sbox;               // their boxes in that order
  int* hsort;                 // the warp back end's hit order (a power-of-two network)
  // components: the merged slot of each component's first vertex, ending
  // with the slot count (filled by the thread back end)
  int *rootB, *rootC;
  // pair-relative successor of each vertex within its component (null: one
  // ring); not carved, set per pair
  const int* bnx = nullptr;
  const int* cnx = nullptr;
};

// successor of vertex i of an n-vertex polygon: the next vertex of its
// component (nx: pair-relative successors, null for one ring)
__device__ __forceinline__ int vsucc(const int* nx, int n, int i) {
  return nx ? nx[i] : (i + 1 == n ? 0 : i + 1);
}

__host__ __device__ __forceinline__ void carve_pool(Carver& cv, int cap, Pool& p) {
  p.x = cv.take<double>(cap);
  p.y = cv.take<double>(cap);
  p.next = cv.take<int>(cap);
  p.prev = cv.take<int>(cap);
  p.nb = cv.take<int>(cap);
  p.label = cv.take<int>(cap);
  p.enex = cv.take<int>(cap);
  p.source = cv.take<unsigned char>(cap);
  p.isect = cv.take<unsigned char>(cap);
  p.src = cv.take<int>(cap);
  p.n = 0;
  p.cap = cap;
}

__host__ __device__ __forceinline__ PairWork carve(Carver& cv, const Caps& c) {
  PairWork w;
  const int E = c.E, n2 = 2 * E, K = c.K;
  w.es = cv.take<double>(E);
  w.ee = cv.take<double>(E);
  w.kes = cv.take<long long>(E);
  w.kee = cv.take<long long>(E);
  w.fbox = cv.take<float4>(E);
  w.sidx = cv.take<int>(n2);
  w.stmp = cv.take<int>(n2);
  w.vl = cv.take<int>(E + 1);
  w.vloc = cv.take<int>(E + 1);
  w.ea = cv.take<double>(c.epcMax);
  w.kea = cv.take<long long>(c.epcMax);
  w.aft = cv.take<int>(E);
  w.bef = cv.take<int>(E);
  w.lr = cv.take<int2>(E);
  w.hb = cv.take<int>(K);
  w.hc = cv.take<int>(K);
  w.ht = cv.take<int>(K);
  w.hord = cv.take<int>(K);
  w.htmp = cv.take<int>(K);
  w.hkey = cv.take<unsigned long long>(K);
  w.hal = cv.take<double>(K);
  w.hbt = cv.take<double>(K);
  w.bAll = cv.take<int>(c.nb + 1);
  w.bND = cv.take<int>(c.nb + 1);
  w.cAll = cv.take<int>(c.nc + 1);
  w.cND = cv.take<int>(c.nc + 1);
  w.cfill = cv.take<int>(c.nc + 1);
  w.csorted = cv.take<int>(K);
  w.isxy = cv.take<double>(2 * K);
  w.aB = cv.take<int>(K);
  w.aC = cv.take<int>(K);
  w.sB = cv.take<int>(K);
  w.sC = cv.take<int>(K);
  w.skey = cv.take<int>(K);
  w.ixB = cv.take<double>(2 * c.nBmax);
  w.ixC = cv.take<double>(2 * c.nQmax);
  w.alB = cv.take<int>(c.nBmax);
  w.alC = cv.take<int>(c.nQmax);
  w.nbB = cv.take<int>(c.nBmax);
  w.nbC = cv.take<int>(c.nQmax);
  w.bNI = cv.take<int>(K);
  w.cNI = cv.take<int>(K);
  w.labB = cv.take<int>(c.nBmax);
  w.labC = cv.take<int>(c.nQmax);
  w.cWin = cv.take<int>(c.nQmax);
  w.srcB = cv.take<int>(c.nBmax);
  w.srcC = cv.take<int>(c.nQmax);
  w.recB = cv.take<int>(c.nBmax);
  w.recC = cv.take<int>(c.nQmax);
  carve_pool(cv, c.capP, w.P);
  carve_pool(cv, c.capQ, w.Q);
  carve_pool(cv, c.capR, w.R);
  w.rroot = cv.take<int>(c.rcap);
  w.counts = cv.take<int>(4);
  w.state = cv.take<int>(4);
  w.splitP = cv.take<unsigned char>(c.capP);
  w.crossP = cv.take<unsigned char>(c.capP);
  w.splitQ = cv.take<unsigned char>(c.capQ);
  w.crossQ = cv.take<unsigned char>(c.capQ);
  w.roff = cv.take<int>(c.rcap + 1);
  w.rxy = cv.take<double>(2 * (long long)c.capR);
  w.tape = cv.take<int4>(c.capR);
  w.phit = cv.take<PwHit>(K);
  w.pw = pw_carve(cv, pw_caps(c.nb, c.nc, K, 1));
  w.ptabn = npow2_dev(2 * (c.nb + c.nc + K) + 2);
  w.ptab = cv.take<int>(w.ptabn);
  w.pbest = cv.take<int>(w.ptabn);
  w.fkey = cv.take<long long>(npow2_dev(n2));
  w.fval = cv.take<int>(npow2_dev(n2));
  w.eflag = cv.take<int>(n2 + 1);
  w.csort = cv.take<unsigned long long>(npow2_dev(c.nc));
  w.sbox = cv.take<float4>(c.nc);
  w.hsort = cv.take<int>(npow2_dev(K));
  w.rootB = cv.take<int>(c.nb + 1);
  w.rootC = cv.take<int>(c.nc + 1);
  return w;
}

__host__ __device__ __forceinline__ size_t arena_bytes(int nb, int nc, int K) {
  Carver cv{nullptr, 0};
  carve(cv, caps_of(nb, nc, K));
  return (cv.off + 255) & ~(size_t)255;
}

// hit capacity of a pair: generous for star-like polygons in the first
// pass; a pair that needs more runs again with the count its first pass
// found (need)
__host__ __device__ __forceinline__ int hit_cap(int nb, int nc, int pass, int need) {
  const long long full = (long long)nb * nc;
  const long long first = (long long)nb + nc + 16;
  long long k = pass == 0 ? (first < full ? first : full) : need;
  if (k > full) k = full;
  return (int)(k > 0 ? k : 1);
}

// findBoarder over S(m) (oacc_segment_tree.cpp:420-460) with the zero
// border slot at z (the same emulation as the pair pipeline), compared on
// order keys: S(m) past the arrays is NaN in the reference, which is neither
// equal to nor below any value; kPastKey (above every finite key) does the same.
constexpr long long kPastKey = 0x7fffffffffffffffll;
struct BordersS {
  const long long* kea;
  int epc, z;
  __device__ long long S(int m) const {
    if (m < 0 || m >= epc) return kPastKey;
    if (m < z) return kea[m + 1];
    if (m == z) return 0;  // okey(0.0)
    return kea[m];
  }
  __device__ int J(int m) const { return m < z ? m : (m == z ? epc - 1 : m - 1); }
};

__device__ int find_border_s(const BordersS& B, long long q) {
  int l = 0, h = B.epc;
  while (l < h) {
    const int m = l + (h - l) / 2;
    const long long sm = B.S(m);
    if (sm == q) {
      if (B.S(m - 1) != q) {
        h = m;
        l = h;
      } else {
        h = m - 1;
      }
    } else if (sm < q) {
      l = m + 1;
    } else {
      h = m - 1;
    }
  }
  if (!(B.S(h) == q)) return -1;
  return h;
}

// emission of base edge b with overlay edge c of this pair (edge indices)
__device__ unsigned emission_s(int b, int c, int cId, const PairWork& w, int logL,
                               unsigned long long* key) {
  return emission_q(w.lr[b], w.lr[c], w.aft[b], w.bef[b], w.aft[c], w.bef[c], c, cId, logL, key);
}

struct PairResult {
  int status;
  int nrings;
  int nverts;
  double area;
  int need;  // PS_CAP: the hit count the candidate stage found
};

// ------------------------------------------------------------------ one pair
// Kernels per pair: the front (rows A1-A7, one warp), the candidate pairs
// (A8, one warp), the warp back end (A9-A18) with the thread back end for the
// pairs it hands over, and the area; w.state carries the front's status,
// logL, the hit count and the back end's route between them.
// Rows A1-A7 of one pair by one warp, in the reference's order
// (edge.h:190-202 edges; oacc_segment_tree.cpp:4513-4692 elementary
// intervals; :203-206 and :616-689 realToInt borders; findBoarder; leaf
// ranges), every loop shared among the lanes: the endpoint sort is a bitonic
// network over (key, endpoint) pairs (the stable order), the elementary
// array comes from a scan of per-endpoint entry counts.  Compares run on
// order keys (okey).
__device__ int clip_pair_front_warp(const double* b, int nb, const double* c, int nc,
                                    const Caps& cp, PairWork& w, int lane) {
  const int E = nb + nc, n2 = 2 * E;
  // ---- A1 edges; the x range on order keys (ties: the earlier vertex)
  long long kmin = LLONG_MAX, kmax = LLONG_MIN;
  int imin = INT_MAX, imax = INT_MAX;
  for (int e = lane; e < E; e += 32) {
    double a0, a1, y0, y1;
    if (e < nb) {
      const int t = vsucc(w.bnx, nb, e);
      a0 = bvx(b, nb, e);
      a1 = bvx(b, nb, t);
      y0 = bvy(b, nb, e);
      y1 = bvy(b, nb, t);
    } else {
      const int t = vsucc(w.cnx, nc, e - nb);
      a0 = bvx(c, nc, e - nb);
      a1 = bvx(c, nc, t);
      y0 = bvy(c, nc, e - nb);
      y1 = bvy(c, nc, t);
    }
    const long long k0 = okey(a0), k1 = okey(a1), ky0 = okey(y0), ky1 = okey(y1);
    if (k0 < k1) {
      w.es[e] = a0;
      w.ee[e] = a1;
      w.kes[e] = k0;
      w.kee[e] = k1;
    } else {
      w.ee[e] = a0;
      w.es[e] = a1;
      w.kee[e] = k0;
      w.kes[e] = k1;
    }
    if (k0 < kmin) {
      kmin = k0;
      imin = e;
    }
    if (k0 > kmax) {
      kmax = k0;
      imax = e;
    }
    const bool xs = k0 < k1, ys = ky0 < ky1;
    w.fbox[e] = make_float4(__double2float_rd(xs ? a0 : a1), __double2float_rd(ys ? y0 : y1),
                            __double2float_ru(xs ? a1 : a0), __double2float_ru(ys ? y1 : y0));
  }
  for (int o = 16; o > 0; o >>= 1) {
    const long long km = __shfl_xor_sync(kFullMask, kmin, o), kx = __shfl_xor_sync(kFullMask, kmax, o);
    const int im = __shfl_xor_sync(kFullMask, imin, o), ix = __shfl_xor_sync(kFullMask, imax, o);
    if (km < kmin || (km == kmin && im < imin)) {
      kmin = km;
      imin = im;
    }
    if (kx > kmax || (kx == kmax && ix < imax)) {
      kmax = kx;
      imax = ix;
    }
  }
  // the vertex values behind the extreme keys (edge e's first vertex)
  auto vx0 = [&](int e) { return e < nb ? bvx(b, nb, e) : bvx(c, nc, e - nb); };
  const double minI = vx0(imin), maxI = vx0(imax);
  __syncwarp();
  // ---- A4 elementary intervals: stable sort of the endpoints by key, the
  // endpoint index breaking ties
  auto kval = [&](int idx) { return (idx & 1) ? w.kee[idx >> 1] : w.kes[idx >> 1]; };
  auto val = [&](int idx) { return (idx & 1) ? w.ee[idx >> 1] : w.es[idx >> 1]; };
  const int np2 = npow2_dev(n2);
  for (int m = lane; m < np2; m += 32) {
    w.fkey[m] = m < n2 ? kval(m) : LLONG_MAX;
    w.fval[m] = m < n2 ? m : INT_MAX;
  }
  __syncwarp();
  // each lane takes compare-exchange pairs (m, m + j), not elements: every
  // lane works in every round
  for (int k = 2; k <= np2; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int q = lane; q < (np2 >> 1); q += 32) {
        const int m = ((q & ~(j - 1)) << 1) | (q & (j - 1)), l = m | j;
        const long long xk = w.fkey[m], yk = w.fkey[l];
        const int xv = w.fval[m], yv = w.fval[l];
        const bool gt = xk > yk || (xk == yk && xv > yv);
        if (gt == ((m & k) == 0)) {
          w.fkey[m] = yk;
          w.fkey[l] = xk;
          w.fval[m] = yv;
          w.fval[l] = xv;
        }
      }
      __syncwarp();
    }
  for (int i = lane; i < n2; i += 32) w.sidx[i] = w.fval[i];
  for (int i = lane; i <= E; i += 32) w.vl[i] = 0;
  __syncwarp();
  for (int j = lane; j < E; j += 32) {
    const int i = w.sidx[j] >> 1;
    if (w.kes[i] == w.kee[i]) w.vl[i] = 1;
  }
  __syncwarp();
  warp_excl_scan(w.vl, E + 1);
  __syncwarp();
  for (int i = lane; i < E; i += 32)
    if (w.vl[i] != w.vl[i + 1]) w.vloc[w.vl[i]] = i;
  __syncwarp();
  // entries per sorted endpoint i (0, 1, or 2 for the last pair), then their places
  for (int i = lane; i < n2 - 1; i += 32) {
    const long long k0 = kval(w.sidx[i]), k1 = kval(w.sidx[i + 1]);
    const int intvi = w.sidx[i] >> 1;
    const int comid = w.vl[i / 2];
    int n = 0;
    if (k0 != k1) {
      n = 1;
    } else if (w.kes[intvi] == w.kee[intvi]) {
      bool keep = comid == 0;
      if (!keep) {
        const int lookup = w.vloc[comid - 1];
        keep = w.kes[lookup] != w.kes[intvi] && w.kee[lookup] != w.kes[intvi];
      }
      n = keep ? 1 : 0;
    }
    if (i == n2 - 2 && k0 != k1) ++n;  // the last slot repeats v0
    w.eflag[i] = n;
  }
  if (lane == 0) w.eflag[n2 - 1] = 0;
  __syncwarp();
  const int count = warp_excl_scan(w.eflag, n2);
  __syncwarp();
  if (count < 1) return PS_UNDEF;
  double* ea = w.ea;
  long long* kea = w.kea;
  for (int i = lane; i < n2 - 1; i += 32) {
    const int at = w.eflag[i], n = (i + 1 < n2 ? w.eflag[i + 1] : count) - at;
    if (n == 0) continue;
    const int si = w.sidx[i];
    const long long k0 = kval(si), k1 = kval(w.sidx[i + 1]);
    if (k0 != k1) {
      for (int t = 0; t < n; ++t) {
        kea[at + t] = k0;
        ea[at + t] = val(si);
      }
    } else {
      kea[at] = w.kes[si >> 1];
      ea[at] = w.es[si >> 1];
    }
  }
  __syncwarp();
  const int epc = npow2_dev(count) + 1;
  for (int i = count + lane; i < epc; i += 32) {
    ea[i] = ea[count - 1];
    kea[i] = kea[count - 1];
  }
  const int L = epc - 1;
  int logL = 0;
  while ((1 << logL) < L) ++logL;
  // ---- A6 borders (realToInt keys, :203-206 with 64-bit; digit sort :616-689)
  const double absMin = fabs(minI);
  const double dv = dadd(maxI, absMin);
  if (!(dv < 2147483647.0)) return PS_UNDEF;
  int digits = 1;
  for (int iv = (int)trunc(dv); iv / 10 > 0; iv /= 10) ++digits;
  double scale = 1.0;
  for (int t = 0; t < 11 - digits; ++t) scale = dmul(scale, 10.0);
  const bool shift = minI < 0;
  __syncwarp();
  int zl = 0;
  bool bad = false;
  {
    auto key = [&](int t) -> long long {
      const double v = shift ? dmul(scale, dadd(ea[t], absMin)) : dmul(scale, ea[t]);
      return (long long)v;
    };
    for (int i = 1 + lane; i < epc; i += 32) {
      const long long ki = key(i);
      if (ki < 0 || ki >= 100000000000LL || (i + 1 < epc && key(i + 1) < ki)) bad = true;
      if (ki == 0) ++zl;
    }
  }
  if (__any_sync(kFullMask, bad)) return PS_UNDEF;
  const int z = __reduce_add_sync(kFullMask, zl);
  const BordersS B{kea, epc, z};
  for (int e = lane; e < E; e += 32) {
    int a = -1, bb = -1;
    const long long kee = w.kee[e], kes = w.kes[e];
    const int en = find_border_s(B, kee);
    const int st = find_border_s(B, kes);
    if (en >= 0) {
      const int j = B.J(en);
      int node = 0;
      if (j <= epc - 2) {
        const int i = j + 1;
        node = L + i;
        if (i != 1 && i + 1 < epc && kea[i] == kea[i + 1]) node = L + i + 1;
      }
      if (node >= L && node < 2 * L && kea[node - L] != kea[node - L + 1]) a = node;
    }
    if (st >= 0) {
      const int j = B.J(st);
      int node = 0;
      if (j <= epc - 2) node = L + j;
      if (node >= L && node < 2 * L && kea[node - L] != kea[node - L + 1]) bb = node;
    }
    w.aft[e] = a;
    w.bef[e] = bb;
    // ---- A7 leaf range [l, r1) of the edge's interval
    int lo = 0, hi = L;
    while (lo < hi) {
      const int m = (lo + hi) >> 1;
      if (kea[m] < kes) lo = m + 1;
      else hi = m;
    }
    const int l = lo;
    lo = 0;
    hi = L;
    while (lo < hi) {
      const int m = (lo + hi) >> 1;
      if (kea[m + 1] <= kee) lo = m + 1;
      else hi = m;
    }
    w.lr[e] = make_int2(l, lo > l ? lo : l);
  }
  __syncwarp();
  if (lane == 0) {
    w.state[1] = logL;
    w.state[2] = 0;
  }
  __syncwarp();
  return PS_OK;
}

// A8 for one pair by one warp: every base x overlay edge pair, float boxes
// first; lanes take the pairs in strides of 32 (coalesced overlay boxes)
// The edge pairs past the float box test and LSMF are queued per warp
// (kCandQ entries of shared memory) and classified 32 at a time, so that
// lineSegmentIntersection's FP64 work runs in full warps: only a few pairs in
// a hundred pass the filters, and FP64 run by a few lanes costs the issue
// slots of all 32.
constexpr int kCandQ = 64;
constexpr long long kSweepMin = 16384;  // pairs with more edge pairs sweep in x
template <bool kSweep, bool kComp>
__device__ void clip_pair_cand(const double* b, int nb, const double* c, int nc, const Caps& cp,
                               PairWork& w, int lane, int2* q) {
  const unsigned full = 0xffffffffu;
  // component successors only in the instantiation for batches with them
  const int* bn = kComp ? w.bnx : nullptr;
  const int* cn = kComp ? w.cnx : nullptr;
  const int logL = w.state[1];
  int nq = 0;  // queued pairs (the same in every lane)
  auto classify = [&](int count) {
    if (lane < count) {
      const int2 e = q[lane];
      const int be = e.x, j = e.y;
      const int bt2 = vsucc(bn, nb, be), ct2 = vsucc(cn, nc, j);
      const double p1x = bvx(b, nb, be), p1y = bvy(b, nb, be);
      const double p2x = bvx(b, nb, bt2), p2y = bvy(b, nb, bt2);
      const double q1x = bvx(c, nc, j), q1y = bvy(c, nc, j);
      const double q2x = bvx(c, nc, ct2), q2y = bvy(c, nc, ct2);
      double al, bt;
      const int ty = seg_isect(p1x, p1y, p2x, p2y, q1x, q1y, q2x, q2y, &al, &bt);
      unsigned long long key;
      if (ty && emission_s(be, nb + j, 2 * j, w, logL, &key) > 0) {
        // out of room: only counted, for the retry's capacity
        const int k = atomicAdd(&w.state[2], 1);
        if (k < cp.K) {
          w.hb[k] = 2 * be;
          w.hc[k] = 2 * j;
          w.ht[k] = ty;
          w.hkey[k] = key;
          w.hal[k] = al;
          w.hbt[k] = bt;
        }
      }
    }
    __syncwarp();
  };
  auto enqueue = [&](bool pass, int be, int j) {
    const unsigned m = __ballot_sync(full, pass);
    if (m == 0u) return;  // nothing to queue (the same on every lane)
    if (pass) q[nq + __popc(m & ((1u << lane) - 1u))] = make_int2(be, j);
    nq += __popc(m);
    __syncwarp();
    if (nq >= 32) {
      classify(32);
      const int rest = nq - 32;
      const int2 t = lane < rest ? q[32 + lane] : make_int2(0, 0);
      __syncwarp();
      if (lane < rest) q[lane] = t;
      nq = rest;
      __syncwarp();
    }
  };
  auto boxes_meet = [](const float4& fb, const float4& fc) {
    return !(fb.x > fc.z || fb.z < fc.x || fb.y > fc.w || fb.w < fc.y);
  };
  if constexpr (kSweep) {
    // Sweep in x: the overlay edges ordered by box min x (float order key,
    // -0 as +0); a base edge's candidates are the overlay edges with min x
    // in [its min x - the largest overlay x extent, its max x], every
    // box-overlapping pair among them.  The order comes from the front's
    // stable endpoint sort (w.sidx, by the exact x keys, so by the rounded-
    // down float keys as well): the overlay edges' min-x endpoints, compacted
    auto fk = [](float f) {
      const unsigned u = __float_as_uint(f == 0.f ? 0.f : f);
      return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    };
    {
      const int n2 = 2 * (nb + nc);
      int cnt = 0;
      for (int i0 = 0; i0 < n2; i0 += 32) {
        const int i = i0 + lane;
        const int id = i < n2 ? w.sidx[i] : 1;
        const bool take = !(id & 1) && (id >> 1) >= nb;
        const unsigned m = __ballot_sync(full, take);
        if (take) {
          const int k = (id >> 1) - nb, at = cnt + __popc(m & ((1u << lane) - 1u));
          const float4 bx = w.fbox[nb + k];
          w.csort[at] = ((unsigned long long)fk(bx.x) << 32) | (unsigned)k;
          w.sbox[at] = bx;
        }
        cnt += __popc(m);
      }
      __syncwarp();
    }
    float ext = 0.f;
    for (int k = lane; k < nc; k += 32) ext = fmaxf(ext, __fsub_ru(w.fbox[nb + k].z, w.fbox[nb + k].x));
    for (int o = 16; o > 0; o >>= 1) ext = fmaxf(ext, __shfl_xor_sync(full, ext, o));
    // first sorted position whose min-x key exceeds kx (or reaches it: ge)
    auto bound = [&](unsigned kx, bool ge) {
      int lo = 0, hi = nc;
      while (lo < hi) {
        const int m = (lo + hi) >> 1;
        const unsigned km = (unsigned)(w.csort[m] >> 32);
        if (ge ? km < kx : km <= kx) lo = m + 1;
        else hi = m;
      }
      return lo;
    };
    for (int be0 = 0; be0 < nb; be0 += 32) {
      const int be = be0 + lane;
      int k = 0, kend = 0;
      float4 fb = make_float4(0.f, 0.f, 0.f, 0.f);
      if (be < nb) {
        fb = w.fbox[be];
        k = bound(fk(__fsub_rd(fb.x, ext)), true);
        kend = bound(fk(fb.z), false);
      }
      while (__any_sync(full, k < kend)) {
        bool pass = false;
        int j = 0;
        if (k < kend) {
          const bool meet = boxes_meet(fb, w.sbox[k]);  // the boxes in sweep order
          if (meet) j = (int)(unsigned)w.csort[k];
          ++k;
          if (meet) {
            const int bt2 = vsucc(bn, nb, be), ct2 = vsucc(cn, nc, j);
            pass = lsmf_d(bvx(b, nb, be), bvy(b, nb, be), bvx(b, nb, bt2), bvy(b, nb, bt2),
                          bvx(c, nc, j), bvy(c, nc, j), bvx(c, nc, ct2), bvy(c, nc, ct2));
          }
        }
        enqueue(pass, be, j);
      }
    }
    if (nq > 0) classify(nq);
    return;
  } else {
    int be = 0, j = lane;
    while (j >= nc && be < nb) {
      j -= nc;
      ++be;
    }
    while (__any_sync(full, be < nb)) {
      bool pass = false;
      if (be < nb && boxes_meet(w.fbox[be], w.fbox[nb + j])) {
        const int bt2 = vsucc(bn, nb, be), ct2 = vsucc(cn, nc, j);
        pass = lsmf_d(bvx(b, nb, be), bvy(b, nb, be), bvx(b, nb, bt2), bvy(b, nb, bt2),
                      bvx(c, nc, j), bvy(c, nc, j), bvx(c, nc, ct2), bvy(c, nc, ct2));
      }
      enqueue(pass, be, j);
      j += 32;
      while (j >= nc && be < nb) {
        j -= nc;
        ++be;
      }
    }
    if (nq > 0) classify(nq);
  }
}

// A9-A13: records, counts, alpha order, merged arrays (one thread per pair)
__device__ PairResult clip_pair_back1(const double* b, int nb, const double* c, int nc,
                                      const Caps& cp, PairWork& w) {
  PairResult res{PS_OK, 0, 0, 0.0, 0};
  const int K = w.state[2];
  if (K > cp.K) {
    res.status = PS_CAP;
    res.need = K;
    return res;
  }
  // ---- A9 unique records in the reference's order: base id, then first key
  for (int i = 0; i < K; ++i) w.hord[i] = i;
  merge_sort(w.hord, w.htmp, K, [&](int x, int y) {
    return w.hb[x] != w.hb[y] ? w.hb[x] < w.hb[y] : w.hkey[x] < w.hkey[y];
  });
  // records in that order: ub/uc/ut = hb/hc/ht through hord
  int* ub = w.htmp;  // reuse: ub[i] = hb[hord[i]]
  for (int i = 0; i < K; ++i) ub[i] = w.hb[w.hord[i]];
  int* uc = w.skey;  // uc[i] = hc[hord[i]]
  for (int i = 0; i < K; ++i) uc[i] = w.hc[w.hord[i]];
  int* ut = w.ht;  // permuted in place through csorted below: keep a copy order
  {
    // permute types into record order using aB as temporary
    for (int i = 0; i < K; ++i) w.aB[i] = w.ht[w.hord[i]];
    for (int i = 0; i < K; ++i) ut[i] = w.aB[i];
  }
  // ---- A10 counts (countEdgeIntersections, src/clip.cpp:522-601) + scans
  for (int i = 0; i <= nb; ++i) w.bAll[i] = w.bND[i] = 0;
  for (int i = 0; i <= nc; ++i) w.cAll[i] = w.cND[i] = w.cfill[i] = 0;
  for (int i = 0; i < K; ++i) {
    const int eb = ub[i] >> 1, ec = uc[i] >> 1;
    w.bAll[eb]++;
    if (nd_b(ut[i])) w.bND[eb]++;
    w.cAll[ec]++;
    if (nd_c(ut[i])) w.cND[ec]++;
  }
  auto excl = [](int* a, int n) {
    int s = 0;
    for (int i = 0; i < n; ++i) {
      const int x = a[i];
      a[i] = s;
      s += x;
    }
  };
  excl(w.bAll, nb + 1);
  excl(w.bND, nb + 1);
  excl(w.cAll, nc + 1);
  excl(w.cND, nc + 1);
  // records stable by overlay id (radixsort of cPolLineIds, :1805)
  for (int i = 0; i < K; ++i) {
    const int ec = uc[i] >> 1;
    w.csorted[w.cAll[ec] + w.cfill[ec]++] = i;
  }
  const int nB = nb + w.bND[nb], nQ = nc + w.cND[nc];
  // components: the merged slot of each one's first vertex (a vertex starts
  // a component when the vertex before it closes its own)
  {
    int nr = 0;
    for (int v = 0; v < nb; ++v)
      if (v == 0 || vsucc(w.bnx, nb, v - 1) != v) w.rootB[nr++] = v + w.bND[v];
    w.rootB[nr] = nB;
    w.counts[2] = nr;
    nr = 0;
    for (int v = 0; v < nc; ++v)
      if (v == 0 || vsucc(w.cnx, nc, v - 1) != v) w.rootC[nr++] = v + w.cND[v];
    w.rootC[nr] = nQ;
    w.counts[3] = nr;
  }
  // ---- A11 records (saveIntersectionsParallel, :7257-7341): the type,
  // alpha and beta the candidate stage's lineSegmentIntersection found (FP64
  // work on one thread per pair costs its issue slots for a whole warp)
  for (int i = 0; i < K; ++i) {
    const int bi = ub[i] >> 1, bi2 = vsucc(w.bnx, nb, bi);
    const double p1x = bvx(b, nb, bi), p1y = bvy(b, nb, bi);
    const double p2x = bvx(b, nb, bi2), p2y = bvy(b, nb, bi2);
    const double q1x = bvx(c, nc, uc[i] >> 1), q1y = bvy(c, nc, uc[i] >> 1);
    const int h = w.hord[i];
    const double al = w.hal[h], bt = w.hbt[h];
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
  }
  // ---- A12 per-edge alpha order (sortIntersectionsAtEdgesParallel, :7436-7473)
  auto alpha_sort = [&](int n, const int* allPS, const int* ndPS, const int* alpha,
                        const int* order, int* sorted) -> bool {
    for (int i = 0; i < K; ++i) sorted[i] = i;
    for (int e = 0; e < n; ++e) {
      const int s = allPS[e], t = allPS[e + 1];
      if (ndPS[e + 1] - ndPS[e] <= 1) continue;
      for (int i = s; i < t; ++i)
        if (alpha[order ? order[i] : i] < 0) return false;
      if (t - s > 32) {  // a long run (an edge crossed many times): stable merge sort
        merge_sort(sorted + s, w.hord + s, t - s, [&](int x, int y) {
          return alpha[order ? order[x] : x] % 1000000000 < alpha[order ? order[y] : y] % 1000000000;
        });
        continue;
      }
      for (int i = s + 1; i < t; ++i) {  // stable insertion by alpha mod 1e9
        const int p = sorted[i];
        const int kp = alpha[order ? order[p] : p] % 1000000000;
        int j = i;
        while (j > s) {
          const int q = sorted[j - 1];
          if (alpha[order ? order[q] : q] % 1000000000 <= kp) break;
          sorted[j] = q;
          --j;
        }
        sorted[j] = p;
      }
    }
    return true;
  };
  if (!alpha_sort(nb, w.bAll, w.bND, w.aB, nullptr, w.sB) ||
      !alpha_sort(nc, w.cAll, w.cND, w.aC, w.csorted, w.sC)) {
    res.status = PS_UNDEF;
    return res;
  }
  // ---- A13 merged arrays (copyIntersectionsParallel, :7508-7664); unwritten
  // slots read 0 as on the reference's zero-filled heap
  for (int i = 0; i < nB; ++i) {
    w.ixB[2 * i] = w.ixB[2 * i + 1] = 0.0;
    w.alB[i] = w.nbB[i] = 0;
    w.srcB[i] = -1;
    w.recB[i] = -1;
  }
  for (int i = 0; i < nQ; ++i) {
    w.ixC[2 * i] = w.ixC[2 * i + 1] = 0.0;
    w.alC[i] = w.nbC[i] = 0;
    w.srcC[i] = -1;
    w.recC[i] = -1;
  }
  for (int id = 0; id < nb; ++id) {
    const int p = id + w.bND[id];
    w.ixB[2 * p] = bvx(b, nb, id);
    w.ixB[2 * p + 1] = bvy(b, nb, id);
    w.alB[p] = -100;
    w.nbB[p] = -100;
    w.srcB[p] = id;
  }
  for (int id = 0; id < nc; ++id) {
    const int p = id + w.cND[id];
    w.ixC[2 * p] = bvx(c, nc, id);
    w.ixC[2 * p + 1] = bvy(c, nc, id);
    w.alC[p] = -100;
    w.nbC[p] = -100;
    w.srcC[p] = id;
  }
  for (int i = 0; i < K; ++i) w.bNI[i] = w.cNI[i] = 0;
  auto copy_runs = [&](bool base, int n, const int* allPS, const int* ndPS, const int* sorted,
                       const int* order, const int* ids, const int* avals, double* ix, int* al,
                       int* NI, int* rec) {
    for (int e = 0; e < n; ++e) {
      const int s = allPS[e];
      if (allPS[e + 1] == s) continue;
      auto entry = [&](int pos) { return order ? order[sorted[pos]] : sorted[pos]; };
      int bid = s;
      int lid = entry(bid);
      const int t = ut[lid];
      const bool deg = base ? (t == 2 || t == 4 || t == 6 || t == 8)
                            : (t == 3 || t == 4 || t == 5 || t == 7 || t == 8);
      if (deg) {
        const int slot = e + ndPS[e];
        al[slot] = avals[lid];
        NI[lid] = slot;
        if (bid < K - 1) lid = entry(++bid);
      }
      const int edge = ids[lid] >> 1;
      if (edge != e) continue;
      const int ns = ndPS[e], ne = ndPS[e + 1];
      for (int q = 0; q < ne - ns; ++q) {
        const int slot = ns + e + 1 + q;
        ix[2 * slot] = w.isxy[2 * lid];
        ix[2 * slot + 1] = w.isxy[2 * lid + 1];
        al[slot] = avals[lid];
        NI[lid] = slot;
        rec[slot] = lid;
        if (bid < K - 1) lid = entry(++bid);
      }
    }
  };
  copy_runs(true, nb, w.bAll, w.bND, w.sB, nullptr, ub, w.aB, w.ixB, w.alB, w.bNI, w.recB);
  copy_runs(false, nc, w.cAll, w.cND, w.sC, w.csorted, uc, w.aC, w.ixC, w.alC, w.cNI, w.recC);
  // neighbours: the last record written to a slot wins
  for (int i = 0; i < K; ++i) {
    w.nbB[w.bNI[i]] = w.cNI[i] + 1;
    w.nbC[w.cNI[i]] = w.bNI[i] + 1;
  }
  return res;
}

// ---- A14 initial labels (calculateInitLabelParallel, :7925-7988), one warp
// per pair, a slot per lane: the orientation tests are FP64, and FP64 run
// by one thread of a warp costs the issue slots of all 32.  Reads the merged
// arrays clip_pair_back1 left in the arena; PS_UNDEF where the reference's
// behaviour is undefined.
// the component [lo, hi) of merged slot i: roots ascending, nr components
__device__ __forceinline__ int2 comp_of_slot(const int* roots, int nr, int i) {
  int lo = 0, hi = nr - 1;
  while (lo < hi) {
    const int m = (lo + hi + 1) >> 1;
    if (roots[m] <= i) lo = m;
    else hi = m - 1;
  }
  return make_int2(roots[lo], roots[lo + 1]);
}

__device__ int clip_pair_labels(int nb, int nc, PairWork& w, int lane) {
  const int nB = nb + w.bND[nb], nQ = nc + w.cND[nc];
  const int nrB = w.counts[2], nrC = w.counts[3];
  for (int q = lane; q < nQ; q += 32) w.cWin[q] = -1;
  __syncwarp();
  bool bad = false;
  for (int i = lane; i < nB; i += 32) {
    w.labB[i] = 0;
    if (w.alB[i] == -100) continue;
    const double cx = w.ixB[2 * i], cy = w.ixB[2 * i + 1];
    // getCircularId (:7826-7834) within the slot's component
    const int2 cb = comp_of_slot(w.rootB, nrB, i);
    const int tm = (i - 1 < cb.x) ? cb.y - 1 : i - 1;
    const double pmx = w.ixB[2 * tm], pmy = w.ixB[2 * tm + 1];
    const int pMN = w.alB[tm] != -100 ? w.nbB[tm] - 1 : -100;
    const int tp = (i + 1 == cb.y) ? cb.x : i + 1;
    const double ppx = w.ixB[2 * tp], ppy = w.ixB[2 * tp + 1];
    const int pPN = w.alB[tp] != -100 ? w.nbB[tp] - 1 : -100;
    const int nId = w.nbB[i] - 1;
    // a neighbour outside the overlay's slots: undefined
    if (nId < 0 || nId >= nQ) {
      bad = true;
      continue;
    }
    const int2 cq = comp_of_slot(w.rootC, nrC, nId);
    int qt[2];
    double s3 = 0.0;
    bool have_s3 = false;
    for (int side = 0; side < 2; ++side) {
      int q = side == 0 ? nId - 1 : nId + 1;
      if (q == cq.y) q = cq.x;
      else if (q == cq.x - 1) q = cq.y - 1;
      const double qx = w.ixC[2 * q], qy = w.ixC[2 * q + 1];
      int r;
      if (pMN != -100 && pMN == q) r = 2;
      else if (pPN != -100 && pPN == q) r = 3;
      else {
        const double s1 = area3(qx, qy, pmx, pmy, cx, cy);
        const double s2 = area3(qx, qy, cx, cy, ppx, ppy);
        if (!have_s3) {
          s3 = area3(pmx, pmy, cx, cy, ppx, ppy);
          have_s3 = true;
        }
        if (s3 > 0) r = (s1 > 0 && s2 > 0) ? 0 : 1;
        else r = (s1 < 0 && s2 < 0) ? 1 : 0;
      }
      qt[side] = r;
    }
    const int qm = qt[0], qp = qt[1];
    int lab;
    if ((qm == 0 && qp == 1) || (qm == 1 && qp == 0)) lab = 1;
    else if ((qm == 0 && qp == 0) || (qm == 1 && qp == 1)) lab = 2;
    else if ((qp == 3 && qm == 1) || (qm == 3 && qp == 1)) lab = 3;
    else if ((qp == 3 && qm == 0) || (qm == 3 && qp == 0)) lab = 4;
    else if ((qp == 3 && qm == 2) || (qm == 3 && qp == 2)) lab = 5;
    else if ((qm == 2 && qp == 1) || (qp == 2 && qm == 1)) lab = 6;
    else if ((qm == 2 && qp == 0) || (qp == 2 && qm == 0)) lab = 7;
    else lab = -102;
    w.labB[i] = lab;
    atomicMax(&w.cWin[nId], i);
  }
  if (__any_sync(0xffffffffu, bad)) return PS_UNDEF;
  __syncwarp();
  for (int q = lane; q < nQ; q += 32) w.labC[q] = w.cWin[q] >= 0 ? w.labB[w.cWin[q]] : 0;
  __syncwarp();
  return PS_OK;
}

// A15-A18 and the rings out, from the labelled merged arrays
__device__ PairResult clip_pair_back2(const double* b, int nb, const double* c, int nc,
                                      const Caps& cp, PairWork& w, int unite) {
  PairResult res{PS_OK, 0, 0, 0.0, 0};
  const int nB = nb + w.bND[nb], nQ = nc + w.cND[nc];
  // the record arrays clip_pair_back1 left: ub/uc in record order, ut
  const int* ub = w.htmp;
  const int* uc = w.skey;
  const int* ut = w.ht;
  // ---- A15-A18 linked-list back end
  SerialArgs a;
  a.P = w.P;
  a.Q = w.Q;
  a.R = w.R;
  a.P.n = a.Q.n = a.R.n = 0;
  a.rroot = w.rroot;
  a.rcap = cp.rcap;
  a.nrings = &w.counts[0];
  a.status = &w.counts[1];
  a.splitP = w.splitP;
  a.splitQ = w.splitQ;
  a.crossP = w.crossP;
  a.crossQ = w.crossQ;
  for (int i = 0; i < cp.capP; ++i) w.splitP[i] = w.crossP[i] = 0;
  for (int i = 0; i < cp.capQ; ++i) w.splitQ[i] = w.crossQ[i] = 0;
  a.bSize = nb;
  a.cSize = nc;
  a.cStart = 0;
  a.nB = nB;
  a.nQ = nQ;
  a.bP = b;
  a.cP = c;
  a.ixB = w.ixB;
  a.ixC = w.ixC;
  a.alB = w.alB;
  a.nbC = w.nbC;
  a.labB = w.labB;
  a.labC = w.labC;
  a.unite = unite;
  a.bnx = w.bnx;
  a.cnx = w.cnx;
  a.rootsP = w.rootB;
  a.rootsQ = w.rootC;
  a.nrP = w.counts[2];
  a.nrQ = w.counts[3];
  *a.nrings = 0;
  int st = ser_build(a);
  if (!st) {
    // list nodes built from the merged arrays sit at their slot index
    for (int v = 0; v < a.P.n; ++v) a.P.src[v] = v;
    for (int v = 0; v < a.Q.n; ++v) a.Q.src[v] = v;
    st = ser_label_trace(a);
  }
  if (!st) ser_cleanup(a);
  if (st) {
    res.status = st == 2 ? PS_UNDEF : PS_CAP;
    return res;
  }
  // ---- rings out: offsets, coordinates, provenance (the area: k_batch_area)
  int nr = 0, nv = 0;
  w.roff[0] = 0;
  for (int r = 0; r < *a.nrings; ++r) {
    const int root = a.rroot[r];
    if (root < 0) continue;
    int v = root;
    do {
      const double x = a.R.x[v], y = a.R.y[v];
      w.rxy[2 * nv] = x;
      w.rxy[2 * nv + 1] = y;
      // provenance: the merged slot the vertex was copied from, as the back
      // end recorded it; a node it made itself (a midpoint) is looked up by
      // its coordinates (base slots first)
      int4 tp = make_int4(-1, 0, 0, 0);
      const int pv = a.R.src[v];
      if (pv >= 0) {
        const int sd = pv >> 30, s = pv & 0x3fffffff;
        const int* srcS = sd ? w.srcC : w.srcB;
        const int* recS = sd ? w.recC : w.recB;
        if (srcS[s] >= 0) {
          tp = make_int4(sd, srcS[s], 0, 0);
        } else if (recS[s] >= 0) {
          const int rr = recS[s];
          tp = ut[rr] == 1 ? make_int4(2, ub[rr] >> 1, uc[rr] >> 1, 0)
                           : ((ut[rr] == 2 || ut[rr] == 6) ? make_int4(0, ub[rr] >> 1, 0, 0)
                                                           : make_int4(1, uc[rr] >> 1, 0, 0));
        }
      }
      for (int s = 0; s < nB && tp.x < 0; ++s) {
        if (w.ixB[2 * s] != x || w.ixB[2 * s + 1] != y) continue;
        if (w.srcB[s] >= 0) tp = make_int4(0, w.srcB[s], 0, 0);
        else if (w.recB[s] >= 0) {
          const int rr = w.recB[s];
          tp = ut[rr] == 1 ? make_int4(2, ub[rr] >> 1, uc[rr] >> 1, 0)
                           : ((ut[rr] == 2 || ut[rr] == 6) ? make_int4(0, ub[rr] >> 1, 0, 0)
                                                           : make_int4(1, uc[rr] >> 1, 0, 0));
        }
      }
      for (int s = 0; s < nQ && tp.x < 0; ++s) {
        if (w.ixC[2 * s] != x || w.ixC[2 * s + 1] != y) continue;
        if (w.srcC[s] >= 0) tp = make_int4(1, w.srcC[s], 0, 0);
        else if (w.recC[s] >= 0) {
          const int rr = w.recC[s];
          tp = ut[rr] == 1 ? make_int4(2, ub[rr] >> 1, uc[rr] >> 1, 0)
                           : ((ut[rr] == 2 || ut[rr] == 6) ? make_int4(0, ub[rr] >> 1, 0, 0)
                                                           : make_int4(1, uc[rr] >> 1, 0, 0));
        }
      }
      w.tape[nv] = tp;
      ++nv;
      v = a.R.next[v];
    } while (v != root);
    w.roff[++nr] = nv;
  }
  res.nrings = nr;
  res.nverts = nv;
  res.area = 0.0;  // k_batch_area
  return res;
}

// The pair's area: the sum over its rings of the shoelace, one warp per pair
// (FP64 products at the full warp rather than on one thread of each warp);
// the lanes' partial sums combine in a fixed order, so the area does not
// depend on how the batch was cut into chunks.
__device__ double pair_area_warp(const int* roff, const double* rxy, int nr, int lane) {
  double area = 0.0;
  for (int r = 0; r < nr; ++r) {
    const int first = roff[r], last = roff[r + 1];
    double s2 = 0.0;
    for (int i = first + lane; i < last; i += 32) {
      const int j = (i + 1 == last) ? first : i + 1;
      s2 = dadd(s2, dsub(dmul(rxy[2 * i], rxy[2 * j + 1]), dmul(rxy[2 * j], rxy[2 * i + 1])));
    }
    for (int o = 16; o > 0; o >>= 1) s2 = dadd(s2, __shfl_xor_sync(0xffffffffu, s2, o));
    area = dadd(area, dmul(0.5, s2));
  }
  return area;
}

// ------------------------------------------------------------------ kernels
__global__ void k_batch_size(int np, const long long* __restrict__ boff,
                             const long long* __restrict__ coff, const int* __restrict__ pass_of,
                             const int* __restrict__ need, long long* __restrict__ bytes, int maxv) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > np) return;
  if (p == np) {
    bytes[p] = 0;
    return;
  }
  const int nb = (int)(boff[p + 1] - boff[p]), nc = (int)(coff[p + 1] - coff[p]);
  const int pass = pass_of ? pass_of[p] : 0;
  const bool ok = nb >= 3 && nc >= 3 && nb <= maxv && nc <= maxv;
  bytes[p] = (ok && pass >= 0)
                 ? (long long)arena_bytes(nb, nc, hit_cap(nb, nc, pass, need ? need[p] : 0))
                 : 0;
}

// The three kernels of a chunk: per pair status, rings, vertices, area (and
// the arena holds its rings and tape).  Arguments common to the three:
struct ClipArgs {
  int np;
  const double* bxy;
  const long long* boff;
  const double* cxy;
  const long long* coff;
  const int* pass_of;  // null: every pair, pass 0

  unsigned char* arena;
  const long long* aoff;
  long long abase;
  int* need;            // written: the hit count of a pair that ran out of room
  const int* need_in;   // read: the retry pass's hit capacity
  int* status;
  int* nrings;
  int* nverts;
  double* area;
  int unite;            // union instead of intersection
  int maxv;             // the small/large split: larger polygons go to the pair pipeline
  // components: pair-relative successor of every vertex within its
  // component, indexed like bxy / cxy (null: every polygon one ring)
  const int* bnx = nullptr;
  const int* cnx = nullptr;
  __device__ bool small(int p, int* nb, int* nc) const {
    *nb = (int)(boff[p + 1] - boff[p]);
    *nc = (int)(coff[p + 1] - coff[p]);
    return *nb >= 3 && *nc >= 3 && *nb <= maxv && *nc <= maxv;
  }
  // more than one component on either side: the last vertex's successor is
  // the first vertex of a later component
  __device__ bool multi(int p, int nb, int nc) const {
    return (bnx && bnx[boff[p] + nb - 1] != 0) || (cnx && cnx[coff[p] + nc - 1] != 0);
  }
  __device__ PairWork work(int p, int nb, int nc, int pass, Caps* cp) const {
    *cp = caps_of(nb, nc, hit_cap(nb, nc, pass, need_in[p]));
    Carver cv{arena + (aoff[p] - abase), 0};
    PairWork w = carve(cv, *cp);
    w.bnx = bnx ? bnx + boff[p] : nullptr;
    w.cnx = cnx ? cnx + coff[p] : nullptr;
    return w;
  }
};

__global__ void __launch_bounds__(128) k_batch_front(ClipArgs A) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if ((t >> 5) >= A.np) return;
  const int p = (int)(t >> 5);
  const int pass = A.pass_of ? A.pass_of[p] : 0;
  if (pass < 0) return;  // settled in an earlier pass, or a large pair
  int nb, nc;
  if (!A.small(p, &nb, &nc)) {
    if (lane == 0) {
      A.status[p] = SBC_EINPUT;
      A.nrings[p] = A.nverts[p] = 0;
      A.area[p] = 0.0;
    }
    return;
  }
  Caps cp;
  PairWork w = A.work(p, nb, nc, pass, &cp);
  const int st =
      clip_pair_front_warp(A.bxy + 2 * A.boff[p], nb, A.cxy + 2 * A.coff[p], nc, cp, w, lane);
  if (lane == 0) {
    w.state[0] = st;
    if (st != PS_OK) {
      A.status[p] = st == PS_UNDEF ? SBC_EUNDEF : SBC_ENOMEM;
      A.nrings[p] = A.nverts[p] = 0;
      A.area[p] = 0.0;
    }
  }
}

// instantiations with their own register budgets: the all-pairs test for
// pairs up to kSweepMin edge pairs, the x sweep above; each with or without
// component successors
template <bool kSweep, bool kComp>
__global__ void __launch_bounds__(128) k_batch_cand(ClipArgs A) {
  __shared__ int2 s_q[4][kCandQ];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if ((t >> 5) >= A.np) return;
  const int p = (int)(t >> 5);
  const int pass = A.pass_of ? A.pass_of[p] : 0;
  int nb, nc;
  if (pass < 0 || !A.small(p, &nb, &nc)) return;
  Caps cp;
  PairWork w = A.work(p, nb, nc, pass, &cp);
  if (w.state[0] != PS_OK || ((long long)nb * nc > kSweepMin) != kSweep) return;
  clip_pair_cand<kSweep, kComp>(A.bxy + 2 * A.boff[p], nb, A.cxy + 2 * A.coff[p], nc, cp, w,
                                lane, s_q[threadIdx.x >> 5]);
}

// The back end in three kernels: A9-A13 on one thread per pair, the labels
// on one warp per pair, A15-A18 on one thread per pair.  w.state[0] carries
// a pair's failure from one to the next.
__device__ void batch_fail(const ClipArgs& A, int p, PairWork& w, int st, int need) {
  A.status[p] = st == PS_UNDEF ? SBC_EUNDEF : SBC_ENOMEM;
  if (st == PS_CAP) A.need[p] = need;
  A.nrings[p] = A.nverts[p] = 0;
  A.area[p] = 0.0;
  w.state[0] = st;
}

// ---- the warp back end: rows A9-A18 of a pair by one warp (sbc_pwpair.cuh)

// pointInPoly against the base side: the pairwise engine's functor without
// its grid (the base is small, so every base edge is tested for membership
// in a run node)
struct PipSmall {
  const double* b;
  int nb;
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
    int part = 0;
    for (int v = lane; v < P.n; v += 32) {
      const int nx = P.next[v];
      part += pip_step(last_x(P, v), last_y(P, v), P.x[nx], P.y[nx], rx, ry);
    }
    for (int u = lane; u < nb; u += 32) {
      const int u2 = u + 1 == nb ? 0 : u + 1;
      const int st = pip_step(b[2 * u], b[2 * u + 1], b[2 * u2], b[2 * u2 + 1], rx, ry);
      if (st && internal(P, u)) part += st;
    }
    return (__reduce_add_sync(kFullMask, part) % 2) != 0;
  }
};

// Provenance of ring vertices by exact coordinates, as the area oracle
// defines it: a base vertex (lowest index) first, then an overlay vertex,
// then a proper crossing (a type-1 record, first in record order).  The
// candidates are numbered in that order (base vertices, overlay vertices,
// records), so the best one for a point is the least number; an open-address
// table keyed by the point's order keys holds, per point, one candidate (to
// compare coordinates) and the least number.
__device__ __forceinline__ unsigned ptab_slot(long long kx, long long ky, int mask) {
  const unsigned long long h = (unsigned long long)kx * 0x9e3779b97f4a7c15ull ^
                               ((unsigned long long)ky + 0x632be59bd9b4e019ull) *
                                   0xc2b2ae3d27d4eb4full;
  return (unsigned)(h >> 32) & (unsigned)mask;
}

__device__ void pair_tape_warp(const double* b, int nb, const double* c, int nc, const PwWork& pw,
                               int K, PairWork& w, int nv, int lane) {
  const int T = w.ptabn, mask = T - 1;
  for (int i = lane; i < T; i += 32) {
    w.ptab[i] = -1;
    w.pbest[i] = INT_MAX;
  }
  __syncwarp();
  auto cx = [&](int t) { return t < nb ? b[2 * t] : (t < nb + nc ? c[2 * (t - nb)] : pw.isxy[2 * (t - nb - nc)]); };
  auto cy = [&](int t) {
    return t < nb ? b[2 * t + 1] : (t < nb + nc ? c[2 * (t - nb) + 1] : pw.isxy[2 * (t - nb - nc) + 1]);
  };
  const int ncand = nb + nc + K;
  for (int t = lane; t < ncand; t += 32) {
    if (t >= nb + nc && pw.ut[t - nb - nc] != 1) continue;  // crossings only
    const long long kx = okey(cx(t)), ky = okey(cy(t));
    unsigned h = ptab_slot(kx, ky, mask);
    for (int probe = 0; probe < T; ++probe) {
      const int old = atomicCAS(&w.ptab[h], -1, t);
      if (old == -1 || (okey(cx(old)) == kx && okey(cy(old)) == ky)) {
        atomicMin(&w.pbest[h], t);
        break;
      }
      h = (h + 1) & (unsigned)mask;
    }
  }
  __syncwarp();
  for (int v = lane; v < nv; v += 32) {
    const long long kx = okey(w.rxy[2 * v]), ky = okey(w.rxy[2 * v + 1]);
    unsigned h = ptab_slot(kx, ky, mask);
    int best = -1;
    for (int probe = 0; probe < T; ++probe) {
      const int t = w.ptab[h];
      if (t == -1) break;
      if (okey(cx(t)) == kx && okey(cy(t)) == ky) {
        best = w.pbest[h];
        break;
      }
      h = (h + 1) & (unsigned)mask;
    }
    int4 tp = make_int4(-1, 0, 0, 0);
    if (best >= 0 && best < nb) tp = make_int4(0, best, 0, 0);
    else if (best >= nb && best < nb + nc) tp = make_int4(1, best - nb, 0, 0);
    else if (best >= nb + nc) tp = make_int4(2, pw.ub[best - nb - nc] >> 1, pw.uc[best - nb - nc] >> 1, 0);
    w.tape[v] = tp;
  }
  __syncwarp();
}

// One warp per pair, in two kernels: the records in the reference's order
// and rows A9-A14 (k_batch_pw, w.state[3] = 2 when done), then rows A15-A18
// (k_batch_pw2).  Two kernels keep each one's code small enough for the
// instruction cache when the warps of an SM are at different steps (a third
// kernel between the lists and the labelling gains nothing).  Both run six
// blocks per SM (80 registers, some spilled): latency-bound, they gain more
// from the extra warps than the spills cost.  A pair
// whose arrays take a path the warp back end does not follow (w.state[3] = 1)
// is clipped by the thread back end below.
__global__ void __launch_bounds__(128, 6) k_batch_pw(ClipArgs A) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if ((t >> 5) >= A.np) return;
  const int p = (int)(t >> 5);
  const int pass = A.pass_of ? A.pass_of[p] : 0;
  int nb, nc;
  if (pass < 0 || !A.small(p, &nb, &nc)) return;
  Caps cp;
  PairWork w = A.work(p, nb, nc, pass, &cp);
  if (w.state[0] != PS_OK) return;
  const int K = w.state[2];
  if (K > cp.K) {
    if (lane == 0) batch_fail(A, p, w, PS_CAP, K);
    return;
  }
  // several components: the thread back end follows them
  if (A.multi(p, nb, nc)) {
    if (lane == 0) w.state[3] = 1;
    return;
  }
  // A9 order (base id, then first emission; the hit index breaks ties, as a
  // stable sort of the hits in index order would): a bitonic network over
  // the hit indices, the lanes on compare-exchange pairs
  {
    const int np = npow2_dev(K);
    for (int m = lane; m < np; m += 32) w.hsort[m] = m < K ? m : INT_MAX;
    __syncwarp();
    auto less = [&](int x, int y) {
      if (y == INT_MAX) return x != INT_MAX;
      if (x == INT_MAX) return false;
      if (w.hb[x] != w.hb[y]) return w.hb[x] < w.hb[y];
      if (w.hkey[x] != w.hkey[y]) return w.hkey[x] < w.hkey[y];
      return x < y;
    };
    for (int k = 2; k <= np; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int q = lane; q < (np >> 1); q += 32) {
          const int m = ((q & ~(j - 1)) << 1) | (q & (j - 1)), l = m | j;
          const int x = w.hsort[m], y = w.hsort[l];
          if (less(y, x) == ((m & k) == 0)) {
            w.hsort[m] = y;
            w.hsort[l] = x;
          }
        }
        __syncwarp();
      }
  }
  for (int i = lane; i < K; i += 32) {
    const int h = w.hsort[i];
    w.phit[i] = PwHit{0, w.hb[h] >> 1, w.hc[h] >> 1, w.ht[h], w.hkey[h], w.hal[h], w.hbt[h]};
  }
  __syncwarp();
  PwWork pw = w.pw;
  PwMid mid;
  const int st = pw_clip_head(A.bxy + 2 * A.boff[p], nb, A.cxy + 2 * A.coff[p], nc, w.phit,
                              pw_caps(nb, nc, K, 1), pw, &mid);
  if (st == PS_UNDEF) {
    if (lane == 0) batch_fail(A, p, w, PS_UNDEF, 0);
    return;
  }
  if (lane == 0) {
    if (st == PS_OK) pw_mid_store(mid, pw.mid);
    w.state[3] = st == PS_OK ? 2 : 1;  // PS_FALLBACK / PS_CAP: the thread back end
  }
}

__global__ void __launch_bounds__(128, 6) k_batch_pw2(ClipArgs A) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if ((t >> 5) >= A.np) return;
  const int p = (int)(t >> 5);
  const int pass = A.pass_of ? A.pass_of[p] : 0;
  int nb, nc;
  if (pass < 0 || !A.small(p, &nb, &nc)) return;
  Caps cp;
  PairWork w = A.work(p, nb, nc, pass, &cp);
  if (w.state[0] != PS_OK || w.state[3] != 2) return;
  const int K = w.state[2];
  const double* b = A.bxy + 2 * A.boff[p];
  const double* c = A.cxy + 2 * A.coff[p];
  const PwCaps pc = pw_caps(nb, nc, K, 1);
  PwWork pw = w.pw;
  PwMid mid = pw_mid_load(pw.mid);
  int nr = 0, nv = 0;
  int st = pw_clip_lists(b, nb, c, nc, pc, pw, &mid);
  if (st == PS_OK)
    st = pw_clip_trace(b, nb, c, nc, pc, pw, mid, PipSmall{b, nb, nullptr, 0}, A.unite, &nr, &nv);
  if (st != PS_OK && st != PS_UNDEF) {
    if (lane == 0) w.state[3] = 1;  // the thread back end takes the pair
    return;
  }
  if (st == PS_UNDEF) {
    if (lane == 0) batch_fail(A, p, w, PS_UNDEF, 0);
    return;
  }
  for (int r = lane; r <= nr; r += 32) w.roff[r] = pw.roff[r];
  for (int i = lane; i < 2 * nv; i += 32) w.rxy[i] = pw.rxy[i];
  __syncwarp();
  pair_tape_warp(b, nb, c, nc, pw, K, w, nv, lane);
  if (lane == 0) {
    w.state[3] = 0;
    A.status[p] = SBC_OK;
    A.nrings[p] = nr;
    A.nverts[p] = nv;
    A.area[p] = 0.0;  // k_batch_area
  }
}

__global__ void __launch_bounds__(kBatchBlock) k_batch_back(ClipArgs A) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.np) return;
  const int p = t;
  const int pass = A.pass_of ? A.pass_of[p] : 0;
  int nb, nc;
  if (pass < 0 || !A.small(p, &nb, &nc)) return;
  Caps cp;
  PairWork w = A.work(p, nb, nc, pass, &cp);
  if (w.state[0] != PS_OK || w.state[3] != 1) return;
  const PairResult r = clip_pair_back1(A.bxy + 2 * A.boff[p], nb, A.cxy + 2 * A.coff[p], nc, cp, w);
  if (r.status != PS_OK) batch_fail(A, p, w, r.status, r.need);
}

__global__ void __launch_bounds__(128) k_batch_labels(ClipArgs A) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if ((t >> 5) >= A.np) return;
  const int p = (int)(t >> 5);
  const int pass = A.pass_of ? A.pass_of[p] : 0;
  int nb, nc;
  if (pass < 0 || !A.small(p, &nb, &nc)) return;
  Caps cp;
  PairWork w = A.work(p, nb, nc, pass, &cp);
  if (w.state[0] != PS_OK || w.state[3] != 1) return;
  const int st = clip_pair_labels(nb, nc, w, lane);
  if (st != PS_OK && lane == 0) batch_fail(A, p, w, st, 0);
}

__global__ void __launch_bounds__(kBatchBlock) k_batch_back2(ClipArgs A) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.np) return;
  const int p = t;
  const int pass = A.pass_of ? A.pass_of[p] : 0;
  int nb, nc;
  if (pass < 0 || !A.small(p, &nb, &nc)) return;
  Caps cp;
  PairWork w = A.work(p, nb, nc, pass, &cp);
  if (w.state[0] != PS_OK || w.state[3] != 1) return;
  const PairResult r =
      clip_pair_back2(A.bxy + 2 * A.boff[p], nb, A.cxy + 2 * A.coff[p], nc, cp, w, A.unite);
  A.status[p] = r.status == PS_OK ? SBC_OK : (r.status == PS_UNDEF ? SBC_EUNDEF : SBC_ENOMEM);
  if (r.status == PS_CAP) A.need[p] = r.need;
  A.nrings[p] = r.nrings;
  A.nverts[p] = r.nverts;
  A.area[p] = r.area;
}

__global__ void __launch_bounds__(128) k_batch_area(ClipArgs A) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if ((t >> 5) >= A.np) return;
  const int p = (int)(t >> 5);
  const int pass = A.pass_of ? A.pass_of[p] : 0;
  int nb, nc;
  if (pass < 0 || !A.small(p, &nb, &nc) || A.status[p] != SBC_OK) return;
  Caps cp;
  PairWork w = A.work(p, nb, nc, pass, &cp);
  const double a = pair_area_warp(w.roff, w.rxy, A.nrings[p], lane);
  if (lane == 0) A.area[p] = a;
}

// the pass arrays of a recorded batch: pass 0 for every pair the forward
// pass ran (-1: a large pair or none), pass 1 for the pairs it retried
__global__ void k_graph_passes(int n, const int* __restrict__ pass, const int* __restrict__ status,
                               int* __restrict__ pass0, int* __restrict__ pass1) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  pass0[p] = (pass[p] >= 0 || status[p] == SBC_EINPUT) ? 0 : -1;
  pass1[p] = pass[p] == 1 ? 1 : -1;
}

// block sizes (threads) of the three kernels: tuning knobs, each at most
// kBatchBlock (128) and a multiple of 32
// the batch's component successors (null: one ring per polygon)
ClipArgs with_components(ClipArgs a, const int* bnx, const int* cnx) {
  a.bnx = bnx;
  a.cnx = cnx;
  return a;
}

void launch_clip(const ClipArgs& A, const BatchShape& sh, double in_bytes, cudaStream_t st) {
  {
    ::sbc::KProbe kp_("k_batch_front", st, in_bytes);
    k_batch_front<<<grid_for(32LL * A.np, sh.front), sh.front, 0, st>>>(A);
  }
  {
    ::sbc::KProbe kp_("k_batch_cand", st, in_bytes);
    if (A.bnx || A.cnx)
      k_batch_cand<false, true><<<grid_for(32LL * A.np, sh.cand), sh.cand, 0, st>>>(A);
    else
      k_batch_cand<false, false><<<grid_for(32LL * A.np, sh.cand), sh.cand, 0, st>>>(A);
  }
  {
    ::sbc::KProbe kp_("k_batch_cand_sweep", st);
    if (A.bnx || A.cnx)
      k_batch_cand<true, true><<<grid_for(32LL * A.np, sh.cand), sh.cand, 0, st>>>(A);
    else
      k_batch_cand<true, false><<<grid_for(32LL * A.np, sh.cand), sh.cand, 0, st>>>(A);
  }
  {
    ::sbc::KProbe kp_("k_batch_pw", st, in_bytes + 20.0 * A.np);
    k_batch_pw<<<grid_for(32LL * A.np, 128), 128, 0, st>>>(A);
  }
  {
    ::sbc::KProbe kp_("k_batch_pw2", st, in_bytes);
    k_batch_pw2<<<grid_for(32LL * A.np, 128), 128, 0, st>>>(A);
  }

  {
    ::sbc::KProbe kp_("k_batch_back", st, in_bytes);
    k_batch_back<<<grid_for(A.np, sh.back), sh.back, 0, st>>>(A);
  }
  {
    ::sbc::KProbe kp_("k_batch_labels", st, in_bytes);
    k_batch_labels<<<grid_for(32LL * A.np, 128), 128, 0, st>>>(A);
  }
  {
    ::sbc::KProbe kp_("k_batch_back2", st, in_bytes + 20.0 * A.np);
    k_batch_back2<<<grid_for(A.np, sh.back), sh.back, 0, st>>>(A);
  }
  {
    ::sbc::KProbe kp_("k_batch_area", st);
    k_batch_area<<<grid_for(32LL * A.np, 128), 128, 0, st>>>(A);
  }
}

__global__ void k_batch_counts(int np, const int* __restrict__ status, const int* __restrict__ nr,
                               const int* __restrict__ nv, long long* __restrict__ rpre,
                               long long* __restrict__ vpre) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > np) return;
  const bool ok = p < np && status[p] == SBC_OK;
  rpre[p] = ok ? nr[p] : 0;
  vpre[p] = ok ? nv[p] : 0;
}

// where a pair's data lives: pass 0 arena, or the retry arena (full
// capacity); offsets are relative to each arena's first pair (abase)
struct Arenas {
  const unsigned char* a0;
  const long long* off0;
  long long abase0;
  const unsigned char* a1;
  const long long* off1;
  long long abase1;
  const int* pass;  // per pair: 0, 1, or -1 (no arena: a large or invalid pair)
  const int* need;  // per pair: the retry pass's hit capacity
  __device__ const unsigned char* at(int p) const {
    return pass[p] == 1 ? a1 + (off1[p] - abase1) : a0 + (off0[p] - abase0);
  }
};

// rings of every pair packed: pair_ring[p] .. pair_ring[p+1] ring offsets;
// one warp per pair, its lanes over the ring offsets and the coordinates
__global__ void k_batch_pack(int np, const long long* __restrict__ boff,
                             const long long* __restrict__ coff, Arenas ar,
                             const int* __restrict__ status,
                             const long long* __restrict__ rpre, const long long* __restrict__ vpre,
                             long long* __restrict__ ring_off, double* __restrict__ xy) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if ((t >> 5) >= np) return;
  const int p = (int)(t >> 5);
  const long long r0 = rpre[p], v0 = vpre[p];
  const int nr = (int)(rpre[p + 1] - r0);
  if (nr == 0 || status[p] != SBC_OK || ar.pass[p] < 0) return;
  const int nb = (int)(boff[p + 1] - boff[p]), nc = (int)(coff[p + 1] - coff[p]);
  const Caps cp = caps_of(nb, nc, hit_cap(nb, nc, ar.pass[p], ar.need[p]));
  Carver cv{const_cast<unsigned char*>(ar.at(p)), 0};
  const PairWork w = carve(cv, cp);
  for (int r = lane; r < nr; r += 32) ring_off[r0 + r] = v0 + w.roff[r];
  const int nv = w.roff[nr];
  for (int i = lane; i < 2 * nv; i += 32) xy[2 * v0 + i] = w.rxy[i];
}

// d(area)/d(vertices), one warp per pair, from the forward pass's tape.  The
// lanes take 32 ring vertices at a time and compute their contributions
// (the crossings' FP64 chain rule in parallel, up to four target vertices
// each, in four rounds).  In each round the lanes naming the same vertex
// form a group (match_any) whose lowest lane sums their values in lane order
// and adds the sum: every gradient entry is summed in an order fixed by the
// rings alone, whatever the launch shape.
__global__ void __launch_bounds__(128)
k_batch_backward(int np, const double* __restrict__ bxy, const long long* __restrict__ boff,
                 const double* __restrict__ cxy, const long long* __restrict__ coff, Arenas ar,
                 const int* __restrict__ status, const int* __restrict__ nrings,
                 const double* __restrict__ gA, const int* __restrict__ bnx,
                 const int* __restrict__ cnx, double* __restrict__ gb, double* __restrict__ gc) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if ((t >> 5) >= np) return;
  const int p = (int)(t >> 5);
  const int nb = (int)(boff[p + 1] - boff[p]), nc = (int)(coff[p + 1] - coff[p]);
  double* gbp = gb + 2 * boff[p];
  double* gcp = gc + 2 * coff[p];
  for (int i = lane; i < 2 * nb; i += 32) gbp[i] = 0.0;
  for (int i = lane; i < 2 * nc; i += 32) gcp[i] = 0.0;
  if (status[p] != SBC_OK || nrings[p] == 0 || ar.pass[p] < 0) return;
  __syncwarp();
  const double* b = bxy + 2 * boff[p];
  const double* c = cxy + 2 * coff[p];
  const int* bn = bnx ? bnx + boff[p] : nullptr;
  const int* cn = cnx ? cnx + coff[p] : nullptr;
  const Caps cp = caps_of(nb, nc, hit_cap(nb, nc, ar.pass[p], ar.need[p]));
  Carver cv{const_cast<unsigned char*>(ar.at(p)), 0};
  const PairWork w = carve(cv, cp);
  const double g = gA[p];
  const int nr = nrings[p];
  for (int r = 0; r < nr; ++r) {
    const int s = w.roff[r], e = w.roff[r + 1];
    for (int i0 = s; i0 < e; i0 += 32) {
      const int i = i0 + lane;
      int tg[4] = {-1, -1, -1, -1};
      double2 vv[4];
      if (i < e) {
        const int ip = (i + 1 == e) ? s : i + 1, im = (i == s) ? e - 1 : i - 1;
        // shoelace: dA/dx_i = (y_{i+1} - y_{i-1}) / 2, dA/dy_i = (x_{i-1} - x_{i+1}) / 2
        const double gx = 0.5 * g * (w.rxy[2 * ip + 1] - w.rxy[2 * im + 1]);
        const double gy = 0.5 * g * (w.rxy[2 * im] - w.rxy[2 * ip]);
        const int4 tp = w.tape[i];
        if (tp.x == 0 || tp.x == 1) {
          tg[0] = (tp.x << 30) | tp.y;
          vv[0] = make_double2(gx, gy);
        } else if (tp.x == 2) {
          // I = (1 - alpha) b1 + alpha b2, alpha = A1 / (A1 - A2),
          // A1 = A(b1, c1, c2), A2 = A(b2, c1, c2)
          const int i1 = tp.y, i2 = vsucc(bn, nb, tp.y), j1 = tp.z, j2 = vsucc(cn, nc, tp.z);
          const double b1x = b[2 * i1], b1y = b[2 * i1 + 1], b2x = b[2 * i2], b2y = b[2 * i2 + 1];
          const double c1x = c[2 * j1], c1y = c[2 * j1 + 1], c2x = c[2 * j2], c2y = c[2 * j2 + 1];
          const double A1 = (c1x - b1x) * (c2y - b1y) - (c1y - b1y) * (c2x - b1x);
          const double A2 = (c1x - b2x) * (c2y - b2y) - (c1y - b2y) * (c2x - b2x);
          const double d = A1 - A2;
          const double al = A1 / d;
          const double ga = gx * (b2x - b1x) + gy * (b2y - b1y);  // dA/dalpha
          const double k1 = -A2 / (d * d) * ga, k2 = A1 / (d * d) * ga;  // dalpha/dA1, dalpha/dA2
          // A(P, Q, R) partials: dP = (Qy - Ry, Rx - Qx), dQ = (Ry - Py, Px - Rx),
          // dR = (Py - Qy, Qx - Px)
          tg[0] = i1;
          vv[0] = make_double2((1.0 - al) * gx + k1 * (c1y - c2y),
                               (1.0 - al) * gy + k1 * (c2x - c1x));
          tg[1] = i2;
          vv[1] = make_double2(al * gx + k2 * (c1y - c2y), al * gy + k2 * (c2x - c1x));
          tg[2] = (1 << 30) | j1;
          vv[2] = make_double2(k1 * (c2y - b1y) + k2 * (c2y - b2y),
                               k1 * (b1x - c2x) + k2 * (b2x - c2x));
          tg[3] = (1 << 30) | j2;
          vv[3] = make_double2(k1 * (b1y - c1y) + k2 * (b2y - c1y),
                               k1 * (c1x - b1x) + k2 * (c1x - b2x));
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const unsigned act = __ballot_sync(0xffffffffu, tg[j] >= 0);
        if (tg[j] >= 0) {
          const unsigned grp = __match_any_sync(act, tg[j]);
          double sx = 0.0, sy = 0.0;
          for (unsigned m = grp; m; m &= m - 1) {
            const int l = __ffs(m) - 1;
            sx += __shfl_sync(grp, vv[j].x, l);
            sy += __shfl_sync(grp, vv[j].y, l);
          }
          if (lane == __ffs(grp) - 1) {
            double* gp = (tg[j] >> 30) ? gcp : gbp;
            const int v = tg[j] & 0x3fffffff;
            gp[2 * v] += sx;
            gp[2 * v + 1] += sy;
          }
        }
        __syncwarp();
      }
    }
  }
}

// ------------------------------------------------------------------ large pairs
// A pair with a polygon above the small/large split (SBC_BATCH_MAX_VERTICES by
// default) is clipped by the pair
// pipeline.  Its ring vertices get the provenance the small-pair engine
// records, by exact coordinates: a base vertex first, then an overlay vertex,
// then a proper crossing (a type-1 record) -- candidates sorted by (x, y),
// ties in that order, and each ring vertex looked up.
__global__ void k_big_cand(int nb, int nc, int K, const double* __restrict__ b,
                           const double* __restrict__ c, const int* __restrict__ ut,
                           const double* __restrict__ isxy, unsigned long long* __restrict__ kx,
                           unsigned long long* __restrict__ ky, unsigned* __restrict__ val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = nb + nc + K;
  if (i >= n) return;
  double x, y;
  bool use = true;
  if (i < nb) {
    x = b[2 * i];
    y = b[2 * i + 1];
  } else if (i < nb + nc) {
    x = c[2 * (i - nb)];
    y = c[2 * (i - nb) + 1];
  } else {
    const int r = i - nb - nc;
    x = isxy[2 * r];
    y = isxy[2 * r + 1];
    use = ut[r] == 1;
  }
  kx[i] = use ? dkey(x) : ~0ull;
  ky[i] = use ? dkey(y) : ~0ull;
  val[i] = (unsigned)i;
}

__global__ void k_big_gather(int n, const unsigned long long* __restrict__ src,
                             const unsigned* __restrict__ val, unsigned long long* __restrict__ dst) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dst[t] = src[val[t]];
}

// tape of each ring vertex: (0, base vertex) / (1, overlay vertex) /
// (2, base edge, overlay edge) for a proper crossing / (-1) none
__global__ void k_big_tape(int nv, const double* __restrict__ xy, int n,
                           const unsigned long long* __restrict__ kxs,
                           const unsigned long long* __restrict__ kys,
                           const unsigned* __restrict__ val, int nb, int nc,
                           const int* __restrict__ ub, const int* __restrict__ uc,
                           int4* __restrict__ tape) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const unsigned long long qx = dkey(xy[2 * v]), qy = dkey(xy[2 * v + 1]);
  int lo = 0, hi = n;
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (kxs[m] < qx || (kxs[m] == qx && kys[m] < qy)) lo = m + 1;
    else hi = m;
  }
  int4 t = make_int4(-1, 0, 0, 0);
  if (lo < n && kxs[lo] == qx && kys[lo] == qy) {
    const int i = (int)val[lo];
    if (i < nb) t = make_int4(0, i, 0, 0);
    else if (i < nb + nc) t = make_int4(1, i - nb, 0, 0);
    else t = make_int4(2, ub[i - nb - nc] >> 1, uc[i - nb - nc] >> 1, 0);
  }
  tape[v] = t;
}

// signed shoelace sum over every ring of one pair: per-block partial sums
// of the vertices' cross terms, then one block adds the partials (a fixed
// order, so the result does not vary between runs)
constexpr int kAreaBlocks = 256;

__global__ void __launch_bounds__(256) k_big_area_part(int nr, int nv, const int* __restrict__ off,
                                                       const double* __restrict__ xy,
                                                       double* __restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
    int lo = 0, hi = nr;  // the ring holding vertex i
    while (hi - lo > 1) {
      const int m = (lo + hi) >> 1;
      if (off[m] <= i) lo = m;
      else hi = m;
    }
    const int j = (i + 1 == off[lo + 1]) ? off[lo] : i + 1;
    s += xy[2 * i] * xy[2 * j + 1] - xy[2 * j] * xy[2 * i + 1];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(kAreaBlocks) k_big_area_sum(const double* __restrict__ part,
                                                              double* __restrict__ area) {
  __shared__ double sh[kAreaBlocks];
  sh[threadIdx.x] = part[threadIdx.x];
  __syncthreads();
  for (int w = kAreaBlocks / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *area = 0.5 * sh[0];
}

// d(area)/d(vertices) of one large pair, one thread per ring vertex
// (contributions are added atomically: their order, and so the last bits of
// the sums, may differ between runs)
__global__ void k_big_backward(int nr, int nv, const int* __restrict__ off,
                               const double* __restrict__ xy, const int4* __restrict__ tape,
                               const double* __restrict__ b, int nb, const double* __restrict__ c,
                               int nc, double g, double* __restrict__ gb, double* __restrict__ gc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  int lo = 0, hi = nr;  // the ring holding vertex i
  while (hi - lo > 1) {
    const int m = (lo + hi) >> 1;
    if (off[m] <= i) lo = m;
    else hi = m;
  }
  const int s = off[lo], e = off[lo + 1];
  const int ip = (i + 1 == e) ? s : i + 1, im = (i == s) ? e - 1 : i - 1;
  const double gx = 0.5 * g * (xy[2 * ip + 1] - xy[2 * im + 1]);
  const double gy = 0.5 * g * (xy[2 * im] - xy[2 * ip]);
  const int4 t = tape[i];
  if (t.x == 0) {
    atomicAdd(&gb[2 * t.y], gx);
    atomicAdd(&gb[2 * t.y + 1], gy);
  } else if (t.x == 1) {
    atomicAdd(&gc[2 * t.y], gx);
    atomicAdd(&gc[2 * t.y + 1], gy);
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
    atomicAdd(&gc[2 * j1], k1 * (c2y - b1y) + k2 * (c2y - b2y));
    atomicAdd(&gc[2 * j1 + 1], k1 * (b1x - c2x) + k2 * (b2x - c2x));
    atomicAdd(&gc[2 * j2], k1 * (b1y - c1y) + k2 * (b2y - c1y));
    atomicAdd(&gc[2 * j2 + 1], k1 * (c1x - b1x) + k2 * (c1x - b2x));
  }
}

}  // namespace


// ------------------------------------------------------------------ host
// Sizes, large pairs and chunks of a batch.  Consecutive pairs whose
// first-pass arenas fit the budget form one chunk; a large pair has no arena.
int BatchRunner::plan(int np_, const long long* d_boff, const long long* d_coff, cudaStream_t st) {
  BufferPool& pool = pl_.pool();
  np = np_;
  aoff[0] = (long long*)pool.get("bt_aoff0", sizeof(long long) * (np + 1));
  aoff[1] = (long long*)pool.get("bt_aoff1", sizeof(long long) * (np + 1));
  pass = (int*)pool.get("bt_pass", sizeof(int) * (np + 1));
  need_ = (int*)pool.get("bt_need", sizeof(int) * (np + 1));
  status = (int*)pool.get("bt_status", sizeof(int) * (np + 1));
  nrings = (int*)pool.get("bt_nrings", sizeof(int) * (np + 1));
  nverts = (int*)pool.get("bt_nverts", sizeof(int) * (np + 1));
  area = (double*)pool.get("bt_area", sizeof(double) * (np + 1));
  sscr_ = pool.get("bt_scan", scan_scratch_bytes(np + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (batch)");
  h_boff_.resize(np + 1);
  h_coff_.resize(np + 1);
  h_aoff0_.resize(np + 1);
  cudaMemcpyAsync(h_boff_.data(), d_boff, sizeof(long long) * (np + 1), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(h_coff_.data(), d_coff, sizeof(long long) * (np + 1), cudaMemcpyDeviceToHost, st);
  {
    ::sbc::KProbe kp_("k_batch_size", st);
    k_batch_size<<<grid_for(np + 1, 256), 256, 0, st>>>(np, d_boff, d_coff, nullptr, nullptr,
                                                       aoff[0], split_now());
  }
  exclusive_scan_i64(aoff[0], np + 1, sscr_, st);
  cudaMemcpyAsync(h_aoff0_.data(), aoff[0], sizeof(long long) * (np + 1), cudaMemcpyDeviceToHost,
                  st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "batch sizes");
  in_verts = (double)(h_boff_[np] + h_coff_[np]);
  big_.clear();
  for (int p = 0; p < np; ++p) {
    const long long nb = h_boff_[p + 1] - h_boff_[p], nc = h_coff_[p + 1] - h_coff_[p];
    if (nb >= 3 && nc >= 3 && (nb > split_now() || nc > split_now())) {
      BigOut b;
      b.p = p;
      big_.push_back(b);
    }
  }
  long long budget = arena_budget;
  if (budget <= 0) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    budget = std::min<long long>(96LL << 30, (long long)(fr / 2));
    budget = std::max<long long>(budget, 1LL << 28);
  }
  chunks_.clear();
  for (int p0 = 0; p0 < np;) {
    // the last p1 with aoff0[p1] - aoff0[p0] <= budget (at least one pair)
    int lo = p0 + 1, hi = np;
    while (lo < hi) {
      const int m = (lo + hi + 1) / 2;
      if (h_aoff0_[m] - h_aoff0_[p0] <= budget) lo = m;
      else hi = m - 1;
    }
    chunks_.push_back({p0, lo});
    p0 = lo;
  }
  resident_ = -1;
  return kOk;
}

// The small pairs of chunk c: pass 0, then the pairs that ran out of hit
// room again with the full product.  The chunk's arenas stay resident.
int BatchRunner::run_chunk(int c, const double* d_bxy, const long long* d_boff,
                           const double* d_cxy, const long long* d_coff, cudaStream_t st) {
  BufferPool& pool = pl_.pool();
  const int p0 = chunks_[c].first, p1 = chunks_[c].second, n = p1 - p0;
  abase_[0] = h_aoff0_[p0];
  arena[0] = (unsigned char*)pool.get("bt_arena0", (size_t)(h_aoff0_[p1] - h_aoff0_[p0]) + 256);
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (batch arena)");
  // large pairs (-1) keep what the pipeline gave them; every other pair runs
  std::vector<char> is_small(n);
  std::vector<int> hp(n);
  for (int i = 0; i < n; ++i) {
    const long long nb = h_boff_[p0 + i + 1] - h_boff_[p0 + i];
    const long long nc = h_coff_[p0 + i + 1] - h_coff_[p0 + i];
    is_small[i] = nb <= split_now() && nc <= split_now();
    hp[i] = (nb >= 3 && nc >= 3 && !is_small[i]) ? -1 : 0;
  }
  cudaMemcpyAsync(pass + p0, hp.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
  // coordinates in; area, status, ring and vertex counts out
  const double in_bytes =
      16.0 * (double)(h_boff_[p1] - h_boff_[p0] + h_coff_[p1] - h_coff_[p0]);
  launch_clip(with_components(ClipArgs{n, d_bxy, d_boff + p0, d_cxy, d_coff + p0, pass + p0,
                                       arena[0], aoff[0] + p0, abase_[0], need_ + p0, need_ + p0,
                                       status + p0, nrings + p0, nverts + p0, area + p0,
                                       unite ? 1 : 0, split_now()},
                              bnx, cnx),
              shape, in_bytes, st);
  std::vector<int> hs(n);
  cudaMemcpyAsync(hs.data(), status + p0, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "batch clip");
  int retry = 0;
  for (int i = 0; i < n; ++i) {
    hp[i] = -1;
    if (is_small[i] && hs[i] == SBC_ENOMEM) {
      hp[i] = 1;
      ++retry;
    }
  }
  arena[1] = arena[0];
  abase_[1] = 0;
  if (retry) {
    cudaMemcpyAsync(pass + p0, hp.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
    {
      ::sbc::KProbe kp_("k_batch_size", st);
      k_batch_size<<<grid_for(n + 1, 256), 256, 0, st>>>(n, d_boff + p0, d_coff + p0, pass + p0,
                                                         need_ + p0, aoff[1] + p0, split_now());
    }
    exclusive_scan_i64(aoff[1] + p0, n + 1, sscr_, st);
    long long total = 0;
    cudaMemcpyAsync(&total, aoff[1] + p1, sizeof(long long), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "batch sizes");
    arena[1] = (unsigned char*)pool.get("bt_arena1", (size_t)total + 256);
    if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (batch arena)");
    launch_clip(with_components(ClipArgs{n, d_bxy, d_boff + p0, d_cxy, d_coff + p0, pass + p0,
                                         arena[1], aoff[1] + p0, 0, need_ + p0, need_ + p0,
                                         status + p0, nrings + p0, nverts + p0, area + p0,
                                         unite ? 1 : 0, split_now()},
                                bnx, cnx),
                shape, in_bytes, st);
  }
  // where each pair's data lives now: pass 0 arena, retry arena, or none
  for (int i = 0; i < n; ++i) {
    const long long nb = h_boff_[p0 + i + 1] - h_boff_[p0 + i];
    const long long nc = h_coff_[p0 + i + 1] - h_coff_[p0 + i];
    const bool ok = nb >= 3 && nc >= 3 && is_small[i];
    hp[i] = !ok ? -1 : (hp[i] == 1 ? 1 : 0);
  }
  cudaMemcpyAsync(pass + p0, hp.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "batch clip");
  resident_ = c;
  return kOk;
}

// Large pairs through the pair pipeline: rings, provenance tape and area.
int BatchRunner::run_big(const double* d_bxy, const double* d_cxy, cudaStream_t st) {
  BufferPool& pool = pl_.pool();
  for (size_t k = 0; k < big_.size(); ++k) {
    BigOut& bo = big_[k];
    const int p = bo.p;
    const int nb = (int)(h_boff_[p + 1] - h_boff_[p]), nc = (int)(h_coff_[p + 1] - h_coff_[p]);
    const double* b = d_bxy + 2 * h_boff_[p];
    const double* c = d_cxy + 2 * h_coff_[p];
    const int sizes[1] = {nc};
    pl_.clear_error();
    int rc = pl_.run(b, nb, c, sizes, 1);
    int hstat = SBC_OK;
    bo.nrings = bo.nverts = 0;
    if (rc == kEInput || rc == kEUndef) {
      hstat = rc == kEInput ? SBC_EINPUT : SBC_EUNDEF;
    } else if (rc) {
      return rc;
    } else {
      const auto& out = pl_.outputs()[0];
      bo.nrings = out.nrings;
      bo.nverts = (int)out.nverts;
      const std::string tag = std::to_string(k);
      bo.off = (int*)pool.get("bt_big_off_" + tag, sizeof(int) * (bo.nrings + 1));
      bo.xy = (double*)pool.get("bt_big_xy_" + tag, sizeof(double) * 2 * (bo.nverts + 1));
      bo.tape = (int4*)pool.get("bt_big_tape_" + tag, sizeof(int4) * (bo.nverts + 1));
      const int K = pl_.dbg_K, n = nb + nc + K;
      auto* kx = (unsigned long long*)pool.get("bt_big_kx", sizeof(unsigned long long) * (n + 1));
      auto* ky = (unsigned long long*)pool.get("bt_big_ky", sizeof(unsigned long long) * (n + 1));
      auto* k2 = (unsigned long long*)pool.get("bt_big_k2", sizeof(unsigned long long) * (n + 1));
      auto* k3 = (unsigned long long*)pool.get("bt_big_k3", sizeof(unsigned long long) * (n + 1));
      auto* val = (unsigned*)pool.get("bt_big_val", sizeof(unsigned) * (n + 1));
      auto* val2 = (unsigned*)pool.get("bt_big_val2", sizeof(unsigned) * (n + 1));
      void* rscr = pool.get("bt_big_rscr", radix_scratch_bytes(n + 1));
      if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (large pair)");
      if (bo.nrings > 0) {
        cudaMemcpyAsync(bo.off, out.d_off, sizeof(int) * (bo.nrings + 1), cudaMemcpyDeviceToDevice,
                        st);
        cudaMemcpyAsync(bo.xy, out.d_xy, sizeof(double) * 2 * bo.nverts, cudaMemcpyDeviceToDevice,
                        st);
        {
          ::sbc::KProbe kp_("k_big_cand", st, 40.0 * n);
          k_big_cand<<<grid_for(n, 256), 256, 0, st>>>(nb, nc, K, b, c, pl_.dbg_ut, pl_.dbg_isxy,
                                                       kx, ky, val);
        }
        // by y, then stably by x: sorted by (x, y), ties in candidate order
        cudaMemcpyAsync(k2, ky, sizeof(unsigned long long) * n, cudaMemcpyDeviceToDevice, st);
        radix_sort_u64(k2, val, k3, val2, n, rscr, st);
        {
          ::sbc::KProbe kp_("k_big_gather", st, 20.0 * n);
          k_big_gather<<<grid_for(n, 256), 256, 0, st>>>(n, kx, val, k2);
        }
        radix_sort_u64(k2, val, k3, val2, n, rscr, st);
        {
          ::sbc::KProbe kp_("k_big_gather", st, 20.0 * n);
          k_big_gather<<<grid_for(n, 256), 256, 0, st>>>(n, ky, val, k3);
        }
        {
          ::sbc::KProbe kp_("k_big_tape", st, 32.0 * bo.nverts);
          k_big_tape<<<grid_for(bo.nverts, 256), 256, 0, st>>>(
              bo.nverts, bo.xy, n, k2, k3, val, nb, nc, pl_.dbg_ub, pl_.dbg_uc, bo.tape);
        }
        {
          double* part = (double*)pool.get("bt_big_part", sizeof(double) * kAreaBlocks);
          if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (large pair)");
          ::sbc::KProbe kp_("k_big_area", st, 16.0 * bo.nverts);
          k_big_area_part<<<kAreaBlocks, 256, 0, st>>>(bo.nrings, bo.nverts, bo.off, bo.xy, part);
          k_big_area_sum<<<1, kAreaBlocks, 0, st>>>(part, area + p);
        }
      } else {
        cudaMemsetAsync(area + p, 0, sizeof(double), st);
      }
    }
    const int hv[3] = {hstat, bo.nrings, bo.nverts};
    cudaMemcpyAsync(status + p, &hv[0], sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(nrings + p, &hv[1], sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(nverts + p, &hv[2], sizeof(int), cudaMemcpyHostToDevice, st);
    if (hstat != SBC_OK) cudaMemsetAsync(area + p, 0, sizeof(double), st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "large pair");
    bo.ok = hstat == SBC_OK;
  }
  pl_.clear_error();
  return kOk;
}

// successor of vertex g within its component, relative to its pair's first
// vertex: comp[] holds the component starts of the batch (ending with the
// vertex count), off[] the pairs' (no component spans two pairs)
__global__ void k_comp_succ(long long nv, const long long* __restrict__ comp, long long ncomp,
                            const long long* __restrict__ off, int np, int* __restrict__ nx) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nv) return;
  auto last_le = [&](const long long* a, long long n, long long v) {
    long long lo = 0, hi = n - 1;  // a[0] <= v < a[n]
    while (lo < hi) {
      const long long m = (lo + hi + 1) >> 1;
      if (a[m] <= v) lo = m;
      else hi = m - 1;
    }
    return lo;
  };
  const long long k = last_le(comp, ncomp, g);
  const long long p = last_le(off, np, g);
  const long long t = g + 1 < comp[k + 1] ? g + 1 : comp[k];
  nx[g] = (int)(t - off[p]);
}

int BatchRunner::set_components(int np_, const long long* d_boff, const long long* d_coff,
                                const long long* d_bcomp, long long nbc,
                                const long long* d_ccomp, long long ncc, long long nbv,
                                long long ncv, cudaStream_t st) {
  key_bcomp = d_bcomp;
  key_ccomp = d_ccomp;
  bnx = cnx = nullptr;
  valid = false;
  BufferPool& pool = pl_.pool();
  int* b = d_bcomp ? (int*)pool.get("bt_bnx", sizeof(int) * (nbv + 1)) : nullptr;
  int* c = d_ccomp ? (int*)pool.get("bt_cnx", sizeof(int) * (ncv + 1)) : nullptr;
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (components)");
  if (b && nbv > 0) {
    ::sbc::KProbe kp_("k_comp_succ", st);
    k_comp_succ<<<grid_for(nbv, 256), 256, 0, st>>>(nbv, d_bcomp, nbc, d_boff, np_, b);
  }
  if (c && ncv > 0) {
    ::sbc::KProbe kp_("k_comp_succ", st);
    k_comp_succ<<<grid_for(ncv, 256), 256, 0, st>>>(ncv, d_ccomp, ncc, d_coff, np_, c);
  }
  bnx = b;
  cnx = c;
  return kOk;
}

int BatchRunner::forward(int np_, const double* d_bxy, const long long* d_boff,
                         const double* d_cxy, const long long* d_coff, cudaStream_t st) {
  valid = false;
  ++generation;
  key_b = d_bxy;
  key_c = d_cxy;
  np = np_;
  if (np <= 0) {
    valid = true;
    return kOk;
  }
  int rc = plan(np_, d_boff, d_coff, st);
  for (size_t c = 0; c < chunks_.size() && !rc; ++c)
    rc = run_chunk((int)c, d_bxy, d_boff, d_cxy, d_coff, st);
  if (!rc) rc = run_big(d_bxy, d_cxy, st);
  if (rc) return rc;
  valid = true;
  return kOk;
}

__global__ void k_big_place(int nr, const int* __restrict__ off, long long v0,
                            long long* __restrict__ ring_off) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nr) ring_off[r] = v0 + off[r];
}

int BatchRunner::rings(const double* d_bxy, const long long* d_boff, const double* d_cxy,
                       const long long* d_coff, cudaStream_t st, long long** pair_ring,
                       long long** ring_off, double** xy, long long* total_rings,
                       long long* total_verts) {
  BufferPool& pool = pl_.pool();
  long long* rpre = (long long*)pool.get("bt_rpre", sizeof(long long) * (np + 1));
  long long* vpre = (long long*)pool.get("bt_vpre", sizeof(long long) * (np + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (batch rings)");
  {
    ::sbc::KProbe kp_("k_batch_counts", st);
    k_batch_counts<<<grid_for(np + 1, 256), 256, 0, st>>>(np, status, nrings, nverts, rpre, vpre);
  }
  exclusive_scan_i64(rpre, np + 1, sscr_, st);
  exclusive_scan_i64(vpre, np + 1, sscr_, st);
  std::vector<long long> hr(np + 1), hv(np + 1);
  cudaMemcpyAsync(hr.data(), rpre, sizeof(long long) * (np + 1), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hv.data(), vpre, sizeof(long long) * (np + 1), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "batch rings");
  long long* roff = (long long*)pool.get("bt_ring_off", sizeof(long long) * (hr[np] + 1));
  double* oxy = (double*)pool.get("bt_xy", sizeof(double) * 2 * (hv[np] + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (batch rings)");
  for (size_t c = 0; c < chunks_.size(); ++c) {
    if (resident_ != (int)c) {  // recompute a chunk whose arenas were reused
      const int rc = run_chunk((int)c, d_bxy, d_boff, d_cxy, d_coff, st);
      if (rc) return rc;
    }
    const int p0 = chunks_[c].first, n = chunks_[c].second - p0;
    const Arenas ar{arena[0], aoff[0] + p0, abase_[0], arena[1], aoff[1] + p0, abase_[1], pass + p0,
                    need_ + p0};
    ::sbc::KProbe kp_("k_batch_pack", st);
    k_batch_pack<<<grid_for(32LL * n, 128), 128, 0, st>>>(n, d_boff + p0, d_coff + p0, ar,
                                                          status + p0, rpre + p0, vpre + p0, roff,
                                                          oxy);
  }
  for (const BigOut& bo : big_) {
    if (!bo.ok || bo.nrings == 0) continue;
    ::sbc::KProbe kp_("k_big_place", st);
    k_big_place<<<grid_for(bo.nrings, 256), 256, 0, st>>>(bo.nrings, bo.off, hv[bo.p],
                                                          roff + hr[bo.p]);
    cudaMemcpyAsync(oxy + 2 * hv[bo.p], bo.xy, sizeof(double) * 2 * bo.nverts,
                    cudaMemcpyDeviceToDevice, st);
  }
  cudaMemcpyAsync(roff + hr[np], &hv[np], sizeof(long long), cudaMemcpyHostToDevice, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "batch pack");
  *pair_ring = rpre;
  *ring_off = roff;
  *xy = oxy;
  *total_rings = hr[np];
  *total_verts = hv[np];
  return kOk;
}

int BatchRunner::backward(const double* d_bxy, const long long* d_boff, const double* d_cxy,
                          const long long* d_coff, const double* d_gA, double* d_gb,
                          double* d_gc, cudaStream_t st) {
  if (np <= 0) return kOk;
  for (size_t c = 0; c < chunks_.size(); ++c) {
    // a batch larger than the arena budget recomputes each chunk's forward
    if (resident_ != (int)c) {
      const int rc = run_chunk((int)c, d_bxy, d_boff, d_cxy, d_coff, st);
      if (rc) return rc;
    }
    const int p0 = chunks_[c].first, p1 = chunks_[c].second, n = p1 - p0;
    const Arenas ar{arena[0], aoff[0] + p0, abase_[0], arena[1], aoff[1] + p0, abase_[1], pass + p0,
                    need_ + p0};
    // coordinates in, one gradient per coordinate out
    ::sbc::KProbe kp_("k_batch_backward", st,
                      32.0 * (double)(h_boff_[p1] - h_boff_[p0] + h_coff_[p1] - h_coff_[p0]) +
                          8.0 * n);
    k_batch_backward<<<grid_for(32LL * n, shape.bwd), shape.bwd, 0, st>>>(
        n, d_bxy, d_boff + p0, d_cxy, d_coff + p0, ar, status + p0, nrings + p0, d_gA + p0, bnx,
        cnx, d_gb, d_gc);
  }
  for (const BigOut& bo : big_) {
    if (!bo.ok || bo.nverts == 0) continue;
    const int p = bo.p;
    const int nb = (int)(h_boff_[p + 1] - h_boff_[p]), nc = (int)(h_coff_[p + 1] - h_coff_[p]);
    double g = 0.0;
    cudaMemcpyAsync(&g, d_gA + p, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "large pair backward");
    ::sbc::KProbe kp_("k_big_backward", st, 48.0 * bo.nverts);
    k_big_backward<<<grid_for(bo.nverts, 256), 256, 0, st>>>(
        bo.nrings, bo.nverts, bo.off, bo.xy, bo.tape, d_bxy + 2 * h_boff_[p], nb,
        d_cxy + 2 * h_coff_[p], nc, g, d_gb + 2 * h_boff_[p], d_gc + 2 * h_coff_[p]);
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "batch backward");
  return kOk;
}

}  // namespace sbc

namespace sbc {

// The batch autotuner: the block size of each of the four kernels, then the
// small/large split, one knob at a time, each setting timed as forward +
// backward (CUDA events on st, the better of two runs); a change is kept only
// if it is faster.  A split below the batch's largest polygons is tried only
// when it moves at most 64 pairs to the pair pipeline (each costs about a
// millisecond there).  Results do not depend on any knob.
int BatchRunner::autotune(int np_, const double* d_bxy, const long long* d_boff,
                          const double* d_cxy, const long long* d_coff, const double* d_gA,
                          double* d_gb, double* d_gc, cudaStream_t st, double* best_ms) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return pl_.fail(kECuda, "autotune events");
  }
  const bool prof = profiling_suspend();
  auto timed = [&](double* ms) -> int {
    double best = 1e300;
    for (int r = 0; r < 2; ++r) {
      cudaEventRecord(e0, st);
      int rc = forward(np_, d_bxy, d_boff, d_cxy, d_coff, st);
      if (!rc) rc = backward(d_bxy, d_boff, d_cxy, d_coff, d_gA, d_gb, d_gc, st);
      cudaEventRecord(e1, st);
      if (rc) return rc;
      if (cudaEventSynchronize(e1) != cudaSuccess) return pl_.fail(kECuda, "autotune timing");
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      best = std::min(best, (double)t);
    }
    *ms = best;
    return kOk;
  };
  double cur = 0.0;
  int rc = timed(&cur);
  int* knobs[4] = {&shape.front, &shape.cand, &shape.back, &shape.bwd};
  for (int i = 0; i < 4 && !rc; ++i) {
    for (int b : {32, 64, 128}) {
      if (b == *knobs[i]) continue;
      const int keep = *knobs[i];
      *knobs[i] = b;
      double t = 0.0;
      rc = timed(&t);
      if (rc || !(t < cur)) *knobs[i] = keep;
      else cur = t;
      if (rc) break;
    }
  }
  for (int sp : {2048, 1024}) {
    if (rc || sp >= split) continue;
    int moved = 0;
    for (int p = 0; p < np && moved <= 64; ++p) {
      const long long nb = h_boff_[p + 1] - h_boff_[p], nc = h_coff_[p + 1] - h_coff_[p];
      const long long m = nb > nc ? nb : nc;
      if (nb >= 3 && nc >= 3 && m > sp && m <= split) ++moved;
    }
    if (moved == 0 || moved > 64) continue;
    const int keep = split;
    split = sp;
    double t = 0.0;
    rc = timed(&t);
    if (rc || !(t < cur)) split = keep;
    else cur = t;
  }
  // leave the forward state of the chosen settings
  if (!rc) rc = forward(np_, d_bxy, d_boff, d_cxy, d_coff, st);
  profiling_restore(prof);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best_ms) *best_ms = cur;
  return rc;
}

// Records the batch's area forward + backward as one CUDA graph.  The normal
// forward pass runs first: it fixes the chunk (one), the arenas and the set
// of pairs that need the retry pass with their hit capacities.  The graph
// replays pass 0, the retry pass and the backward pass on those buffers.
int BatchRunner::graph_record(int np_, const double* d_bxy, const long long* d_boff,
                              const double* d_cxy, const long long* d_coff, const double* d_gA,
                              double* d_gb, double* d_gc, double* out_area, int* out_status,
                              cudaStream_t st, cudaGraphExec_t* exec,
                              unsigned long long* kernels) {
  int rc = forward(np_, d_bxy, d_boff, d_cxy, d_coff, st);
  if (rc) return rc;
  if (np <= 0 || chunks_.size() != 1 || !big_.empty())
    return pl_.fail(kEInput, "graph capture needs a non-empty batch in one arena chunk with no "
                             "polygon above the small/large split (SBC_BATCH_MAX_VERTICES by "
                             "default)");
  BufferPool& pool = pl_.pool();
  int* pass0 = (int*)pool.get("bt_g_pass0", sizeof(int) * (np + 1));
  int* pass1 = (int*)pool.get("bt_g_pass1", sizeof(int) * (np + 1));
  int* need_rec = (int*)pool.get("bt_g_need_rec", sizeof(int) * (np + 1));
  int* need_scr = (int*)pool.get("bt_g_need_scr", sizeof(int) * (np + 1));
  if (pool.failed) return pl_.fail(kENoMem, "device allocation failed (graph)");
  {
    ::sbc::KProbe kp_("k_graph_passes", st);
    k_graph_passes<<<grid_for(np, 256), 256, 0, st>>>(np, pass, status, pass0, pass1);
  }
  cudaMemcpyAsync(need_rec, need_, sizeof(int) * np, cudaMemcpyDeviceToDevice, st);
  std::vector<int> hp(np);
  cudaMemcpyAsync(hp.data(), pass, sizeof(int) * np, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return pl_.fail(kECuda, "graph setup");
  bool retry = false;
  for (int p = 0; p < np; ++p) retry |= hp[p] == 1;
  const double in_bytes = 16.0 * in_verts;
  const bool prof = profiling_suspend();
  const unsigned long long l0 = g_launches;
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    launch_clip(with_components(ClipArgs{np, d_bxy, d_boff, d_cxy, d_coff, pass0, arena[0],
                                         aoff[0], abase_[0], need_scr, need_rec, status, nrings,
                                         nverts, area, unite ? 1 : 0, split_now()},
                                bnx, cnx),
                shape, in_bytes, st);
    if (retry)
      launch_clip(with_components(ClipArgs{np, d_bxy, d_boff, d_cxy, d_coff, pass1, arena[1],
                                           aoff[1], 0, need_scr, need_rec, status, nrings, nverts,
                                           area, unite ? 1 : 0, split_now()},
                                  bnx, cnx),
                  shape, in_bytes, st);
    const Arenas ar{arena[0], aoff[0], abase_[0], arena[1], aoff[1], 0, pass, need_rec};
    {
      ::sbc::KProbe kp_("k_batch_backward", st);
      k_batch_backward<<<grid_for(32LL * np, shape.bwd), shape.bwd, 0, st>>>(
          np, d_bxy, d_boff, d_cxy, d_coff, ar, status, nrings, d_gA, bnx, cnx, d_gb, d_gc);
    }
    if (out_area) cudaMemcpyAsync(out_area, area, sizeof(double) * np, cudaMemcpyDeviceToDevice, st);
    if (out_status)
      cudaMemcpyAsync(out_status, status, sizeof(int) * np, cudaMemcpyDeviceToDevice, st);
    e = cudaStreamEndCapture(st, &graph);
  }
  profiling_restore(prof);
  *kernels = g_launches - l0;
  g_launches = l0;
  if (e != cudaSuccess || !graph) return pl_.fail(kECuda, "graph capture");
  e = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return pl_.fail(kECuda, "graph instantiation");
  return kOk;
}

}  // namespace sbc
