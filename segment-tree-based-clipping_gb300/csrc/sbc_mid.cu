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
// order.  The candidate stage (sbc_cand.cu) gives each unique hit the key of
// its first emission in that order; the hits of one base edge are put in key
// order here, which is the reference's first-occurrence order after its
// stable radix sort by base id.
#include <cstdio>

#include "sbc_pipeline.cuh"

namespace sbc {

namespace {

// ---------------------------------------------------------------- A9 dedup
__global__ void k_iota_keys(const int* __restrict__ rb, long long n, unsigned* __restrict__ keys,
                            unsigned* __restrict__ vals) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keys[i] = (unsigned)rb[i];
  vals[i] = (unsigned)i;
}

// hits grouped by base edge (bId = 2 x vertex index): counts, then positions
__global__ void k_bucket_count(const int* __restrict__ rb, long long n, int* __restrict__ cnt) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  atomicAdd(&cnt[rb[i] >> 1], 1);
}

__global__ void k_bucket_scatter(const int* __restrict__ rb, long long n,
                                 const int* __restrict__ start, int* __restrict__ fill,
                                 unsigned* __restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int b = rb[i] >> 1;
  out[start[b] + atomicAdd(&fill[b], 1)] = (unsigned)i;
}

// Segments (hits of one base edge, or records of one edge) longer than
// kSegShort go to a warp-per-segment ranking kernel; shorter ones are sorted
// by one thread.
constexpr int kSegShort = 16;
constexpr int kSegChunk = 256;  // entries staged per warp in shared memory

__global__ void k_dedup(const int* __restrict__ start, int nseg, const unsigned* __restrict__ svals,
                        const unsigned long long* __restrict__ rkey, const int* __restrict__ rc,
                        unsigned* __restrict__ ord, int* __restrict__ keep,
                        int* __restrict__ long_list, unsigned* __restrict__ long_count) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  int a = start[s], b = start[s + 1];
  int m = b - a;
  if (m > kSegShort) {
    long_list[atomicAdd(long_count, 1u)] = s;
    return;
  }
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

// Long segments, one warp each: an entry's place in key order is the number
// of smaller keys in its segment (keys are unique), and it is a first
// occurrence unless a smaller key has the same overlay edge.
__global__ void __launch_bounds__(256)
k_dedup_long(const int* __restrict__ start, const int* __restrict__ long_list,
             const unsigned* __restrict__ long_count, const unsigned* __restrict__ svals,
             const unsigned long long* __restrict__ rkey, const int* __restrict__ rc,
             unsigned* __restrict__ ord, int* __restrict__ keep) {
  __shared__ unsigned long long kj[8][kSegChunk];
  __shared__ int cj[8][kSegChunk];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned nl = *long_count;
  const long long nw = (long long)gridDim.x * 8;
  for (long long w = (long long)blockIdx.x * 8 + wid; w < nl; w += nw) {
    const int s = long_list[w];
    const int a = start[s], m = start[s + 1] - a;
    for (int i0 = 0; i0 < m; i0 += 32) {
      const int i = i0 + lane;
      const bool valid = i < m;
      const unsigned ri = valid ? svals[a + i] : 0u;
      const unsigned long long ki = valid ? rkey[ri] : 0ull;
      const int ci = valid ? rc[ri] : 0;
      int rank = 0;
      bool dup = false;
      for (int j0 = 0; j0 < m; j0 += kSegChunk) {
        const int cnt = min(kSegChunk, m - j0);
        __syncwarp();
        for (int t = lane; t < cnt; t += 32) {
          const unsigned r = svals[a + j0 + t];
          kj[wid][t] = rkey[r];
          cj[wid][t] = rc[r];
        }
        __syncwarp();
        for (int t = 0; t < cnt; ++t) {
          if (kj[wid][t] < ki) {
            ++rank;
            dup |= cj[wid][t] == ci;
          }
        }
      }
      if (valid) {
        ord[a + rank] = ri;
        keep[a + rank] = dup ? 0 : 1;
      }
    }
  }
}

__global__ void k_dedup_write(const unsigned* __restrict__ ord, const int* __restrict__ pos,
                              long long n, const int* __restrict__ rb, const int* __restrict__ rc,
                              const int* __restrict__ rt, const double2* __restrict__ rab,
                              int* __restrict__ ub, int* __restrict__ uc, int* __restrict__ ut,
                              double2* __restrict__ uab) {
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  if (pos[p + 1] == pos[p]) return;
  int j = pos[p];
  unsigned r = ord[p];
  ub[j] = rb[r];
  uc[j] = rc[r];
  ut[j] = rt[r];
  if (rab) uab[j] = rab[r];
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
// uab: the (alpha, beta) the exact stage computed for each record (its type
// already in ut), or nullptr to compute them here
__global__ void k_records(const int* __restrict__ ub, const int* __restrict__ uc,
                          int* __restrict__ ut, const double2* __restrict__ uab, int K,
                          const double* __restrict__ bP, const double* __restrict__ cP,
                          double* __restrict__ isxy, int* __restrict__ aB, int* __restrict__ aC) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= K) return;
  const double* b = bP + ub[j];
  const double* c = cP + uc[j];
  double al = 0.0, be = 0.0;
  int ty;
  if (uab) {
    ty = ut[j];
    const double2 ab = uab[j];
    al = ab.x;
    be = ab.y;
  } else {
    ty = seg_isect(b[0], b[1], b[2], b[3], c[0], c[1], c[2], c[3], &al, &be);
  }
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
// The identity order over all K records (coalesced), and the edges whose
// records need sorting (more than one non-degenerate intersection) appended
// to the short list (up to kSegShort records) or the long list, one atomic
// per warp and list.  Edges with at most one such record keep the identity
// (the reference sorts only those with more, :7436-7473).
__global__ void k_alpha_classify(int n, int K, const int* __restrict__ allPS,
                                 const int* __restrict__ ndPS, int* __restrict__ sorted,
                                 int* __restrict__ short_list, unsigned* __restrict__ counts,
                                 int* __restrict__ long_list) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nth = (long long)gridDim.x * blockDim.x;
  for (long long i = tid; i < K; i += nth) sorted[i] = (int)i;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  // whole warps walk the edges (the loop bound is the same for a warp)
  for (long long base = tid - lane; base < n; base += nth) {
    const long long e = base + lane;
    bool sh = false, lg = false;
    if (e < n && ndPS[e + 1] - ndPS[e] > 1) {
      lg = allPS[e + 1] - allPS[e] > kSegShort;
      sh = !lg;
    }
    const unsigned ms = __ballot_sync(0xffffffffu, sh), ml = __ballot_sync(0xffffffffu, lg);
    unsigned bs = 0, bl = 0;
    if (lane == 0) {
      if (ms) bs = atomicAdd(&counts[0], (unsigned)__popc(ms));
      if (ml) bl = atomicAdd(&counts[1], (unsigned)__popc(ml));
    }
    bs = __shfl_sync(0xffffffffu, bs, 0);
    bl = __shfl_sync(0xffffffffu, bl, 0);
    if (sh) short_list[bs + __popc(ms & lt)] = (int)e;
    if (lg) long_list[bl + __popc(ml & lt)] = (int)e;
  }
}

// Short edges of the list, one thread each: stable insertion by alpha mod 1e9.
__global__ void k_alpha_sort(const int* __restrict__ list, const unsigned* __restrict__ count,
                             const int* __restrict__ allPS, const int* __restrict__ alpha,
                             const int* __restrict__ order, int* __restrict__ sorted,
                             unsigned* __restrict__ flags) {
  const unsigned x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= *count) return;
  const int e = list[x];
  const int s = allPS[e], m = allPS[e + 1] - s;  // 2 <= m <= kSegShort
  // The run's (key, record) pairs in registers, padded past m, sorted by an
  // odd-even transposition network on (key, record): fixed indices keep the
  // arrays in registers, and the record breaking ties gives the stable order.
  int kk[kSegShort], ii[kSegShort];
  bool neg = false;
#pragma unroll
  for (int i = 0; i < kSegShort; ++i) {
    if (i < m) {
      const int a = alpha[order ? order[s + i] : s + i];
      neg |= a < 0;
      kk[i] = a % 1000000000;
      ii[i] = s + i;
    } else {
      kk[i] = INT_MAX;
      ii[i] = INT_MAX;
    }
  }
  if (neg) {
    atomicOr(flags, (unsigned)kFlagUndef);
    return;
  }
#pragma unroll
  for (int r = 0; r < kSegShort; ++r) {
#pragma unroll
    for (int i = r & 1; i + 1 < kSegShort; i += 2) {
      const bool sw = kk[i] > kk[i + 1] || (kk[i] == kk[i + 1] && ii[i] > ii[i + 1]);
      const int k0 = sw ? kk[i + 1] : kk[i], k1 = sw ? kk[i] : kk[i + 1];
      const int i0 = sw ? ii[i + 1] : ii[i], i1 = sw ? ii[i] : ii[i + 1];
      kk[i] = k0;
      kk[i + 1] = k1;
      ii[i] = i0;
      ii[i + 1] = i1;
    }
  }
#pragma unroll
  for (int i = 0; i < kSegShort; ++i)
    if (i < m) sorted[s + i] = ii[i];
}

// Long edges, one warp each: the stable position of record i is the number
// of records with a smaller alpha digit string, plus the equal ones before it.
__global__ void __launch_bounds__(256)
k_alpha_sort_long(const int* __restrict__ allPS, const int* __restrict__ long_list,
                  const unsigned* __restrict__ long_count, const int* __restrict__ alpha,
                  const int* __restrict__ order, int* __restrict__ sorted,
                  unsigned* __restrict__ flags) {
  __shared__ int kj[8][kSegChunk];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned nl = *long_count;
  const long long nw = (long long)gridDim.x * 8;
  for (long long w = (long long)blockIdx.x * 8 + wid; w < nl; w += nw) {
    const int e = long_list[w];
    const int s = allPS[e], m = allPS[e + 1] - s;
    bool neg = false;
    for (int i = lane; i < m; i += 32) neg |= alpha[order ? order[s + i] : s + i] < 0;
    if (__any_sync(0xffffffffu, neg)) {
      // undefined in the reference (a negative radix digit): the call fails
      if (lane == 0) atomicOr(flags, (unsigned)kFlagUndef);
      for (int i = lane; i < m; i += 32) sorted[s + i] = s + i;
      continue;
    }
    for (int i0 = 0; i0 < m; i0 += 32) {
      const int i = i0 + lane;
      const bool valid = i < m;
      const int ki = valid ? alpha[order ? order[s + i] : s + i] % 1000000000 : 0;
      int rank = 0;
      for (int j0 = 0; j0 < m; j0 += kSegChunk) {
        const int cnt = min(kSegChunk, m - j0);
        __syncwarp();
        for (int t = lane; t < cnt; t += 32)
          kj[wid][t] = alpha[order ? order[s + j0 + t] : s + j0 + t] % 1000000000;
        __syncwarp();
        for (int t = 0; t < cnt; ++t) {
          const int kk = kj[wid][t];
          rank += (kk < ki) || (kk == ki && j0 + t < i);
        }
      }
      if (valid) sorted[s + rank] = s + i;
    }
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
// initial label of intersection slot i (alpha != -100) of the merged base
// list.  The orientation of (prev, current, next) does not depend on the
// overlay neighbour: it is computed once, when first needed.
__device__ __forceinline__ void label_slot(int i, int nB, int nQ, const double* __restrict__ ixB,
                                           const double* __restrict__ ixC,
                                           const int* __restrict__ alB,
                                           const int* __restrict__ nbB, int* __restrict__ labB,
                                           int* __restrict__ cWin, unsigned* __restrict__ flags) {
  labB[i] = 0;
  double cx = ixB[2 * i], cy = ixB[2 * i + 1];
  int tm = (i - 1 == -1) ? nB - 1 : i - 1;  // getCircularId
  double pmx = ixB[2 * tm], pmy = ixB[2 * tm + 1];
  int pMN = alB[tm] != -100 ? nbB[tm] - 1 : -100;
  int tp = (i + 1 == nB) ? 0 : i + 1;
  double ppx = ixB[2 * tp], ppy = ixB[2 * tp + 1];
  int pPN = alB[tp] != -100 ? nbB[tp] - 1 : -100;
  int nId = nbB[i] - 1;
  int qt[2];
  double s3 = 0.0;
  bool have_s3 = false;
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
      if (!have_s3) {
        s3 = area3(pmx, pmy, cx, cy, ppx, ppy);
        have_s3 = true;
      }
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

// Only intersection slots (alpha != -100) have work, about a third of the
// slots and spread over every warp.  The orientation tests are FP64, and an
// FP64 instruction costs its issue slots whatever its active lanes: each
// block gathers its tile's intersection slots into shared memory and works
// through them with full warps.
constexpr int kLabThreads = 256, kLabItems = 8;
__global__ void __launch_bounds__(kLabThreads)
    k_labels(int nB, int nQ, const double* __restrict__ ixB, const double* __restrict__ ixC,
             const int* __restrict__ alB, const int* __restrict__ nbB, int* __restrict__ labB,
             int* __restrict__ cWin, unsigned* __restrict__ flags) {
  __shared__ int list[kLabThreads * kLabItems];
  __shared__ int wsum[kLabThreads / 32];
  __shared__ int total;
  const long long base = (long long)blockIdx.x * (kLabThreads * kLabItems);
  unsigned act = 0;
  for (int j = 0; j < kLabItems; ++j) {
    const long long i = base + (long long)j * kLabThreads + threadIdx.x;
    if (i < nB) {
      if (alB[i] != -100) act |= 1u << j;
      else labB[i] = 0;
    }
  }
  const int cnt = __popc(act);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int k2 = 0; k2 < kLabThreads / 32; ++k2) {
      const int t = wsum[k2];
      wsum[k2] = acc;
      acc += t;
    }
    total = acc;
  }
  __syncthreads();
  int pos = wsum[w] + inc - cnt;
  for (int j = 0; j < kLabItems; ++j)
    if ((act >> j) & 1u) list[pos++] = (int)(base + (long long)j * kLabThreads + threadIdx.x);
  __syncthreads();
  const int n = total;
  for (int t = threadIdx.x; t < n; t += kLabThreads)
    label_slot(list[t], nB, nQ, ixB, ixC, alB, nbB, labB, cWin, flags);
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
  // ---- A8 candidate pairs: unique hits with the key of their first emission
  int *rb = nullptr, *rc = nullptr, *rt = nullptr;
  unsigned long long* rkey = nullptr;
  long long nraw = 0;
  {
    int rc0 = stage_candidates(cType, &rb, &rc, &rt, &rkey, &nraw, out);
    if (rc0) return rc0;
  }
  return stage_records(cType, rb, rc, rt, rkey, nraw, out);
}

// A9-A18 from the candidate hits of overlay cType: base ids rb, overlay ids
// rc (offsets into the interleaved arrays), types rt, first-emission keys.
// With `unique_sorted` the hits are already A9's output (unique pairs in base
// id, then key order) and A9 is skipped.
int Pipeline::stage_records(int cType, const int* rb, const int* rc, const int* rt,
                            const unsigned long long* rkey, long long nraw, OverlayOut& out,
                            bool unique_sorted) {
  cudaStream_t st = st_;
  const int cListId = cType - 1;
  const int bSize = nb;
  const int cStart = hcS[cListId];
  const int cSize = hcS[cType] - hcS[cListId] - 1;

  // ---- A9 dedup: hits grouped by base edge (counting sort), put in key order
  // per edge, first occurrence per overlay edge kept
  long long R = nraw;
  auto* sv = (unsigned*)pool_.get("dd_vals", sizeof(unsigned) * (R + 1));
  int* segstart = (int*)pool_.get("dd_segstart", sizeof(int) * ((long long)bSize + 2));
  int* bfill = (int*)pool_.get("dd_bfill", sizeof(int) * ((long long)bSize + 2));
  auto* ord = (unsigned*)pool_.get("dd_ord", sizeof(unsigned) * (R + 1));
  int* keep = (int*)pool_.get("dd_keep", sizeof(int) * (R + 2));
  void* sscr2 = pool_.get_zeroed("scan_scr5", scan_scratch_bytes(R + 2 > bSize + 2 ? R + 2 : bSize + 2), st);
  if (pool_.failed) return fail(kENoMem, "device allocation failed (dedup)");
  int K = 0;
  const int nseg = bSize;
  if (unique_sorted) K = (int)R;
  if (R > 0 && !unique_sorted) {
    cudaMemsetAsync(segstart, 0, sizeof(int) * ((long long)bSize + 1), st);
    cudaMemsetAsync(bfill, 0, sizeof(int) * ((long long)bSize + 1), st);
    {
      ::sbc::KProbe kp_("k_bucket_count", st);
      k_bucket_count<<<grid_for(R, 256), 256, 0, st>>>(rb, R, segstart);
    }
    exclusive_scan_i32(segstart, (long long)bSize + 1, sscr2, st, true);
    {
      ::sbc::KProbe kp_("k_bucket_scatter", st);
      k_bucket_scatter<<<grid_for(R, 256), 256, 0, st>>>(rb, R, segstart, bfill, sv);
    }
    int* long_list = (int*)pool_.get("seg_long_list", sizeof(int) * ((long long)nseg + 1));
    auto* long_count = (unsigned*)pool_.get("seg_long_count", 256);
    if (pool_.failed) return fail(kENoMem, "device allocation failed (dedup lists)");
    cudaMemsetAsync(long_count, 0, sizeof(unsigned), st);
    {
      ::sbc::KProbe kp_("k_dedup", st);
      k_dedup<<<grid_for(nseg, 128), 128, 0, st>>>(segstart, nseg, sv, rkey, rc, ord, keep,
                                                   long_list, long_count);
    }
    {
      ::sbc::KProbe kp_("k_dedup_long", st);
      k_dedup_long<<<grid_for((long long)nseg * 32, 256) < 1024 ? grid_for((long long)nseg * 32, 256)
                                                                  : 1024,
                     256, 0, st>>>(segstart, long_list, long_count, sv, rkey, rc, ord, keep);
    }
    cudaMemsetAsync(keep + R, 0, sizeof(int), st);
    exclusive_scan_i32(keep, R + 1, sscr2, st, true);
    const int* r_K = rd_.get(keep + R, HostReads::kMid, st);
    cudaStreamSynchronize(st);
    K = *r_K;
  }
  out.unique = K;
  int* ub = (int*)pool_.get("u_b", sizeof(int) * (K + 1));
  int* uc = (int*)pool_.get("u_c", sizeof(int) * (K + 1));
  int* ut = (int*)pool_.get("u_t", sizeof(int) * (K + 1));
  // the exact stage's (alpha, beta) per hit, carried through the dedup
  const double2* rab = unique_sorted ? nullptr : raw_ab_;
  auto* uab = rab ? (double2*)pool_.get("u_ab", sizeof(double2) * (K + 1)) : nullptr;
  if (pool_.failed) return fail(kENoMem, "device allocation failed (unique)");
  if (K > 0 && unique_sorted) {
    cudaMemcpyAsync(ub, rb, sizeof(int) * K, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(uc, rc, sizeof(int) * K, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(ut, rt, sizeof(int) * K, cudaMemcpyDeviceToDevice, st);
  } else if (K > 0) {
    {
      ::sbc::KProbe kp_("k_dedup_write", st);
      k_dedup_write<<<grid_for(R, 256), 256, 0, st>>>(ord, keep, R, rb, rc, rt, rab, ub, uc, ut,
                                                      uab);
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
  void* sscr3 = pool_.get_zeroed(
      "scan_scr6", scan_set_scratch_bytes((long long)(bSize > cSize ? bSize : cSize) + 1, 4), st);
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
  {
    int* const arrs[4] = {bAll, bND, cAll, cND};
    const long long ns[4] = {bSize + 1, bSize + 1, cSize + 1, cSize + 1};
    exclusive_scan_i32_set(arrs, ns, 4, sscr3, st, true);
  }
  const int* r_hb = rd_.get(bND + bSize, HostReads::kMid + 1, st);
  const int* r_hc = rd_.get(cND + cSize, HostReads::kMid + 2, st);
  cudaStreamSynchronize(st);
  const int hb = *r_hb, hc = *r_hc;
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
      k_records<<<grid_for(K, 256), 256, 0, st>>>(ub, uc, ut, rab ? uab : nullptr, K, bP, cP,
                                                  isxy, aB, aC);
    }
    // ---- A12 per-edge alpha sorts
    int* along = (int*)pool_.get("alpha_long_list", sizeof(int) * ((long long)(bSize > cSize ? bSize : cSize) + 1));
    int* ashort = (int*)pool_.get("alpha_short_list", sizeof(int) * ((long long)(bSize > cSize ? bSize : cSize) + 1));
    auto* acounts = (unsigned*)pool_.get("alpha_counts", 256);  // [0] short, [1] long
    unsigned* acount = acounts + 1;
    if (pool_.failed) return fail(kENoMem, "device allocation failed (alpha lists)");
    // edges with two or more records to sort: at most K / 2 of them
    const unsigned sg = grid_for(K / 2 + 1, 128);
    const unsigned cg = grid_for((long long)(bSize > cSize ? bSize : cSize), 256) < 2048
                            ? grid_for((long long)(bSize > cSize ? bSize : cSize), 256)
                            : 2048;
    const unsigned ag = grid_for((long long)(bSize > cSize ? bSize : cSize) * 32, 256) < 1024
                            ? grid_for((long long)(bSize > cSize ? bSize : cSize) * 32, 256)
                            : 1024;
    cudaMemsetAsync(acounts, 0, 2 * sizeof(unsigned), st);
    {
      ::sbc::KProbe kp_("k_alpha_classify", st, 8.0 * bSize + 4.0 * K);
      k_alpha_classify<<<cg, 256, 0, st>>>(bSize, K, bAll, bND, sB, ashort, acounts, along);
    }
    {
      ::sbc::KProbe kp_("k_alpha_sort", st);
      k_alpha_sort<<<sg, 128, 0, st>>>(ashort, acounts, bAll, aB, nullptr, sB, d_flags);
    }
    {
      ::sbc::KProbe kp_("k_alpha_sort_long", st);
      k_alpha_sort_long<<<ag, 256, 0, st>>>(bAll, along, acount, aB, nullptr, sB, d_flags);
    }
    cudaMemsetAsync(acounts, 0, 2 * sizeof(unsigned), st);
    {
      ::sbc::KProbe kp_("k_alpha_classify", st, 8.0 * cSize + 4.0 * K);
      k_alpha_classify<<<cg, 256, 0, st>>>(cSize, K, cAll, cND, sC, ashort, acounts, along);
    }
    {
      ::sbc::KProbe kp_("k_alpha_sort", st);
      k_alpha_sort<<<sg, 128, 0, st>>>(ashort, acounts, cAll, aC, csorted, sC, d_flags);
    }
    {
      ::sbc::KProbe kp_("k_alpha_sort_long", st);
      k_alpha_sort_long<<<ag, 256, 0, st>>>(cAll, along, acount, aC, csorted, sC, d_flags);
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
    k_labels<<<grid_for(nB, kLabThreads * kLabItems), kLabThreads, 0, st>>>(
        nB, nQ, ixB, ixC, alB, nbB, labB, winC, d_flags);
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
