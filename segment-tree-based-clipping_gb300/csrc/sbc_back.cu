// sbc_back.cu -- Greiner-Hormann / Foster back end on the merged ring arrays
// (reference rows A15-A19):
//
//  A15  copyToLinkedList        src/clip.cpp:606-695
//  A16  labelIntersections2     foster/polyclip.h:337-709
//  A17  createResult2           foster/polyclip.h:717-759
//  A18  cleanUpResult2          foster/polyclip.h:767-787
//
// The reference walks linked lists one vertex at a time.  Here the linked
// lists are the slot arrays themselves (list order == slot order), and the
// common case runs data-parallel:
//   * entry/exit flags are a prefix parity over crossing vertices, seeded by
//     a parallel point-in-polygon reduction;
//   * ring starts come from pointer jumping (the first crossing vertex of a
//     ring in list order starts it);
//   * rings are traced segment by segment (one thread per ring, O(segments)),
//     then every vertex is copied in parallel;
//   * collinear clean-up is a parallel test, with an exact per-ring pass
//     only for rings that lose vertices.
// Inputs the data-parallel path does not cover (intersection chains, bouncing
// split pairs, polygons made only of intersection vertices, inconsistent
// entry/exit structure, coordinate collisions in the list bridge) are
// detected on the device and run through `k_serial_backend`, a single-thread
// kernel that follows the reference's linked-list algorithm step by step.
#include <cooperative_groups.h>
#include <cstdio>
#include <mutex>

#include "../../include/sbclip.h"
#include "sbc_pipeline.cuh"
#include "sbc_serial.cuh"

namespace sbc {

namespace {

// scalars the fast path computes (one struct, one read-back)
struct BkScalars {
  unsigned anomaly;
  int crossCount[2];
  int firstFree[2];     // first slot that is not an intersection vertex
  int notOnOn[2];       // vertices whose label is not ON_ON
  int winding[2];       // winding number of the seed point against the other ring
  int nRings;
  int pad;
};

// ---------------------------------------------------------------- list bridge (A15)
// The per-side steps below run for P (the base list) and Q (the overlay
// list) in one launch each: blockIdx.y picks the side.

// source slots of the merged list, and copyToLinkedList's bridge check: it
// matches list vertices by coordinates, so an inserted entry equal to the
// next source vertex would be taken for it (anomaly).  Coordinates compare
// through their order keys (integer compares; ±0 equal as for the doubles).
struct SrcSide {
  int nSrc, nSlots, polyOff;
  const int* ndPS;
  const double* ix;
  const double* poly;
  unsigned char* src;
};
__global__ void k_mark_bridge(SrcSide s0, SrcSide s1, BkScalars* sc) {
  const SrcSide& a = blockIdx.y ? s1 : s0;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.nSrc) return;
  const int p = k + a.ndPS[k];
  a.src[p] = 1;
  const int b = (k + 1 < a.nSrc) ? (k + 1 + a.ndPS[k + 1]) : a.nSlots;
  const int nx = (k + 1 < a.nSrc) ? k + 1 : 0;
  const long long vx = okey(a.poly[2 * (a.polyOff + nx)]);
  const long long vy = okey(a.poly[2 * (a.polyOff + nx) + 1]);
  for (int i = p + 1; i < b; ++i)
    if (okey(a.ix[2 * i]) == vx && okey(a.ix[2 * i + 1]) == vy) atomicOr(&sc->anomaly, 1u);
}

// P: intersection flag, label; Q: flag, label, neighbour (copyToLinkedList)
struct InitArgs {
  int nB, nQ;
  const unsigned char *srcP, *srcQ;
  const int *alB, *labB, *nbC, *labC;
  unsigned char *isP, *isQ;
  int *labP, *labQ, *nbQ, *winP;
};
__global__ void k_init_PQ(InitArgs A, BkScalars* sc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (blockIdx.y == 0) {
    if (i >= A.nB) return;
    A.isP[i] = (!A.srcP[i] || A.alB[i] != -100) ? 1 : 0;
    A.labP[i] = A.labB[i];
    return;
  }
  if (i >= A.nQ) return;
  const bool is = !A.srcQ[i] || A.nbC[i] != -100;
  A.isQ[i] = is ? 1 : 0;
  A.labQ[i] = A.labC[i];
  A.nbQ[i] = -1;
  if (is) {
    const int t = A.nbC[i] - 1;
    if (t < 0 || t >= A.nB) {
      atomicOr(&sc->anomaly, 2u);
      return;
    }
    A.nbQ[i] = t;
    atomicMax(&A.winP[t], i);  // the last C vertex linked to t wins
  }
}

struct ListSide {
  int n;
  const unsigned char* isect;
  const int* lab;
};

// per-side statistics: crossing count, first non-intersection slot, ON_ON;
// chains of ON labels are an anomaly on P only
__global__ void k_side_stats(ListSide s0, ListSide s1, BkScalars* sc) {
  const ListSide& a = blockIdx.y ? s1 : s0;
  const int side = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int cross = 0, notonon = 0;
  unsigned free_i = 0xffffffffu;  // first slot without an intersection, per warp first
  if (i < a.n) {
    const int l = a.lab[i];
    const bool is = a.isect[i] != 0;
    if (is && l == L_CROSSING) cross = 1;
    if (l != L_ON_ON) notonon = 1;
    if (!is) free_i = (unsigned)i;
    if (side == 0 && is && (l == L_LEFT_ON || l == L_RIGHT_ON)) atomicOr(&sc->anomaly, 4u);
    if (l == L_DCROSS || l == L_DBOUNCE) atomicOr(&sc->anomaly, 4u);
  }
  cross = block_sum(cross);
  notonon = block_sum(notonon);
  free_i = block_min(free_i);
  if (threadIdx.x == 0) {
    if (cross) atomicAdd(&sc->crossCount[side], cross);
    if (notonon) atomicAdd(&sc->notOnOn[side], notonon);
    if (free_i != 0xffffffffu) atomicMin(&sc->firstFree[side], (int)free_i);
  }
}

// pointInPoly (foster/polygon.h:427-448) as a reduction over the ring's
// edges: side 0 tests P's first free slot against ring Q (winding[0]), side
// 1 Q's first free slot against ring P.  The crossing tests compare order
// keys; the orientation test stays FP64.
struct PipSide {
  int n;
  const double* ring;
  const double* sp;
};
__global__ void k_pip(PipSide s0, PipSide s1, BkScalars* sc) {
  const PipSide& a = blockIdx.y ? s1 : s0;
  const int side = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = sc->firstFree[side];
  const double rx = a.sp[2 * s], ry = a.sp[2 * s + 1];
  const long long kx = okey(rx), ky = okey(ry);
  int w = 0;
  if (i < a.n) {
    const int j = (i + 1 == a.n) ? 0 : i + 1;
    const double x0 = a.ring[2 * i], y0 = a.ring[2 * i + 1];
    const double x1 = a.ring[2 * j], y1 = a.ring[2 * j + 1];
    const long long ky0 = okey(y0), ky1 = okey(y1);
    if ((ky0 < ky) != (ky1 < ky)) {
      const int d = 2 * (ky1 > ky0) - 1;
      const long long kx0 = okey(x0), kx1 = okey(x1);
      if (kx0 >= kx) {
        if (kx1 > kx) w = d;
        else if ((area3(x0, y0, x1, y1, rx, ry) > 0) == (ky1 > ky0)) w = d;
      } else if (kx1 > kx) {
        if ((area3(x0, y0, x1, y1, rx, ry) > 0) == (ky1 > ky0)) w = d;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
  if ((threadIdx.x & 31) == 0 && w) atomicAdd(&sc->winding[side], w);
}

// ---------------------------------------------------------------- entry/exit (A16 step 4)
__global__ void k_cross_flags(ListSide s0, ListSide s1, int* __restrict__ c0,
                              int* __restrict__ c1) {
  const ListSide& a = blockIdx.y ? s1 : s0;
  int* c = blockIdx.y ? c1 : c0;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > a.n) return;
  c[i] = (i < a.n && a.isect[i] && a.lab[i] == L_CROSSING) ? 1 : 0;
}

// status before vertex i = ENTRY ^ inside(V) ^ parity(crossings from V to i)
struct EnexSide {
  int n;
  const unsigned char* isect;
  const int* lab;
  const int* pre;
  unsigned char* enex;
  unsigned char* split;
  int* list;
};
__global__ void k_enex(EnexSide s0, EnexSide s1, const BkScalars* __restrict__ sc) {
  const EnexSide& a = blockIdx.y ? s1 : s0;
  const int side = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int V = sc->firstFree[side];
  const int total = a.pre[a.n];
  const int r = (i >= V) ? (a.pre[i] - a.pre[V]) : (a.pre[i] + total - a.pre[V]);
  const int status0 = (sc->winding[side] & 1) ? EX_EXIT : EX_ENTRY;
  const int status = (r & 1) ? (1 - status0) : status0;
  const int l = a.lab[i];
  unsigned char e = EX_NEITHER;
  if (a.isect[i] && l == L_CROSSING) {
    e = (unsigned char)status;
    a.list[a.pre[i]] = i;
  }
  a.enex[i] = e;
  a.split[i] = (a.isect[i] && l == L_BOUNCING && status == EX_EXIT) ? 1 : 0;
}

// a bouncing vertex whose neighbour is also a split candidate needs the
// split-pair insertion of step 5 (serial path)
__global__ void k_split_check(int nB, const unsigned char* __restrict__ splitP,
                              const unsigned char* __restrict__ splitQ, const int* __restrict__ winP,
                              BkScalars* sc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nB) return;
  if (!splitP[i]) return;
  int q = winP[i];
  if (q >= 0 && splitQ[q]) atomicOr(&sc->anomaly, 8u);
}

// ---------------------------------------------------------------- tracing (A17)
// enex vertices are indexed 0..cP-1 (P, slot order) then cP..cP+cQ-1 (Q)
struct Trace {
  int nB, nQ, cP, cQ;
  const int* listP;   // enex slots of P in slot order
  const int* listQ;
  const unsigned char* enexP;
  const unsigned char* enexQ;
  const int* winP;    // neighbour of P slot (Q slot) or -1
  const int* nbQ;     // neighbour of Q slot (P slot) or -1
  const int* rankP;   // slot -> enex index (valid for enex slots)
  const int* rankQ;
};

__device__ __forceinline__ int tr_slot(const Trace& T, int x) {
  return x < T.cP ? T.listP[x] : T.listQ[x - T.cP];
}

// target: next EXIT forward from an ENTRY vertex, previous ENTRY backward from
// an EXIT vertex; with alternating flags this is the adjacent enex vertex
__device__ __forceinline__ int tr_target(const Trace& T, int x) {
  if (x < T.cP) {
    int e = T.enexP[T.listP[x]];
    return e == EX_ENTRY ? (x + 1 == T.cP ? 0 : x + 1) : (x == 0 ? T.cP - 1 : x - 1);
  }
  int y = x - T.cP;
  int e = T.enexQ[T.listQ[y]];
  int z = e == EX_ENTRY ? (y + 1 == T.cQ ? 0 : y + 1) : (y == 0 ? T.cQ - 1 : y - 1);
  return T.cP + z;
}

// neighbour jump from enex vertex t (-1 if the neighbour is no enex vertex)
__device__ __forceinline__ int tr_jump(const Trace& T, int t) {
  if (t < T.cP) {
    int q = T.winP[T.listP[t]];
    if (q < 0 || T.enexQ[q] == EX_NEITHER) return -1;
    return T.cP + T.rankQ[q];
  }
  int p = T.nbQ[T.listQ[t - T.cP]];
  if (p < 0 || T.enexP[p] == EX_NEITHER) return -1;
  return T.rankP[p];
}

__global__ void k_rank(int n0, const int* __restrict__ list0, int* __restrict__ rank0, int n1,
                       const int* __restrict__ list1, int* __restrict__ rank1) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (blockIdx.y == 0) {
    if (x < n0) rank0[list0[x]] = x;
  } else if (x < n1) {
    rank1[list1[x]] = x;
  }
}

__global__ void k_tr_init(Trace T, int* __restrict__ jmp, int* __restrict__ mval, BkScalars* sc) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int n = T.cP + T.cQ;
  if (x >= n) return;
  int t = tr_target(T, x);
  // alternation: the target must carry the opposite flag
  int ex = x < T.cP ? T.enexP[T.listP[x]] : T.enexQ[T.listQ[x - T.cP]];
  int et = t < T.cP ? T.enexP[T.listP[t]] : T.enexQ[T.listQ[t - T.cP]];
  if (ex == et) atomicOr(&sc->anomaly, 16u);
  int s = tr_jump(T, t);
  if (s < 0) {
    atomicOr(&sc->anomaly, 32u);
    s = x;
  }
  jmp[x] = s;
  int a = x < T.cP ? T.listP[x] : 0x7fffffff;
  int b = t < T.cP ? T.listP[t] : 0x7fffffff;
  mval[x] = a < b ? a : b;
}

__global__ void k_tr_jump(int n, const int* __restrict__ jin, const int* __restrict__ min_,
                          int* __restrict__ jout, int* __restrict__ mout) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
  int j = jin[x];
  int a = min_[x], b = min_[j];
  mout[x] = a < b ? a : b;
  jout[x] = jin[j];
}

// The two pointer-jumping passes below as one cooperative launch each,
// rounds separated by grid-wide barriers and ended on the device as soon as
// a round changes nothing that is read afterwards:
//  * orbit minimum (k_tr_jump): after round r every element holds the
//    minimum over the next 2^(r+1) elements of its orbit; a round that
//    changes no minimum means every orbit is covered (the orbit's minimum is
//    unique, and it would reach a new element in every round until then);
//  * weighted list ranking (k_lr_jump): after round r an element's pointer
//    is -1 iff it is fewer than 2^(r+1) hops from its path's end; a path
//    holding an element 2^r hops from its end ends one in round r, so a
//    round that ends none leaves no path unfinished (orbits that never meet
//    the break stay cycles and are not read).
// The flag of round r is flags[r % 3]; thread 0 clears flags[(r + 1) % 3] at
// the start of round r, which every thread last read before the barrier that
// ended round r - 1.  Every thread reads the same flag after the same
// barrier, so all leave the loop in the same round.  The result is left in
// the A arrays.
constexpr int kJumpBatch = 4;

__global__ void k_tr_jump_coop(int n, int* __restrict__ jA, int* __restrict__ mA,
                               int* __restrict__ jB, int* __restrict__ mB,
                               unsigned* __restrict__ flags, int max_rounds) {
  cooperative_groups::grid_group grid = cooperative_groups::this_grid();
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nth = (long long)gridDim.x * blockDim.x;
  int *jin = jA, *min_ = mA, *jout = jB, *mout = mB;
  for (int r = 0; r < max_rounds; ++r) {
    if (tid == 0) flags[(r + 1) % 3] = 0u;
    bool ch = false;
    // kJumpBatch elements per thread at a time: their loads are issued
    // together, so a round costs two dependent L2 round trips per batch
    for (long long x0 = tid; x0 < n; x0 += kJumpBatch * nth) {
      int j[kJumpBatch], a[kJumpBatch], b[kJumpBatch], jj[kJumpBatch];
#pragma unroll
      for (int u = 0; u < kJumpBatch; ++u) {
        const long long x = x0 + u * nth;
        j[u] = x < n ? jin[x] : 0;
        a[u] = x < n ? min_[x] : 0;
      }
#pragma unroll
      for (int u = 0; u < kJumpBatch; ++u) {
        const long long x = x0 + u * nth;
        b[u] = x < n ? min_[j[u]] : 0;
        jj[u] = x < n ? jin[j[u]] : 0;
      }
#pragma unroll
      for (int u = 0; u < kJumpBatch; ++u) {
        const long long x = x0 + u * nth;
        if (x < n) {
          const int m = a[u] < b[u] ? a[u] : b[u];
          mout[x] = m;
          jout[x] = jj[u];
          ch |= m != a[u];
        }
      }
    }
    if (__any_sync(0xffffffffu, ch) && (threadIdx.x & 31) == 0) atomicOr(&flags[r % 3], 1u);
    grid.sync();
    int* t0 = jin; jin = jout; jout = t0;
    int* t1 = min_; min_ = mout; mout = t1;
    if (*(volatile unsigned*)&flags[r % 3] == 0u) break;
  }
  if (min_ != mA)
    for (long long x = tid; x < n; x += nth) {
      mA[x] = min_[x];
      jA[x] = jin[x];
    }
}

__global__ void k_lr_jump_coop(int n, int* __restrict__ nA, long long* __restrict__ SA,
                               int* __restrict__ nB, long long* __restrict__ SB,
                               unsigned* __restrict__ flags, int max_rounds) {
  cooperative_groups::grid_group grid = cooperative_groups::this_grid();
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nth = (long long)gridDim.x * blockDim.x;
  int *nin = nA, *nout = nB;
  long long *Sin = SA, *Sout = SB;
  for (int r = 0; r < max_rounds; ++r) {
    if (tid == 0) flags[(r + 1) % 3] = 0u;
    bool ch = false;
    for (long long x0 = tid; x0 < n; x0 += kJumpBatch * nth) {
      int j[kJumpBatch], jj[kJumpBatch];
      long long sa[kJumpBatch], sb[kJumpBatch];
#pragma unroll
      for (int u = 0; u < kJumpBatch; ++u) {
        const long long x = x0 + u * nth;
        j[u] = x < n ? nin[x] : -1;
        sa[u] = x < n ? Sin[x] : 0;
      }
#pragma unroll
      for (int u = 0; u < kJumpBatch; ++u) {
        jj[u] = j[u] >= 0 ? nin[j[u]] : -1;
        sb[u] = j[u] >= 0 ? Sin[j[u]] : 0;
      }
#pragma unroll
      for (int u = 0; u < kJumpBatch; ++u) {
        const long long x = x0 + u * nth;
        if (x < n) {
          nout[x] = j[u] < 0 ? -1 : jj[u];
          Sout[x] = sa[u] + sb[u];
          ch |= j[u] >= 0 && jj[u] < 0;
        }
      }
    }
    if (__any_sync(0xffffffffu, ch) && (threadIdx.x & 31) == 0) atomicOr(&flags[r % 3], 1u);
    grid.sync();
    int* t0 = nin; nin = nout; nout = t0;
    long long* t1 = Sin; Sin = Sout; Sout = t1;
    if (*(volatile unsigned*)&flags[r % 3] == 0u) break;
  }
  if (nin != nA)
    for (long long x = tid; x < n; x += nth) {
      nA[x] = nin[x];
      SA[x] = Sin[x];
    }
}

// every enex vertex must agree with its successor and its target on the
// ring minimum (rings are closed under both)
__global__ void k_tr_consistent(Trace T, const int* __restrict__ mval, BkScalars* sc) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int n = T.cP + T.cQ;
  if (x >= n) return;
  int t = tr_target(T, x);
  int s = tr_jump(T, t);
  if (s < 0 || mval[x] != mval[t] || mval[x] != mval[s]) atomicOr(&sc->anomaly, 64u);
}

__global__ void k_tr_starts(Trace T, const int* __restrict__ mval, int* __restrict__ isStart) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x > T.cP) return;
  isStart[x] = (x < T.cP && mval[x] == T.listP[x]) ? 1 : 0;
}

__global__ void k_tr_startlist(int cP, const int* __restrict__ pre, int* __restrict__ starts) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= cP) return;
  if (pre[x + 1] != pre[x]) starts[pre[x]] = x;
}

__device__ __forceinline__ int tr_len(const Trace& T, int x, int t) {
  int n = x < T.cP ? T.nB : T.nQ;
  int sx = tr_slot(T, x), st = tr_slot(T, t);
  bool fwd = (x < T.cP ? T.enexP[sx] : T.enexQ[sx]) == EX_ENTRY;
  int d = fwd ? st - sx : sx - st;
  if (d <= 0) d += n;
  return d;
}

// createResult2 as weighted list ranking.  A ring is the orbit of its start I
// under succ(x) = neighbour(target(x)); segment x contributes the vertices
// after x up to target(x).  Breaking each orbit before I and pointer jumping
// gives every segment the number of ring vertices from it to the ring's end,
// hence its output position; vertices of the opposite orbit of the same ring
// never reach the break and are not part of the output.
__global__ void k_lr_init(Trace T, const int* __restrict__ mval, int* __restrict__ nxt,
                          long long* __restrict__ S, int* __restrict__ ringI,
                          int* __restrict__ indeg, BkScalars* sc) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int n = T.cP + T.cQ;
  if (x >= n) return;
  if (mval[x] < 0 || mval[x] >= T.nB) {  // every ring holds a P crossing vertex
    atomicOr(&sc->anomaly, 2048u);
    ringI[x] = x;
    nxt[x] = -1;
    S[x] = 0;
    return;
  }
  int I = T.rankP[mval[x]];
  int t = tr_target(T, x);
  int s = tr_jump(T, t);
  ringI[x] = I;
  nxt[x] = (s == I) ? -1 : s;
  S[x] = tr_len(T, x, t);
  if (s >= 0) atomicAdd(&indeg[s], 1);
}

__global__ void k_lr_jump(int n, const int* __restrict__ nin, const long long* __restrict__ Sin,
                          int* __restrict__ nout, long long* __restrict__ Sout) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
  int j = nin[x];
  if (j < 0) {
    nout[x] = -1;
    Sout[x] = Sin[x];
  } else {
    nout[x] = nin[j];
    Sout[x] = Sin[x] + Sin[j];
  }
}

// succ must be a permutation, every ring start must reach its orbit's end,
// and no segment of a start's orbit may end at the start vertex itself (that
// stops the reference's walk early; the serial path covers it)
__global__ void k_lr_check(Trace T, const int* __restrict__ nxt, const int* __restrict__ ringI,
                           const int* __restrict__ indeg, BkScalars* sc) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int n = T.cP + T.cQ;
  if (x >= n) return;
  if (indeg[x] != 1) atomicOr(&sc->anomaly, 512u);
  if (ringI[x] == x && nxt[x] != -1) atomicOr(&sc->anomaly, 1024u);
  if (nxt[x] == -1 && tr_target(T, x) == ringI[x]) atomicOr(&sc->anomaly, 256u);
}

// rlen[r] for r <= cap: ring r's length, 0 from the ring count on
__global__ void k_lr_ringlen(int cap, const int* __restrict__ nRings_p,
                             const int* __restrict__ starts, const long long* __restrict__ S,
                             int* __restrict__ rlen) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > cap) return;
  const int nRings = *nRings_p;
  rlen[r] = r < nRings ? (int)S[starts[r]] : 0;
}

// Segments of up to kSegInline vertices are copied by their own warp (so a
// warp copies at most 32 x kSegInline vertices); longer ones are cut into
// pieces of kSegPiece vertices that k_lr_copy_long copies one warp per piece.
// Otherwise one warp holding long ring stretches would run long after the
// others.
constexpr int kSegInline = 32;
constexpr int kSegPiece = 256;

// the output placement of segment x (an enex vertex of a start's orbit)
struct SegCopy {
  long long base;
  int len, m, sx;
  bool onP, fwd;
};
__device__ __forceinline__ SegCopy seg_copy_of(const Trace& T, int x, const long long* S,
                                               const int* ringI, const int* startPre,
                                               const int* vOff) {
  SegCopy c;
  const int I = ringI[x];
  c.base = vOff[startPre[I]] + S[I] - S[x];
  const int t = tr_target(T, x);
  c.len = tr_len(T, x, t);
  c.onP = x < T.cP;
  c.m = c.onP ? T.nB : T.nQ;
  c.sx = tr_slot(T, x);
  c.fwd = (c.onP ? T.enexP[c.sx] : T.enexQ[c.sx]) == EX_ENTRY;
  return c;
}

// a piece of a long segment: its placement and steps [step0, step0 + count)
struct SegPiece {
  long long base;
  int sx, m, step0, count, onP, fwd;
};

// vertex `step` (1-based) of a segment
__device__ __forceinline__ void seg_copy_step(const SegCopy& c, int step, const double* ixB,
                                              const double* ixC, double* out) {
  int slot = c.fwd ? c.sx + step : c.sx - step;
  if (slot >= c.m) slot -= c.m;
  if (slot < 0) slot += c.m;
  const double2 v = reinterpret_cast<const double2*>(c.onP ? ixB : ixC)[slot];
  reinterpret_cast<double2*>(out)[c.base + step - 1] = v;
}

__global__ void k_lr_copy(Trace T, const int* __restrict__ nxt, const long long* __restrict__ S,
                          const int* __restrict__ ringI, const int* __restrict__ startPre,
                          const int* __restrict__ vOff, const double* __restrict__ ixB,
                          const double* __restrict__ ixC, double* __restrict__ out,
                          SegPiece* __restrict__ pieces, unsigned* __restrict__ npieces,
                          long long pcap) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int n = T.cP + T.cQ;
  bool mine = x < n && nxt[x] == -1;  // only segments of a start's orbit
  long long base = 0;
  int len = 0, m = 1, sx = 0;
  bool onP = false, fwd = false;
  if (mine) {
    const SegCopy c = seg_copy_of(T, x, S, ringI, startPre, vOff);
    if (c.len > kSegInline) {
      // to the long-segment queue, one entry per piece
      const int np = (c.len + kSegPiece - 1) / kSegPiece;
      const unsigned q = atomicAdd(npieces, (unsigned)np);
      for (int i = 0; i < np; ++i)
        if (q + i < pcap) {
          const int s0 = i * kSegPiece + 1;
          pieces[q + i] = SegPiece{c.base, c.sx, c.m, s0, min(kSegPiece, c.len - s0 + 1),
                                   (int)c.onP, (int)c.fwd};
        }
      mine = false;
    } else {
      base = c.base;
      len = c.len;
      m = c.m;
      sx = c.sx;
      onP = c.onP;
      fwd = c.fwd;
    }
  }
  // the warp's segments laid end to end, 32 output vertices per round: each
  // lane finds the segment of its vertex by a binary search over the lanes'
  // inclusive length prefix, so every lane copies whatever the lengths
  const unsigned full = 0xffffffffu;
  int incl = mine ? len : 0;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(full, incl, o);
    if (lane >= o) incl += y;
  }
  const int excl = incl - (mine ? len : 0);
  const int total = __shfl_sync(full, incl, 31);
  for (int o0 = 0; o0 < total; o0 += 32) {
    const int o = o0 + lane;
    int sl = 0;  // lanes whose segments end at or before o
#pragma unroll
    for (int b = 16; b >= 1; b >>= 1)
      if (__shfl_sync(full, incl, sl + b - 1) <= o) sl += b;
    const long long b0 = __shfl_sync(full, base, sl);
    const int e0 = __shfl_sync(full, excl, sl);
    const int s0 = __shfl_sync(full, sx, sl);
    const int m0 = __shfl_sync(full, m, sl);
    const bool f0 = __shfl_sync(full, (int)fwd, sl) != 0;
    const bool p0 = __shfl_sync(full, (int)onP, sl) != 0;
    if (o < total) {
      const SegCopy c{b0, 0, m0, s0, p0, f0};
      seg_copy_step(c, o - e0 + 1, ixB, ixC, out);
    }
  }
}

// the pieces of the long segments, one warp per piece
__global__ void k_lr_copy_long(const double* __restrict__ ixB, const double* __restrict__ ixC,
                               double* __restrict__ out, const SegPiece* __restrict__ pieces,
                               const unsigned* __restrict__ npieces, long long pcap) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const long long np = min((long long)*npieces, pcap);
  for (long long i = w; i < np; i += ((long long)gridDim.x * blockDim.x) >> 5) {
    const SegPiece pc = pieces[i];
    const SegCopy c{pc.base, 0, pc.m, pc.sx, pc.onP != 0, pc.fwd != 0};
    for (int k = lane; k < pc.count; k += 32) seg_copy_step(c, pc.step0 + k, ixB, ixC, out);
  }
}

// ---------------------------------------------------------------- clean-up (A18)
// ring of vertex v: last ring whose offset is <= v (empty rings are skipped)
__global__ void k_ring_of(long long nv, int nRings, const int* __restrict__ off,
                          int* __restrict__ ringOf) {
  long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  int lo = 0, hi = nRings;
  while (hi - lo > 1) {
    int m = (lo + hi) >> 1;
    if (off[m] <= v) lo = m;
    else hi = m;
  }
  ringOf[v] = lo;
}

// a ring can only lose vertices if one of them is collinear with its
// original neighbours (removals only ever follow such a vertex)
__global__ void k_collinear(long long nv, const int* __restrict__ off,
                            const int* __restrict__ ringOf, const double* __restrict__ xy,
                            int* __restrict__ ringFlag, int* __restrict__ keep,
                            int* __restrict__ flagV, int* __restrict__ nxt, int* __restrict__ prv) {
  long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v > nv) return;
  if (v == nv) {
    keep[v] = 0;
    flagV[v] = 0;
    return;
  }
  keep[v] = 1;
  int r = ringOf[v];
  int a = off[r], b = off[r + 1];
  long long p = v == a ? b - 1 : v - 1;
  long long q = v + 1 == b ? a : v + 1;
  nxt[v] = (int)q;
  prv[v] = (int)p;
  int f = fabs(area3(xy[2 * p], xy[2 * p + 1], xy[2 * v], xy[2 * v + 1], xy[2 * q], xy[2 * q + 1])) <
          kEps;
  flagV[v] = f;
  if (f) ringFlag[r] = 1;
}

__global__ void k_flag_list(long long nv, const int* __restrict__ fpre, int* __restrict__ list) {
  long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  if (fpre[v + 1] != fpre[v]) list[fpre[v]] = (int)v;
}

// cleanUpResult2 (foster/polyclip.h:767-787) on one flagged ring, thread per
// ring.  The linked-list steps are the reference's; vertices whose links are
// still the original ones and that are not collinear with their original
// neighbours cannot be removed, so the walk jumps over them: it visits the
// flagged vertices, the successor of every removed vertex and the last
// vertex (whose next is the root the root loop left).  The reference keeps
// iterating from a deleted vertex through its old next pointer; so does this.
__global__ void k_cleanup_ring(int nRings, const int* __restrict__ off,
                               const int* __restrict__ ringFlag, const int* __restrict__ flist,
                               const int* __restrict__ nflag_p, const double* __restrict__ xy,
                               int* __restrict__ nxt, int* __restrict__ prv,
                               int* __restrict__ keep) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nRings) return;
  int a = off[r], b = off[r + 1];
  if (!ringFlag[r] || b == a) return;
  const int nflag = *nflag_p;
  auto A = [&](int v) {
    int p = prv[v], q = nxt[v];
    return fabs(area3(xy[2 * p], xy[2 * p + 1], xy[2 * v], xy[2 * v + 1], xy[2 * q], xy[2 * q + 1]));
  };
  int root = a;
  auto remove = [&](int V) {
    if (root == V) {
      root = nxt[V];
      if (nxt[root] == root) root = -1;
    }
    nxt[prv[V]] = nxt[V];
    prv[nxt[V]] = prv[V];
    keep[V] = 0;
  };
  while (root >= 0 && A(root) < kEps) remove(root);
  if (root < 0) return;  // every vertex was removed (each keep flag cleared)
  const bool prefixRemoved = root != a;
  int lo = 0, hi = nflag;  // first flagged vertex >= root
  while (lo < hi) {
    int m = (lo + hi) >> 1;
    if (flist[m] < root) lo = m + 1;
    else hi = m;
  }
  int fi = lo;
  int V = root;
  while (true) {
    bool removed = A(V) < kEps;
    if (removed) remove(V);
    int cand = 0x7fffffff;
    if (removed && V + 1 < b) cand = V + 1;
    while (fi < nflag && flist[fi] <= V) ++fi;
    if (fi < nflag && flist[fi] < b && flist[fi] < cand) cand = flist[fi];
    if (prefixRemoved && V < b - 1 && b - 1 < cand) cand = b - 1;
    if (cand >= b) break;
    V = cand;
  }
}

// rings that lost every vertex print nothing (foster/polygon.h:577)
__global__ void k_ring_nonempty(int nRings, const int* __restrict__ off, const int* __restrict__ kpv,
                                int* __restrict__ ne) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > nRings) return;
  ne[r] = (r < nRings && kpv[off[r + 1]] > kpv[off[r]]) ? 1 : 0;
}

// kept vertices keep their ring order: the reference's root is the first
// vertex surviving the root loop, and later removals never touch it
__global__ void k_compact_xy(long long nv, const int* __restrict__ kpv,
                             const double* __restrict__ xy, double* __restrict__ oxy) {
  long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv || kpv[v + 1] == kpv[v]) return;  // flag = difference of the prefix
  long long w = kpv[v];
  oxy[2 * w] = xy[2 * v];
  oxy[2 * w + 1] = xy[2 * v + 1];
}

__global__ void k_compact_off(int nRings, long long nv, const int* __restrict__ off,
                              const int* __restrict__ kpv, const int* __restrict__ rpre,
                              int* __restrict__ ooff) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > nRings) return;
  if (r == nRings) {
    ooff[rpre[nRings]] = kpv[nv];
    return;
  }
  if (rpre[r + 1] != rpre[r]) ooff[rpre[r]] = kpv[off[r]];
}

// ---------------------------------------------------------------- whole-list rings (A16 step 3.5)
__global__ void k_copy_list(int n, const double* __restrict__ src, double* __restrict__ dst) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * n) return;
  dst[i] = src[i];
}

__global__ void k_serial_backend(SerialArgs a) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  *a.status = 0;
  *a.nrings = 0;
  int st = ser_build(a);
  if (!st) st = ser_label_trace(a);
  if (!st) ser_cleanup(a);
  *a.status = st;
}

// serial output: ring vertex counts and coordinates in ring order
__global__ void k_serial_emit(SerialArgs a, int* __restrict__ ooff, double* __restrict__ oxy,
                              long long cap, int* __restrict__ counts) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  long long w = 0;
  int nr = 0;
  ooff[0] = 0;
  for (int r = 0; r < *a.nrings; ++r) {
    int root = a.rroot[r];
    if (root < 0) continue;
    int v = root;
    do {
      if (w < cap) {
        oxy[2 * w] = a.R.x[v];
        oxy[2 * w + 1] = a.R.y[v];
      }
      ++w;
      v = a.R.next[v];
    } while (v != root);
    ooff[++nr] = (int)w;
  }
  counts[0] = nr;
  counts[1] = (int)w;
}

}  // namespace

// ============================================================== host driver
// One cooperative launch of a jump kernel above over n elements, with as
// many blocks as can be resident at once (grid-wide barriers need them all
// running); false if the launch is refused, and the caller then runs the
// plain launch loop.
template <typename A>
static bool jump_coop(void (*kern)(int, int*, A*, int*, A*, unsigned*, int), int n, int* pA,
                      A* vA, int* pB, A* vB, unsigned* flags, int rounds, cudaStream_t st) {
  if (n <= 0) return true;
  static std::mutex mu;
  static int cap[64][2] = {};  // per device and value type: co-resident blocks of 256 threads
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
  const int kind = sizeof(A) == 8 ? 1 : 0;
  int maxb = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!cap[dev][kind]) {
      int per = 0, sms = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)kern, 256, 0) !=
              cudaSuccess ||
          cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
          per < 1)
        return false;
      cap[dev][kind] = per * sms;
    }
    maxb = cap[dev][kind];
  }
  const int blocks = (int)std::min<long long>(((long long)n + 255) / 256, (long long)maxb);
  if (cudaMemsetAsync(flags, 0, 3 * sizeof(unsigned), st) != cudaSuccess) return false;
  void* args[] = {&n, &pA, &vA, &pB, &vB, &flags, &rounds};
  ::sbc::KProbe kp_(kind ? "k_lr_jump_coop" : "k_tr_jump_coop", st);
  if (cudaLaunchCooperativeKernel((const void*)kern, dim3(blocks), dim3(256), args, 0, st) ==
      cudaSuccess)
    return true;
  cudaGetLastError();  // this refused launch's own error: the loop below replaces it
  return false;
}

static int serial_backend(Pipeline& pl, const Merged& m, OverlayOut& out, int tag) {
  cudaStream_t st = pl.stream();
  BufferPool& bp = pl.pool();
  int extra = 2 * m.K + 8;
  int capP = m.nB + extra, capQ = m.nQ + extra, capR = m.nB + m.nQ + 2 * extra + 16;
  auto mk = [&](const char* nm, int cap, Pool& p) {
    std::string s(nm);
    p.x = (double*)bp.get(s + "_x", sizeof(double) * cap);
    p.y = (double*)bp.get(s + "_y", sizeof(double) * cap);
    p.next = (int*)bp.get(s + "_next", sizeof(int) * cap);
    p.prev = (int*)bp.get(s + "_prev", sizeof(int) * cap);
    p.nb = (int*)bp.get(s + "_nb", sizeof(int) * cap);
    p.label = (int*)bp.get(s + "_label", sizeof(int) * cap);
    p.enex = (int*)bp.get(s + "_enex", sizeof(int) * cap);
    p.source = (unsigned char*)bp.get(s + "_src", cap);
    p.isect = (unsigned char*)bp.get(s + "_isect", cap);
    p.n = 0;
    p.cap = cap;
  };
  SerialArgs a;
  mk("serP", capP, a.P);
  mk("serQ", capQ, a.Q);
  mk("serR", capR, a.R);
  a.rcap = m.nB + 16;
  a.rroot = (int*)bp.get("ser_roots", sizeof(int) * a.rcap);
  a.nrings = (int*)bp.get("ser_nrings", 256);
  a.status = (int*)bp.get("ser_status", 256);
  a.splitP = (unsigned char*)bp.get("ser_splitP", capP);
  a.splitQ = (unsigned char*)bp.get("ser_splitQ", capQ);
  a.crossP = (unsigned char*)bp.get("ser_crossP", capP);
  a.crossQ = (unsigned char*)bp.get("ser_crossQ", capQ);
  if (bp.failed) return pl.fail(kENoMem, "device allocation failed (serial back end)");
  cudaMemsetAsync(a.splitP, 0, capP, st);
  cudaMemsetAsync(a.splitQ, 0, capQ, st);
  cudaMemsetAsync(a.crossP, 0, capP, st);
  cudaMemsetAsync(a.crossQ, 0, capQ, st);
  a.bSize = m.bSize;
  a.cSize = m.cSize;
  a.cStart = m.cStart;
  a.nB = m.nB;
  a.nQ = m.nQ;
  a.bP = m.bP;
  a.cP = m.cP;
  a.ixB = m.ixB;
  a.ixC = m.ixC;
  a.alB = m.alB;
  a.nbC = m.nbC;
  a.labB = m.labB;
  a.labC = m.labC;
  a.unite = pl.unite ? 1 : 0;
  {
    ::sbc::KProbe kp_("k_serial_backend", st);
    k_serial_backend<<<1, 1, 0, st>>>(a);
  }
  int hst = 0;
  cudaMemcpyAsync(&hst, a.status, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  if (hst == 2) return pl.fail(kEUndef, "reference behaviour undefined in the linked-list back end");
  if (hst == 3) return pl.fail(kEInternal, "serial back end capacity exceeded");
  std::string t = std::to_string(tag);
  long long cap = capR;
  int* ooff = (int*)bp.get("ring_off_" + t, sizeof(int) * (a.rcap + 1));
  double* oxy = (double*)bp.get("ring_xy_" + t, sizeof(double) * 2 * cap);
  int* counts = (int*)bp.get("ser_counts", 256);
  if (bp.failed) return pl.fail(kENoMem, "device allocation failed (rings)");
  {
    ::sbc::KProbe kp_("k_serial_emit", st);
    k_serial_emit<<<1, 1, 0, st>>>(a, ooff, oxy, cap, counts);
  }
  int hc[2];
  cudaMemcpyAsync(hc, counts, sizeof(hc), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  out.nrings = hc[0];
  out.nverts = hc[1];
  out.d_off = ooff;
  out.d_xy = oxy;
  out.slow_path = 1;
  return kOk;
}

int run_backend(Pipeline& pl, const Merged& m, OverlayOut& out) {
  cudaStream_t st = pl.stream();
  BufferPool& bp = pl.pool();
  const int ovTag = (int)(&out - &pl.outputs()[0]);
  // union mode has only the exact serial back end
  if (pl.force_serial_backend || pl.unite) return serial_backend(pl, m, out, ovTag);
  const int nB = m.nB, nQ = m.nQ;
  auto* sc = (BkScalars*)bp.get("bk_scalars", sizeof(BkScalars));
  auto* srcP = (unsigned char*)bp.get("bk_srcP", nB);
  auto* srcQ = (unsigned char*)bp.get("bk_srcQ", nQ);
  auto* isP = (unsigned char*)bp.get("bk_isP", nB);
  auto* isQ = (unsigned char*)bp.get("bk_isQ", nQ);
  int* labP = (int*)bp.get("bk_labP", sizeof(int) * nB);
  int* labQ = (int*)bp.get("bk_labQ", sizeof(int) * nQ);
  int* nbQ = (int*)bp.get("bk_nbQ", sizeof(int) * nQ);
  int* winP = (int*)bp.get("bk_winP", sizeof(int) * nB);
  if (bp.failed) return pl.fail(kENoMem, "device allocation failed (back end)");
  BkScalars init;
  memset(&init, 0, sizeof init);
  init.firstFree[0] = init.firstFree[1] = 0x7fffffff;
  cudaMemcpyAsync(sc, &init, sizeof init, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(srcP, 0, nB, st);
  cudaMemsetAsync(srcQ, 0, nQ, st);
  cudaMemsetAsync(winP, 0xff, sizeof(int) * nB, st);
  auto grid2 = [](long long n0, long long n1, int per) {
    return dim3(grid_for(n0 > n1 ? n0 : n1, per), 2);
  };
  {
    const SrcSide s0{m.bSize, nB, 0, m.bND, m.ixB, m.bP, srcP};
    const SrcSide s1{m.cSize, nQ, m.cStart, m.cND, m.ixC, m.cP, srcQ};
    ::sbc::KProbe kp_("k_mark_bridge", st);
    k_mark_bridge<<<grid2(m.bSize, m.cSize, 128), 128, 0, st>>>(s0, s1, sc);
  }
  {
    const InitArgs ia{nB, nQ, srcP, srcQ, m.alB, m.labB, m.nbC, m.labC,
                      isP, isQ, labP, labQ, nbQ, winP};
    ::sbc::KProbe kp_("k_init_PQ", st);
    k_init_PQ<<<grid2(nB, nQ, 256), 256, 0, st>>>(ia, sc);
  }
  const ListSide lsP{nB, isP, labP}, lsQ{nQ, isQ, labQ};
  {
    ::sbc::KProbe kp_("k_side_stats", st);
    k_side_stats<<<grid2(nB, nQ, 256), 256, 0, st>>>(lsP, lsQ, sc);
  }
  static_assert(sizeof(BkScalars) <= 8 * 8, "BkScalars fits the back end's host words");
  HostReads& rd = pl.reads();
  BkScalars h;
  const BkScalars* r_sc = rd.get(sc, HostReads::kBack, st);
  cudaStreamSynchronize(st);
  h = *r_sc;
  if (h.anomaly) return serial_backend(pl, m, out, ovTag);
  const bool noP = h.crossCount[0] == 0, noQ = h.crossCount[1] == 0;
  if (noP != noQ) return serial_backend(pl, m, out, ovTag);
  if (h.firstFree[0] == 0x7fffffff || h.firstFree[1] == 0x7fffffff)
    return serial_backend(pl, m, out, ovTag);
  if (noP && (h.notOnOn[0] == 0 || h.notOnOn[1] == 0)) return serial_backend(pl, m, out, ovTag);

  // seeds: the first non-intersection vertex of each side (sc->firstFree)
  // against the other side
  {
    const PipSide p0{nQ, m.ixC, m.ixB}, p1{nB, m.ixB, m.ixC};
    ::sbc::KProbe kp_("k_pip", st);
    k_pip<<<grid2(nQ, nB, 256), 256, 0, st>>>(p0, p1, sc);
  }

  std::string tg = std::to_string(ovTag);
  if (noP) {
    // both polygons without crossings: each one inside the other is a ring
    r_sc = rd.get(sc, HostReads::kBack, st);
    cudaStreamSynchronize(st);
    h = *r_sc;
    bool inP = (h.winding[0] % 2) != 0, inQ = (h.winding[1] % 2) != 0;
    int nr = (inP ? 1 : 0) + (inQ ? 1 : 0);
    long long nv = (inP ? nB : 0) + (inQ ? nQ : 0);
    double* xy = (double*)bp.get("bk_rxy", sizeof(double) * 2 * (nv + 1));
    int* off = (int*)bp.get("bk_roff", sizeof(int) * 4);
    if (bp.failed) return pl.fail(kENoMem, "device allocation failed (rings)");
    int hoff[3] = {0, 0, 0};
    long long w = 0;
    int r = 0;
    if (inP) {
      {
        ::sbc::KProbe kp_("k_copy_list", st);
        k_copy_list<<<grid_for(2 * nB, 256), 256, 0, st>>>(nB, m.ixB, xy);
      }
      w += nB;
      hoff[++r] = (int)w;
    }
    if (inQ) {
      {
        ::sbc::KProbe kp_("k_copy_list", st);
        k_copy_list<<<grid_for(2 * nQ, 256), 256, 0, st>>>(nQ, m.ixC, xy + 2 * w);
      }
      w += nQ;
      hoff[++r] = (int)w;
    }
    cudaMemcpyAsync(off, hoff, sizeof hoff, cudaMemcpyHostToDevice, st);
    out.d_off = off;
    out.d_xy = xy;
    out.nrings = nr;
    out.nverts = nv;
  } else {
    // ---- entry/exit flags
    int* preP = (int*)bp.get("bk_preP", sizeof(int) * (nB + 1));
    int* preQ = (int*)bp.get("bk_preQ", sizeof(int) * (nQ + 1));
    auto* enexP = (unsigned char*)bp.get("bk_enexP", nB);
    auto* enexQ = (unsigned char*)bp.get("bk_enexQ", nQ);
    auto* splitP = (unsigned char*)bp.get("bk_splitP", nB);
    auto* splitQ = (unsigned char*)bp.get("bk_splitQ", nQ);
    int* listP = (int*)bp.get("bk_listP", sizeof(int) * (h.crossCount[0] + 1));
    int* listQ = (int*)bp.get("bk_listQ", sizeof(int) * (h.crossCount[1] + 1));
    int* rankP = (int*)bp.get("bk_rankP", sizeof(int) * nB);
    int* rankQ = (int*)bp.get("bk_rankQ", sizeof(int) * nQ);
    const long long nmax = (long long)(nB > nQ ? nB : nQ) + 1;
    const size_t scr_b = std::max(scan_scratch_bytes((long long)nB + nQ + 4),
                                  scan_set_scratch_bytes(nmax, 2));
    void* sscr = bp.get_zeroed("bk_scan", scr_b, st);
    if (bp.failed) return pl.fail(kENoMem, "device allocation failed (entry/exit)");
    {
      ::sbc::KProbe kp_("k_cross_flags", st);
      k_cross_flags<<<grid2(nB + 1, nQ + 1, 256), 256, 0, st>>>(lsP, lsQ, preP, preQ);
    }
    {
      int* const arrs[2] = {preP, preQ};
      const long long ns[2] = {(long long)nB + 1, (long long)nQ + 1};
      exclusive_scan_i32_set(arrs, ns, 2, sscr, st, true);
    }
    {
      const EnexSide e0{nB, isP, labP, preP, enexP, splitP, listP};
      const EnexSide e1{nQ, isQ, labQ, preQ, enexQ, splitQ, listQ};
      ::sbc::KProbe kp_("k_enex", st);
      k_enex<<<grid2(nB, nQ, 256), 256, 0, st>>>(e0, e1, sc);
    }
    {
      ::sbc::KProbe kp_("k_split_check", st);
      k_split_check<<<grid_for(nB, 256), 256, 0, st>>>(nB, splitP, splitQ, winP, sc);
    }
    const int cPn = h.crossCount[0], cQn = h.crossCount[1];
    if ((cPn & 1) || (cQn & 1)) return serial_backend(pl, m, out, ovTag);
    {
      ::sbc::KProbe kp_("k_rank", st);
      k_rank<<<grid2(cPn, cQn, 256), 256, 0, st>>>(cPn, listP, rankP, cQn, listQ, rankQ);
    }
    Trace T{nB, nQ, cPn, cQn, listP, listQ, enexP, enexQ, winP, nbQ, rankP, rankQ};
    const int nE = cPn + cQn;
    int* jmpA = (int*)bp.get("bk_jmpA", sizeof(int) * (nE + 1));
    int* jmpB = (int*)bp.get("bk_jmpB", sizeof(int) * (nE + 1));
    int* mA = (int*)bp.get("bk_mA", sizeof(int) * (nE + 1));
    int* mB = (int*)bp.get("bk_mB", sizeof(int) * (nE + 1));
    int* isStart = (int*)bp.get("bk_isStart", sizeof(int) * (cPn + 1));
    if (bp.failed) return pl.fail(kENoMem, "device allocation failed (rings)");
    {
      ::sbc::KProbe kp_("k_tr_init", st);
      k_tr_init<<<grid_for(nE, 256), 256, 0, st>>>(T, jmpA, mA, sc);
    }
    int rounds = 0;
    for (int span = 1; span < nE; span <<= 1) ++rounds;
    unsigned* jflags = (unsigned*)bp.get("bk_jump_flags", 256);
    if (bp.failed) return pl.fail(kENoMem, "device allocation failed (rings)");
    if (!jump_coop(k_tr_jump_coop, nE, jmpA, mA, jmpB, mB, jflags, rounds, st)) {
      for (int r = 0; r < rounds; ++r) {
        {
          ::sbc::KProbe kp_("k_tr_jump", st);
          k_tr_jump<<<grid_for(nE, 256), 256, 0, st>>>(nE, jmpA, mA, jmpB, mB);
        }
        std::swap(jmpA, jmpB);
        std::swap(mA, mB);
      }
    }
    {
      ::sbc::KProbe kp_("k_tr_consistent", st);
      k_tr_consistent<<<grid_for(nE, 256), 256, 0, st>>>(T, mA, sc);
    }
    // An anomaly found so far is read with the ring count below: the
    // kernels in between stay in bounds whatever the orbit minima hold
    // (k_lr_init checks them, and ring starts are ranks of P crossings).

    // ---- ring starts and segment walks.  There are at most cPn rings (a
    // ring starts at a P crossing): the ring arrays are sized for that, and
    // the ring count stays on the device until the one read below.
    {
      ::sbc::KProbe kp_("k_tr_starts", st);
      k_tr_starts<<<grid_for(cPn + 1, 256), 256, 0, st>>>(T, mA, isStart);
    }
    exclusive_scan_i32(isStart, cPn + 1, sscr, st, true);
    int* starts = (int*)bp.get("bk_starts", sizeof(int) * (cPn + 1));
    int* rlen = (int*)bp.get("bk_rlen", sizeof(int) * (cPn + 2));
    int* nxA = (int*)bp.get("bk_lrnA", sizeof(int) * (nE + 1));
    int* nxB = (int*)bp.get("bk_lrnB", sizeof(int) * (nE + 1));
    long long* SA = (long long*)bp.get("bk_lrSA", sizeof(long long) * (nE + 1));
    long long* SB = (long long*)bp.get("bk_lrSB", sizeof(long long) * (nE + 1));
    int* ringI = (int*)bp.get("bk_lrI", sizeof(int) * (nE + 1));
    int* indeg = (int*)bp.get("bk_lrdeg", sizeof(int) * (nE + 1));
    if (bp.failed) return pl.fail(kENoMem, "device allocation failed (rings)");
    {
      ::sbc::KProbe kp_("k_tr_startlist", st);
      k_tr_startlist<<<grid_for(cPn, 256), 256, 0, st>>>(cPn, isStart, starts);
    }
    cudaMemsetAsync(indeg, 0, sizeof(int) * (nE + 1), st);
    {
      ::sbc::KProbe kp_("k_lr_init", st);
      k_lr_init<<<grid_for(nE, 256), 256, 0, st>>>(T, mA, nxA, SA, ringI, indeg, sc);
    }
    if (!jump_coop(k_lr_jump_coop, nE, nxA, SA, nxB, SB, jflags, rounds, st)) {
      for (int r = 0; r < rounds; ++r) {
        ::sbc::KProbe kp_("k_lr_jump", st);
        k_lr_jump<<<grid_for(nE, 256), 256, 0, st>>>(nE, nxA, SA, nxB, SB);
        std::swap(nxA, nxB);
        std::swap(SA, SB);
      }
    }
    {
      ::sbc::KProbe kp_("k_lr_check", st);
      k_lr_check<<<grid_for(nE, 256), 256, 0, st>>>(T, nxA, ringI, indeg, sc);
    }
    {
      ::sbc::KProbe kp_("k_lr_ringlen", st);
      k_lr_ringlen<<<grid_for(cPn + 1, 256), 256, 0, st>>>(cPn, isStart + cPn, starts, SA, rlen);
    }
    // zero lengths past the last ring: rlen[cPn] is the vertex total
    exclusive_scan_i32(rlen, cPn + 1, sscr, st, true);
    const int* r_nr = rd.get(isStart + cPn, HostReads::kBack + 8, st);
    const int* r_nv = rd.get(rlen + cPn, HostReads::kBack + 9, st);
    r_sc = rd.get(sc, HostReads::kBack, st);
    cudaStreamSynchronize(st);
    h = *r_sc;
    if (h.anomaly) return serial_backend(pl, m, out, ovTag);
    const int nRings = *r_nr;
    const long long nv = *r_nv;
    double* rxy = (double*)bp.get("bk_rxy", sizeof(double) * 2 * (nv + 1));
    // long-segment pieces: at most nv / kSegPiece + (segments above kSegInline)
    const long long pcap = nv / kSegPiece + nv / kSegInline + 2;
    auto* pieces = (SegPiece*)bp.get("bk_pieces", sizeof(SegPiece) * pcap);
    auto* npieces = (unsigned*)bp.get("bk_npieces", 256);
    if (bp.failed) return pl.fail(kENoMem, "device allocation failed (ring vertices)");
    cudaMemsetAsync(npieces, 0, sizeof(unsigned), st);
    {
      ::sbc::KProbe kp_("k_lr_copy", st);
      k_lr_copy<<<grid_for(nE, 128), 128, 0, st>>>(T, nxA, SA, ringI, isStart, rlen, m.ixB, m.ixC,
                                                    rxy, pieces, npieces, pcap);
    }
    {
      ::sbc::KProbe kp_("k_lr_copy_long", st);
      k_lr_copy_long<<<grid_for(((long long)pcap + 1) * 32, 256) < 1216u
                           ? grid_for(((long long)pcap + 1) * 32, 256)
                           : 1216u,
                       256, 0, st>>>(m.ixB, m.ixC, rxy, pieces, npieces, pcap);
    }
    out.d_off = rlen;  // exclusive prefix of ring lengths, nRings+1 entries
    out.d_xy = rxy;
    out.nrings = nRings;
    out.nverts = nv;
  }

  // ---- clean-up and compaction
  {
    const int nR = out.nrings;
    const long long nv = out.nverts;
    int* ringOf = (int*)bp.get("cl_ringOf", sizeof(int) * (nv + 1));
    int* ringFlag = (int*)bp.get("cl_flag", sizeof(int) * (nR + 1));
    int* nxt = (int*)bp.get("cl_next", sizeof(int) * (nv + 1));
    int* prv = (int*)bp.get("cl_prev", sizeof(int) * (nv + 1));
    int* keep = (int*)bp.get("cl_keep", sizeof(int) * (nv + 1));
    int* flagV = (int*)bp.get("cl_flagV", sizeof(int) * (nv + 1));
    int* flist = (int*)bp.get("cl_flist", sizeof(int) * (nv + 1));
    int* rpre = (int*)bp.get("cl_rpre", sizeof(int) * (nR + 2));
    int* ooff = (int*)bp.get("ring_off_" + tg, sizeof(int) * (nR + 2));
    double* oxy = (double*)bp.get("ring_xy_" + tg, sizeof(double) * 2 * (nv + 1));
    void* sscr = bp.get_zeroed("cl_scan", scan_scratch_bytes(nv + nR + 4), st);
    if (bp.failed) return pl.fail(kENoMem, "device allocation failed (clean-up)");
    cudaMemsetAsync(ringFlag, 0, sizeof(int) * (nR + 1), st);
    if (nv > 0) {
      ::sbc::KProbe kp_("k_ring_of", st);
      k_ring_of<<<grid_for(nv, 256), 256, 0, st>>>(nv, nR, out.d_off, ringOf);
    }
    {
      ::sbc::KProbe kp_("k_collinear", st);
      k_collinear<<<grid_for(nv + 1, 256), 256, 0, st>>>(nv, out.d_off, ringOf, out.d_xy, ringFlag,
                                                        keep, flagV, nxt, prv);
    }
    exclusive_scan_i32(flagV, nv + 1, sscr, st, true);
    // the flagged-vertex count stays on the device (flagV[nv]); rings
    // without a flagged vertex leave k_cleanup_ring at once
    if (nv > 0) {
      {
        ::sbc::KProbe kp_("k_flag_list", st);
        k_flag_list<<<grid_for(nv, 256), 256, 0, st>>>(nv, flagV, flist);
      }
      ::sbc::KProbe kp_("k_cleanup_ring", st);
      k_cleanup_ring<<<grid_for(nR, 128), 128, 0, st>>>(nR, out.d_off, ringFlag, flist,
                                                      flagV + nv, out.d_xy, nxt, prv, keep);
    }
    int* kpv = keep;  // exclusive prefix of the keep flags (nv+1 entries)
    exclusive_scan_i32(kpv, nv + 1, sscr, st, true);
    {
      ::sbc::KProbe kp_("k_ring_nonempty", st);
      k_ring_nonempty<<<grid_for(nR + 1, 128), 128, 0, st>>>(nR, out.d_off, kpv, rpre);
    }
    exclusive_scan_i32(rpre, nR + 1, sscr, st, true);
    if (nv > 0) {
      ::sbc::KProbe kp_("k_compact_xy", st);
      k_compact_xy<<<grid_for(nv, 256), 256, 0, st>>>(nv, kpv, out.d_xy, oxy);
    }
    {
      ::sbc::KProbe kp_("k_compact_off", st);
      k_compact_off<<<grid_for(nR + 1, 128), 128, 0, st>>>(nR, nv, out.d_off, kpv, rpre, ooff);
    }
    // the two counts land with the caller's next wait on the stream
    // (Pipeline::finish_counts); both sit in one host word of this overlay
    int* hh = (int*)rd.word(HostReads::kCounts + ovTag);
    cudaMemcpyAsync(hh, rpre + nR, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(hh + 1, kpv + nv, sizeof(int), cudaMemcpyDeviceToHost, st);
    out.counts = hh;
    out.d_off = ooff;
    out.d_xy = oxy;
  }
  return kOk;
}

}  // namespace sbc

// ================================================= allocation-free tracing
// sbc_trace_rings_noalloc (include/sbclip.h) runs k_serial_backend and
// k_serial_emit, unchanged, with every pool carved out of one file-scope
// device array instead of context buffers, so the call allocates nothing.
// It serves callers that may not allocate device memory: plug-in hosts that
// own the GPU's memory and hand out fixed buffers, and processes under a hard
// device-memory cap.  The array is shared by every call on a device and keeps
// the last call's contents; calls whose device work overlaps race on it.

// Device-side scratch: every GPU that loads this library holds it until the
// process exits.  In host code this name only stands in for the symbol; its
// device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char sbc_noalloc_scratch[SBC_NOALLOC_SCRATCH_BYTES];

namespace sbc {
namespace {

constexpr size_t na_align(size_t x) { return (x + 255) & ~(size_t)255; }

// bytes of one node pool of `cap` nodes (x, y, next, prev, nb, label, enex,
// source, isect), each sub-array 256-byte aligned
constexpr size_t na_pool_bytes(long long cap) {
  return 2 * na_align(sizeof(double) * cap) + 5 * na_align(sizeof(int) * cap) + 2 * na_align(cap);
}

// Capacities the context path uses for the same pair (serial_backend above).
struct NaCaps {
  long long capP, capQ, capR, rcap;
};
constexpr NaCaps na_caps(long long nB, long long nQ, long long K) {
  return NaCaps{nB + 2 * K + 8, nQ + 2 * K + 8, nB + nQ + 2 * (2 * K + 8) + 16, nB + 16};
}

// Scratch bytes of one call: three pools, ring roots, one 256-byte block of
// counters, four byte-flag arrays.  The layout in na_carve follows this sum.
constexpr size_t na_bytes(long long nB, long long nQ, long long K) {
  return na_pool_bytes(na_caps(nB, nQ, K).capP) + na_pool_bytes(na_caps(nB, nQ, K).capQ) +
         na_pool_bytes(na_caps(nB, nQ, K).capR) + na_align(sizeof(int) * na_caps(nB, nQ, K).rcap) +
         256 + 2 * na_align(na_caps(nB, nQ, K).capP) + 2 * na_align(na_caps(nB, nQ, K).capQ);
}

// The pools need 2*(nB + nQ + 4K) + const nodes and the ring roots nB + 16
// entries, so under nB + nQ + 4K <= SBC_NOALLOC_MAX_UNITS the largest need
// is at nB = SBC_NOALLOC_MAX_UNITS, nQ = K = 0.
static_assert(na_bytes(SBC_NOALLOC_MAX_UNITS, 0, 0) <= SBC_NOALLOC_SCRATCH_BYTES,
              "allocation-free scratch array too small for its stated limit");

struct NaBump {
  unsigned char* p;
  template <class T>
  T* take(long long n) {
    T* r = (T*)p;
    p += na_align(sizeof(T) * n);
    return r;
  }
};

void na_pool(NaBump& b, long long cap, Pool& pool) {
  pool.x = b.take<double>(cap);
  pool.y = b.take<double>(cap);
  pool.next = b.take<int>(cap);
  pool.prev = b.take<int>(cap);
  pool.nb = b.take<int>(cap);
  pool.label = b.take<int>(cap);
  pool.enex = b.take<int>(cap);
  pool.source = b.take<unsigned char>(cap);
  pool.isect = b.take<unsigned char>(cap);
  pool.n = 0;
  pool.cap = (int)cap;
}

constexpr int kNaMaxDevices = 64;
std::mutex g_na_mu;
void* g_na_ptr[kNaMaxDevices] = {};

int na_fail(char* err, int err_len, int code, const char* msg, long long v0 = 0, long long v1 = 0) {
  if (err && err_len > 0) snprintf(err, (size_t)err_len, msg, v0, v1);
  return code;
}

}  // namespace
}  // namespace sbc

extern "C" int sbc_trace_rings_noalloc(const sbc_merged_lists* in, int* ring_offsets,
                                       int offsets_cap, double* ring_xy, long long xy_cap_verts,
                                       int* nrings_out, long long* nverts_out, void* stream,
                                       char* err, int err_len) {
  using namespace sbc;
  if (err && err_len > 0) err[0] = 0;
  if (!in || !ring_offsets || (!ring_xy && xy_cap_verts > 0) || !nrings_out || !nverts_out)
    return na_fail(err, err_len, SBC_EINPUT, "null argument");
  if (!in->b_xy || !in->c_xy || !in->merged_bxy || !in->merged_balpha || !in->label_b ||
      !in->merged_cxy || !in->merged_cnb || !in->label_c)
    return na_fail(err, err_len, SBC_EINPUT, "null input array");
  if (in->nb < 3 || in->nc < 3)
    return na_fail(err, err_len, SBC_EINPUT, "polygons need at least 3 vertices (base %lld, overlay %lld)",
                   in->nb, in->nc);
  if (in->n_slots_b < in->nb || in->n_slots_c < in->nc || in->n_isect < 0 || xy_cap_verts < 0)
    return na_fail(err, err_len, SBC_EINPUT,
                   "merged lists shorter than their polygons (slots %lld / %lld)", in->n_slots_b,
                   in->n_slots_c);
  const long long units = (long long)in->n_slots_b + in->n_slots_c + 4LL * in->n_isect;
  if (units > SBC_NOALLOC_MAX_UNITS)
    return na_fail(err, err_len, SBC_EINPUT,
                   "n_slots_b + n_slots_c + 4*n_isect = %lld exceeds the allocation-free limit %lld",
                   units, (long long)SBC_NOALLOC_MAX_UNITS);
  if ((long long)offsets_cap < (long long)in->n_slots_b + 17)
    return na_fail(err, err_len, SBC_EINPUT, "ring_offsets holds %lld ints, needs n_slots_b + 17 = %lld",
                   offsets_cap, (long long)in->n_slots_b + 17);
  const long long nB = in->n_slots_b, nQ = in->n_slots_c, K = in->n_isect;
  if (na_bytes(nB, nQ, K) > (size_t)SBC_NOALLOC_SCRATCH_BYTES)
    return na_fail(err, err_len, SBC_EINPUT, "scratch need %lld bytes exceeds the array (%lld)",
                   (long long)na_bytes(nB, nQ, K), (long long)SBC_NOALLOC_SCRATCH_BYTES);

  // per-device set-up: the array's device address, looked up once per device
  int dev = -1;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess)
    return na_fail(err, err_len, SBC_ECUDA, "cudaGetDevice failed (%lld)", (long long)ce);
  if (dev < 0 || dev >= kNaMaxDevices)
    return na_fail(err, err_len, SBC_EINPUT, "device ordinal %lld out of range", dev);
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[dev]) {
      void* p = nullptr;
      ce = cudaGetSymbolAddress(&p, sbc_noalloc_scratch);
      if (ce != cudaSuccess || !p)
        return na_fail(err, err_len, SBC_ECUDA, "cudaGetSymbolAddress failed (%lld)", (long long)ce);
      g_na_ptr[dev] = p;
    }
    base = (unsigned char*)g_na_ptr[dev];
  }

  // carve the pools in the order na_bytes counts them
  const NaCaps cp = na_caps(nB, nQ, K);
  SerialArgs a;
  NaBump b{base};
  na_pool(b, cp.capP, a.P);
  na_pool(b, cp.capQ, a.Q);
  na_pool(b, cp.capR, a.R);
  a.rcap = (int)cp.rcap;
  a.rroot = b.take<int>(cp.rcap);
  int* block = b.take<int>(64);    // [0..1] emit counts, [2] status, [4] ring counter
  unsigned char* flags = b.p;      // splitP, crossP (capP each), splitQ, crossQ (capQ each)
  a.splitP = b.take<unsigned char>(cp.capP);
  a.crossP = b.take<unsigned char>(cp.capP);
  a.splitQ = b.take<unsigned char>(cp.capQ);
  a.crossQ = b.take<unsigned char>(cp.capQ);
  const size_t flag_bytes = (size_t)(b.p - flags);
  a.status = block + 2;
  a.nrings = block + 4;
  a.bSize = in->nb;
  a.cSize = in->nc;
  a.cStart = 0;
  a.nB = (int)nB;
  a.nQ = (int)nQ;
  a.bP = in->b_xy;
  a.cP = in->c_xy;
  a.ixB = in->merged_bxy;
  a.ixC = in->merged_cxy;
  a.alB = in->merged_balpha;
  a.nbC = in->merged_cnb;
  a.labB = in->label_b;
  a.labC = in->label_c;

  // the flags and counters must start at zero; the pools are written before
  // they are read
  // Every runtime call's own return code is checked, and the kernels go
  // through cudaLaunchKernel, whose return is that launch's status alone: an
  // error the caller left pending on this thread is neither reported as this
  // call's nor cleared.
  cudaStream_t st = (cudaStream_t)stream;
  ce = cudaMemsetAsync(block, 0, 256, st);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(flags, 0, flag_bytes, st);
  if (ce != cudaSuccess)
    return na_fail(err, err_len, SBC_ECUDA, "cudaMemsetAsync failed (%lld)", (long long)ce);
  ++g_launches;
  {
    void* args[] = {&a};
    ce = cudaLaunchKernel((const void*)k_serial_backend, dim3(1), dim3(1), args, 0, st);
  }
  if (ce != cudaSuccess)
    return na_fail(err, err_len, SBC_ECUDA, "back-end launch failed (%lld)", (long long)ce);
  int hst = 0;
  ce = cudaMemcpyAsync(&hst, a.status, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess)
    return na_fail(err, err_len, SBC_ECUDA, "CUDA error %lld in the allocation-free back end", (long long)ce);
  if (hst == 2)
    return na_fail(err, err_len, SBC_EUNDEF, "reference behaviour undefined in the linked-list back end");
  if (hst != 0)
    return na_fail(err, err_len, SBC_EINTERNAL, "linked-list back end capacity exceeded (status %lld)", hst);
  ++g_launches;
  {
    void* args[] = {&a, &ring_offsets, &ring_xy, &xy_cap_verts, &block};
    ce = cudaLaunchKernel((const void*)k_serial_emit, dim3(1), dim3(1), args, 0, st);
  }
  if (ce != cudaSuccess)
    return na_fail(err, err_len, SBC_ECUDA, "ring-output launch failed (%lld)", (long long)ce);
  int hc[2] = {0, 0};
  ce = cudaMemcpyAsync(hc, block, sizeof(hc), cudaMemcpyDeviceToHost, st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess)
    return na_fail(err, err_len, SBC_ECUDA, "CUDA error %lld in the allocation-free ring output", (long long)ce);
  *nrings_out = hc[0];
  *nverts_out = hc[1];
  if (hc[1] > xy_cap_verts)
    return na_fail(err, err_len, SBC_EINPUT, "ring_xy holds %lld vertices, the rings need %lld",
                   xy_cap_verts, (long long)hc[1]);
  return SBC_OK;
}
