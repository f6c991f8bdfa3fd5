/*
 * sbc_oracle.h -- CPU restatement of the reference's segment-tree polygon
 * clipping path (TEST INFRASTRUCTURE ONLY: the checker, never the product).
 *
 * Restates src/clip.cpp:1415-2115 (multicore_clipping) of the reference with
 * the behaviour of its 1-thread CPU build under the two harness patches
 * (64-bit realToInt, zero-filled heap), stage by stage, so every intermediate
 * array can be compared with the CUDA path.
 */
#ifndef SBC_ORACLE_H
#define SBC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sbco_run sbco_run;

/* Which intermediate array of overlay `ov` (1-based overlay index). */
enum sbco_array {
  SBCO_RAW_B = 0, SBCO_RAW_C, SBCO_RAW_T,          /* raw candidate hits (ints) */
  SBCO_UNIQ_B, SBCO_UNIQ_C, SBCO_UNIQ_T,           /* deduplicated (ints) */
  SBCO_ISECT_XY, SBCO_ISECT_AB, SBCO_ISECT_AC,     /* records (doubles, ints, ints) */
  SBCO_MERGED_BXY, SBCO_MERGED_CXY,                /* merged vertex arrays (doubles) */
  SBCO_MERGED_BALPHA, SBCO_MERGED_CALPHA,          /* ints */
  SBCO_MERGED_BNB, SBCO_MERGED_CNB,                /* ints (1-based neighbour slot or -100) */
  SBCO_LABEL_B, SBCO_LABEL_C,                      /* initial labels (ints) */
  SBCO_RING_OFFSETS,                               /* ints: nrings+1 vertex offsets */
  SBCO_RING_XY,                                    /* doubles */
  SBCO_NUM_ARRAYS
};

/* Tree-level statistics (overlay-independent). */
enum sbco_stat {
  SBCO_STAT_EDGES = 0, SBCO_STAT_ELEM_COUNT, SBCO_STAT_TREE_SIZE,
  SBCO_STAT_COVER_TOTAL, SBCO_STAT_LEAF_END_TOTAL, SBCO_STAT_NUM
};

/* Tree-level arrays (overlay-independent), for direct checks of the tree
 * build: the padded elementary points (A4), the leaf end lists as CSR by leaf
 * (A6: leaf q's entries leaf_edge[leaf_off[q] .. leaf_off[q+1]), edge
 * indices, an edge's end entry before its start entry) and the cover lists
 * as CSR by node (A7: node v's edges cov_edge[cov_off[v] .. cov_off[v+1]),
 * ascending edge index). */
enum sbco_tree_array {
  SBCO_TREE_EA = 0,         /* doubles, epc */
  SBCO_TREE_LEAF_OFF,       /* ints, numLeaves+1 */
  SBCO_TREE_LEAF_EDGE,      /* ints */
  SBCO_TREE_COV_OFF,        /* ints, ts+1 */
  SBCO_TREE_COV_EDGE,       /* ints */
  SBCO_TREE_NUM
};
long sbco_tree_len(const sbco_run *r, int which);
const void *sbco_tree_data(const sbco_run *r, int which);

/*
 * Run the whole path for one base polygon (nb vertices, interleaved xy) and k
 * overlays (concatenated interleaved xy, sizes in c_sizes).  No closing
 * duplicate vertex.  Returns NULL only on allocation failure; check
 * sbco_status().
 */
sbco_run *sbco_clip(const double *b_xy, int nb, const double *c_xy, const int *c_sizes, int k);
/* One base against one overlay, each made of components (Foster's .poly
 * format, lib/optimizedFostersAlgorithm/README.md:43-62): component i of the
 * base is vertices [bcomp[i], bcomp[i+1]) (nbc components, bcomp[nbc] = nb),
 * likewise for the overlay.  Every component closes on its own first
 * vertex; labelling and tracing run over all components in the order of
 * Foster's multi-component code (lib/optimizedFostersAlgorithm/
 * polyclip.cpp:335-780).  One component each gives sbco_clip's result. */
sbco_run *sbco_clip_components(const double *b_xy, int nb, const int *bcomp, int nbc,
                               const double *c_xy, int nc, const int *ccomp, int ncc);
/* Union instead of intersection in the back end (the Foster code's UNION
 * switch, foster/polyclip.h:39); applies to later sbco_clip calls. */
void sbco_set_union(int on);
int sbco_status(const sbco_run *r);              /* 0 = ok, else SBCO_E* */
const char *sbco_message(const sbco_run *r);
long sbco_len(const sbco_run *r, int ov, int which);  /* element count */
const void *sbco_data(const sbco_run *r, int ov, int which);
long sbco_stat(const sbco_run *r, int which);
void sbco_free(sbco_run *r);

/* Single edge-pair classifier (reference lineSegmentIntersection). */
int sbco_segment_intersection(const double *p1, const double *p2, const double *q1,
                              const double *q2, double *alpha, double *beta);

#define SBCO_OK 0
#define SBCO_EINPUT 1      /* malformed input (fewer than 3 vertices ...) */
#define SBCO_EUNDEF 2      /* the reference's behaviour is undefined here */
#define SBCO_ENOMEM 3

#ifdef __cplusplus
}
#endif
#endif
