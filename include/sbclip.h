/*
 * sbclip.h -- C ABI of the GB300 segment-tree polygon clipping library
 * (libsbclip.so).  Plain pointers and sizes; no C++ or torch types.
 *
 * The reference exposes this path only as the `seg` command line
 * (src/clip.cpp:2117-2130 `main` -> `multicore_clipping`, src/clip.cpp:1415);
 * these entry points replace multicore_clipping one to one, and the drop-in
 * `seg` binary of this package is a thin reader/writer around them.
 *
 * Conventions
 *  - Every function returns an int status: SBC_OK (0) or one of SBC_E*.
 *    The library never exits the process; sbc_last_error() explains a failure.
 *  - Polygons are interleaved x,y doubles, one ring each, no repeated closing
 *    vertex (the reference's input file format, src/clip.cpp:181-298).
 *  - Results are rings in the reference's output order: `offsets` has
 *    nrings+1 entries (vertex offsets), `xy` 2*nverts doubles.  Result memory
 *    belongs to the context and stays valid until its next clipping call.
 *  - `stream` is a cudaStream_t (NULL: the context's own stream).
 *  - One context per host thread; contexts hold all state, no globals.
 */
#ifndef SBCLIP_H
#define SBCLIP_H

#ifdef __cplusplus
extern "C" {
#endif

#define SBC_OK 0
#define SBC_EINPUT 1     /* malformed input: < 3 vertices, non-finite coordinate, ... */
#define SBC_EUNDEF 2     /* input on which the reference's behaviour is undefined */
#define SBC_ENOMEM 3     /* device or host allocation failed */
#define SBC_ECUDA 4      /* CUDA runtime error */
#define SBC_EINTERNAL 5

typedef struct sbc_ctx sbc_ctx;

typedef struct sbc_options {
  int device;       /* CUDA device ordinal */
  int flags;        /* SBC_FLAG_* */
} sbc_options;

#define SBC_FLAG_TIMING 1          /* record per-phase CUDA-event times (sbc_stats) */
#define SBC_FLAG_SERIAL_BACKEND 2  /* run the back end's exact single-thread emulation */
#define SBC_FLAG_UNION 4           /* union instead of intersection: the Foster back end's
                                      UNION switch (foster/polyclip.h:39), which the
                                      reference's seg driver leaves off; every clipping
                                      call of the context (pair, one-to-many, batches,
                                      pairwise) then returns union rings */
#define SBC_FLAG_ENDPOINT_SORT 8   /* build the elementary intervals from a sort of all 2E edge
                                      endpoints instead of the E vertices (a test hook: the
                                      arrays and rings are the same either way) */
#define SBC_FLAG_WIDE_VERTEX_SORT 16 /* sort the vertices on their 64-bit order keys instead of
                                      32-bit keys plus the fix-up of equal-key runs (a test
                                      hook: same arrays and rings) */

typedef struct sbc_rings {
  int nrings;
  long long nverts;
  const int* offsets;   /* nrings+1 */
  const double* xy;     /* 2*nverts */
} sbc_rings;

/* Create / destroy a context (replaces the reference's process-wide state:
 * SegTree and the Foster globals bPolysList / cPolysList / rPolyList,
 * foster/polyclip.h:35-37). */
int sbc_create(const sbc_options* opt, sbc_ctx** out);
void sbc_destroy(sbc_ctx* ctx);
const char* sbc_last_error(const sbc_ctx* ctx);

/* Intersection of a base polygon with k overlays in one segment tree, exactly
 * as multicore_clipping (src/clip.cpp:1415-2115) computes it for
 * `seg base overlay_1 ... overlay_k`: out[i] receives overlay i+1's rings
 * (the reference's ../results/Fig-def-R<i+1>.txt).  Host buffers in and out;
 * host<->device copies happen inside the call. */
int sbc_clip_one_to_many(sbc_ctx* ctx, const double* b_xy, int nb, const double* c_xy,
                         const int* c_sizes, int k, sbc_rings* out, void* stream);

/* The single-pair case of sbc_clip_one_to_many (k = 1). */
int sbc_clip_pair(sbc_ctx* ctx, const double* b_xy, int nb, const double* c_xy, int nc,
                  sbc_rings* out, void* stream);

/* Device-resident variant: inputs are device pointers; `out` receives device
 * pointers (offsets and xy in device memory owned by the context). */
int sbc_clip_pair_device(sbc_ctx* ctx, const double* d_b_xy, int nb, const double* d_c_xy,
                         int nc, sbc_rings* out, void* stream);

/* Diagnostics of the last call, written into out[0..n): see SBC_STAT_*. */
#define SBC_STAT_EDGES 0
#define SBC_STAT_ELEMENTARY_POINTS 1
#define SBC_STAT_TREE_SIZE 2
#define SBC_STAT_COVER_ENTRIES 3
#define SBC_STAT_LEAF_END_ENTRIES 4
#define SBC_STAT_CANDIDATES_TESTED 5    /* overlay 1: box-overlapping edge pairs passing LSMF */
#define SBC_STAT_RAW_HITS 6             /* overlay 1: the reference's raw candidate hits */
#define SBC_STAT_UNIQUE 7               /* overlay 1: unique intersecting edge pairs */
#define SBC_STAT_SLOTS_B 8
#define SBC_STAT_SLOTS_C 9
#define SBC_STAT_SERIAL_BACKEND 10      /* 1 if the exact serial back end ran */
#define SBC_STAT_WORK_UNITS 11          /* overlay 1: edge-box pairs tested by the grid join */
#define SBC_STAT_GRID_PAIRS 12          /* overlay 1: box-overlapping edge pairs the grid found */
#define SBC_STAT_VERTEX_SORT 13         /* the endpoint order came from: 0 the endpoint sort,
                                           1 the vertex sort on 64-bit keys, 2 the vertex sort
                                           on 32-bit keys with equal-key runs fixed up */
#define SBC_STAT_OUTSIDE_CMBR 14        /* edges whose box misses the common MBR of the base and
                                           the overlays (left out of the candidate search; the
                                           reference's getCMBR, src/clip.cpp:743-777) */
#define SBC_STAT_NUM 15
int sbc_stats(const sbc_ctx* ctx, long long* out, int n);

/* Per-phase device milliseconds of the last call when SBC_FLAG_TIMING is set:
 * [setup, elementary, end lists, cover lists, candidates+merge, back end,
 *  device->host, total]. */
int sbc_phase_times(const sbc_ctx* ctx, float* out_ms, int n);

/* Intermediate arrays of the last overlay of the last call (for parity
 * checks), copied to host memory: see SBC_ARR_*.  Returns the element count
 * in *count (the copy is truncated to cap elements). */
#define SBC_ARR_UNIQ_B 0       /* int */
#define SBC_ARR_UNIQ_C 1       /* int */
#define SBC_ARR_UNIQ_T 2       /* int */
#define SBC_ARR_ISECT_XY 3     /* double */
#define SBC_ARR_ISECT_AB 4     /* int */
#define SBC_ARR_ISECT_AC 5     /* int */
#define SBC_ARR_MERGED_BXY 6   /* double */
#define SBC_ARR_MERGED_CXY 7   /* double */
#define SBC_ARR_MERGED_BALPHA 8
#define SBC_ARR_MERGED_CALPHA 9
#define SBC_ARR_MERGED_BNB 10
#define SBC_ARR_MERGED_CNB 11
#define SBC_ARR_LABEL_B 12
#define SBC_ARR_LABEL_C 13
/* tree arrays of the last call (overlay-independent) */
#define SBC_ARR_ELEMENTARY 14  /* double: the padded elementary points (2^k+1) */
#define SBC_ARR_LEAF_AFTER 15  /* int per edge: leaf node of its end-list entry from its end, or -1 */
#define SBC_ARR_LEAF_BEFORE 16 /* int per edge: leaf node of its entry from its start, or -1 */
#define SBC_ARR_LEAF_RANGE 17  /* int pairs per edge: leaves [l, r1) its cover lists span */
int sbc_debug_array(sbc_ctx* ctx, int which, void* host_dst, long long cap, long long* count);

/* Edge-pair classification of n pairs (p1,p2,q1,q2 as 8 doubles per pair,
 * host memory) on the device: the reference's lineSegmentIntersection
 * (p_seg_tree/oacc_segment_tree.cpp:5426-5517) with alphaToInt
 * (:7247-7252).  types/alpha/beta/alpha_int/beta_int receive n values each
 * (any output pointer may be NULL). */
int sbc_classify_pairs(sbc_ctx* ctx, const double* pairs, int n, int* types, double* alpha,
                       double* beta, int* alpha_int, int* beta_int);

/* ---- Batches of independent pairs --------------------------------------
 * Many base/overlay pairs in one call: the result for every pair equals
 * sbc_clip_pair on that pair (the reference's `seg base overlay`, run once
 * per pair; the reference itself has no batched call).  Polygons are
 * concatenated: pair p's base is vertices [b_off[p], b_off[p+1]) of b_xy, its
 * overlay vertices [c_off[p], c_off[p+1]) of c_xy.  A pair whose polygons
 * have at most SBC_BATCH_MAX_VERTICES vertices is clipped by one device
 * thread, all such pairs in one launch per chunk (consecutive pairs whose
 * scratch arenas fit the budget, sbc_batch_set_arena_budget); a pair with a
 * larger polygon is clipped by the single-pair pipeline.  A polygon needs at
 * least 3 vertices; a pair with a smaller one gets status SBC_EINPUT and no
 * rings.  Per-pair failures (SBC_EUNDEF where the reference's behaviour is
 * undefined) are reported in the per-pair status; the call itself fails only
 * on argument, allocation or CUDA errors. */
#define SBC_BATCH_MAX_VERTICES 4096
typedef struct sbc_batch {
  int npairs;
  const double* b_xy;
  const long long* b_off;     /* npairs+1 */
  const double* c_xy;
  const long long* c_off;     /* npairs+1 */
} sbc_batch;

typedef struct sbc_batch_rings {
  int npairs;
  long long nrings, nverts;
  const long long* pair_ring; /* npairs+1: pair p owns rings [pair_ring[p], pair_ring[p+1]) */
  const long long* ring_off;  /* nrings+1 vertex offsets into xy */
  const double* xy;           /* 2*nverts */
  const int* status;          /* npairs */
} sbc_batch_rings;

/* Rings of every pair.  sbc_clip_batch: host arrays in, host arrays out
 * (owned by the context until its next call).  _device: device arrays in,
 * device arrays out (owned by the context). */
int sbc_clip_batch(sbc_ctx* ctx, const sbc_batch* batch, sbc_batch_rings* out, void* stream);
int sbc_clip_batch_device(sbc_ctx* ctx, const sbc_batch* batch, sbc_batch_rings* out,
                          void* stream);

/* Intersection area of every pair: the sum of the shoelace areas of its rings
 * (0 for pairs whose status is not SBC_OK).  area[npairs], status[npairs]
 * (status may be NULL).  Host arrays, or device arrays for _device. */
int sbc_area_forward(sbc_ctx* ctx, const sbc_batch* batch, double* area, int* status,
                     void* stream);
int sbc_area_forward_device(sbc_ctx* ctx, const sbc_batch* batch, double* area, int* status,
                            void* stream);

/* Gradient of sum_p grad_area[p] * area[p] with respect to every vertex
 * coordinate, with the combinatorial structure of each result held fixed:
 * grad_b receives 2 * b_off[npairs] doubles, grad_c 2 * c_off[npairs].  A ring
 * vertex that is a proper crossing passes its gradient to both edges through
 * I = (1 - alpha) b1 + alpha b2, alpha = A(b1,c1,c2) / (A(b1,c1,c2) - A(b2,c1,c2)).
 * _device reuses the records of the last sbc_area_forward_device call on this
 * context when it was given the same batch (same arrays and count), and runs
 * the forward pass first otherwise; the host variant always runs it. */
int sbc_area_backward(sbc_ctx* ctx, const sbc_batch* batch, const double* grad_area,
                      double* grad_b, double* grad_c, void* stream);
int sbc_area_backward_device(sbc_ctx* ctx, const sbc_batch* batch, const double* grad_area,
                             double* grad_b, double* grad_c, void* stream);

/* ---- Polygons with several components (holes, islands) ------------------
 * A polygon may be made of components, as in the .poly files of the
 * reference's Foster program (lib/optimizedFostersAlgorithm/README.md:43-62:
 * `x y,` per vertex, `;` closing a component); the seg driver itself reads
 * one ring per file (gpc_read_multi_polygon, src/clip.cpp:172-311).  Every
 * component closes on its own first vertex.  Labelling and tracing follow
 * Foster's multi-component code (lib/optimizedFostersAlgorithm/
 * polyclip.cpp:335-780): a point is inside a polygon when an odd number of
 * its components contain it, a component without crossings is kept whole
 * when it lies inside the other polygon, an identical component is kept when
 * both are holes or neither is.  With one component per polygon the result
 * is the batch engine's (and the reference's) ring for ring.
 *
 * b_comp lists the first vertex of every base component of the batch in
 * ascending order and ends with b_off[npairs] (nb_comp + 1 entries,
 * b_comp[0] = 0); every non-empty polygon starts a component, so none spans
 * two pairs, and every component has at least 3 vertices.  Likewise c_comp.
 * A null array: one ring per polygon on that side.  Pairs with components
 * are clipped by the batch engine whatever their size. */
typedef struct sbc_components {
  const long long* b_comp;
  long long nb_comp;
  const long long* c_comp;
  long long nc_comp;
} sbc_components;

/* sbc_clip_batch with components (host arrays; _device: device arrays, the
 * offsets read back once to be checked). */
int sbc_clip_batch_components(sbc_ctx* ctx, const sbc_batch* batch, const sbc_components* comps,
                              sbc_batch_rings* out, void* stream);
int sbc_clip_batch_components_device(sbc_ctx* ctx, const sbc_batch* batch,
                                     const sbc_components* comps, sbc_batch_rings* out,
                                     void* stream);
/* One pair, host arrays: base components [b_comp[i], b_comp[i+1]) of b_xy
 * (nb_comp components, b_comp[0] = 0), likewise the overlay.  The call fails
 * with the pair's status (SBC_EUNDEF, ...) when the pair fails. */
int sbc_clip_components(sbc_ctx* ctx, const double* b_xy, const int* b_comp, int nb_comp,
                        const double* c_xy, const int* c_comp, int nc_comp, sbc_rings* out,
                        void* stream);
/* Area forward / backward (sbc_area_forward_device, sbc_area_backward_device)
 * with components; the backward reuses the forward's records when given the
 * same batch and component arrays. */
int sbc_area_forward_components_device(sbc_ctx* ctx, const sbc_batch* batch,
                                       const sbc_components* comps, double* area, int* status,
                                       void* stream);
int sbc_area_backward_components_device(sbc_ctx* ctx, const sbc_batch* batch,
                                        const sbc_components* comps, const double* grad_area,
                                        double* grad_b, double* grad_c, void* stream);

/* ---- One base against many overlays, pairwise ---------------------------
 * The rings of `seg base overlay_i` for every overlay i (each equal to
 * sbc_clip_pair(base, overlay_i)); the reference has no such call and is run
 * once per overlay for it (multicore_clipping, src/clip.cpp:1415-2115, with
 * one overlay).  Unlike sbc_clip_one_to_many, whose results follow the
 * reference's single tree over all overlays (at most 9), every overlay here
 * gets the result of its own pair, for any number of overlays.  The base is
 * prepared once; overlay i is vertices [c_off[i], c_off[i+1]) of c_xy.  An
 * overlay with fewer than 3 vertices gets status SBC_EINPUT and no rings;
 * SBC_EUNDEF marks a pair on which the reference's behaviour is undefined.
 * Output as for sbc_clip_batch (npairs = noverlays): host arrays owned by the
 * context for sbc_clip_pairwise, device arrays for _device. */
typedef struct sbc_pairwise_job {
  const double* b_xy;         /* 2*nb */
  int nb;
  int noverlays;
  const double* c_xy;
  const long long* c_off;     /* noverlays+1 */
} sbc_pairwise_job;
int sbc_clip_pairwise(sbc_ctx* ctx, const sbc_pairwise_job* job, sbc_batch_rings* out,
                      void* stream);
int sbc_clip_pairwise_device(sbc_ctx* ctx, const sbc_pairwise_job* job, sbc_batch_rings* out,
                             void* stream);
/* Area of every overlay's result (the signed shoelace sum of its rings, 0
 * where the status is not SBC_OK) and its gradient, for device arrays:
 * sbc_pairwise_area_device clips the job (as sbc_clip_pairwise_device) and
 * writes area[noverlays] and, if status is not NULL, status[noverlays].
 * sbc_pairwise_area_backward_device writes d(sum_i grad_area[i] area[i]) /
 * d(vertex) with the combinatorial structure held fixed: grad_b (2*nb
 * doubles, summed over every overlay) and grad_c (2*c_off[noverlays]); it
 * reuses the last pairwise call's rings when given the same job arrays and
 * clips first otherwise.  A ring vertex's provenance is found by exact
 * coordinates: a base vertex first, then an overlay vertex, then a proper
 * crossing I = (1 - a) b1 + a b2.  Contributions are added atomically, so the
 * last bits of the sums may differ between runs. */
int sbc_pairwise_area_device(sbc_ctx* ctx, const sbc_pairwise_job* job, double* area, int* status,
                             void* stream);
int sbc_pairwise_area_backward_device(sbc_ctx* ctx, const sbc_pairwise_job* job,
                                      const double* grad_area, double* grad_b, double* grad_c,
                                      void* stream);
/* Diagnostics of the last sbc_clip_pairwise call: out[0] overlays clipped by
 * the single-pair pipeline (inputs outside the batched path's conditions),
 * out[1] unique intersecting edge pairs, out[2] box-overlapping edge pairs
 * tested, out[3] cells of the base grid, out[4] overlays whose records went
 * through the single-pair pipeline's data-parallel rows A9-A18 (see
 * sbc_pairwise_set_split). */
int sbc_pairwise_info(const sbc_ctx* ctx, long long* out, int n);
/* Base-grid cell width of sbc_clip_pairwise in units of
 * max(sqrt(base bounding-box area / nb), 1.5 mean base edge extents); default
 * 1.  A tuning knob: results do not depend on it. */
int sbc_pairwise_set_cell_factor(sbc_ctx* ctx, double factor);
/* Overlays with at least `records` intersecting edge pairs leave the
 * one-warp-per-pair back end for the data-parallel one (several such overlays
 * at a time, each on its own stream); default 8192.  A tuning knob: results
 * do not depend on it. */
int sbc_pairwise_set_split(sbc_ctx* ctx, int records);
/* Host worker threads (each with its own stream) that clip the big overlays
 * concurrently with the one-warp-per-pair kernel; default 8, 1 to 64.  A
 * tuning knob: results do not depend on it (1 serialises the big overlays,
 * which per-kernel profiling needs).  sbc_pairwise_get_workers reads it. */
int sbc_pairwise_set_workers(sbc_ctx* ctx, int workers);
int sbc_pairwise_get_workers(const sbc_ctx* ctx);
/* Autotuner: runs the job (device arrays, as for sbc_clip_pairwise_device)
 * under several splits, block-slot reserves and worker counts for the big
 * overlays, and cell widths, keeps the fastest setting in the
 * context and reports it (any output may be NULL).  The rings of the last run
 * are left as sbc_clip_pairwise_device would leave them. */
int sbc_pairwise_autotune(sbc_ctx* ctx, const sbc_pairwise_job* job, int* split,
                          double* cell_factor, double* best_ms, void* stream);

/* The area forward + backward of one batch as a single CUDA graph launch.
 * sbc_area_graph_create runs the batch once (device arrays, as for the
 * _device calls) to fix its arena chunk, scratch buffers and the pairs that
 * need a second pass with more hit room, then records pass one, the second
 * pass, the backward pass and copies of area and status (either may be NULL)
 * into a graph.  sbc_area_graph_launch replays it on `stream`: the batch's
 * arrays are read anew, so new coordinates of the same polygons give new
 * areas and gradients; a pair that now needs more hit room than recorded
 * reports SBC_ENOMEM in its status (re-create the graph then).  The graph
 * uses the context's batch buffers: a later batched call on the context makes
 * it stale and sbc_area_graph_launch then fails with SBC_EINPUT.  Needs a
 * batch that fits one arena chunk with no polygon above SBC_BATCH_MAX_VERTICES
 * vertices. */
typedef struct sbc_graph sbc_graph;
int sbc_area_graph_create(sbc_ctx* ctx, const sbc_batch* batch, const double* grad_area,
                          double* grad_b, double* grad_c, double* area, int* status,
                          void* stream, sbc_graph** out);
int sbc_area_graph_launch(sbc_graph* graph, void* stream);
void sbc_area_graph_destroy(sbc_graph* graph);

/* Bytes of per-pair scratch arenas one chunk of a batch may hold (0: the
 * smaller of 96 GiB and half of the device's free memory).  A batch larger
 * than one chunk runs chunk by chunk; its backward pass then recomputes each
 * chunk's forward pass instead of keeping every intersection record. */
int sbc_batch_set_arena_budget(sbc_ctx* ctx, long long bytes);
/* Shape of the last batch call: out[0] chunks, out[1] pairs clipped by the
 * single-pair pipeline because a polygon exceeds the small/large split. */
int sbc_batch_info(const sbc_ctx* ctx, long long* out, int n);
/* Tuning knobs of the batch engine, shape[5]: block sizes (threads: 32, 64,
 * 96 or 128) of the per-pair front kernel, the warp-per-pair candidate
 * kernel, the per-pair back end and the backward kernel, then the small/large
 * split (a pair with a polygon above it is clipped by the single-pair
 * pipeline; 3 to SBC_BATCH_MAX_VERTICES, default SBC_BATCH_MAX_VERTICES).
 * Results do not depend on them.  A graph (sbc_area_graph_create) needs a
 * batch with no polygon above the split. */
int sbc_batch_set_shape(sbc_ctx* ctx, const int* shape);
int sbc_batch_get_shape(const sbc_ctx* ctx, int* shape);
/* Autotuner: times the batch's area forward + backward (device arrays, as for
 * the _device calls; grad_b and grad_c are overwritten) under each knob's
 * settings in turn, keeps the fastest in the context and reports it in
 * shape[5] and best_ms (either may be NULL).  A split below the batch's
 * largest polygons is tried only when it moves at most 64 pairs to the
 * single-pair pipeline.  The reference has no counterpart: it clips pairs one
 * at a time. */
int sbc_batch_autotune(sbc_ctx* ctx, const sbc_batch* batch, const double* grad_area,
                       double* grad_b, double* grad_c, int* shape, double* best_ms,
                       void* stream);

/* Allocation-free ring tracing.  No counterpart in the reference: it exists
 * for callers that are not allowed to allocate device memory themselves or
 * through this library -- for example an engine that owns every byte of the
 * GPU and hands each plug-in fixed input and output buffers, or a process
 * running against a hard device-memory cap where a cudaMalloc would fail or
 * spoil the host's accounting.  Every other entry point grows
 * context-owned device buffers on demand; this one allocates nothing.
 *
 * It runs the library's exact linked-list back end (the reference's
 * copyToLinkedList, labelIntersections2, createResult2 and cleanUpResult2,
 * applied one step at a time by a single device thread) on the merged
 * vertex/intersection lists of ONE base/overlay pair.  Those lists are the
 * arrays sbc_debug_array exports after a clipping call: merged_bxy and
 * merged_cxy (SBC_ARR_MERGED_BXY / _CXY), merged_balpha (SBC_ARR_MERGED_BALPHA),
 * merged_cnb (SBC_ARR_MERGED_CNB), label_b and label_c (SBC_ARR_LABEL_B / _C);
 * n_isect is the number of unique intersecting edge pairs (SBC_ARR_UNIQ_B's
 * count).  The result equals sbc_clip_pair's rings for that pair.  Array
 * contents are not validated: pass the lists of one pair unchanged.
 *
 * Limits and sharing:
 *  - The node pools live in one file-scope device array of
 *    SBC_NOALLOC_SCRATCH_BYTES (24 MiB), which every GPU that loads the
 *    library holds until the process exits.  A call must satisfy
 *    n_slots_b + n_slots_c + 4 * n_isect <= SBC_NOALLOC_MAX_UNITS; larger
 *    calls are rejected with SBC_EINPUT before any device work.
 *  - The first call on a device looks up that array's device address (once
 *    per device, with the device current); make that first call before any
 *    stream capture begins.
 *  - All calls on a device share the array, and it keeps the last call's
 *    contents.  Calls whose device work overlaps (different streams, or
 *    different host threads, without ordering between them) race on it;
 *    order them, e.g. by issuing them on one stream.
 *  - Runs on the calling thread's current device; `stream` must belong to
 *    it (NULL: the legacy default stream).  The call waits for its own work
 *    on `stream` before it returns.
 *
 * Inputs are device pointers.  Outputs: ring_offsets (device, at least
 * n_slots_b + 17 ints, checked), ring_xy (device, room for xy_cap_verts
 * vertices = 2*xy_cap_verts doubles), *nrings_out and *nverts_out (host).
 * If the rings need more than xy_cap_verts vertices the call returns
 * SBC_EINPUT with *nverts_out set to the number needed.  A message for any
 * non-zero status is written to err (err_len bytes, may be NULL). */
#define SBC_NOALLOC_MAX_UNITS 262144
#define SBC_NOALLOC_SCRATCH_BYTES (24 * 1024 * 1024)
typedef struct sbc_merged_lists {
  const double* b_xy;          /* base polygon, nb vertices (2*nb doubles) */
  int nb;
  const double* c_xy;          /* overlay polygon, nc vertices */
  int nc;
  const double* merged_bxy;    /* 2*n_slots_b doubles */
  const int* merged_balpha;    /* n_slots_b */
  const int* label_b;          /* n_slots_b */
  int n_slots_b;
  const double* merged_cxy;    /* 2*n_slots_c doubles */
  const int* merged_cnb;       /* n_slots_c */
  const int* label_c;          /* n_slots_c */
  int n_slots_c;
  int n_isect;
} sbc_merged_lists;
int sbc_trace_rings_noalloc(const sbc_merged_lists* in, int* ring_offsets, int offsets_cap,
                            double* ring_xy, long long xy_cap_verts, int* nrings_out,
                            long long* nverts_out, void* stream, char* err, int err_len);

/* Number of this library's kernel launches in the process so far. */
unsigned long long sbc_kernel_launches(void);

/* Per-kernel device times (diagnostics; no counterpart in the reference).
 * Between sbc_profile_begin and sbc_profile_end every launch of this library
 * is bracketed by CUDA events on its stream.  sbc_profile_end writes up to
 * `cap` kernels: NUL-separated names into `names` (names_len bytes), total
 * milliseconds into ms[i], launch counts into counts[i], and the launches'
 * summed algorithmic bytes (inputs read and outputs written once, 0 where a
 * launch states none) into bytes[i]; *n_out = kernels.  Any output pointer
 * may be NULL. */
int sbc_profile_begin(void);
int sbc_profile_end(char* names, int names_len, float* ms, int* counts, double* bytes, int cap,
                    int* n_out);
/* The launches of the window the last sbc_profile_end closed, in launch
 * order (a device timeline; diagnostics): up to `cap` NUL-separated names,
 * start_ms[i] from the first launch's start to launch i's start, dur_ms[i],
 * and stream[i], the streams numbered in order of first use.  Gaps between
 * one launch's end and the next one's start on a stream are idle time: host
 * round trips and launch latency.  *n_out = launches; any output pointer may
 * be NULL. */
int sbc_profile_timeline(char* names, int names_len, float* start_ms, float* dur_ms, int* stream,
                         int cap, int* n_out);

/* Library version string. */
const char* sbc_version(void);

#ifdef __cplusplus
}
#endif
#endif
