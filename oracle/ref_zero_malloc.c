/*
 * Zero-filling malloc for the reference CPU build (oracle harness only).
 *
 * The reference reads heap memory it never wrote: the vertical-line flags and
 * the elementary-index flags (p_seg_tree/oacc_segment_tree.cpp:4562-4576), the
 * last border slot (oacc_segment_tree.cpp:1985-2007 writes epc-1 of epc
 * entries) and never-initialised omp locks (segment_tree.h:150-156).  Routing
 * malloc through glibc's calloc makes every such read return zero, so the
 * binary is deterministic and its behaviour is the one this repository
 * restates.
 */
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

extern void *__libc_calloc(size_t nmemb, size_t size);

void *malloc(size_t n) { return __libc_calloc(1, n); }

#ifdef __cplusplus
}
#endif
