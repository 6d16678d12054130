/*
 * grazelle_phases.h -- drop-in replacement for Grazelle's include/phases.h on the GB300.
 *
 * Same names, argument meaning and call order as the reference:
 *   perform_edge_pull_phase_{pr,cc,bfs}   include/phases.h:77-78   (asm: source/phase_edge_pull_*.asm)
 *   perform_edge_push_phase_{pr,cc,bfs}   include/phases.h:81-82   (asm: source/phase_edge_push_*.asm)
 *   perform_vertex_phase_{pr,cc,bfs}      include/phases.h:85-86   (asm: source/phase_vertex_*.asm)
 *   phase_op_reset_global_accum           include/phases.h:53-54   (source/phases.asm:24-30)
 *   phase_op_write_global_accum_to_buf    include/phases.h:57-58   (source/phases.asm:34-44)
 *   phase_op_combine_global_var_from_buf  include/phases.h:61-62   (source/phases.c:27-37)
 *   edge_pull_op_merge_with_merge_buffer  include/phases.h:70      (source/phases.c:41-70)
 * and the reference's compile-time application macros (include/phases.h:28-46).
 *
 * Differences that a caller sees:
 *   - The phases act on the graph bound with grz_phases_bind() instead of on process
 *     globals.  `edge_list` is that graph's device list (grz_graph_info_t.pull_list_device /
 *     push_list_device) or any 32-byte-aligned vector offset into it, and `count` is a
 *     vector count, as in the reference.
 *   - The edge-list pointer is `const void*` because <immintrin.h> does not exist on the Arm
 *     host of a GB300.  The ABI is unchanged: one pointer argument.
 *   - One host thread makes the calls (the reference's SPMD threads become the GPU grid).
 *     Calls enqueue work on the graph's stream.  phase_op_write_global_accum_to_buf and
 *     phase_op_combine_global_var_from_buf synchronise that stream, because they return
 *     host data.
 *   - The functions return void like the reference.  A failure is recorded and can be
 *     read with grz_phases_last_status(); the host driver maps it to exit code 255, as
 *     graphdata.c:965-966 does for a bad file.
 *   - The GPU edge-pull phase combines destinations that cross work units itself.  The
 *     merge buffer it leaves has no used entry, so edge_pull_op_merge_with_merge_buffer
 *     (kept for callers, exact reference semantics on host arrays) finds nothing to merge.
 */
#ifndef GRAZELLE_PHASES_H
#define GRAZELLE_PHASES_H

#include <stdint.h>

#include "grazelle_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* element of the merge buffer, as include/graphtypes.h:27-34 */
typedef struct mergeaccum_t {
    uint64_t initial_vertex_id;
    uint64_t final_vertex_id;
    double final_partial_value;
    uint64_t __padding__;
} mergeaccum_t;

/* -------- application selection (include/phases.h:28-46) -------- */
#if defined(BREADTH_FIRST_SEARCH)
#define perform_edge_pull_phase perform_edge_pull_phase_bfs
#define perform_edge_push_phase perform_edge_push_phase_bfs
#define perform_vertex_phase perform_vertex_phase_bfs
#elif defined(CONNECTED_COMPONENTS)
#define perform_edge_pull_phase perform_edge_pull_phase_cc
#define perform_edge_push_phase perform_edge_push_phase_cc
#define perform_vertex_phase perform_vertex_phase_cc
#else
#define perform_edge_pull_phase perform_edge_pull_phase_pr
#define perform_edge_push_phase perform_edge_push_phase_pr
#define perform_vertex_phase perform_vertex_phase_pr
#endif

/* binds the graph and application that the calls below act on */
int grz_phases_bind(grz_graph* g, int app);
/* status of the last failed phase call since the last query (GRZ_OK if none); clears it */
int grz_phases_last_status(void);

/* -------- common phase operators -------- */
void phase_op_reset_global_accum(void);
void phase_op_write_global_accum_to_buf(uint64_t* reduce_buffer);
uint64_t phase_op_combine_global_var_from_buf(uint64_t* reduce_buffer);

/* -------- edge-pull engine operators -------- */
void edge_pull_op_merge_with_merge_buffer(mergeaccum_t* merge_buffer, uint64_t count, double* vertex_accumulators);

/* -------- phase control functions -------- */
void perform_edge_pull_phase_pr(const void* edge_list, const uint64_t edge_list_count);
void perform_edge_pull_phase_cc(const void* edge_list, const uint64_t edge_list_count);
void perform_edge_pull_phase_bfs(const void* edge_list, const uint64_t edge_list_count);
void perform_edge_push_phase_pr(const void* edge_list, const uint64_t edge_list_count);
void perform_edge_push_phase_cc(const void* edge_list, const uint64_t edge_list_count);
void perform_edge_push_phase_bfs(const void* edge_list, const uint64_t edge_list_count);
void perform_vertex_phase_pr(const uint64_t vertex_start, const uint64_t vertex_count, const uint64_t* reduce_buffer);
void perform_vertex_phase_cc(const uint64_t vertex_start, const uint64_t vertex_count, const uint64_t* reduce_buffer);
void perform_vertex_phase_bfs(const uint64_t vertex_start, const uint64_t vertex_count, const uint64_t* reduce_buffer);

#ifdef __cplusplus
}
#endif

#endif
