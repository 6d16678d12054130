// grz_phases.cu -- the reference's phase entry points (include/phases.h) on the GB300 engine.
//
// The reference's phases read and write process globals (include/graphdata.h:29-114) and keep
// per-thread state in reserved vector registers between calls (include/registers.inc:24,75).
// Here that state lives in the graph bound by grz_phases_bind(), and the global accumulator
// (the reference's ymm2 low lane, reset by phases.asm:24-30) is the graph's device-side exact
// accumulator.
#include <string.h>

#include "grz_internal.cuh"
#include "../../include/grazelle_phases.h"

int grz_pr_edge_pull(grz_graph* g, uint64_t first, uint64_t count);
int grz_pr_vertex(grz_graph* g, uint64_t first, uint64_t count, double S);
int grz_pr_push_phase(grz_graph* g, uint64_t first_vec, uint64_t count);
int grz_pr_vertex_after_push(grz_graph* g, uint64_t first, uint64_t count, double S);
int grz_cc_phase(grz_graph* g, int pull, uint64_t first_vec, uint64_t count);
int grz_bfs_phase(grz_graph* g, int pull, uint64_t first_vec, uint64_t count);
int grz_frontier_vertex_phase(grz_graph* g, uint64_t first, uint64_t count);

static grz_graph* g_bound = nullptr;
static int g_app = GRZ_APP_PAGERANK;
static int g_status = GRZ_OK;

static void note(int rc)
{
    if (rc != GRZ_OK && g_status == GRZ_OK) g_status = rc;
}

extern "C" int grz_phases_bind(grz_graph* g, int app)
{
    if (!g || app < GRZ_APP_PAGERANK || app > GRZ_APP_BREADTH_FIRST_SEARCH) return GRZ_ERR_ARG;
    g_bound = g;
    g_app = app;
    g_status = GRZ_OK;
    return GRZ_OK;
}

extern "C" int grz_phases_last_status(void)
{
    const int s = g_status;
    g_status = GRZ_OK;
    return s;
}

// maps (edge_list, count) onto a vector range of one of the bound graph's lists
static int resolve(const void* edge_list, uint64_t count, int want_push, uint64_t* first)
{
    grz_graph* g = g_bound;
    if (!g) return GRZ_ERR_STATE;
    grz_list* L = want_push ? &g->push : &g->pull;
    if (!L->nbr) return grz_set_error(g, GRZ_ERR_STATE, "%s list not loaded", want_push ? "push" : "pull");
    const int rc = grz_list_reference(g, L);  // the caller's pointer came from these vectors
    if (rc) return rc;
    const uintptr_t base = (uintptr_t)L->vs, p = (uintptr_t)edge_list;
    if (p < base || ((p - base) & 31) != 0) return grz_set_error(g, GRZ_ERR_ARG, "edge_list is not a vector of the bound graph's list");
    const uint64_t off = (p - base) / 32;
    if (off + count > L->nvec) return grz_set_error(g, GRZ_ERR_ARG, "vector range beyond the list");
    *first = off;
    return GRZ_OK;
}

// -------- common phase operators (source/phases.asm:24-44, source/phases.c:27-37) --------

extern "C" void phase_op_reset_global_accum(void)
{
    grz_graph* g = g_bound;
    if (!g) { note(GRZ_ERR_STATE); return; }
    cudaError_t e = cudaMemsetAsync(g->glob, 0, sizeof(u128) * GRZ_SUM_SLOTS, g->stream);
    if (e == cudaSuccess && g->fr.vote)
        e = cudaMemsetAsync(g->fr.vote, 0, sizeof(unsigned long long) * GRZ_VOTE_SLOTS * GRZ_VOTE_STRIDE, g->stream);
    note(grz_cuda_check(g, e, "reset global accum"));
}

// Writes the global accumulator into the calling thread's slot of the reduce buffer.  One host
// thread drives the GPU, so that is slot 0.  PageRank stores the FP64 sum's bit pattern, as the
// reference does from ymm2's low lane; CC and BFS store the vote as an integer.
extern "C" void phase_op_write_global_accum_to_buf(uint64_t* reduce_buffer)
{
    grz_graph* g = g_bound;
    if (!g || !reduce_buffer) { note(GRZ_ERR_STATE); return; }
    if (g_app == GRZ_APP_PAGERANK) {
        u128 slots[GRZ_SUM_SLOTS];
        cudaError_t e = cudaMemcpyAsync(slots, g->glob, sizeof(slots), cudaMemcpyDeviceToHost, g->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
        if (e != cudaSuccess) { note(grz_cuda_check(g, e, "read global accum")); return; }
        const double d = fx_to_double(u128_host_sum(slots, GRZ_SUM_SLOTS));
        memcpy(&reduce_buffer[0], &d, sizeof(double));
    } else {
        uint64_t v = 0;
        if (g->fr.vote) {
            const int rc = grz_read_vote(g, &v);
            if (rc) { note(rc); return; }
        }
        g->fr.vote_host = v;
        reduce_buffer[0] = v;
    }
}

// source/phases.c:27-37 over the host threads that wrote the buffer (one)
extern "C" uint64_t phase_op_combine_global_var_from_buf(uint64_t* reduce_buffer)
{
    if (!reduce_buffer) { note(GRZ_ERR_ARG); return 0; }
    return reduce_buffer[0];
}

// source/phases.c:41-70 on host arrays, SCALAR_REDUCE_OP of the bound application
// (include/execution.h:39,51,63)
extern "C" void edge_pull_op_merge_with_merge_buffer(mergeaccum_t* mb, uint64_t count, double* acc)
{
    if (!mb || !acc) return;
    const bool is_min = g_app != GRZ_APP_PAGERANK;
    uint64_t i = 0;
    while (i < count && !(mb[i].initial_vertex_id & 0x8000000000000000ull)) {
        double p = mb[i].final_partial_value;
        uint64_t j;
        for (j = i + 1; j < count && mb[j].final_vertex_id == mb[i].final_vertex_id; ++j)
            p = is_min ? (p < mb[j].final_partial_value ? p : mb[j].final_partial_value) : p + mb[j].final_partial_value;
        if (j < count && mb[j].initial_vertex_id == mb[i].final_vertex_id) {
            const double a = acc[mb[j].initial_vertex_id];
            p = is_min ? (p < a ? p : a) : p + a;
        }
        acc[mb[i].final_vertex_id] = p;
        i = j;
    }
}

// -------- phase control functions --------

extern "C" void perform_edge_pull_phase_pr(const void* edge_list, const uint64_t count)
{
    uint64_t first = 0;
    int rc = resolve(edge_list, count, 0, &first);
    if (rc == GRZ_OK) rc = grz_pr_edge_pull(g_bound, first, count);
    note(rc);
}

extern "C" void perform_edge_push_phase_pr(const void* edge_list, const uint64_t count)
{
    uint64_t first = 0;
    int rc = resolve(edge_list, count, 1, &first);
    if (rc == GRZ_OK) rc = grz_pr_push_phase(g_bound, first, count);
    note(rc);
}

// 4-wide reduce-buffer sum of source/phase_vertex_pr.asm:45-63 for one writing thread
static double reduce_buffer_sum(const uint64_t* rb)
{
    double a[4];
    memcpy(a, rb, sizeof(a));
    return (a[2] + a[3]) + (a[0] + a[1]);
}

extern "C" void perform_vertex_phase_pr(const uint64_t first, const uint64_t count, const uint64_t* reduce_buffer)
{
    grz_graph* g = g_bound;
    if (!g || !reduce_buffer) { note(GRZ_ERR_STATE); return; }
    note(grz_pr_vertex(g, first, count, reduce_buffer_sum(reduce_buffer)));
}

extern "C" void perform_edge_pull_phase_cc(const void* edge_list, const uint64_t count)
{
    uint64_t first = 0;
    int rc = resolve(edge_list, count, 0, &first);
    if (rc == GRZ_OK) rc = grz_cc_phase(g_bound, 1, first, count);
    note(rc);
}

extern "C" void perform_edge_push_phase_cc(const void* edge_list, const uint64_t count)
{
    uint64_t first = 0;
    int rc = resolve(edge_list, count, 1, &first);
    if (rc == GRZ_OK) rc = grz_cc_phase(g_bound, 0, first, count);
    note(rc);
}

extern "C" void perform_vertex_phase_cc(const uint64_t first, const uint64_t count, const uint64_t* reduce_buffer)
{
    (void)reduce_buffer;
    if (!g_bound) { note(GRZ_ERR_STATE); return; }
    note(grz_frontier_vertex_phase(g_bound, first, count));
}

extern "C" void perform_edge_pull_phase_bfs(const void* edge_list, const uint64_t count)
{
    uint64_t first = 0;
    int rc = resolve(edge_list, count, 0, &first);
    if (rc == GRZ_OK) rc = grz_bfs_phase(g_bound, 1, first, count);
    note(rc);
}

extern "C" void perform_edge_push_phase_bfs(const void* edge_list, const uint64_t count)
{
    uint64_t first = 0;
    int rc = resolve(edge_list, count, 1, &first);
    if (rc == GRZ_OK) rc = grz_bfs_phase(g_bound, 0, first, count);
    note(rc);
}

extern "C" void perform_vertex_phase_bfs(const uint64_t first, const uint64_t count, const uint64_t* reduce_buffer)
{
    (void)reduce_buffer;
    if (!g_bound) { note(GRZ_ERR_STATE); return; }
    note(grz_frontier_vertex_phase(g_bound, first, count));
}
