/*
 * grz_oracle.c -- CPU restatement of Grazelle's hot path (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py load this library, and only to check or time
 * the GPU product against it.  The product never links, loads or calls it.
 *
 * Each function restates one piece of the reference, which is x86-64 AVX2
 * assembly plus C, in portable scalar C.  The file:line citations point into
 * the reference tree.  The serial functions follow the single-thread (-n 1)
 * behaviour of the reference exactly:
 *   - work units are processed in index order, as one thread claims them
 *     (include/scheduler_pull.inc:63-87);
 *   - the per-vector FP64 sum order is (g2+g3)+(g0+g1), then acc = s + acc
 *     (source/phase_edge_pull_pr.asm:146-149);
 *   - the merge-buffer fold is in unit order (source/phases.c:41-70);
 *   - the vertex phase uses separate multiply and add, no FMA
 *     (source/phase_vertex_pr.asm:116-128).
 * At -n 1 their output is therefore bit-identical to the reference.  The
 * tests in tests/test_oracle_vs_reference.py check this against the
 * reference binary built by oracle/build_ref.py.
 *
 * The oracle_*_mt functions are the multi-threaded CPU baseline.  They use
 * OpenMP with the same work-unit split and dynamic unit claiming as the
 * reference's SPMD threads (source/main.c:75-90).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_VALID 0x8000000000000000ull
#define ORC_ID48 0x0000ffffffffffffull
#define ORC_NO_EDGES 0x7fffffffffffffffull
#define ORC_PAST_END 0xffffffffffffffffull

/* ------------------------------------------------------------------------- */
/* A1: vector-sparse edge vectors                                             */
/* ------------------------------------------------------------------------- */

/* Shared (spread-encoded) vertex of one 4-lane vector; source/graphdata.c:114-120. */
static inline uint64_t orc_shared(const uint64_t* v)
{
    return ((v[0] & 0x7fff000000000000ull) >> 48) | ((v[1] & 0x7fff000000000000ull) >> 33) |
           ((v[2] & 0x7fff000000000000ull) >> 18) | ((v[3] & 0x0007000000000000ull) >> 3);
}

uint64_t oracle_shared_id(const uint64_t* v) { return orc_shared(v); }

/* One vector from a stash; source/graphdata.c:143-173 (graph_helper_write_edge_vector). */
static inline void orc_write_vector(uint64_t* out, uint64_t shared, const uint64_t* ids, uint32_t count)
{
    const uint64_t piece[4] = { (shared & 0x0000000000007fffull) >> 0, (shared & 0x000000003fff8000ull) >> 15,
                                (shared & 0x00001fffc0000000ull) >> 30, (shared & 0x0000e00000000000ull) >> 45 };
    for (int k = 0; k < 4; ++k)
        out[k] = ((count > (uint32_t)k ? 1ull : 0ull) << 63) | (piece[k] << 48) | ids[k];
}

/*
 * Packs an edge list (interleaved src,dst pairs, already grouped by the shared
 * vertex) into 4-lane vectors; source/graphdata.c:618-701 (in-edges, shared = dst)
 * and :705-788 (out-edges, shared = src).  A vector is flushed when the shared
 * vertex changes or the stash holds 4.  Invalid lanes keep the stale neighbour
 * IDs left in the stash (the stash is never cleared), and one final vector is
 * always written, even for an empty list.  Returns the vector count; `out` must
 * hold max(E,1) vectors (4 words each).
 */
uint64_t oracle_pack_vectors(const uint64_t* pairs, uint64_t num_edges, int shared_is_dst, uint64_t* out)
{
    uint64_t stash[4] = { 0, 0, 0, 0 };
    uint64_t stash_shared = 0;
    uint32_t stash_count = 0;
    uint64_t n = 0;
    for (uint64_t e = 0; e < num_edges; ++e) {
        const uint64_t src = pairs[2 * e], dst = pairs[2 * e + 1];
        const uint64_t sh = shared_is_dst ? dst : src;
        const uint64_t nb = shared_is_dst ? src : dst;
        if ((stash_count != 0 && stash_shared != sh) || stash_count == 4) {
            orc_write_vector(out + 4 * n, stash_shared, stash, stash_count);
            ++n;
            stash_count = 0;
        }
        stash_shared = sh;
        stash[stash_count++] = nb;
    }
    orc_write_vector(out + 4 * n, stash_shared, stash, stash_count);
    return n + 1;
}

/*
 * A2: per-vertex index of the first vector; source/graphdata.c:219-267.
 * index_count is V + 64 in the reference (graphdata.c:371,408).
 */
void oracle_vertex_index(const uint64_t* vec, uint64_t nvec, uint64_t* index, uint64_t index_count,
                         uint64_t* start_out, uint64_t* end_out)
{
    uint64_t cur = orc_shared(vec);
    for (uint64_t i = 0; i < cur; ++i) index[i] = ORC_NO_EDGES;
    index[cur] = 0;
    uint64_t last = cur;
    *start_out = cur;
    for (uint64_t i = 1; i < nvec; ++i) {
        cur = orc_shared(vec + 4 * i);
        if (last != cur) {
            while (last < cur - 1) index[++last] = ORC_NO_EDGES;
            index[cur] = i;
            last = cur;
        }
    }
    *end_out = cur;
    for (uint64_t i = cur + 1; i < index_count; ++i) index[i] = ORC_PAST_END;
}

/* A3: outdegree credit per source over the -pull file; source/graphdata.c:792-821. */
void oracle_outdegrees(const uint64_t* pairs, uint64_t num_edges, uint64_t num_vertices, double* outdeg)
{
    memset(outdeg, 0, sizeof(double) * num_vertices);
    for (uint64_t e = 0; e < num_edges; ++e) outdeg[pairs[2 * e]] += 1.0;
}

/* A4: unit u covers [q*u + min(r,u), +q+(u<r)); include/scheduler_pull.inc:94-138. */
static inline void orc_unit_range(uint64_t nvec, uint64_t units, uint64_t u, uint64_t* lo, uint64_t* hi)
{
    const uint64_t q = nvec / units, r = nvec % units;
    *lo = q * u + (u < r ? u : r);
    *hi = *lo + q + (u < r ? 1 : 0);
}

/* ------------------------------------------------------------------------- */
/* PageRank                                                                    */
/* ------------------------------------------------------------------------- */

typedef struct orc_merge { uint64_t initial, final_; double partial; uint64_t pad; } orc_merge;

/* A6: source/phases.c:41-70 with SCALAR_REDUCE_OP = + (include/execution.h:63). */
static void orc_merge_sum(const orc_merge* mb, uint64_t count, double* accum)
{
    uint64_t i = 0;
    while (i < count && !(mb[i].initial & ORC_VALID)) {
        double p = mb[i].partial;
        uint64_t j;
        for (j = i + 1; j < count && mb[j].final_ == mb[i].final_; ++j) p = p + mb[j].partial;
        if (j < count && mb[j].initial == mb[i].final_) p = p + accum[mb[j].initial];
        accum[mb[i].final_] = p;
        i = j;
    }
}

/*
 * A5: one unit of perform_edge_pull_phase_pr; source/phase_edge_pull_pr.asm:45-183, 244-290.
 * Returns the unit's contribution to the thread's global accumulator, in the
 * order the asm adds it (one add per finished run, then the merge-entry add).
 */
static double orc_pr_pull_unit(const uint64_t* vec, uint64_t lo, uint64_t hi, const double* prop, double* accum,
                               orc_merge* entry, double glob)
{
    uint64_t prev = orc_shared(vec + 4 * lo);
    entry->initial = prev;
    double acc = 0.0;
    for (uint64_t i = lo; i < hi; ++i) {
        const uint64_t* v = vec + 4 * i;
        double g[4];
        for (int k = 0; k < 4; ++k) g[k] = (v[k] & ORC_VALID) ? prop[v[k] & ORC_ID48] : 0.0;
        const uint64_t dst = orc_shared(v);
        if (prev != dst) {
            accum[prev] = acc;
            glob = glob + acc;
            acc = 0.0;
        }
        prev = dst;
        const double s = (g[2] + g[3]) + (g[0] + g[1]);
        acc = s + acc;
    }
    glob = glob + acc;
    entry->final_ = prev;
    entry->partial = acc;
    return glob;
}

/*
 * A7: perform_vertex_phase_pr; source/phase_vertex_pr.asm:27-134.
 * S is the reduce-buffer total; G = (1 - S) / V; (1-d)/V from include/phasehelpers.inc:48-53.
 */
static void orc_pr_vertex(uint64_t first, uint64_t count, const double* accum, const double* outdeg, double* prop,
                          double S, double num_vertices, double damping)
{
    const double G = (1.0 - S) / num_vertices;
    const double c = (1.0 - damping) / num_vertices;
    for (uint64_t v = first; v < first + count; ++v) {
        const double deg = outdeg[v] == 0.0 ? num_vertices : outdeg[v];
        double t = accum[v] + G;
        t = t * damping;
        t = t + c;
        prop[v] = t / deg;
    }
}

/* A8: execution_initialize_vertex_prop_pr; source/execution_pr.c:85-88. */
void oracle_pr_init(uint64_t num_vertices, const double* outdeg, double* prop, double* accum)
{
    const double V = (double)num_vertices;
    for (uint64_t v = 0; v < num_vertices; ++v) {
        prop[v] = (1.0 / V) / (outdeg[v] == 0.0 ? V : outdeg[v]);
        accum[v] = 0.0;
    }
}

/* The 4-wide reduce-buffer sum of the vertex phase (phase_vertex_pr.asm:45-63). */
static double orc_reduce_buffer_sum(const double* rb, uint64_t threads)
{
    double a[4] = { 0, 0, 0, 0 };
    const uint64_t blocks = ((threads - 1) >> 2) + 1;
    for (uint64_t b = 0; b < blocks; ++b)
        for (int k = 0; k < 4; ++k) a[k] = a[k] + rb[4 * b + k];
    return (a[2] + a[3]) + (a[0] + a[1]);
}

/*
 * PageRank with the pull engine, single thread (execution_impl_pr,
 * source/execution_pr.c:92-168).  `units` = 32 x threads by default
 * (source/main.c:75-90).  prop/accum must be initialised (oracle_pr_init).
 * damping is 0.875 in the reference (source/constants.asm:75-79).
 */
void oracle_pr_pull(const uint64_t* vec, uint64_t nvec, const double* outdeg, uint64_t num_vertices, uint32_t iters,
                    double damping, uint64_t units, double* prop, double* accum)
{
    orc_merge* mb = (orc_merge*)malloc(sizeof(orc_merge) * units);
    double rb[8];
    for (uint32_t it = 0; it < iters; ++it) {
        for (uint64_t u = 0; u < units; ++u) { mb[u].initial = ~0ull; mb[u].final_ = ~0ull; mb[u].partial = 0.0; }
        double glob = 0.0;
        for (uint64_t u = 0; u < units; ++u) {
            uint64_t lo, hi;
            orc_unit_range(nvec, units, u, &lo, &hi);
            if (lo >= hi) continue;
            glob = orc_pr_pull_unit(vec, lo, hi, prop, accum, &mb[u], glob);
        }
        orc_merge_sum(mb, units, accum);
        memset(rb, 0, sizeof(rb));
        rb[0] = glob;
        const double S = orc_reduce_buffer_sum(rb, 1);
        orc_pr_vertex(0, num_vertices, accum, outdeg, prop, S, (double)num_vertices, damping);
    }
    free(mb);
}

/*
 * PageRank with the push engine (EDGE_FORCE_PUSH), single thread:
 * source/phase_edge_push_pr.asm:42-354 (accum[dst] += prop[src] per valid lane,
 * glob += prop[src] per lane), then the vertex phase resets the accumulators
 * (phase_vertex_pr.asm:101-106).
 */
void oracle_pr_push(const uint64_t* vec, uint64_t nvec, const double* outdeg, uint64_t num_vertices, uint32_t iters,
                    double damping, double* prop, double* accum)
{
    for (uint32_t it = 0; it < iters; ++it) {
        double glob = 0.0;
        for (uint64_t i = 0; i < nvec; ++i) {
            const uint64_t* v = vec + 4 * i;
            const double msg = prop[orc_shared(v)];
            for (int k = 0; k < 4; ++k) {
                if (!(v[k] & ORC_VALID)) continue;
                accum[v[k] & ORC_ID48] += msg;
                glob += msg;
            }
        }
        orc_pr_vertex(0, num_vertices, accum, outdeg, prop, glob, (double)num_vertices, damping);
        for (uint64_t v = 0; v < num_vertices; ++v) accum[v] = 0.0;
    }
}

/* PageRank Sum check of source/main.c:132-138. */
double oracle_pr_sum(const double* prop, const double* outdeg, uint64_t num_vertices)
{
    double s = 0.0;
    for (uint64_t v = 0; v < num_vertices; ++v)
        s += prop[v] * (outdeg[v] == 0.0 ? (double)num_vertices : outdeg[v]);
    return s;
}

/* ------------------------------------------------------------------------- */
/* Multi-threaded PageRank pull: the CPU baseline                              */
/* ------------------------------------------------------------------------- */

/*
 * Same units, per-unit arithmetic and merge as oracle_pr_pull, but the units
 * are claimed dynamically by `threads` OpenMP threads, as in the reference.
 * Each thread keeps its own global accumulator, and the per-thread partials
 * are summed in thread order, so S depends on the thread count just as the
 * reference's does.  The vertex phase is split statically over the threads.
 * Returns the number of threads actually used.
 */
int oracle_pr_pull_mt(const uint64_t* vec, uint64_t nvec, const double* outdeg, uint64_t num_vertices, uint32_t iters,
                      double damping, uint64_t units, int threads, double* prop, double* accum)
{
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#else
    threads = 1;
#endif
    orc_merge* mb = (orc_merge*)malloc(sizeof(orc_merge) * units);
    double* part = (double*)calloc((size_t)threads + 8, sizeof(double));
    for (uint32_t it = 0; it < iters; ++it) {
        for (uint64_t u = 0; u < units; ++u) { mb[u].initial = ~0ull; mb[u].final_ = ~0ull; mb[u].partial = 0.0; }
#pragma omp parallel num_threads(threads)
        {
            int tid = 0;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
            double glob = 0.0;
#pragma omp for schedule(dynamic, 1)
            for (int64_t u = 0; u < (int64_t)units; ++u) {
                uint64_t lo, hi;
                orc_unit_range(nvec, units, (uint64_t)u, &lo, &hi);
                if (lo < hi) glob = orc_pr_pull_unit(vec, lo, hi, prop, accum, &mb[u], glob);
            }
            part[tid] = glob;
        }
        orc_merge_sum(mb, units, accum);
        const double S = orc_reduce_buffer_sum(part, (uint64_t)threads);
        const double V = (double)num_vertices;
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int64_t b = 0; b < (int64_t)((num_vertices + 4095) / 4096); ++b) {
            const uint64_t first = (uint64_t)b * 4096;
            const uint64_t cnt = (first + 4096 <= num_vertices) ? 4096 : num_vertices - first;
            orc_pr_vertex(first, cnt, accum, outdeg, prop, S, V, damping);
        }
    }
    free(part);
    free(mb);
    return threads;
}

/* ------------------------------------------------------------------------- */
/* Frontier bitmaps                                                            */
/* ------------------------------------------------------------------------- */

static inline int orc_bit(const uint64_t* bm, uint64_t v) { return (int)((bm[v >> 6] >> (v & 63)) & 1ull); }
static inline void orc_set(uint64_t* bm, uint64_t v) { bm[v >> 6] |= 1ull << (v & 63); }
static inline void orc_clr(uint64_t* bm, uint64_t v) { bm[v >> 6] &= ~(1ull << (v & 63)); }

/* Vote increment; include/phasehelpers.inc:388-399 (count and/or outdegree). */
static inline uint64_t orc_vote(const double* outdeg, uint64_t v, int without_count, int without_outdeg)
{
    uint64_t d = 0;
    if (!without_count) d += 1;
    if (!without_outdeg) d += (uint64_t)llrint(outdeg[v]);
    return d;
}

/* flags for the CC/BFS drivers (Makefile EXPERIMENTS names) */
#define ORC_FORCE_PULL 1
#define ORC_FORCE_PUSH 2
#define ORC_WITHOUT_COUNT 4
#define ORC_WITHOUT_OUTDEG 8

/* Engine choice; source/execution_cc.c:120-142 and source/execution_bfs.c:146-168. */
static int orc_use_pull(int flags, uint64_t vote, uint64_t V, uint64_t E)
{
    if (flags & ORC_FORCE_PULL) return 1;
    if (flags & ORC_FORCE_PUSH) return 0;
    const uint64_t threshold = (flags & ORC_WITHOUT_OUTDEG) ? V / 2 : E / 5;
    return vote > threshold;
}

/* ------------------------------------------------------------------------- */
/* Connected Components                                                        */
/* ------------------------------------------------------------------------- */

/* Scalar-reduce write of one destination; phase_edge_pull_cc.asm:183-233 and :357-392. */
static inline uint64_t orc_cc_write(double* prop, uint64_t* has_next, const double* outdeg, uint64_t v, double run,
                                    int flags)
{
    const double old = prop[v];
    const double nw = run < old ? run : old;
    if (nw == old) return 0;
    prop[v] = nw;
    orc_set(has_next, v);
    return orc_vote(outdeg, v, flags & ORC_WITHOUT_COUNT, flags & ORC_WITHOUT_OUTDEG);
}

/* perform_edge_pull_phase_cc, one thread, units in order; phase_edge_pull_cc.asm:50-392, 398-529. */
static uint64_t orc_cc_pull_phase(const uint64_t* vec, uint64_t nvec, uint64_t units, double* prop, uint64_t* has_next,
                                  const double* outdeg, int flags)
{
    uint64_t vote = 0;
    for (uint64_t u = 0; u < units; ++u) {
        uint64_t lo, hi;
        orc_unit_range(nvec, units, u, &lo, &hi);
        if (lo >= hi) continue;
        uint64_t prev = orc_shared(vec + 4 * lo);
        double acc = INFINITY;
        for (uint64_t i = lo; i < hi; ++i) {
            const uint64_t* v = vec + 4 * i;
            const uint64_t dst = orc_shared(v);
            double g[4];
            for (int k = 0; k < 4; ++k) g[k] = (v[k] & ORC_VALID) ? prop[v[k] & ORC_ID48] : INFINITY;
            if (prev != dst) {
                vote += orc_cc_write(prop, has_next, outdeg, prev, acc, flags);
                acc = INFINITY;
            }
            prev = dst;
            double m = g[0];
            for (int k = 1; k < 4; ++k) m = g[k] < m ? g[k] : m;
            acc = m < acc ? m : acc;
        }
        vote += orc_cc_write(prop, has_next, outdeg, prev, acc, flags);
    }
    return vote;
}

/*
 * perform_edge_push_phase_cc, one thread; phase_edge_push_cc.asm:51-573 (CAS path).
 * A source is processed when its HasInfo bit is set at the moment the scan
 * reaches it (strong frontier, include/phasehelpers.inc:137-213).  A changed
 * destination also sets HasInfo at once (asynchronous frontier, :212-215).
 */
static uint64_t orc_cc_push_phase(const uint64_t* vec, uint64_t nvec, double* prop, uint64_t* has, uint64_t* has_next,
                                  const double* outdeg, int flags)
{
    uint64_t vote = 0;
    for (uint64_t i = 0; i < nvec; ++i) {
        const uint64_t* v = vec + 4 * i;
        const uint64_t src = orc_shared(v);
        if (!orc_bit(has, src)) continue;
        const double msg = prop[src];
        for (int k = 0; k < 4; ++k) {
            if (!(v[k] & ORC_VALID)) continue;
            const uint64_t dst = v[k] & ORC_ID48;
            const double old = prop[dst];
            const double nw = old < msg ? old : msg;
            if (!(nw != old)) continue;
            prop[dst] = nw;
            orc_set(has, dst);
            orc_set(has_next, dst);
            vote += orc_vote(outdeg, dst, flags & ORC_WITHOUT_COUNT, flags & ORC_WITHOUT_OUTDEG);
        }
    }
    return vote;
}

/*
 * Connected Components driver, single thread: execution_impl_cc
 * (source/execution_cc.c:94-268), init values execution_cc.c:66-90.
 * labels[V] (double, out).  iter_out[0..2] = total, pull, push iterations.
 * engine_log (optional, capacity max_log): 1 = pull, 0 = push per iteration.
 */
void oracle_cc(const uint64_t* pull_vec, uint64_t pull_nvec, const uint64_t* push_vec, uint64_t push_nvec,
               const double* outdeg, uint64_t V, uint64_t E, uint64_t units, int flags, double* labels,
               uint64_t* iter_out, uint8_t* engine_log, uint64_t max_log)
{
    const uint64_t words = (V >> 6) + ((V & 63) ? 1 : 0);
    uint64_t* has = (uint64_t*)malloc(sizeof(uint64_t) * (words + 1));
    uint64_t* has_next = (uint64_t*)calloc(words + 1, sizeof(uint64_t));
    for (uint64_t w = 0; w < words; ++w) has[w] = ~0ull;
    for (uint64_t v = 0; v < V; ++v) labels[v] = (double)v;
    uint64_t vote = 0;
    if (!(flags & ORC_WITHOUT_OUTDEG)) vote += E;
    if (!(flags & ORC_WITHOUT_COUNT)) vote += V;
    uint64_t ctr = 0, npull = 0, npush = 0;
    for (;;) {
        ++ctr;
        const int pull = orc_use_pull(flags, vote, V, E);
        if (engine_log && ctr - 1 < max_log) engine_log[ctr - 1] = (uint8_t)pull;
        if (pull) {
            ++npull;
            vote = orc_cc_pull_phase(pull_vec, pull_nvec, units, labels, has_next, outdeg, flags);
        } else {
            ++npush;
            vote = orc_cc_push_phase(push_vec, push_nvec, labels, has, has_next, outdeg, flags);
        }
        if (vote == 0) break;
        uint64_t* t = has; has = has_next; has_next = t;  /* execution_cc.c:245-250 */
        memset(has_next, 0, sizeof(uint64_t) * words);    /* perform_vertex_phase_cc, phase_vertex_cc.asm:37-46 */
    }
    iter_out[0] = ctr; iter_out[1] = npull; iter_out[2] = npush;
    free(has); free(has_next);
}

/* ------------------------------------------------------------------------- */
/* Breadth-First Search                                                        */
/* ------------------------------------------------------------------------- */

/*
 * perform_edge_pull_phase_bfs, one thread; phase_edge_pull_bfs.asm:53-211.
 * A destination is processed while its WantsInfo bit is set (strong check).
 * The first of its vectors that holds a HasInfo source (weak check) gives the
 * parent: the largest such source ID in that vector (:175-190).  Its
 * WantsInfo bit is then cleared, so later vectors are skipped.
 */
static uint64_t orc_bfs_pull_phase(const uint64_t* vec, uint64_t nvec, double* parent, const uint64_t* has,
                                   uint64_t* has_next, uint64_t* wants, const double* outdeg, int flags)
{
    uint64_t vote = 0;
    for (uint64_t i = 0; i < nvec; ++i) {
        const uint64_t* v = vec + 4 * i;
        const uint64_t dst = orc_shared(v);
        if (!orc_bit(wants, dst)) continue;
        int any = 0;
        uint64_t best = 0;
        for (int k = 0; k < 4; ++k) {
            if (!(v[k] & ORC_VALID)) continue;
            const uint64_t s = v[k] & ORC_ID48;
            if (!orc_bit(has, s)) continue;
            if (!any || s > best) best = s;
            any = 1;
        }
        if (!any) continue;
        parent[dst] = (double)(int64_t)best;
        orc_set(has_next, dst);
        orc_clr(wants, dst);
        vote += orc_vote(outdeg, dst, flags & ORC_WITHOUT_COUNT, flags & ORC_WITHOUT_OUTDEG);
    }
    return vote;
}

/*
 * perform_edge_push_phase_bfs, one thread; phase_edge_push_bfs.asm:53-202.
 * For a source in HasInfo, the WantsInfo bits of all four destinations are
 * read first (weak check, :108-114).  Each marked destination is then visited
 * in lane order: its WantsInfo bit is cleared, HasInfo* is set, and its
 * parent becomes the source.
 */
static uint64_t orc_bfs_push_phase(const uint64_t* vec, uint64_t nvec, double* parent, const uint64_t* has,
                                   uint64_t* has_next, uint64_t* wants, const double* outdeg, int flags)
{
    uint64_t vote = 0;
    for (uint64_t i = 0; i < nvec; ++i) {
        const uint64_t* v = vec + 4 * i;
        const uint64_t src = orc_shared(v);
        if (!orc_bit(has, src)) continue;
        int mark[4];
        for (int k = 0; k < 4; ++k) mark[k] = (v[k] & ORC_VALID) && orc_bit(wants, v[k] & ORC_ID48);
        for (int k = 0; k < 4; ++k) {
            if (!mark[k]) continue;
            const uint64_t dst = v[k] & ORC_ID48;
            orc_clr(wants, dst);
            orc_set(has_next, dst);
            parent[dst] = (double)(int64_t)src;
            vote += orc_vote(outdeg, dst, flags & ORC_WITHOUT_COUNT, flags & ORC_WITHOUT_OUTDEG);
        }
    }
    return vote;
}

/*
 * BFS driver from root 0, single thread: execution_impl_bfs
 * (source/execution_bfs.c:120-276), init values :56-116.  parent[V] (double,
 * -1 = unvisited or the root).  iter_out as in oracle_cc.
 */
void oracle_bfs(const uint64_t* pull_vec, uint64_t pull_nvec, const uint64_t* push_vec, uint64_t push_nvec,
                const double* outdeg, uint64_t V, uint64_t E, int flags, double* parent, uint64_t* iter_out,
                uint8_t* engine_log, uint64_t max_log)
{
    const uint64_t words = (V >> 6) + ((V & 63) ? 1 : 0);
    uint64_t* has = (uint64_t*)calloc(words + 1, sizeof(uint64_t));
    uint64_t* has_next = (uint64_t*)calloc(words + 1, sizeof(uint64_t));
    uint64_t* wants = (uint64_t*)calloc(words + 1, sizeof(uint64_t));
    for (uint64_t w = 0; w < words; ++w) wants[w] = ~0ull;
    orc_set(has, 0);
    orc_clr(wants, 0);
    for (uint64_t v = 0; v < V; ++v) parent[v] = -1.0;
    uint64_t vote = 0;
    if (!(flags & ORC_WITHOUT_OUTDEG)) vote += (uint64_t)outdeg[0];
    if (!(flags & ORC_WITHOUT_COUNT)) vote += 1;
    uint64_t ctr = 0, npull = 0, npush = 0;
    for (;;) {
        ++ctr;
        const int pull = orc_use_pull(flags, vote, V, E);
        if (engine_log && ctr - 1 < max_log) engine_log[ctr - 1] = (uint8_t)pull;
        if (pull) {
            ++npull;
            vote = orc_bfs_pull_phase(pull_vec, pull_nvec, parent, has, has_next, wants, outdeg, flags);
        } else {
            ++npush;
            vote = orc_bfs_push_phase(push_vec, push_nvec, parent, has, has_next, wants, outdeg, flags);
        }
        if (vote == 0) break;
        uint64_t* t = has; has = has_next; has_next = t;
        memset(has_next, 0, sizeof(uint64_t) * words);
    }
    iter_out[0] = ctr; iter_out[1] = npull; iter_out[2] = npush;
    free(has); free(has_next); free(wants);
}

/* ------------------------------------------------------------------------- */
/* Checkers                                                                    */
/* ------------------------------------------------------------------------- */

/*
 * BFS levels from the root by a plain queue BFS over the -push pairs
 * (src-sorted; CSR offsets built here).  level[v] = -1 if unreachable.
 */
void oracle_bfs_levels(const uint64_t* push_pairs, uint64_t E, uint64_t V, uint64_t root, int64_t* level)
{
    uint64_t* off = (uint64_t*)calloc(V + 1, sizeof(uint64_t));
    for (uint64_t e = 0; e < E; ++e) off[push_pairs[2 * e] + 1]++;
    for (uint64_t v = 0; v < V; ++v) off[v + 1] += off[v];
    uint64_t* adj = (uint64_t*)malloc(sizeof(uint64_t) * (E ? E : 1));
    uint64_t* fill = (uint64_t*)malloc(sizeof(uint64_t) * (V ? V : 1));
    memcpy(fill, off, sizeof(uint64_t) * V);
    for (uint64_t e = 0; e < E; ++e) adj[fill[push_pairs[2 * e]]++] = push_pairs[2 * e + 1];
    for (uint64_t v = 0; v < V; ++v) level[v] = -1;
    uint64_t* q = (uint64_t*)malloc(sizeof(uint64_t) * (V ? V : 1));
    uint64_t qh = 0, qt = 0;
    level[root] = 0;
    q[qt++] = root;
    while (qh < qt) {
        const uint64_t u = q[qh++];
        for (uint64_t k = off[u]; k < off[u + 1]; ++k) {
            const uint64_t w = adj[k];
            if (level[w] < 0) { level[w] = level[u] + 1; q[qt++] = w; }
        }
    }
    free(q); free(fill); free(adj); free(off);
}

/*
 * Checks that `parent` (root stays -1, as in the reference) is a legal BFS
 * tree for `level`: every reached non-root v has a parent p with an edge
 * p->v and level[p] == level[v]-1; unreached vertices have parent -1.
 * Returns 0 if legal, else 1 + the first offending vertex.
 */
uint64_t oracle_bfs_check_tree(const uint64_t* push_pairs, uint64_t E, uint64_t V, uint64_t root,
                               const int64_t* level, const int64_t* parent)
{
    /* edge membership via the src-sorted pairs: binary search in each source's range */
    uint64_t* off = (uint64_t*)calloc(V + 1, sizeof(uint64_t));
    for (uint64_t e = 0; e < E; ++e) off[push_pairs[2 * e] + 1]++;
    for (uint64_t v = 0; v < V; ++v) off[v + 1] += off[v];
    uint64_t bad = 0;
    for (uint64_t v = 0; v < V && !bad; ++v) {
        if (v == root) { if (parent[v] != -1) bad = v + 1; continue; }
        if (level[v] < 0) { if (parent[v] != -1) bad = v + 1; continue; }
        const int64_t p = parent[v];
        if (p < 0 || (uint64_t)p >= V || level[p] != level[v] - 1) { bad = v + 1; continue; }
        uint64_t lo = off[p], hi = off[p + 1];
        int found = 0;
        while (lo < hi) {
            const uint64_t mid = (lo + hi) / 2;
            const uint64_t d = push_pairs[2 * mid + 1];
            if (d == v) { found = 1; break; }
            if (d < v) lo = mid + 1; else hi = mid;
        }
        if (!found) bad = v + 1;
    }
    free(off);
    return bad;
}

/* ------------------------------------------------------------------------- */
/* Multi-threaded CC / BFS: the CPU baseline on machines where the reference  */
/* (x86-64 AVX2 only) cannot run.  Same SPMD semantics as the reference:      */
/* dynamic work units, CAS-min label updates, asynchronous HasInfo updates in */
/* CC push, unsynchronised parent stores in BFS, strong-frontier skip-ahead   */
/* through the vertex index (include/phasehelpers.inc:137-213).               */
/* ------------------------------------------------------------------------- */

static inline int orc_abit(const uint64_t* bm, uint64_t v)
{
    return (int)((__atomic_load_n(&bm[v >> 6], __ATOMIC_RELAXED) >> (v & 63)) & 1ull);
}
static inline void orc_aset(uint64_t* bm, uint64_t v) { __atomic_fetch_or(&bm[v >> 6], 1ull << (v & 63), __ATOMIC_RELAXED); }
static inline void orc_aclr(uint64_t* bm, uint64_t v) { __atomic_fetch_and(&bm[v >> 6], ~(1ull << (v & 63)), __ATOMIC_RELAXED); }

static inline double orc_aload(const double* p)
{
    uint64_t b = __atomic_load_n((const uint64_t*)p, __ATOMIC_RELAXED);
    double d;
    memcpy(&d, &b, 8);
    return d;
}

/* CAS-min of a non-negative double label (lock cmpxchg loop, phase_edge_pull_cc.asm:188-202);
 * returns 1 if this call lowered it */
static inline int orc_cas_min(double* p, double x)
{
    uint64_t* q = (uint64_t*)p;
    uint64_t old = __atomic_load_n(q, __ATOMIC_RELAXED);
    for (;;) {
        double od;
        memcpy(&od, &old, 8);
        if (!(x < od)) return 0;
        uint64_t nb;
        memcpy(&nb, &x, 8);
        if (__atomic_compare_exchange_n(q, &old, nb, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return 1;
    }
}

/* next vertex >= v that is set in `bm` and owns vectors (vindex entry without bit 62/63);
 * returns its first vector, or UINT64_MAX if none (strong frontier search) */
static uint64_t orc_next_active(const uint64_t* bm, const uint64_t* vindex, uint64_t v, uint64_t words)
{
    for (;;) {
        uint64_t w = v >> 6;
        if (w >= words) return UINT64_MAX;
        uint64_t x = __atomic_load_n(&bm[w], __ATOMIC_RELAXED) & (~0ull << (v & 63));
        while (!x) {
            if (++w >= words) return UINT64_MAX;
            x = __atomic_load_n(&bm[w], __ATOMIC_RELAXED);
        }
        const uint64_t cand = (w << 6) + (uint64_t)__builtin_ctzll(x);
        const uint64_t idx = vindex[cand];
        if (idx & 0x8000000000000000ull) return UINT64_MAX;   /* beyond the last vertex */
        if (!(idx & 0x4000000000000000ull)) return idx;         /* has vectors */
        v = cand + 1;
    }
}

typedef struct orc_mt_graph {
    const uint64_t* pull_vec; uint64_t pull_nvec; const uint64_t* pull_index;
    const uint64_t* push_vec; uint64_t push_nvec; const uint64_t* push_index;
    const double* outdeg; uint64_t V, E;
} orc_mt_graph;

/*
 * Multi-threaded CC or BFS (app 1 / 2) from root 0: the reference's execution_impl_{cc,bfs}
 * run by `threads` OpenMP threads.  props[V] out (labels / parents as doubles), iter_out[3]
 * out.  Returns the thread count used.
 */
int oracle_frontier_mt(const uint64_t* pull_vec, uint64_t pull_nvec, const uint64_t* pull_index,
                       const uint64_t* push_vec, uint64_t push_nvec, const uint64_t* push_index,
                       const double* outdeg, uint64_t V, uint64_t E, int app, int flags, int threads,
                       double* props, uint64_t* iter_out)
{
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#else
    threads = 1;
#endif
    const uint64_t words = (V >> 6) + ((V & 63) ? 1 : 0);
    uint64_t* has = (uint64_t*)calloc(words + 1, sizeof(uint64_t));
    uint64_t* has_next = (uint64_t*)calloc(words + 1, sizeof(uint64_t));
    uint64_t* wants = (uint64_t*)calloc(words + 1, sizeof(uint64_t));
    const int wc = (flags & ORC_WITHOUT_COUNT) != 0, wo = (flags & ORC_WITHOUT_OUTDEG) != 0;
    uint64_t vote = 0;
    if (app == 1) {
        for (uint64_t w = 0; w < words; ++w) has[w] = wants[w] = ~0ull;
        for (uint64_t v = 0; v < V; ++v) props[v] = (double)v;
        if (!wo) vote += E;
        if (!wc) vote += V;
    } else {
        for (uint64_t w = 0; w < words; ++w) wants[w] = ~0ull;
        orc_set(has, 0);
        orc_clr(wants, 0);
        for (uint64_t v = 0; v < V; ++v) props[v] = -1.0;
        if (!wo) vote += (uint64_t)outdeg[0];
        if (!wc) vote += 1;
    }
    const uint64_t units = (uint64_t)threads << 5;
    uint64_t ctr = 0, npull = 0, npush = 0;
    for (;;) {
        ++ctr;
        const int pull = orc_use_pull(flags, vote, V, E);
        if (pull) ++npull; else ++npush;
        uint64_t nv = 0;
        const uint64_t* vec = pull ? pull_vec : push_vec;
        const uint64_t nvec = pull ? pull_nvec : push_nvec;
        const uint64_t* vindex = pull ? pull_index : push_index;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1) reduction(+ : nv)
        for (int64_t uu = 0; uu < (int64_t)units; ++uu) {
            uint64_t lo, hi;
            orc_unit_range(nvec, units, (uint64_t)uu, &lo, &hi);
            if (lo >= hi) continue;
            if (app == 1 && pull) {
                /* CC pull: phase_edge_pull_cc.asm, write at each destination change and unit end */
                uint64_t prev = orc_shared(vec + 4 * lo);
                double acc = INFINITY;
                for (uint64_t i = lo; i < hi; ++i) {
                    const uint64_t* v = vec + 4 * i;
                    const uint64_t dst = orc_shared(v);
                    double m = INFINITY;
                    for (int k = 0; k < 4; ++k)
                        if (v[k] & ORC_VALID) { const double x = orc_aload(&props[v[k] & ORC_ID48]); m = x < m ? x : m; }
                    if (prev != dst) {
                        if (orc_cas_min(&props[prev], acc)) {
                            orc_aset(has_next, prev);
                            nv += orc_vote(outdeg, prev, wc, wo);
                        }
                        acc = INFINITY;
                    }
                    prev = dst;
                    acc = m < acc ? m : acc;
                }
                if (orc_cas_min(&props[prev], acc)) { orc_aset(has_next, prev); nv += orc_vote(outdeg, prev, wc, wo); }
            } else {
                /* strong frontier on the shared vertex: HasInfo (push) or WantsInfo (BFS pull) */
                const uint64_t* strong = pull ? wants : has;
                uint64_t i = lo;
                while (i < hi) {
                    const uint64_t* v = vec + 4 * i;
                    const uint64_t sh = orc_shared(v);
                    if (!orc_abit(strong, sh)) {
                        const uint64_t nx = orc_next_active(strong, vindex, sh + 1, words);
                        if (nx == UINT64_MAX) break;
                        i = nx > i ? nx : i + 1;
                        continue;
                    }
                    if (app == 2 && pull) {
                        /* BFS pull: phase_edge_pull_bfs.asm:104-207 */
                        int any = 0;
                        uint64_t best = 0;
                        for (int k = 0; k < 4; ++k) {
                            if (!(v[k] & ORC_VALID)) continue;
                            const uint64_t s = v[k] & ORC_ID48;
                            if (!orc_abit(has, s)) continue;
                            if (!any || s > best) best = s;
                            any = 1;
                        }
                        if (any) {
                            __atomic_store_n((uint64_t*)&props[sh], 0, __ATOMIC_RELAXED);
                            const double pd = (double)(int64_t)best;
                            uint64_t pb;
                            memcpy(&pb, &pd, 8);
                            __atomic_store_n((uint64_t*)&props[sh], pb, __ATOMIC_RELAXED);
                            orc_aset(has_next, sh);
                            orc_aclr(wants, sh);
                            nv += orc_vote(outdeg, sh, wc, wo);
                        }
                    } else if (app == 2) {
                        /* BFS push: phase_edge_push_bfs.asm:104-198 */
                        int mark[4];
                        for (int k = 0; k < 4; ++k) mark[k] = (v[k] & ORC_VALID) && orc_abit(wants, v[k] & ORC_ID48);
                        const double pd = (double)(int64_t)sh;
                        uint64_t pb;
                        memcpy(&pb, &pd, 8);
                        for (int k = 0; k < 4; ++k) {
                            if (!mark[k]) continue;
                            const uint64_t d = v[k] & ORC_ID48;
                            orc_aclr(wants, d);
                            orc_aset(has_next, d);
                            __atomic_store_n((uint64_t*)&props[d], pb, __ATOMIC_RELAXED);
                            nv += orc_vote(outdeg, d, wc, wo);
                        }
                    } else {
                        /* CC push: phase_edge_push_cc.asm:130-225, asynchronous HasInfo */
                        const double msg = orc_aload(&props[sh]);
                        for (int k = 0; k < 4; ++k) {
                            if (!(v[k] & ORC_VALID)) continue;
                            const uint64_t d = v[k] & ORC_ID48;
                            if (orc_cas_min(&props[d], msg)) {
                                orc_aset(has, d);
                                orc_aset(has_next, d);
                                nv += orc_vote(outdeg, d, wc, wo);
                            }
                        }
                    }
                    ++i;
                }
            }
        }
        vote = nv;
        if (vote == 0) break;
        uint64_t* t = has; has = has_next; has_next = t;
        memset(has_next, 0, sizeof(uint64_t) * words);
    }
    iter_out[0] = ctr; iter_out[1] = npull; iter_out[2] = npush;
    free(has); free(has_next); free(wants);
    return threads;
}

/* ------------------------------------------------------------------------- */
/* Batched personalized PageRank and multi-root BFS levels (checkers)          */
/* ------------------------------------------------------------------------- */

/*
 * K personalized PageRank instances on one graph, the serial definition of
 * oracle/ppr.py with the instances side by side: the reference's PageRank
 * iteration (edge pull source/phase_edge_pull_pr.asm:45-171, vertex phase
 * source/phase_vertex_pr.asm:75-134) with the teleport term and the dangling
 * mass sent to the seed:
 *   prop[u]  = rank[u] / deg'(u)   (deg' = outdegree, or V when 0)
 *   accum[v] = sum over in-edges (u, v) of prop[u], in the -pull file's order
 *   S        = sum over v of accum[v]
 *   rank'[v] = d * accum[v] + [v == seed] * (d * (1 - S) + (1 - d))
 * from rank = one-hot(seed).  pull_pairs is the -pull list (sorted by
 * destination).  ranks is [V][K]; seeds[k] >= V leaves column k at zero.
 * OpenMP over destinations; S is summed per thread, then over threads.
 */
void oracle_ppr_multi(const uint64_t* pull_pairs, uint64_t E, uint64_t V, const uint32_t* seeds, uint32_t K,
                      uint32_t iters, double d, int threads, double* ranks)
{
    uint64_t* off = (uint64_t*)calloc(V + 1, sizeof(uint64_t));
    double* degp = (double*)malloc(sizeof(double) * (V ? V : 1));
    double* prop = (double*)malloc(sizeof(double) * (V ? V : 1) * K);
    double* S = (double*)calloc(K, sizeof(double));
    for (uint64_t v = 0; v < V; ++v) degp[v] = 0.0;
    for (uint64_t e = 0; e < E; ++e) {
        degp[pull_pairs[2 * e]] += 1.0;
        off[pull_pairs[2 * e + 1] + 1]++;
    }
    for (uint64_t v = 0; v < V; ++v) {
        off[v + 1] += off[v];
        if (degp[v] == 0.0) degp[v] = (double)V;
    }
    memset(ranks, 0, sizeof(double) * V * K);
    for (uint32_t k = 0; k < K; ++k)
        if (seeds[k] < V) ranks[(uint64_t)seeds[k] * K + k] = 1.0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    for (uint32_t it = 0; it < iters; ++it) {
        for (uint32_t k = 0; k < K; ++k) S[k] = 0.0;
#pragma omp parallel
        {
            double* Sl = (double*)calloc(K, sizeof(double));
#pragma omp for schedule(static)
            for (uint64_t v = 0; v < V; ++v)
                for (uint32_t k = 0; k < K; ++k) prop[v * K + k] = ranks[v * K + k] / degp[v];
#pragma omp for schedule(dynamic, 4096)
            for (uint64_t v = 0; v < V; ++v) {
                double acc[64];
                for (uint32_t k = 0; k < K; ++k) acc[k] = 0.0;
                for (uint64_t e = off[v]; e < off[v + 1]; ++e) {
                    const double* p = prop + pull_pairs[2 * e] * K;
                    for (uint32_t k = 0; k < K; ++k) acc[k] += p[k];
                }
                for (uint32_t k = 0; k < K; ++k) {
                    Sl[k] += acc[k];
                    ranks[v * K + k] = d * acc[k];
                }
            }
#pragma omp critical
            for (uint32_t k = 0; k < K; ++k) S[k] += Sl[k];
            free(Sl);
        }
        for (uint32_t k = 0; k < K; ++k)
            if (seeds[k] < V) ranks[(uint64_t)seeds[k] * K + k] += d * (1.0 - S[k]) + (1.0 - d);
    }
    free(S); free(prop); free(degp); free(off);
}

/*
 * BFS levels from n roots over the -push pairs (the CSR is built once, the
 * roots run on parallel threads): level[r * V + v], -1 if unreachable.
 */
void oracle_bfs_levels_multi(const uint64_t* push_pairs, uint64_t E, uint64_t V, const uint64_t* roots, uint32_t n,
                             int threads, int64_t* level)
{
    uint64_t* off = (uint64_t*)calloc(V + 1, sizeof(uint64_t));
    for (uint64_t e = 0; e < E; ++e) off[push_pairs[2 * e] + 1]++;
    for (uint64_t v = 0; v < V; ++v) off[v + 1] += off[v];
    uint64_t* adj = (uint64_t*)malloc(sizeof(uint64_t) * (E ? E : 1));
    uint64_t* fill = (uint64_t*)malloc(sizeof(uint64_t) * (V ? V : 1));
    memcpy(fill, off, sizeof(uint64_t) * V);
    for (uint64_t e = 0; e < E; ++e) adj[fill[push_pairs[2 * e]]++] = push_pairs[2 * e + 1];
    free(fill);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (uint32_t r = 0; r < n; ++r) {
        int64_t* lv = level + (uint64_t)r * V;
        uint64_t* q = (uint64_t*)malloc(sizeof(uint64_t) * (V ? V : 1));
        uint64_t qh = 0, qt = 0;
        for (uint64_t v = 0; v < V; ++v) lv[v] = -1;
        lv[roots[r]] = 0;
        q[qt++] = roots[r];
        while (qh < qt) {
            const uint64_t u = q[qh++];
            for (uint64_t k = off[u]; k < off[u + 1]; ++k) {
                const uint64_t w = adj[k];
                if (lv[w] < 0) { lv[w] = lv[u] + 1; q[qt++] = w; }
            }
        }
        free(q);
    }
    free(adj); free(off);
}

/*
 * Connected Components labels straight from the -pull pairs (sorted by
 * destination), for graphs whose vector lists would not fit a bounded host
 * sample: label[v] = the smallest vertex ID that reaches v (v included),
 * which is the fixpoint the reference's CC reaches on a directed or
 * symmetric graph (pull: label[d] = min over its sources and itself,
 * source/phase_edge_pull_cc.asm:183-233; push: CAS-min into the
 * destinations, source/phase_edge_push_cc.asm:130-225; the vertex IDs are the
 * initial labels, source/execution_cc.c:66-90).  Sweeps of in-place
 * min-propagation over the destination ranges (OpenMP, relaxed atomic reads
 * and writes: labels only decrease) until a sweep changes nothing.  Returns
 * the number of sweeps.
 */
uint32_t oracle_cc_min_labels(const uint64_t* pull_pairs, uint64_t E, uint64_t V, int threads, uint32_t* label)
{
    for (uint64_t v = 0; v < V; ++v) label[v] = (uint32_t)v;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    /* chunk boundaries on destination changes, so that one thread owns each destination */
    const uint64_t nch = E / 65536 + 1;
    uint64_t* cut = (uint64_t*)malloc(sizeof(uint64_t) * (nch + 1));
    for (uint64_t c = 0; c <= nch; ++c) {
        uint64_t e = E * c / nch;
        while (e > 0 && e < E && pull_pairs[2 * e + 1] == pull_pairs[2 * (e - 1) + 1]) ++e;
        cut[c] = e;
    }
    uint32_t sweeps = 0;
    for (;;) {
        uint64_t changed = 0;
        ++sweeps;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : changed)
        for (uint64_t c = 0; c < nch; ++c) {
            uint64_t e = cut[c];
            const uint64_t end = cut[c + 1];
            while (e < end) {
                const uint64_t d = pull_pairs[2 * e + 1];
                uint32_t m = __atomic_load_n(&label[d], __ATOMIC_RELAXED);
                const uint32_t m0 = m;
                for (; e < end && pull_pairs[2 * e + 1] == d; ++e) {
                    const uint32_t x = __atomic_load_n(&label[pull_pairs[2 * e]], __ATOMIC_RELAXED);
                    if (x < m) m = x;
                }
                if (m < m0) {
                    __atomic_store_n(&label[d], m, __ATOMIC_RELAXED);
                    ++changed;
                }
            }
        }
        if (!changed) break;
    }
    free(cut);
    return sweeps;
}

/*
 * One PageRank iteration from the initial props, checked on a sample of
 * destinations only, straight from the -pull pairs (sorted by destination):
 * for graphs whose vector lists would not fit a bounded host sample.
 *   prop0[u] = (1/V) / deg'(u)                 source/execution_pr.c:85-88
 *   accum[v] = sum over v's in-edges of prop0  source/phase_edge_pull_pr.asm:45-171
 *   S        = sum over u of prop0[u] * outdeg(u)   (= sum of all accumulators)
 *   prop1[v] = ((accum[v] + (1-S)/V) * d + (1-d)/V) / deg'(v)   source/phase_vertex_pr.asm:75-134
 * deg' = outdegree from the -pull pairs, or V when 0.  samples[] are
 * destinations; out[i] is prop1[samples[i]] (a binary search finds each
 * destination's edges).
 */
void oracle_pr_sample_iteration(const uint64_t* pull_pairs, uint64_t E, uint64_t V, double d, int threads,
                                const uint64_t* samples, uint64_t n, double* out)
{
    uint32_t* deg = (uint32_t*)calloc(V ? V : 1, sizeof(uint32_t));
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for schedule(static)
    for (uint64_t e = 0; e < E; ++e) __atomic_fetch_add(&deg[pull_pairs[2 * e]], 1u, __ATOMIC_RELAXED);
    const double dV = (double)V;
    double S = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : S)
    for (uint64_t u = 0; u < V; ++u)
        if (deg[u]) S += ((1.0 / dV) / (double)deg[u]) * (double)deg[u];
    const double G = (1.0 - S) / dV;
#pragma omp parallel for schedule(dynamic, 64)
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t v = samples[i];
        uint64_t lo = 0, hi = E;  /* first edge with destination >= v */
        while (lo < hi) {
            const uint64_t mid = lo + (hi - lo) / 2;
            if (pull_pairs[2 * mid + 1] < v) lo = mid + 1; else hi = mid;
        }
        double acc = 0.0;
        for (uint64_t e = lo; e < E && pull_pairs[2 * e + 1] == v; ++e) {
            const uint64_t u = pull_pairs[2 * e];
            acc += (1.0 / dV) / (double)deg[u];  /* a source of an edge has deg >= 1 */
        }
        const double dp = deg[v] ? (double)deg[v] : dV;
        out[i] = ((acc + G) * d + (1.0 - d) / dV) / dp;
    }
    free(deg);
}
