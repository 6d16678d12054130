/*
 * grazelle_main.c -- the C host driver of the GB300 engine.
 *
 * Plays the part of the reference's source/main.c, source/cmdline.c and
 * source/execution_{pr,cc,bfs}.c.  It uses the same command line (-i -n -N -o
 * -s -u -V -h), the same exit codes, the same stats block and output file
 * format, and compile-time application selection: build with -DPAGERANK
 * (default), -DCONNECTED_COMPONENTS or -DBREADTH_FIRST_SEARCH, plus the
 * reference's EXPERIMENT_* engine flags.  Every edge and vertex phase goes
 * through the drop-in phases.h entry points (include/grazelle_phases.h), in
 * the call order of the reference's execution_impl_* loops.
 *
 * Differences from the reference host code:
 *   - one host thread drives the GPU, so -n and -u are accepted and reported but do not
 *     spawn threads;
 *   - graph_data_read_from_file becomes grz_graph_load_files (the pairs stream to the GPU, which
 *     builds the layout); CC and BFS without a -push file derive that list on the device;
 *   - the CC/BFS HasInfo / HasInfo* pointer swap (execution_cc.c:245-250) happens inside
 *     perform_vertex_phase_*, because the bitmaps live on the device;
 *   - the run is timed with CLOCK_MONOTONIC (the reference uses CLOCK_REALTIME_COARSE,
 *     source/benchmark.c:40,55).
 */
#include <ctype.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <unistd.h>

#include "grazelle_phases.h"

#define VERSION "1.0.1-ppopp18-gb300"

#ifdef EXPERIMENT_ITERATION_PROFILE
/* the frontier column of the per-iteration profile (source/main.c:43-55) */
#if defined(EXPERIMENT_THRESHOLD_WITHOUT_OUTDEGREES) && defined(EXPERIMENT_THRESHOLD_WITHOUT_COUNT)
#error "Cannot profile iterations with both outdegrees and count disabled for engine selection."
#elif defined(EXPERIMENT_THRESHOLD_WITHOUT_OUTDEGREES)
#define PROFILE_FRONTIER_COLUMN "HasInfo Vertices / Total Vertices"
#elif defined(EXPERIMENT_THRESHOLD_WITHOUT_COUNT)
#define PROFILE_FRONTIER_COLUMN "HasInfo Edges / Total Edges"
#else
#define PROFILE_FRONTIER_COLUMN "HasInfo (Vertices + Edges) / Total Edges"
#endif
#endif

#if defined(BREADTH_FIRST_SEARCH)
#define APP GRZ_APP_BREADTH_FIRST_SEARCH
#define APP_NAME "Breadth-First Search"
#elif defined(CONNECTED_COMPONENTS)
#define APP GRZ_APP_CONNECTED_COMPONENTS
#define APP_NAME "Connected Components"
#else
#define APP GRZ_APP_PAGERANK
#define APP_NAME "PageRank"
#endif

/* -------- command line (source/cmdline.c) -------- */

typedef struct opts_t {
    char input[1024];
    const char* output;
    uint32_t iterations;
    uint32_t threads;
    uint64_t granularity;
    int device;
} opts_t;

static void die_unknown(const char* a0, const char* o)
{
    printf("%s: Unrecognized option `%s'.\nTry `%s -h' for more information.\n", a0, o, a0);
    exit(1);
}

static void die_invalid(const char* a0, const char* o, const char* v)
{
    printf("%s: Invalid value `%s' for option `%s'.\nTry `%s -h' for more information.\n", a0, v, o, a0);
    exit(2);
}

static void die_missing_value(const char* a0, const char* o)
{
    printf("%s: Missing argument for option `%s'.\nTry `%s -h' for more information.\n", a0, o, a0);
    exit(3);
}

static void die_extraneous(const char* a0, const char* o)
{
    printf("%s: Option `%s' does not accept an argument.\nTry `%s -h' for more information.\n", a0, o, a0);
    exit(4);
}

static void usage(const char* a0)
{
    printf("Usage: %s [options] -i input-graph\n       %s -h\n       %s -V\n\n", a0, a0, a0);
    printf("Required:\n  -i input-graph\n        Path of the input graph, without the -pull / -push suffix.\n\n");
    printf("Options:\n  -h\n        Prints this information and exits.\n");
    printf("  -n num-threads\n        Accepted for compatibility; one host thread drives the GPU.\n");
    printf("  -N num-iterations\n        Number of PageRank iterations (ignored by CC and BFS). Defaults to 1.\n");
    printf("  -o output-file\n        Path of the file to write as output.\n");
    printf("  -s vectors-per-unit\n        Accepted for compatibility; the GPU schedules per vector.\n");
    printf("  -u node1[,node2...]\n        Accepted for compatibility; only node 0 is used.\n");
    printf("  -d device\n        CUDA device ordinal. Defaults to 0.\n");
    printf("  -V\n        Prints version information and exits.\n");
    exit(0);
}

static int takes_value(char c) { return c == 'i' || c == 'n' || c == 'N' || c == 'o' || c == 's' || c == 'u' || c == 'd'; }
static int known(char c) { return takes_value(c) || c == 'h' || c == '?' || c == 'V'; }

static void parse(int argc, char** argv, opts_t* o)
{
    memset(o, 0, sizeof(*o));
    o->iterations = 1;
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        if ((a[0] != '-' && a[0] != '/') || a[1] == '\0' || a[2] != '\0') die_unknown(argv[0], a);
        const char c = a[1];
        if (!known(c)) die_unknown(argv[0], a);
        const char* v = (i + 1 < argc && argv[i + 1][0] != '-') ? argv[i + 1] : NULL;
        if (takes_value(c) && !v) die_missing_value(argv[0], a);
        if (!takes_value(c) && v) die_extraneous(argv[0], a);
        if (v) ++i;
        char* end = NULL;
        switch (c) {
            case 'h': case '?': usage(argv[0]); break;
            case 'V': printf("%s %s (%s)\n", argv[0], VERSION, APP_NAME); exit(0);
            case 'i': snprintf(o->input, sizeof(o->input), "%s", v); break;
            case 'o': o->output = v; break;
            case 'n': o->threads = (uint32_t)strtoul(v, &end, 10); if (*end) die_invalid(argv[0], a, v); break;
            case 'N': o->iterations = (uint32_t)strtoul(v, &end, 10); if (*end || o->iterations < 1) die_invalid(argv[0], a, v); break;
            case 's': o->granularity = strtoull(v, &end, 10); if (*end || o->granularity < 1) die_invalid(argv[0], a, v); break;
            case 'd': o->device = (int)strtol(v, &end, 10); if (*end || o->device < 0) die_invalid(argv[0], a, v); break;
            case 'u':
                for (const char* p = v; *p; ++p)
                    if (!isdigit((unsigned char)*p) && *p != ',') die_invalid(argv[0], a, v);
                if (strtol(v, NULL, 10) != 0 || strchr(v, ',')) die_invalid(argv[0], a, v);
                break;
        }
    }
    if (!o->input[0]) {
        printf("%s: Missing required option `-i'.\nTry `%s -h' for more information.\n", argv[0], argv[0]);
        exit(5);
    }
}

/* -------- the host check of source/graphdata.c:957-967 before touching the GPU -------- */

/* 1 when the file exists; exits like the reference when a required file is missing or malformed */
static int check_file_or_die(const char* base, const char* suffix, int required)
{
    char p[1100];
    snprintf(p, sizeof(p), "%s%s", base, suffix);
    FILE* f = fopen(p, "rb");
    uint64_t hdr[2];
    if (!f) {
        if (!required) return 0;
        fprintf(stderr, "Error: unable to read file \"%s\"\n", p);
        exit(255);
    }
    const size_t got = fread(hdr, sizeof(uint64_t), 2, f);
    fseek(f, 0, SEEK_END);
    const long long sz = ftell(f);
    fclose(f);
    if (got != 2 || sz != (long long)(16 + 16 * hdr[1])) {
        fprintf(stderr, "Error: unable to read file \"%s\"\n", p);
        exit(255);
    }
    return 1;
}

static double now_ms(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec * 1e3 + (double)t.tv_nsec / 1e6;
}

#ifdef EXPERIMENT_ITERATION_PROFILE
static uint64_t now_ns(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (uint64_t)t.tv_sec * 1000000000ull + (uint64_t)t.tv_nsec;
}
#endif

static void gpu_or_die(int rc, grz_graph* g, const char* what)
{
    if (rc == GRZ_OK) return;
    fprintf(stderr, "Error: %s: %s (%s)\n", what, g ? grz_graph_last_error(g) : "", grz_error_string(rc));
    exit(255);
}

/* -------- execution_impl_* (source/execution_{pr,cc,bfs}.c) -------- */

static uint64_t total_iterations, iterations_pull, iterations_push;

#ifdef EXPERIMENT_ITERATION_STATS
/* vectors and edges the edge phase processed in each iteration (execution_cc.c:209-231) */
static uint64_t* stat_vectors;
static uint64_t* stat_edges;
static uint64_t stat_cap;

static void stats_record(grz_graph* g, uint64_t iteration)
{
    uint64_t v = 0, e = 0;
    gpu_or_die(grz_stats_take(g, &v, &e), g, "iteration stats");
    if (iteration >= stat_cap) {
        stat_cap = stat_cap ? 2 * stat_cap : 64;
        stat_vectors = (uint64_t*)realloc(stat_vectors, sizeof(uint64_t) * stat_cap);
        stat_edges = (uint64_t*)realloc(stat_edges, sizeof(uint64_t) * stat_cap);
        if (!stat_vectors || !stat_edges) { fprintf(stderr, "Error: out of memory\n"); exit(255); }
    }
    stat_vectors[iteration] = v;
    stat_edges[iteration] = e;
}
#endif

static void execution_impl(grz_graph* g, const grz_graph_info_t* info, const opts_t* o)
{
    uint64_t reduce_buffer[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };  /* sz_reduce_buffer for one thread, execution_*.c:37-45 */
    const void* pull_list = info->pull_list_device;
    const void* push_list = info->push_list_device;
#if APP == GRZ_APP_PAGERANK
    /* the merge buffer of graphdata.c:1053-1072 (32 units per thread); the GPU edge phase leaves it unused */
    mergeaccum_t merge_buffer[32];
    for (int i = 0; i < 32; ++i) { merge_buffer[i].initial_vertex_id = ~0ull; merge_buffer[i].final_vertex_id = ~0ull; merge_buffer[i].final_partial_value = 0.0; }
    double unused_accumulator = 0.0;
    (void)push_list;
    for (uint64_t ctr = 0; ctr < o->iterations; ++ctr) {
#ifndef EXPERIMENT_EDGE_FORCE_PUSH
        iterations_pull += 1;
        phase_op_reset_global_accum();
        perform_edge_pull_phase(pull_list, info->pull_vectors);
        edge_pull_op_merge_with_merge_buffer(merge_buffer, 32, &unused_accumulator);
        phase_op_write_global_accum_to_buf(reduce_buffer);
#else
        iterations_push += 1;
        phase_op_reset_global_accum();
        perform_edge_push_phase(push_list, info->push_vectors);
        phase_op_write_global_accum_to_buf(reduce_buffer);
#endif
        perform_vertex_phase(0, info->num_vertices, reduce_buffer);
        total_iterations += 1;
    }
#else
    int flags = 0;
#if defined(EXPERIMENT_EDGE_FORCE_PULL)
    flags |= GRZ_FLAG_FORCE_PULL;
#endif
#if defined(EXPERIMENT_EDGE_FORCE_PUSH)
    flags |= GRZ_FLAG_FORCE_PUSH;
#endif
#if defined(EXPERIMENT_THRESHOLD_WITHOUT_COUNT)
    flags |= GRZ_FLAG_WITHOUT_COUNT;
#endif
#if defined(EXPERIMENT_THRESHOLD_WITHOUT_OUTDEGREES)
    flags |= GRZ_FLAG_WITHOUT_OUTDEG;
#endif
    gpu_or_die(grz_frontier_begin(g, APP, 0, flags), g, "frontier init");
    uint64_t converge_vote = 0;
    gpu_or_die(grz_frontier_current_vote(g, &converge_vote, NULL), g, "initial vote");
    (void)o;
#ifdef EXPERIMENT_ITERATION_PROFILE
    /* execution_bfs.c:127-139, execution_cc.c: the vote over the edges (the vertices without outdegrees) */
#ifdef EXPERIMENT_THRESHOLD_WITHOUT_OUTDEGREES
    const double profile_comparator = (double)info->num_vertices;
#else
    const double profile_comparator = (double)info->num_edges;
#endif
#endif
#ifdef EXPERIMENT_ITERATION_STATS
    gpu_or_die(grz_stats_enable(g, 1), g, "iteration stats");
#endif
    for (;;) {
        total_iterations += 1;
#if defined(EXPERIMENT_EDGE_FORCE_PULL)
        const int use_pull = 1;
#elif defined(EXPERIMENT_EDGE_FORCE_PUSH)
        const int use_pull = 0;
#elif defined(EXPERIMENT_THRESHOLD_WITHOUT_OUTDEGREES)
        const int use_pull = converge_vote > info->num_vertices / 2;
#else
        const int use_pull = converge_vote > info->num_edges / 5;
#endif
#ifdef EXPERIMENT_ITERATION_PROFILE
        const double profile_frontier = (double)converge_vote / profile_comparator;
        const uint64_t profile_t0 = now_ns();
#endif
        phase_op_reset_global_accum();
        if (use_pull) {
            iterations_pull += 1;
            perform_edge_pull_phase(pull_list, info->pull_vectors);
        } else {
            iterations_push += 1;
            perform_edge_push_phase(push_list, info->push_vectors);
        }
        phase_op_write_global_accum_to_buf(reduce_buffer);
#ifdef EXPERIMENT_ITERATION_PROFILE
        /* source/execution_bfs.c:172-215: one row per iteration; the edge phase in nanoseconds of
           wall time (the GPU finished it before the vote came back), not TSC cycles */
        gpu_or_die(grz_sync(g), g, "edge phase");
        fprintf(stderr, "%llu,%s,%llu,%.10lf\n", (unsigned long long)total_iterations, use_pull ? "Pull" : "Push",
                (unsigned long long)(now_ns() - profile_t0), profile_frontier);
#endif
        converge_vote = phase_op_combine_global_var_from_buf(reduce_buffer);
#ifdef EXPERIMENT_ITERATION_STATS
        stats_record(g, total_iterations - 1);
#endif
        if (0 == converge_vote) break;
        perform_vertex_phase(0, info->num_vertices, NULL);
    }
#endif
}

int main(int argc, char** argv)
{
    opts_t o;
    parse(argc, argv, &o);
    check_file_or_die(o.input, "-pull", 1);
    const int have_push = check_file_or_die(o.input, "-push", 0);

    grz_graph* g = NULL;
    gpu_or_die(grz_graph_create(&g, o.device, NULL), NULL, "GPU");
    const double t_load = now_ms();
#if APP == GRZ_APP_PAGERANK
    (void)have_push;
    gpu_or_die(grz_graph_load_files(g, o.input), g, "load");
#else
    /* CC and BFS need the -push list: without the file, it is derived on the device */
    gpu_or_die(grz_graph_load_files_ex(g, o.input, have_push ? 0 : GRZ_LOAD_DERIVE_PUSH), g, "load");
#endif
    grz_graph_info_t info;
    grz_graph_get_info(g, &info);
    printf("In-edges:  created %llu vectors, efficiency = %.1lf%%\n", (unsigned long long)info.pull_vectors,
           (double)info.num_edges / (double)info.pull_vectors / 4.0 * 100.0);
    if (info.push_vectors)
        printf("Out-edges: created %llu vectors, efficiency = %.1lf%%\n", (unsigned long long)info.push_vectors,
               (double)info.num_edges / (double)info.push_vectors / 4.0 * 100.0);
#ifdef EXPERIMENT_MODEL_LONG_VECTORS
    /* graphdata.c:919-923, 946-950: the same lists with 8- and 16-lane vectors */
    {
        const int lists[2] = { GRZ_LIST_PULL, GRZ_LIST_PUSH };
        const char* names[2] = { "In-edges: ", "Out-edges:" };
        for (int l = 0; l < 2; ++l) {
            if (l == 1 && !info.push_vectors) break;
            for (uint32_t lanes = 8; lanes <= 16; lanes *= 2) {
                uint64_t n = 0;
                gpu_or_die(grz_graph_vector_model(g, lists[l], lanes, &n), g, "vector model");
                printf("%s VL%u: created %llu vectors, efficiency = %.1lf%%\n", names[l], lanes, (unsigned long long)n,
                       (double)info.num_edges / (double)n / (double)lanes * 100.0);
            }
        }
    }
#endif
    /* graphdata.c:435-470 (one node: every vertex), then main.c:73-89 */
    printf("Vertices:  assigned using in-edge list\n");
    printf("Vertices:  node %u gets %llu vertices (%llu to %llu, %.2lf%% of total)\n", 0u, (unsigned long long)info.num_vertices,
           0ull, (unsigned long long)(info.num_vertices - 1), 100.0);
    {
        uint64_t threads = o.threads;
        if (threads == 0) {
            const long n = sysconf(_SC_NPROCESSORS_ONLN);
            threads = n > 0 ? (uint64_t)n : 1;
        }
        const uint64_t units = o.granularity ? info.pull_vectors / o.granularity : threads << 5;
        if (units == 0) {
            printf("Unable to set requested scheduler granularity because the graph is too small.\n");
            grz_graph_destroy(g);
            return 1;
        }
        printf("Scheduler: total units = %llu, vectors per unit = %llu\n", (unsigned long long)units,
               (unsigned long long)(info.pull_vectors / units));
    }
    printf("Loading graph took %.2lfms.\n", now_ms() - t_load);
#ifdef EXPERIMENT_MODEL_LONG_VECTORS
    printf("Not executing application, since this was a modelling experiment.\n");
    grz_graph_destroy(g);
    return 0;
#endif
#if APP == GRZ_APP_PAGERANK
    gpu_or_die(grz_pr_init(g, 0.875), g, "PageRank init");
#endif
    gpu_or_die(grz_phases_bind(g, APP), g, "bind");
    printf("Starting execution.\n");
#ifdef EXPERIMENT_ITERATION_PROFILE
    fprintf(stderr, "Iteration,Selected Engine,Edge Phase Execution Time (ns),%s\n", PROFILE_FRONTIER_COLUMN);
#endif
    const double t0 = now_ms();
    execution_impl(g, &info, &o);
    gpu_or_die(grz_sync(g), g, "execution");
    const double ms = now_ms() - t0;
    gpu_or_die(grz_phases_last_status(), g, "phase");
    printf("Execution completed.\n");

    const uint64_t V = info.num_vertices;
    double* props = (double*)malloc(sizeof(double) * (V ? V : 1));
    double* outdeg = (double*)malloc(sizeof(double) * (V ? V : 1));
    gpu_or_die(grz_read_props(g, props, V), g, "read props");
    gpu_or_die(grz_graph_copy_outdegrees(g, outdeg, V), g, "read outdegrees");

    printf("\n------------ EXECUTION STATISTICS ------------\n");
    printf("%-25s = %.2lfms\n", "Running Time", ms);
#if APP == GRZ_APP_PAGERANK
    printf("%-25s = %.0lf Medges/sec\n", "Processing Rate", (double)info.num_edges * (double)o.iterations / ms / 1000.0);
    double sum = 0.0;
    for (uint64_t v = 0; v < V; ++v) sum += props[v] * (outdeg[v] == 0.0 ? (double)V : outdeg[v]);
    printf("%-25s = %.10lf\n", "PageRank Sum", sum);
#else
    printf("%-25s = %.0lf Medges/sec\n", "Effective Processing Rate", (double)info.num_edges * (double)total_iterations / ms / 1000.0);
#endif
    printf("%-25s = %llu\n", "Total Iterations", (unsigned long long)total_iterations);
    printf("%-25s = %llu\n", "Pull-Based Iterations", (unsigned long long)iterations_pull);
    printf("%-25s = %llu\n", "Push-Based Iterations", (unsigned long long)iterations_push);
    printf("----------------------------------------------\n");
#if defined(EXPERIMENT_ITERATION_STATS) && APP != GRZ_APP_PAGERANK
    /* main.c:147-157 */
    fprintf(stderr, "%s,%s,%s\n", "Iteration", "# Vectors", "Packing Efficiency");
    for (uint64_t i = 0; i < total_iterations; ++i) {
        const uint64_t nv = stat_vectors[i];
        const double eff = nv == 0 ? 0.0 : (double)stat_edges[i] / (4.0 * (double)nv);
        fprintf(stderr, "%llu,%llu,%lf\n", (unsigned long long)(1 + i), (unsigned long long)nv, eff);
    }
#endif

    if (o.output) {
        /* graph_data_write_ranks_to_file, source/graphdata.c:1119-1138 */
        FILE* f = fopen(o.output, "w");
        if (f) {
            for (uint64_t v = 0; v < V; ++v) {
#if APP == GRZ_APP_PAGERANK
                fprintf(f, "%llu %.5le\n", (unsigned long long)v, props[v] * (outdeg[v] == 0.0 ? (double)V : outdeg[v]));
#else
                fprintf(f, "%llu %.0lf\n", (unsigned long long)v, props[v]);
#endif
            }
            fclose(f);
        }
    }
    free(props);
    free(outdeg);
    grz_graph_destroy(g);
    return 0;
}
