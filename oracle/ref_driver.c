/*
 * Full-precision dump driver for the unmodified Grazelle reference.
 *
 * Test infrastructure only.  Linked (by oracle/build_ref.py) against every
 * object of the reference except source/main.c.o.  It repeats the start-up
 * sequence of source/main.c:62-117 (NUMA init, command line, execution_init,
 * graph_data_read_from_file, scheduler unit counts from main.c:75-90, merge
 * buffers) and then runs the same threads_spawn(execution_impl) call, timed
 * with CLOCK_MONOTONIC instead of the coarse clock of source/benchmark.c.
 *
 * Outputs, selected by environment variables:
 *   GRZ_REF_DUMP=<file>        header + graph_vertex_props[V] + graph_vertex_outdegrees[V]
 *   GRZ_REF_DUMP_LISTS=<file>  the in-edge (gather) and out-edge (scatter) vector lists
 *                              and their vertex indices, written before execution
 *
 * The printed stats block keeps the reference's labels (main.c:123-145).
 */
#include "cmdline.h"
#include "execution.h"
#include "graphdata.h"
#include "numanodes.h"
#include "scheduler.h"
#include "threads.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <time.h>

#define GRZ_REF_MAGIC 0x3130464552525a47ull /* "GZRREF01" little-endian */

static void write_or_die(const void* p, size_t sz, size_t n, FILE* f)
{
    if (n && fwrite(p, sz, n, f) != n) { fprintf(stderr, "ref_driver: short write\n"); exit(254); }
}

static void dump_lists(const char* path)
{
    FILE* f = fopen(path, "wb");
    if (!f) { fprintf(stderr, "ref_driver: cannot open %s\n", path); exit(254); }
    const uint64_t vi_count = graph_num_vertices + 8ull * sizeof(uint64_t);
    uint64_t hdr[4] = { graph_num_vertices, graph_num_edges, 0, 0 };
    hdr[2] = graph_edges_gather_list_block_counts_numa[0][0];
    hdr[3] = (graph_edges_scatter_list_block_counts_numa != NULL) ? graph_edges_scatter_list_block_counts_numa[0][0] : 0ull;
    write_or_die(hdr, sizeof(uint64_t), 4, f);
    write_or_die(graph_edges_gather_list_block_bufs_numa[0][0], 32, hdr[2], f);
    write_or_die(graph_vertex_gather_index_numa[0], sizeof(uint64_t), vi_count, f);
    if (hdr[3]) {
        write_or_die(graph_edges_scatter_list_block_bufs_numa[0][0], 32, hdr[3], f);
        write_or_die(graph_vertex_scatter_index_numa[0], sizeof(uint64_t), vi_count, f);
    }
    fclose(f);
}

int main(int argc, char* argv[])
{
    numanodes_initialize();
    cmdline_parse_options_or_die(argc, argv);
    const cmdline_opts_t* s = cmdline_get_current_settings();

    execution_init();
    graph_data_read_from_file(s->graph_input_filename_gather, s->graph_input_filename_scatter, s->num_numa_nodes, s->numa_nodes);

    if (0ull == s->sched_granularity) {
        sched_pull_units_per_node = (s->num_threads / s->num_numa_nodes) << 5ull;
    } else {
        sched_pull_units_per_node = graph_edges_gather_list_vector_count / (uint64_t)s->num_numa_nodes / s->sched_granularity;
        if (0ull == sched_pull_units_per_node) {
            printf("Unable to set requested scheduler granularity because the graph is too small.\n");
            return 1;
        }
    }
    sched_pull_units_total = sched_pull_units_per_node * s->num_numa_nodes;
    graph_data_allocate_merge_buffers(s->num_threads, s->num_numa_nodes, s->numa_nodes);
#ifdef EXPERIMENT_ITERATION_STATS
    graph_data_allocate_stats(s->num_threads, s->numa_nodes[0]);
#endif

    const char* lists = getenv("GRZ_REF_DUMP_LISTS");
    if (lists && lists[0]) dump_lists(lists);

    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    threads_spawn(s->num_threads, s->num_numa_nodes, s->numa_nodes, 0, execution_impl, NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    const uint64_t ns = (uint64_t)(t1.tv_sec - t0.tv_sec) * 1000000000ull + (uint64_t)(t1.tv_nsec - t0.tv_nsec);
    const double ms = (double)ns / 1e6;

    printf("%-25s = %.3lfms\n", "Running Time", ms);
    printf("%-25s = %llu\n", "Total Iterations", (unsigned long long)total_iterations_executed);
    printf("%-25s = %llu\n", "Pull-Based Iterations", (unsigned long long)total_iterations_used_gather);
    printf("%-25s = %llu\n", "Push-Based Iterations", (unsigned long long)total_iterations_used_scatter);
    printf("%-25s = %u\n", "Threads", s->num_threads);
    printf("%-25s = %llu\n", "Pull Units", (unsigned long long)sched_pull_units_total);

    const char* dump = getenv("GRZ_REF_DUMP");
    if (dump && dump[0]) {
        FILE* f = fopen(dump, "wb");
        if (!f) { fprintf(stderr, "ref_driver: cannot open %s\n", dump); return 254; }
        uint64_t hdr[8] = { GRZ_REF_MAGIC, graph_num_vertices, graph_num_edges, total_iterations_executed,
                            total_iterations_used_gather, total_iterations_used_scatter, ns, s->num_threads };
        write_or_die(hdr, sizeof(uint64_t), 8, f);
        write_or_die(graph_vertex_props, sizeof(double), graph_num_vertices, f);
        write_or_die(graph_vertex_outdegrees, sizeof(double), graph_num_vertices, f);
        fclose(f);
    }
    return 0;
}
