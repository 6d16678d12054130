// grz_ccbfs.cu -- Connected Components and BFS phases (placeholder until the kernels land).
#include "grz_internal.cuh"

int grz_cc_phase(grz_graph* g, int pull, uint64_t first_vec, uint64_t count)
{
    (void)pull; (void)first_vec; (void)count;
    return grz_set_error(g, GRZ_ERR_STATE, "connected components not available");
}

int grz_bfs_phase(grz_graph* g, int pull, uint64_t first_vec, uint64_t count)
{
    (void)pull; (void)first_vec; (void)count;
    return grz_set_error(g, GRZ_ERR_STATE, "bfs not available");
}

int grz_frontier_vertex_phase(grz_graph* g, uint64_t first, uint64_t count)
{
    (void)first; (void)count;
    return grz_set_error(g, GRZ_ERR_STATE, "frontier vertex phase not available");
}
