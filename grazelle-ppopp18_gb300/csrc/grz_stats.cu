// grz_stats.cu -- the reference's measurement experiments, as device reductions.
//
// ITERATION_STATS (source/execution_cc.c:209-231, source/execution_bfs.c:217-239, printed at
// source/main.c:147-157; counted by phase_helper_iteration_stats, include/phasehelpers.inc:
// 401-428): per iteration, the vectors the edge phase worked through and their valid lanes
// (edges), whose ratio over 4 per vector is the packing efficiency.  Here the edge phases
// count, when stats are on, the vectors they process: a pull over a vector range counts the
// range, a compacted pull or push counts the selected vertices' vectors.
//
// MODEL_LONG_VECTORS (source/graphdata.c:628-675, printed at :919-923 and :946-950): the vectors
// a list would need with 8 or 16 lanes, i.e. the sum over shared vertices of ceil(run / lanes).
#include "grz_internal.cuh"
#include "../../include/grazelle_gb300.h"

namespace {

constexpr int ST_T = 256;

__device__ __forceinline__ uint32_t valid_lanes(const uint4 n)
{
    return (n.x != GRZ_INVALID_ID) + (n.y != GRZ_INVALID_ID) + (n.z != GRZ_INVALID_ID) + (n.w != GRZ_INVALID_ID);
}

__device__ __forceinline__ void add_warp(unsigned long long* out, unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(out, v);
}

// valid lanes of vectors [first, first + count) into out[1]
__global__ void k_stat_range(const uint4* __restrict__ nbr, uint64_t first, uint64_t count, unsigned long long* __restrict__ out)
{
    unsigned long long e = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * ST_T + threadIdx.x; i < count; i += (uint64_t)gridDim.x * ST_T)
        e += valid_lanes(nbr[first + i]);
    add_warp(out + 1, e);
}

// vectors and valid lanes of the compacted selection (counters[0] vertices in `sel`)
__global__ void k_stat_selected(const uint32_t* __restrict__ sel, const uint32_t* __restrict__ counters,
                                const uint32_t* __restrict__ rowptr, const uint4* __restrict__ nbr,
                                unsigned long long* __restrict__ out)
{
    const uint32_t n = counters[0];
    unsigned long long vec = 0, e = 0;
    for (uint32_t i = blockIdx.x * ST_T + threadIdx.x; i < n; i += gridDim.x * ST_T) {
        const uint32_t v = sel[i];
        for (uint32_t k = rowptr[v]; k < rowptr[v + 1]; ++k) {
            ++vec;
            e += valid_lanes(nbr[k]);
        }
    }
    add_warp(out, vec);
    add_warp(out + 1, e);
}

// sum over shared vertices of ceil(run / lanes); a run is 4 per full vector plus the lanes of its
// last vector
__global__ void k_vector_model(const uint32_t* __restrict__ rowptr, const uint4* __restrict__ nbr, uint64_t V, uint32_t lanes,
                               unsigned long long* __restrict__ out)
{
    unsigned long long s = 0;
    for (uint64_t v = (uint64_t)blockIdx.x * ST_T + threadIdx.x; v < V; v += (uint64_t)gridDim.x * ST_T) {
        const uint32_t c = rowptr[v + 1] - rowptr[v];
        if (c == 0) continue;
        const uint64_t run = 4ull * (c - 1) + valid_lanes(nbr[rowptr[v + 1] - 1]);
        s += (run + lanes - 1) / lanes;
    }
    add_warp(out, s);
}

unsigned stat_grid(const grz_graph* g) { return (unsigned)g->num_sms * 4; }

}  // namespace

// ---- hooks of the edge phases (grz_ccbfs.cu), active only while stats are on ----

int grz_stats_count_range(grz_graph* g, const grz_list* L, uint64_t first, uint64_t count)
{
    if (!g->stats_on || count == 0) return GRZ_OK;
    g->stats_host[0] += count;
    k_stat_range<<<stat_grid(g), ST_T, 0, g->stream>>>(L->nbr, first, count, g->stats_dev); GRZ_COUNT_LAUNCH(g);
    return grz_cuda_check(g, cudaGetLastError(), "iteration stats");
}

int grz_stats_count_selected(grz_graph* g, const grz_list* L, const uint32_t* sel, const uint32_t* counters)
{
    if (!g->stats_on) return GRZ_OK;
    k_stat_selected<<<stat_grid(g), ST_T, 0, g->stream>>>(sel, counters, L->rowptr, L->nbr, g->stats_dev); GRZ_COUNT_LAUNCH(g);
    return grz_cuda_check(g, cudaGetLastError(), "iteration stats");
}

// ---- C ABI ----

extern "C" int grz_stats_enable(grz_graph* g, int on)
{
    if (!g) return GRZ_ERR_ARG;
    GRZ_CK(g, cudaSetDevice(g->device));
    if (on && !g->stats_dev) GRZ_CK(g, cudaMalloc((void**)&g->stats_dev, sizeof(unsigned long long) * 2));
    if (g->stats_dev) GRZ_CK(g, cudaMemsetAsync(g->stats_dev, 0, sizeof(unsigned long long) * 2, g->stream));
    g->stats_host[0] = 0;
    g->stats_on = on ? 1 : 0;
    return GRZ_OK;
}

extern "C" int grz_stats_take(grz_graph* g, uint64_t* vectors, uint64_t* edges)
{
    if (!g || !vectors || !edges) return GRZ_ERR_ARG;
    if (!g->stats_dev) return grz_set_error(g, GRZ_ERR_STATE, "iteration stats not enabled");
    unsigned long long h[2] = { 0, 0 };
    GRZ_CK(g, cudaMemcpyAsync(h, g->stats_dev, sizeof(h), cudaMemcpyDeviceToHost, g->stream));
    GRZ_CK(g, cudaMemsetAsync(g->stats_dev, 0, sizeof(h), g->stream));
    GRZ_CK(g, cudaStreamSynchronize(g->stream));
    *vectors = h[0] + g->stats_host[0];
    *edges = h[1];
    g->stats_host[0] = 0;
    return GRZ_OK;
}

extern "C" int grz_graph_vector_model(grz_graph* g, int list, uint32_t lanes, uint64_t* vectors)
{
    if (!g || !vectors || lanes == 0) return GRZ_ERR_ARG;
    const grz_list* L = list == GRZ_LIST_PUSH ? &g->push : &g->pull;
    if (!L->nbr) return grz_set_error(g, GRZ_ERR_STATE, "list not built");
    GRZ_CK(g, cudaSetDevice(g->device));
    unsigned long long* d = nullptr;
    unsigned long long h = 0;
    GRZ_CK(g, cudaMallocAsync((void**)&d, sizeof(h), g->stream));
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(h), g->stream);
    if (e == cudaSuccess && g->V) {
        k_vector_model<<<stat_grid(g), ST_T, 0, g->stream>>>(L->rowptr, L->nbr, g->V, lanes, d); GRZ_COUNT_LAUNCH(g);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, g->stream);
    cudaFreeAsync(d, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    GRZ_CK(g, e);
    *vectors = h;
    return GRZ_OK;
}
