// grz_layout.cu -- builds Grazelle's vector-sparse layout on the device from an edge list.
//
// Input: the (src, dst) pairs of a -pull file (grouped by dst) or a -push file (grouped by src),
// already in device memory.  Output, per list (see grz_internal.cuh for the HBM layout):
//   * the reference's 256-bit vectors, bit-identical to graph_helper_write_edge_vector
//     (source/graphdata.c:143-173) as driven by the stash logic of graphdata.c:618-701 / 705-788,
//     including the stale neighbour IDs that invalid lanes inherit from the never-cleared stash;
//   * the reference vertex index (graphdata.c:219-267);
//   * the execution layout: uint4 neighbour IDs, per-vector shared vertex, CSR row pointers.
// Outdegrees follow graphdata.c:792-821 (credit per source of the -pull list).
//
// The execution form is built in three passes: the edge range [start, end) of each shared
// vertex (one pass over the pairs: run heads and tails), the vector offsets (ceil(run / 4) per
// vertex, one scan over V), and the vectors themselves (the edge whose position in its run is a
// multiple of 4 writes one vector, since the reference's stash flushes on a change of shared
// vertex or when full).  The reference-format vectors, whose invalid lanes inherit the stale
// stash values, are derived from the execution form on first request (grz_list_reference).
#include <algorithm>
#include <vector>

#include "grz_internal.cuh"

namespace {

constexpr int BT = 256;

static inline unsigned grid_blocks_for(uint64_t n) { return (unsigned)((n + BT - 1) / BT); }

// shared-vertex pieces of the spread encoding (graphdata.c:145-150)
__device__ __forceinline__ uint64_t piece_of(uint64_t s, int lane)
{
    switch (lane) {
        case 0: return (s & 0x0000000000007fffull) >> 0;
        case 1: return (s & 0x000000003fff8000ull) >> 15;
        case 2: return (s & 0x00001fffc0000000ull) >> 30;
        default: return (s & 0x0000e00000000000ull) >> 45;
    }
}

// edge range of each shared vertex: start[s] = its first edge, end[s] = one past its last (both
// 0 without edges).  flags[0]: not grouped in ascending order, flags[1]: an ID >= V.
__global__ void k_group_bounds(const uint64_t* __restrict__ pairs, uint64_t E, uint64_t V, int shared_is_dst,
                               uint32_t* __restrict__ start, uint32_t* __restrict__ end, unsigned* __restrict__ flags)
{
    const uint64_t e = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (e >= E) return;
    const int sh = shared_is_dst ? 1 : 0;
    const uint64_t s = pairs[2 * e + sh];
    const uint64_t nb = pairs[2 * e + (1 - sh)];
    if (s >= V || nb >= V) atomicOr(&flags[1], 1u);
    bool head = true, tail = true;
    if (e > 0) {
        const uint64_t sp = pairs[2 * (e - 1) + sh];
        head = sp != s;
        if (sp > s) atomicOr(&flags[0], 1u);
    }
    if (e + 1 < E) tail = pairs[2 * (e + 1) + sh] != s;
    if (s < V) {
        if (head) start[s] = (uint32_t)e;
        if (tail) end[s] = (uint32_t)(e + 1);
    }
}

// vectors of each shared vertex (entry V is 0 for the exclusive scan's total); edges of each
// shared vertex into `edges` when asked
__global__ void k_group_vectors(const uint32_t* __restrict__ start, const uint32_t* __restrict__ end, uint64_t V,
                                uint32_t* __restrict__ cnt, uint32_t* __restrict__ edges)
{
    const uint64_t v = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (v < V) {
        const uint32_t d = end[v] - start[v];
        cnt[v] = (d + 3u) / 4u;
        if (edges) edges[v] = d;
    } else if (v == V) {
        cnt[v] = 0;
    }
}

// the edge at a multiple-of-4 position of its run writes that vector: up to four neighbours,
// the rest of the lanes invalid, and the shared vertex
__global__ void k_vector_write(const uint64_t* __restrict__ pairs, uint64_t E, int shared_is_dst,
                               const uint32_t* __restrict__ start, const uint32_t* __restrict__ end,
                               const uint32_t* __restrict__ rowptr, uint4* __restrict__ nbr, uint32_t* __restrict__ shared)
{
    const uint64_t e = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (e >= E) return;
    const int sh = shared_is_dst ? 1 : 0;
    const uint32_t s = (uint32_t)pairs[2 * e + sh];
    const uint32_t pos = (uint32_t)e - __ldg(start + s);
    if (pos & 3u) return;
    const uint32_t n = min(4u, __ldg(end + s) - (uint32_t)e);
    uint32_t ids[4] = { GRZ_INVALID_ID, GRZ_INVALID_ID, GRZ_INVALID_ID, GRZ_INVALID_ID };
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k)
        if (k < n) ids[k] = (uint32_t)pairs[2 * (e + k) + (1 - sh)];
    const uint32_t vec = __ldg(rowptr + s) + pos / 4u;
    nbr[vec] = make_uint4(ids[0], ids[1], ids[2], ids[3]);
    shared[vec] = s;
}

// the reference vertex index (graphdata.c:219-267): first vector of each vertex with edges,
// 0x7fff... for one without edges up to the last shared vertex, 0xffff... beyond it
__global__ void k_vindex(const uint32_t* __restrict__ start, const uint32_t* __restrict__ end,
                         const uint32_t* __restrict__ rowptr, uint64_t V, uint64_t count, uint64_t last_shared,
                         uint64_t* __restrict__ vindex)
{
    const uint64_t i = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (i >= count) return;
    if (i < V && end[i] > start[i]) vindex[i] = rowptr[i];
    else vindex[i] = (i > last_shared) ? 0xffffffffffffffffull : 0x7fffffffffffffffull;
}

// the empty list: one vector with no valid lane and shared vertex 0 (graphdata.c:700), which the
// index and row pointers attribute to vertex 0
__global__ void k_empty_list(uint64_t* vs, uint4* nbr, uint32_t* shared)
{
    for (int l = 0; l < 4; ++l) vs[l] = 0;
    nbr[0] = make_uint4(GRZ_INVALID_ID, GRZ_INVALID_ID, GRZ_INVALID_ID, GRZ_INVALID_ID);
    shared[0] = 0;
}

__global__ void k_empty_index(uint64_t* __restrict__ vindex, uint64_t count, uint32_t* __restrict__ rowptr, uint64_t V)
{
    const uint64_t i = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (i < count) vindex[i] = i == 0 ? 0ull : 0xffffffffffffffffull;
    if (i <= V) rowptr[i] = i == 0 ? 0u : 1u;
}

// key = v+1 when lane l of vector v holds a neighbour, else 0 (inclusive max scan -> last filler)
__global__ void k_lane_keys(const uint4* __restrict__ nbr, uint64_t nvec, uint32_t* __restrict__ last1,
                            uint32_t* __restrict__ last2, uint32_t* __restrict__ last3)
{
    const uint64_t v = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (v >= nvec) return;
    const uint4 n = nbr[v];
    last1[v] = n.y != GRZ_INVALID_ID ? (uint32_t)(v + 1) : 0u;
    last2[v] = n.z != GRZ_INVALID_ID ? (uint32_t)(v + 1) : 0u;
    last3[v] = n.w != GRZ_INVALID_ID ? (uint32_t)(v + 1) : 0u;
}

// reference 256-bit vectors; invalid lanes take the stale stash value (0 before any fill).
// Hub-encoded neighbours are decoded back to their vertex IDs.
__global__ void k_vector_encode(const uint32_t* __restrict__ shared, const uint4* __restrict__ nbr,
                                const uint32_t* __restrict__ last1, const uint32_t* __restrict__ last2,
                                const uint32_t* __restrict__ last3, uint64_t nvec, const uint32_t* __restrict__ hub_vid,
                                uint32_t nhub, uint64_t* __restrict__ vs)
{
    const uint64_t v = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (v >= nvec) return;
    const uint64_t s = shared[v];
    const uint4 n = nbr[v];
    const uint32_t own[4] = { n.x, n.y, n.z, n.w };
    const uint32_t* last[4] = { nullptr, last1, last2, last3 };
    for (int l = 0; l < 4; ++l) {
        uint64_t word = piece_of(s, l) << 48;
        if (own[l] != GRZ_INVALID_ID) {
            word |= (1ull << 63) | (uint64_t)grz_hub_decode(own[l], hub_vid, nhub);
        } else if (l > 0) {
            const uint32_t src = last[l][v];  // 1 + vector that last filled lane l (< v)
            if (src) {
                const uint4 m = nbr[src - 1];
                const uint32_t mm[4] = { m.x, m.y, m.z, m.w };
                word |= (uint64_t)grz_hub_decode(mm[l], hub_vid, nhub);
            }
        }
        vs[4 * v + l] = word;
    }
}

// outdegree credit per source of the -pull list (graphdata.c:792-821); lanes of a warp that
// name the same source add once
__global__ void k_degree(const uint64_t* __restrict__ pairs, uint64_t E, uint32_t* __restrict__ degree)
{
    const uint64_t e = (uint64_t)blockIdx.x * BT + threadIdx.x;
    const bool live = e < E;
    const uint32_t s = live ? (uint32_t)pairs[2 * e] : GRZ_INVALID_ID;
    const unsigned peers = __match_any_sync(0xffffffffu, s);
    if (live && (int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&degree[s], (uint32_t)__popc(peers));
}

__global__ void k_degree_to_double(const uint32_t* __restrict__ degree, uint64_t V, double* __restrict__ outdeg,
                                   double* __restrict__ inv_deg)
{
    const uint64_t v = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (v >= V) return;
    const double d = (double)degree[v];
    outdeg[v] = d;
    inv_deg[v] = 1.0 / (d == 0.0 ? (double)V : d);
}

}  // namespace

// The rest of a list build once the run bounds [start, end) of every shared vertex are known
// (k_group_bounds, or the fused ingest of grz_sort.cu): vector offsets, vectors, vertex index.
// last_shared: the shared vertex of the last edge; first_shared: of the first.
// The edges come as pairs (written_cap 0), or L->nbr and L->shared (written_cap vectors) already
// hold the vectors and only the offsets and the index are built.  Everything, the temporaries
// included, is ordered on `st`.
int grz_build_list_from_bounds(grz_graph* g, grz_list* L, const uint64_t* d_pairs, uint64_t E, int shared_is_dst,
                               const uint32_t* start, const uint32_t* end, uint64_t first_shared, uint64_t last_shared,
                               uint32_t* run_len, cudaStream_t st, uint64_t written_cap)
{
    const uint64_t V = g->V;
    const uint64_t vi_count = V + 64;
    uint32_t *cnt = nullptr, *tot = nullptr;
    uint32_t nv32 = 0;
    int rc = GRZ_OK;
#define LCK(call) do { cudaError_t e__ = (call); if (e__ != cudaSuccess) { rc = grz_cuda_check(g, e__, #call); goto done; } } while (0)
    LCK(cudaMallocAsync((void**)&cnt, sizeof(uint32_t) * (V + 1), st));
    LCK(cudaMallocAsync((void**)&tot, sizeof(uint32_t), st));
    k_group_vectors<<<grid_blocks_for(V + 1), BT, 0, st>>>(start, end, V, cnt, run_len); GRZ_COUNT_LAUNCH(g);
    LCK(cudaGetLastError());
    rc = grz_exclusive_sum_u32_on(g, cnt, L->rowptr, V + 1, tot, st);
    if (rc) goto done;
    LCK(cudaMemcpyAsync(&nv32, tot, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    LCK(cudaStreamSynchronize(st));
    L->nvec = nv32;
    if (written_cap) {
        // the caller allocated the vectors (written_cap of them) and wrote them already
        if (L->nvec > written_cap) { rc = grz_set_error(g, GRZ_ERR_STATE, "list needs %llu vectors, %llu were written",
                                                         (unsigned long long)L->nvec, (unsigned long long)written_cap); goto done; }
    } else {
        LCK(cudaMallocAsync((void**)&L->nbr, sizeof(uint4) * L->nvec, st));
        LCK(cudaMallocAsync((void**)&L->shared, sizeof(uint32_t) * L->nvec, st));
        k_vector_write<<<grid_blocks_for(E), BT, 0, st>>>(d_pairs, E, shared_is_dst, start, end, L->rowptr, L->nbr, L->shared);
        GRZ_COUNT_LAUNCH(g);
        LCK(cudaGetLastError());
    }
    k_vindex<<<grid_blocks_for(vi_count), BT, 0, st>>>(start, end, L->rowptr, V, vi_count, last_shared, L->vindex); GRZ_COUNT_LAUNCH(g);
    LCK(cudaGetLastError());
    L->vindex_start = first_shared;
    L->vindex_end = last_shared;
    L->vs = nullptr;  // reference-format vectors: on first request
done:
    if (cnt) cudaFreeAsync(cnt, st);
    if (tot) cudaFreeAsync(tot, st);
#undef LCK
    return rc;
}

int grz_build_list(grz_graph* g, grz_list* L, const uint64_t* d_pairs, uint64_t E, int shared_is_dst, uint32_t* run_len)
{
    const uint64_t V = g->V;
    cudaStream_t st = g->stream;
    if (E >= 0xffffffffull) return grz_set_error(g, GRZ_ERR_RANGE, "edge count %llu too large (limit 2^32-2)", (unsigned long long)E);
    const uint64_t vi_count = V + 64;
    uint32_t *start = nullptr, *end = nullptr;
    unsigned* flags = nullptr;
    int rc = GRZ_OK;
#define LCK(call) do { cudaError_t e__ = (call); if (e__ != cudaSuccess) { rc = grz_cuda_check(g, e__, #call); goto done; } } while (0)
    LCK(cudaMallocAsync((void**)&L->vindex, sizeof(uint64_t) * vi_count, st));
    LCK(cudaMallocAsync((void**)&L->rowptr, sizeof(uint32_t) * (V + 1), st));
    if (E == 0) {
        L->nvec = 1;
        LCK(cudaMallocAsync((void**)&L->vs, sizeof(uint64_t) * 4, st));
        LCK(cudaMallocAsync((void**)&L->nbr, sizeof(uint4), st));
        LCK(cudaMallocAsync((void**)&L->shared, sizeof(uint32_t), st));
        k_empty_list<<<1, 1, 0, st>>>(L->vs, L->nbr, L->shared); GRZ_COUNT_LAUNCH(g);
        k_empty_index<<<grid_blocks_for(std::max<uint64_t>(vi_count, V + 1)), BT, 0, st>>>(L->vindex, vi_count, L->rowptr, V); GRZ_COUNT_LAUNCH(g);
        LCK(cudaGetLastError());
        L->vindex_start = L->vindex_end = 0;
    } else {
        unsigned flags_h[2] = { 0, 0 };
        uint64_t ends_h[2] = { 0, 0 };
        const int sh = shared_is_dst ? 1 : 0;
        LCK(cudaMallocAsync((void**)&flags, 2 * sizeof(unsigned), st));
        LCK(cudaMallocAsync((void**)&start, sizeof(uint32_t) * (V + 1), st));
        LCK(cudaMallocAsync((void**)&end, sizeof(uint32_t) * (V + 1), st));
        LCK(cudaMemsetAsync(flags, 0, 2 * sizeof(unsigned), st));
        LCK(cudaMemsetAsync(start, 0, sizeof(uint32_t) * (V + 1), st));
        LCK(cudaMemsetAsync(end, 0, sizeof(uint32_t) * (V + 1), st));
        k_group_bounds<<<grid_blocks_for(E), BT, 0, st>>>(d_pairs, E, V, shared_is_dst, start, end, flags); GRZ_COUNT_LAUNCH(g);
        LCK(cudaGetLastError());
        LCK(cudaMemcpyAsync(flags_h, flags, sizeof(flags_h), cudaMemcpyDeviceToHost, st));
        LCK(cudaMemcpyAsync(&ends_h[0], d_pairs + sh, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
        LCK(cudaMemcpyAsync(&ends_h[1], d_pairs + 2 * (E - 1) + sh, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
        LCK(cudaStreamSynchronize(st));
        if (flags_h[0]) { rc = grz_set_error(g, GRZ_ERR_UNSORTED, "%s list is not grouped by %s in ascending order", shared_is_dst ? "pull" : "push", shared_is_dst ? "destination" : "source"); goto done; }
        if (flags_h[1]) { rc = grz_set_error(g, GRZ_ERR_RANGE, "%s list holds a vertex ID >= V (%llu)", shared_is_dst ? "pull" : "push", (unsigned long long)V); goto done; }
        rc = grz_build_list_from_bounds(g, L, d_pairs, E, shared_is_dst, start, end, ends_h[0], ends_h[1], run_len, g->stream, 0);
    }
done:
    for (void* p : { (void*)flags, (void*)start, (void*)end })
        if (p) cudaFreeAsync(p, st);
#undef LCK
    if (rc == GRZ_OK) rc = grz_cuda_check(g, cudaStreamSynchronize(st), "build list");
    return rc;
}

// The reference-format vectors of a built list (graphdata.c:143-173 with the stash of
// graphdata.c:618-788), derived from the execution form: a lane the vector leaves empty holds
// the neighbour of the last earlier vector that filled that lane (the never-cleared stash).
int grz_list_reference(grz_graph* g, grz_list* L)
{
    if (L->vs || !L->nbr) return GRZ_OK;
    cudaStream_t st = g->stream;
    const uint64_t nvec = L->nvec;
    uint32_t* l1 = nullptr;
    int rc = GRZ_OK;
#define LCK(call) do { cudaError_t e__ = (call); if (e__ != cudaSuccess) { rc = grz_cuda_check(g, e__, #call); goto done; } } while (0)
    LCK(cudaMallocAsync((void**)&L->vs, sizeof(uint64_t) * 4 * nvec, st));
    LCK(cudaMallocAsync((void**)&l1, sizeof(uint32_t) * nvec * 3, st));
    k_lane_keys<<<grid_blocks_for(nvec), BT, 0, st>>>(L->nbr, nvec, l1, l1 + nvec, l1 + 2 * nvec); GRZ_COUNT_LAUNCH(g);
    LCK(cudaGetLastError());
    for (int k = 0; k < 3 && rc == GRZ_OK; ++k) rc = grz_inclusive_max_u32(g, l1 + k * nvec, l1 + k * nvec, nvec);
    if (rc) goto done;
    k_vector_encode<<<grid_blocks_for(nvec), BT, 0, st>>>(L->shared, L->nbr, l1, l1 + nvec, l1 + 2 * nvec, nvec, L->hub_vid,
                                                          L->nhub, L->vs); GRZ_COUNT_LAUNCH(g);
    LCK(cudaGetLastError());
done:
    if (l1) cudaFreeAsync(l1, st);
#undef LCK
    if (rc == GRZ_OK) rc = grz_cuda_check(g, cudaStreamSynchronize(st), "reference vectors");
    if (rc != GRZ_OK && L->vs) {
        cudaFree(L->vs);
        L->vs = nullptr;
    }
    return rc;
}

// the outdegree arrays, degree zeroed
int grz_alloc_outdegrees(grz_graph* g)
{
    const uint64_t V = g->V;
    if (g->degree) return GRZ_OK;
    int rc = grz_dev_alloc(g, (void**)&g->degree, sizeof(uint32_t) * (V + 1));
    if (!rc) rc = grz_dev_alloc(g, (void**)&g->outdeg, sizeof(double) * (V + 8));
    if (!rc) rc = grz_dev_alloc(g, (void**)&g->inv_deg, sizeof(double) * (V + 1));
    if (rc) return rc;
    GRZ_CK(g, cudaMemsetAsync(g->degree, 0, sizeof(uint32_t) * (V + 1), g->stream));
    return GRZ_OK;
}

// Outdegrees: counted from the -pull pairs, or (d_pull_pairs null) already in g->degree, where
// grz_build_list put the run lengths of a -push list derived from those pairs.
int grz_build_outdegrees(grz_graph* g, const uint64_t* d_pull_pairs, uint64_t E, cudaStream_t st)
{
    const uint64_t V = g->V;
    if (!st) st = g->stream;
    int rc = grz_alloc_outdegrees(g);
    if (rc) return rc;
    GRZ_CK(g, cudaMemsetAsync(g->outdeg + V, 0, sizeof(double) * 8, st));  // the padding; k_degree_to_double writes the rest
    if (E > 0 && d_pull_pairs) {
        k_degree<<<grid_blocks_for(E), BT, 0, st>>>(d_pull_pairs, E, g->degree); GRZ_COUNT_LAUNCH(g);
        GRZ_CK(g, cudaGetLastError());
    }
    if (V > 0) {
        k_degree_to_double<<<grid_blocks_for(V), BT, 0, st>>>(g->degree, V, g->outdeg, g->inv_deg); GRZ_COUNT_LAUNCH(g);
        GRZ_CK(g, cudaGetLastError());
    }
    return GRZ_OK;
}

// ---------------------------------------------------------------------------------------------
// Hub sources of the pull list (see GRZ_HUB_BASE).  The hubs are the vertices with the highest
// out-degree (number of pull-list lanes that name them).  Selection: a histogram of
// min(degree, HUB_BINS - 1) gives the smallest degree bin above which at most max_hubs
// vertices lie; those candidates are compacted in ID order, sorted on the host by (degree
// descending, ID) and cut to max_hubs; the list's neighbour fields are then rewritten.

namespace {

constexpr uint32_t HUB_BINS = 8192;

__global__ void __launch_bounds__(BT) k_deg_hist(const uint32_t* __restrict__ degree, uint64_t V, uint32_t* __restrict__ hist)
{
    __shared__ uint32_t h[HUB_BINS];
    for (uint32_t i = threadIdx.x; i < HUB_BINS; i += BT) h[i] = 0;
    __syncthreads();
    for (uint64_t v = (uint64_t)blockIdx.x * BT + threadIdx.x; v < V; v += (uint64_t)gridDim.x * BT)
        atomicAdd(&h[min(degree[v], HUB_BINS - 1)], 1u);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < HUB_BINS; i += BT)
        if (h[i]) atomicAdd(hist + i, h[i]);
}

__global__ void k_hub_flags(const uint32_t* __restrict__ degree, uint64_t V, uint32_t tbin, uint32_t* __restrict__ flags)
{
    const uint64_t v = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (v < V) flags[v] = min(degree[v], HUB_BINS - 1) > tbin ? 1u : 0u;
}

__global__ void k_hub_compact(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ pos, uint64_t V,
                              const uint32_t* __restrict__ degree, uint32_t* __restrict__ cand, uint32_t* __restrict__ cand_deg)
{
    const uint64_t v = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (v < V && flags[v]) {
        cand[pos[v]] = (uint32_t)v;
        cand_deg[pos[v]] = degree[v];
    }
}

__global__ void k_hub_slots(const uint32_t* __restrict__ hub_vid, uint32_t nhub, uint32_t* __restrict__ slot_of)
{
    const uint32_t i = blockIdx.x * BT + threadIdx.x;
    if (i < nhub) slot_of[hub_vid[i]] = i;
}

__global__ void k_hub_encode(uint4* __restrict__ nbr, uint64_t nvec, const uint32_t* __restrict__ slot_of, uint32_t V)
{
    const uint64_t v = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (v >= nvec) return;
    uint4 s = nbr[v];
    uint32_t* f[4] = { &s.x, &s.y, &s.z, &s.w };
    bool any = false;
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        const uint32_t x = *f[l];
        if (x < V) {
            const uint32_t sl = slot_of[x];
            if (sl != GRZ_INVALID_ID) { *f[l] = GRZ_HUB_BASE + sl; any = true; }
        }
    }
    if (any) nbr[v] = s;
}

}  // namespace

int grz_build_hubs(grz_graph* g, grz_list* L, uint32_t max_hubs)
{
    const uint64_t V = g->V;
    cudaStream_t st = g->stream;
    L->nhub = 0;
    if (max_hubs > GRZ_HUB_MAX) max_hubs = GRZ_HUB_MAX;
    if (max_hubs == 0 || V == 0 || V >= GRZ_HUB_BASE || !L->nbr || L->nvec == 0) return GRZ_OK;
    int rc = GRZ_OK;
    uint32_t *hist = nullptr, *flags = nullptr, *pos = nullptr, *tot = nullptr, *cand = nullptr, *cdeg = nullptr, *slot_of = nullptr;
    std::vector<uint32_t> h(HUB_BINS);
#define HCK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { rc = grz_cuda_check(g, e_, #x); goto done; } } while (0)
    {
        HCK(cudaMallocAsync((void**)&hist, sizeof(uint32_t) * HUB_BINS, st));
        HCK(cudaMemsetAsync(hist, 0, sizeof(uint32_t) * HUB_BINS, st));
        const unsigned grid = (unsigned)std::min<uint64_t>(grid_blocks_for(V), (uint64_t)g->num_sms * 4);
        k_deg_hist<<<grid, BT, 0, st>>>(g->degree, V, hist); GRZ_COUNT_LAUNCH(g);
        HCK(cudaGetLastError());
        HCK(cudaMemcpyAsync(h.data(), hist, sizeof(uint32_t) * HUB_BINS, cudaMemcpyDeviceToHost, st));
        HCK(cudaStreamSynchronize(st));
        // smallest tbin >= 1 with count(bin > tbin) <= max_hubs; a hub has degree >= 2
        uint64_t above = 0;
        uint32_t tbin = HUB_BINS - 1;
        while (tbin > 1 && above + h[tbin] <= max_hubs) above += h[tbin--];
        if (tbin == HUB_BINS - 1) tbin = HUB_BINS - 2;  // more top-bin vertices than slots: sort them all
        HCK(cudaMallocAsync((void**)&flags, sizeof(uint32_t) * V, st));
        HCK(cudaMallocAsync((void**)&pos, sizeof(uint32_t) * V, st));
        HCK(cudaMallocAsync((void**)&tot, sizeof(uint32_t), st));
        k_hub_flags<<<grid_blocks_for(V), BT, 0, st>>>(g->degree, V, tbin, flags); GRZ_COUNT_LAUNCH(g);
        HCK(cudaGetLastError());
        rc = grz_exclusive_sum_u32(g, flags, pos, V, tot);
        if (rc) goto done;
        uint32_t ncand = 0;
        HCK(cudaMemcpyAsync(&ncand, tot, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        HCK(cudaStreamSynchronize(st));
        if (ncand == 0) goto done;
        HCK(cudaMallocAsync((void**)&cand, sizeof(uint32_t) * ncand, st));
        HCK(cudaMallocAsync((void**)&cdeg, sizeof(uint32_t) * ncand, st));
        k_hub_compact<<<grid_blocks_for(V), BT, 0, st>>>(flags, pos, V, g->degree, cand, cdeg); GRZ_COUNT_LAUNCH(g);
        HCK(cudaGetLastError());
        std::vector<uint32_t> hc(ncand), hd(ncand);
        HCK(cudaMemcpyAsync(hc.data(), cand, sizeof(uint32_t) * ncand, cudaMemcpyDeviceToHost, st));
        HCK(cudaMemcpyAsync(hd.data(), cdeg, sizeof(uint32_t) * ncand, cudaMemcpyDeviceToHost, st));
        HCK(cudaStreamSynchronize(st));
        std::vector<uint32_t> order(ncand);
        for (uint32_t i = 0; i < ncand; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return hd[a] > hd[b]; });
        const uint32_t nhub = std::min<uint32_t>(ncand, max_hubs);
        std::vector<uint32_t> vid(nhub);
        for (uint32_t i = 0; i < nhub; ++i) vid[i] = hc[order[i]];
        HCK(cudaMallocAsync((void**)&L->hub_vid, sizeof(uint32_t) * nhub, st));
        HCK(cudaMemcpyAsync(L->hub_vid, vid.data(), sizeof(uint32_t) * nhub, cudaMemcpyHostToDevice, st));
        HCK(cudaMallocAsync((void**)&slot_of, sizeof(uint32_t) * V, st));
        HCK(cudaMemsetAsync(slot_of, 0xff, sizeof(uint32_t) * V, st));
        k_hub_slots<<<grid_blocks_for(nhub), BT, 0, st>>>(L->hub_vid, nhub, slot_of); GRZ_COUNT_LAUNCH(g);
        k_hub_encode<<<grid_blocks_for(L->nvec), BT, 0, st>>>(L->nbr, L->nvec, slot_of, (uint32_t)V); GRZ_COUNT_LAUNCH(g);
        HCK(cudaGetLastError());
        HCK(cudaStreamSynchronize(st));
        L->nhub = nhub;
    }
done:
#undef HCK
    for (uint32_t* p : { hist, flags, pos, tot, cand, cdeg, slot_of })
        if (p) cudaFreeAsync(p, st);
    return rc;
}
