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
// Edge e starts a new vector when it starts a run of its shared vertex or when its position in
// the run is a multiple of 4 (the stash flushes on a change of shared vertex or when full), so
// vector numbers come from a scan over those flags, and a lane is (position in run) mod 4.
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

// flags[0]: unsorted, flags[1]: id out of range
__global__ void k_edge_heads(const uint64_t* __restrict__ pairs, uint64_t E, uint64_t V, int shared_is_dst,
                             uint32_t* __restrict__ head_pos, unsigned* __restrict__ flags)
{
    const uint64_t e = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (e >= E) return;
    const uint64_t s = pairs[2 * e + (shared_is_dst ? 1 : 0)];
    const uint64_t nb = pairs[2 * e + (shared_is_dst ? 0 : 1)];
    bool head = (e == 0);
    if (e > 0) {
        const uint64_t sp = pairs[2 * (e - 1) + (shared_is_dst ? 1 : 0)];
        head = (sp != s);
        if (sp > s) atomicOr(&flags[0], 1u);
    }
    if (s >= V || nb >= V) atomicOr(&flags[1], 1u);
    head_pos[e] = head ? (uint32_t)e : 0u;
}

__global__ void k_vector_starts(const uint32_t* __restrict__ run_start, uint64_t E, uint32_t* __restrict__ vstart)
{
    const uint64_t e = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (e >= E) return;
    const uint32_t pos = (uint32_t)e - run_start[e];
    vstart[e] = (pos & 3u) == 0 ? 1u : 0u;  // a run start has pos 0
}

// vfirst[v] = first edge of vector v; written by the edge that starts it
__global__ void k_vector_first(const uint32_t* __restrict__ vstart, const uint32_t* __restrict__ vnum_excl, uint64_t E,
                               uint32_t* __restrict__ vfirst)
{
    const uint64_t e = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (e >= E) return;
    if (vstart[e]) vfirst[vnum_excl[e]] = (uint32_t)e;
}

// per vector: lane count, shared vertex, valid neighbours; keys for the stale-lane scans
__global__ void k_vector_fill(const uint64_t* __restrict__ pairs, int shared_is_dst, const uint32_t* __restrict__ vfirst,
                              uint64_t nvec, uint64_t E, uint32_t* __restrict__ shared_out, uint4* __restrict__ nbr_out,
                              uint32_t* __restrict__ last1, uint32_t* __restrict__ last2, uint32_t* __restrict__ last3)
{
    const uint64_t v = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (v >= nvec) return;
    const uint64_t f = vfirst[v];
    const uint64_t nx = (v + 1 < nvec) ? vfirst[v + 1] : E;
    const uint32_t cnt = (uint32_t)(nx - f);
    uint32_t ids[4] = { GRZ_INVALID_ID, GRZ_INVALID_ID, GRZ_INVALID_ID, GRZ_INVALID_ID };
    for (uint32_t k = 0; k < cnt && k < 4; ++k) ids[k] = (uint32_t)pairs[2 * (f + k) + (shared_is_dst ? 0 : 1)];
    shared_out[v] = (uint32_t)pairs[2 * f + (shared_is_dst ? 1 : 0)];
    nbr_out[v] = make_uint4(ids[0], ids[1], ids[2], ids[3]);
    // key = v+1 when lane l is filled by this vector, else 0 (inclusive max scan -> last filler)
    last1[v] = cnt > 1 ? (uint32_t)(v + 1) : 0u;
    last2[v] = cnt > 2 ? (uint32_t)(v + 1) : 0u;
    last3[v] = cnt > 3 ? (uint32_t)(v + 1) : 0u;
}

// reference 256-bit vectors; invalid lanes take the stale stash value (0 before any fill)
__global__ void k_vector_encode(const uint32_t* __restrict__ shared, const uint4* __restrict__ nbr,
                                const uint32_t* __restrict__ last1, const uint32_t* __restrict__ last2,
                                const uint32_t* __restrict__ last3, uint64_t nvec, uint64_t* __restrict__ vs)
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
            word |= (1ull << 63) | (uint64_t)own[l];
        } else if (l > 0) {
            const uint32_t src = last[l][v];  // 1 + vector that last filled lane l (<= v, not v itself)
            if (src) {
                const uint4 m = nbr[src - 1];
                const uint32_t mm[4] = { m.x, m.y, m.z, m.w };
                word |= (uint64_t)mm[l];
            }
        }
        vs[4 * v + l] = word;
    }
}

// the empty list: one vector with no valid lane and shared vertex 0 (graphdata.c:700)
__global__ void k_empty_list(uint64_t* vs, uint4* nbr, uint32_t* shared)
{
    for (int l = 0; l < 4; ++l) vs[l] = 0;
    nbr[0] = make_uint4(GRZ_INVALID_ID, GRZ_INVALID_ID, GRZ_INVALID_ID, GRZ_INVALID_ID);
    shared[0] = 0;
}

__global__ void k_vindex_fill(uint64_t* __restrict__ vindex, uint64_t count, uint64_t first_shared, uint64_t last_shared)
{
    const uint64_t i = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (i >= count) return;
    vindex[i] = (i > last_shared) ? 0xffffffffffffffffull : 0x7fffffffffffffffull;
}

__global__ void k_vindex_heads(const uint32_t* __restrict__ shared, uint64_t nvec, uint64_t* __restrict__ vindex)
{
    const uint64_t v = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (v >= nvec) return;
    if (v == 0 || shared[v - 1] != shared[v]) vindex[shared[v]] = v;
}

// vectors per vertex, written at the last vector of each run
__global__ void k_row_counts(const uint32_t* __restrict__ shared, uint64_t nvec, const uint64_t* __restrict__ vindex,
                             uint32_t* __restrict__ cnt)
{
    const uint64_t v = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (v >= nvec) return;
    const uint32_t s = shared[v];
    if (v + 1 == nvec || shared[v + 1] != s) cnt[s] = (uint32_t)(v + 1 - vindex[s]);
}

__global__ void k_degree(const uint64_t* __restrict__ pairs, uint64_t E, uint32_t* __restrict__ degree)
{
    const uint64_t e = (uint64_t)blockIdx.x * BT + threadIdx.x;
    if (e >= E) return;
    atomicAdd(&degree[pairs[2 * e]], 1u);
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

int grz_build_list(grz_graph* g, grz_list* L, const uint64_t* d_pairs, uint64_t E, int shared_is_dst)
{
    const uint64_t V = g->V;
    cudaStream_t st = g->stream;
    if (E >= 0xffffffffull) return grz_set_error(g, GRZ_ERR_RANGE, "edge count %llu too large (limit 2^32-2)", (unsigned long long)E);
    uint64_t nvec = 1;
    unsigned flags_h[2] = { 0, 0 };
    uint32_t *head = nullptr, *vstart = nullptr, *vexcl = nullptr, *vfirst = nullptr, *l1 = nullptr, *l2 = nullptr, *l3 = nullptr;
    unsigned* flags = nullptr;
    int rc = GRZ_OK;
    const uint64_t vi_count = V + 64;

#define LCK(call) do { cudaError_t e__ = (call); if (e__ != cudaSuccess) { rc = grz_cuda_check(g, e__, #call); goto done; } } while (0)
    if (E > 0) {
        LCK(cudaMallocAsync((void**)&flags, 2 * sizeof(unsigned), st));
        LCK(cudaMemsetAsync(flags, 0, 2 * sizeof(unsigned), st));
        LCK(cudaMallocAsync((void**)&head, sizeof(uint32_t) * E, st));
        LCK(cudaMallocAsync((void**)&vstart, sizeof(uint32_t) * E, st));
        LCK(cudaMallocAsync((void**)&vexcl, sizeof(uint32_t) * (E + 1), st));
        k_edge_heads<<<grid_blocks_for(E), BT, 0, st>>>(d_pairs, E, V, shared_is_dst, head, flags); GRZ_COUNT_LAUNCH(g);
        LCK(cudaGetLastError());
        LCK(cudaMemcpyAsync(flags_h, flags, sizeof(flags_h), cudaMemcpyDeviceToHost, st));
        LCK(cudaStreamSynchronize(st));
        if (flags_h[0]) { rc = grz_set_error(g, GRZ_ERR_UNSORTED, "%s list is not grouped by %s in ascending order", shared_is_dst ? "pull" : "push", shared_is_dst ? "destination" : "source"); goto done; }
        if (flags_h[1]) { rc = grz_set_error(g, GRZ_ERR_RANGE, "%s list holds a vertex ID >= V (%llu)", shared_is_dst ? "pull" : "push", (unsigned long long)V); goto done; }
        rc = grz_inclusive_max_u32(g, head, head, E);  // head[] now holds each edge's run start
        if (rc) goto done;
        k_vector_starts<<<grid_blocks_for(E), BT, 0, st>>>(head, E, vstart); GRZ_COUNT_LAUNCH(g);
        LCK(cudaGetLastError());
        rc = grz_exclusive_sum_u32(g, vstart, vexcl, E, vexcl + E);
        if (rc) goto done;
        uint32_t nv32 = 0;
        LCK(cudaMemcpyAsync(&nv32, vexcl + E, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        LCK(cudaStreamSynchronize(st));
        nvec = nv32;
    }
    L->nvec = nvec;
    LCK(cudaMallocAsync((void**)&L->vs, sizeof(uint64_t) * 4 * nvec, st));
    LCK(cudaMallocAsync((void**)&L->nbr, sizeof(uint4) * nvec, st));
    LCK(cudaMallocAsync((void**)&L->shared, sizeof(uint32_t) * nvec, st));
    LCK(cudaMallocAsync((void**)&L->vindex, sizeof(uint64_t) * vi_count, st));
    LCK(cudaMallocAsync((void**)&L->rowptr, sizeof(uint32_t) * (V + 1), st));
    if (E > 0) {
        LCK(cudaMallocAsync((void**)&vfirst, sizeof(uint32_t) * nvec, st));
        LCK(cudaMallocAsync((void**)&l1, sizeof(uint32_t) * nvec * 3, st));
        l2 = l1 + nvec;
        l3 = l2 + nvec;
        k_vector_first<<<grid_blocks_for(E), BT, 0, st>>>(vstart, vexcl, E, vfirst); GRZ_COUNT_LAUNCH(g);
        LCK(cudaGetLastError());
        k_vector_fill<<<grid_blocks_for(nvec), BT, 0, st>>>(d_pairs, shared_is_dst, vfirst, nvec, E, L->shared, L->nbr, l1, l2, l3); GRZ_COUNT_LAUNCH(g);
        LCK(cudaGetLastError());
        if ((rc = grz_inclusive_max_u32(g, l1, l1, nvec))) goto done;
        if ((rc = grz_inclusive_max_u32(g, l2, l2, nvec))) goto done;
        if ((rc = grz_inclusive_max_u32(g, l3, l3, nvec))) goto done;
        k_vector_encode<<<grid_blocks_for(nvec), BT, 0, st>>>(L->shared, L->nbr, l1, l2, l3, nvec, L->vs); GRZ_COUNT_LAUNCH(g);
        LCK(cudaGetLastError());
    } else {
        k_empty_list<<<1, 1, 0, st>>>(L->vs, L->nbr, L->shared); GRZ_COUNT_LAUNCH(g);
        LCK(cudaGetLastError());
    }
    {
        uint32_t fs = 0, ls = 0;
        LCK(cudaMemcpyAsync(&fs, L->shared, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        LCK(cudaMemcpyAsync(&ls, L->shared + (nvec - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        LCK(cudaStreamSynchronize(st));
        L->vindex_start = fs;
        L->vindex_end = ls;
        k_vindex_fill<<<grid_blocks_for(vi_count), BT, 0, st>>>(L->vindex, vi_count, fs, ls); GRZ_COUNT_LAUNCH(g);
        LCK(cudaGetLastError());
        k_vindex_heads<<<grid_blocks_for(nvec), BT, 0, st>>>(L->shared, nvec, L->vindex); GRZ_COUNT_LAUNCH(g);
        LCK(cudaGetLastError());
        uint32_t* cnt = nullptr;
        LCK(cudaMallocAsync((void**)&cnt, sizeof(uint32_t) * (V + 1), st));
        LCK(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * (V + 1), st));
        k_row_counts<<<grid_blocks_for(nvec), BT, 0, st>>>(L->shared, nvec, L->vindex, cnt); GRZ_COUNT_LAUNCH(g);
        LCK(cudaGetLastError());
        rc = grz_exclusive_sum_u32(g, cnt, L->rowptr, V + 1, nullptr);
        cudaFreeAsync(cnt, st);
        if (rc) goto done;
    }
done:
    if (flags) cudaFreeAsync(flags, st);
    if (head) cudaFreeAsync(head, st);
    if (vstart) cudaFreeAsync(vstart, st);
    if (vexcl) cudaFreeAsync(vexcl, st);
    if (vfirst) cudaFreeAsync(vfirst, st);
    if (l1) cudaFreeAsync(l1, st);
#undef LCK
    if (rc == GRZ_OK) rc = grz_cuda_check(g, cudaStreamSynchronize(st), "build list");
    return rc;
}

int grz_build_outdegrees(grz_graph* g, const uint64_t* d_pull_pairs, uint64_t E)
{
    const uint64_t V = g->V;
    cudaStream_t st = g->stream;
    int rc = grz_dev_alloc(g, (void**)&g->degree, sizeof(uint32_t) * (V + 1));
    if (!rc) rc = grz_dev_alloc(g, (void**)&g->outdeg, sizeof(double) * (V + 8));
    if (!rc) rc = grz_dev_alloc(g, (void**)&g->inv_deg, sizeof(double) * (V + 1));
    if (rc) return rc;
    GRZ_CK(g, cudaMemsetAsync(g->degree, 0, sizeof(uint32_t) * (V + 1), st));
    GRZ_CK(g, cudaMemsetAsync(g->outdeg, 0, sizeof(double) * (V + 8), st));
    if (E > 0) {
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
