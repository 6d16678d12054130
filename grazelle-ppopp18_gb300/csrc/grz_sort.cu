// grz_sort.cu -- pull-only ingest: the -pull list, the -push list and the outdegrees from the
// -pull pairs alone.
//
// The reference reads two files holding the same edges: -pull sorted by (dst, src) and -push
// sorted by (src, dst) (source/graphdata.c:957-1049).  Given only the -pull pairs, a stable sort
// by source turns them into the -push order: the input is already ascending in dst within every
// source, and a stable sort keeps that.  Duplicate edges are kept, as the reference keeps them.
//
// 1. One fused pass reads the -pull pairs where they are (pinned host memory over the host link,
//    or device memory) and, while the link is the bottleneck, also writes the sort keys
//    (src << 32 | dst, the pairs in half the bytes), the run bounds of every destination (the
//    -pull list's first build step), the per-tile histogram of the first radix digit, and the
//    outdegrees (graphdata.c:792-821 credits the sources of the -pull list).
// 2. The -pull list is finished from the run bounds and the keys (grz_build_list_from_bounds),
//    before the sort permutes them.
// 3. The -push list's offsets come from the outdegrees: its runs are the sources' out-edges.
// 4. LSD radix sort over the source's 8-bit digits (as many passes as V needs): per pass,
//    per-tile digit histograms, one exclusive scan in (digit, tile) order, and a stable scatter
//    that sorts each tile by digit in shared memory before writing it out.  The last pass writes
//    each edge straight into its -push vector lane: its final position p in the (src, dst) order
//    is lane (p - first edge of src) of that source's vectors.
// Stability inside a tile: each warp owns a contiguous eighth of the tile and walks it in input
// order; ballots rank equal digits within a round, and the warps' positions per digit follow
// warp order.
#include "grz_internal.cuh"

namespace {

constexpr int ST = 256;                 // threads per block
constexpr int SI = 8;                   // keys per thread per tile (GB300 sweep of 4-16: 8 fastest)
constexpr int STILE = ST * SI;          // keys per tile
constexpr int RBITS = 8;
constexpr int RBINS = 1 << RBITS;
static_assert(ST == RBINS, "the histogram and digit passes give each thread one digit");

// Step 1 over one tile of STILE pairs.  The tile's destinations go through shared memory so that
// each pair crosses the link once; only the two neighbours outside the tile are read again.
__global__ void __launch_bounds__(ST) k_ingest(const ulonglong2* __restrict__ in, uint64_t E, uint64_t V,
                                              unsigned long long* __restrict__ keys,
                                              uint32_t* __restrict__ start, uint32_t* __restrict__ end,
                                              uint32_t* __restrict__ deg, uint32_t ntiles, uint32_t* __restrict__ hist,
                                              unsigned* __restrict__ flags)
{
    __shared__ unsigned long long s_dst[STILE];
    __shared__ uint32_t cnt[RBINS];
    cnt[threadIdx.x] = 0;
    const uint64_t base = (uint64_t)blockIdx.x * STILE;
    ulonglong2 p[SI];
#pragma unroll
    for (int c = 0; c < SI; ++c) {
        const uint64_t e = base + (uint64_t)c * ST + threadIdx.x;
        p[c] = e < E ? in[e] : make_ulonglong2(~0ull, ~0ull);
    }
#pragma unroll
    for (int c = 0; c < SI; ++c) s_dst[c * ST + threadIdx.x] = p[c].y;
    __syncthreads();
    bool bad_order = false, bad_range = false;
#pragma unroll
    for (int c = 0; c < SI; ++c) {
        const int i = c * ST + threadIdx.x;
        const uint64_t e = base + (uint64_t)i;
        if (e >= E) continue;
        const uint64_t s = p[c].x, d = p[c].y;
        const uint64_t dp = i > 0 ? s_dst[i - 1] : (e > 0 ? in[e - 1].y : d);
        const uint64_t dn = i + 1 < STILE ? s_dst[i + 1] : (e + 1 < E ? in[e + 1].y : d);
        keys[e] = (s << 32) | (d & 0xffffffffull);
        if (s >= V || d >= V) bad_range = true;
        if (e > 0 && dp > d) bad_order = true;
        const bool head = e == 0 || dp != d;
        const bool tail = e + 1 == E || dn != d;
        if (d < V) {
            if (head) start[d] = (uint32_t)e;
            if (tail) end[d] = (uint32_t)(e + 1);
        }
        if (s < V) {
            atomicAdd(&cnt[(uint32_t)s & (RBINS - 1)], 1u);
            atomicAdd(deg + s, 1u);
        }
    }
    if (bad_order) atomicOr(&flags[0], 1u);
    if (bad_range) atomicOr(&flags[1], 1u);
    __syncthreads();
    hist[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(ST) k_sort_hist(const unsigned long long* __restrict__ keys, uint64_t n, int shift,
                                                  uint32_t ntiles, uint32_t* __restrict__ hist)
{
    __shared__ uint32_t cnt[RBINS];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * STILE;
#pragma unroll 4
    for (int i = 0; i < SI; ++i) {
        const uint64_t k = base + (uint64_t)i * ST + threadIdx.x;
        if (k < n) atomicAdd(&cnt[(uint32_t)(keys[k] >> (32 + shift)) & (RBINS - 1)], 1u);
    }
    __syncthreads();
    hist[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

// lanes of the warp whose digit equals this lane's (dead lanes form their own group): one ballot
// per digit bit
__device__ __forceinline__ unsigned digit_peers(uint32_t d, bool live)
{
    const unsigned lv = __ballot_sync(0xffffffffu, live);
    unsigned m = live ? lv : ~lv;
#pragma unroll
    for (int b = 0; b < RBITS; ++b) {
        const bool bit = (d >> b) & 1u;
        const unsigned bb = __ballot_sync(0xffffffffu, bit);
        m &= bit ? bb : ~bb;
    }
    return m;
}

// Where the last pass puts an edge: lane (p - pstart[src]) of the source's -push vectors.
struct PushOut {
    uint32_t* nbr32;         // the -push list's neighbour lanes (pre-filled with GRZ_INVALID_ID)
    uint32_t* shared;        // shared vertex of each -push vector
    const uint32_t* pstart;  // first (src, dst)-order position of each source
    const uint32_t* prowptr; // first vector of each source
};

// stable scatter of one tile (ToVectors: the last pass, into the -push vectors).
// Warp w owns the tile's keys [STILE/8 w, STILE/8 (w+1)) and walks them in rounds of 32 in
// input order.  (1) Each warp counts its digits into its own shared-memory row (digit_peers: one
// leader per digit per round, so no atomics).  (2) One thread per digit turns the rows into
// tile-local positions: the digit's start in the tile (a block scan over the digit totals) plus
// the counts of the warps before.  (3) Each warp places its keys in shared memory at those
// positions (a key's rank: its digit's running count in the warp plus its lane rank among equal
// digits of the round), so the tile sits in shared memory sorted by digit, stably.  (4) The
// block writes the tile out in that order: each digit's keys go to one contiguous run of the
// output, so the stores coalesce.
template <bool ToVectors>
__global__ void __launch_bounds__(ST) k_sort_scatter(const unsigned long long* __restrict__ keys, uint64_t n, int shift,
                                                     uint32_t ntiles, const uint32_t* __restrict__ offs,
                                                     unsigned long long* __restrict__ keys_out, const PushOut po)
{
    constexpr int NW = ST / 32;
    __shared__ unsigned long long s_keys[STILE];
    __shared__ uint32_t wrun[NW][RBINS];
    __shared__ uint32_t s_local[RBINS];   // digit's first position in the tile
    __shared__ uint32_t s_glob[RBINS];    // digit's first position in the output (this tile's share)
    __shared__ uint32_t s_wsum[NW];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < NW * RBINS; i += ST) (&wrun[0][0])[i] = 0;
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    const uint64_t tile0 = (uint64_t)blockIdx.x * STILE;
    const uint32_t tcount = n - tile0 < (uint64_t)STILE ? (uint32_t)(n - tile0) : (uint32_t)STILE;
    const uint64_t base = tile0 + (uint64_t)warp * (SI * 32);
    unsigned long long key[SI];
    unsigned peers[SI];
#pragma unroll
    for (int c = 0; c < SI; ++c) {
        const uint64_t k = base + (uint64_t)c * 32 + lane;
        key[c] = k < n ? keys[k] : 0ull;
    }
#pragma unroll
    for (int c = 0; c < SI; ++c) {
        const bool live = base + (uint64_t)c * 32 + lane < n;
        const uint32_t d = (uint32_t)(key[c] >> (32 + shift)) & (RBINS - 1);
        peers[c] = digit_peers(d, live);
        if (live && (peers[c] & lt) == 0) wrun[warp][d] += __popc(peers[c]);
        __syncwarp();
    }
    __syncthreads();
    // (2) thread d owns digit d
    {
        const int d = threadIdx.x;
        uint32_t tot = 0;
        for (int w = 0; w < NW; ++w) tot += wrun[w][d];
        uint32_t incl = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) s_wsum[warp] = incl;
        __syncthreads();
        uint32_t before = 0;
        for (int w = 0; w < warp; ++w) before += s_wsum[w];
        const uint32_t local = before + incl - tot;
        s_local[d] = local;
        s_glob[d] = offs[(uint64_t)d * ntiles + blockIdx.x];
        uint32_t run = local;
        for (int w = 0; w < NW; ++w) {
            const uint32_t c = wrun[w][d];
            wrun[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
    // (3) place the keys, stably, in digit order
#pragma unroll
    for (int c = 0; c < SI; ++c) {
        const bool live = base + (uint64_t)c * 32 + lane < n;
        const uint32_t d = (uint32_t)(key[c] >> (32 + shift)) & (RBINS - 1);
        uint32_t b0 = 0;
        if (live && (peers[c] & lt) == 0) {
            b0 = wrun[warp][d];
            wrun[warp][d] = b0 + __popc(peers[c]);
        }
        b0 = __shfl_sync(0xffffffffu, b0, __ffs(peers[c]) - 1);
        __syncwarp();
        if (live) s_keys[b0 + __popc(peers[c] & lt)] = key[c];
    }
    __syncthreads();
    // (4) write out in digit order: consecutive positions of one digit are consecutive outputs
    for (uint32_t i = threadIdx.x; i < tcount; i += ST) {
        const unsigned long long kk = s_keys[i];
        const uint32_t d = (uint32_t)(kk >> (32 + shift)) & (RBINS - 1);
        const uint64_t dest = (uint64_t)s_glob[d] + (i - s_local[d]);
        if (ToVectors) {
            const uint32_t src = (uint32_t)(kk >> 32);
            const uint32_t q = (uint32_t)dest - __ldg(po.pstart + src);
            const uint32_t vec = __ldg(po.prowptr + src) + (q >> 2);
            po.nbr32[4 * (uint64_t)vec + (q & 3u)] = (uint32_t)(kk & 0xffffffffull);
            if ((q & 3u) == 0) po.shared[vec] = src;
        } else {
            keys_out[dest] = kk;
        }
    }
}

// vectors of each source's run (entry V is 0 for the exclusive scan's total)
__global__ void k_run_vectors(const uint32_t* __restrict__ deg, uint64_t V, uint32_t* __restrict__ cnt)
{
    const uint64_t v = (uint64_t)blockIdx.x * ST + threadIdx.x;
    if (v < V) cnt[v] = (deg[v] + 3u) / 4u;
    else if (v == V) cnt[v] = 0;
}

// the reference vertex index of a list whose runs are `deg` (graphdata.c:219-267)
__global__ void k_run_vindex(const uint32_t* __restrict__ deg, const uint32_t* __restrict__ rowptr, uint64_t V, uint64_t count,
                             uint64_t last_shared, uint64_t* __restrict__ vindex)
{
    const uint64_t i = (uint64_t)blockIdx.x * ST + threadIdx.x;
    if (i >= count) return;
    if (i < V && deg[i] > 0) vindex[i] = rowptr[i];
    else vindex[i] = (i > last_shared) ? 0xffffffffffffffffull : 0x7fffffffffffffffull;
}

inline unsigned blocks_of(uint64_t n) { return (unsigned)((n + ST - 1) / ST); }

}  // namespace

// Both lists and the outdegrees from E > 0 -pull pairs at `pull` (pinned host memory or device
// memory).  Temporaries come from the graph's pool; g->pull, g->push and the outdegree arrays
// must be empty.
int grz_ingest_pull_derive(grz_graph* g, const uint64_t* pull, uint64_t E)
{
    const uint64_t V = g->V;
    cudaStream_t st = g->stream;
    if (E >= 0xffffffffull) return grz_set_error(g, GRZ_ERR_RANGE, "edge count %llu too large (limit 2^32-2)", (unsigned long long)E);
    int passes = 0;
    for (uint64_t v = V ? V - 1 : 0; v; v >>= RBITS) ++passes;
    if (passes == 0) passes = 1;
    const uint32_t ntiles = (uint32_t)((E + STILE - 1) / STILE);
    const uint64_t vi_count = V + 64;
    grz_list* P = &g->pull;
    grz_list* Q = &g->push;
    unsigned long long *ka = nullptr, *kb = nullptr;
    uint32_t *hist = nullptr, *start = nullptr, *end = nullptr, *pstart = nullptr, *cnt = nullptr, *tot = nullptr;
    unsigned* flags = nullptr;
    unsigned flags_h[2] = { 0, 0 };
    uint64_t ends_h[2] = { 0, 0 };
    uint32_t nv32 = 0;
    uint32_t qends[2] = { 0, 0 };
    int rc = GRZ_OK;
#define ICK(call) do { cudaError_t e__ = (call); if (e__ != cudaSuccess) { rc = grz_cuda_check(g, e__, #call); goto done; } } while (0)
#define IRC(expr) do { rc = (expr); if (rc) goto done; } while (0)
    IRC(grz_dev_alloc(g, (void**)&ka, sizeof(unsigned long long) * E));
    if (passes > 1) IRC(grz_dev_alloc(g, (void**)&kb, sizeof(unsigned long long) * E));
    IRC(grz_dev_alloc(g, (void**)&hist, sizeof(uint32_t) * RBINS * (uint64_t)ntiles));
    IRC(grz_dev_alloc(g, (void**)&start, sizeof(uint32_t) * (V + 1)));
    IRC(grz_dev_alloc(g, (void**)&end, sizeof(uint32_t) * (V + 1)));
    IRC(grz_dev_alloc(g, (void**)&flags, sizeof(unsigned) * 2));
    IRC(grz_alloc_outdegrees(g));  // g->degree zeroed
    ICK(cudaMemsetAsync(start, 0, sizeof(uint32_t) * (V + 1), st));
    ICK(cudaMemsetAsync(end, 0, sizeof(uint32_t) * (V + 1), st));
    ICK(cudaMemsetAsync(flags, 0, sizeof(unsigned) * 2, st));
    // 1. the fused pass over the pairs
    k_ingest<<<ntiles, ST, 0, st>>>(reinterpret_cast<const ulonglong2*>(pull), E, V, ka, start, end, g->degree, ntiles,
                                    hist, flags); GRZ_COUNT_LAUNCH(g);
    ICK(cudaGetLastError());
    {
        unsigned long long kends[2] = { 0, 0 };
        ICK(cudaMemcpyAsync(flags_h, flags, sizeof(flags_h), cudaMemcpyDeviceToHost, st));
        ICK(cudaMemcpyAsync(&kends[0], ka, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        ICK(cudaMemcpyAsync(&kends[1], ka + (E - 1), sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        ICK(cudaStreamSynchronize(st));
        ends_h[0] = kends[0] & 0xffffffffull;  // first and last destination
        ends_h[1] = kends[1] & 0xffffffffull;
        if (flags_h[0]) { rc = grz_set_error(g, GRZ_ERR_UNSORTED, "pull list is not grouped by destination in ascending order"); goto done; }
        if (flags_h[1]) { rc = grz_set_error(g, GRZ_ERR_RANGE, "pull list holds a vertex ID >= V (%llu)", (unsigned long long)V); goto done; }
        // 2. the -pull list from its run bounds
        ICK(cudaMallocAsync((void**)&P->vindex, sizeof(uint64_t) * vi_count, st));
        ICK(cudaMallocAsync((void**)&P->rowptr, sizeof(uint32_t) * (V + 1), st));
        IRC(grz_build_list_from_bounds(g, P, nullptr, E, 1, start, end, ends_h[0], ends_h[1], nullptr, ka));
    }
    // 3. the -push list's offsets from the outdegrees
    IRC(grz_dev_alloc(g, (void**)&pstart, sizeof(uint32_t) * (V + 1)));
    IRC(grz_dev_alloc(g, (void**)&cnt, sizeof(uint32_t) * (V + 1)));
    IRC(grz_dev_alloc(g, (void**)&tot, sizeof(uint32_t)));
    ICK(cudaMallocAsync((void**)&Q->vindex, sizeof(uint64_t) * vi_count, st));
    ICK(cudaMallocAsync((void**)&Q->rowptr, sizeof(uint32_t) * (V + 1), st));
    IRC(grz_exclusive_sum_u32(g, g->degree, pstart, V + 1, nullptr));
    k_run_vectors<<<blocks_of(V + 1), ST, 0, st>>>(g->degree, V, cnt); GRZ_COUNT_LAUNCH(g);
    ICK(cudaGetLastError());
    IRC(grz_exclusive_sum_u32(g, cnt, Q->rowptr, V + 1, tot));
    ICK(cudaMemcpyAsync(&nv32, tot, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    ICK(cudaStreamSynchronize(st));
    Q->nvec = nv32;
    ICK(cudaMallocAsync((void**)&Q->nbr, sizeof(uint4) * Q->nvec, st));
    ICK(cudaMallocAsync((void**)&Q->shared, sizeof(uint32_t) * Q->nvec, st));
    ICK(cudaMemsetAsync(Q->nbr, 0xff, sizeof(uint4) * Q->nvec, st));
    // 4. the sort; its last pass fills the -push vectors
    {
        PushOut po;
        po.nbr32 = reinterpret_cast<uint32_t*>(Q->nbr);
        po.shared = Q->shared;
        po.pstart = pstart;
        po.prowptr = Q->rowptr;
        for (int p = 0; p < passes; ++p) {
            const int shift = p * RBITS;
            if (p > 0) {
                k_sort_hist<<<ntiles, ST, 0, st>>>(ka, E, shift, ntiles, hist); GRZ_COUNT_LAUNCH(g);
                ICK(cudaGetLastError());
            }
            IRC(grz_exclusive_sum_u32(g, hist, hist, (uint64_t)RBINS * ntiles, nullptr));
            if (p + 1 == passes) {
                k_sort_scatter<true><<<ntiles, ST, 0, st>>>(ka, E, shift, ntiles, hist, nullptr, po); GRZ_COUNT_LAUNCH(g);
            } else {
                k_sort_scatter<false><<<ntiles, ST, 0, st>>>(ka, E, shift, ntiles, hist, kb, po); GRZ_COUNT_LAUNCH(g);
            }
            ICK(cudaGetLastError());
            unsigned long long* t = ka;
            ka = kb;
            kb = t;
        }
    }
    // the -push vertex index: its first and last shared vertices are those of its end vectors
    ICK(cudaMemcpyAsync(&qends[0], Q->shared, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    ICK(cudaMemcpyAsync(&qends[1], Q->shared + (Q->nvec - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    ICK(cudaStreamSynchronize(st));
    Q->vindex_start = qends[0];
    Q->vindex_end = qends[1];
    Q->vs = nullptr;
    k_run_vindex<<<blocks_of(vi_count), ST, 0, st>>>(g->degree, Q->rowptr, V, vi_count, qends[1], Q->vindex); GRZ_COUNT_LAUNCH(g);
    ICK(cudaGetLastError());
    IRC(grz_build_outdegrees(g, nullptr, E));
done:
#undef ICK
#undef IRC
    grz_dev_free(g, ka);
    grz_dev_free(g, kb);
    for (void* q : { (void*)hist, (void*)start, (void*)end, (void*)pstart, (void*)cnt, (void*)tot, (void*)flags })
        grz_dev_free(g, q);
    if (rc == GRZ_OK) rc = grz_cuda_check(g, cudaStreamSynchronize(st), "pull-only ingest");
    return rc;
}
