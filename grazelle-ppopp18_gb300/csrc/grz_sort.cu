// grz_sort.cu -- pull-only ingest: the -pull list, the -push list and the outdegrees from the
// -pull pairs alone.
//
// The reference reads two files holding the same edges: -pull sorted by (dst, src) and -push
// sorted by (src, dst) (source/graphdata.c:957-1049).  Given only the -pull pairs, a stable sort
// by source turns them into the -push order: the input is already ascending in dst within every
// source, and a stable sort keeps that.  Duplicate edges are kept, as the reference keeps them.
//
// The pairs are cut into chunks of whole tiles, in input order.  Pairs in pinned host memory
// cross the host link chunk by chunk on the copy engine, into a ring of device slots, while the
// SMs process the chunks already in (pairs in device memory are read in place).  Per chunk, on
// the graph's stream:
// - one pass writes the sort keys (src << 32 | dst: the pairs in half the bytes), the run bounds
//   of every destination (the -pull list's first build step) and the chunk's per-tile histogram
//   of the first radix digit; the slot is then free for a later chunk;
// - the chunk's -pull vectors are written (k_pull_heads, k_pull_write);
// - an LSD radix sort over the source's 8-bit digits sorts the chunk (per pass: per-tile digit
//   histograms, one exclusive scan in (digit, tile) order, and a stable scatter that sorts each
//   tile by digit in shared memory before writing it out);
// - each edge of the sorted chunk gets its rank among its source's edges: the source's edges in
//   earlier chunks (a running count per source, which ends as the outdegree that
//   graphdata.c:792-821 credits) plus its place in the chunk's run of that source.
// Chunks are in input order and each chunk's sort is stable, so an edge's rank is its position
// in the source's (dst, input order) run, exactly what one stable sort of all pairs would give.
// Once every chunk is ranked, the -pull list's offsets and index follow from the run bounds, the
// -push list's offsets come from the outdegrees, and one pass puts every edge into lane (rank) of
// its source's -push vectors.  Only the last chunk's work and these steps follow the link.
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
constexpr uint64_t CHUNK_EDGES = 1ull << 24;  // pairs per ingest chunk by default (GB300 sweep at 520M pairs:
constexpr uint64_t AUTO_CHUNKS_MAX = 64;      // 8 chunks 45.4 ms, 24 43.7, 32-64 43.5; one chunk 65.1)
constexpr int TAIL_SPLITS = 3;                // the last regular chunk is cut into halves, quarters, ...
constexpr uint64_t STAGE_SLOTS = 3;           // device slots the chunks of pinned host pairs are copied into
constexpr uint64_t PLACE_BLOCK_BYTES = 24ull << 20;  // -push vectors per placement block (L2: 126 MB)
constexpr uint64_t PLACE_MAX_BLOCKS = 4096;
constexpr uint64_t PLACE_EDGES_PER_THREAD = 4;
static_assert(ST == RBINS, "the histogram and digit passes give each thread one digit");

// The first pass over one chunk, a block per tile of STILE pairs: chunk holds the chunk's pairs
// (e0 .. e0 + n - 1, in a staging slot or in place), all of them is any pair's device-readable
// address (read only for the two neighbours outside the chunk).  A tile's destinations go through
// shared memory; only the neighbours outside the tile are read again.  hist is the chunk's
// [digit][tile] histogram of the sources' lowest digit.
__global__ void __launch_bounds__(ST) k_ingest(const ulonglong2* __restrict__ chunk, const ulonglong2* __restrict__ all,
                                              uint64_t E, uint64_t V, uint64_t e0, uint64_t n, uint32_t ntiles,
                                              unsigned long long* __restrict__ keys, uint32_t* __restrict__ start,
                                              uint32_t* __restrict__ end, uint32_t* __restrict__ hist, unsigned* __restrict__ flags)
{
    __shared__ unsigned long long s_dst[STILE];
    __shared__ uint32_t cnt[RBINS];
    cnt[threadIdx.x] = 0;
    const uint64_t base = (uint64_t)blockIdx.x * STILE;  // within the chunk
    auto dst_at = [&](uint64_t e) { return e >= e0 && e < e0 + n ? chunk[e - e0].y : all[e].y; };
    ulonglong2 p[SI];
#pragma unroll
    for (int c = 0; c < SI; ++c) {
        const uint64_t i = base + (uint64_t)c * ST + threadIdx.x;
        p[c] = i < n ? chunk[i] : make_ulonglong2(~0ull, ~0ull);
    }
#pragma unroll
    for (int c = 0; c < SI; ++c) s_dst[c * ST + threadIdx.x] = p[c].y;
    __syncthreads();
    bool bad_order = false, bad_range = false;
#pragma unroll
    for (int c = 0; c < SI; ++c) {
        const int i = c * ST + threadIdx.x;
        if (base + i >= n) continue;
        const uint64_t e = e0 + base + i;
        const uint64_t s = p[c].x, d = p[c].y;
        const uint64_t dp = i > 0 ? s_dst[i - 1] : (e > 0 ? dst_at(e - 1) : d);
        const uint64_t dn = i + 1 < STILE ? s_dst[i + 1] : (e + 1 < E ? dst_at(e + 1) : d);
        keys[e] = (s << 32) | (d & 0xffffffffull);
        if (s >= V || d >= V) bad_range = true;
        if (e > 0 && dp > d) bad_order = true;
        const bool head = e == 0 || dp != d;
        const bool tail = e + 1 == E || dn != d;
        if (d < V) {
            if (head) start[d] = (uint32_t)e;
            if (tail) end[d] = (uint32_t)(e + 1);
        }
        // every key, in range or not: the chunk is sorted before the range check is read
        atomicAdd(&cnt[(uint32_t)s & (RBINS - 1)], 1u);
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

// stable scatter of one tile.
// Warp w owns the tile's keys [STILE/8 w, STILE/8 (w+1)) and walks them in rounds of 32 in
// input order.  (1) Each warp counts its digits into its own shared-memory row (digit_peers: one
// leader per digit per round, so no atomics).  (2) One thread per digit turns the rows into
// tile-local positions: the digit's start in the tile (a block scan over the digit totals) plus
// the counts of the warps before.  (3) Each warp places its keys in shared memory at those
// positions (a key's rank: its digit's running count in the warp plus its lane rank among equal
// digits of the round), so the tile sits in shared memory sorted by digit, stably.  (4) The
// block writes the tile out in that order: each digit's keys go to one contiguous run of the
// output, so the stores coalesce.
__global__ void __launch_bounds__(ST) k_sort_scatter(const unsigned long long* __restrict__ keys, uint64_t n, int shift,
                                                     uint32_t ntiles, const uint32_t* __restrict__ offs,
                                                     unsigned long long* __restrict__ keys_out)
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
        keys_out[(uint64_t)s_glob[d] + (i - s_local[d])] = kk;
    }
}

// The -pull list's vectors of one chunk, written while later chunks cross the link.  A
// destination's vectors start at the edges at multiple-of-4 positions of its run (the heads), and
// vector k of the list is the k-th head in input order.  Once a chunk is in, every run start of
// its destinations is known (its runs start in it or in an earlier chunk), so its heads can be
// counted per tile, numbered by a scan plus the heads of the earlier chunks (carry[c]), and
// written; lanes past the chunk's end are read from the pairs.  Thread j of a tile takes its
// edges 8j .. 8j+7.  Destinations >= V (input that fails the range check) and vector numbers
// >= cap (heads of unsorted input) are skipped.
__device__ __forceinline__ bool pull_head(uint32_t d, uint64_t e, uint64_t V, const uint32_t* __restrict__ start)
{
    return d < V && (((uint32_t)e - __ldg(start + d)) & 3u) == 0;
}

__global__ void __launch_bounds__(ST) k_pull_heads(const unsigned long long* __restrict__ keys, uint64_t e0, uint64_t n, uint64_t V,
                                                  const uint32_t* __restrict__ start, uint32_t* __restrict__ tcount)
{
    __shared__ uint32_t wsum[ST / 32];
    const uint64_t first = e0 + (uint64_t)blockIdx.x * STILE + (uint64_t)threadIdx.x * SI;
    uint32_t h = 0;
#pragma unroll
    for (int k = 0; k < SI; ++k) {
        const uint64_t e = first + k;
        if (e < e0 + n) h += pull_head((uint32_t)(keys[e] & 0xffffffffull), e, V, start);
    }
    h = __reduce_add_sync(0xffffffffu, h);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = h;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < ST / 32; ++w) t += wsum[w];
        tcount[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(ST) k_pull_write(const unsigned long long* __restrict__ keys, const ulonglong2* __restrict__ in,
                                                  uint64_t E, uint64_t e0, uint64_t n, uint64_t V,
                                                  const uint32_t* __restrict__ start, const uint32_t* __restrict__ toff,
                                                  const uint32_t* __restrict__ carry, uint64_t cap,
                                                  uint4* __restrict__ nbr, uint32_t* __restrict__ shared)
{
    __shared__ uint32_t wsum[ST / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t first = e0 + (uint64_t)blockIdx.x * STILE + (uint64_t)threadIdx.x * SI;
    const uint64_t chunk_end = e0 + n;
    uint32_t d[SI];
    unsigned hm = 0;
#pragma unroll
    for (int k = 0; k < SI; ++k) {
        const uint64_t e = first + k;
        d[k] = e < chunk_end ? (uint32_t)(keys[e] & 0xffffffffull) : 0xffffffffu;
        if (e < chunk_end && pull_head(d[k], e, V, start)) hm |= 1u << k;
    }
    // exclusive rank of this thread's first head among the tile's heads
    const uint32_t h = __popc(hm);
    uint32_t incl = h;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    uint64_t vec = (uint64_t)__ldg(carry) + __ldg(toff + blockIdx.x) + before + incl - h;
    for (int k = 0; k < SI; ++k) {
        if (!((hm >> k) & 1u)) continue;
        const uint64_t e = first + k;
        if (vec < cap) {
            uint32_t ids[4];
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const uint64_t x = e + l;
                uint32_t src = GRZ_INVALID_ID, dst = 0xffffffffu;
                if (x < chunk_end) {
                    const unsigned long long kk = keys[x];
                    src = (uint32_t)(kk >> 32);
                    dst = (uint32_t)(kk & 0xffffffffull);
                } else if (x < E) {
                    const ulonglong2 pr = in[x];
                    src = (uint32_t)pr.x;
                    dst = pr.y == d[k] ? d[k] : 0xffffffffu;
                }
                ids[l] = dst == d[k] ? src : GRZ_INVALID_ID;
            }
            nbr[vec] = make_uint4(ids[0], ids[1], ids[2], ids[3]);
            shared[vec] = d[k];
        }
        ++vec;
    }
}

// heads of the chunks so far: carry[c + 1] = carry[c] + the chunk's heads
__global__ void k_pull_carry(uint32_t* carry, uint32_t c) { carry[c + 1] += carry[c]; }

// Ranks of a sorted chunk's edges among their sources' edges, in two steps.  run[s]: the
// source's edges in earlier chunks.  At the head p of the chunk's run of s, off[s] = run[s] - p,
// so an edge at p ranks off[s] + p; the tail of the run leaves run[s] = its rank + 1.  Sources
// >= V (a list that fails the range check) are skipped.
__global__ void k_src_heads(const unsigned long long* __restrict__ keys, uint64_t n, uint64_t V,
                            const uint32_t* __restrict__ run, uint32_t* __restrict__ off)
{
    const uint64_t p = (uint64_t)blockIdx.x * ST + threadIdx.x;
    if (p >= n) return;
    const uint32_t s = (uint32_t)(keys[p] >> 32);
    if (s < V && (p == 0 || (uint32_t)(keys[p - 1] >> 32) != s)) off[s] = run[s] - (uint32_t)p;
}

__global__ void k_src_ranks(const unsigned long long* __restrict__ keys, uint64_t n, uint64_t V,
                            const uint32_t* __restrict__ off, uint32_t* __restrict__ rank, uint32_t* __restrict__ run)
{
    const uint64_t p = (uint64_t)blockIdx.x * ST + threadIdx.x;
    if (p >= n) return;
    const uint32_t s = (uint32_t)(keys[p] >> 32);
    if (s >= V) { rank[p] = 0; return; }
    const uint32_t r = off[s] + (uint32_t)p;
    rank[p] = r;
    if (p + 1 == n || (uint32_t)(keys[p + 1] >> 32) != s) run[s] = r + 1;
}

// The placement goes by source blocks: block b holds the sources whose -push vectors start in
// [b nvec / nb, (b + 1) nvec / nb), a region that fits in L2.  seg[c][b] is the first position of
// chunk c's sorted keys whose source lies in block b or later (seg[c][nb] = the chunk's end), so
// the edges of block b from every chunk are placed together and the partial-sector writes of the
// chunks meet in L2 instead of in DRAM.
// the chunks' first edges, passed by value so that no host buffer has to outlive the launch
struct ChunkStarts {
    uint64_t v[GRZ_INGEST_MAX_CHUNKS + TAIL_SPLITS + 2];
};

__global__ void k_chunk_starts(ChunkStarts cs, uint32_t n, uint64_t* __restrict__ out)
{
    const uint32_t i = threadIdx.x;
    if (i < n) out[i] = cs.v[i];
}

__global__ void k_seg_bounds(const unsigned long long* __restrict__ keys, const uint64_t* __restrict__ cstart, uint32_t nchunks,
                             const uint32_t* __restrict__ rowptr, uint64_t V, uint64_t nvec, uint32_t nb,
                             uint64_t* __restrict__ seg)
{
    const uint64_t i = (uint64_t)blockIdx.x * ST + threadIdx.x;
    if (i >= (uint64_t)nchunks * (nb + 1)) return;
    const uint32_t c = (uint32_t)(i / (nb + 1)), b = (uint32_t)(i % (nb + 1));
    const uint64_t lo0 = cstart[c], hi0 = cstart[c + 1];
    if (b == nb) { seg[i] = hi0; return; }
    // first source of the block: the smallest s with rowptr[s] >= b nvec / nb
    const uint64_t target = (uint64_t)b * nvec / nb;
    uint64_t lo = 0, hi = V;
    while (lo < hi) {
        const uint64_t m = (lo + hi) / 2;
        if (rowptr[m] < target) lo = m + 1; else hi = m;
    }
    const uint32_t s0 = (uint32_t)lo;
    // first position of the chunk with source >= s0
    uint64_t a = lo0, z = hi0;
    while (a < z) {
        const uint64_t m = (a + z) / 2;
        if ((uint32_t)(keys[m] >> 32) < s0) a = m + 1; else z = m;
    }
    seg[i] = a;
}

// every edge into lane (rank & 3) of vector (rank >> 2) of its source's -push vectors; the edge in
// lane 0 also writes the vector's shared vertex and marks the lanes past the run invalid.  Block
// (b, c, x) of the grid walks chunk c's part of source block b with stride xs threads.
__global__ void k_push_place(const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ rank,
                             const uint64_t* __restrict__ seg, uint32_t nchunks, uint32_t nb, uint32_t xs,
                             const uint32_t* __restrict__ deg, const uint32_t* __restrict__ rowptr,
                             uint32_t* __restrict__ nbr32, uint32_t* __restrict__ shared)
{
    const uint32_t x = blockIdx.x % xs, c = (blockIdx.x / xs) % nchunks, b = blockIdx.x / (xs * nchunks);
    const uint64_t lo = seg[(uint64_t)c * (nb + 1) + b], hi = seg[(uint64_t)c * (nb + 1) + b + 1];
    for (uint64_t p = lo + (uint64_t)x * ST + threadIdx.x; p < hi; p += (uint64_t)xs * ST) {
        const unsigned long long kk = keys[p];
        const uint32_t s = (uint32_t)(kk >> 32);
        const uint32_t r = rank[p];
        const uint32_t vec = __ldg(rowptr + s) + (r >> 2);
        nbr32[4 * (uint64_t)vec + (r & 3u)] = (uint32_t)(kk & 0xffffffffull);
        if ((r & 3u) == 0) {
            shared[vec] = s;
            const uint32_t left = __ldg(deg + s) - r;  // edges from this lane on, >= 1
            for (uint32_t l = left; l < 4; ++l) nbr32[4 * (uint64_t)vec + l] = GRZ_INVALID_ID;
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

// Both lists and the outdegrees from E > 0 -pull pairs.  pull: their device-readable address
// (device memory, or pinned host memory read over the link); host: their pinned host address, to
// copy them chunk by chunk through staging slots (the copy engine keeps the link busy while the
// SMs process the chunks already in), or null to read pull in place.  Temporaries come from the
// graph's pool; g->pull, g->push and the outdegree arrays must be empty.
int grz_ingest_pull_derive(grz_graph* g, const uint64_t* pull, uint64_t E, const uint64_t* host)
{
    const uint64_t V = g->V;
    cudaStream_t st = g->stream;
    if (E >= 0xffffffffull) return grz_set_error(g, GRZ_ERR_RANGE, "edge count %llu too large (limit 2^32-2)", (unsigned long long)E);
    int passes = 0;
    for (uint64_t v = V ? V - 1 : 0; v; v >>= RBITS) ++passes;
    if (passes == 0) passes = 1;
    const uint64_t ntiles = (E + STILE - 1) / STILE;
    // chunks of whole tiles: by edge count unless tuned
    uint64_t nchunks = g->tune.ingest_chunks;
    if (nchunks == 0) nchunks = std::min<uint64_t>(AUTO_CHUNKS_MAX, std::max<uint64_t>(1, (E + CHUNK_EDGES - 1) / CHUNK_EDGES));
    nchunks = std::min<uint64_t>(nchunks, ntiles);
    const uint64_t tpc = (ntiles + nchunks - 1) / nchunks;  // tiles per chunk
    // chunk c is tiles [ct[c], ct[c + 1]): tpc each, and the rest (at most tpc) in halves, so
    // that the last chunk, whose work follows the link, is small
    uint64_t ct[GRZ_INGEST_MAX_CHUNKS + TAIL_SPLITS + 2];
    nchunks = 0;
    {
        uint64_t t = 0;
        while (ntiles - t > tpc) { ct[nchunks++] = t; t += tpc; }
        uint64_t rest = ntiles - t;
        for (int k = 0; k < TAIL_SPLITS && rest > 1; ++k) {
            const uint64_t piece = (rest + 1) / 2;
            ct[nchunks++] = t;
            t += piece;
            rest -= piece;
        }
        ct[nchunks++] = t;
        ct[nchunks] = ntiles;
    }
    const uint64_t vi_count = V + 64;
    const ulonglong2* all = reinterpret_cast<const ulonglong2*>(pull);
    grz_list* P = &g->pull;
    grz_list* Q = &g->push;
    unsigned long long* kbuf[3] = { nullptr, nullptr, nullptr };  // input-order keys, then the sort's two buffers
    uint32_t *hist = nullptr, *start = nullptr, *end = nullptr, *off = nullptr, *rank = nullptr, *cnt = nullptr, *tot = nullptr;
    uint32_t *heads = nullptr, *carry = nullptr;
    uint64_t* cstart = nullptr;  // first edge of each chunk, and E
    // the -pull list's vectors, numbered as they are written: at most E/4 + one partial vector per destination
    const uint64_t pcap = E / 4 + std::min<uint64_t>(V, E) + 1;
    unsigned* flags = nullptr;
    uint64_t* seg = nullptr;
    unsigned flags_h[2] = { 0, 0 };
    unsigned long long kends[2] = { 0, 0 };
    uint32_t nv32 = 0;
    uint32_t qends[2] = { 0, 0 };
    // ev[c]: chunk c is in its slot; ev[nchunks + c]: its slot is free again; ev[2 nchunks]: set-up done
    cudaEvent_t ev[2 * (GRZ_INGEST_MAX_CHUNKS + TAIL_SPLITS + 1) + 1] = {};
    int nev = 0;
    cudaStream_t cs = nullptr;
    const uint64_t nslots = host ? std::min<uint64_t>(nchunks, STAGE_SLOTS) : 0;
    ulonglong2* slot[STAGE_SLOTS] = {};
    const unsigned long long* sorted = nullptr;
    auto copy_chunk = [&](uint64_t c) -> cudaError_t {
        const uint64_t e0 = ct[c] * STILE, n = std::min<uint64_t>(ct[c + 1] * STILE, E) - e0;
        cudaError_t e = cudaSuccess;
        if (c >= nslots) e = cudaStreamWaitEvent(cs, ev[nchunks + c - nslots], 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(slot[c % nslots], host + 2 * e0, sizeof(ulonglong2) * n, cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess) e = cudaEventRecord(ev[c], cs);
        return e;
    };
    int rc = GRZ_OK;
#define ICK(call) do { cudaError_t e__ = (call); if (e__ != cudaSuccess) { rc = grz_cuda_check(g, e__, #call); goto done; } } while (0)
#define IRC(expr) do { rc = (expr); if (rc) goto done; } while (0)
    for (; nev < 2 * (int)nchunks + 1; ++nev) ICK(cudaEventCreateWithFlags(&ev[nev], cudaEventDisableTiming));
    for (int b = 0; b < 3; ++b)
        if (b < 2 || passes > 1) IRC(grz_dev_alloc(g, (void**)&kbuf[b], sizeof(unsigned long long) * E));
    for (uint64_t r = 0; r < nslots; ++r) IRC(grz_dev_alloc(g, (void**)&slot[r], sizeof(ulonglong2) * tpc * STILE));
    // 1. the first chunks start crossing the link as soon as their slots exist
    if (host) {
        ICK(grz_copy_stream(g));
        cs = g->copy_stream;
        ICK(cudaEventRecord(ev[2 * nchunks], st));  // after the slots' allocation
        ICK(cudaStreamWaitEvent(cs, ev[2 * nchunks], 0));
        for (uint64_t c = 0; c < nslots; ++c) ICK(copy_chunk(c));
    }
    IRC(grz_dev_alloc(g, (void**)&rank, sizeof(uint32_t) * E));
    IRC(grz_dev_alloc(g, (void**)&hist, sizeof(uint32_t) * RBINS * ntiles));
    IRC(grz_dev_alloc(g, (void**)&start, sizeof(uint32_t) * (V + 1)));
    IRC(grz_dev_alloc(g, (void**)&end, sizeof(uint32_t) * (V + 1)));
    IRC(grz_dev_alloc(g, (void**)&off, sizeof(uint32_t) * (V + 1)));
    IRC(grz_dev_alloc(g, (void**)&flags, sizeof(unsigned) * 2));
    IRC(grz_dev_alloc(g, (void**)&heads, sizeof(uint32_t) * ntiles));
    IRC(grz_dev_alloc(g, (void**)&carry, sizeof(uint32_t) * (nchunks + 1)));
    ICK(cudaMallocAsync((void**)&P->nbr, sizeof(uint4) * pcap, st));
    ICK(cudaMallocAsync((void**)&P->shared, sizeof(uint32_t) * pcap, st));
    ICK(cudaMemsetAsync(carry, 0, sizeof(uint32_t) * (nchunks + 1), st));
    IRC(grz_alloc_outdegrees(g));  // g->degree zeroed: the running count per source
    ICK(cudaMemsetAsync(start, 0, sizeof(uint32_t) * (V + 1), st));
    ICK(cudaMemsetAsync(end, 0, sizeof(uint32_t) * (V + 1), st));
    ICK(cudaMemsetAsync(flags, 0, sizeof(unsigned) * 2, st));
    // 2. per chunk, once it is in: the first pass, its -pull vectors, its sort by source and its
    //    edges' ranks; its slot then takes the chunk nslots further on
    for (uint64_t c = 0; c < nchunks; ++c) {
        const uint64_t t0 = ct[c], nt = ct[c + 1] - t0;
        const uint64_t e0 = t0 * STILE, n = std::min<uint64_t>(nt * STILE, E - e0);
        uint32_t* h = hist + RBINS * t0;
        if (host) ICK(cudaStreamWaitEvent(st, ev[c], 0));
        k_ingest<<<(unsigned)nt, ST, 0, st>>>(host ? slot[c % nslots] : all + e0, all, E, V, e0, n, (uint32_t)nt, kbuf[0], start,
                                               end, h, flags); GRZ_COUNT_LAUNCH(g);
        ICK(cudaGetLastError());
        if (host) {
            ICK(cudaEventRecord(ev[nchunks + c], st));
            if (c + nslots < nchunks) ICK(copy_chunk(c + nslots));
        }
        k_pull_heads<<<(unsigned)nt, ST, 0, st>>>(kbuf[0], e0, n, V, start, heads + t0); GRZ_COUNT_LAUNCH(g);
        ICK(cudaGetLastError());
        IRC(grz_exclusive_sum_u32_on(g, heads + t0, heads + t0, nt, carry + c + 1, st));
        k_pull_carry<<<1, 1, 0, st>>>(carry, (uint32_t)c); GRZ_COUNT_LAUNCH(g);
        k_pull_write<<<(unsigned)nt, ST, 0, st>>>(kbuf[0], all, E, e0, n, V, start, heads + t0, carry + c, pcap, P->nbr, P->shared);
        GRZ_COUNT_LAUNCH(g);
        ICK(cudaGetLastError());
        const unsigned long long* in = kbuf[0] + e0;
        int out = 1;
        for (int p = 0; p < passes; ++p) {
            if (p > 0) {
                k_sort_hist<<<(unsigned)nt, ST, 0, st>>>(in, n, p * RBITS, (uint32_t)nt, h); GRZ_COUNT_LAUNCH(g);
                ICK(cudaGetLastError());
            }
            IRC(grz_exclusive_sum_u32_on(g, h, h, (uint64_t)RBINS * nt, nullptr, st));
            k_sort_scatter<<<(unsigned)nt, ST, 0, st>>>(in, n, p * RBITS, (uint32_t)nt, h, kbuf[out] + e0); GRZ_COUNT_LAUNCH(g);
            ICK(cudaGetLastError());
            in = kbuf[out] + e0;
            out = 3 - out;
        }
        k_src_heads<<<blocks_of(n), ST, 0, st>>>(in, n, V, g->degree, off); GRZ_COUNT_LAUNCH(g);
        k_src_ranks<<<blocks_of(n), ST, 0, st>>>(in, n, V, off, rank + e0, g->degree); GRZ_COUNT_LAUNCH(g);
        ICK(cudaGetLastError());
        sorted = in - e0;
    }
    // 3. after the last chunk: the input checks and the -push list's offsets (from the outdegrees,
    //    its run lengths) on the graph's stream
    IRC(grz_dev_alloc(g, (void**)&cnt, sizeof(uint32_t) * (V + 1)));
    IRC(grz_dev_alloc(g, (void**)&tot, sizeof(uint32_t)));
    ICK(cudaMallocAsync((void**)&Q->vindex, sizeof(uint64_t) * vi_count, st));
    ICK(cudaMallocAsync((void**)&Q->rowptr, sizeof(uint32_t) * (V + 1), st));
    ICK(cudaMallocAsync((void**)&P->vindex, sizeof(uint64_t) * vi_count, st));
    ICK(cudaMallocAsync((void**)&P->rowptr, sizeof(uint32_t) * (V + 1), st));
    ICK(cudaMemcpyAsync(flags_h, flags, sizeof(flags_h), cudaMemcpyDeviceToHost, st));
    ICK(cudaMemcpyAsync(&kends[0], kbuf[0], sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    ICK(cudaMemcpyAsync(&kends[1], kbuf[0] + (E - 1), sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    k_run_vectors<<<blocks_of(V + 1), ST, 0, st>>>(g->degree, V, cnt); GRZ_COUNT_LAUNCH(g);
    ICK(cudaGetLastError());
    IRC(grz_exclusive_sum_u32(g, cnt, Q->rowptr, V + 1, tot));
    ICK(cudaMemcpyAsync(&nv32, tot, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    ICK(cudaStreamSynchronize(st));
    if (flags_h[0]) { rc = grz_set_error(g, GRZ_ERR_UNSORTED, "pull list is not grouped by destination in ascending order"); goto done; }
    if (flags_h[1]) { rc = grz_set_error(g, GRZ_ERR_RANGE, "pull list holds a vertex ID >= V (%llu)", (unsigned long long)V); goto done; }
    Q->nvec = nv32;
    ICK(cudaMallocAsync((void**)&Q->nbr, sizeof(uint4) * Q->nvec, st));
    ICK(cudaMallocAsync((void**)&Q->shared, sizeof(uint32_t) * Q->nvec, st));
    {
        const uint64_t nb = std::min<uint64_t>(PLACE_MAX_BLOCKS, std::max<uint64_t>(1, Q->nvec * sizeof(uint4) / PLACE_BLOCK_BYTES));
        const uint64_t per = (E + nb * nchunks - 1) / (nb * nchunks);  // edges per (block, chunk) on average
        const uint64_t xs = std::max<uint64_t>(1, (per + PLACE_EDGES_PER_THREAD * ST - 1) / (PLACE_EDGES_PER_THREAD * ST));
        ChunkStarts cs_h;
        for (uint64_t c = 0; c <= nchunks; ++c) cs_h.v[c] = std::min<uint64_t>(ct[c] * STILE, E);
        IRC(grz_dev_alloc(g, (void**)&seg, sizeof(uint64_t) * nchunks * (nb + 1)));
        IRC(grz_dev_alloc(g, (void**)&cstart, sizeof(uint64_t) * (nchunks + 1)));
        static_assert(GRZ_INGEST_MAX_CHUNKS + TAIL_SPLITS + 2 <= 128, "one block writes the chunk starts");
        k_chunk_starts<<<1, 128, 0, st>>>(cs_h, (uint32_t)(nchunks + 1), cstart); GRZ_COUNT_LAUNCH(g);
        k_seg_bounds<<<blocks_of(nchunks * (nb + 1)), ST, 0, st>>>(sorted, cstart, (uint32_t)nchunks, Q->rowptr, V, Q->nvec,
                                                                  (uint32_t)nb, seg); GRZ_COUNT_LAUNCH(g);
        k_push_place<<<(unsigned)(nb * nchunks * xs), ST, 0, st>>>(sorted, rank, seg, (uint32_t)nchunks, (uint32_t)nb, (uint32_t)xs,
                                                                  g->degree, Q->rowptr, reinterpret_cast<uint32_t*>(Q->nbr),
                                                                  Q->shared); GRZ_COUNT_LAUNCH(g);
        ICK(cudaGetLastError());
    }
    // 4. meanwhile on the second stream: the -pull list's offsets and index (its vectors are
    //    written) and the outdegrees as doubles
    ICK(grz_copy_stream(g));
    cs = g->copy_stream;
    ICK(cudaEventRecord(ev[2 * nchunks], st));
    ICK(cudaStreamWaitEvent(cs, ev[2 * nchunks], 0));
    IRC(grz_build_list_from_bounds(g, P, nullptr, E, 1, start, end, kends[0] & 0xffffffffull, kends[1] & 0xffffffffull, nullptr,
                                   cs, pcap));
    IRC(grz_build_outdegrees(g, nullptr, E, cs));
    // the -push vertex index: its first and last shared vertices are those of its end vectors
    ICK(cudaMemcpyAsync(&qends[0], Q->shared, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    ICK(cudaMemcpyAsync(&qends[1], Q->shared + (Q->nvec - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    ICK(cudaStreamSynchronize(st));
    Q->vindex_start = qends[0];
    Q->vindex_end = qends[1];
    Q->vs = nullptr;
    k_run_vindex<<<blocks_of(vi_count), ST, 0, st>>>(g->degree, Q->rowptr, V, vi_count, qends[1], Q->vindex); GRZ_COUNT_LAUNCH(g);
    ICK(cudaGetLastError());
done:
#undef ICK
#undef IRC
    // the temporaries are freed on the graph's stream once the second stream's work is done too
    if (cs && (cudaEventRecord(g->copy_ev[1], cs) != cudaSuccess || cudaStreamWaitEvent(st, g->copy_ev[1], 0) != cudaSuccess))
        cudaStreamSynchronize(cs);
    for (void* q : { (void*)kbuf[0], (void*)kbuf[1], (void*)kbuf[2], (void*)rank, (void*)hist, (void*)start, (void*)end, (void*)off,
                     (void*)cnt, (void*)tot, (void*)flags, (void*)seg, (void*)heads, (void*)carry, (void*)cstart })
        grz_dev_free(g, q);
    for (void* q : slot) grz_dev_free(g, q);
    for (int i = 0; i < nev; ++i) cudaEventDestroy(ev[i]);
    if (rc == GRZ_OK) rc = grz_cuda_check(g, cudaStreamSynchronize(st), "pull-only ingest");
    else cudaStreamSynchronize(st);
    return rc;
}
