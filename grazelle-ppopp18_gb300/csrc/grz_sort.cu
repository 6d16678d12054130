// grz_sort.cu -- the -push edge list derived on the device from the -pull list.
//
// The reference reads two files holding the same edges: -pull sorted by (dst, src) and -push
// sorted by (src, dst) (source/graphdata.c:957-1049).  Given only the -pull pairs, a stable sort
// by source turns them into the -push order: the input is already ascending in dst within every
// source, and a stable sort keeps that.  Duplicate edges are kept, as the reference keeps them.
//
// LSD radix sort over the source's 8-bit digits (as many passes as V needs), keys packed as
// (src << 32 | dst).  Per pass: per-tile digit histograms, one exclusive scan over the histogram
// in (digit, tile) order, and a stable scatter that sorts each tile by digit in shared memory
// before writing it out (each digit's keys of a tile form one contiguous output run).
// Stability inside a tile: each warp owns a contiguous eighth of the tile and walks it in input
// order; __match_any_sync ranks equal digits within a round, and the warps' positions per digit
// follow warp order.  The last pass writes the interleaved 64-bit (src, dst) pairs the layout
// builder reads.
#include "grz_internal.cuh"

namespace {

constexpr int ST = 256;                 // threads per block
constexpr int SI = 8;                   // keys per thread per tile (GB300 sweep of 4-16: 8 fastest)
constexpr int STILE = ST * SI;          // keys per tile
constexpr int RBITS = 8;
constexpr int RBINS = 1 << RBITS;
static_assert(ST == RBINS, "the scatter's digit pass gives each thread one digit");

__global__ void k_pack_keys(const uint64_t* __restrict__ pairs, uint64_t E, unsigned long long* __restrict__ keys)
{
    const uint64_t e = (uint64_t)blockIdx.x * ST + threadIdx.x;
    if (e < E) keys[e] = (pairs[2 * e] << 32) | (pairs[2 * e + 1] & 0xffffffffull);
}

__global__ void __launch_bounds__(ST) k_sort_hist(const unsigned long long* __restrict__ keys, uint64_t n, int shift,
                                                  uint32_t ntiles, uint32_t* __restrict__ hist)
{
    __shared__ uint32_t cnt[RBINS];
    for (int b = threadIdx.x; b < RBINS; b += ST) cnt[b] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * STILE;
#pragma unroll 4
    for (int i = 0; i < SI; ++i) {
        const uint64_t k = base + (uint64_t)i * ST + threadIdx.x;
        if (k < n) atomicAdd(&cnt[(uint32_t)(keys[k] >> (32 + shift)) & (RBINS - 1)], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < RBINS; b += ST) hist[(uint64_t)b * ntiles + blockIdx.x] = cnt[b];
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

// stable scatter of one tile; `pairs_out` (last pass) gets interleaved (src, dst) uint64 pairs.
// Warp w owns the tile's keys [512 w, 512 w + 512) and walks them in rounds of 32 in input
// order.  (1) Each warp counts its digits into its own shared-memory row (digit_peers: one
// leader per digit per round, so no atomics).  (2) One thread per digit turns the rows into tile-local
// positions: the digit's start in the tile (a block scan over the digit totals) plus the counts
// of the warps before.  (3) Each warp places its keys in shared memory at those positions (a
// key's rank: its digit's running count in the warp plus its lane rank among equal digits of
// the round), so the tile sits in shared memory sorted by digit, stably.  (4) The block writes
// the tile out in that order: each digit's keys go to one contiguous run of the output, so the
// stores coalesce.
__global__ void __launch_bounds__(ST) k_sort_scatter(const unsigned long long* __restrict__ keys, uint64_t n, int shift,
                                                     uint32_t ntiles, const uint32_t* __restrict__ offs,
                                                     unsigned long long* __restrict__ keys_out, uint64_t* __restrict__ pairs_out)
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
        const bool live = k < n;
        key[c] = live ? keys[k] : 0ull;
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
    // (2) ST == RBINS: thread d owns digit d
    {
        const int d = threadIdx.x;
        uint32_t tot = 0;
        for (int w = 0; w < NW; ++w) tot += wrun[w][d];
        // exclusive block scan of the digit totals
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
        if (pairs_out) {
            reinterpret_cast<ulonglong2*>(pairs_out)[dest] = make_ulonglong2(kk >> 32, kk & 0xffffffffull);
        } else {
            keys_out[dest] = kk;
        }
    }
}

}  // namespace

// pull_pairs (device, E interleaved (src, dst) in (dst, src) order) -> push_out (device, the same
// edges in (src, dst) order).  Temporaries come from the graph's pool.
int grz_derive_push_pairs(grz_graph* g, const uint64_t* pull_pairs, uint64_t E, uint64_t* push_out)
{
    if (E == 0) return GRZ_OK;
    if (E >= 0xffffffffull) return grz_set_error(g, GRZ_ERR_RANGE, "edge count too large to sort");
    cudaStream_t st = g->stream;
    int passes = 0;
    for (uint64_t v = g->V ? g->V - 1 : 0; v; v >>= RBITS) ++passes;
    if (passes == 0) passes = 1;
    const uint32_t ntiles = (uint32_t)((E + STILE - 1) / STILE);
    unsigned long long *ka = nullptr, *kb = nullptr;
    uint32_t* hist = nullptr;
    int rc = grz_dev_alloc(g, (void**)&ka, sizeof(unsigned long long) * E);
    if (!rc && passes > 1) rc = grz_dev_alloc(g, (void**)&kb, sizeof(unsigned long long) * E);
    if (!rc) rc = grz_dev_alloc(g, (void**)&hist, sizeof(uint32_t) * RBINS * (uint64_t)ntiles);
    if (!rc) {
        k_pack_keys<<<(unsigned)((E + ST - 1) / ST), ST, 0, st>>>(pull_pairs, E, ka); GRZ_COUNT_LAUNCH(g);
        rc = grz_cuda_check(g, cudaGetLastError(), "pack keys");
    }
    for (int p = 0; p < passes && !rc; ++p) {
        const int shift = p * RBITS;
        k_sort_hist<<<ntiles, ST, 0, st>>>(ka, E, shift, ntiles, hist); GRZ_COUNT_LAUNCH(g);
        rc = grz_cuda_check(g, cudaGetLastError(), "sort histogram");
        if (!rc) rc = grz_exclusive_sum_u32(g, hist, hist, (uint64_t)RBINS * ntiles, nullptr);
        if (rc) break;
        const bool last = p + 1 == passes;
        k_sort_scatter<<<ntiles, ST, 0, st>>>(ka, E, shift, ntiles, hist, last ? nullptr : kb, last ? push_out : nullptr); GRZ_COUNT_LAUNCH(g);
        rc = grz_cuda_check(g, cudaGetLastError(), "sort scatter");
        unsigned long long* t = ka;
        ka = kb;
        kb = t;
    }
    grz_dev_free(g, ka);
    grz_dev_free(g, kb);
    grz_dev_free(g, hist);
    return rc;
}
