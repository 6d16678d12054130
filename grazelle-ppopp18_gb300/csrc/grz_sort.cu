// grz_sort.cu -- the -push edge list derived on the device from the -pull list.
//
// The reference reads two files holding the same edges: -pull sorted by (dst, src) and -push
// sorted by (src, dst) (source/graphdata.c:957-1049).  Given only the -pull pairs, a stable sort
// by source turns them into the -push order: the input is already ascending in dst within every
// source, and a stable sort keeps that.  Duplicate edges are kept, as the reference keeps them.
//
// LSD radix sort over the source's 8-bit digits (as many passes as V needs), keys packed as
// (src << 32 | dst).  Per pass: per-tile digit histograms, one exclusive scan over the histogram
// in (digit, tile) order, and a stable scatter.  Stability inside a tile: the tile is walked in
// chunks of 256 keys in input order; within a warp, __match_any_sync ranks equal digits; across
// the warps of a chunk, the warps take their offsets from per-digit shared counters in warp
// order.  The last pass writes the interleaved 64-bit (src, dst) pairs the layout builder reads.
#include "grz_internal.cuh"

namespace {

constexpr int ST = 256;                 // threads per block
constexpr int SI = 16;                  // keys per thread per tile
constexpr int STILE = ST * SI;          // keys per tile
constexpr int RBITS = 8;
constexpr int RBINS = 1 << RBITS;

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

// stable scatter of one tile; `pairs_out` (last pass) gets interleaved (src, dst) uint64 pairs
__global__ void __launch_bounds__(ST) k_sort_scatter(const unsigned long long* __restrict__ keys, uint64_t n, int shift,
                                                     uint32_t ntiles, const uint32_t* __restrict__ offs,
                                                     unsigned long long* __restrict__ keys_out, uint64_t* __restrict__ pairs_out)
{
    __shared__ uint32_t run[RBINS];   // keys of each digit already placed from this tile
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int b = threadIdx.x; b < RBINS; b += ST) run[b] = offs[(uint64_t)b * ntiles + blockIdx.x];
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    const uint64_t base = (uint64_t)blockIdx.x * STILE;
    for (int c = 0; c < SI; ++c) {
        const uint64_t k = base + (uint64_t)c * ST + threadIdx.x;
        const bool live = k < n;
        const unsigned long long key = live ? keys[k] : 0ull;
        const uint32_t digit = live ? ((uint32_t)(key >> (32 + shift)) & (RBINS - 1)) : RBINS;  // dead lanes: own group
        const unsigned peers = __match_any_sync(0xffffffffu, digit);
        const uint32_t rank = __popc(peers & lt);
        const bool leader = (peers & lt) == 0;
        uint32_t dest = 0;
        // warps of the chunk take their offsets in warp order (input order)
        for (int w = 0; w < ST / 32; ++w) {
            if (warp == w) {
                uint32_t b0 = 0;
                if (leader && live) {
                    b0 = run[digit];
                    run[digit] = b0 + __popc(peers);
                }
                b0 = __shfl_sync(0xffffffffu, b0, __ffs(peers) - 1);
                dest = b0 + rank;
            }
            __syncthreads();
        }
        if (live) {
            if (pairs_out) {
                pairs_out[2 * (uint64_t)dest] = key >> 32;
                pairs_out[2 * (uint64_t)dest + 1] = key & 0xffffffffull;
            } else {
                keys_out[dest] = key;
            }
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
