// grz_scan.cu -- device-wide scans over uint32 arrays (reduce-then-scan, no inter-block waits).
//
// Used by the on-device layout builder: run starts (inclusive max), vector numbering and CSR
// row pointers (exclusive sum).  Three passes: per-tile reduction, scan of the tile totals
// (recursively), per-tile scan seeded with the tile's offset.  Memory-bound; it runs once per
// graph load.
#include "grz_internal.cuh"

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // 4096 elements per block

struct OpSum {
    __device__ static uint32_t id() { return 0u; }
    __device__ static uint32_t op(uint32_t a, uint32_t b) { return a + b; }
};
struct OpMax {
    __device__ static uint32_t id() { return 0u; }
    __device__ static uint32_t op(uint32_t a, uint32_t b) { return a > b ? a : b; }
};

template <class Op>
__device__ uint32_t block_reduce(uint32_t v, uint32_t* sm)
{
    for (int o = 16; o > 0; o >>= 1) v = Op::op(v, __shfl_down_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sm[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (l < SCAN_THREADS / 32) ? sm[l] : Op::id();
        for (int o = 16; o > 0; o >>= 1) v = Op::op(v, __shfl_down_sync(0xffffffffu, v, o));
    }
    return v;
}

// exclusive block scan of one value per thread; returns the thread's exclusive prefix
template <class Op>
__device__ uint32_t block_exclusive(uint32_t v, uint32_t* sm, uint32_t* total)
{
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (l >= o) x = Op::op(y, x);
    }
    if (l == 31) sm[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t s = (l < SCAN_THREADS / 32) ? sm[l] : Op::id();
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (l >= o) s = Op::op(y, s);
        }
        if (l < SCAN_THREADS / 32) sm[l] = s;  // inclusive warp totals
    }
    __syncthreads();
    const uint32_t warp_prefix = w ? sm[w - 1] : Op::id();
    const uint32_t incl = Op::op(warp_prefix, x);
    uint32_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (l == 0) excl = warp_prefix;
    if (total) *total = sm[SCAN_THREADS / 32 - 1];
    return excl;
}

template <class Op>
__global__ void k_tile_reduce(const uint32_t* __restrict__ in, uint64_t n, uint32_t* __restrict__ tile_tot)
{
    __shared__ uint32_t sm[32];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    uint32_t v = Op::id();
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        const uint64_t k = base + (uint64_t)i * SCAN_THREADS + threadIdx.x;
        if (k < n) v = Op::op(v, in[k]);
    }
    v = block_reduce<Op>(v, sm);
    if (threadIdx.x == 0) tile_tot[blockIdx.x] = v;
}

// scans a tile; each thread owns SCAN_ITEMS consecutive elements.  The tile moves between global
// and shared memory in striped order (coalesced), and each thread works on its consecutive items
// in shared memory.
template <class Op, bool Inclusive>
__global__ void __launch_bounds__(SCAN_THREADS) k_tile_scan(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                            uint64_t n, const uint32_t* __restrict__ tile_off,
                                                            uint32_t* __restrict__ grand_total)
{
    __shared__ uint32_t sm[32];
    __shared__ uint32_t tile[SCAN_TILE + SCAN_TILE / 32];  // one pad word per 32 against bank conflicts
    const uint64_t tbase = (uint64_t)blockIdx.x * SCAN_TILE;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        const uint32_t e = (uint32_t)i * SCAN_THREADS + threadIdx.x;
        const uint64_t k = tbase + e;
        tile[e + (e >> 5)] = (k < n) ? in[k] : Op::id();
    }
    __syncthreads();
    uint32_t v[SCAN_ITEMS];
    uint32_t acc = Op::id();
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        const uint32_t e = threadIdx.x * SCAN_ITEMS + i;
        v[i] = tile[e + (e >> 5)];
        acc = Op::op(acc, v[i]);
    }
    uint32_t tot;
    uint32_t run = block_exclusive<Op>(acc, sm, &tot);
    if (tile_off) run = Op::op(tile_off[blockIdx.x], run);
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        const uint32_t e = threadIdx.x * SCAN_ITEMS + i;
        const uint32_t nxt = Op::op(run, v[i]);
        tile[e + (e >> 5)] = Inclusive ? nxt : run;
        run = nxt;
    }
    if (grand_total && threadIdx.x == SCAN_THREADS - 1 && blockIdx.x == gridDim.x - 1) *grand_total = run;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        const uint32_t e = (uint32_t)i * SCAN_THREADS + threadIdx.x;
        const uint64_t k = tbase + e;
        if (k < n) out[k] = tile[e + (e >> 5)];
    }
}

template <class Op, bool Inclusive>
int scan_impl(grz_graph* g, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total_dev, cudaStream_t st)
{
    if (n == 0) {
        if (total_dev) GRZ_CK(g, cudaMemsetAsync(total_dev, 0, sizeof(uint32_t), st));
        return GRZ_OK;
    }
    const uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 1) {
        k_tile_scan<Op, Inclusive><<<1, SCAN_THREADS, 0, st>>>(in, out, n, nullptr, total_dev);
        return grz_cuda_check(g, cudaGetLastError(), "k_tile_scan");
    }
    uint32_t* tot = nullptr;
    GRZ_CK(g, cudaMallocAsync((void**)&tot, sizeof(uint32_t) * (2 * tiles + 1), st));
    uint32_t* off = tot + tiles;
    k_tile_reduce<Op><<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(in, n, tot);
    int rc = grz_cuda_check(g, cudaGetLastError(), "k_tile_reduce");
    if (rc == GRZ_OK) rc = scan_impl<Op, false>(g, tot, off, tiles, nullptr, st);
    if (rc == GRZ_OK) {
        k_tile_scan<Op, Inclusive><<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(in, out, n, off, total_dev);
        rc = grz_cuda_check(g, cudaGetLastError(), "k_tile_scan");
    }
    cudaFreeAsync(tot, st);
    return rc;
}

}  // namespace

int grz_exclusive_sum_u32(grz_graph* g, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total_out_dev)
{
    return scan_impl<OpSum, false>(g, in, out, n, total_out_dev, g->stream);
}

int grz_exclusive_sum_u32_on(grz_graph* g, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total_out_dev,
                             cudaStream_t st)
{
    return scan_impl<OpSum, false>(g, in, out, n, total_out_dev, st);
}

int grz_inclusive_max_u32(grz_graph* g, const uint32_t* in, uint32_t* out, uint64_t n)
{
    return scan_impl<OpMax, true>(g, in, out, n, nullptr, g->stream);
}
