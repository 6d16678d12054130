// grz_pr.cu -- PageRank edge-pull and vertex phases on the vector-sparse layout.
//
// Reference semantics (source/phase_edge_pull_pr.asm:45-171, source/phase_vertex_pr.asm:27-134):
//   accum[v] = sum over v's in-edge vectors of the props of the valid source lanes
//   S        = sum of all accumulators (the "PageRank sum" of the reduce buffer)
//   prop[v]  = ((accum[v] + (1 - S)/V) * d + (1 - d)/V) / (outdeg[v] == 0 ? V : outdeg[v])
//
// GB300 design:
//   * Accumulation is exact in unsigned 4.124 fixed point (u128).  The gathered values are the
//     props converted exactly from double.  Integer addition is associative, so each sum is the
//     exact sum of the reference's double inputs, rounded once to double.  The result is
//     independent of tile shape, thread count and scheduling.  GB300's FP64 pipe runs at ~1/58
//     of its integer rate, so FP64 adds per edge would bound the kernel.
//   * The gather kernel runs one thread per vector at full occupancy, so that as many random
//     16-byte gathers as possible are in flight.  The gathers bound the iteration: about one line
//     request per SM clock.  A warp-segmented scan sums the vectors of each destination.
//     Destinations cut by a warp edge are combined with exact u128 atomics, in any order.
//     This replaces the reference's work-unit merge buffer (source/phases.c:41-70); no thread
//     ever waits on another.
//   * The apply kernel is the vertex phase.  It also accumulates S_{k+1} = sum_u outdeg[u] *
//     prop_{k+1}[u] exactly, which equals iteration k+1's sum of accumulators, so an iteration is
//     two kernels with no host round trip.
//   * The vertex formula is fma(acc, d, G*d + (1-d)/V) times a precomputed 1/deg'.  It stays
//     within a few roundings of the reference's ((acc + G)*d + (1-d)/V) / deg': two FP64 ops
//     per vertex instead of three plus a division, on a part whose FP64 rate is low.
#include <string.h>

#include <algorithm>
#include <vector>

#include "grz_internal.cuh"

namespace {

constexpr int PR_THREADS = 256;

__device__ __forceinline__ u128 ld_fx(const u128* p, uint32_t i)
{
#if GRZ_GATHER_LD == 1
    u128 r;
    asm("ld.global.nc.L1::evict_last.v2.u64 {%0, %1}, [%2];" : "=l"(r.lo), "=l"(r.hi) : "l"(p + i));
    return r;
#else
    const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(p) + i);
    u128 r;
    r.lo = v.x;
    r.hi = v.y;
    return r;
#endif
}

// a gathered prop as fixed point: stored so (16 bytes), or as the double it exactly converts
// from (8 bytes: half the gathered working set, the same sums)
__device__ __forceinline__ u128 ld_prop(const u128* p, uint32_t i) { return ld_fx(p, i); }
__device__ __forceinline__ u128 ld_prop(const double* p, uint32_t i) { return fx_from_double(__ldg(p + i)); }

// The same through the coherent path (ld.global, L1-cached): for the persistent kernel, whose
// apply phase rewrites the props that a later gather phase of the same launch reads, which the
// read-only (non-coherent) path does not allow.
__device__ __forceinline__ u128 ld_prop_coh(const u128* p, uint32_t i)
{
    u128 r;
    asm volatile("ld.global.v2.u64 {%0, %1}, [%2];" : "=l"(r.lo), "=l"(r.hi) : "l"(p + i));
    return r;
}
__device__ __forceinline__ u128 ld_prop_coh(const double* p, uint32_t i)
{
    double x;
    asm volatile("ld.global.f64 %0, [%1];" : "=d"(x) : "l"(p + i));
    return fx_from_double(x);
}

// per-iteration constants handed from the gather kernel to the apply kernel
struct PRConst {
    const u128* part_in;  // per-block partial sums whose total is S_k (exact)
    uint32_t nparts;
    double* K_out;        // G*d + (1-d)/V
    double damping, c, nverts;
};

__device__ __forceinline__ u128 u128_shfl_up(u128 v, int off)
{
    u128 r;
    r.lo = __shfl_up_sync(0xffffffffu, v.lo, off);
    r.hi = __shfl_up_sync(0xffffffffu, v.hi, off);
    return r;
}

// Edge-pull gather: one thread per vector.  Each vector's four source props are summed exactly
// in the reference's lane order (g2+g3)+(g0+g1) (phase_edge_pull_pr.asm:146-149); integer
// addition makes the order immaterial anyway.  A warp-segmented inclusive scan over the
// destination keys then sums the vectors of each destination within the warp.  A destination
// whose vectors all lie in this warp is stored with one plain store.  One that continues into a
// neighbouring warp is combined across the block and stored once; only a destination whose
// vectors straddle the block's tile edge is added with exact u128 atomics, so only those
// accumulators must be zero on entry (the fused apply clears exactly those, marked in pr_cut).
// A destination with no in-edges is never touched and stays 0.  The loads of nbr/dst are
// streamed once (evict-first); the prop gathers go through L1.  P is the gathered props' type:
// u128 fixed point, or double (converted exactly to fixed point after the load).
__device__ __forceinline__ u128 block_reduce_u128(u128 s, u128* red);

// shared memory of the gather's block combine
struct GatherSmem {
    static constexpr int NW = PR_THREADS / 32;
    uint32_t key[2][NW];
    u128 sum[2][NW];
    uint32_t flag[2][NW];  // bit0 present, bit1 head real, bit2 tail real
    u128 red[NW];
};

// once per iteration (block 0 of the gather): S_k from the previous apply's per-block partials,
// then K = G*d + (1-d)/V with G = (1 - S_k)/V
__device__ __forceinline__ void pr_publish_K(const PRConst& pc, u128* red)
{
    u128 S = u128_zero();
    for (uint32_t b = threadIdx.x; b < pc.nparts; b += PR_THREADS) S = u128_add(S, pc.part_in[b]);
    S = block_reduce_u128(S, red);
    if (threadIdx.x == 0) *pc.K_out = __fma_rn((1.0 - fx_to_double(S)) / pc.nverts, pc.damping, pc.c);
}

// The gather over tiles blockIdx.x, blockIdx.x + nblocks, ... of PR_THREADS vectors.
// ADD: the accumulators already hold the sums of earlier launches (source segments); a destination
// owned by one warp or block is added by a plain read-modify-write, one cut by a tile edge atomically.
__device__ __forceinline__ void rowacc_put(u128* rowacc, uint32_t key, u128 val, bool add)
{
    ulonglong2* p = reinterpret_cast<ulonglong2*>(rowacc) + key;
    if (add) {
        const ulonglong2 o = __ldcg(p);
        u128 a;
        a.lo = o.x;
        a.hi = o.y;
        val = u128_add(val, a);
    }
    __stcg(p, make_ulonglong2(val.lo, val.hi));
}

template <typename P, bool COH, bool ADD = false>
__device__ __forceinline__ void pr_gather_tiles(const uint4* __restrict__ nbr, const uint32_t* __restrict__ dstv, uint64_t first,
                                                uint64_t nvec, uint64_t list_nvec, const P* __restrict__ prop_fx, uint32_t V,
                                                u128* __restrict__ rowacc, const uint32_t* __restrict__ hub_vid, uint32_t nhub,
                                                uint32_t block, uint32_t nblocks, GatherSmem& sm)
{
    constexpr int NW = GatherSmem::NW;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // vector indices stay below 2^32 (the lists' limit), so the index arithmetic is 32-bit
    const uint32_t ntiles = (uint32_t)((nvec + PR_THREADS - 1) / PR_THREADS);
    const uint32_t first32 = (uint32_t)first, nvec32 = (uint32_t)nvec, list32 = (uint32_t)list_nvec;
    for (uint32_t tile = block; tile < ntiles; tile += nblocks) {
        if (lane < 2) sm.flag[lane][warp] = 0;
        const uint32_t i = tile * PR_THREADS + threadIdx.x;
        const uint32_t v = first32 + i;
        const bool live = i < nvec32;
        uint32_t key = 0xffffffffu;
        u128 val = u128_zero();
        if (live) {
            const uint4 s = ld_stream(nbr + v);
            key = ld_stream(dstv + v);
            const uint32_t i0 = min(grz_hub_decode(s.x, hub_vid, nhub), V), i1 = min(grz_hub_decode(s.y, hub_vid, nhub), V);
            const uint32_t i2 = min(grz_hub_decode(s.z, hub_vid, nhub), V), i3 = min(grz_hub_decode(s.w, hub_vid, nhub), V);
            const u128 g0 = COH ? ld_prop_coh(prop_fx, i0) : ld_prop(prop_fx, i0);
            const u128 g1 = COH ? ld_prop_coh(prop_fx, i1) : ld_prop(prop_fx, i1);
            const u128 g2 = COH ? ld_prop_coh(prop_fx, i2) : ld_prop(prop_fx, i2);
            const u128 g3 = COH ? ld_prop_coh(prop_fx, i3) : ld_prop(prop_fx, i3);
            val = u128_add(u128_add(g2, g3), u128_add(g0, g1));
        }
        uint32_t prevkey = __shfl_up_sync(0xffffffffu, key, 1);
        uint32_t nextkey = __shfl_down_sync(0xffffffffu, key, 1);
        // neighbours across the warp edge come from the whole list, so a destination cut by the edge of
        // a caller's vector range is also added atomically, from both sides
        if (lane == 0) prevkey = (live && v > 0) ? __ldg(dstv + v - 1) : 0xfffffffeu;
        if (lane == 31) nextkey = (live && v + 1 < list32) ? __ldg(dstv + v + 1) : 0xfffffffeu;
        const bool head = key != prevkey;  // the previous vector has another destination
        const bool tail = key != nextkey;  // the next vector has another destination
        const unsigned real_heads = __ballot_sync(0xffffffffu, head);
        const unsigned seg_heads = real_heads | 1u;  // warp-local segments
        const int segstart = 31 - __clz(seg_heads & (0xffffffffu >> (31 - lane)));
        const int maxlen = __reduce_max_sync(0xffffffffu, (unsigned)(lane - segstart + 1));
        for (int off = 1; off < maxlen; off <<= 1) {
            const u128 o = u128_shfl_up(val, off);
            if (lane - off >= segstart) val = u128_add(val, o);
        }
        __syncwarp();
        if (live && (tail || lane == 31)) {
            const bool head_real = (real_heads >> segstart) & 1u;
            if (tail && head_real) {
                // every vector of this destination is in this warp
                rowacc_put(rowacc, key, val, ADD);
            } else {
                // open on the left (slot 0) or on the right only (slot 1): combined across the block below
                const int slot = (segstart == 0 && !head_real) ? 0 : 1;
                sm.key[slot][warp] = key;
                sm.sum[slot][warp] = val;
                sm.flag[slot][warp] = 1u | (head_real ? 2u : 0u) | (tail ? 4u : 0u);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            // Walk the warps' open pieces in order.  A destination that starts and ends inside the
            // block is stored once.  Only destinations that cross the block edge (at most the first
            // and the last) are added to global memory atomically.
            bool open = false, open_head = false;
            uint32_t ok = 0;
            u128 os = u128_zero();
            for (int w = 0; w < NW; ++w) {
                const uint32_t f0 = sm.flag[0][w];
                if (f0 & 1u) {
                    if (!open) { open = true; open_head = false; ok = sm.key[0][w]; os = u128_zero(); }
                    os = u128_add(os, sm.sum[0][w]);
                    if (f0 & 4u) {
                        if (open_head) rowacc_put(rowacc, ok, os, ADD);
                        else if (os.lo | os.hi) u128_atomic_add(rowacc + ok, os);
                        open = false;
                    }
                }
                const uint32_t f1 = sm.flag[1][w];
                if (f1 & 1u) { open = true; open_head = (f1 & 2u) != 0; ok = sm.key[1][w]; os = sm.sum[1][w]; }
            }
            if (open && (os.lo | os.hi)) u128_atomic_add(rowacc + ok, os);
        }
        __syncthreads();  // the walk has read this tile's pieces
    }
}

// 8 resident blocks per SM asked of the compiler: 32 registers, the most gathers in flight (a
// 16-byte spill in the fixed-point form).  Unbounded, the compiler takes 80 registers (3 blocks
// per SM), which measured 47% slower at R-MAT 20.
constexpr int PR_GATHER_MIN_BLOCKS = 8;

template <typename P, bool ADD = false>
__global__ void __launch_bounds__(PR_THREADS, PR_GATHER_MIN_BLOCKS) k_pr_gather(const uint4* __restrict__ nbr, const uint32_t* __restrict__ dstv,
                                                          uint64_t first, uint64_t nvec, uint64_t list_nvec,
                                                          const P* __restrict__ prop_fx, uint32_t V, u128* __restrict__ rowacc,
                                                          const uint32_t* __restrict__ hub_vid, uint32_t nhub, const PRConst pc)
{
    __shared__ GatherSmem sm;
    if (pc.K_out && blockIdx.x == 0) pr_publish_K(pc, sm.red);
    pr_gather_tiles<P, false, ADD>(nbr, dstv, first, nvec, list_nvec, prop_fx, V, rowacc, hub_vid, nhub, blockIdx.x, gridDim.x, sm);
}

__device__ __forceinline__ u128 block_reduce_u128(u128 s, u128* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    s = u128_zero();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < PR_THREADS / 32) ? red[threadIdx.x] : u128_zero();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
    }
    return s;
}

// Vertex phase fused with reading the accumulators (phase_vertex_pr.asm:75-134):
//   prop[v] = (acc[v]*d + G*d + (1-d)/V) / deg'[v],  G = (1 - S)/V
// computed as fma + multiply by the precomputed 1/deg'.  It writes the new props in fixed point,
// or as doubles when the next gather reads doubles (plus the reference-format doubles when
// asked), and accumulates S' = sum deg[v]*prop[v] exactly; S' is the next
// iteration's sum of accumulators.  Of the accumulators it clears only those the next gather
// adds to atomically (bit set in `cut`); the others are overwritten by the next gather's stores.
// The grid strides over the vertices, PR_APPLY_U vertices per thread at a time whose
// accumulators are loaded before anything is stored; one partial of S' per block.  GB300 sweep of
// vertices in flight per thread x blocks per SM: 8 x 3 (80 registers) 16.7 us at V = 2^20 and
// 2.08 ms at V = 2^27; 4 x 4 14.5 us; 2 x 6 14.5 us and 1.25 ms; 1 x 8 (31 registers) 14.5 us and
// 1.15 ms (5.2 TB/s of 44V bytes).  Occupancy hides the latency better than loads in flight.
#ifndef GRZ_PR_APPLY_U
#define GRZ_PR_APPLY_U 1
#endif
#ifndef GRZ_PR_APPLY_MINB
#define GRZ_PR_APPLY_MINB 8
#endif
constexpr int PR_APPLY_U = GRZ_PR_APPLY_U;
constexpr int PR_APPLY_RESIDENT = GRZ_PR_APPLY_MINB;  // blocks per SM that the launch bounds fit

// the apply over vertices block*PR_THREADS + tid, strided by nblocks*PR_THREADS, U vertices per
// thread loaded before any is stored; returns the block's partial of S' (valid in thread 0;
// every thread of the block must call it)
template <int U>
__device__ __forceinline__ u128 pr_apply_range(u128* __restrict__ rowacc, const uint32_t* __restrict__ cut, bool clear_all,
                                               const double* __restrict__ inv_deg, const uint32_t* __restrict__ degree, uint64_t V,
                                               double sK, double damping, u128* __restrict__ prop_fx, double* __restrict__ prop_d,
                                               double* __restrict__ prop_out, uint32_t block, uint32_t nblocks, u128* red)
{
    const uint64_t stride = (uint64_t)nblocks * PR_THREADS;
    u128 s = u128_zero();
    for (uint64_t base = (uint64_t)block * PR_THREADS + threadIdx.x; base < V; base += stride * U) {
        ulonglong2 a[U];
        uint32_t cw[U];
#pragma unroll
        for (int j = 0; j < U; ++j) {
            const uint64_t v = base + (uint64_t)j * stride;
            a[j] = make_ulonglong2(0ull, 0ull);
            cw[j] = 0;
            if (v < V) {
                a[j] = __ldcs(reinterpret_cast<const ulonglong2*>(rowacc) + v);
                cw[j] = clear_all ? 0u : __ldg(cut + (v >> 5));
            }
        }
#pragma unroll
        for (int j = 0; j < U; ++j) {
            const uint64_t v = base + (uint64_t)j * stride;
            if (v >= V) break;
            if ((a[j].x | a[j].y) && (clear_all || ((cw[j] >> (v & 31)) & 1u)))
                *(reinterpret_cast<ulonglong2*>(rowacc) + v) = make_ulonglong2(0ull, 0ull);
            u128 acc;
            acc.lo = a[j].x;
            acc.hi = a[j].y;
            const double p = __dmul_rn(__fma_rn(fx_to_double(acc), damping, sK), __ldg(inv_deg + v));
            const u128 pf = fx_from_double(p);
            if (prop_d) __stcg(prop_d + v, p);  // the next gather reads doubles
            else __stcg(reinterpret_cast<ulonglong2*>(prop_fx) + v, make_ulonglong2(pf.lo, pf.hi));
            if (prop_out) prop_out[v] = p;
            s = u128_add(s, u128_mul32(pf, __ldg(degree + v)));
        }
    }
    return block_reduce_u128(s, red);
}

__global__ void __launch_bounds__(PR_THREADS, PR_APPLY_RESIDENT) k_pr_apply(u128* __restrict__ rowacc, const uint32_t* __restrict__ cut,
                                                                            int clear_all, const double* __restrict__ inv_deg,
                                                                            const uint32_t* __restrict__ degree, uint64_t V,
                                                                            const double* __restrict__ Kp, u128* __restrict__ part_out,
                                                                            double damping, u128* __restrict__ prop_fx,
                                                                            double* __restrict__ prop_d, double* __restrict__ prop_out)
{
    __shared__ u128 red[PR_THREADS / 32];
    const u128 s = pr_apply_range<PR_APPLY_U>(rowacc, cut, clear_all != 0, inv_deg, degree, V, *Kp, damping, prop_fx, prop_d, prop_out, blockIdx.x, gridDim.x,
                                  red);
    if (threadIdx.x == 0) part_out[blockIdx.x] = s;  // summed by the next gather kernel's block 0
}

// ---------------------------------------------------------------------------------------------
// Persistent form: all iterations in one cooperative launch, gather and apply separated by a
// grid-wide barrier (the reference's pull phase -> threads_barrier -> perform_vertex_phase_pr,
// source/phase_vertex_pr.asm:190-285, barrier source/threads.asm:181-204).  Every wait of the
// barrier is bounded: past the deadline (%globaltimer) a block sets the error word and every
// block returns at its next barrier, so a launch always ends and the host reads the error.

struct PRBar {
    unsigned int count;     // arrivals at the current barrier
    unsigned int gen;       // barriers completed
    unsigned int err;       // 1: a wait ran out
    unsigned int where;     // the barrier (1-based) whose wait ran out
    unsigned long long gather_ns[64];  // per iteration, block 0's view: gather phase (the barrier included)
    unsigned long long apply_ns[64];   // apply phase
};

constexpr unsigned long long PR_BAR_SPIN_MAX = 1ull << 26;  // iteration bound of one wait (besides the deadline)

__device__ __forceinline__ unsigned long long pr_now_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// true when every block arrived; false when a wait gave up (or another block's did).
// `withhold` leaves this block's arrival out (host-side fault injection for the tests).
__device__ __forceinline__ bool pr_grid_barrier(PRBar* bar, unsigned nblocks, unsigned long long limit_ns, unsigned idx, bool withhold)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile unsigned int* vgen = &bar->gen;
        volatile unsigned int* verr = &bar->err;
        const unsigned int g0 = *vgen;
        __threadfence();
        if (*verr) {
            ok = 0;
        } else if (!withhold && atomicAdd(&bar->count, 1u) + 1u == nblocks) {
            bar->count = 0u;
            __threadfence();
            atomicAdd(&bar->gen, 1u);
        } else {
            const unsigned long long t0 = pr_now_ns();
            for (unsigned long long spin = 0; *vgen == g0; ++spin) {
                if (*verr) { ok = 0; break; }
                if (spin >= PR_BAR_SPIN_MAX || pr_now_ns() - t0 > limit_ns) {
                    if (atomicExch(&bar->err, 1u) == 0u) bar->where = idx;
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

struct PRPersist {
    const uint4* nbr;
    const uint32_t* dstv;
    uint64_t nvec;
    uint32_t V;
    const uint32_t* hub_vid;
    uint32_t nhub;
    u128* rowacc;
    const uint32_t* cut;
    const double* inv_deg;
    const uint32_t* degree;
    u128* fx[2];            // props, fixed point (ping-pong)
    double* d[2];           // props, doubles (ping-pong; gathered in doubles mode)
    int dmode;
    int cur;                // which buffer holds the current props
    u128* sum[2];           // per-block partials of S (ping-pong)
    uint32_t nparts0;       // partials in sum[sum_cur] at the start
    int sum_cur;
    double* K;
    double damping, c, nverts;
    uint32_t iters;
    double* prop_out;       // reference-format doubles after the last iteration, or null
    PRBar* bar;
    unsigned long long limit_ns;
    int withhold_block;     // -1: none
    int time_phases;        // block 0 records the phase durations into bar
};

// registers bounded so that MINB blocks of 256 threads stay resident per SM (the gather wants as
// many random loads in flight as possible: 6 leaves the apply unspilled, 8 is the two-kernel
// gather's occupancy); the apply loads 2 vertices per thread ahead
constexpr int PR_PERSIST_APPLY_U = 2;

template <typename P, int MINB>
__global__ void __launch_bounds__(PR_THREADS, MINB) k_pr_persistent(const PRPersist q)
{
    __shared__ GatherSmem sm;
    const unsigned nb = gridDim.x;
    unsigned bi = 0;
    int cur = q.cur, sc = q.sum_cur;
    uint32_t nparts = q.nparts0;
    for (uint32_t it = 0; it < q.iters; ++it) {
        const unsigned long long t0 = (q.time_phases && blockIdx.x == 0 && threadIdx.x == 0) ? pr_now_ns() : 0ull;
        if (blockIdx.x == 0) {
            PRConst pc;
            pc.part_in = q.sum[sc];
            pc.nparts = nparts;
            pc.K_out = q.K;
            pc.damping = q.damping;
            pc.c = q.c;
            pc.nverts = q.nverts;
            pr_publish_K(pc, sm.red);
        }
        const P* props = q.dmode ? (const P*)q.d[cur] : (const P*)q.fx[cur];
        pr_gather_tiles<P, true>(q.nbr, q.dstv, 0, q.nvec, q.nvec, props, q.V, q.rowacc, q.hub_vid, q.nhub, blockIdx.x, nb, sm);
        if (!pr_grid_barrier(q.bar, nb, q.limit_ns, ++bi, (int)blockIdx.x == q.withhold_block)) return;
        const unsigned long long t1 = (q.time_phases && blockIdx.x == 0 && threadIdx.x == 0) ? pr_now_ns() : 0ull;
        const double sK = *(volatile double*)q.K;
        const u128 s = pr_apply_range<PR_PERSIST_APPLY_U>(q.rowacc, q.cut, false, q.inv_deg, q.degree, q.V, sK, q.damping, q.fx[cur ^ 1],
                                      q.dmode ? q.d[cur ^ 1] : nullptr, it + 1 == q.iters ? q.prop_out : nullptr, blockIdx.x, nb,
                                      sm.red);
        if (threadIdx.x == 0) q.sum[sc ^ 1][blockIdx.x] = s;
        if (!pr_grid_barrier(q.bar, nb, q.limit_ns, ++bi, false)) return;
        if (q.time_phases && blockIdx.x == 0 && threadIdx.x == 0 && it < 64) {
            const unsigned long long t2 = pr_now_ns();
            q.bar->gather_ns[it] = t1 - t0;
            q.bar->apply_ns[it] = t2 - t1;
        }
        cur ^= 1;
        sc ^= 1;
        nparts = nb;
    }
}

// bit j of word t: vertex 32t + j has pull vectors in two or more gather tiles of PR_THREADS
// vectors (its accumulator is summed with atomics)
__global__ void k_pr_cutbits(const uint32_t* __restrict__ rowptr, uint64_t V, uint32_t* __restrict__ cut)
{
    const uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool c = false;
    if (v < V) {
        const uint32_t r0 = rowptr[v], r1 = rowptr[v + 1];
        c = r1 > r0 && r0 / PR_THREADS != (r1 - 1) / PR_THREADS;
    }
    const unsigned m = __ballot_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0 && v < V) cut[v >> 5] = m;
}

// ---------------------------------------------------------------------------------------------
// Source-segmented pull lists.  A destination's in-edges are its vectors' lanes in order, sorted
// by source (the -pull order), so the edges from source segment s form one run of lanes
// [a_s, b_s).  Segment s's list has ceil((b_s - a_s) / 4) vectors per destination, grouped by
// destination in ascending order; the segment lists are concatenated in segment order.

// source of lane L of a destination whose vectors start at r0
__device__ __forceinline__ uint32_t lane_src(const uint32_t* __restrict__ nbr32, uint32_t r0, uint32_t L)
{
    return __ldg(nbr32 + (uint64_t)r0 * 4 + L);
}

// valid lanes of the destination with vectors [r0, r1) (only its last vector can be partial)
__device__ __forceinline__ uint32_t dst_lanes(const uint4* __restrict__ nbr, uint32_t r0, uint32_t r1)
{
    const uint4 t = __ldg(nbr + r1 - 1);
    return 4 * (r1 - r0 - 1) + (t.x != GRZ_INVALID_ID) + (t.y != GRZ_INVALID_ID) + (t.z != GRZ_INVALID_ID) + (t.w != GRZ_INVALID_ID);
}

// first lane in [lo, hi) whose source is >= key, else hi
__device__ __forceinline__ uint32_t lane_lower_bound(const uint32_t* __restrict__ nbr32, uint32_t r0, uint32_t lo, uint32_t hi,
                                                     uint64_t key)
{
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if ((uint64_t)lane_src(nbr32, r0, mid) < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// first lane at or after p + 1 whose source is >= key (lane p's source is below key): galloping,
// then a binary search, so a run of n lanes costs O(log n) reads
__device__ __forceinline__ uint32_t lane_gallop(const uint32_t* __restrict__ nbr32, uint32_t r0, uint32_t p, uint32_t L, uint64_t key)
{
    uint32_t lo = p + 1, step = 1, hi = p + 1;
    while (hi < L && (uint64_t)lane_src(nbr32, r0, hi) < key) {
        lo = hi + 1;
        step <<= 1;
        hi = (p + step < L) ? p + step : L;
    }
    return lane_lower_bound(nbr32, r0, lo, hi < L ? hi : L, key);
}

// vectors of every (segment, destination): cnt[s * (V + 1) + d]; entries of empty pairs stay 0
__global__ void k_seg_count(const uint4* __restrict__ nbr, const uint32_t* __restrict__ rowptr, uint32_t V, uint32_t bits,
                            uint32_t* __restrict__ cnt)
{
    const uint32_t* nbr32 = reinterpret_cast<const uint32_t*>(nbr);
    for (uint64_t d = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; d < V; d += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t r0 = __ldg(rowptr + d), r1 = __ldg(rowptr + d + 1);
        if (r0 == r1) continue;
        const uint32_t L = dst_lanes(nbr, r0, r1);
        uint32_t p = 0;
        while (p < L) {
            const uint32_t sg = lane_src(nbr32, r0, p) >> bits;
            const uint32_t q = lane_gallop(nbr32, r0, p, L, (uint64_t)(sg + 1) << bits);
            cnt[(uint64_t)sg * (V + 1) + d] = (q - p + 3) / 4;
            p = q;
        }
    }
}

// run of one (segment, destination) pair too long for one thread: written by a whole block
struct SegBig {
    uint32_t d, a, b, out;  // destination, lanes [a, b), first output vector (within the segment)
};
constexpr uint32_t SEG_BIG_VECTORS = 32;

__device__ __forceinline__ void seg_write_vector(const uint32_t* __restrict__ nbr32, uint32_t r0, uint32_t a, uint32_t b, uint32_t j,
                                                 uint32_t d, uint4* __restrict__ out_nbr, uint32_t* __restrict__ out_dst, uint64_t o)
{
    const uint32_t L0 = a + 4 * j;
    uint4 v;
    v.x = L0 + 0 < b ? lane_src(nbr32, r0, L0 + 0) : GRZ_INVALID_ID;
    v.y = L0 + 1 < b ? lane_src(nbr32, r0, L0 + 1) : GRZ_INVALID_ID;
    v.z = L0 + 2 < b ? lane_src(nbr32, r0, L0 + 2) : GRZ_INVALID_ID;
    v.w = L0 + 3 < b ? lane_src(nbr32, r0, L0 + 3) : GRZ_INVALID_ID;
    out_nbr[o] = v;
    out_dst[o] = d;
}

// segment sg: each destination with a run writes its vectors at base + off[d]; runs of more than
// SEG_BIG_VECTORS vectors are listed for k_seg_write_big instead
__global__ void k_seg_write(const uint4* __restrict__ nbr, const uint32_t* __restrict__ rowptr, uint32_t V, uint32_t bits, uint32_t sg,
                            const uint32_t* __restrict__ off, uint64_t base, uint4* __restrict__ out_nbr, uint32_t* __restrict__ out_dst,
                            SegBig* __restrict__ big, uint32_t* __restrict__ nbig)
{
    const uint32_t* nbr32 = reinterpret_cast<const uint32_t*>(nbr);
    for (uint64_t d = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; d < V; d += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t o0 = __ldg(off + d), n = __ldg(off + d + 1) - o0;
        if (n == 0) continue;
        const uint32_t r0 = __ldg(rowptr + d), r1 = __ldg(rowptr + d + 1);
        const uint32_t L = dst_lanes(nbr, r0, r1);
        const uint32_t a = lane_lower_bound(nbr32, r0, 0, L, (uint64_t)sg << bits);
        const uint32_t b = lane_lower_bound(nbr32, r0, a, L, (uint64_t)(sg + 1) << bits);
        if (n > SEG_BIG_VECTORS) {
            const uint32_t k = atomicAdd(nbig, 1u);
            SegBig e;
            e.d = (uint32_t)d; e.a = a; e.b = b; e.out = o0;
            big[k] = e;
            continue;
        }
        for (uint32_t j = 0; j < n; ++j) seg_write_vector(nbr32, r0, a, b, j, (uint32_t)d, out_nbr, out_dst, base + o0 + j);
    }
}

__global__ void k_seg_write_big(const uint4* __restrict__ nbr, const uint32_t* __restrict__ rowptr, const SegBig* __restrict__ big,
                                const uint32_t* __restrict__ nbig, uint64_t base, uint4* __restrict__ out_nbr, uint32_t* __restrict__ out_dst)
{
    const uint32_t* nbr32 = reinterpret_cast<const uint32_t*>(nbr);
    const uint32_t m = *nbig;
    for (uint32_t k = blockIdx.x; k < m; k += gridDim.x) {
        const SegBig e = big[k];
        const uint32_t r0 = __ldg(rowptr + e.d);
        const uint32_t n = (e.b - e.a + 3) / 4;
        for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) seg_write_vector(nbr32, r0, e.a, e.b, j, e.d, out_nbr, out_dst, base + e.out + j);
    }
}

// Edge-pull phase alone (the phases.h boundary): accumulators as doubles plus their exact sum
// into the global accumulator; clears rowacc.
__global__ void __launch_bounds__(PR_THREADS) k_pr_accum_out(u128* __restrict__ rowacc, uint64_t V, double* __restrict__ accum,
                                                             u128* __restrict__ glob)
{
    __shared__ u128 red[PR_THREADS / 32];
    const uint64_t v = (uint64_t)blockIdx.x * PR_THREADS + threadIdx.x;
    u128 s = u128_zero();
    if (v < V) {
        s = rowacc[v];
        rowacc[v] = u128_zero();
        accum[v] = fx_to_double(s);
    }
    s = block_reduce_u128(s, red);
    if (threadIdx.x == 0) u128_slot_add(glob, s);
}

// perform_vertex_phase_pr over [first, first+count): double accumulators -> props (double and fixed)
__global__ void k_pr_vertex(const double* __restrict__ accum, const double* __restrict__ inv_deg,
                            double* __restrict__ prop, u128* __restrict__ prop_fx, uint64_t first, uint64_t count,
                            double damping, double K)
{
    const uint64_t i = (uint64_t)blockIdx.x * PR_THREADS + threadIdx.x;
    if (i >= count) return;
    const uint64_t v = first + i;
    const double p = __dmul_rn(__fma_rn(accum[v], damping, K), inv_deg[v]);
    prop[v] = p;
    prop_fx[v] = fx_from_double(p);
}

// execution_initialize_vertex_prop_pr (source/execution_pr.c:85-88): (1/V) / deg'
__global__ void k_pr_init(const double* __restrict__ outdeg, const uint32_t* __restrict__ degree, uint64_t V,
                          double* __restrict__ prop, double* __restrict__ accum, u128* __restrict__ prop_fx,
                          double* __restrict__ prop_d, u128* __restrict__ part0)
{
    __shared__ u128 red[PR_THREADS / 32];
    const uint64_t v = (uint64_t)blockIdx.x * PR_THREADS + threadIdx.x;
    u128 s = u128_zero();
    if (v < V) {
        const double dV = (double)V;
        const double p = (1.0 / dV) / (outdeg[v] == 0.0 ? dV : outdeg[v]);
        prop[v] = p;
        accum[v] = 0.0;
        const u128 pf = fx_from_double(p);
        prop_fx[v] = pf;
        if (prop_d) prop_d[v] = p;
        s = u128_mul32(pf, degree[v]);
    }
    s = block_reduce_u128(s, red);
    if (threadIdx.x == 0) part0[blockIdx.x] = s;
}

__global__ void k_fx_to_double(const u128* __restrict__ fx, uint64_t V, double* __restrict__ out)
{
    const uint64_t v = (uint64_t)blockIdx.x * PR_THREADS + threadIdx.x;
    if (v < V) out[v] = fx_to_double(fx[v]);
}

// double props -> the fixed-point props they convert to (and, when asked, back to the double
// the fixed-point value rounds to, which is what the fixed-point path reports)
__global__ void k_double_to_fx(const double* __restrict__ d, uint64_t V, u128* __restrict__ fx, double* __restrict__ out)
{
    const uint64_t v = (uint64_t)blockIdx.x * PR_THREADS + threadIdx.x;
    if (v >= V) return;
    const u128 f = fx_from_double(d[v]);
    if (fx) fx[v] = f;
    if (out) out[v] = fx_to_double(f);
}

unsigned blocks_for(uint64_t n) { return (unsigned)((n + PR_THREADS - 1) / PR_THREADS); }

}  // namespace

// The current props live in pr_fx[pr_cur] (fixed point) or, after fused iterations that gather
// doubles, in pr_d[pr_cur]; each form is brought up to date from the other before a path that
// reads it.
static int pr_sync_fx(grz_graph* g)
{
    if (!g->pr_fx_stale) return GRZ_OK;
    k_double_to_fx<<<blocks_for(g->V), PR_THREADS, 0, g->stream>>>(g->pr_d[g->pr_cur], g->V, g->pr_fx[g->pr_cur], nullptr); GRZ_COUNT_LAUNCH(g);
    GRZ_CK(g, cudaGetLastError());
    g->pr_fx_stale = 0;
    return GRZ_OK;
}

static int pr_sync_d(grz_graph* g)
{
    if (!g->pr_d_stale) return GRZ_OK;
    k_fx_to_double<<<blocks_for(g->V), PR_THREADS, 0, g->stream>>>(g->pr_fx[g->pr_cur], g->V, g->pr_d[g->pr_cur]); GRZ_COUNT_LAUNCH(g);
    GRZ_CK(g, cudaGetLastError());
    g->pr_d_stale = 0;
    return GRZ_OK;
}

// The phase-API gathers and the push phase add into every accumulator: after fused iterations,
// which leave the accumulators of non-straddling destinations holding their last sums, clear all.
int grz_pr_rowacc_clean(grz_graph* g)
{
    if (g->pr_rowacc && g->pr_rowacc_stale) {
        GRZ_CK(g, cudaMemsetAsync(g->pr_rowacc, 0, sizeof(u128) * (g->V + 1), g->stream));
        g->pr_rowacc_stale = 0;
    }
    return GRZ_OK;
}

static int pr_build_segments(grz_graph* g, uint32_t bits);

// Sources per segment (log2) of the segmented lists, 0 for none: the tuned size, else, when the
// double props exceed 4x L2 (or `force`), the largest segment whose props are at most 1.25x L2
// (see grz_pr_prepare); never more than GRZ_PR_MAX_SEGMENTS segments.
static uint32_t pr_segment_bits(const grz_graph* g, int force)
{
    const uint64_t V = g->V;
    uint32_t bits = 0;
    const uint32_t sb = g->tune.pr_segment_bits;
    if (sb >= 8) {
        bits = sb;
    } else if (sb == 0 && (force || (uint64_t)sizeof(double) * V > 4ull * (uint64_t)g->l2_bytes)) {
        bits = 8;
        while ((8ull << (bits + 1)) <= (uint64_t)g->l2_bytes * 5 / 4) ++bits;
    }
    while (bits && ((V + (1ull << bits) - 1) >> bits) > GRZ_PR_MAX_SEGMENTS) ++bits;
    return bits;
}

int grz_pr_ensure_segments(grz_graph* g, int force)
{
    const uint32_t bits = pr_segment_bits(g, force);
    if (!bits || g->pull.nhub || !g->pull.nvec) return GRZ_OK;
    return pr_build_segments(g, bits);
}

int grz_pr_prepare(grz_graph* g)
{
    const uint64_t V = g->V;
    if (!g->pr_fx[0]) {
        GRZ_CK(g, cudaMalloc((void**)&g->pr_fx[0], sizeof(u128) * (V + 1)));
        GRZ_CK(g, cudaMalloc((void**)&g->pr_fx[1], sizeof(u128) * (V + 1)));
        GRZ_CK(g, cudaMalloc((void**)&g->pr_sum, sizeof(u128) * 2 * (blocks_for(V) + 1)));
        GRZ_CK(g, cudaMalloc((void**)&g->pr_K, sizeof(double) * 2));
        GRZ_CK(g, cudaMalloc((void**)&g->pr_rowacc, sizeof(u128) * (V + 1)));
        GRZ_CK(g, cudaMalloc((void**)&g->pr_cut, sizeof(uint32_t) * ((V + 31) / 32 + 1)));
        g->pr_lists_changed = 1;
    }
    if (g->pr_lists_changed) {
        // (also after a reload with the same V, which kept the arrays)
        GRZ_CK(g, cudaMemsetAsync(g->pr_rowacc, 0, sizeof(u128) * (V + 1), g->stream));
        g->pr_rowacc_stale = 0;
        if (V) {
            k_pr_cutbits<<<blocks_for(V), PR_THREADS, 0, g->stream>>>(g->pull.rowptr, V, g->pr_cut); GRZ_COUNT_LAUNCH(g);
            GRZ_CK(g, cudaGetLastError());
        }
        // entry V of both prop arrays is a permanent zero that invalid lanes gather
        GRZ_CK(g, cudaMemsetAsync(g->pr_fx[0], 0, sizeof(u128) * (V + 1), g->stream));
        GRZ_CK(g, cudaMemsetAsync(g->pr_fx[1], 0, sizeof(u128) * (V + 1), g->stream));
        for (double* d : g->pr_d)
            if (d) GRZ_CK(g, cudaMemsetAsync(d, 0, sizeof(double) * (V + 1), g->stream));
        g->pr_lists_changed = 0;
    }
    // Doubles gathered instead of 16-byte fixed point: chosen, or when the fixed-point props
    // exceed 6x L2.  Below that the gathers are bound by the L1/L2 path and the per-edge
    // conversion costs more than the smaller working set saves; above it the DRAM sectors of the
    // random gathers dominate and halving the props wins.  GB300 sweep (16 iterations,
    // fixed vs doubles): R-MAT 24 25.7 vs 31.8 ms, 25 64.6 vs 67.4 ms, 26 179.1 vs 156.4 ms,
    // 27 413 vs 371 ms.
    const int pick = g->tune.pr_props;
    g->pr_dmode = pick == 2 || (pick == 0 && (uint64_t)sizeof(u128) * V > 6ull * (uint64_t)g->l2_bytes);
    // Source segments when even the double props are far larger than L2 (or when chosen): each
    // segment's props (8 bytes x 2^bits) mostly stay in L2 while its edges stream, instead of one
    // random DRAM sector per gathered prop.  Segment props of about the size of L2 are best: on
    // GB300 at R-MAT 27 (16 iterations) the gather took 23.2 ms unsegmented and 17.8 / 18.1 /
    // 19.0 / 20.5 ms with 2^24 / 2^23 / 2^22 / 2^21 sources per segment (128 MB of props for
    // 2^24 against 126 MB of L2); smaller segments add more (segment, destination)
    // read-modify-writes and partial vectors than they save.  Needs sources in ascending order
    // along each destination's lanes, which hub encoding breaks.
    const uint32_t bits = pr_segment_bits(g, 0);
    g->pr_segmode = 0;
    if (bits && g->pull.nhub == 0 && g->pull.nvec) {
        const int rc = pr_build_segments(g, bits);
        if (rc) return rc;
        g->pr_segmode = 1;
        g->pr_dmode = 1;  // the segments gather the props as doubles
    }
    if (g->pr_dmode && !g->pr_d[0]) {
        GRZ_CK(g, cudaMalloc((void**)&g->pr_d[0], sizeof(double) * (V + 1)));
        GRZ_CK(g, cudaMalloc((void**)&g->pr_d[1], sizeof(double) * (V + 1)));
        GRZ_CK(g, cudaMemsetAsync(g->pr_d[0], 0, sizeof(double) * (V + 1), g->stream));
        GRZ_CK(g, cudaMemsetAsync(g->pr_d[1], 0, sizeof(double) * (V + 1), g->stream));
    }
    return GRZ_OK;
}

// Builds the source-segmented pull lists with 2^bits sources per segment (once per lists and bits).
static int pr_build_segments(grz_graph* g, uint32_t bits)
{
    if (g->seg_nbr && g->seg_bits == bits) return GRZ_OK;
    grz_dev_free(g, g->seg_nbr);
    grz_dev_free(g, g->seg_dst);
    g->seg_nbr = nullptr;
    g->seg_dst = nullptr;
    g->seg_bits = 0;
    const uint64_t V = g->V;
    const uint32_t nseg = (uint32_t)((V + (1ull << bits) - 1) >> bits);
    if (nseg == 0 || nseg > GRZ_PR_MAX_SEGMENTS) return grz_set_error(g, GRZ_ERR_RANGE, "%u source segments (at most %d)", nseg, GRZ_PR_MAX_SEGMENTS);
    cudaStream_t st = g->stream;
    uint32_t *cnt = nullptr, *tot = nullptr, *nbig = nullptr;
    SegBig* big = nullptr;
    const uint64_t ncnt = (uint64_t)nseg * (V + 1);
    int rc = grz_dev_alloc(g, (void**)&cnt, sizeof(uint32_t) * ncnt);
    if (!rc) rc = grz_dev_alloc(g, (void**)&tot, sizeof(uint32_t) * (nseg + 1));
    if (!rc) rc = grz_cuda_check(g, cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * ncnt, st), "memset");
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(blocks_for(V), (uint64_t)g->num_sms * 8));
    if (!rc) {
        k_seg_count<<<grid, PR_THREADS, 0, st>>>(g->pull.nbr, g->pull.rowptr, (uint32_t)V, bits, cnt); GRZ_COUNT_LAUNCH(g);
        rc = grz_cuda_check(g, cudaGetLastError(), "k_seg_count");
    }
    for (uint32_t sg = 0; sg < nseg && !rc; ++sg)
        rc = grz_exclusive_sum_u32_on(g, cnt + (uint64_t)sg * (V + 1), cnt + (uint64_t)sg * (V + 1), V + 1, tot + sg, st);
    std::vector<uint32_t> th(nseg);
    if (!rc) rc = grz_cuda_check(g, cudaMemcpyAsync(th.data(), tot, sizeof(uint32_t) * nseg, cudaMemcpyDeviceToHost, st), "D2H");
    if (!rc) rc = grz_cuda_check(g, cudaStreamSynchronize(st), "segment counts");
    uint64_t total = 0, maxn = 0;
    if (!rc) {
        for (uint32_t sg = 0; sg < nseg; ++sg) {
            g->seg_first[sg] = total;
            total += th[sg];
            maxn = std::max<uint64_t>(maxn, th[sg]);
        }
        g->seg_first[nseg] = total;
        if (total >= 0xffffffffull) rc = grz_set_error(g, GRZ_ERR_RANGE, "segmented lists of %llu vectors", (unsigned long long)total);
    }
    if (!rc) rc = grz_dev_alloc(g, (void**)&g->seg_nbr, sizeof(uint4) * std::max<uint64_t>(total, 1));
    if (!rc) rc = grz_dev_alloc(g, (void**)&g->seg_dst, sizeof(uint32_t) * std::max<uint64_t>(total, 1));
    // long runs: at most one per SEG_BIG_VECTORS + 1 vectors of a segment
    if (!rc) rc = grz_dev_alloc(g, (void**)&big, sizeof(SegBig) * (maxn / (SEG_BIG_VECTORS + 1) + 1));
    if (!rc) rc = grz_dev_alloc(g, (void**)&nbig, sizeof(uint32_t));
    for (uint32_t sg = 0; sg < nseg && !rc; ++sg) {
        if (!th[sg]) continue;
        rc = grz_cuda_check(g, cudaMemsetAsync(nbig, 0, sizeof(uint32_t), st), "memset");
        if (rc) break;
        k_seg_write<<<grid, PR_THREADS, 0, st>>>(g->pull.nbr, g->pull.rowptr, (uint32_t)V, bits, sg, cnt + (uint64_t)sg * (V + 1),
                                                 g->seg_first[sg], g->seg_nbr, g->seg_dst, big, nbig); GRZ_COUNT_LAUNCH(g);
        k_seg_write_big<<<(unsigned)g->num_sms * 4, PR_THREADS, 0, st>>>(g->pull.nbr, g->pull.rowptr, big, nbig, g->seg_first[sg],
                                                                        g->seg_nbr, g->seg_dst); GRZ_COUNT_LAUNCH(g);
        rc = grz_cuda_check(g, cudaGetLastError(), "k_seg_write");
    }
    for (void* q : { (void*)cnt, (void*)tot, (void*)big, (void*)nbig }) grz_dev_free(g, q);
    if (rc) {
        grz_dev_free(g, g->seg_nbr);
        grz_dev_free(g, g->seg_dst);
        g->seg_nbr = nullptr;
        g->seg_dst = nullptr;
        return rc;
    }
    g->seg_bits = bits;
    g->nseg = nseg;
    return GRZ_OK;
}

// PageRank initial state (props, zero accumulators, S_0)
int grz_pr_init_state(grz_graph* g, double damping)
{
    int rc = grz_pr_prepare(g);
    if (rc) return rc;
    g->pr_damping = damping;
    g->pr_cur = 0;
    g->pr_fx_stale = g->pr_d_stale = 0;
    g->pr_sum_cur = 0;
    g->pr_iters_done = 0;
    GRZ_CK(g, cudaMemsetAsync(g->pr_sum, 0, sizeof(u128) * 2 * (blocks_for(g->V) + 1), g->stream));
    GRZ_CK(g, cudaMemsetAsync(g->accum, 0, sizeof(double) * (g->V + 8), g->stream));
    g->pr_nparts[0] = g->pr_nparts[1] = blocks_for(g->V);
    if (g->V) {
        k_pr_init<<<blocks_for(g->V), PR_THREADS, 0, g->stream>>>(g->outdeg, g->degree, g->V, g->prop, g->accum, g->pr_fx[0],
                                                                 g->pr_dmode ? g->pr_d[0] : nullptr, g->pr_sum); GRZ_COUNT_LAUNCH(g);
        GRZ_CK(g, cudaGetLastError());
    }
    return GRZ_OK;
}

// resident blocks per SM of the gather kernel (its grid is persistent: SMs x resident)
template <typename P, bool ADD>
static int pr_gather_resident(grz_graph* g)
{
    static int resident[64] = {};
    if (g->device < 0 || g->device >= 64) return 1;
    if (!resident[g->device]) {
        int r = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_pr_gather<P, ADD>, PR_THREADS, 0) != cudaSuccess || r < 1) {
            cudaGetLastError();
            r = 1;
        }
        resident[g->device] = r;
    }
    return resident[g->device];
}

// one gather launch over vectors [first, first + count) of a list of list_nvec vectors
template <typename P, bool ADD>
static void pr_gather_launch(grz_graph* g, const uint4* nbr, const uint32_t* dstv, uint64_t first, uint64_t count, uint64_t list_nvec,
                             const P* props, const uint32_t* hub_vid, uint32_t nhub, const PRConst& pc)
{
    const uint64_t want = g->tune.pr_grid ? g->tune.pr_grid : (uint64_t)g->num_sms * pr_gather_resident<P, ADD>(g);
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(blocks_for(count), want));
    k_pr_gather<P, ADD><<<grid, PR_THREADS, 0, g->stream>>>(nbr, dstv, first, count, list_nvec, props, (uint32_t)g->V, g->pr_rowacc,
                                                            hub_vid, nhub, pc);
    GRZ_COUNT_LAUNCH(g);
}

template <typename P>
static int pr_gather(grz_graph* g, uint64_t first, uint64_t count, const PRConst& pc, const P* props)
{
    if (count == 0) return GRZ_OK;
    grz_prof_begin(g, GRZ_PROF_PR_GATHER);
    pr_gather_launch<P, false>(g, g->pull.nbr, g->pull.shared, first, count, g->pull.nvec, props, g->pull.hub_vid, g->pull.nhub, pc);
    grz_prof_end(g);
    return grz_cuda_check(g, cudaGetLastError(), "k_pr_gather");
}

// The gather over the source segments in order, each adding into the accumulators (which the
// apply of segmented iterations leaves all zero).  One profiler record spans all segments.
static int pr_gather_segments(grz_graph* g, const PRConst& pc0, const double* props)
{
    grz_prof_begin(g, GRZ_PROF_PR_GATHER);
    bool first = true;
    for (uint32_t sg = 0; sg < g->nseg; ++sg) {
        const uint64_t a = g->seg_first[sg], n = g->seg_first[sg + 1] - a;
        if (n == 0) continue;
        PRConst pc = pc0;
        if (!first) pc.K_out = nullptr;  // the iteration's constant once
        first = false;
        pr_gather_launch<double, true>(g, g->seg_nbr, g->seg_dst, a, n, g->seg_first[g->nseg], props, nullptr, 0u, pc);
    }
    if (first) {
        // no edges at all: the constant still has to be published
        k_pr_gather<double, true><<<1, PR_THREADS, 0, g->stream>>>(g->seg_nbr, g->seg_dst, 0, 0, 0, props, (uint32_t)g->V, g->pr_rowacc,
                                                                   nullptr, 0u, pc0); GRZ_COUNT_LAUNCH(g);
    }
    grz_prof_end(g);
    return grz_cuda_check(g, cudaGetLastError(), "k_pr_gather (segments)");
}

// one PageRank iteration: edge-pull gather + vertex phase (two kernels)
int grz_pr_fused_iteration(grz_graph* g, int write_double_props)
{
    if (g->V == 0) return GRZ_OK;
    const int k = g->pr_sum_cur;
    const double dV = (double)g->V;
    const uint32_t stride = blocks_for(g->V) + 1;  // each half of pr_sum holds up to blocks_for(V) partials
    PRConst pc;
    pc.part_in = g->pr_sum + (size_t)k * stride;
    pc.nparts = g->pr_nparts[k];
    pc.K_out = g->pr_K;
    pc.damping = g->pr_damping;
    pc.c = (1.0 - g->pr_damping) / dV;
    pc.nverts = dV;
    int rc = GRZ_OK;
    if (g->pr_segmode) {
        rc = pr_sync_d(g);
        if (rc == GRZ_OK) rc = pr_gather_segments(g, pc, (const double*)g->pr_d[g->pr_cur]);
    } else if (g->pr_dmode) {
        rc = pr_sync_d(g);
        if (rc == GRZ_OK) rc = pr_gather(g, 0, g->pull.nvec, pc, (const double*)g->pr_d[g->pr_cur]);
    } else {
        rc = pr_sync_fx(g);
        if (rc == GRZ_OK) rc = pr_gather(g, 0, g->pull.nvec, pc, (const u128*)g->pr_fx[g->pr_cur]);
    }
    if (rc) return rc;
    grz_prof_begin(g, GRZ_PROF_PR_APPLY);
    const uint64_t agrid = std::max<uint64_t>(1, std::min<uint64_t>((g->V + (uint64_t)PR_THREADS * PR_APPLY_U - 1) /
                                                                        ((uint64_t)PR_THREADS * PR_APPLY_U),
                                                                    (uint64_t)g->num_sms * PR_APPLY_RESIDENT));
    k_pr_apply<<<(unsigned)agrid, PR_THREADS, 0, g->stream>>>(g->pr_rowacc, g->pr_cut, g->pr_segmode, g->inv_deg, g->degree, g->V, g->pr_K,
                                                              g->pr_sum + (size_t)(k ^ 1) * stride, g->pr_damping, g->pr_fx[g->pr_cur ^ 1],
                                                              g->pr_dmode ? g->pr_d[g->pr_cur ^ 1] : nullptr,
                                                              write_double_props ? g->prop : nullptr); GRZ_COUNT_LAUNCH(g);
    grz_prof_end(g);
    GRZ_CK(g, cudaGetLastError());
    g->pr_nparts[k ^ 1] = (uint32_t)agrid;
    g->pr_fx_stale = g->pr_dmode;  // the new props are only in pr_d
    g->pr_rowacc_stale = 1;
    g->pr_cur ^= 1;
    g->pr_sum_cur = k ^ 1;
    g->pr_iters_done++;
    return GRZ_OK;
}

// resident blocks per SM of the persistent kernel (a cooperative launch needs them all resident)
template <typename P, int MINB>
static int pr_persistent_resident(grz_graph* g)
{
    static int resident[64] = {};
    if (g->device < 0 || g->device >= 64) return 1;
    if (!resident[g->device]) {
        int r = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_pr_persistent<P, MINB>, PR_THREADS, 0) != cudaSuccess || r < 1) {
            cudaGetLastError();
            r = 1;
        }
        resident[g->device] = r;
    }
    return resident[g->device];
}

// Whether grz_pr_iterate runs its iterations in one persistent launch.  Measured on GB300 (R-MAT
// 20, 16 iterations): two kernels 93 us per iteration, the persistent kernel (6 blocks per SM)
// 109 us: its gather must read the props through the coherent path (its apply rewrites them in
// the same launch) and holds fewer blocks per SM.  Two kernels stay the default.
int grz_pr_use_persistent(const grz_graph* g) { return g->tune.pr_persistent >= 2 && !g->pr_segmode; }

// `iters` PageRank iterations (gather + apply each) in one cooperative launch.  Synchronises the
// graph's stream to read the barrier's error word.  A wait that runs out returns GRZ_ERR_TIMEOUT
// and leaves the PageRank state uninitialised (grz_pr_init starts over).
int grz_pr_persistent_iterations(grz_graph* g, uint32_t iters)
{
    if (iters == 0 || g->V == 0) return GRZ_OK;
    if (!g->pr_bar) {
        GRZ_CK(g, cudaMalloc(&g->pr_bar, sizeof(PRBar)));
        GRZ_CK(g, cudaMallocHost(&g->pr_bar_host, sizeof(PRBar)));
    }
    int rc = g->pr_dmode ? pr_sync_d(g) : pr_sync_fx(g);
    if (rc) return rc;
    const bool eight = g->tune.pr_persistent == 3;
    const int resident = eight ? (g->pr_dmode ? pr_persistent_resident<double, 8>(g) : pr_persistent_resident<u128, 8>(g))
                               : (g->pr_dmode ? pr_persistent_resident<double, 6>(g) : pr_persistent_resident<u128, 6>(g));
    uint64_t want = g->tune.pr_grid ? g->tune.pr_grid : (uint64_t)g->num_sms * resident;
    want = std::min<uint64_t>(want, (uint64_t)g->num_sms * resident);  // co-resident
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, blocks_for(g->V)));  // partial slots
    const uint32_t stride = blocks_for(g->V) + 1;
    const bool timing = g->prof && g->prof->on;
    PRPersist q;
    memset(&q, 0, sizeof(q));
    q.nbr = g->pull.nbr;
    q.dstv = g->pull.shared;
    q.nvec = g->pull.nvec;
    q.V = (uint32_t)g->V;
    q.hub_vid = g->pull.hub_vid;
    q.nhub = g->pull.nhub;
    q.rowacc = g->pr_rowacc;
    q.cut = g->pr_cut;
    q.inv_deg = g->inv_deg;
    q.degree = g->degree;
    q.fx[0] = g->pr_fx[0];
    q.fx[1] = g->pr_fx[1];
    q.d[0] = g->pr_d[0];
    q.d[1] = g->pr_d[1];
    q.dmode = g->pr_dmode;
    q.cur = g->pr_cur;
    q.sum[0] = g->pr_sum;
    q.sum[1] = g->pr_sum + stride;
    q.sum_cur = g->pr_sum_cur;
    q.nparts0 = g->pr_nparts[g->pr_sum_cur];
    q.K = g->pr_K;
    q.damping = g->pr_damping;
    q.nverts = (double)g->V;
    q.c = (1.0 - g->pr_damping) / q.nverts;
    q.iters = iters;
    q.prop_out = nullptr;
    q.bar = (PRBar*)g->pr_bar;
    q.limit_ns = (unsigned long long)(g->tune.pr_wait_limit_us ? g->tune.pr_wait_limit_us : 2000000u) * 1000ull;
    q.withhold_block = (int)g->tune.pr_withhold - 1;
    q.time_phases = timing ? 1 : 0;
    GRZ_CK(g, cudaMemsetAsync(g->pr_bar, 0, 4 * sizeof(unsigned int), g->stream));
    void* args[] = { &q };
    const void* fn = eight ? (g->pr_dmode ? (const void*)k_pr_persistent<double, 8> : (const void*)k_pr_persistent<u128, 8>)
                           : (g->pr_dmode ? (const void*)k_pr_persistent<double, 6> : (const void*)k_pr_persistent<u128, 6>);
    GRZ_CK(g, cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(PR_THREADS), args, 0, g->stream));
    GRZ_COUNT_LAUNCH(g);
    const size_t rb = timing ? sizeof(PRBar) : 4 * sizeof(unsigned int);
    GRZ_CK(g, cudaMemcpyAsync(g->pr_bar_host, g->pr_bar, rb, cudaMemcpyDeviceToHost, g->stream));
    GRZ_CK(g, cudaStreamSynchronize(g->stream));
    const PRBar* hb = (const PRBar*)g->pr_bar_host;
    if (hb->err) {
        // the iteration stopped part-way: the accumulators and props are inconsistent
        GRZ_CK(g, cudaMemsetAsync(g->pr_rowacc, 0, sizeof(u128) * (g->V + 1), g->stream));
        g->pr_rowacc_stale = 0;
        g->pr_lists_changed = 1;
        return grz_set_error(g, GRZ_ERR_TIMEOUT, "PageRank grid barrier %u: a wait ran out after %u us", hb->where,
                             g->tune.pr_wait_limit_us ? g->tune.pr_wait_limit_us : 2000000u);
    }
    if (timing)
        for (uint32_t i = 0; i < iters && i < 64; ++i) {
            grz_prof_direct(g, GRZ_PROF_PR_GATHER, (float)(hb->gather_ns[i] * 1e-6));
            grz_prof_direct(g, GRZ_PROF_PR_APPLY, (float)(hb->apply_ns[i] * 1e-6));
        }
    if (iters & 1) {
        g->pr_cur ^= 1;
        g->pr_sum_cur ^= 1;
    }
    g->pr_nparts[g->pr_sum_cur] = grid;
    g->pr_fx_stale = g->pr_dmode;
    g->pr_rowacc_stale = 1;
    g->pr_iters_done += iters;
    return GRZ_OK;
}

// Edge-pull phase alone, over vectors [first, first+count).  Slices of the list (the reference's
// per-NUMA-node lists) may come in separate calls, in list order.  The call whose slice ends the
// list publishes the double accumulators and their exact sum into g->glob.
int grz_pr_edge_pull(grz_graph* g, uint64_t first, uint64_t count)
{
    if (g->V == 0) return GRZ_OK;
    int rc = grz_pr_rowacc_clean(g);
    if (rc == GRZ_OK) rc = pr_sync_fx(g);
    if (rc) return rc;
    PRConst pc;
    memset(&pc, 0, sizeof(pc));
    rc = pr_gather(g, first, count, pc, (const u128*)g->pr_fx[g->pr_cur]);
    if (rc) return rc;
    if (first + count < g->pull.nvec) return GRZ_OK;
    k_pr_accum_out<<<blocks_for(g->V), PR_THREADS, 0, g->stream>>>(g->pr_rowacc, g->V, g->accum, g->glob); GRZ_COUNT_LAUNCH(g);
    GRZ_CK(g, cudaGetLastError());
    return GRZ_OK;
}

// vertex phase over [first, first+count) with S from the reduce buffer
int grz_pr_vertex(grz_graph* g, uint64_t first, uint64_t count, double S)
{
    if (first >= g->V) return GRZ_OK;
    if (first + count > g->V) count = g->V - first;
    const double dV = (double)g->V;
    const double G = (1.0 - S) / dV;
    const double c = (1.0 - g->pr_damping) / dV;
    const double K = fma(G, g->pr_damping, c);
    int rc = pr_sync_fx(g);
    if (rc) return rc;
    g->pr_d_stale = g->pr_d[0] != nullptr;  // the props change in the fixed-point form only
    // the props being gathered are rewritten in place: the boundary path keeps one live copy
    k_pr_vertex<<<blocks_for(count), PR_THREADS, 0, g->stream>>>(g->accum, g->inv_deg, g->prop, g->pr_fx[g->pr_cur],
                                                                 first, count, g->pr_damping, K); GRZ_COUNT_LAUNCH(g);
    GRZ_CK(g, cudaGetLastError());
    return GRZ_OK;
}

// reference-format props (double) from the current fixed-point props
int grz_pr_props_to_double(grz_graph* g)
{
    if (g->V == 0) return GRZ_OK;
    if (g->pr_fx_stale) {
        // the double props convert exactly to the fixed-point ones; report what those round to
        k_double_to_fx<<<blocks_for(g->V), PR_THREADS, 0, g->stream>>>(g->pr_d[g->pr_cur], g->V, nullptr, g->prop); GRZ_COUNT_LAUNCH(g);
    } else {
        k_fx_to_double<<<blocks_for(g->V), PR_THREADS, 0, g->stream>>>(g->pr_fx[g->pr_cur], g->V, g->prop); GRZ_COUNT_LAUNCH(g);
    }
    GRZ_CK(g, cudaGetLastError());
    return GRZ_OK;
}

// ---------------------------------------------------------------------------------------------
// PageRank push (EDGE_FORCE_PUSH): source/phase_edge_push_pr.asm:42-354.  Each valid lane adds
// the source's prop to the destination's accumulator.  Here the accumulator is an exact u128
// (two 64-bit atomics with carry), so push and pull give bit-identical sums, in any order.

namespace {

__global__ void k_pr_push(const uint4* __restrict__ nbr, const uint32_t* __restrict__ shared, uint64_t first,
                          uint64_t count, const u128* __restrict__ prop_fx, u128* __restrict__ acc_fx,
                          u128* __restrict__ glob)
{
    __shared__ u128 red[PR_THREADS / 32];
    const uint64_t i = (uint64_t)blockIdx.x * PR_THREADS + threadIdx.x;
    u128 s = u128_zero();
    if (i < count) {
        const uint64_t v = first + i;
        const uint4 n = __ldg(nbr + v);
        const u128 msg = ld_fx(prop_fx, shared[v]);
        const uint32_t ids[4] = { n.x, n.y, n.z, n.w };
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            if (ids[l] == GRZ_INVALID_ID) continue;
            u128_atomic_add(&acc_fx[ids[l]], msg);
            s = u128_add(s, msg);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < PR_THREADS / 32) ? red[threadIdx.x] : u128_zero();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
        if (threadIdx.x == 0) u128_slot_add(glob, s);
    }
}

// accumulators (exact) -> double accumulators, then reset (phase_vertex_pr.asm:101-106)
__global__ void k_pr_push_accum_out(u128* __restrict__ acc_fx, double* __restrict__ accum, uint64_t first, uint64_t count)
{
    const uint64_t i = (uint64_t)blockIdx.x * PR_THREADS + threadIdx.x;
    if (i >= count) return;
    const uint64_t v = first + i;
    accum[v] = fx_to_double(acc_fx[v]);
    acc_fx[v] = u128_zero();
}

}  // namespace

int grz_pr_push_phase(grz_graph* g, uint64_t first_vec, uint64_t count)
{
    if (!g->push.nbr) return grz_set_error(g, GRZ_ERR_STATE, "push list not loaded");
    if (count == 0) return GRZ_OK;
    // the pull accumulators double as the push accumulators (all zero between uses)
    int rc = grz_pr_rowacc_clean(g);
    if (rc == GRZ_OK) rc = pr_sync_fx(g);
    if (rc) return rc;
    k_pr_push<<<blocks_for(count), PR_THREADS, 0, g->stream>>>(g->push.nbr, g->push.shared, first_vec, count,
                                                               g->pr_fx[g->pr_cur], g->pr_rowacc, g->glob); GRZ_COUNT_LAUNCH(g);
    GRZ_CK(g, cudaGetLastError());
    k_pr_push_accum_out<<<blocks_for(g->V), PR_THREADS, 0, g->stream>>>(g->pr_rowacc, g->accum, 0, g->V); GRZ_COUNT_LAUNCH(g);
    GRZ_CK(g, cudaGetLastError());
    return GRZ_OK;
}
