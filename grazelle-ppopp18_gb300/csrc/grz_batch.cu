// grz_batch.cu -- many personalized-PageRank and multi-source BFS instances over many graphs
// of uneven size, each run as one CUDA graph launch.
//
// The reference has no batching and no personalized PageRank.  PPR here is the reference's
// PageRank vertex phase (source/phase_vertex_pr.asm:75-134) with the teleport term and the
// dangling mass sent to the seed instead of spread over all vertices:
//   accum[v]   = sum over v's in-edges (u, v) of prop[u]        (edge-pull, phase_edge_pull_pr.asm)
//   S          = sum over v of accum[v]
//   rank'[v]   = d * accum[v] + [v == seed] * (d * (1 - S) + (1 - d))
//   prop'[v]   = rank'[v] / deg'(v)                              (deg' as the reference: V if 0)
// starting from rank = one-hot(seed).  Ranks sum to 1 in every iteration.
//
// GB300 design:
//   * The graphs become one block-diagonal union graph: each graph's vertex IDs are offset by
//     the vertices of the graphs before it, and the union is loaded as one grz_graph.  Kernels
//     never need to know where one graph ends; only the per-graph sums S do.
//   * Up to GRZ_BATCH_K (8) instances per graph share one pass over the edges.  Props are stored
//     [vertex][instance] in 4.124 fixed point (the apply converts each prop once), so the 8 lanes
//     that serve one vector's instances read one aligned 128-byte row per source: the random
//     gather costs one line for 8 instances instead of 8 lines, and no conversion per edge.
//   * PPR gather: a warp owns a tile of 32 vectors and walks it 4 vectors x 8 instances at a
//     time.  Lane (vector, instance) sums its four sources exactly; a shuffle scan over the 4
//     vectors and a carried running sum complete each destination inside the warp, with no
//     shared memory and no barrier.  Destinations complete inside the tile are stored, the (at
//     most two) cut by the tile edge are added with exact u128 atomics.  Sums are exact, so
//     results do not depend on the launch shape.
//   * PPR apply: thread per (vertex, instance); it reads S of its graph and instance (summed
//     exactly by the previous apply as sum deg(u) * prop(u)), writes the new props and clears
//     the accumulators.  The next S is summed in registers per graph, then per block in shared
//     memory, and reaches global memory with one atomic per block, graph and instance (one
//     cache line per graph would otherwise take an atomic from every 32 vertices).
//   * Multi-source BFS: bit-parallel, 8 roots per graph.  visited / frontier are one byte per
//     vertex (bit i = instance i).  Pull: a vector's new bits are the OR of its sources'
//     frontier bytes, reduced per destination within the warp, minus the visited bits; the
//     vertex pass sets level = iteration for each new bit.  Levels are exact (level-synchronous).
//   * The PPR iteration loop (fixed count) and the BFS loop (WHILE until no new bit, decided on
//     the device) are each captured once as a CUDA graph and replayed.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "grz_internal.cuh"
#include "../../include/grazelle_gb300.h"

namespace {

constexpr int K = GRZ_BATCH_K;  // instances per graph (8)
constexpr int GT = 256;         // threads per block: 32 vectors (or vertices) x 8 instances
constexpr int TV = GT / K;      // vectors per gather tile
constexpr uint32_t NONE = 0xffffffffu;
constexpr int MAX_GRAPHS = 1024;

__device__ __forceinline__ u128 shfl_up_u128(u128 v, int off)
{
    u128 r;
    r.lo = __shfl_up_sync(0xffffffffu, v.lo, off);
    r.hi = __shfl_up_sync(0xffffffffu, v.hi, off);
    return r;
}

// graph of union vertex v (voff: G+1 ascending offsets in shared memory)
__device__ __forceinline__ uint32_t graph_of(const uint32_t* voff, uint32_t G, uint32_t v)
{
    uint32_t lo = 0, hi = G - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (voff[mid] <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// initial PPR state: prop = one-hot(seed) / deg'; S = deg(seed) * prop(seed) per (graph, instance).
// The props are 4.124 fixed point (prop) or the doubles they are the exact conversions of (propd).
__global__ void k_ppr_init(const uint32_t* __restrict__ seeds, uint32_t G, const double* __restrict__ inv_deg,
                           const uint32_t* __restrict__ degree, u128* __restrict__ prop, double* __restrict__ propd,
                           u128* __restrict__ S)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= G * K) return;
    const uint32_t s = seeds[t];
    const uint32_t i = t % K;
    u128 v = u128_zero();
    if (s != NONE) {
        const u128 p = fx_from_double(inv_deg[s]);
        if (propd) propd[(uint64_t)s * K + i] = inv_deg[s];
        else prop[(uint64_t)s * K + i] = p;
        v = u128_mul32(p, degree[s]);
    }
    S[t] = v;
}

__device__ __forceinline__ u128 ldg_u128(const u128* p)
{
    const ulonglong2 q = __ldg(reinterpret_cast<const ulonglong2*>(p));
    u128 r;
    r.lo = q.x;
    r.hi = q.y;
    return r;
}

// edge-pull of all instances (see the file comment).  Warp-level tiles of TV = 32 vectors,
// persistent over the grid's warps.  A warp walks its tile in 8 steps of 4 vectors x 8 instances
// (lane = 8 * slot + instance): it sums each lane's four sources exactly, scans the step's 4
// vectors per instance (keys ascend, so equal keys form one run), and carries the open
// destination's running sum into the next step.  A destination whose vectors all lie in the
// tile is stored once by the lane of its last vector; one cut by the tile edge is added with
// exact u128 atomics.  Block 0 first clears S_next for the apply that follows.
constexpr int GSTEPS = TV / 4;  // steps of 4 vectors per tile
constexpr int GCHUNK = 2;       // steps whose loads are issued together
// 6 blocks per SM: occupancy beats deeper per-warp load batches (GB300 sweep over steps per
// chunk 1-8 and 4-8 blocks per SM: 99.8 ms per 256-instance run here, 102-163 ms elsewhere)
constexpr int GATHER_RESIDENT = 6;

// a gathered prop in fixed point: read as such, or converted (exactly) from the double it came from
__device__ __forceinline__ u128 ld_prop(const u128* p) { return ldg_u128(p); }
__device__ __forceinline__ u128 ld_prop(const double* p) { return fx_from_double(__ldg(p)); }

__device__ __forceinline__ u128 shfl_u128(u128 v, int src)
{
    u128 r;
    r.lo = __shfl_sync(0xffffffffu, v.lo, src);
    r.hi = __shfl_sync(0xffffffffu, v.hi, src);
    return r;
}

template <typename P>
__global__ void __launch_bounds__(GT, GATHER_RESIDENT) k_ppr_gather(const uint4* __restrict__ nbr, const uint32_t* __restrict__ dstv,
                                                   uint64_t nvec, uint32_t V, const P* __restrict__ prop,
                                                   u128* __restrict__ rowacc, u128* __restrict__ S_next, uint32_t nS)
{
    if (blockIdx.x == 0)
        for (uint32_t k = threadIdx.x; k < nS; k += GT) S_next[k] = u128_zero();
    const int lane = threadIdx.x & 31;
    const int q = lane / K, inst = lane % K;
    const uint64_t ntiles = (nvec + TV - 1) / TV;
    const uint64_t nwarps = (uint64_t)gridDim.x * (GT / 32);
    for (uint64_t tile = (uint64_t)blockIdx.x * (GT / 32) + (threadIdx.x >> 5); tile < ntiles; tile += nwarps) {
        const uint64_t v0 = tile * TV;
        // the tile's 32 keys, one per lane (NONE past the list), and the keys either side of it
        const uint32_t kall = v0 + lane < nvec ? __ldcs(dstv + v0 + lane) : NONE;
        const uint32_t kbefore = v0 > 0 ? __ldg(dstv + v0 - 1) : NONE - 1;
        const uint32_t kafter = v0 + TV < nvec ? __ldg(dstv + v0 + TV) : NONE - 1;
        u128 carry = u128_zero();
        uint32_t ckey = NONE - 1;  // destination of the open run carried from the previous step
#pragma unroll
        for (int h = 0; h < GSTEPS; h += GCHUNK) {
            u128 val[GCHUNK];
#pragma unroll
            for (int j = 0; j < GCHUNK; ++j) {
                const uint64_t v = v0 + (uint64_t)(h + j) * 4 + q;
                val[j] = u128_zero();
                if (v < nvec) {
                    const uint4 sv = __ldg(nbr + v);
                    const uint32_t ids[4] = { sv.x, sv.y, sv.z, sv.w };
#pragma unroll
                    for (int l = 0; l < 4; ++l)
                        if (ids[l] < V) val[j] = u128_add(val[j], ld_prop(prop + (uint64_t)ids[l] * K + inst));
                }
            }
#pragma unroll
            for (int j = 0; j < GCHUNK; ++j) {
                const int pos = (h + j) * 4 + q;  // vector of this lane within the tile
                u128 x = val[j];
                const uint32_t k = __shfl_sync(0xffffffffu, kall, pos);
#pragma unroll
                for (int off = 1; off < 4; off <<= 1) {
                    const u128 o = shfl_up_u128(x, off * K);
                    const uint32_t ko = __shfl_sync(0xffffffffu, kall, pos >= off ? pos - off : 0);
                    if (q >= off && ko == k) x = u128_add(x, o);
                }
                if (k == ckey) x = u128_add(x, carry);
                const uint32_t kn_in = __shfl_sync(0xffffffffu, kall, (pos + 1) & (TV - 1));  // every lane shuffles
                const uint32_t kn = pos + 1 < TV ? kn_in : kafter;
                const bool tail = kn != k;
                if (k != NONE && (tail || pos == TV - 1)) {
                    u128* dst = rowacc + (uint64_t)k * K + inst;
                    if (tail && k != kbefore) *dst = x;                // every vector of k is in this tile
                    else if (x.lo | x.hi) u128_atomic_add(dst, x);     // cut by the tile edge
                }
                carry = shfl_u128(x, 3 * K + inst);
                ckey = __shfl_sync(0xffffffffu, k, 3 * K + inst);
            }
        }
    }
}

constexpr int APPLY_SLOTS = 64;  // graphs whose next S a block sums in shared memory (beyond: global atomics)
#ifndef GRZ_PPR_APPLY_U
#define GRZ_PPR_APPLY_U 1
#endif
#ifndef GRZ_PPR_APPLY_MINB
#define GRZ_PPR_APPLY_MINB 8
#endif
// Tiles whose accumulators a thread loads before it stores anything, and resident apply blocks
// per SM.  GB300 sweep (256 PPR x 20 iterations on the 32-graph batch): 8 tiles at 3 blocks per SM
// (80 registers) 100.9 ms, 4 at 4 95.3 ms, 2 at 6 91.5 ms, 1 at 8 (32 registers) 89.7 ms: the
// apply wants every warp slot more than loads in flight per thread.
constexpr int APPLY_U = GRZ_PPR_APPLY_U;

// bit j of word t: vertex 32t + j has pull vectors in two or more gather tiles, so its
// accumulator is summed with atomics and the apply must clear it.  Every other accumulator is
// either stored whole by each gather or never written (no in-edges), and needs no clearing.
__global__ void k_ppr_cutbits(const uint32_t* __restrict__ rowptr, uint32_t V, uint32_t* __restrict__ cut)
{
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    bool c = false;
    if (v < V) {
        const uint32_t r0 = rowptr[v], r1 = rowptr[v + 1];
        c = r1 > r0 && r0 / TV != (r1 - 1) / TV;
    }
    const unsigned m = __ballot_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0 && v < V) cut[v / 32] = m;
}

__device__ __forceinline__ void s_flush(u128* s_part, u128* S_next, uint32_t g, int inst, u128 x)
{
    if ((x.lo | x.hi) == 0) return;
    if (g < (uint32_t)APPLY_SLOTS) u128_atomic_add(s_part + g * K + inst, x);
    else u128_atomic_add(S_next + (uint64_t)g * K + inst, x);
}

// vertex phase of all instances; thread per (vertex, instance).  The grid strides over tiles of
// 32 vertices (all blocks on one moving front of the arrays), APPLY_U tiles at a time: their
// accumulators are loaded first, then the tiles are finished in order.
__global__ void __launch_bounds__(GT, GRZ_PPR_APPLY_MINB) k_ppr_apply(u128* __restrict__ rowacc, const uint32_t* __restrict__ cut,
                                                     const double* __restrict__ inv_deg,
                                                     const uint32_t* __restrict__ degree, uint32_t V,
                                                     const uint32_t* __restrict__ voff_g, uint32_t G,
                                                     const uint32_t* __restrict__ seeds, double damping,
                                                     const u128* __restrict__ S_cur, u128* __restrict__ S_next,
                                                     u128* __restrict__ prop_out, double* __restrict__ propd_out,
                                                     double* __restrict__ rank_out)
{
    __shared__ uint32_t voff[MAX_GRAPHS + 1];
    __shared__ u128 s_part[APPLY_SLOTS * K];
    const uint32_t nslots = (G < (uint32_t)APPLY_SLOTS ? G : (uint32_t)APPLY_SLOTS) * K;
    for (uint32_t k = threadIdx.x; k <= G; k += GT) voff[k] = voff_g[k];
    for (uint32_t k = threadIdx.x; k < nslots; k += GT) s_part[k] = u128_zero();
    __syncthreads();
    const uint64_t ntiles = ((uint64_t)V + TV - 1) / TV;
    const int inst = threadIdx.x % K, lv = threadIdx.x / K;
    // per-thread state of the graph of its current vertex (vertices ascend); the seed's teleport
    // term d * (1 - S) + (1 - d) is computed once per graph
    uint32_t g = 0, gend = 0, seed = NONE;
    double cseed = 0.0;
    u128 acc = u128_zero();
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += (uint64_t)APPLY_U * gridDim.x) {
        u128 a[APPLY_U];
        uint32_t cw[APPLY_U];
#pragma unroll
        for (int j = 0; j < APPLY_U; ++j) {
            const uint64_t t = tile + (uint64_t)j * gridDim.x;
            const uint64_t v = t * TV + lv;
            a[j] = u128_zero();
            cw[j] = 0;
            if (v < V) {
                const ulonglong2 q = *(reinterpret_cast<const ulonglong2*>(rowacc) + v * K + inst);
                a[j].lo = q.x;
                a[j].hi = q.y;
                cw[j] = __ldg(cut + t);
            }
        }
#pragma unroll
        for (int j = 0; j < APPLY_U; ++j) {
            const uint64_t v64 = (tile + (uint64_t)j * gridDim.x) * TV + lv;
            if (v64 >= V) break;
            const uint32_t v = (uint32_t)v64;
            if (v >= gend) {
                s_flush(s_part, S_next, g, inst, acc);
                acc = u128_zero();
                g = graph_of(voff, G, v);
                gend = voff[g + 1];
                seed = seeds[g * K + inst];
                const double S = fx_to_double(S_cur[g * K + inst]);
                cseed = __dadd_rn(__dmul_rn(damping, 1.0 - S), 1.0 - damping);
            }
            const uint64_t idx = (uint64_t)v * K + inst;
            const bool mass = (a[j].lo | a[j].hi) != 0;
            if (mass && ((cw[j] >> lv) & 1u)) rowacc[idx] = u128_zero();
            // rank' = fma(accum, d, [v == seed] * teleport); zero without mass (most vertices early on)
            double rank = 0.0, pd = 0.0;
            u128 p = u128_zero();
            if (seed != NONE && (mass || v == seed)) {
                rank = __fma_rn(fx_to_double(a[j]), damping, v == seed ? cseed : 0.0);
                pd = __dmul_rn(rank, __ldg(inv_deg + v));
                p = fx_from_double(pd);
                if (p.lo | p.hi) acc = u128_add(acc, u128_mul32(p, __ldg(degree + v)));
            }
            if (propd_out) propd_out[idx] = pd;  // the gather converts it to p
            else *(reinterpret_cast<ulonglong2*>(prop_out) + idx) = make_ulonglong2(p.lo, p.hi);
            if (rank_out) rank_out[idx] = rank;
        }
    }
    s_flush(s_part, S_next, g, inst, acc);
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < nslots; k += GT) {
        const u128 x = s_part[k];
        if (x.lo | x.hi) u128_atomic_add(S_next + k, x);
    }
}

// ----------------------------------------------------------------------------------------------
// multi-source BFS

__global__ void k_msbfs_init(const uint32_t* __restrict__ roots, uint32_t n, uint8_t* __restrict__ visited,
                             uint8_t* __restrict__ frontier, int32_t* __restrict__ level, uint32_t* __restrict__ iter)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0 && iter) *iter = 1;  // the first iteration
    if (t >= n) return;
    const uint32_t r = roots[t];
    if (r == NONE) return;
    const uint32_t bit = 1u << (t % K);
    // several instances may share a root: byte-wise OR through the containing word
    atomicOr(reinterpret_cast<unsigned*>(visited) + (r >> 2), bit << (8 * (r & 3)));
    atomicOr(reinterpret_cast<unsigned*>(frontier) + (r >> 2), bit << (8 * (r & 3)));
    level[(uint64_t)r * K + t % K] = 0;
}

// pull: new bits of each destination = OR of its sources' frontier bytes, minus its visited bits
__global__ void __launch_bounds__(256) k_msbfs_pull(const uint4* __restrict__ nbr, const uint32_t* __restrict__ dstv, uint64_t nvec,
                                                    uint32_t V, const uint8_t* __restrict__ frontier,
                                                    const uint8_t* __restrict__ visited, unsigned* __restrict__ next_words)
{
    const int lane = threadIdx.x & 31;
    const uint64_t ntiles = (nvec + 255) / 256;
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const uint64_t v = t * 256 + threadIdx.x;
        uint32_t key = NONE, m = 0;
        if (v < nvec) {
            key = __ldcs(dstv + v);
            if (visited[key] != 0xffu) {
                const uint4 s = __ldcs(nbr + v);
                const uint32_t ids[4] = { s.x, s.y, s.z, s.w };
#pragma unroll
                for (int l = 0; l < 4; ++l)
                    if (ids[l] < V) m |= frontier[ids[l]];
            }
        }
        const uint32_t prevkey = __shfl_up_sync(0xffffffffu, key, 1);
        const uint32_t nextkey = __shfl_down_sync(0xffffffffu, key, 1);
        const bool head = lane == 0 || key != prevkey;
        const bool tail = lane == 31 || key != nextkey;
        const unsigned heads = __ballot_sync(0xffffffffu, head);
        const int segstart = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
        const int maxlen = __reduce_max_sync(0xffffffffu, (unsigned)(lane - segstart + 1));
        for (int off = 1; off < maxlen; off <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, m, off);
            if (lane - off >= segstart) m |= o;
        }
        if (tail && key != NONE) {
            const uint32_t nb = m & ~(uint32_t)visited[key] & 0xffu;
            if (nb) atomicOr(next_words + (key >> 2), nb << (8 * (key & 3)));
        }
    }
}

// vertex pass: four vertices (one word) per thread; counts the new bits
__global__ void __launch_bounds__(256) k_msbfs_vertex(unsigned* __restrict__ next_words, unsigned* __restrict__ visited_words,
                                                      unsigned* __restrict__ frontier_words, int32_t* __restrict__ level,
                                                      uint32_t V, const uint32_t* __restrict__ iter,
                                                      unsigned long long* __restrict__ changed)
{
    const uint32_t W = (V + 3) / 4;
    const uint32_t k = *iter;
    unsigned long long cnt = 0;
    for (uint32_t w = blockIdx.x * 256 + threadIdx.x; w < W; w += gridDim.x * 256) {
        const unsigned nx = next_words[w];
        const unsigned vis = visited_words[w];
        const unsigned nb = nx & ~vis;
        frontier_words[w] = nb;
        if (nx) next_words[w] = 0;
        if (nb) {
            visited_words[w] = vis | nb;
            cnt += __popc(nb);
            for (int b = 0; b < 4; ++b) {
                unsigned bits = (nb >> (8 * b)) & 0xffu;
                const uint32_t v = w * 4 + b;
                while (bits) {
                    const int i = __ffs(bits) - 1;
                    bits &= bits - 1;
                    level[(uint64_t)v * K + i] = (int32_t)k;
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(changed, cnt);
}

// %globaltimer into *out (one thread): the branch timers of the combined PPR + BFS graph
__global__ void k_stamp(unsigned long long* __restrict__ out)
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *out = t;
}

// end of a BFS iteration: stop when no bit changed or the bound is reached; next iteration number
__global__ void k_msbfs_decide(unsigned long long* __restrict__ ctl, uint32_t* __restrict__ iter, uint32_t max_iter,
                               cudaGraphConditionalHandle loop)
{
    // ctl[0] changed in this iteration, ctl[1] iterations with a change, ctl[2] bound hit
    // (1: iterations, 2: time), ctl[3] %globaltimer of the first decision
    unsigned long long now;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
    if (ctl[3] == 0) ctl[3] = now;
    const unsigned long long c = ctl[0];
    ctl[0] = 0;
    unsigned run = c != 0;
    if (run) ctl[1] += 1;
    if (run && *iter >= max_iter) { run = 0; ctl[2] = 1; }
    if (run && now - ctl[3] > 120ull * 1000000000ull) { run = 0; ctl[2] = 2; }
    if (run) *iter += 1;
    cudaGraphSetConditional(loop, run);
}

}  // namespace

// ----------------------------------------------------------------------------------------------

struct grz_batch {
    int device;
    cudaStream_t stream;
    int own_stream;
    grz_graph* u;                        // the union graph
    std::vector<uint32_t> voff;          // G+1 vertex offsets
    std::vector<uint64_t> Vg, Eg;
    std::vector<std::vector<uint64_t>> pairs;  // pending pull pairs per graph (until build)
    uint32_t* d_voff;
    uint32_t* d_seeds;                   // [G][K] union vertex IDs or NONE
    // PPR
    u128* prop[2];                       // [vertex][instance] 4.124 fixed point
    double* propd[2];                    // the same props as the doubles they convert from exactly
    int ppr_props;                       // tuning: 0 or 1 fixed point, 2 doubles
    int ppr_dmode;                       // the captured loop gathers propd
    double* rank;
    u128* rowacc;
    uint32_t* cut;                       // [V/32] accumulators the apply clears (k_ppr_cutbits)
    u128* S[2];
    cudaGraphExec_t ppr_exec;
    uint32_t ppr_iters;
    double ppr_damping;
    int ppr_final;                        // which prop buffer the last replay wrote
    // BFS
    uint8_t* visited;
    uint8_t* frontier;
    unsigned* next_words;
    int32_t* level;
    unsigned long long* ctl;             // changed, iterations, bound hit
    uint32_t* iter;
    cudaGraphExec_t bfs_exec;
    // PPR and BFS together: one graph whose two branches run the two loops side by side
    uint32_t* d_roots;                   // [G][K] BFS roots of the combined run
    cudaGraphExec_t run_exec;
    uint32_t run_iters;
    double run_damping;
    int run_dmode;
    unsigned long long* stamps;          // PPR start / end, BFS start / end (%globaltimer, written inside the graph)
    int ppr_blocks, bfs_blocks;          // resident blocks per SM of the persistent kernels
    void* mail;                          // pinned host read-back
    char err[256];
};

static int bset(grz_batch* b, int code, const char* msg)
{
    snprintf(b->err, sizeof(b->err), "%s", msg);
    return code;
}

static int bck(grz_batch* b, cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return GRZ_OK;
    cudaGetLastError();
    snprintf(b->err, sizeof(b->err), "%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? GRZ_ERR_NOMEM : GRZ_ERR_CUDA;
}
#define BCK(b, x) do { int rc_ = bck((b), (x), #x); if (rc_) return rc_; } while (0)

static unsigned persistent_grid(const grz_batch* b, uint64_t work_blocks, int per_sm)
{
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(work_blocks, (uint64_t)b->u->num_sms * per_sm));
}

extern "C" int grz_batch_create(grz_batch** out, int device, void* stream)
{
    if (!out) return GRZ_ERR_ARG;
    *out = nullptr;
    grz_batch* b = new (std::nothrow) grz_batch();
    if (!b) return GRZ_ERR_NOMEM;
    b->device = device;
    int rc = grz_graph_create(&b->u, device, stream);
    if (rc) { delete b; return rc; }
    b->stream = b->u->stream;
    b->voff.push_back(0);
    b->ppr_blocks = 8;
    b->bfs_blocks = 8;
    *out = b;
    return GRZ_OK;
}

static void free_state(grz_batch* b)
{
    void* p[] = { b->d_voff, b->d_seeds, b->d_roots, b->stamps, b->prop[0], b->prop[1], b->propd[0], b->propd[1], b->rank, b->rowacc, b->cut, b->S[0], b->S[1],
                  b->visited, b->frontier, b->next_words, b->level, b->ctl, b->iter };
    for (void* x : p) cudaFree(x);
    b->d_voff = b->d_seeds = b->d_roots = nullptr;
    b->stamps = nullptr;
    b->prop[0] = b->prop[1] = nullptr;
    b->propd[0] = b->propd[1] = nullptr;
    b->rank = nullptr;
    b->rowacc = b->S[0] = b->S[1] = nullptr;
    b->cut = nullptr;
    b->visited = b->frontier = nullptr;
    b->next_words = nullptr;
    b->level = nullptr;
    b->ctl = nullptr;
    b->iter = nullptr;
    if (b->ppr_exec) cudaGraphExecDestroy(b->ppr_exec);
    if (b->bfs_exec) cudaGraphExecDestroy(b->bfs_exec);
    if (b->run_exec) cudaGraphExecDestroy(b->run_exec);
    b->ppr_exec = b->bfs_exec = b->run_exec = nullptr;
}

extern "C" void grz_batch_destroy(grz_batch* b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    free_state(b);
    if (b->mail) cudaFreeHost(b->mail);

    grz_graph_destroy(b->u);
    delete b;
}

extern "C" const char* grz_batch_last_error(const grz_batch* b) { return b ? b->err : ""; }

// Adds one graph: V vertices, E edges as interleaved (src, dst) pairs sorted by (dst, src) (the
// -pull order, source/graphdata.c:957).  Copied; the union is built by grz_batch_build.
extern "C" int grz_batch_add_graph(grz_batch* b, uint64_t V, uint64_t E, const uint64_t* pull_pairs)
{
    if (!b || V == 0 || (E > 0 && !pull_pairs)) return GRZ_ERR_ARG;
    if (b->voff.size() > MAX_GRAPHS) return bset(b, GRZ_ERR_RANGE, "too many graphs");
    if (V < TV) return bset(b, GRZ_ERR_RANGE, "a batched graph needs at least 32 vertices");
    const uint64_t base = b->voff.back();
    if (base + V >= GRZ_HUB_BASE) return bset(b, GRZ_ERR_RANGE, "the union exceeds 2^31 vertices");
    std::vector<uint64_t> p(2 * E);
    for (uint64_t e = 0; e < E; ++e) {
        const uint64_t s = pull_pairs[2 * e], d = pull_pairs[2 * e + 1];
        if (s >= V || d >= V) return bset(b, GRZ_ERR_RANGE, "vertex ID out of range");
        if (e > 0) {
            const uint64_t ps = pull_pairs[2 * e - 2], pd = pull_pairs[2 * e - 1];
            if (d < pd || (d == pd && s < ps)) return bset(b, GRZ_ERR_UNSORTED, "pairs are not in (dst, src) order");
        }
        p[2 * e] = s + base;
        p[2 * e + 1] = d + base;
    }
    b->pairs.push_back(std::move(p));
    b->Vg.push_back(V);
    b->Eg.push_back(E);
    b->voff.push_back((uint32_t)(base + V));
    return GRZ_OK;
}

extern "C" int grz_batch_build(grz_batch* b)
{
    if (!b || b->pairs.empty()) return GRZ_ERR_ARG;
    BCK(b, cudaSetDevice(b->device));
    free_state(b);
    uint64_t E = 0;
    for (uint64_t e : b->Eg) E += e;
    std::vector<uint64_t> all;
    all.reserve(2 * E);
    for (auto& p : b->pairs) all.insert(all.end(), p.begin(), p.end());
    const uint64_t V = b->voff.back();
    int rc = grz_graph_load_pairs(b->u, V, E, E ? all.data() : nullptr, nullptr);
    if (rc) return bset(b, rc, grz_graph_last_error(b->u));
    const uint32_t G = (uint32_t)b->Vg.size();
    BCK(b, cudaMalloc((void**)&b->d_voff, sizeof(uint32_t) * (G + 1)));
    BCK(b, cudaMemcpy(b->d_voff, b->voff.data(), sizeof(uint32_t) * (G + 1), cudaMemcpyHostToDevice));
    BCK(b, cudaMalloc((void**)&b->d_seeds, sizeof(uint32_t) * G * K));
    BCK(b, cudaMalloc((void**)&b->d_roots, sizeof(uint32_t) * G * K));
    if (!b->mail) BCK(b, cudaMallocHost(&b->mail, 64));
    return GRZ_OK;
}

extern "C" int grz_batch_info(const grz_batch* b, uint64_t* graphs, uint64_t* vertices, uint64_t* edges, uint64_t* vectors)
{
    if (!b) return GRZ_ERR_ARG;
    if (graphs) *graphs = b->Vg.size();
    if (vertices) *vertices = b->voff.back();
    if (edges) *edges = b->u->E;
    if (vectors) *vectors = b->u->pull.nvec;
    return GRZ_OK;
}

static int upload_seeds(grz_batch* b, const uint32_t* local, uint32_t k, uint32_t* dst = nullptr)
{
    if (!dst) dst = b->d_seeds;
    const uint32_t G = (uint32_t)b->Vg.size();
    std::vector<uint32_t> s((size_t)G * K, NONE);
    for (uint32_t g = 0; g < G; ++g)
        for (uint32_t i = 0; i < k; ++i) {
            const uint32_t x = local[(size_t)g * k + i];
            if (x == NONE) continue;
            if (x >= b->Vg[g]) return bset(b, GRZ_ERR_ARG, "seed or root outside its graph");
            s[(size_t)g * K + i] = b->voff[g] + x;
        }
    BCK(b, cudaMemcpyAsync(dst, s.data(), sizeof(uint32_t) * s.size(), cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    return GRZ_OK;
}

// Enqueues the fixed-length PPR loop (gather + apply per iteration) on cs, which is capturing.
// Returns the prop buffer the last iteration wrote.
static int enqueue_ppr_chain(grz_batch* b, cudaStream_t cs, uint32_t iterations, double damping, int dmode, const uint32_t* seeds,
                             int* final_cur)
{
    grz_graph* u = b->u;
    const uint32_t V = (uint32_t)u->V, G = (uint32_t)b->Vg.size();
    // the gather's unit is a warp tile of TV vectors; blocks beyond residency would only queue
    int gres = 0;
    const cudaError_t oe = dmode ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&gres, k_ppr_gather<double>, GT, 0)
                                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&gres, k_ppr_gather<u128>, GT, 0);
    if (oe != cudaSuccess || gres < 1) {
        cudaGetLastError();
        gres = 1;
    }
    const uint64_t gtiles = (u->pull.nvec + TV - 1) / TV;
    const unsigned ggrid = persistent_grid(b, (gtiles + GT / 32 - 1) / (GT / 32), std::min(b->ppr_blocks, gres));
    // GRZ_PPR_APPLY_MINB blocks per SM fit the apply's registers
    const unsigned agrid = persistent_grid(b, (V + TV - 1) / TV, std::min(b->ppr_blocks, GRZ_PPR_APPLY_MINB));
    int cur = 0;
    for (uint32_t it = 0; it < iterations; ++it) {
        if (dmode)
            k_ppr_gather<<<ggrid, GT, 0, cs>>>(u->pull.nbr, u->pull.shared, u->pull.nvec, V, b->propd[cur], b->rowacc, b->S[cur ^ 1], G * K);
        else
            k_ppr_gather<<<ggrid, GT, 0, cs>>>(u->pull.nbr, u->pull.shared, u->pull.nvec, V, b->prop[cur], b->rowacc, b->S[cur ^ 1], G * K);
        k_ppr_apply<<<agrid, GT, 0, cs>>>(b->rowacc, b->cut, u->inv_deg, u->degree, V, b->d_voff, G, seeds, damping, b->S[cur],
                                         b->S[cur ^ 1], b->prop[cur ^ 1], dmode ? b->propd[cur ^ 1] : nullptr,
                                         it + 1 == iterations ? b->rank : nullptr);
        cur ^= 1;
        const int rc = bck(b, cudaGetLastError(), "ppr launch");
        if (rc) return rc;
    }
    *final_cur = cur;
    return GRZ_OK;
}

// the fixed-length PPR iteration loop as one CUDA graph (gather + apply per iteration)
static int build_ppr_graph(grz_batch* b, uint32_t iterations, double damping, int dmode)
{
    if (b->ppr_exec) { cudaGraphExecDestroy(b->ppr_exec); b->ppr_exec = nullptr; }
    cudaStream_t cs = nullptr;
    BCK(b, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    int cur = 0;
    int rc = bck(b, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (!rc) rc = enqueue_ppr_chain(b, cs, iterations, damping, dmode, b->d_seeds, &cur);
    const cudaError_t e = cudaStreamEndCapture(cs, &graph);
    if (!rc) rc = bck(b, e, "end capture");
    if (!rc) rc = bck(b, cudaGraphInstantiate(&b->ppr_exec, graph, 0), "instantiate");
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (rc) { b->ppr_exec = nullptr; return rc; }
    b->ppr_iters = iterations;
    b->ppr_damping = damping;
    b->ppr_final = cur;
    b->ppr_dmode = dmode;
    return GRZ_OK;
}

// the PPR state (props, ranks, accumulators, straddle bits), allocated on first use
static int ppr_alloc(grz_batch* b, int dmode)
{
    grz_graph* u = b->u;
    const uint64_t V = u->V;
    const uint32_t G = (uint32_t)b->Vg.size();
    if (!b->prop[0]) {
        BCK(b, cudaMalloc((void**)&b->prop[0], sizeof(u128) * V * K));
        BCK(b, cudaMalloc((void**)&b->prop[1], sizeof(u128) * V * K));
        BCK(b, cudaMalloc((void**)&b->rank, sizeof(double) * V * K));
        BCK(b, cudaMalloc((void**)&b->rowacc, sizeof(u128) * (V + 1) * K));
        BCK(b, cudaMalloc((void**)&b->S[0], sizeof(u128) * G * K));
        BCK(b, cudaMalloc((void**)&b->S[1], sizeof(u128) * G * K));
        BCK(b, cudaMemsetAsync(b->rowacc, 0, sizeof(u128) * (V + 1) * K, b->stream));
        BCK(b, cudaMalloc((void**)&b->cut, sizeof(uint32_t) * ((V + 31) / 32)));
        k_ppr_cutbits<<<(unsigned)((V + 255) / 256), 256, 0, b->stream>>>(u->pull.rowptr, (uint32_t)V, b->cut);
        BCK(b, cudaGetLastError());
    }
    if (dmode && !b->propd[0]) {
        BCK(b, cudaMalloc((void**)&b->propd[0], sizeof(double) * V * K));
        BCK(b, cudaMalloc((void**)&b->propd[1], sizeof(double) * V * K));
    }
    return GRZ_OK;
}

// k seeds per graph (local vertex IDs, NONE = unused instance), `iterations` PPR iterations;
// ranks out as [union vertex][k] (graph g's vertex v at row voff[g] + v)
extern "C" int grz_batch_ppr(grz_batch* b, const uint32_t* seeds, uint32_t k, uint32_t iterations, double damping,
                             double* ranks_out, grz_run_stats_t* stats)
{
    if (!b || !seeds || k == 0 || k > (uint32_t)K || iterations == 0 || !(damping >= 0.0 && damping <= 1.0)) return GRZ_ERR_ARG;
    if (!b->d_seeds) return bset(b, GRZ_ERR_STATE, "grz_batch_build not called");
    BCK(b, cudaSetDevice(b->device));
    grz_graph* u = b->u;
    const uint64_t V = u->V;
    const uint32_t G = (uint32_t)b->Vg.size();
    // Doubles gathered instead of 16-byte fixed point only when chosen: each row of a source's 8
    // instances is 64 bytes instead of 128, and the gather converts each double exactly to the
    // fixed point the apply would have stored, so the sums and results are the same bit for bit.
    // The gather is bound by L1TEX and instructions, not DRAM, so the conversions cost more than
    // the halved rows save: GB300, the 32-graph batch (1.9 GB of fixed-point rows, 15x L2), 256
    // instances x 20 iterations: 101 ms fixed point, 155 ms doubles.
    const int dmode = b->ppr_props == 2;
    int rc = ppr_alloc(b, dmode);
    if (rc) return rc;
    rc = upload_seeds(b, seeds, k);
    if (rc) return rc;
    if (!b->ppr_exec || b->ppr_iters != iterations || b->ppr_damping != damping || b->ppr_dmode != dmode) {
        rc = build_ppr_graph(b, iterations, damping, dmode);
        if (rc) return rc;
    }
    cudaEvent_t e0, e1;
    BCK(b, cudaEventCreate(&e0));
    BCK(b, cudaEventCreate(&e1));
    cudaStream_t st = b->stream;
    rc = bck(b, cudaEventRecord(e0, st), "event");
    if (!rc && dmode) rc = bck(b, cudaMemsetAsync(b->propd[0], 0, sizeof(double) * V * K, st), "memset");
    if (!rc && !dmode) rc = bck(b, cudaMemsetAsync(b->prop[0], 0, sizeof(u128) * V * K, st), "memset");
    if (!rc) {
        k_ppr_init<<<(G * K + 255) / 256, 256, 0, st>>>(b->d_seeds, G, u->inv_deg, u->degree, b->prop[0], dmode ? b->propd[0] : nullptr,
                                                        b->S[0]);
        rc = bck(b, cudaGetLastError(), "ppr init");
    }
    if (!rc) rc = bck(b, cudaGraphLaunch(b->ppr_exec, st), "graph launch");
    if (!rc) rc = bck(b, cudaEventRecord(e1, st), "event");
    if (!rc && ranks_out) {
        if (k == (uint32_t)K) {
            rc = bck(b, cudaMemcpyAsync(ranks_out, b->rank, sizeof(double) * V * K, cudaMemcpyDeviceToHost, st), "D2H");
        } else {
            rc = bck(b, cudaMemcpy2DAsync(ranks_out, sizeof(double) * k, b->rank, sizeof(double) * K, sizeof(double) * k, V,
                                          cudaMemcpyDeviceToHost, st), "D2H");
        }
    }
    if (!rc) rc = bck(b, cudaStreamSynchronize(st), "run");
    if (!rc && stats) {
        memset(stats, 0, sizeof(*stats));
        stats->iterations = iterations;
        stats->pull_iterations = iterations;
        cudaEventElapsedTime(&stats->ms, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    u->nlaunch += 1 + 2ull * iterations;
    return rc;
}

// Adds to `graph`, after `deps`, the BFS loop: WHILE (a bit changed) { pull; vertex pass; decide }.
static int add_bfs_loop(grz_batch* b, cudaGraph_t graph, const cudaGraphNode_t* deps, size_t ndeps, cudaGraphNode_t* node_out)
{
    grz_graph* u = b->u;
    const uint32_t V = (uint32_t)u->V;
    cudaGraphConditionalHandle loop = 0;
    int rc = bck(b, cudaGraphConditionalHandleCreate(&loop, graph, 1, cudaGraphCondAssignDefault), "handle");
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = loop;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    if (!rc) rc = bck(b, cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &p), "while node");
    cudaStream_t cs = nullptr;
    if (!rc) rc = bck(b, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "stream");
    if (!rc) rc = bck(b, cudaStreamBeginCaptureToGraph(cs, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                      cudaStreamCaptureModeThreadLocal), "capture");
    if (!rc) {
        const unsigned pgrid = persistent_grid(b, (u->pull.nvec + 255) / 256, b->bfs_blocks);
        const unsigned vgrid = persistent_grid(b, ((V + 3) / 4 + 255) / 256, b->bfs_blocks);
        k_msbfs_pull<<<pgrid, 256, 0, cs>>>(u->pull.nbr, u->pull.shared, u->pull.nvec, V, b->frontier, b->visited, b->next_words);
        k_msbfs_vertex<<<vgrid, 256, 0, cs>>>(b->next_words, reinterpret_cast<unsigned*>(b->visited),
                                              reinterpret_cast<unsigned*>(b->frontier), b->level, V, b->iter, b->ctl);
        k_msbfs_decide<<<1, 1, 0, cs>>>(b->ctl, b->iter, V + 1, loop);
        rc = bck(b, cudaGetLastError(), "bfs launch");
        cudaGraph_t g2 = nullptr;
        const cudaError_t e = cudaStreamEndCapture(cs, &g2);
        if (!rc) rc = bck(b, e, "end capture");
    }
    if (cs) cudaStreamDestroy(cs);
    *node_out = node;
    return rc;
}

// the BFS loop as one CUDA graph
static int build_bfs_graph(grz_batch* b)
{
    if (b->bfs_exec) { cudaGraphExecDestroy(b->bfs_exec); b->bfs_exec = nullptr; }
    cudaGraph_t top = nullptr;
    BCK(b, cudaGraphCreate(&top, 0));
    cudaGraphNode_t node = nullptr;
    int rc = add_bfs_loop(b, top, nullptr, 0, &node);
    if (!rc) rc = bck(b, cudaGraphInstantiate(&b->bfs_exec, top, 0), "instantiate");
    cudaGraphDestroy(top);
    if (rc) b->bfs_exec = nullptr;
    return rc;
}

// the multi-source BFS state, allocated on first use
static int bfs_alloc(grz_batch* b)
{
    const uint64_t V = b->u->V;
    const uint64_t Vw = (V + 3) / 4 * 4;
    if (!b->visited) {
        BCK(b, cudaMalloc((void**)&b->visited, Vw));
        BCK(b, cudaMalloc((void**)&b->frontier, Vw));
        BCK(b, cudaMalloc((void**)&b->next_words, Vw));
        BCK(b, cudaMalloc((void**)&b->level, sizeof(int32_t) * V * K));
        BCK(b, cudaMalloc((void**)&b->ctl, sizeof(unsigned long long) * 4));
        BCK(b, cudaMalloc((void**)&b->iter, sizeof(uint32_t)));
    }
    return GRZ_OK;
}

// the last node of the work captured so far on cs (one node), then ends the capture
static int end_capture_sink(grz_batch* b, cudaStream_t cs, cudaGraphNode_t* sink)
{
    cudaStreamCaptureStatus st;
    const cudaGraphNode_t* deps = nullptr;
    size_t n = 0;
    const cudaError_t e = cudaStreamGetCaptureInfo(cs, &st, nullptr, nullptr, &deps, nullptr, &n);
    const cudaGraphNode_t last = (e == cudaSuccess && n == 1) ? deps[0] : nullptr;
    cudaGraph_t out = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(cs, &out);
    if (e != cudaSuccess) return bck(b, e, "capture info");
    if (e2 != cudaSuccess) return bck(b, e2, "end capture");
    if (sink) {
        if (!last) return bset(b, GRZ_ERR_STATE, "captured work does not end in one node");
        *sink = last;
    }
    return GRZ_OK;
}

// PPR and multi-source BFS as one CUDA graph with two independent branches, each from its initial
// state to its results: branch 1 the PPR loop (d_seeds), branch 2 the BFS loop (d_roots).  Event
// records at both ends of each branch time them inside the one launch.
static int build_run_graph(grz_batch* b, uint32_t iterations, double damping, int dmode)
{
    if (b->run_exec) { cudaGraphExecDestroy(b->run_exec); b->run_exec = nullptr; }
    if (!b->stamps) BCK(b, cudaMalloc((void**)&b->stamps, 4 * sizeof(unsigned long long)));
    grz_graph* u = b->u;
    const uint64_t V = u->V;
    const uint64_t Vw = (V + 3) / 4 * 4;
    const uint32_t G = (uint32_t)b->Vg.size();
    cudaGraph_t top = nullptr;
    BCK(b, cudaGraphCreate(&top, 0));
    cudaStream_t cs = nullptr;
    int rc = bck(b, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "stream");
    int cur = 0;
    // branch 1: PPR
    if (!rc) rc = bck(b, cudaStreamBeginCaptureToGraph(cs, top, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal), "capture");
    if (!rc) {
        k_stamp<<<1, 1, 0, cs>>>(b->stamps + 0);
        if (dmode) cudaMemsetAsync(b->propd[0], 0, sizeof(double) * V * K, cs);
        else cudaMemsetAsync(b->prop[0], 0, sizeof(u128) * V * K, cs);
        k_ppr_init<<<(G * K + 255) / 256, 256, 0, cs>>>(b->d_seeds, G, u->inv_deg, u->degree, b->prop[0], dmode ? b->propd[0] : nullptr,
                                                        b->S[0]);
        rc = bck(b, cudaGetLastError(), "ppr init");
        if (!rc) rc = enqueue_ppr_chain(b, cs, iterations, damping, dmode, b->d_seeds, &cur);
        k_stamp<<<1, 1, 0, cs>>>(b->stamps + 1);
        const int rc2 = end_capture_sink(b, cs, nullptr);
        if (!rc) rc = rc2;
    }
    // branch 2: BFS (no dependency on branch 1)
    cudaGraphNode_t init = nullptr, loop = nullptr;
    if (!rc) rc = bck(b, cudaStreamBeginCaptureToGraph(cs, top, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal), "capture");
    if (!rc) {
        k_stamp<<<1, 1, 0, cs>>>(b->stamps + 2);
        cudaMemsetAsync(b->visited, 0, Vw, cs);
        cudaMemsetAsync(b->frontier, 0, Vw, cs);
        cudaMemsetAsync(b->next_words, 0, Vw, cs);
        cudaMemsetAsync(b->level, 0xff, sizeof(int32_t) * V * K, cs);
        cudaMemsetAsync(b->ctl, 0, sizeof(unsigned long long) * 4, cs);
        k_msbfs_init<<<(G * K + 255) / 256, 256, 0, cs>>>(b->d_roots, G * K, b->visited, b->frontier, b->level, b->iter);
        rc = bck(b, cudaGetLastError(), "bfs init");
        const int rc2 = end_capture_sink(b, cs, &init);
        if (!rc) rc = rc2;
    }
    if (!rc) rc = add_bfs_loop(b, top, &init, 1, &loop);
    if (!rc) rc = bck(b, cudaStreamBeginCaptureToGraph(cs, top, &loop, nullptr, 1, cudaStreamCaptureModeThreadLocal), "capture");
    if (!rc) {
        k_stamp<<<1, 1, 0, cs>>>(b->stamps + 3);
        rc = bck(b, cudaGetLastError(), "stamp");
        const int rc2 = end_capture_sink(b, cs, nullptr);
        if (!rc) rc = rc2;
    }
    if (cs) cudaStreamDestroy(cs);
    if (!rc) rc = bck(b, cudaGraphInstantiate(&b->run_exec, top, 0), "instantiate");
    cudaGraphDestroy(top);
    if (rc) { b->run_exec = nullptr; return rc; }
    b->run_iters = iterations;
    b->run_damping = damping;
    b->run_dmode = dmode;
    b->ppr_final = cur;
    return GRZ_OK;
}

// k roots per graph (local IDs, NONE = unused instance); levels out as [union vertex][k]
// (-1 = unreached)
extern "C" int grz_batch_msbfs(grz_batch* b, const uint32_t* roots, uint32_t k, int32_t* levels_out, grz_run_stats_t* stats)
{
    if (!b || !roots || k == 0 || k > (uint32_t)K) return GRZ_ERR_ARG;
    if (!b->d_seeds) return bset(b, GRZ_ERR_STATE, "grz_batch_build not called");
    BCK(b, cudaSetDevice(b->device));
    grz_graph* u = b->u;
    const uint64_t V = u->V;
    const uint32_t G = (uint32_t)b->Vg.size();
    const uint64_t Vw = (V + 3) / 4 * 4;
    int rc = bfs_alloc(b);
    if (rc) return rc;
    rc = upload_seeds(b, roots, k);
    if (rc) return rc;
    if (!b->bfs_exec) {
        rc = build_bfs_graph(b);
        if (rc) return rc;
    }
    cudaStream_t st = b->stream;
    cudaEvent_t e0, e1;
    BCK(b, cudaEventCreate(&e0));
    BCK(b, cudaEventCreate(&e1));
    const uint32_t one = 1;
    rc = bck(b, cudaEventRecord(e0, st), "event");
    if (!rc) rc = bck(b, cudaMemsetAsync(b->visited, 0, Vw, st), "memset");
    if (!rc) rc = bck(b, cudaMemsetAsync(b->frontier, 0, Vw, st), "memset");
    if (!rc) rc = bck(b, cudaMemsetAsync(b->next_words, 0, Vw, st), "memset");
    if (!rc) rc = bck(b, cudaMemsetAsync(b->level, 0xff, sizeof(int32_t) * V * K, st), "memset");
    if (!rc) rc = bck(b, cudaMemsetAsync(b->ctl, 0, sizeof(unsigned long long) * 4, st), "memset");
    if (!rc) {
        memcpy(b->mail, &one, sizeof(one));
        rc = bck(b, cudaMemcpyAsync(b->iter, b->mail, sizeof(uint32_t), cudaMemcpyHostToDevice, st), "H2D");
    }
    if (!rc) {
        k_msbfs_init<<<(G * K + 255) / 256, 256, 0, st>>>(b->d_seeds, G * K, b->visited, b->frontier, b->level, nullptr);
        rc = bck(b, cudaGetLastError(), "bfs init");
    }
    if (!rc) rc = bck(b, cudaGraphLaunch(b->bfs_exec, st), "graph launch");
    if (!rc) rc = bck(b, cudaEventRecord(e1, st), "event");
    if (!rc) rc = bck(b, cudaMemcpyAsync(b->mail, b->ctl, sizeof(unsigned long long) * 3, cudaMemcpyDeviceToHost, st), "D2H");
    if (!rc && levels_out) {
        if (k == (uint32_t)K)
            rc = bck(b, cudaMemcpyAsync(levels_out, b->level, sizeof(int32_t) * V * K, cudaMemcpyDeviceToHost, st), "D2H");
        else
            rc = bck(b, cudaMemcpy2DAsync(levels_out, sizeof(int32_t) * k, b->level, sizeof(int32_t) * K, sizeof(int32_t) * k, V,
                                          cudaMemcpyDeviceToHost, st), "D2H");
    }
    if (!rc) rc = bck(b, cudaStreamSynchronize(st), "run");
    unsigned long long c[3];
    memcpy(c, b->mail, sizeof(c));
    if (!rc && c[2] == 1) rc = bset(b, GRZ_ERR_TIMEOUT, "BFS did not converge within V + 1 iterations");
    if (!rc && c[2] == 2) rc = bset(b, GRZ_ERR_TIMEOUT, "BFS stopped by its time bound");
    if (!rc && stats) {
        memset(stats, 0, sizeof(*stats));
        stats->iterations = (uint32_t)c[1] + 1;  // the last iteration found nothing new
        stats->pull_iterations = stats->iterations;
        cudaEventElapsedTime(&stats->ms, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    u->nlaunch += 1 + 3ull * (c[1] + 1);
    return rc;
}

// PPR (seeds, k per graph, `iterations`) and multi-source BFS (roots, kb per graph) in one CUDA
// graph launch: the two loops run side by side as independent branches of one graph, each from
// its initial state.  Results and per-branch device times as grz_batch_ppr / grz_batch_msbfs;
// *total_ms is the launch's device time.
extern "C" int grz_batch_run(grz_batch* b, const uint32_t* seeds, uint32_t k, uint32_t iterations, double damping,
                             const uint32_t* roots, uint32_t kb, double* ranks_out, int32_t* levels_out,
                             grz_run_stats_t* ppr_stats, grz_run_stats_t* bfs_stats, float* total_ms)
{
    if (!b || !seeds || !roots || k == 0 || k > (uint32_t)K || kb == 0 || kb > (uint32_t)K || iterations == 0 ||
        !(damping >= 0.0 && damping <= 1.0))
        return GRZ_ERR_ARG;
    if (!b->d_seeds) return bset(b, GRZ_ERR_STATE, "grz_batch_build not called");
    BCK(b, cudaSetDevice(b->device));
    grz_graph* u = b->u;
    const uint64_t V = u->V;
    const int dmode = b->ppr_props == 2;
    int rc = ppr_alloc(b, dmode);
    if (!rc) rc = bfs_alloc(b);
    if (!rc) rc = upload_seeds(b, seeds, k, b->d_seeds);
    if (!rc) rc = upload_seeds(b, roots, kb, b->d_roots);
    if (rc) return rc;
    if (!b->run_exec || b->run_iters != iterations || b->run_damping != damping || b->run_dmode != dmode) {
        rc = build_run_graph(b, iterations, damping, dmode);
        if (rc) return rc;
    }
    cudaStream_t st = b->stream;
    cudaEvent_t e0, e1;
    BCK(b, cudaEventCreate(&e0));
    BCK(b, cudaEventCreate(&e1));
    rc = bck(b, cudaEventRecord(e0, st), "event");
    if (!rc) rc = bck(b, cudaGraphLaunch(b->run_exec, st), "graph launch");
    if (!rc) rc = bck(b, cudaEventRecord(e1, st), "event");
    if (!rc) rc = bck(b, cudaMemcpyAsync(b->mail, b->ctl, sizeof(unsigned long long) * 3, cudaMemcpyDeviceToHost, st), "D2H");
    if (!rc) rc = bck(b, cudaMemcpyAsync((unsigned long long*)b->mail + 4, b->stamps, 4 * sizeof(unsigned long long),
                                         cudaMemcpyDeviceToHost, st), "D2H");
    if (!rc && ranks_out) {
        if (k == (uint32_t)K) {
            rc = bck(b, cudaMemcpyAsync(ranks_out, b->rank, sizeof(double) * V * K, cudaMemcpyDeviceToHost, st), "D2H");
        } else {
            rc = bck(b, cudaMemcpy2DAsync(ranks_out, sizeof(double) * k, b->rank, sizeof(double) * K, sizeof(double) * k, V,
                                          cudaMemcpyDeviceToHost, st), "D2H");
        }
    }
    if (!rc && levels_out) {
        if (kb == (uint32_t)K)
            rc = bck(b, cudaMemcpyAsync(levels_out, b->level, sizeof(int32_t) * V * K, cudaMemcpyDeviceToHost, st), "D2H");
        else
            rc = bck(b, cudaMemcpy2DAsync(levels_out, sizeof(int32_t) * kb, b->level, sizeof(int32_t) * K, sizeof(int32_t) * kb, V,
                                          cudaMemcpyDeviceToHost, st), "D2H");
    }
    if (!rc) rc = bck(b, cudaStreamSynchronize(st), "run");
    unsigned long long c[3];
    memcpy(c, b->mail, sizeof(c));
    if (!rc && c[2] == 1) rc = bset(b, GRZ_ERR_TIMEOUT, "BFS did not converge within V + 1 iterations");
    if (!rc && c[2] == 2) rc = bset(b, GRZ_ERR_TIMEOUT, "BFS stopped by its time bound");
    if (!rc) {
        const unsigned long long* ts = (const unsigned long long*)b->mail + 4;
        if (ppr_stats) {
            memset(ppr_stats, 0, sizeof(*ppr_stats));
            ppr_stats->iterations = ppr_stats->pull_iterations = iterations;
            ppr_stats->ms = (float)((double)(ts[1] - ts[0]) * 1e-6);
        }
        if (bfs_stats) {
            memset(bfs_stats, 0, sizeof(*bfs_stats));
            bfs_stats->iterations = bfs_stats->pull_iterations = (uint32_t)c[1] + 1;
            bfs_stats->ms = (float)((double)(ts[3] - ts[2]) * 1e-6);
        }
        if (total_ms) cudaEventElapsedTime(total_ms, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    u->nlaunch += 2 + 2ull * iterations + 1 + 3ull * (c[1] + 1);
    return rc;
}

extern "C" int grz_batch_tune_set(grz_batch* b, int param, int64_t value)
{
    if (!b) return GRZ_ERR_ARG;
    if (param == GRZ_BATCH_TUNE_PPR_PROPS) {
        if (value < 0 || value > 2) return bset(b, GRZ_ERR_RANGE, "PPR props must be 0 (by size), 1 (fixed point) or 2 (doubles)");
        b->ppr_props = (int)value;  // the next run captures its loop again if the mode changes
        return GRZ_OK;
    }
    if (value < 1 || value > 32) return bset(b, GRZ_ERR_RANGE, "blocks per SM must be 1..32");
    int* slot = param == GRZ_BATCH_TUNE_PPR_BLOCKS ? &b->ppr_blocks : (param == GRZ_BATCH_TUNE_BFS_BLOCKS ? &b->bfs_blocks : nullptr);
    if (!slot) return bset(b, GRZ_ERR_ARG, "unknown batch tuning parameter");
    if (*slot != (int)value) {
        *slot = (int)value;
        // the captured loops bake the grid in: capture again at the next run
        cudaSetDevice(b->device);
        if (param == GRZ_BATCH_TUNE_PPR_BLOCKS && b->ppr_exec) { cudaGraphExecDestroy(b->ppr_exec); b->ppr_exec = nullptr; }
        if (param == GRZ_BATCH_TUNE_BFS_BLOCKS && b->bfs_exec) { cudaGraphExecDestroy(b->bfs_exec); b->bfs_exec = nullptr; }
        if (b->run_exec) { cudaGraphExecDestroy(b->run_exec); b->run_exec = nullptr; }
    }
    return GRZ_OK;
}

extern "C" int grz_batch_tune_get(const grz_batch* b, int param, int64_t* value)
{
    if (!b || !value) return GRZ_ERR_ARG;
    if (param == GRZ_BATCH_TUNE_PPR_BLOCKS) *value = b->ppr_blocks;
    else if (param == GRZ_BATCH_TUNE_BFS_BLOCKS) *value = b->bfs_blocks;
    else if (param == GRZ_BATCH_TUNE_PPR_PROPS) *value = b->ppr_props;
    else return GRZ_ERR_ARG;
    return GRZ_OK;
}

extern "C" unsigned long long grz_batch_launch_count(const grz_batch* b) { return b ? b->u->nlaunch : 0ull; }
