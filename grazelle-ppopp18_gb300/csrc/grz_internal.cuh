// grz_internal.cuh -- shared device/host definitions of the GB300 Grazelle engine.
//
// Data layout in HBM for one graph (V vertices, E edges, N vector-sparse vectors per list):
//
//   Reference layout (bit-identical to Grazelle's host packer, source/graphdata.c:143-173; the
//   vectors are derived from the execution layout when first asked for):
//     list[l].vs        uint64[4N]   4-lane 256-bit vectors: valid bit 63, spread shared ID in
//                                    bits 62:48, 48-bit neighbour ID in bits 47:0
//     list[l].vindex    uint64[V+64] first vector of each shared vertex (graphdata.c:219-267)
//   Execution layout (what the kernels stream):
//     list[l].nbr       uint4[N]     the four neighbour IDs as uint32, invalid lane = 0xffffffff
//     list[l].shared    uint32[N]    shared vertex of each vector (dst for pull, src for push)
//     list[l].rowptr    uint32[V+1]  CSR over vectors: vectors of vertex v are [rowptr[v], rowptr[v+1])
//   Per-vertex state:
//     outdeg            double[V+8]  outdegree from the -pull list (graphdata.c:792-821)
//     degree            uint32[V]    same, integer
//     inv_deg           double[V]    1 / (outdeg == 0 ? V : outdeg)
//     pr_fx[2]          u128[V]      PageRank props as unsigned 4.124 fixed point (ping-pong)
//
// All IDs on the device are 32-bit, so V and N must stay below 2^32 - 1.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define GRZ_INVALID_ID 0xffffffffu
#define GRZ_FX_FRAC 124  // fractional bits of the u128 fixed-point PageRank values

// ----------------------------------------------------------------------------------------------
// error codes (also in include/grazelle_gb300.h)
#define GRZ_OK 0
#define GRZ_ERR_ARG -1
#define GRZ_ERR_CUDA -2
#define GRZ_ERR_NOMEM -3
#define GRZ_ERR_UNSORTED -4
#define GRZ_ERR_RANGE -5
#define GRZ_ERR_STATE -6
#define GRZ_ERR_IO -7
#define GRZ_ERR_TIMEOUT -8

#define GRZ_APP_PAGERANK 0
#define GRZ_APP_CONNECTED_COMPONENTS 1
#define GRZ_APP_BREADTH_FIRST_SEARCH 2

// ----------------------------------------------------------------------------------------------
// 128-bit unsigned fixed point

struct __align__(16) u128 {
    unsigned long long lo, hi;
};

__host__ __device__ __forceinline__ u128 u128_zero() { u128 r; r.lo = 0; r.hi = 0; return r; }

__host__ __device__ __forceinline__ u128 u128_add(u128 a, u128 b)
{
    u128 r;
#ifdef __CUDA_ARCH__
    asm("add.cc.u64 %0, %2, %4;\n\taddc.u64 %1, %3, %5;" : "=l"(r.lo), "=l"(r.hi) : "l"(a.lo), "l"(a.hi), "l"(b.lo), "l"(b.hi));
#else
    r.lo = a.lo + b.lo;
    r.hi = a.hi + b.hi + (r.lo < a.lo ? 1ull : 0ull);
#endif
    return r;
}

// a * d (mod 2^128); exact when the true product is below 2^128
__device__ __forceinline__ u128 u128_mul32(u128 a, uint32_t d)
{
    u128 r;
    r.lo = a.lo * (unsigned long long)d;
    r.hi = a.hi * (unsigned long long)d + __umul64hi(a.lo, (unsigned long long)d);
    return r;
}

// Exact conversion of a non-negative double below 16 to 4.124 fixed point.  Values below
// 2^-72 lose their bits beneath 2^-124 (truncation); zero and subnormals map to 0.
__host__ __device__ __forceinline__ u128 fx_from_double(double x)
{
    unsigned long long b;
#ifdef __CUDA_ARCH__
    b = (unsigned long long)__double_as_longlong(x);
#else
    __builtin_memcpy(&b, &x, 8);
#endif
    const int e = (int)((b >> 52) & 0x7ff);
    u128 r = u128_zero();
    if (e == 0) return r;
    const unsigned long long m = (b & 0x000fffffffffffffull) | 0x0010000000000000ull;
    const int sh = e - 1075 + GRZ_FX_FRAC;  // x = m * 2^(e-1075)
    if (sh >= 0) {
        if (sh == 0) { r.lo = m; }
        else if (sh < 64) { r.lo = m << sh; r.hi = m >> (64 - sh); }
        else if (sh < 128) { r.hi = m << (sh - 64); }
    } else if (sh > -64) {
        r.lo = m >> (-sh);
    }
    return r;
}

// Round-to-nearest-even conversion of 4.124 fixed point to double, integer arithmetic only.
__host__ __device__ __forceinline__ double fx_to_double(u128 a)
{
    if ((a.hi | a.lo) == 0) return 0.0;
#ifdef __CUDA_ARCH__
    const int lz = a.hi ? __clzll((long long)a.hi) : 64 + __clzll((long long)a.lo);
#else
    const int lz = a.hi ? __builtin_clzll(a.hi) : 64 + __builtin_clzll(a.lo);
#endif
    const int msb = 127 - lz;
    unsigned long long m;
    int exp2 = msb - GRZ_FX_FRAC;  // value in [2^exp2, 2^(exp2+1))
    if (msb <= 52) {
        // fits: shift left so the leading bit lands on bit 52 (msb <= 52 implies a.hi == 0)
        m = a.lo << (52 - msb);
    } else {
        const int sh = msb - 52;  // 1..75
        unsigned long long rem_hi_bit, rem_rest;
        // m = a >> sh (53 bits); round bit = bit (sh-1); sticky = bits below
        if (sh < 64) {
            m = (a.lo >> sh) | (sh ? (a.hi << (64 - sh)) : 0ull);
            rem_hi_bit = (a.lo >> (sh - 1)) & 1ull;
            rem_rest = (sh >= 2) ? (a.lo & ((1ull << (sh - 1)) - 1ull)) : 0ull;
        } else if (sh == 64) {
            m = a.hi;
            rem_hi_bit = a.lo >> 63;
            rem_rest = a.lo & 0x7fffffffffffffffull;
        } else {
            m = a.hi >> (sh - 64);
            const int rb = sh - 1;  // round bit position (>= 64)
            rem_hi_bit = (a.hi >> (rb - 64)) & 1ull;
            rem_rest = ((rb - 64) ? (a.hi & ((1ull << (rb - 64)) - 1ull)) : 0ull) | a.lo;
        }
        if (rem_hi_bit && (rem_rest || (m & 1ull))) {
            ++m;
            if (m == (1ull << 53)) { m >>= 1; ++exp2; }
        }
    }
    const unsigned long long bits = ((unsigned long long)(exp2 + 1023) << 52) | (m & 0x000fffffffffffffull);
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)bits);
#else
    double d;
    __builtin_memcpy(&d, &bits, 8);
    return d;
#endif
}

// Exact global u128 accumulation: two 64-bit atomics; the low-word wrap-around is carried.
__device__ __forceinline__ void u128_atomic_add(u128* dst, u128 v)
{
    const unsigned long long old = atomicAdd(&dst->lo, v.lo);
    const unsigned long long carry = (old + v.lo < old) ? 1ull : 0ull;
    if (v.hi | carry) atomicAdd(&dst->hi, v.hi + carry);
}

// Exact sums that every block adds into are spread over GRZ_SUM_SLOTS slots (block mod slots):
// thousands of atomics to one address would serialise on one L2 slice.
#define GRZ_SUM_SLOTS 64

__device__ __forceinline__ void u128_slot_add(u128* slots, u128 v)
{
    if (v.lo | v.hi) u128_atomic_add(slots + (blockIdx.x & (GRZ_SUM_SLOTS - 1)), v);
}

__device__ __forceinline__ u128 u128_shfl_down(u128 v, int off)
{
    u128 r;
    r.lo = __shfl_down_sync(0xffffffffu, v.lo, off);
    r.hi = __shfl_down_sync(0xffffffffu, v.hi, off);
    return r;
}

// ----------------------------------------------------------------------------------------------
// Bulk copies global -> shared memory on the copy engine (cp.async.bulk, completion counted on an
// mbarrier in shared memory).  Addresses and sizes must be multiples of 16 bytes.  Waits are
// bounded (iterations and %globaltimer): a wait that runs out returns false.

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// makes initialised mbarriers visible to the copy engine (the async proxy)
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// orders this thread's earlier shared-memory accesses before later bulk copies into the same bytes
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait_parity(unsigned long long* bar, unsigned parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Cache policy of the edge stream (read once per pass) and of the label gathers.
// GRZ_STREAM_LD: 0 = ld.global.cs (evict-first), 1 = non-coherent load that does not allocate
// in L1 (L1 capacity left to the gathers), 2 = coherent load that does not allocate in L1.
// GRZ_GATHER_LD: 0 = plain coherent load, 1 = L1::evict_last (gathered lines kept over others).
#ifndef GRZ_STREAM_LD
#define GRZ_STREAM_LD 0
#endif
#ifndef GRZ_GATHER_LD
#define GRZ_GATHER_LD 0
#endif
__device__ __forceinline__ uint4 ld_stream(const uint4* p)
{
#if GRZ_STREAM_LD == 1
    uint4 r;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
    return r;
#elif GRZ_STREAM_LD == 2
    uint4 r;
    asm volatile("ld.global.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
    return r;
#else
    return __ldcs(p);
#endif
}
__device__ __forceinline__ uint32_t ld_stream(const uint32_t* p)
{
#if GRZ_STREAM_LD == 1
    uint32_t r;
    asm("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(r) : "l"(p));
    return r;
#elif GRZ_STREAM_LD == 2
    uint32_t r;
    asm volatile("ld.global.L1::no_allocate.u32 %0, [%1];" : "=r"(r) : "l"(p));
    return r;
#else
    return __ldcs(p);
#endif
}
// a label that may change during the phase (coherent load)
__device__ __forceinline__ uint32_t ld_label(const uint32_t* p)
{
#if GRZ_GATHER_LD == 1
    uint32_t r;
    asm volatile("ld.global.L1::evict_last.u32 %0, [%1];" : "=r"(r) : "l"(p));
    return r;
#else
    return *p;
#endif
}

// waits for the phase with the given parity to complete; false when the wait ran out (1 s)
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity)
{
    if (mbar_try_wait_parity(bar, parity)) return true;
    unsigned long long t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (unsigned i = 0; i < (1u << 24); ++i) {
        if (mbar_try_wait_parity(bar, parity)) return true;
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 > 1000000000ull) break;
    }
    return false;
}

// ----------------------------------------------------------------------------------------------
// graph context

struct grz_list {
    uint64_t nvec;          // number of 4-lane vectors
    uint64_t* vs;           // reference-format vectors, 4 words each (built on first request)
    uint64_t* vindex;       // uint64[V+64]
    uint64_t vindex_start;  // first shared vertex with vectors
    uint64_t vindex_end;    // last shared vertex with vectors
    uint4* nbr;             // uint4[nvec]; pull list: hub sources encoded as GRZ_HUB_BASE + slot
    uint32_t* shared;       // uint32[nvec]
    uint32_t* rowptr;       // uint32[V+1]
    uint32_t* hub_vid;      // pull list: vertex of each hub slot, slots by out-degree, highest first
    uint32_t nhub;
};

// Hub sources of the pull list.  In power-law graphs a few thousand vertices are the source of
// most edges.  The device pull list stores such a source as GRZ_HUB_BASE + slot, so the pull
// kernels can serve it from a copy of the hubs' values in shared memory instead of a gather
// through L1.  Invalid lanes stay GRZ_INVALID_ID; other sources are plain IDs (< V < 2^31).
#define GRZ_HUB_BASE 0x80000000u
#define GRZ_HUB_MAX 49152u
#define GRZ_INGEST_MAX_CHUNKS 64
#define GRZ_PR_MAX_SEGMENTS 256

#define GRZ_BATCH_K 8  // instances per graph of a batch (grz_batch.cu)

// the vertex a pull-list neighbour field names (GRZ_INVALID_ID stays invalid)
__device__ __forceinline__ uint32_t grz_hub_decode(uint32_t x, const uint32_t* __restrict__ hub_vid, uint32_t nhub)
{
    const uint32_t sl = x - GRZ_HUB_BASE;
    return sl < nhub ? __ldg(hub_vid + sl) : x;
}

struct grz_prof;

// engine flags (the reference's EXPERIMENTS that change the CC/BFS driver, Makefile:59-176)
#define GRZ_FLAG_FORCE_PULL 1       // EXPERIMENT_EDGE_FORCE_PULL
#define GRZ_FLAG_FORCE_PUSH 2       // EXPERIMENT_EDGE_FORCE_PUSH
#define GRZ_FLAG_WITHOUT_COUNT 4    // EXPERIMENT_THRESHOLD_WITHOUT_COUNT
#define GRZ_FLAG_WITHOUT_OUTDEG 8   // EXPERIMENT_THRESHOLD_WITHOUT_OUTDEGREES
#define GRZ_FLAG_HOST_LOOP 16       // run the iteration loop on the host

// the vote is added into GRZ_VOTE_SLOTS counters, 128 bytes apart (block mod slots)
#define GRZ_VOTE_SLOTS 64
#define GRZ_VOTE_STRIDE 16

// learned switch (grz_switch.cu)
#define GRZ_MLP_FEATURES 12
#define GRZ_MLP_HIDDEN 32
#define GRZ_MLP_PARAMS 1505  // 32*12 + 32 + 32*32 + 32 + 32 + 1
#define GRZ_POLICY_THRESHOLD 0
#define GRZ_POLICY_LEARNED 1
struct grz_mlp;

#define GRZ_TUNE_HUBS 0
#define GRZ_TUNE_CC_CACHE 1
#define GRZ_TUNE_CC_THREADS 2
#define GRZ_TUNE_CC_GRID 3
#define GRZ_TUNE_PR_GRID 4
#define GRZ_TUNE_BFS_PULL_SCAN 5
#define GRZ_TUNE_PR_PROPS 6
#define GRZ_TUNE_INGEST_CHUNKS 7
#define GRZ_TUNE_PR_PERSISTENT 8
#define GRZ_TUNE_PR_WAIT_LIMIT_US 9
#define GRZ_TUNE_PR_WITHHOLD 10
#define GRZ_TUNE_RUN_MAX_ITERATIONS 11
#define GRZ_TUNE_RUN_LIMIT_US 12
#define GRZ_TUNE_PULL_STAGING 13
#define GRZ_TUNE_PR_SEGMENT_BITS 14
#define GRZ_TUNE_CC_SEGMENTS 16
#define GRZ_TUNE_BFS_PULL_FIRST 17
#define GRZ_TUNE_CC_PULL_FIRST 18
#define GRZ_TUNE_HUBS_LOADED 100

// kernel shapes chosen per graph (grz_tune_set; the autotuner searches them)
struct grz_tuning {
    uint32_t hub_max;      // hub sources encoded when a graph is loaded (0: none)
    uint32_t cc_cache;     // hub labels the CC pull kernel keeps in shared memory
    uint32_t cc_threads;   // threads per block of the CC pull kernel (256, 512, 1024)
    uint32_t cc_grid;      // blocks of the persistent CC pull kernel (0: SMs x resident blocks)
    uint32_t pr_grid;      // blocks of the persistent PageRank gather kernel (0: SMs x resident blocks)
    uint32_t bfs_pull_scan;  // 1: BFS pull scans every vector; 0: only the wanted destinations' (compacted)
    uint32_t pr_props;     // props the PageRank gather reads: 0 by size, 1 fixed point, 2 doubles
    uint32_t ingest_chunks;  // chunks of the pull-only ingest (0: by edge count)
    uint32_t pr_persistent;  // PageRank iterations: 0 by default rule, 1 two kernels each, 2 one cooperative launch
    uint32_t pr_wait_limit_us;  // bound of one grid-barrier wait of the persistent kernel (0: 2 s)
    uint32_t pr_withhold;    // tests: block + 1 whose first barrier arrival is withheld (0: none)
    uint32_t run_max_iterations;  // CC/BFS iteration bound (0: V + 2)
    uint32_t run_limit_us;   // CC/BFS time bound of a run in microseconds (0: 300 s)
    uint32_t pull_staging;   // CC pull's edge stream: 0 plain streaming loads, 1 bulk copies into shared memory
    uint32_t pr_segment_bits;  // PageRank source segments: 0 by size, 1 none, b in [8, 31]: 2^b sources per segment
    uint32_t cc_segments; // CC full pull over the source segments: 0 when built, 1 never, 2 build them by size
    uint32_t bfs_pull_first;  // BFS pull: vectors a wanted destination reads in the early-exit pass (0: no such pass)
    uint32_t cc_pull_first;   // CC: each destination's first vector before the whole-list pass of a first pull (0: off)
};

// Device control block of a CC/BFS run executed as one CUDA graph (grz_ccbfs.cu): the
// decision kernel at the end of each iteration updates it and sets the graph's conditional
// handles.  The host writes it before the launch and reads it after.
struct grz_runctl {
    unsigned long long vote;         // vote of the last iteration
    unsigned long long cnt_f;        // popcount accumulators of the decision kernel (zero between uses)
    unsigned long long cnt_u;
    unsigned long long ticket;       // last-block ticket of the decision kernel (zero between uses)
    uint32_t running;                // 1 until an iteration ends with vote 0
    uint32_t engine;                 // engine of the iteration about to run: 1 pull, 0 push
    uint32_t level;                  // number of the iteration about to run (1-based) = BFS level
    uint32_t npull, npush;
    uint32_t last_engine;
    uint32_t max_level;              // iteration bound: the run stops with `overrun` = 1 beyond it
    uint32_t overrun;                // 2: stopped by the time bound
    unsigned long long t0_ns;        // %globaltimer at the initial decision
    unsigned long long limit_ns;     // time bound of the run
    // the engine policy, read at run time so that one captured graph serves every policy
    const float* params;             // MLP parameters (learned policy) or null
    double threshold;                // vote threshold (E/5 or V/2)
    int32_t force;                   // 1 pull, 0 push, -1 the policy decides
    float features[GRZ_MLP_FEATURES];
};

// CC / BFS state (grz_ccbfs.cu)
struct grz_frontier_state {
    int app, flags;
    uint32_t root, iter, npull, npush;
    uint64_t vote_host;              // the last phase's vote (converge_vote in the reference)
    uint32_t* label;                 // CC labels / BFS parents, uint32[V+1] (entry V = +inf)
    uint32_t* level;                 // BFS level of each vertex
    unsigned long long* has;         // HasInfo bitmap
    unsigned long long* has_next;    // HasInfo*
    unsigned long long* wants;       // WantsInfo
    unsigned long long* nonempty_push;  // vertices with out-vectors
    unsigned long long* nonempty_pull;  // vertices with in-vectors
    unsigned long long* unres;       // BFS pull: wanted destinations the early-exit pass left undecided
    uint32_t* frontier;              // compacted active sources
    uint32_t* voff;                  // push: offset of each source's first vector among the frontier's
    uint32_t* vdelta;                // push: first vector index in the list minus voff (mod 2^32)
    uint32_t* tile_first;            // push: frontier entry owning the first vector of each tile
    uint32_t* fr_part;               // push: per-block source and vector totals (scanned)
    uint32_t* touched;               // BFS destinations reached in this phase
    unsigned long long* cand64;      // BFS pull: (vector index, ~source) per destination
    uint32_t* cand32;                // BFS push: smallest source per destination
    uint32_t* counters;              // [0] frontier size, [1] touched count
    unsigned long long* vote;        // GRZ_VOTE_SLOTS * GRZ_VOTE_STRIDE
    unsigned long long* chg;         // CC: smallest label written per iteration, tagged (2 words, grz_ccbfs.cu)
    unsigned long long mail_chg[2];  // host copy of the initial chg words (outlives the async copy)
    int cc_partial;                  // a phases.h pull covered part of the list: no converged-destination skip
    unsigned* dev_err;               // set by an edge phase whose bounded wait gave up
    // engine policy
    int policy;                      // GRZ_POLICY_*
    grz_mlp* mlp;
    int next_pull;                   // learned decision for the next iteration
    int last_engine;
    float last_features[GRZ_MLP_FEATURES];
    void* sw_out;                    // device: vote, decision, counts, ticket, features
    void* mail;                      // pinned host: read-back of the vote slots or of sw_out
    float last_edge_ms;              // edge-phase time of the last step when timing is on
    int time_edges;
    cudaEvent_t ev[2];
    // the run as one CUDA graph (WHILE over two iterations with IF nodes per engine)
    grz_runctl* ctl;                 // device
    const uint32_t* level_dev;       // set while capturing: BFS level read from ctl->level
    cudaGraphExec_t run_exec;
    unsigned long long* run_bm[2];   // the HasInfo buffers in the graph's even-iteration roles
    int run_key[2];                  // app, flags of the captured graph
    grz_tuning run_tune;             // kernel shapes of the captured graph
    const uint4* run_seg;            // source-segmented lists the captured graph reads (or null)
    // snapshot for timing both engines from one state
    void* snap;
    uint64_t snap_bytes;
    uint64_t snap_scalars[8];
    // the buffers outlive a reload of a graph with the same V (cudaMalloc and cudaFree synchronise
    // the device); what depends on the lists is rebuilt at the next initialisation
    uint64_t alloc_V;                // V the per-vertex buffers are sized for
    uint64_t tile_cap;               // entries of tile_first
    int lists_changed;
};

struct grz_graph {
    int device;
    cudaStream_t stream;
    int own_stream;
    cudaStream_t copy_stream;  // second H2D copy of a load, overlapped with the first list's build
    cudaEvent_t copy_ev[2];
    uint64_t V, E;
    grz_list pull, push;
    double* outdeg;       // double[V+8]
    uint32_t* degree;     // uint32[V]
    double* inv_deg;      // double[V]
    // PageRank state
    u128* pr_fx[2];
    int pr_cur;           // which pr_fx holds the current props
    u128* pr_sum;         // u128[2][V/256]: per-block partials of S_k (ping-pong)
    double* pr_K;         // per-iteration constant G*d + (1-d)/V, written by the gather kernel
    int pr_sum_cur;
    u128* pr_rowacc;      // u128[V+1] exact per-destination accumulators
    uint32_t* pr_cut;     // uint32[V/32]: destinations whose pull vectors straddle a gather tile
    int pr_rowacc_stale;  // fused iterations cleared only the straddling accumulators
    int pr_lists_changed; // the PageRank arrays were kept across a reload with the same V
    uint32_t pr_nparts[2];  // partials in each half of pr_sum
    // source-segmented pull lists (grz_pr.cu): vectors of the edges whose source lies in segment s
    // (sources [s << seg_bits, (s + 1) << seg_bits)), grouped by destination, concatenated in
    // segment order; built at grz_pr_init when the gathered props exceed L2
    uint32_t seg_bits;    // 0: not built
    uint32_t nseg;
    uint64_t seg_first[GRZ_PR_MAX_SEGMENTS + 1];
    uint4* seg_nbr;
    uint32_t* seg_dst;
    int pr_segmode;       // fused iterations gather segment by segment
    void* pr_bar;         // grid barrier and phase timer of the persistent PageRank kernel (device)
    void* pr_bar_host;    // pinned read-back of its error word and phase times
    double* pr_d[2];      // double[V+1]: the props as doubles, gathered instead of pr_fx in pr_dmode
    int pr_dmode;         // fused iterations gather pr_d
    int pr_fx_stale;      // pr_fx[pr_cur] is behind pr_d[pr_cur]
    int pr_d_stale;       // pr_d[pr_cur] is behind pr_fx[pr_cur]
    double pr_damping;
    uint32_t pr_iters_done;
    double* prop;         // double[V+8]: reference-format vertex props (PR props, CC labels, BFS parents)
    double* accum;        // double[V+8]: reference accumulators (PR) / HasInfo* bitmap (CC, BFS)
    // scratch
    void* scratch;
    size_t scratch_bytes;
    // global accumulator of the phase API (exact)
    u128* glob;           // u128[GRZ_SUM_SLOTS] device
    int app;              // 0 PR, 1 CC, 2 BFS
    int num_sms;
    int l2_bytes;
    // iteration stats (grz_stats.cu): vectors and valid lanes the edge phases processed
    int stats_on;
    unsigned long long* stats_dev;  // [vectors counted on the device, valid lanes]
    unsigned long long* prof_work;  // while profiling: vectors the CC open-destination pulls read [first pulls, later pulls]
    uint64_t stats_host[1];         // vectors of whole ranges, counted on the host
    uint32_t max_degree;
    int max_degree_known;
    grz_frontier_state fr;
    grz_prof* prof;       // kernel timing (null unless enabled)
    unsigned long long nlaunch;  // kernels launched by this graph (grz_launch_count)
    grz_tuning tune;
    char err[256];
};

#define GRZ_COUNT_LAUNCH(g) ((g)->nlaunch++)

// CC/BFS state that belongs to the loaded lists: a reload with the same V keeps the buffers
// but marks them stale until grz_frontier_init rebuilds what depends on the lists
static inline bool grz_frontier_live(const grz_graph* g) { return g->fr.label && !g->fr.lists_changed; }
// PageRank state of the loaded lists (grz_pr_init since the last load)
static inline bool grz_pr_live(const grz_graph* g) { return g->pr_fx[0] && !g->pr_lists_changed; }

// The streamed device arrays of a graph (vector lists, row pointers, degrees, the edge pairs of a
// load, temporaries) come from its device's stream-ordered pool, allocated and freed on the
// graph's stream.  The pool keeps freed memory (its release threshold is raised once per device
// when a graph is created), so reloading a graph reuses memory without synchronising the device.
// Arrays that kernels gather from at random (labels, frontier bitmaps, PageRank props) use
// cudaMalloc: random gathers from pool memory measured 12% slower on GB300.
int grz_dev_alloc(grz_graph* g, void** p, size_t bytes);
void grz_dev_free(grz_graph* g, void* p);

// record an event pair around a launch when profiling is on
void grz_prof_begin(grz_graph* g, int kind);
void grz_prof_end(grz_graph* g);

// warp 0 of the calling block: exact sum of GRZ_SUM_SLOTS slots (result valid in lane 0)
__device__ __forceinline__ u128 u128_warp_sum_slots(const u128* slots)
{
    const int lane = threadIdx.x & 31;
    u128 s = u128_add(slots[lane], slots[lane + 32]);
    for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
    return s;
}

static inline u128 u128_host_sum(const u128* slots, int n)
{
    u128 s = u128_zero();
    for (int i = 0; i < n; ++i) s = u128_add(s, slots[i]);
    return s;
}

// ----------------------------------------------------------------------------------------------
// kernel-level profiling (CUDA event pairs around launches), the GPU analogue of the reference's
// EXPERIMENT_ITERATION_PROFILE cycle counts (source/execution_bfs.c:172-215)

#define GRZ_PROF_MAX 8192
enum grz_prof_kind {
    GRZ_PROF_PR_GATHER = 1, GRZ_PROF_PR_APPLY, GRZ_PROF_PR_PUSH, GRZ_PROF_PR_VERTEX,
    GRZ_PROF_CC_PULL, GRZ_PROF_CC_PUSH, GRZ_PROF_BFS_PULL, GRZ_PROF_BFS_PUSH,
    GRZ_PROF_FRONTIER, GRZ_PROF_VERTEX, GRZ_PROF_ITERATION, GRZ_PROF_MLP, GRZ_PROF_BATCH,
    GRZ_PROF_BFS_VISIT, GRZ_PROF_PUSH_COMPACT,
    GRZ_PROF_KINDS
};

struct grz_prof {
    int on;
    int n;
    int kind[GRZ_PROF_MAX];
    cudaEvent_t ev[GRZ_PROF_MAX][2];
    float direct_ms[GRZ_PROF_MAX];  // >= 0: a duration measured on the device (%globaltimer), no events
    int created;
};
// a record whose duration the device measured itself (phases of a persistent kernel)
void grz_prof_direct(grz_graph* g, int kind, float ms);

// host helpers (grz_api.cu)
int grz_set_error(grz_graph* g, int code, const char* fmt, ...);
int grz_cuda_check(grz_graph* g, cudaError_t e, const char* what);
int grz_scratch(grz_graph* g, size_t bytes, void** out);

#define GRZ_TRY(expr) do { const int rc_try_ = (expr); if (rc_try_) return rc_try_; } while (0)
#define GRZ_CK(g, call)                                         \
    do {                                                        \
        cudaError_t e__ = (call);                               \
        if (e__ != cudaSuccess) return grz_cuda_check((g), e__, #call); \
    } while (0)

// CC / BFS (grz_ccbfs.cu)
int grz_frontier_init(grz_graph* g, int app, int flags, uint32_t root);
int grz_frontier_step(grz_graph* g, int engine, int* engine_out, uint64_t* vote_out);
int grz_frontier_vertex_phase(grz_graph* g, uint64_t first, uint64_t count);
int grz_frontier_props(grz_graph* g);
int grz_engine_threshold(const grz_graph* g, uint64_t vote);
int grz_read_vote(grz_graph* g, uint64_t* out);
int grz_frontier_mail(grz_graph* g);
int grz_frontier_run_graph(grz_graph* g, uint64_t* launches);
int grz_frontier_check_waits(grz_graph* g);
// builds the source-segmented pull lists by the size rule of grz_pr_init (grz_pr.cu); `force`:
// also below the size threshold, with the tuned or the default segment size
int grz_pr_ensure_segments(grz_graph* g, int force);
void grz_frontier_run_prepare(grz_graph* g);
int grz_frontier_digest(grz_graph* g, uint64_t* out3);
int grz_switch_max_degree(grz_graph* g);
void grz_switch_policy_ctl(grz_graph* g, grz_runctl* c);
int grz_switch_launch_run_decide(grz_graph* g, const unsigned long long* next_frontier, unsigned long long* clear_bm, int initial,
                                 unsigned long long hloop, unsigned long long hpull, unsigned long long hpush);
// learned switch: features of a state + the policy's decision; frontier = HasInfo of the
// iteration the decision is for; vote_override = ~0 to read the vote slots
int grz_switch_decide(grz_graph* g, const unsigned long long* frontier, uint64_t vote_override, uint32_t iter,
                      uint64_t* vote, int* next_pull, float* features);
void grz_frontier_free(grz_graph* g);
void grz_frontier_park(grz_graph* g);  // before a reload with the same V: keep the buffers

// layout (grz_layout.cu)
// run_len (optional, uint32[V]): edges of each shared vertex
int grz_build_list(grz_graph* g, grz_list* L, const uint64_t* d_pairs, uint64_t E, int shared_is_dst,
                   uint32_t* run_len = nullptr);
int grz_list_reference(grz_graph* g, grz_list* L);  // reference-format vectors, built on first request
int grz_stats_count_range(grz_graph* g, const grz_list* L, uint64_t first, uint64_t count);
int grz_stats_count_selected(grz_graph* g, const grz_list* L, const uint32_t* sel, const uint32_t* counters);
int grz_build_hubs(grz_graph* g, grz_list* L, uint32_t max_hubs);
// both lists and the outdegrees from E > 0 -pull pairs in pinned host or device memory (grz_sort.cu)
// (pull: device-readable pairs; host: the same pairs' pinned host address, to copy them chunk by
// chunk, or null when pull is device memory)
int grz_ingest_pull_derive(grz_graph* g, const uint64_t* pull, uint64_t E, const uint64_t* host);
cudaError_t grz_copy_stream(grz_graph* g);
int grz_build_list_from_bounds(grz_graph* g, grz_list* L, const uint64_t* d_pairs, uint64_t E, int shared_is_dst,
                               const uint32_t* start, const uint32_t* end, uint64_t first_shared, uint64_t last_shared,
                               uint32_t* run_len, cudaStream_t st, uint64_t written_cap);
#define GRZ_LOAD_DERIVE_PUSH 1
int grz_alloc_outdegrees(grz_graph* g);
int grz_build_outdegrees(grz_graph* g, const uint64_t* d_pull_pairs, uint64_t E, cudaStream_t st = nullptr);

// scans (grz_scan.cu): exclusive sum of uint32 into uint32 (n < 2^32), inclusive max of uint32
int grz_exclusive_sum_u32(grz_graph* g, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total_out_dev);
int grz_exclusive_sum_u32_on(grz_graph* g, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total_out_dev,
                             cudaStream_t st);  // ordered on st
int grz_inclusive_max_u32(grz_graph* g, const uint32_t* in, uint32_t* out, uint64_t n);
