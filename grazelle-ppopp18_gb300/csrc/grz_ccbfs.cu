// grz_ccbfs.cu -- Connected Components and Breadth-First Search: edge-pull, edge-push on a
// compacted frontier, vertex (frontier) phase, and the engine-switching driver loops.
//
// Reference semantics (paths in the Grazelle tree):
//   CC pull   source/phase_edge_pull_cc.asm:50-392   label[d] = min(label[d], min over valid sources)
//   CC push   source/phase_edge_push_cc.asm:51-573   for sources in HasInfo: CAS-min into label[dst]
//   BFS pull  source/phase_edge_pull_bfs.asm:53-211  for dst in WantsInfo: parent = max HasInfo source
//                                                    of the first vector that holds one
//   BFS push  source/phase_edge_push_bfs.asm:53-202  for sources in HasInfo: visit dst in WantsInfo
//   vertex    source/phase_vertex_{cc,bfs}.asm:37-46 zero HasInfo* after the pointer swap
//   driver    source/execution_cc.c:94-268, source/execution_bfs.c:120-276
//   vote      include/phasehelpers.inc:388-399       1 + outdeg per changed vertex
//
// GPU form:
//   * Labels and parents live on the device as uint32 (IDs are below 2^32).  The reference's
//     double props are produced only when the result is read back.  Entry V of the label
//     array is a permanent +infinity that invalid lanes gather.
//   * Pull: one thread per vector, a warp-segmented reduction per destination, one atomic per
//     (warp, destination).  Labels are updated in place, as the reference's CAS loop does, so
//     a later vector may already see a lowered label.
//   * Push: HasInfo is compacted, in vertex order, into a list of active sources that have
//     out-edges, with a scan of their vector counts.  The concatenation of their vector ranges
//     is expanded in tiles of 1024 vectors over the whole grid, so neither threads nor blocks
//     wait on high-degree sources.
//   * Each changed vertex is counted once per iteration: the first setter of its HasInfo* bit
//     adds 1 + outdeg to the vote.  The reference can count a destination that straddles two
//     work units twice.  The vote only steers the engine choice.
//   * BFS parent rules are deterministic, so parents equal the single-thread reference: pull
//     keeps the largest HasInfo source of the lowest-indexed vector that holds one (a 64-bit
//     atomicMin on (vector index, ~source)); push keeps the smallest HasInfo source (atomicMin).
//     A vertex's BFS level is the iteration that visits it, so levels are exact by construction.
#include <string.h>

#include <algorithm>
#include <type_traits>

#include "grz_internal.cuh"

namespace {

constexpr int T = 256;
constexpr uint32_t INF = 0xffffffffu;
// BFS visit: sweep all vertices instead of the touched list when more than V / this were touched
constexpr uint64_t VISIT_DENSE_RATIO = 128;
// tiles of T vectors per step of the BFS pull kernel
constexpr int BFS_PULL_TILES = 4;
// bitmap words (64 destinations each) a warp of the first-vector passes owns, and their blocks per SM
#ifndef GRZ_BFS_FW
#define GRZ_BFS_FW 2
#endif
#ifndef GRZ_BFS_MINB
#define GRZ_BFS_MINB 8
#endif
constexpr int FW = GRZ_BFS_FW;

unsigned blocks_for(uint64_t n) { return (unsigned)((n + T - 1) / T); }

__device__ __forceinline__ bool bit_of(const unsigned long long* bm, uint32_t v) { return (bm[v >> 6] >> (v & 63)) & 1ull; }

// sets bit v; true if this call set it (it was clear)
__device__ __forceinline__ bool bit_set_first(unsigned long long* bm, uint32_t v)
{
    const unsigned long long m = 1ull << (v & 63);
    return !(atomicOr(bm + (v >> 6), m) & m);
}

__device__ __forceinline__ void vote_add(unsigned long long* vote, unsigned long long x)
{
    // one add per block (the callers aggregate the block first), spread over the vote slots
    if (x) atomicAdd(vote + (blockIdx.x & (GRZ_VOTE_SLOTS - 1)) * GRZ_VOTE_STRIDE, x);
}

__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long x, unsigned long long* red)
{
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    x = 0;
    if (threadIdx.x < 32) {
        x = (threadIdx.x < T / 32) ? red[threadIdx.x] : 0ull;
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    }
    return x;
}

// Appends `val` to the BFS touched list for the lanes with `pred`, one atomicAdd per warp (all 32
// lanes call it together; the callers' loops are warp-uniform), until the list holds
// V / VISIT_DENSE_RATIO + 1 entries.  From there on k_bfs_visit sweeps all vertices instead of
// reading the list (the count only grows), so further appends are skipped: a plain load of the
// counter replaces the atomic, and a large iteration no longer queues millions of atomics on one
// address.  Each destination is first-touched once per phase, so the list never outgrows V.
__device__ __forceinline__ bool touched_full(const uint32_t* count, uint32_t V)
{
    return *(volatile const uint32_t*)count >= (uint32_t)((uint64_t)V / VISIT_DENSE_RATIO + 1);
}

// `full`: touched_full as the caller last read it (once per tile or step, warp-uniform); the
// count can pass the bound between two reads, which only lets a few more appends through
__device__ __forceinline__ void touched_append(bool pred, uint32_t val, uint32_t* __restrict__ list, uint32_t* __restrict__ count,
                                               bool full)
{
    if (full) return;
    const unsigned m = __ballot_sync(0xffffffffu, pred);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pred) list[base + __popc(m & ((1u << lane) - 1u))] = val;
}

struct VoteCfg {
    const uint32_t* degree;
    int without_count, without_outdeg;
    __device__ __forceinline__ unsigned long long of(uint32_t v) const
    {
        return (without_count ? 0ull : 1ull) + (without_outdeg ? 0ull : (unsigned long long)degree[v]);
    }
};

// ---------------------------------------------------------------------------------------------
// CC pull

// Smallest label written by a CC iteration, for the next iteration's converged-destination
// skip.  Iteration k adds ((k << 32) | ~m) into word k & 1 with atomicMax, m the smallest label
// it wrote; the words are never reset: a tag other than k - 1 means "unknown" and the reader
// does not skip.  Why the skip is exact: after a complete iteration (a pull over the
// whole list, or a push from the whole frontier) every destination d holds at most the labels
// its sources had when d was last evaluated, so only a source that changed since can lower d.
// Every such change happened in iteration k - 1 (earlier ones were evaluated or pushed in
// k - 1) or happens during iteration k (recorded in HasInfo*, handled in k + 1).  A change in
// k - 1 wrote a label >= m(k - 1); so if label[d] <= m(k - 1), iteration k cannot lower d.
// Iteration 1 follows the initial state, in which every vertex counts as changed: no skip.
__device__ __forceinline__ bool cc_prev_min(const unsigned long long* __restrict__ chg, uint32_t k, uint32_t* m)
{
    if (k < 2) return false;
    const unsigned long long w = chg[(k - 1) & 1];
    if ((uint32_t)(w >> 32) != k - 1) return false;
    *m = ~(uint32_t)w;
    return true;
}

// block-wide minimum of one value per thread, then one tagged atomicMax (threadIdx.x 0 only)
template <int BT>
__device__ __forceinline__ void cc_record_min(uint32_t my_min, uint32_t* red32, unsigned long long* __restrict__ chg, uint32_t k)
{
    my_min = __reduce_min_sync(0xffffffffu, my_min);
    if ((threadIdx.x & 31) == 0) red32[threadIdx.x >> 5] = my_min;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t x = threadIdx.x < BT / 32 ? red32[threadIdx.x] : INF;
        x = __reduce_min_sync(0xffffffffu, x);
        if (threadIdx.x == 0 && x != INF) atomicMax(chg + (k & 1), ((unsigned long long)k << 32) | (unsigned long long)(~x));
    }
}

// Persistent, BT threads per block, one thread per vector per tile of BT vectors.  The labels
// of the first `ncache` hub slots are copied into shared memory when the block starts; lanes
// that name them read shared memory instead of gathering through L1 (in a power-law graph most
// lanes).  Those copies may fall behind the in-place updates of this phase, which the
// reference's asynchronous CAS loop allows as well: a label only ever decreases, every value
// read is one the source really had, and an iteration that changes nothing is still a fixpoint.
// Iteration k (epoch_dev, else epoch) skips destinations whose label is at most the smallest
// label written in iteration k - 1 (cc_prev_min; only with use_prev, i.e. when k - 1 was a
// complete iteration): it reads their destination and label, not their vectors.  R-MAT's
// hubs have the smallest IDs, so after the first iteration most of the giant component holds
// label 0 and the second pull reads little more than the destinations.
// tiles whose destination and label loads the skip mode issues together
constexpr int SKIP_TILES = 4;

// double-buffered staging of the edge stream in shared memory (the bulk-copy form)
template <int BT>
struct CCStage {
    uint4 nbr[2][BT];
    uint32_t dst[2][BT];
    unsigned long long bar[2];
};
struct CCNoStage {};

template <int BT, bool BULK>
__global__ void __launch_bounds__(BT) k_cc_pull(const uint4* __restrict__ nbr, const uint32_t* __restrict__ dstv, uint64_t first,
                                                uint64_t nvec, uint32_t V, uint32_t* __restrict__ label,
                                                const uint32_t* __restrict__ hub_vid, uint32_t nhub, uint32_t ncache,
                                                unsigned long long* __restrict__ has_next, VoteCfg vc,
                                                unsigned long long* __restrict__ vote, unsigned long long* __restrict__ chg,
                                                uint32_t epoch, const uint32_t* __restrict__ epoch_dev, int use_prev,
                                                unsigned* __restrict__ err)
{
    extern __shared__ uint32_t s_hub[];
    __shared__ unsigned long long red[BT / 32];
    __shared__ uint32_t red32[BT / 32];
    __shared__ __align__(16) typename std::conditional<BULK, CCStage<BT>, CCNoStage>::type stg;
    for (uint32_t k = threadIdx.x; k < ncache; k += BT) s_hub[k] = label[__ldg(hub_vid + k)];
    const uint32_t ep = epoch_dev ? *epoch_dev : epoch;
    uint32_t mprev = 0;
    bool skip = use_prev && cc_prev_min(chg, ep, &mprev);
    // use_prev 2: a source-segment pass, which runs only when the skip is off (the full pass);
    // use_prev 3: the pass over the whole list that runs only when it is on (the grid agrees)
    if ((use_prev == 2 && skip) || (use_prev == 3 && !skip)) return;
    // use_prev 4: after k_cc_pull_first, which ran because the skip is off: the destinations
    // whose label is already 0, the smallest there is, need none of their vectors
    // use_prev 5: the same, but only then (a later iteration is left to the open-destination pass)
    if (use_prev == 5 && skip) return;
    if ((use_prev == 4 || use_prev == 5) && !skip) {
        skip = true;
        mprev = 0;
    }
    const int lane = threadIdx.x & 31;
    unsigned long long my_vote = 0;
    uint32_t my_min = INF;
    const uint64_t ntiles = (nvec + BT - 1) / BT;
    const uint64_t nfull = nvec / BT;  // tiles the bulk copies serve (whole tiles only)
    // The bulk form copies each whole tile's vectors and destinations into shared memory on the
    // copy engine, two tiles ahead, so the SM's load path serves only the label gathers.  Not in
    // skip mode (it reads most vectors' destinations only) nor for a vector sub-range.
    const bool bulk = BULK && !skip && first == 0;
    unsigned par = 0u;  // bit j: the parity stage j waits for next
    if constexpr (BULK) {
        if (bulk && threadIdx.x == 0) {
            mbar_init(&stg.bar[0], 1);
            mbar_init(&stg.bar[1], 1);
            mbar_fence_init();
            for (int j = 0; j < 2; ++j) {
                const uint64_t t = blockIdx.x + (uint64_t)j * gridDim.x;
                if (t < nfull) {
                    mbar_arrive_expect_tx(&stg.bar[j], BT * (sizeof(uint4) + sizeof(uint32_t)));
                    bulk_copy_g2s(stg.nbr[j], nbr + t * BT, BT * sizeof(uint4), &stg.bar[j]);
                    bulk_copy_g2s(stg.dst[j], dstv + t * BT, BT * sizeof(uint32_t), &stg.bar[j]);
                }
            }
        }
    }
    __syncthreads();
    // one tile's reduction and updates, once its destinations (key), their labels if known (labd,
    // skip mode) and its vectors (staged, or loaded here when needed) are at hand
    auto finish = [&](uint64_t v, bool live, uint32_t key, uint32_t labd, bool need, bool staged, uint4 sv) {
        uint32_t m = INF;
        if (need) {
            const uint4 s4 = staged ? sv : ld_stream(nbr + v);
            const uint32_t x[4] = { s4.x, s4.y, s4.z, s4.w };
            auto fetch = [&](uint32_t xl) -> uint32_t {
                const uint32_t sl = xl - GRZ_HUB_BASE;
                if (sl < ncache) return s_hub[sl];
                // labels change in place during the phase: plain (coherent) loads
                const uint32_t id = sl < nhub ? __ldg(hub_vid + sl) : min(xl, V);
                return ld_label(label + id);
            };
            // A vector's lanes hold its sources in ascending order, so lane 0 is the
            // smallest-ID source: in a power-law graph often a hub whose label is already 0.
            // Then the minimum is 0 and the other three gathers are not issued.
            m = fetch(x[0]);
            if (m != 0) m = min(m, min(min(fetch(x[1]), fetch(x[2])), fetch(x[3])));
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
            if (lane - off >= segstart) m = min(m, o);
        }
        if (live && tail && m != INF && m < (skip ? labd : label[key])) {
            const uint32_t old = atomicMin(label + key, m);
            if (m < old) {
                my_min = min(my_min, m);
                if (bit_set_first(has_next, key)) my_vote += vc.of(key);
            }
        }
    };
    if (skip) {
        // Skip mode: a vector is read only if its destination's label can still drop.  Each
        // block takes SKIP_TILES consecutive tiles at a time and issues all their destination
        // loads, then all their label loads, before any tile goes on: the chain destination ->
        // label -> vector is latency-bound, so this keeps SKIP_TILES times more loads in flight.
        constexpr int U = SKIP_TILES;
        for (uint64_t t0 = (uint64_t)blockIdx.x * U; t0 < ntiles; t0 += (uint64_t)gridDim.x * U) {
            uint32_t keys[U], labs[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint64_t i = (t0 + u) * BT + threadIdx.x;
                keys[u] = i < nvec ? ld_stream(dstv + first + i) : INF;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) labs[u] = keys[u] != INF ? ld_label(label + keys[u]) : INF;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint64_t i = (t0 + u) * BT + threadIdx.x;
                const bool live = i < nvec;
                const bool need = live && labs[u] > mprev;
                if (!__any_sync(0xffffffffu, need)) continue;  // warp-uniform
                finish(first + i, live, keys[u], labs[u], need, false, make_uint4(INF, INF, INF, INF));
            }
        }
    } else {
        uint64_t j = 0;
        for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++j) {
            const uint64_t i = t * BT + threadIdx.x;
            const uint64_t v = first + i;
            const bool live = i < nvec;
            uint32_t key = INF;
            bool staged = false;
            uint4 sv = make_uint4(INF, INF, INF, INF);
            if constexpr (BULK) {
                if (bulk && t < nfull) {
                    const int st = (int)(j & 1);
                    const bool ok = mbar_wait_bounded(&stg.bar[st], (par >> st) & 1u);
                    if (__syncthreads_or(!ok)) {
                        if (threadIdx.x == 0) atomicExch(err, 1u);
                        return;
                    }
                    par ^= 1u << st;
                    sv = stg.nbr[st][threadIdx.x];
                    key = stg.dst[st][threadIdx.x];
                    staged = true;
                    __syncthreads();  // every thread has read the stage
                    const uint64_t tn = t + 2ull * gridDim.x;
                    if (threadIdx.x == 0 && tn < nfull) {
                        fence_proxy_async_smem();
                        mbar_arrive_expect_tx(&stg.bar[st], BT * (sizeof(uint4) + sizeof(uint32_t)));
                        bulk_copy_g2s(stg.nbr[st], nbr + tn * BT, BT * sizeof(uint4), &stg.bar[st]);
                        bulk_copy_g2s(stg.dst[st], dstv + tn * BT, BT * sizeof(uint32_t), &stg.bar[st]);
                    }
                }
            }
            if (live && !staged) key = ld_stream(dstv + v);
            finish(v, live, key, INF, live, staged, sv);
        }
    }
    for (int o = 16; o > 0; o >>= 1) my_vote += __shfl_down_sync(0xffffffffu, my_vote, o);
    if (lane == 0) red[threadIdx.x >> 5] = my_vote;
    cc_record_min<BT>(my_min, red32, chg, ep);  // (contains the __syncthreads the vote sum needs)
    if (threadIdx.x < 32) {
        unsigned long long x = threadIdx.x < BT / 32 ? red[threadIdx.x] : 0ull;
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (threadIdx.x == 0) vote_add(vote, x);
    }
}

// CC pull, first-vector pass of an iteration without a usable previous minimum (the first pull of
// a run).  Each destination's first vector holds its smallest-ID sources; in a power-law graph
// one of them is usually a hub whose label is 0 by the time it is read (in place, as the full
// pass reads them), and then the destination's label is final for this iteration: 0 cannot be
// lowered.  This pass evaluates every destination's first vector (lane 0 first, as in
// k_cc_pull), one destination per thread, and writes the new labels.  What follows reads the
// other vectors of the destinations still above 0, so the iteration's result is the full pull's:
// in the default form (GRZ_TUNE_CC_PULL_FIRST 4) the compaction of the destinations this pass
// marks in `unres` (open_all: every one still above 0) and k_cc_pull_expand over all their
// vectors; in form 2 the same for the remaining vectors of those with more than one; in forms 1
// and 3 the pass over the whole list (k_cc_pull with use_prev 4 or 5) that skips the
// destinations at 0.  A warp owns CFW bitmap words (64 destinations each), so it writes their
// HasInfo* and `unres` bits without atomics; the pass records its smallest label written for the
// next iteration's skip, and sets *gate to 1 in an iteration it runs, 0 in one it leaves to the
// later-pull kernels.
#ifndef GRZ_CC_FW
#define GRZ_CC_FW 1
#endif
// bitmap words a warp of k_cc_pull_first owns (GB300, R-MAT 24 sym: 1 word 0.42 ms for the first pull,
// 2 words 0.46 ms, with 60 bytes of spills at 32 registers)
constexpr int CFW = GRZ_CC_FW;

__global__ void __launch_bounds__(T, 8) k_cc_pull_first(const uint32_t* __restrict__ rowptr, const uint4* __restrict__ nbr,
                                                      uint32_t V, uint64_t W, uint32_t* __restrict__ label,
                                                      const uint32_t* __restrict__ hub_vid, uint32_t nhub,
                                                      unsigned long long* __restrict__ has_next, VoteCfg vc,
                                                      unsigned long long* __restrict__ vote, unsigned long long* __restrict__ chg,
                                                      uint32_t epoch, const uint32_t* __restrict__ epoch_dev,
                                                      unsigned long long* __restrict__ unres, uint32_t* __restrict__ gate,
                                                      int open_all)
{
    __shared__ unsigned long long red[T / 32];
    __shared__ uint32_t red32[T / 32];
    const uint32_t ep = epoch_dev ? *epoch_dev : epoch;
    uint32_t mprev = 0;
    const bool skip_iteration = cc_prev_min(chg, ep, &mprev);  // the same on every thread
    if (gate && blockIdx.x == 0 && threadIdx.x == 0) *gate = skip_iteration ? 0u : 1u;
    if (skip_iteration) return;  // the skip pass does this iteration alone
    constexpr int Q = 2 * CFW;
    const int lane = threadIdx.x & 31;
    unsigned long long my_vote = 0;
    uint32_t my_min = INF;
    auto fetch = [&](uint32_t xl) -> uint32_t {
        const uint32_t sl = xl - GRZ_HUB_BASE;
        const uint32_t id = sl < nhub ? __ldg(hub_vid + sl) : min(xl, V);
        return ld_label(label + id);
    };
    const uint64_t nwarps = (uint64_t)gridDim.x * (T / 32);
    // row pointers of a group of destinations (a and b: start and end of each slot's range)
    auto rows = [&](uint64_t w, uint32_t* a, uint32_t* b) {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const uint64_t v = 64 * w + 32 * (uint64_t)q + lane;
            a[q] = b[q] = 0;
            if (w < W && v < V) {
                a[q] = rowptr[v];
                b[q] = rowptr[v + 1];
            }
        }
    };
    uint64_t w0 = ((uint64_t)blockIdx.x * (T / 32) + (threadIdx.x >> 5)) * CFW;
    uint32_t ra[Q], rb[Q];
    rows(w0, ra, rb);
    for (; w0 < W; w0 += nwarps * CFW) {  // warp-uniform
        uint32_t r0[Q], n[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            r0[q] = ra[q];
            n[q] = rb[q] - ra[q];
        }
        uint4 sv[Q];
        uint32_t cur[Q];  // the destinations' own labels, loaded with their first vectors
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            sv[q] = n[q] ? ld_stream(nbr + r0[q]) : make_uint4(INF, INF, INF, INF);
            cur[q] = n[q] ? ld_label(label + (uint32_t)(64 * w0 + 32 * (uint64_t)q + lane)) : 0u;
        }
        uint32_t m[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) m[q] = n[q] ? fetch(sv[q].x) : INF;
#pragma unroll
        for (int q = 0; q < Q; ++q)
            if (m[q] != 0 && n[q]) m[q] = min(m[q], min(min(fetch(sv[q].y), fetch(sv[q].z)), fetch(sv[q].w)));
#pragma unroll
        for (int f = 0; f < CFW; ++f) {
            // word w0 + f: new labels of its 64 destinations, then its HasInfo* bits (set by lane 0;
            // a destination counts in the vote if its bit was clear)
            unsigned long long hn = 0ull, un = 0ull;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int q = 2 * f + h;
                const uint32_t v = (uint32_t)(64 * w0 + 32 * (uint64_t)q + lane);
                bool ch = false, more = false;
                if (n[q]) {
                    // this thread is the destination's only writer in this pass, so its label read
                    // with the vector is still current
                    if (m[q] < cur[q]) {
                        label[v] = m[q];
                        my_min = min(my_min, m[q]);
                        ch = true;
                    }
                    // still open: its other vectors (open_all: all of them again) are read next
                    more = (open_all || n[q] > 1) && min(m[q], cur[q]) != 0;
                }
                hn |= (unsigned long long)__ballot_sync(0xffffffffu, ch) << (32 * h);
                un |= (unsigned long long)__ballot_sync(0xffffffffu, more) << (32 * h);
            }
            if (unres && lane == 0 && w0 + f < W) unres[w0 + f] = un;
            if (!hn) continue;  // warp-uniform
            unsigned long long old = 0ull;
            if (lane == 0) {
                old = has_next[w0 + f];
                has_next[w0 + f] = old | hn;
            }
            const unsigned long long fresh = hn & ~__shfl_sync(0xffffffffu, old, 0);
#pragma unroll
            for (int h = 0; h < 2; ++h)
                if ((fresh >> (32 * h + lane)) & 1ull) my_vote += vc.of((uint32_t)(64 * (w0 + f) + 32 * h + lane));
        }
        // the next group's row pointers (issuing them at the top of the step instead, to overlap
        // this group's chain, needed more registers than the 32 of 8 blocks per SM and measured no
        // faster on GB300; loading the destinations' own labels with their first vectors, one
        // dependent round trip less, took the first pull at R-MAT 24 sym from 0.33 to 0.32 ms)
        rows(w0 + nwarps * CFW, ra, rb);
    }
    my_vote = block_sum_u64(my_vote, red);
    if (threadIdx.x == 0) vote_add(vote, my_vote);
    __syncthreads();
    cc_record_min<T>(my_min, red32, chg, ep);
}

// CC pull of an iteration with a usable previous minimum m (the skip of k_cc_pull): marks in
// `unres` the destinations with in-vectors whose label is above m, the only ones the iteration can
// lower, for the compaction and k_cc_pull_expand; *gate = 1.  In an iteration without a usable
// minimum it only sets *gate = 0.  A warp per bitmap word: each lane reads two labels.
__global__ void __launch_bounds__(T) k_cc_mark_open(const uint32_t* __restrict__ label, const unsigned long long* __restrict__ nonempty,
                                                    uint64_t V, uint64_t W, const unsigned long long* __restrict__ chg, uint32_t epoch,
                                                    const uint32_t* __restrict__ epoch_dev, unsigned long long* __restrict__ unres,
                                                    uint32_t* __restrict__ gate)
{
    const uint32_t ep = epoch_dev ? *epoch_dev : epoch;
    uint32_t mprev = 0;
    const bool skip_iteration = cc_prev_min(chg, ep, &mprev);
    if (gate && blockIdx.x == 0 && threadIdx.x == 0) *gate = skip_iteration ? 1u : 0u;
    if (!skip_iteration) return;
    const int lane = threadIdx.x & 31;
    const uint64_t nwarps = (uint64_t)gridDim.x * (T / 32);
    for (uint64_t w = (uint64_t)blockIdx.x * (T / 32) + (threadIdx.x >> 5); w < W; w += nwarps) {  // warp-uniform
        const uint64_t v0 = 64 * w + lane, v1 = v0 + 32;
        const bool o0 = v0 < V && ld_label(label + v0) > mprev;
        const bool o1 = v1 < V && ld_label(label + v1) > mprev;
        const unsigned long long m = (unsigned long long)__ballot_sync(0xffffffffu, o0) |
                                     ((unsigned long long)__ballot_sync(0xffffffffu, o1) << 32);
        if (lane == 0) unres[w] = m & nonempty[w];
    }
}

// ---------------------------------------------------------------------------------------------
// BFS pull

// BFS pull (phase_edge_pull_bfs.asm:53-211), persistent over tiles of T vectors.  For a
// wanted destination, a vector's candidate is (vector index, ~largest HasInfo source); the
// smallest candidate per destination wins: the reference's parent rule (the largest frontier
// source of the first vector that has one).  Vectors of one destination are reduced within
// the warp first, so only one atomicMin per (warp, destination) reaches memory.
__global__ void __launch_bounds__(T) k_bfs_pull(const uint4* __restrict__ nbr, const uint32_t* __restrict__ dstv, uint64_t first,
                                                uint64_t nvec, uint32_t V, const unsigned long long* __restrict__ has,
                                                const unsigned long long* __restrict__ wants,
                                                unsigned long long* __restrict__ cand, uint32_t* __restrict__ touched,
                                                uint32_t* __restrict__ ntouched, const uint32_t* __restrict__ hub_vid, uint32_t nhub,
                                                unsigned long long* __restrict__ has_next)
{
    // U tiles per step: their destination loads, then their WantsInfo loads, are issued together
    // (enough bytes in flight per SM to cover DRAM latency);
    // late in a BFS most destinations are visited and a warp without a wanted one skips its tile
    constexpr int U = BFS_PULL_TILES;
    const int lane = threadIdx.x & 31;
    const uint64_t ntiles = (nvec + T - 1) / T;
    for (uint64_t t0 = (uint64_t)blockIdx.x * U; t0 < ntiles; t0 += (uint64_t)gridDim.x * U) {
        uint32_t keys[U];
        bool want[U];
#pragma unroll
        for (int j = 0; j < U; ++j) {
            const uint64_t i = (t0 + j) * T + threadIdx.x;
            keys[j] = i < nvec ? __ldcs(dstv + first + i) : INF;
        }
#pragma unroll
        for (int j = 0; j < U; ++j) want[j] = keys[j] != INF && bit_of(wants, keys[j]);  // strong check
        const bool full = __shfl_sync(0xffffffffu, lane == 0 ? touched_full(ntouched, V) : false, 0);
#pragma unroll
        for (int j = 0; j < U; ++j) {
            if (!__ballot_sync(0xffffffffu, want[j])) continue;  // warp-uniform
            const uint64_t v = first + (t0 + j) * T + threadIdx.x;
            const uint32_t key = keys[j];
            unsigned long long k = ~0ull;
            if (want[j]) {
                const uint4 s = __ldcs(nbr + v);
                const uint32_t ids[4] = { grz_hub_decode(s.x, hub_vid, nhub), grz_hub_decode(s.y, hub_vid, nhub),
                                          grz_hub_decode(s.z, hub_vid, nhub), grz_hub_decode(s.w, hub_vid, nhub) };
                uint32_t best = 0;
                bool any = false;
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    const uint32_t id = ids[l];
                    if (id < V && bit_of(has, id)) {  // weak check on the source
                        best = any ? max(best, id) : id;
                        any = true;
                    }
                }
                if (any) k = ((unsigned long long)v << 32) | (unsigned long long)(~best);
            }
            // segmented min of k over runs of equal keys within the warp
            const uint32_t prevkey = __shfl_up_sync(0xffffffffu, key, 1);
            const uint32_t nextkey = __shfl_down_sync(0xffffffffu, key, 1);
            const bool head = lane == 0 || key != prevkey;
            const bool tail = lane == 31 || key != nextkey;
            const unsigned heads = __ballot_sync(0xffffffffu, head);
            const int segstart = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
            const int maxlen = __reduce_max_sync(0xffffffffu, (unsigned)(lane - segstart + 1));
            for (int off = 1; off < maxlen; off <<= 1) {
                const unsigned long long o = __shfl_up_sync(0xffffffffu, k, off);
                if (lane - off >= segstart) k = min(k, o);
            }
            bool first_touch = false;
            if (tail && k != ~0ull && k < cand[key]) {
                first_touch = atomicMin(cand + key, k) == ~0ull;
                if (first_touch) atomicOr(has_next + (key >> 6), 1ull << (key & 63));
            }
            touched_append(first_touch, key, touched, ntouched, full);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Push: frontier compaction and edge-balanced expansion.
//
// The active sources that have out-vectors are compacted in vertex order, each with the offset
// of its first vector in the concatenation of their vector ranges.  The expansion then splits
// that concatenation into tiles of PUSH_TILE vectors spread over the grid, so a hub's vectors
// are spread over many blocks.  tile_first[t] is the frontier entry that owns the first vector
// of tile t.  Passes: k_fr_count (per block of bitmap words: sources and vectors),
// k_fr_scan (one block: exclusive scan of the block totals), k_fr_write (frontier entries,
// their vector offsets and the tile owners), k_push_expand.

constexpr uint32_t PUSH_TILE = 1024;

// block-wide exclusive scan of two u32 values; returns the block totals through the references
__device__ __forceinline__ void block_scan2(uint32_t& a, uint32_t& b, uint32_t& tot_a, uint32_t& tot_b, uint32_t* sa,
                                            uint32_t* sb)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t xa = a, xb = b;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t ya = __shfl_up_sync(0xffffffffu, xa, o);
        const uint32_t yb = __shfl_up_sync(0xffffffffu, xb, o);
        if (lane >= o) { xa += ya; xb += yb; }
    }
    if (lane == 31) { sa[warp] = xa; sb[warp] = xb; }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t ra = 0, rb = 0;
        for (int k = 0; k < T / 32; ++k) {
            const uint32_t ta = sa[k], tb = sb[k];
            sa[k] = ra; sb[k] = rb;
            ra += ta; rb += tb;
        }
        sa[T / 32] = ra; sb[T / 32] = rb;
    }
    __syncthreads();
    a = sa[warp] + xa - a;
    b = sb[warp] + xb - b;
    tot_a = sa[T / 32];
    tot_b = sb[T / 32];
}

// The compaction kernels give each thread CU = 32 consecutive vertices (half a bitmap word) and
// each block CCHUNK consecutive vertices, so a block needs a single block-wide scan and a block
// with nothing selected exits after reading its words.  A thread with a selected vertex reads its
// 33 row pointers with 128-bit loads issued together and works from registers.  Selected: the bit
// is set in both bitmaps (HasInfo and out-vectors for push; WantsInfo and in-vectors for the BFS
// pull).
constexpr int CU = 32;
constexpr uint32_t CCHUNK = T * CU;

// selection bits of vertices [v0, v0 + CU), v0 a multiple of CU
__device__ __forceinline__ uint32_t selected_bits(const unsigned long long* __restrict__ bm1,
                                                  const unsigned long long* __restrict__ bm2, uint64_t v0, uint64_t V)
{
    if (v0 >= V) return 0u;
    const uint64_t w = v0 >> 6;
    uint32_t bits = (uint32_t)((bm1[w] & bm2[w]) >> (v0 & 63));
    if (v0 + CU > V) bits &= (1u << (V - v0)) - 1u;
    return bits;
}

// r[0..CU] = rowptr[v0 .. v0 + CU] (entries past V are not read; their bits are clear)
__device__ __forceinline__ void load_rowptr(const uint32_t* __restrict__ rowptr, uint64_t v0, uint64_t V, uint32_t* r)
{
    if (v0 + CU <= V) {
        const uint4* p = reinterpret_cast<const uint4*>(rowptr + v0);  // v0 * 4 bytes is a multiple of 128
#pragma unroll
        for (int q = 0; q < CU / 4; ++q) {
            const uint4 x = p[q];
            r[4 * q] = x.x; r[4 * q + 1] = x.y; r[4 * q + 2] = x.z; r[4 * q + 3] = x.w;
        }
        r[CU] = rowptr[v0 + CU];
    } else {
#pragma unroll
        for (int j = 0; j <= CU; ++j) r[j] = (v0 + j <= V) ? rowptr[v0 + j] : 0u;
    }
}

__global__ void __launch_bounds__(T) k_fr_count(const unsigned long long* __restrict__ bm1,
                                                const unsigned long long* __restrict__ bm2, uint64_t V,
                                                const uint32_t* __restrict__ rowptr, uint32_t skip, const uint32_t* __restrict__ gate,
                                                uint32_t* __restrict__ part_n, uint32_t* __restrict__ part_vec)
{
    __shared__ uint32_t sa[T / 32 + 1], sb[T / 32 + 1];
    // a zero gate selects nothing (the bitmaps were not written in this phase): k_fr_scan then
    // reports an empty list without reading the partials, and k_fr_write returns at once
    if (gate && *gate == 0u) return;
    const uint64_t v0 = (uint64_t)blockIdx.x * CCHUNK + (uint64_t)threadIdx.x * CU;
    const uint32_t bits = selected_bits(bm1, bm2, v0, V);
    if (!__syncthreads_or(bits)) {
        if (threadIdx.x == 0) { part_n[blockIdx.x] = 0; part_vec[blockIdx.x] = 0; }
        return;
    }
    uint32_t n = __popc(bits), vec = 0;
    if (bits) {
        uint32_t r[CU + 1];
        load_rowptr(rowptr, v0, V, r);
#pragma unroll
        for (int j = 0; j < CU; ++j)
            if ((bits >> j) & 1u) vec += r[j + 1] - r[j] - skip;
    }
    uint32_t tn, tv;
    block_scan2(n, vec, tn, tv, sa, sb);
    if (threadIdx.x == 0) { part_n[blockIdx.x] = tn; part_vec[blockIdx.x] = tv; }
}

// one block of SCAN_T threads: exclusive scan of the per-block totals in place (each thread a
// contiguous segment); counters[0] = selected vertices, counters[2] = their vectors
constexpr int SCAN_T = 1024;

__global__ void __launch_bounds__(SCAN_T) k_fr_scan(uint32_t* __restrict__ part_n, uint32_t* __restrict__ part_vec, uint32_t nb,
                                                    uint32_t* __restrict__ counters, const uint32_t* __restrict__ gate)
{
    __shared__ uint32_t sa[SCAN_T / 32 + 1], sb[SCAN_T / 32 + 1];
    if (gate && *gate == 0u) {  // gated off: an empty list (the partials were not written)
        if (threadIdx.x == 0) { counters[0] = 0; counters[2] = 0; }
        return;
    }
    const uint32_t per = (nb + SCAN_T - 1) / SCAN_T;
    const uint32_t lo = min(nb, threadIdx.x * per), hi = min(nb, lo + per);
    uint32_t sn = 0, sv = 0;
#pragma unroll 8
    for (uint32_t i = lo; i < hi; ++i) { sn += part_n[i]; sv += part_vec[i]; }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t xa = sn, xb = sv;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t ya = __shfl_up_sync(0xffffffffu, xa, o);
        const uint32_t yb = __shfl_up_sync(0xffffffffu, xb, o);
        if (lane >= o) { xa += ya; xb += yb; }
    }
    if (lane == 31) { sa[warp] = xa; sb[warp] = xb; }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t ra = 0, rb = 0;
        for (int k = 0; k < SCAN_T / 32; ++k) {
            const uint32_t ta = sa[k], tb = sb[k];
            sa[k] = ra; sb[k] = rb;
            ra += ta; rb += tb;
        }
        counters[0] = ra;
        counters[2] = rb;
    }
    __syncthreads();
    uint32_t en = sa[warp] + xa - sn, ev = sb[warp] + xb - sv;
    for (uint32_t i = lo; i < hi; ++i) {
        const uint32_t tn = part_n[i], tv = part_vec[i];
        part_n[i] = en;
        part_vec[i] = ev;
        en += tn;
        ev += tv;
    }
}

// frontier[i] = i-th selected vertex (ID order), voff[i] = offset of its first vector among the
// selected vertices' vectors, vdelta[i] = its first vector's index in the list minus voff[i]
// (mod 2^32); tile_first[t] for the tiles that start in its range.  voff[count] = total vectors.
// `skip` leaves out the first vectors of every selected vertex (each selected one has more).
__global__ void __launch_bounds__(T) k_fr_write(const unsigned long long* __restrict__ bm1,
                                                const unsigned long long* __restrict__ bm2, uint64_t V,
                                                const uint32_t* __restrict__ rowptr, uint32_t skip, const uint32_t* __restrict__ base_n,
                                                const uint32_t* __restrict__ base_vec, const uint32_t* __restrict__ counters,
                                                uint32_t nb, uint32_t* __restrict__ frontier, uint32_t* __restrict__ voff,
                                                uint32_t* __restrict__ vdelta, uint32_t* __restrict__ tile_first,
                                                const uint32_t* __restrict__ gate)
{
    __shared__ uint32_t sa[T / 32 + 1], sb[T / 32 + 1];
    if (gate && *gate == 0u) return;  // gated off: nothing selected
    if (blockIdx.x == 0 && threadIdx.x == 0) voff[counters[0]] = counters[2];
    const uint32_t b0 = base_n[blockIdx.x];
    const uint32_t b1 = blockIdx.x + 1 < nb ? base_n[blockIdx.x + 1] : counters[0];
    if (b0 == b1) return;  // nothing selected in this block (uniform)
    const uint64_t v0 = (uint64_t)blockIdx.x * CCHUNK + (uint64_t)threadIdx.x * CU;
    const uint32_t bits = selected_bits(bm1, bm2, v0, V);
    uint32_t r[CU + 1];
    uint32_t n = __popc(bits), vec = 0;
    if (bits) {
        load_rowptr(rowptr, v0, V, r);
#pragma unroll
        for (int j = 0; j < CU; ++j)
            if ((bits >> j) & 1u) vec += r[j + 1] - r[j] - skip;
    }
    uint32_t tn, tv;
    block_scan2(n, vec, tn, tv, sa, sb);
    if (!bits) return;
    uint32_t pos = b0 + n, vo = base_vec[blockIdx.x] + vec;
#pragma unroll
    for (int j = 0; j < CU; ++j) {
        if (!((bits >> j) & 1u)) continue;
        const uint32_t cnt = r[j + 1] - r[j] - skip;
        frontier[pos] = (uint32_t)(v0 + j);
        voff[pos] = vo;
        vdelta[pos] = r[j] + skip - vo;
        for (uint64_t t = ((uint64_t)vo + PUSH_TILE - 1) / PUSH_TILE; t * PUSH_TILE < (uint64_t)vo + cnt; ++t) tile_first[t] = pos;
        ++pos;
        vo += cnt;
    }
}

// Expand the compacted frontier, one tile of PUSH_TILE vectors at a time (grid-stride over
// tiles; the totals stay on the device).  The tile's owners are staged in shared memory and
// each vector finds its owner by a binary search there.
template <bool IsBfs>
__global__ void __launch_bounds__(T) k_push_expand(const uint32_t* __restrict__ frontier, const uint32_t* __restrict__ voff,
                                                   const uint32_t* __restrict__ vdelta, const uint32_t* __restrict__ tile_first,
                                                   const uint32_t* __restrict__ counters, const uint4* __restrict__ nbr,
                                                   uint32_t V, uint32_t* __restrict__ label,
                                                   unsigned long long* __restrict__ has_next, const unsigned long long* __restrict__ wants,
                                                   uint32_t* __restrict__ cand32, uint32_t* __restrict__ touched,
                                                   uint32_t* __restrict__ ntouched, VoteCfg vc, unsigned long long* __restrict__ vote,
                                                   unsigned long long* __restrict__ chg, uint32_t epoch,
                                                   const uint32_t* __restrict__ epoch_dev)
{
    __shared__ uint32_t s_src[PUSH_TILE + 1];
    __shared__ uint32_t red32[T / 32];
    uint32_t my_min = INF;  // CC: the smallest label written (cc_prev_min of the next iteration)
    __shared__ uint32_t s_off[PUSH_TILE + 1];
    __shared__ uint32_t s_delta[PUSH_TILE + 1];
    __shared__ unsigned long long red[T / 32];
    __shared__ bool s_full;  // BFS: the touched list is long enough for the visit to sweep (read per tile)
    const uint32_t nf = counters[0], total = counters[2];
    const uint32_t ntiles = (total + PUSH_TILE - 1) / PUSH_TILE;
    unsigned long long my_vote = 0;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint32_t first = tile_first[tile];
        const uint32_t t0 = tile * PUSH_TILE;
        const uint32_t tend = min(total, t0 + PUSH_TILE);
        // entries first .. first+nw-1 own every vector of the tile (each owns at least one)
        const uint32_t nw = min(PUSH_TILE, nf - first);
        for (uint32_t i = threadIdx.x; i <= nw; i += T) {
            s_off[i] = voff[first + i];
            if (i < nw) {
                s_src[i] = frontier[first + i];
                s_delta[i] = vdelta[first + i];
            }
        }
        if (IsBfs && threadIdx.x == 0) s_full = touched_full(ntouched, V);
        __syncthreads();
        for (uint32_t base = t0; base < tend; base += T) {  // warp-uniform trip count
            const uint32_t gv = base + threadIdx.x;
            const bool live = gv < tend;
            uint32_t u = 0;
            uint4 s = make_uint4(INF, INF, INF, INF);
            if (live) {
                int lo = 0, hi = (int)nw - 1;  // last entry with s_off <= gv
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s_off[mid] <= gv) lo = mid; else hi = mid - 1;
                }
                u = s_src[lo];
                s = __ldcs(nbr + (uint32_t)(gv + s_delta[lo]));
            }
            const uint32_t ids[4] = { s.x, s.y, s.z, s.w };
            if (IsBfs) {
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    const uint32_t d = ids[l];
                    bool first_touch = false;
                    if (d < V && bit_of(wants, d) && u < cand32[d]) {
                        first_touch = atomicMin(cand32 + d, u) == INF;
                        if (first_touch) atomicOr(has_next + (d >> 6), 1ull << (d & 63));
                    }
                    touched_append(first_touch, d, touched, ntouched, s_full);
                }
            } else if (live) {
                const uint32_t msg = label[u];
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    const uint32_t d = ids[l];
                    if (d < V && msg < label[d]) {
                        const uint32_t old = atomicMin(label + d, msg);
                        if (msg < old) {
                            my_min = min(my_min, msg);
                            if (bit_set_first(has_next, d)) my_vote += vc.of(d);
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
    if (!IsBfs) {
        my_vote = block_sum_u64(my_vote, red);
        if (threadIdx.x == 0) vote_add(vote, my_vote);
        cc_record_min<T>(my_min, red32, chg, epoch_dev ? *epoch_dev : epoch);
    }
}

// BFS pull over the compacted wanted destinations (WantsInfo and in-vectors): only their vectors
// are read, in tiles of PUSH_TILE vectors.  The vectors of one destination are consecutive in the
// concatenation, so the per-destination minimum candidate (the reference's parent rule, as in
// k_bfs_pull) is reduced within the warp before one atomicMin.
// Early exit: the candidate is (first vector with a frontier source, ~largest such source), so
// once a destination has a candidate, its later vectors cannot win.  Blocks take runs of
// PULL_CHUNK consecutive tiles from a queue (balanced, and a long destination's tiles are
// processed roughly in order), and a vector past its destination's first LONG_RUN vectors is
// skipped (no neighbour or frontier reads) when the candidate already names an earlier vector.
// In R-MAT the sources of a destination ascend and the hubs have small IDs, so a long
// destination next to a frontier hub stops after its first vectors.
constexpr uint32_t PULL_CHUNK = 2;  // GB300 sweep of 2-16 (queue of runs): 2 keeps small pulls cheapest
constexpr uint32_t LONG_RUN = 32;

__global__ void __launch_bounds__(T) k_bfs_pull_expand(const uint32_t* __restrict__ dests, const uint32_t* __restrict__ voff,
                                                       const uint32_t* __restrict__ vdelta, const uint32_t* __restrict__ tile_first,
                                                       const uint32_t* __restrict__ counters, const uint4* __restrict__ nbr,
                                                       uint32_t V, const unsigned long long* __restrict__ has,
                                                       unsigned long long* __restrict__ cand, uint32_t* __restrict__ touched,
                                                       uint32_t* __restrict__ ntouched, const uint32_t* __restrict__ hub_vid,
                                                       uint32_t nhub, unsigned long long* __restrict__ has_next,
                                                       uint32_t* __restrict__ queue)
{
    __shared__ uint32_t s_dst[PUSH_TILE + 1];
    __shared__ uint32_t s_off[PUSH_TILE + 1];
    __shared__ uint32_t s_delta[PUSH_TILE + 1];
    __shared__ uint32_t s_chunk;
    __shared__ bool s_full;  // the touched list is long enough for the visit to sweep (read per tile)
    const uint32_t nd = counters[0], total = counters[2];
    const uint32_t ntiles = (total + PUSH_TILE - 1) / PUSH_TILE;
    const int lane = threadIdx.x & 31;
    for (;;) {
        if (threadIdx.x == 0) s_chunk = atomicAdd(queue, 1u);
        __syncthreads();
        const uint32_t chunk = s_chunk;
        __syncthreads();  // every thread has read s_chunk before it is replaced
        if ((uint64_t)chunk * PULL_CHUNK >= ntiles) break;
        const uint32_t chunk_end = min(ntiles, (chunk + 1) * PULL_CHUNK);
        for (uint32_t tile = chunk * PULL_CHUNK; tile < chunk_end; ++tile) {
            const uint32_t first = tile_first[tile];
            const uint32_t t0 = tile * PUSH_TILE;
            const uint32_t tend = min(total, t0 + PUSH_TILE);
            const uint32_t nw = min(PUSH_TILE, nd - first);
            for (uint32_t i = threadIdx.x; i <= nw; i += T) {
                s_off[i] = voff[first + i];
                if (i < nw) {
                    s_dst[i] = dests[first + i];
                    s_delta[i] = vdelta[first + i];
                }
            }
            if (threadIdx.x == 0) s_full = touched_full(ntouched, V);
            __syncthreads();
            for (uint32_t base = t0; base < tend; base += T) {  // warp-uniform trip count
                const uint32_t gv = base + threadIdx.x;
                uint32_t key = INF;
                unsigned long long k = ~0ull;
                if (gv < tend) {
                    int lo = 0, hi = (int)nw - 1;  // last entry with s_off <= gv
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (s_off[mid] <= gv) lo = mid; else hi = mid - 1;
                    }
                    key = s_dst[lo];
                    const uint32_t vec = gv + s_delta[lo];
                    bool skip = false;
                    if (gv >= s_off[lo] + LONG_RUN) {
                        const unsigned long long c = __ldcg(cand + key);  // atomics of other blocks land in L2
                        skip = c != ~0ull && (uint32_t)(c >> 32) < vec;
                    }
                    if (!skip) {
                        const uint4 s = __ldcs(nbr + vec);
                        const uint32_t ids[4] = { grz_hub_decode(s.x, hub_vid, nhub), grz_hub_decode(s.y, hub_vid, nhub),
                                                  grz_hub_decode(s.z, hub_vid, nhub), grz_hub_decode(s.w, hub_vid, nhub) };
                        uint32_t best = 0;
                        bool any = false;
    #pragma unroll
                        for (int l = 0; l < 4; ++l) {
                            const uint32_t id = ids[l];
                            if (id < V && bit_of(has, id)) {
                                best = any ? max(best, id) : id;
                                any = true;
                            }
                        }
                        if (any) k = ((unsigned long long)vec << 32) | (unsigned long long)(~best);
                    }
                }
                if (!__any_sync(0xffffffffu, k != ~0ull)) continue;  // no frontier source in the warp's vectors
                const uint32_t prevkey = __shfl_up_sync(0xffffffffu, key, 1);
                const uint32_t nextkey = __shfl_down_sync(0xffffffffu, key, 1);
                const bool head = lane == 0 || key != prevkey;
                const bool tail = lane == 31 || key != nextkey;
                const unsigned heads = __ballot_sync(0xffffffffu, head);
                const int segstart = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
                const int maxlen = __reduce_max_sync(0xffffffffu, (unsigned)(lane - segstart + 1));
                for (int off = 1; off < maxlen; off <<= 1) {
                    const unsigned long long o = __shfl_up_sync(0xffffffffu, k, off);
                    if (lane - off >= segstart) k = min(k, o);
                }
                bool first_touch = false;
                if (tail && k != ~0ull && k < cand[key]) {
                    first_touch = atomicMin(cand + key, k) == ~0ull;
                    if (first_touch) atomicOr(has_next + (key >> 6), 1ull << (key & 63));
                }
                touched_append(first_touch, key, touched, ntouched, s_full);
            }
            __syncthreads();
        }
    }
}

// CC pull over the remaining vectors of the destinations k_cc_pull_first left open (label above 0
// after their first vector), compacted with their vector ranges as the BFS pull's are (the same
// tiles, queue and binary search as k_bfs_pull_expand).  A vector whose destination reached 0
// meanwhile needs no gathers; the others take the minimum of their lanes' labels (lane 0 first),
// reduced per destination within the warp, and the run's last lane lowers the label in place.
__global__ void __launch_bounds__(T) k_cc_pull_expand(const uint32_t* __restrict__ dests, const uint32_t* __restrict__ voff,
                                                      const uint32_t* __restrict__ vdelta, const uint32_t* __restrict__ tile_first,
                                                      const uint32_t* __restrict__ counters, const uint4* __restrict__ nbr,
                                                      uint32_t V, uint32_t* __restrict__ label, const uint32_t* __restrict__ hub_vid,
                                                      uint32_t nhub, unsigned long long* __restrict__ has_next, VoteCfg vc,
                                                      unsigned long long* __restrict__ vote, unsigned long long* __restrict__ chg,
                                                      uint32_t epoch, const uint32_t* __restrict__ epoch_dev,
                                                      uint32_t* __restrict__ queue, unsigned long long* __restrict__ work)
{
    __shared__ uint32_t s_dst[PUSH_TILE + 1];
    __shared__ uint32_t s_off[PUSH_TILE + 1];
    __shared__ uint32_t s_delta[PUSH_TILE + 1];
    __shared__ uint32_t s_chunk;
    __shared__ unsigned long long red[T / 32];
    __shared__ uint32_t red32[T / 32];
    const uint32_t ep = epoch_dev ? *epoch_dev : epoch;
    const uint32_t nd = counters[0], total = counters[2];
    const uint32_t ntiles = (total + PUSH_TILE - 1) / PUSH_TILE;
    const int lane = threadIdx.x & 31;
    unsigned long long my_vote = 0, my_vecs = 0;
    uint32_t my_min = INF;
    auto fetch = [&](uint32_t xl) -> uint32_t {
        const uint32_t sl = xl - GRZ_HUB_BASE;
        const uint32_t id = sl < nhub ? __ldg(hub_vid + sl) : min(xl, V);
        return ld_label(label + id);
    };
    for (;;) {
        if (threadIdx.x == 0) s_chunk = atomicAdd(queue, 1u);
        __syncthreads();
        const uint32_t chunk = s_chunk;
        __syncthreads();  // every thread has read s_chunk before it is replaced
        if ((uint64_t)chunk * PULL_CHUNK >= ntiles) break;
        const uint32_t chunk_end = min(ntiles, (chunk + 1) * PULL_CHUNK);
        for (uint32_t tile = chunk * PULL_CHUNK; tile < chunk_end; ++tile) {
            const uint32_t first = tile_first[tile];
            const uint32_t t0 = tile * PUSH_TILE;
            const uint32_t tend = min(total, t0 + PUSH_TILE);
            const uint32_t nw = min(PUSH_TILE, nd - first);
            for (uint32_t i = threadIdx.x; i <= nw; i += T) {
                s_off[i] = voff[first + i];
                if (i < nw) {
                    s_dst[i] = dests[first + i];
                    s_delta[i] = vdelta[first + i];
                }
            }
            __syncthreads();
            for (uint32_t base = t0; base < tend; base += T) {  // warp-uniform trip count
                const uint32_t gv = base + threadIdx.x;
                uint32_t key = INF, m = INF;
                if (gv < tend) {
                    int lo = 0, hi = (int)nw - 1;  // last entry with s_off <= gv
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (s_off[mid] <= gv) lo = mid; else hi = mid - 1;
                    }
                    key = s_dst[lo];
                    if (ld_label(label + key) != 0) {
                        ++my_vecs;
                        const uint4 sv = ld_stream(nbr + (uint32_t)(gv + s_delta[lo]));
                        m = fetch(sv.x);
                        if (m != 0) m = min(m, min(min(fetch(sv.y), fetch(sv.z)), fetch(sv.w)));
                    }
                }
                if (!__any_sync(0xffffffffu, m != INF)) continue;
                const uint32_t prevkey = __shfl_up_sync(0xffffffffu, key, 1);
                const uint32_t nextkey = __shfl_down_sync(0xffffffffu, key, 1);
                const bool head = lane == 0 || key != prevkey;
                const bool tail = lane == 31 || key != nextkey;
                const unsigned heads = __ballot_sync(0xffffffffu, head);
                const int segstart = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
                const int maxlen = __reduce_max_sync(0xffffffffu, (unsigned)(lane - segstart + 1));
                for (int off = 1; off < maxlen; off <<= 1) {
                    const uint32_t o = __shfl_up_sync(0xffffffffu, m, off);
                    if (lane - off >= segstart) m = min(m, o);
                }
                if (tail && m != INF && m < ld_label(label + key)) {
                    const uint32_t old = atomicMin(label + key, m);
                    if (m < old) {
                        my_min = min(my_min, m);
                        if (bit_set_first(has_next, key)) my_vote += vc.of(key);
                    }
                }
            }
            __syncthreads();
        }
    }
    my_vote = block_sum_u64(my_vote, red);
    if (threadIdx.x == 0) vote_add(vote, my_vote);
    __syncthreads();
    if (work) {  // profiling: vectors read, by kind of iteration
        uint32_t mp = 0;
        const int slot = cc_prev_min(chg, ep, &mp) ? 1 : 0;
        my_vecs = block_sum_u64(my_vecs, red);
        if (threadIdx.x == 0 && my_vecs) atomicAdd(work + slot, my_vecs);
        __syncthreads();
    }
    cc_record_min<T>(my_min, red32, chg, ep);
}

// BFS pull, early-exit pass.  Every in-neighbour of a wanted (unvisited) destination that has been
// visited is in the frontier (it was visited in the previous iteration, else it would have
// visited the destination already), so in the big pull iterations most wanted destinations find
// a frontier source in their first vector.  Each wanted destination reads its first `first_n`
// vectors in order and stops at the first one with a frontier source; that vector's largest
// frontier source is its parent, which is the full scan's rule (smallest vector index, then
// largest source) because no earlier vector has one.  A destination decided here is visited here
// (parent, level, WantsInfo cleared, HasInfo* set, vote), so it needs no candidate word and no
// place in the touched list, whose single counter would serialise millions of appends.  One
// still undecided that has more vectors is marked in `unres`, and the tiled pass
// (k_bfs_pull_expand, then k_bfs_visit) reads the rest of its vectors.  A warp owns FW whole
// bitmap words (64 destinations each; lane l of slot q holds destination 64 w0 + 32 q + l), so
// it writes their WantsInfo, HasInfo* and unres words without atomics, and the first-vector
// loads of its 2 FW slots are issued together.

__global__ void __launch_bounds__(T, GRZ_BFS_MINB) k_bfs_pull_first(unsigned long long* __restrict__ wants,
                                                      const unsigned long long* __restrict__ nonempty,
                                                      const uint32_t* __restrict__ rowptr, const uint4* __restrict__ nbr,
                                                      uint32_t V, uint64_t W, const unsigned long long* __restrict__ has,
                                                      const uint32_t* __restrict__ hub_vid, uint32_t nhub,
                                                      unsigned long long* __restrict__ has_next,
                                                      unsigned long long* __restrict__ unres, uint32_t first_n,
                                                      uint32_t* __restrict__ parent, uint32_t* __restrict__ level,
                                                      uint32_t iter_host, const uint32_t* __restrict__ iter_dev, VoteCfg vc,
                                                      unsigned long long* __restrict__ vote)
{
    __shared__ unsigned long long red[T / 32];
    constexpr int Q = 2 * FW;
    const int lane = threadIdx.x & 31;
    const uint32_t iter = iter_dev ? *iter_dev : iter_host;
    unsigned long long my_vote = 0;
    // the largest frontier source of vector `vec`, or INF without one
    auto vec_best = [&](uint32_t vec) -> uint32_t {
        const uint4 s = __ldcs(nbr + vec);
        const uint32_t ids[4] = { grz_hub_decode(s.x, hub_vid, nhub), grz_hub_decode(s.y, hub_vid, nhub),
                                  grz_hub_decode(s.z, hub_vid, nhub), grz_hub_decode(s.w, hub_vid, nhub) };
        bool in[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) in[l] = ids[l] < V && bit_of(has, ids[l]);
        // lanes ascend by source: the largest frontier source is the last lane with one
        return in[3] ? ids[3] : in[2] ? ids[2] : in[1] ? ids[1] : in[0] ? ids[0] : INF;
    };
    const uint64_t nwarps = (uint64_t)gridDim.x * (T / 32);
    for (uint64_t w0 = ((uint64_t)blockIdx.x * (T / 32) + (threadIdx.x >> 5)) * FW; w0 < W; w0 += nwarps * FW) {  // warp-uniform
        unsigned long long sel[FW];
#pragma unroll
        for (int f = 0; f < FW; ++f) sel[f] = w0 + f < W ? wants[w0 + f] & nonempty[w0 + f] : 0ull;
        uint32_t r0[Q], n[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const uint64_t v = 64 * w0 + 32 * (uint64_t)q + lane;
            n[q] = 0;
            if (v < V && ((sel[q >> 1] >> (32 * (q & 1) + lane)) & 1ull)) {
                r0[q] = rowptr[v];
                n[q] = rowptr[v + 1] - r0[q];
            }
        }
        uint32_t p[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) p[q] = n[q] ? vec_best(r0[q]) : INF;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const uint32_t m = min(n[q], first_n);
            for (uint32_t j = 1; j < m && p[q] == INF; ++j) p[q] = vec_best(r0[q] + j);
        }
        unsigned long long un[FW], hn[FW];
#pragma unroll
        for (int f = 0; f < FW; ++f) un[f] = hn[f] = 0ull;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const uint32_t v = (uint32_t)(64 * w0 + 32 * (uint64_t)q + lane);
            const bool hit = p[q] != INF;
            if (hit) {
                parent[v] = p[q];
                level[v] = iter;
                my_vote += vc.of(v);
            }
            const unsigned mh = __ballot_sync(0xffffffffu, hit);
            const unsigned mu = __ballot_sync(0xffffffffu, !hit && n[q] > first_n);
            hn[q >> 1] |= (unsigned long long)mh << (32 * (q & 1));
            un[q >> 1] |= (unsigned long long)mu << (32 * (q & 1));
        }
        if (lane == 0) {
#pragma unroll
            for (int f = 0; f < FW; ++f) {
                if (w0 + f >= W) break;
                unres[w0 + f] = un[f];
                if (hn[f]) {
                    has_next[w0 + f] |= hn[f];
                    wants[w0 + f] &= ~hn[f];
                }
            }
        }
    }
    my_vote = block_sum_u64(my_vote, red);
    if (threadIdx.x == 0) vote_add(vote, my_vote);
}

// BFS: visit the touched destinations (pull: decode the winning (vector, source) key; push: the
// smallest source), in one pass over the touched list
template <bool FromPull>
__global__ void __launch_bounds__(T) k_bfs_visit(const uint32_t* __restrict__ touched, const uint32_t* __restrict__ ntouched,
                                                 unsigned long long* __restrict__ cand64, uint32_t* __restrict__ cand32,
                                                 uint32_t* __restrict__ parent, uint32_t* __restrict__ level, uint32_t iter_host,
                                                 const uint32_t* __restrict__ iter_dev,
                                                 unsigned long long* __restrict__ wants, const unsigned long long* __restrict__ has_next,
                                                 VoteCfg vc, unsigned long long* __restrict__ vote, uint32_t V)
{
    __shared__ unsigned long long red[T / 32];
    const uint32_t n = *ntouched;
    const uint32_t iter = iter_dev ? *iter_dev : iter_host;
    unsigned long long my_vote = 0;
    auto visit = [&](uint32_t d) {
        uint32_t p;
        if (FromPull) {
            p = ~(uint32_t)(cand64[d] & 0xffffffffull);
            cand64[d] = ~0ull;
        } else {
            p = cand32[d];
            cand32[d] = INF;
        }
        parent[d] = p;
        level[d] = iter;
        my_vote += vc.of(d);
    };
    if ((uint64_t)n * VISIT_DENSE_RATIO <= V) {
        // few: the touched list (first-touch order)
        for (uint32_t i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) {
            const uint32_t d = touched[i];
            visit(d);
            atomicAnd(wants + (d >> 6), ~(1ull << (d & 63)));
        }
    } else {
        // many: every vertex, in ID order, 4 per thread per step with the loads of the 4 issued
        // together (coalesced, no per-thread dependence chains).  A vertex was touched in this
        // call when its HasInfo* bit is set (at first touch) and its WantsInfo bit still is (a
        // caller's earlier vector range of this iteration visited and cleared its own).  Each
        // vertex is read and written by one thread only, so cand and degree go through the
        // read-only path.
        constexpr int U = 4;
        const uint32_t lane = threadIdx.x & 31;
        for (uint64_t base = (uint64_t)blockIdx.x * T * U; base < V; base += (uint64_t)gridDim.x * T * U) {  // warp-uniform
            uint32_t d[U];
            bool hit[U];
#pragma unroll
            for (int j = 0; j < U; ++j) {
                d[j] = (uint32_t)(base + (uint64_t)j * T + threadIdx.x);
                hit[j] = d[j] < V && (((has_next[d[j] >> 6] & wants[d[j] >> 6]) >> (d[j] & 63)) & 1ull);
            }
            uint32_t p[U], deg[U];
#pragma unroll
            for (int j = 0; j < U; ++j) {
                if (hit[j]) {
                    p[j] = FromPull ? ~(uint32_t)(__ldg(cand64 + d[j]) & 0xffffffffull) : __ldg(cand32 + d[j]);
                    deg[j] = __ldg(vc.degree + d[j]);
                }
            }
#pragma unroll
            for (int j = 0; j < U; ++j) {
                if (hit[j]) {
                    if (FromPull) cand64[d[j]] = ~0ull; else cand32[d[j]] = INF;
                    parent[d[j]] = p[j];
                    level[d[j]] = iter;
                    my_vote += (vc.without_count ? 0ull : 1ull) + (vc.without_outdeg ? 0ull : (unsigned long long)deg[j]);
                }
                // the warp's 32 vertices lie in one 64-bit word: one atomicAnd clears their WantsInfo bits
                const unsigned m = __ballot_sync(0xffffffffu, hit[j]);
                if (m && lane == (uint32_t)(__ffs(m) - 1)) {
                    const uint32_t d0 = d[j] - lane;
                    atomicAnd(wants + (d0 >> 6), ~((unsigned long long)m << (d0 & 63)));
                }
            }
        }
    }
    my_vote = block_sum_u64(my_vote, red);
    if (threadIdx.x == 0) vote_add(vote, my_vote);
}

// ---------------------------------------------------------------------------------------------
// init / output

// execution_initialize_vertex_prop_cc: (double)id; entry V = +inf.  Four labels per thread with one
// 16-byte store (the array is 256-byte aligned), the last few one by one.
__global__ void k_cc_init(uint32_t* __restrict__ label, uint64_t V)
{
    const uint64_t q = (uint64_t)blockIdx.x * T + threadIdx.x;
    const uint64_t v = 4 * q;
    if (v + 3 < V) {
        reinterpret_cast<uint4*>(label)[q] = make_uint4((uint32_t)v, (uint32_t)v + 1, (uint32_t)v + 2, (uint32_t)v + 3);
    } else {
        for (uint64_t k = v; k <= V && k < v + 4; ++k) label[k] = k < V ? (uint32_t)k : INF;
    }
}

// parent and level of entries [0, V] = INF: four of each per thread with 16-byte stores (the arrays
// are 256-byte aligned), the last few one by one
__global__ void k_bfs_init(uint32_t* __restrict__ parent, uint32_t* __restrict__ level, uint64_t V)
{
    const uint64_t q = (uint64_t)blockIdx.x * T + threadIdx.x;
    const uint64_t v = 4 * q;
    const uint4 inf4 = make_uint4(INF, INF, INF, INF);
    if (v + 3 <= V) {
        reinterpret_cast<uint4*>(parent)[q] = inf4;
        reinterpret_cast<uint4*>(level)[q] = inf4;
    } else {
        for (uint64_t u = v; u <= V; ++u) { parent[u] = INF; level[u] = INF; }
    }
}

// bitmaps: `all_ones` sets bits [0, V); bits at and beyond V stay clear
__global__ void k_bitmap_init(unsigned long long* __restrict__ bm, uint64_t words, uint64_t V, int all_ones)
{
    const uint64_t w = (uint64_t)blockIdx.x * T + threadIdx.x;
    if (w >= words) return;
    unsigned long long x = 0;
    if (all_ones) {
        const uint64_t lo = w * 64;
        if (lo + 64 <= V) x = ~0ull;
        else if (lo < V) x = (1ull << (V - lo)) - 1ull;
    }
    bm[w] = x;
}

// bitmap of vertices that own at least one vector in a list: a thread per vertex, a warp per
// 32-bit half of a bitmap word (the words are little-endian), all `words` words written
__global__ void k_nonempty(const uint32_t* __restrict__ rowptr, uint64_t V, unsigned long long* __restrict__ bm, uint64_t words)
{
    const uint64_t v = (uint64_t)blockIdx.x * T + threadIdx.x;
    const bool in = v < 64 * words;  // uniform per warp: 64 words is a multiple of 32
    const bool bit = in && v < V && rowptr[v + 1] > rowptr[v];
    const unsigned m = __ballot_sync(0xffffffffu, bit);
    if (in && (threadIdx.x & 31) == 0) reinterpret_cast<uint32_t*>(bm)[v >> 5] = m;
}

// reference-format output: CC labels as double; BFS parents as double with -1 for unvisited
// vertices and the root (source/execution_bfs.c:113-116)
__global__ void k_u32_to_double(const uint32_t* __restrict__ x, uint64_t V, double* __restrict__ out, int bfs)
{
    const uint64_t v = (uint64_t)blockIdx.x * T + threadIdx.x;
    if (v >= V) return;
    const uint32_t a = x[v];
    out[v] = (bfs && a == INF) ? -1.0 : (double)a;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// host side

static uint64_t words_of(uint64_t V) { return (V >> 6) + 2; }
static int frontier_list_state(grz_graph* g);

static int ensure_frontier_state(grz_graph* g)
{
    grz_frontier_state& f = g->fr;
    if (f.label && !f.lists_changed) return GRZ_OK;
    const uint64_t V = g->V, W = words_of(V);
    const uint64_t tiles = std::max(g->push.nvec, g->pull.nvec) / PUSH_TILE + 2;
    if (f.label) {
        // kept from the graph loaded before, which had the same V
        if (f.alloc_V != V) return grz_set_error(g, GRZ_ERR_STATE, "frontier buffers sized for another graph");
        if (tiles > f.tile_cap) {
            GRZ_CK(g, cudaFree(f.tile_first));
            f.tile_first = nullptr;
            GRZ_CK(g, cudaMalloc((void**)&f.tile_first, sizeof(uint32_t) * tiles));
            f.tile_cap = tiles;
        }
        f.lists_changed = 0;
        return frontier_list_state(g);
    }
    f.alloc_V = V;
    f.tile_cap = tiles;
    GRZ_CK(g, cudaMalloc((void**)&f.label, sizeof(uint32_t) * (V + 1)));
    GRZ_CK(g, cudaMalloc((void**)&f.level, sizeof(uint32_t) * (V + 1)));
    GRZ_CK(g, cudaMalloc((void**)&f.has, sizeof(unsigned long long) * W));
    GRZ_CK(g, cudaMalloc((void**)&f.has_next, sizeof(unsigned long long) * W));
    GRZ_CK(g, cudaMalloc((void**)&f.wants, sizeof(unsigned long long) * W));
    GRZ_CK(g, cudaMalloc((void**)&f.nonempty_push, sizeof(unsigned long long) * W));
    GRZ_CK(g, cudaMalloc((void**)&f.frontier, sizeof(uint32_t) * (V + 1)));
    GRZ_CK(g, cudaMalloc((void**)&f.voff, sizeof(uint32_t) * (V + 1)));
    GRZ_CK(g, cudaMalloc((void**)&f.vdelta, sizeof(uint32_t) * (V + 1)));
    GRZ_CK(g, cudaMalloc((void**)&f.tile_first, sizeof(uint32_t) * tiles));
    GRZ_CK(g, cudaMalloc((void**)&f.fr_part, sizeof(uint32_t) * 2 * (V / CCHUNK + 1)));
    GRZ_CK(g, cudaMalloc((void**)&f.nonempty_pull, sizeof(unsigned long long) * W));
    GRZ_CK(g, cudaMalloc((void**)&f.unres, sizeof(unsigned long long) * W));
    GRZ_CK(g, cudaMalloc((void**)&f.touched, sizeof(uint32_t) * (V + 1)));
    GRZ_CK(g, cudaMalloc((void**)&f.cand64, sizeof(unsigned long long) * (V + 1)));
    GRZ_CK(g, cudaMalloc((void**)&f.cand32, sizeof(uint32_t) * (V + 1)));
    GRZ_CK(g, cudaMalloc((void**)&f.counters, sizeof(uint32_t) * 8));
    GRZ_CK(g, cudaMalloc((void**)&f.vote, sizeof(unsigned long long) * GRZ_VOTE_SLOTS * GRZ_VOTE_STRIDE));
    GRZ_CK(g, cudaMalloc((void**)&f.chg, sizeof(unsigned long long) * 2));
    GRZ_CK(g, cudaMalloc((void**)&f.dev_err, sizeof(unsigned)));
    return frontier_list_state(g);
}

// the state that depends on the loaded lists, and the scratch values the kernels expect
static int frontier_list_state(grz_graph* g)
{
    const uint64_t V = g->V, W = words_of(V);
    grz_frontier_state& f = g->fr;
    GRZ_CK(g, cudaMemsetAsync(f.vote, 0, sizeof(unsigned long long) * GRZ_VOTE_SLOTS * GRZ_VOTE_STRIDE, g->stream));
    GRZ_CK(g, cudaMemsetAsync(f.cand64, 0xff, sizeof(unsigned long long) * (V + 1), g->stream));
    GRZ_CK(g, cudaMemsetAsync(f.cand32, 0xff, sizeof(uint32_t) * (V + 1), g->stream));
    GRZ_CK(g, cudaMemsetAsync(f.nonempty_push, 0, sizeof(unsigned long long) * W, g->stream));
    GRZ_CK(g, cudaMemsetAsync(f.nonempty_pull, 0, sizeof(unsigned long long) * W, g->stream));
    if (g->pull.rowptr && V) {
        k_nonempty<<<blocks_for(64 * W), T, 0, g->stream>>>(g->pull.rowptr, V, f.nonempty_pull, W); GRZ_COUNT_LAUNCH(g);
        GRZ_CK(g, cudaGetLastError());
    }
    if (g->push.rowptr && V) {
        k_nonempty<<<blocks_for(64 * W), T, 0, g->stream>>>(g->push.rowptr, V, f.nonempty_push, W); GRZ_COUNT_LAUNCH(g);
        GRZ_CK(g, cudaGetLastError());
    }
    return GRZ_OK;
}

static VoteCfg vote_cfg(const grz_graph* g)
{
    VoteCfg vc;
    vc.degree = g->degree;
    vc.without_count = (g->fr.flags & GRZ_FLAG_WITHOUT_COUNT) ? 1 : 0;
    vc.without_outdeg = (g->fr.flags & GRZ_FLAG_WITHOUT_OUTDEG) ? 1 : 0;
    return vc;
}

int grz_frontier_init(grz_graph* g, int app, int flags, uint32_t root)
{
    if (!g->outdeg) return grz_set_error(g, GRZ_ERR_STATE, "no graph loaded");
    int rc = ensure_frontier_state(g);
    if (rc) return rc;
    if (app == GRZ_APP_CONNECTED_COMPONENTS && g->tune.cc_segments == 2) {
        rc = grz_pr_ensure_segments(g, 1);
        if (rc) return rc;
    }
    const uint64_t V = g->V, W = words_of(V);
    grz_frontier_state& f = g->fr;
    f.app = app;
    f.flags = flags;
    f.root = root;
    f.iter = 0;
    f.npull = f.npush = 0;
    f.last_engine = 1;
    f.next_pull = 1;
    f.cc_partial = 0;
    cudaStream_t st = g->stream;
    GRZ_CK(g, cudaMemsetAsync(f.dev_err, 0, sizeof(unsigned), st));
    if (app == GRZ_APP_CONNECTED_COMPONENTS) {
        k_cc_init<<<blocks_for(V / 4 + 1), T, 0, st>>>(f.label, V); GRZ_COUNT_LAUNCH(g);
        k_bitmap_init<<<blocks_for(W), T, 0, st>>>(f.has, W, V, 1); GRZ_COUNT_LAUNCH(g);      // HasInfo = all (execution_cc.c:66-73)
        k_bitmap_init<<<blocks_for(W), T, 0, st>>>(f.wants, W, V, 1); GRZ_COUNT_LAUNCH(g);
        // before iteration 1 every vertex counts as changed, the smallest label being 0 (tag 0)
        const unsigned long long chg0[2] = { 0x00000000ffffffffull, 0ull };
        memcpy(f.mail_chg, chg0, sizeof(chg0));
        GRZ_CK(g, cudaMemcpyAsync(f.chg, f.mail_chg, sizeof(chg0), cudaMemcpyHostToDevice, st));
        f.vote_host = 0;
        if (!(flags & GRZ_FLAG_WITHOUT_OUTDEG)) f.vote_host += g->E;     // execution_cc.c:106-112
        if (!(flags & GRZ_FLAG_WITHOUT_COUNT)) f.vote_host += V;
    } else {
        if (root >= V) return grz_set_error(g, GRZ_ERR_ARG, "root %u >= V", root);
        k_bfs_init<<<blocks_for((V + 1) / 4 + 1), T, 0, st>>>(f.label, f.level, V); GRZ_COUNT_LAUNCH(g);
        k_bitmap_init<<<blocks_for(W), T, 0, st>>>(f.has, W, V, 0); GRZ_COUNT_LAUNCH(g);
        k_bitmap_init<<<blocks_for(W), T, 0, st>>>(f.wants, W, V, 1); GRZ_COUNT_LAUNCH(g);
        const unsigned long long rbit = 1ull << (root & 63);
        unsigned long long w0 = 0, w1 = 0;
        GRZ_CK(g, cudaMemcpyAsync(&w1, f.wants + (root >> 6), 8, cudaMemcpyDeviceToHost, st));
        GRZ_CK(g, cudaStreamSynchronize(st));
        w0 = rbit;
        w1 &= ~rbit;
        GRZ_CK(g, cudaMemcpyAsync(f.has + (root >> 6), &w0, 8, cudaMemcpyHostToDevice, st));
        GRZ_CK(g, cudaMemcpyAsync(f.wants + (root >> 6), &w1, 8, cudaMemcpyHostToDevice, st));
        const uint32_t zero = 0;
        GRZ_CK(g, cudaMemcpyAsync(f.level + root, &zero, 4, cudaMemcpyHostToDevice, st));
        double od = 0;
        GRZ_CK(g, cudaMemcpyAsync(&od, g->outdeg + root, 8, cudaMemcpyDeviceToHost, st));
        GRZ_CK(g, cudaStreamSynchronize(st));
        f.vote_host = 0;
        if (!(flags & GRZ_FLAG_WITHOUT_OUTDEG)) f.vote_host += (uint64_t)od;  // execution_bfs.c:132-137
        if (!(flags & GRZ_FLAG_WITHOUT_COUNT)) f.vote_host += 1;
    }
    GRZ_CK(g, cudaMemsetAsync(f.has_next, 0, sizeof(unsigned long long) * W, st));
    GRZ_CK(g, cudaGetLastError());
    return GRZ_OK;
}

// the reference's threshold engine choice (execution_bfs.c:146-168, execution_cc.c:120-142)
int grz_engine_threshold(const grz_graph* g, uint64_t vote)
{
    const int flags = g->fr.flags;
    if (flags & GRZ_FLAG_FORCE_PULL) return 1;
    if (flags & GRZ_FLAG_FORCE_PUSH) return 0;
    const uint64_t thr = (flags & GRZ_FLAG_WITHOUT_OUTDEG) ? g->V / 2 : g->E / 5;
    return vote > thr ? 1 : 0;
}

// BFS visit grid: full occupancy (8 blocks of 256 per SM), fewer for small graphs
static unsigned visit_grid(const grz_graph* g)
{
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(blocks_for((g->V + 3) / 4), (uint64_t)g->num_sms * 8));
}

// Whether the CC pull's full pass reads the source-segmented lists (built by grz_pr_init, or by
// grz_frontier_init under GRZ_TUNE_CC_SEGMENTS = 2); they need a pull list without hub encoding.
static bool cc_use_segments(const grz_graph* g)
{
    return g->tune.cc_segments != 1 && g->seg_nbr && g->nseg && g->pull.nhub == 0 && !g->tune.cc_pull_first;
}

// kernels one segmented CC pull launches per source segment (the empty segments are skipped)
static uint64_t cc_segment_launches(const grz_graph* g)
{
    uint64_t n = 0;
    for (uint32_t sg = 0; sg < g->nseg; ++sg) n += g->seg_first[sg + 1] > g->seg_first[sg];
    return n;
}

// Shared-memory opt-in and resident blocks per SM of the CC pull kernel, per device, block size
// and staging form.
template <int BT, bool BULK>
static int cc_pull_config(grz_graph* g, size_t smem, int* resident)
{
    static int configured[64] = {};
    const int bit = (BT == 256 ? 1 : (BT == 512 ? 2 : 4)) << (BULK ? 3 : 0);
    if (g->device < 0 || g->device >= 64) return GRZ_ERR_ARG;
    if (!(configured[g->device] & bit)) {
        cudaFuncAttributes fa;
        int optin = 0;
        GRZ_CK(g, cudaFuncGetAttributes(&fa, k_cc_pull<BT, BULK>));
        GRZ_CK(g, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, g->device));
        GRZ_CK(g, cudaFuncSetAttribute(k_cc_pull<BT, BULK>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
        configured[g->device] |= bit;
    }
    GRZ_CK(g, cudaOccupancyMaxActiveBlocksPerMultiprocessor(resident, k_cc_pull<BT, BULK>, BT, smem));
    if (*resident < 1) return grz_set_error(g, GRZ_ERR_ARG, "CC pull: %d threads with %zu bytes of shared memory do not fit", BT, smem);
    return GRZ_OK;
}

template <int BT>
static int cc_pull_config_any(grz_graph* g, size_t smem, int* resident)
{
    return g->tune.pull_staging ? cc_pull_config<BT, true>(g, smem, resident) : cc_pull_config<BT, false>(g, smem, resident);
}

// Compacts the vertices selected by bm1 & bm2 (defined below)
static void compact(grz_graph* g, const unsigned long long* bm1, const unsigned long long* bm2, const uint32_t* rowptr,
                    uint32_t skip = 0, const uint32_t* gate = nullptr);

template <int BT, bool BULK>
static int launch_cc_pull_bt(grz_graph* g, uint64_t first, uint64_t count, const VoteCfg& vc)
{
    grz_frontier_state& f = g->fr;
    const uint32_t ncache = std::min<uint32_t>(g->tune.cc_cache, g->pull.nhub);
    const size_t smem = sizeof(uint32_t) * ncache;
    int resident = 0;
    int rc = cc_pull_config<BT, BULK>(g, smem, &resident);
    if (rc) return rc;
    const uint64_t tiles = (count + BT - 1) / BT;
    uint64_t grid = g->tune.cc_grid ? g->tune.cc_grid : (uint64_t)g->num_sms * resident;
    grid = std::max<uint64_t>(1, std::min<uint64_t>(grid, tiles));
    // the skip needs every earlier iteration to have been complete (the whole list, or the whole
    // frontier): true for the driver loops, not once a phases.h call covered part of the list
    const bool whole = !f.cc_partial && first == 0 && count == g->pull.nvec;
    if (whole && g->tune.cc_pull_first) {
        // Each destination's first vector (k_cc_pull_first, which decides on the device whether
        // this is an iteration without a usable previous minimum and otherwise returns at once).
        // Form 1: the whole list without the destinations at 0.  Form 2: the destinations it left
        // open are compacted with their remaining vectors and pulled (gated, empty in a skip
        // iteration), and the skip pass over the whole list runs only in a skip iteration; its
        // first pull is shorter, but it propagates less in place and the runs take one iteration
        // more (GB300, R-MAT 24 sym: 0.81 against 0.76 ms per run).
        const bool open_list = g->tune.cc_pull_first == 2;
        uint32_t* gate = f.counters + 6;
        const uint64_t W = words_of(g->V), groups = (W + CFW - 1) / CFW;
        const unsigned fgrid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((groups + T / 32 - 1) / (T / 32),
                                                                                   (uint64_t)g->num_sms * 8));
        const bool open_all = g->tune.cc_pull_first == 4;
        k_cc_pull_first<<<fgrid, T, 0, g->stream>>>(g->pull.rowptr, g->pull.nbr, (uint32_t)g->V, W, f.label, g->pull.hub_vid,
                                                     g->pull.nhub, f.has_next, vc, f.vote, f.chg, f.iter, f.level_dev,
                                                     (open_list || open_all) ? f.unres : nullptr, gate, open_all ? 1 : 0); GRZ_COUNT_LAUNCH(g);
        unsigned long long* work = nullptr;
        if (g->prof && g->prof->on) {
            if (!g->prof_work) {
                GRZ_CK(g, cudaMalloc((void**)&g->prof_work, sizeof(unsigned long long) * 2));
                GRZ_CK(g, cudaMemsetAsync(g->prof_work, 0, sizeof(unsigned long long) * 2, g->stream));
            }
            work = g->prof_work;
        }
        auto expand = [&]() {
            k_cc_pull_expand<<<(unsigned)g->num_sms * 8, T, 0, g->stream>>>(f.frontier, f.voff, f.vdelta, f.tile_first, f.counters,
                                                                           g->pull.nbr, (uint32_t)g->V, f.label, g->pull.hub_vid,
                                                                           g->pull.nhub, f.has_next, vc, f.vote, f.chg, f.iter,
                                                                           f.level_dev, f.counters + 5, work); GRZ_COUNT_LAUNCH(g);
        };
        if (open_all) {
            // form 4: every pull over the open destinations only, marked by the first-vector pass
            // (first iteration: every vector of those still above 0) or by k_cc_mark_open (later
            // iterations); one of the two writes the whole bitmap in each iteration
            const unsigned mgrid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((W + T / 32 - 1) / (T / 32),
                                                                                       (uint64_t)g->num_sms * 8));
            k_cc_mark_open<<<mgrid, T, 0, g->stream>>>(f.label, f.nonempty_pull, g->V, W, f.chg, f.iter, f.level_dev, f.unres,
                                                        nullptr); GRZ_COUNT_LAUNCH(g);
            compact(g, f.unres, f.nonempty_pull, g->pull.rowptr, 0, nullptr);
            expand();
            return GRZ_OK;
        }
        if (open_list) {
            compact(g, f.unres, f.unres, g->pull.rowptr, 1, gate);
            expand();
        }
        // form 3: the whole list only in the first iteration; in a skip iteration the destinations
        // above the previous minimum are marked, compacted and pulled instead of the whole list
        const bool open_skip = g->tune.cc_pull_first == 3;
        k_cc_pull<BT, BULK><<<(unsigned)grid, BT, smem, g->stream>>>(g->pull.nbr, g->pull.shared, first, count, (uint32_t)g->V, f.label,
                                                                    g->pull.hub_vid, g->pull.nhub, ncache, f.has_next, vc, f.vote, f.chg,
                                                                    f.iter, f.level_dev, open_list ? 3 : (open_skip ? 5 : 4),
                                                                    f.dev_err); GRZ_COUNT_LAUNCH(g);
        if (open_skip) {
            uint32_t* gate2 = f.counters + 7;
            const unsigned mgrid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((W + T / 32 - 1) / (T / 32),
                                                                                       (uint64_t)g->num_sms * 8));
            k_cc_mark_open<<<mgrid, T, 0, g->stream>>>(f.label, f.nonempty_pull, g->V, W, f.chg, f.iter, f.level_dev, f.unres,
                                                        gate2); GRZ_COUNT_LAUNCH(g);
            compact(g, f.unres, f.nonempty_pull, g->pull.rowptr, 0, gate2);
            expand();
        }
        return GRZ_OK;
    }
    if (whole && cc_use_segments(g)) {
        // The full pass (no skip yet) reads the source-segmented lists, so that each segment's
        // labels stay in L2 while its edges stream; the pass with the skip reads the whole list
        // (it reads destinations, not sources).  Which of them does the work is decided on the
        // device, so one captured run graph holds both.
        for (uint32_t sg = 0; sg < g->nseg; ++sg) {
            const uint64_t a = g->seg_first[sg], n = g->seg_first[sg + 1] - a;
            if (n == 0) continue;
            const uint64_t sgrid = std::max<uint64_t>(1, std::min<uint64_t>(grid, (n + BT - 1) / BT));
            k_cc_pull<BT, false><<<(unsigned)sgrid, BT, 0, g->stream>>>(g->seg_nbr, g->seg_dst, a, n, (uint32_t)g->V, f.label, nullptr,
                                                                       0u, 0u, f.has_next, vc, f.vote, f.chg, f.iter, f.level_dev, 2,
                                                                       f.dev_err); GRZ_COUNT_LAUNCH(g);
        }
        k_cc_pull<BT, BULK><<<(unsigned)grid, BT, smem, g->stream>>>(g->pull.nbr, g->pull.shared, first, count, (uint32_t)g->V, f.label,
                                                                    g->pull.hub_vid, g->pull.nhub, ncache, f.has_next, vc, f.vote, f.chg,
                                                                    f.iter, f.level_dev, 3, f.dev_err); GRZ_COUNT_LAUNCH(g);
        return GRZ_OK;
    }
    k_cc_pull<BT, BULK><<<(unsigned)grid, BT, smem, g->stream>>>(g->pull.nbr, g->pull.shared, first, count, (uint32_t)g->V, f.label,
                                                                g->pull.hub_vid, g->pull.nhub, ncache, f.has_next, vc, f.vote, f.chg,
                                                                f.iter, f.level_dev, whole ? 1 : 0, f.dev_err); GRZ_COUNT_LAUNCH(g);
    return GRZ_OK;
}

static int launch_cc_pull(grz_graph* g, uint64_t first, uint64_t count, const VoteCfg& vc)
{
    const bool b = g->tune.pull_staging != 0;
    switch (g->tune.cc_threads) {
    case 256: return b ? launch_cc_pull_bt<256, true>(g, first, count, vc) : launch_cc_pull_bt<256, false>(g, first, count, vc);
    case 1024: return b ? launch_cc_pull_bt<1024, true>(g, first, count, vc) : launch_cc_pull_bt<1024, false>(g, first, count, vc);
    default: return b ? launch_cc_pull_bt<512, true>(g, first, count, vc) : launch_cc_pull_bt<512, false>(g, first, count, vc);
    }
}

// Compacts the vertices selected by bm1 & bm2, with their vector ranges in `rowptr`, into
// fr.frontier / voff / vdelta / tile_first (counts on the device in counters[0], [2]).
static void compact(grz_graph* g, const unsigned long long* bm1, const unsigned long long* bm2, const uint32_t* rowptr,
                    uint32_t skip, const uint32_t* gate)
{
    grz_frontier_state& f = g->fr;
    cudaStream_t st = g->stream;
    const unsigned nb = (unsigned)(g->V / CCHUNK + 1);
    k_fr_count<<<nb, T, 0, st>>>(bm1, bm2, g->V, rowptr, skip, gate, f.fr_part, f.fr_part + nb); GRZ_COUNT_LAUNCH(g);
    k_fr_scan<<<1, SCAN_T, 0, st>>>(f.fr_part, f.fr_part + nb, nb, f.counters, gate); GRZ_COUNT_LAUNCH(g);
    k_fr_write<<<nb, T, 0, st>>>(bm1, bm2, g->V, rowptr, skip, f.fr_part, f.fr_part + nb, f.counters, nb, f.frontier, f.voff,
                                 f.vdelta, f.tile_first, gate); GRZ_COUNT_LAUNCH(g);
}

// One edge phase on a vector range of the pull (pull=1) or push list.  Leaves the vote of the
// phase in fr.vote[0] on the device.  The push engine always expands the whole compacted frontier.
static int edge_phase(grz_graph* g, int pull, uint64_t first, uint64_t count)
{
    grz_frontier_state& f = g->fr;
    const uint32_t V = (uint32_t)g->V;
    const uint64_t W = words_of(g->V);
    cudaStream_t st = g->stream;
    const VoteCfg vc = vote_cfg(g);
    const bool bfs = f.app == GRZ_APP_BREADTH_FIRST_SEARCH;
    GRZ_CK(g, cudaMemsetAsync(f.counters, 0, sizeof(uint32_t) * 8, st));
    if (pull) {
        if (!g->pull.nbr) return grz_set_error(g, GRZ_ERR_STATE, "pull list not loaded");
        if (count == 0) return GRZ_OK;
        const bool compacted = bfs && first == 0 && count == g->pull.nvec && !g->tune.bfs_pull_scan;
        const uint32_t first_n = g->tune.bfs_pull_first;
        if (compacted && first_n) {
            // the whole list: each wanted destination's first vectors up to the first frontier
            // source, then the remaining vectors of those left undecided
            if (g->stats_on) {  // the work counted is the reference's: every vector of the wanted destinations
                compact(g, f.wants, f.nonempty_pull, g->pull.rowptr);
                GRZ_TRY(grz_stats_count_selected(g, &g->pull, f.frontier, f.counters));
            }
            grz_prof_begin(g, GRZ_PROF_BFS_PULL);
            const uint64_t pgroups = (W + FW - 1) / FW;
            const unsigned fgrid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((pgroups + T / 32 - 1) / (T / 32),
                                                                                       (uint64_t)g->num_sms * GRZ_BFS_MINB));
            k_bfs_pull_first<<<fgrid, T, 0, st>>>(f.wants, f.nonempty_pull, g->pull.rowptr, g->pull.nbr, V, W, f.has,
                                                  g->pull.hub_vid, g->pull.nhub, f.has_next, f.unres, first_n, f.label, f.level,
                                                  f.iter, f.level_dev, vc, f.vote); GRZ_COUNT_LAUNCH(g);
            compact(g, f.unres, f.unres, g->pull.rowptr, first_n);
            k_bfs_pull_expand<<<(unsigned)g->num_sms * 8, T, 0, st>>>(f.frontier, f.voff, f.vdelta, f.tile_first, f.counters,
                                                                     g->pull.nbr, V, f.has, f.cand64, f.touched, f.counters + 1,
                                                                     g->pull.hub_vid, g->pull.nhub, f.has_next, f.counters + 5); GRZ_COUNT_LAUNCH(g);
        } else if (compacted) {
            // the whole list: only the vectors of wanted destinations
            grz_prof_begin(g, GRZ_PROF_PUSH_COMPACT);
            compact(g, f.wants, f.nonempty_pull, g->pull.rowptr);
            grz_prof_end(g);
            GRZ_TRY(grz_stats_count_selected(g, &g->pull, f.frontier, f.counters));
            grz_prof_begin(g, GRZ_PROF_BFS_PULL);
            k_bfs_pull_expand<<<(unsigned)g->num_sms * 8, T, 0, st>>>(f.frontier, f.voff, f.vdelta, f.tile_first, f.counters,
                                                                     g->pull.nbr, V, f.has, f.cand64, f.touched, f.counters + 1,
                                                                     g->pull.hub_vid, g->pull.nhub, f.has_next, f.counters + 5); GRZ_COUNT_LAUNCH(g);
        } else {
            GRZ_TRY(grz_stats_count_range(g, &g->pull, first, count));
            grz_prof_begin(g, bfs ? GRZ_PROF_BFS_PULL : GRZ_PROF_CC_PULL);
        }
        if (bfs && !compacted) {
            const unsigned pgrid = (unsigned)std::min<uint64_t>(blocks_for(count), (uint64_t)g->num_sms * 8);
            k_bfs_pull<<<pgrid, T, 0, st>>>(g->pull.nbr, g->pull.shared, first, count, V, f.has, f.wants, f.cand64,
                                                       f.touched, f.counters + 1, g->pull.hub_vid, g->pull.nhub, f.has_next); GRZ_COUNT_LAUNCH(g);
        }
        if (bfs) {
            grz_prof_end(g);
            grz_prof_begin(g, GRZ_PROF_BFS_VISIT);
            k_bfs_visit<true><<<visit_grid(g), T, 0, st>>>(f.touched, f.counters + 1, f.cand64, f.cand32, f.label, f.level,
                                                            f.iter, f.level_dev, f.wants, f.has_next, vc, f.vote, V); GRZ_COUNT_LAUNCH(g);
        } else {
            int rc = launch_cc_pull(g, first, count, vc);
            if (rc) return rc;
        }
        grz_prof_end(g);
    } else {
        if (!g->push.nbr) return grz_set_error(g, GRZ_ERR_STATE, "push list not loaded");
        grz_prof_begin(g, GRZ_PROF_PUSH_COMPACT);
        compact(g, f.has, f.nonempty_push, g->push.rowptr);
        grz_prof_end(g);
        GRZ_TRY(grz_stats_count_selected(g, &g->push, f.frontier, f.counters));
        grz_prof_begin(g, bfs ? GRZ_PROF_BFS_PUSH : GRZ_PROF_CC_PUSH);
        const unsigned grid = (unsigned)g->num_sms * 8;
        if (bfs) {
            k_push_expand<true><<<grid, T, 0, st>>>(f.frontier, f.voff, f.vdelta, f.tile_first, f.counters, g->push.nbr, V, f.label,
                                                    f.has_next, f.wants, f.cand32, f.touched, f.counters + 1, vc, f.vote,
                                                    nullptr, 0, nullptr); GRZ_COUNT_LAUNCH(g);
            grz_prof_end(g);
            grz_prof_begin(g, GRZ_PROF_BFS_VISIT);
            k_bfs_visit<false><<<visit_grid(g), T, 0, st>>>(f.touched, f.counters + 1, f.cand64, f.cand32, f.label, f.level,
                                                             f.iter, f.level_dev, f.wants, f.has_next, vc, f.vote, V); GRZ_COUNT_LAUNCH(g);
        } else {
            k_push_expand<false><<<grid, T, 0, st>>>(f.frontier, f.voff, f.vdelta, f.tile_first, f.counters, g->push.nbr, V, f.label,
                                                     f.has_next, f.wants, f.cand32, f.touched, f.counters + 1, vc, f.vote,
                                                     f.chg, f.iter, f.level_dev); GRZ_COUNT_LAUNCH(g);
        }
        grz_prof_end(g);
    }
    return grz_cuda_check(g, cudaGetLastError(), "edge phase");
}

// perform_vertex_phase_{cc,bfs}: HasInfo <- HasInfo*, HasInfo* <- 0 (pointer swap + clear)
int grz_frontier_vertex_phase(grz_graph* g, uint64_t first, uint64_t count)
{
    (void)first;
    (void)count;
    grz_frontier_state& f = g->fr;
    if (!grz_frontier_live(g)) return grz_set_error(g, GRZ_ERR_STATE, "frontier state not initialised for the loaded graph");
    unsigned long long* t = f.has;
    f.has = f.has_next;
    f.has_next = t;
    GRZ_CK(g, cudaMemsetAsync(f.has_next, 0, sizeof(unsigned long long) * words_of(g->V), g->stream));
    return GRZ_OK;
}

// the phases.h entry points: one edge phase with a fresh vote, counted into the iteration total
int grz_cc_phase(grz_graph* g, int pull, uint64_t first_vec, uint64_t count)
{
    if (!grz_frontier_live(g) || g->fr.app != GRZ_APP_CONNECTED_COMPONENTS) {
        int rc = grz_frontier_init(g, GRZ_APP_CONNECTED_COMPONENTS, 0, 0);
        if (rc) return rc;
    }
    // An edge phase per call, numbered like the driver loops' iterations.  A pull over part of
    // the list leaves the converged-destination skip off for the rest of this state (the tag
    // 2^32 - 1 never matches; grz_frontier_init starts over).
    grz_frontier_state& f = g->fr;
    const bool whole = !pull || (first_vec == 0 && count == g->pull.nvec);
    if (!whole) f.cc_partial = 1;
    f.iter++;
    const int rc = edge_phase(g, pull, first_vec, count);
    if (rc) return rc;
    if (f.cc_partial) GRZ_CK(g, cudaMemsetAsync(f.chg, 0xff, 2 * sizeof(unsigned long long), g->stream));
    return GRZ_OK;
}

int grz_bfs_phase(grz_graph* g, int pull, uint64_t first_vec, uint64_t count)
{
    if (!grz_frontier_live(g) || g->fr.app != GRZ_APP_BREADTH_FIRST_SEARCH) {
        int rc = grz_frontier_init(g, GRZ_APP_BREADTH_FIRST_SEARCH, 0, 0);
        if (rc) return rc;
    }
    grz_frontier_state& f = g->fr;
    f.iter++;  // a BFS level per edge phase; the root is level 0
    return edge_phase(g, pull, first_vec, count);
}

// Runs one iteration: engine choice from the current vote (or the caller's choice), the edge
// phase, the vote read-back and, unless converged, the vertex phase.  Returns 1 while not
// converged, 0 when the vote is 0, negative on error.  *engine_out = 1 pull / 0 push.
int grz_frontier_step(grz_graph* g, int engine, int* engine_out, uint64_t* vote_out)
{
    grz_frontier_state& f = g->fr;
    const bool learned = f.policy == GRZ_POLICY_LEARNED && f.mlp;
    int rc;
    if (engine < 0 && learned && f.iter == 0) {
        // first iteration: decide from the initial frontier and the initial vote
        uint64_t v0 = 0;
        rc = grz_switch_decide(g, f.has, f.vote_host, 1, &v0, &f.next_pull, f.last_features);
        if (rc) return rc;
    }
    const bool forced = (f.flags & (GRZ_FLAG_FORCE_PULL | GRZ_FLAG_FORCE_PUSH)) != 0;
    const int pull = engine >= 0 ? engine : ((learned && !forced) ? f.next_pull : grz_engine_threshold(g, f.vote_host));
    if (engine_out) *engine_out = pull;
    GRZ_CK(g, cudaMemsetAsync(f.vote, 0, sizeof(unsigned long long) * GRZ_VOTE_SLOTS * GRZ_VOTE_STRIDE, g->stream));
    f.iter++;
    if (f.time_edges) GRZ_CK(g, cudaEventRecord(f.ev[0], g->stream));
    rc = edge_phase(g, pull, 0, pull ? g->pull.nvec : g->push.nvec);
    if (rc) return rc;
    if (f.time_edges) GRZ_CK(g, cudaEventRecord(f.ev[1], g->stream));
    if (pull) f.npull++; else f.npush++;
    f.last_engine = pull;
    uint64_t v = 0;
    if (learned) {
        // the vote and the next engine in one read-back; the next frontier is HasInfo*
        rc = grz_switch_decide(g, f.has_next, ~0ull, f.iter + 1, &v, &f.next_pull, f.last_features);
    } else {
        rc = grz_read_vote(g, &v);
    }
    if (rc) return rc;
    if (f.time_edges) {
        GRZ_CK(g, cudaEventSynchronize(f.ev[1]));
        GRZ_CK(g, cudaEventElapsedTime(&f.last_edge_ms, f.ev[0], f.ev[1]));
    }
    f.vote_host = v;
    if (vote_out) *vote_out = v;
    if (v == 0) return 0;
    rc = grz_frontier_vertex_phase(g, 0, g->V);
    return rc ? rc : 1;
}

// GRZ_ERR_TIMEOUT if a bounded device-side wait of an edge phase gave up since grz_frontier_init
// (synchronises the stream)
int grz_frontier_check_waits(grz_graph* g)
{
    grz_frontier_state& f = g->fr;
    if (!f.dev_err) return GRZ_OK;
    unsigned e = 0;
    GRZ_CK(g, cudaMemcpyAsync(&e, f.dev_err, sizeof(e), cudaMemcpyDeviceToHost, g->stream));
    GRZ_CK(g, cudaStreamSynchronize(g->stream));
    if (e) return grz_set_error(g, GRZ_ERR_TIMEOUT, "an edge phase's wait for its staged vectors ran out");
    return GRZ_OK;
}

// the pinned host buffer the per-iteration read-backs go through
int grz_frontier_mail(grz_graph* g)
{
    if (!g->fr.mail) GRZ_CK(g, cudaMallocHost(&g->fr.mail, sizeof(unsigned long long) * GRZ_VOTE_SLOTS * GRZ_VOTE_STRIDE));
    return GRZ_OK;
}

// sum of the vote slots (synchronises the stream)
int grz_read_vote(grz_graph* g, uint64_t* out)
{
    const int rc = grz_frontier_mail(g);
    if (rc) return rc;
    const size_t bytes = sizeof(unsigned long long) * GRZ_VOTE_SLOTS * GRZ_VOTE_STRIDE;
    GRZ_CK(g, cudaMemcpyAsync(g->fr.mail, g->fr.vote, bytes, cudaMemcpyDeviceToHost, g->stream));
    GRZ_CK(g, cudaStreamSynchronize(g->stream));
    const unsigned long long* slots = (const unsigned long long*)g->fr.mail;
    uint64_t v = 0;
    for (int i = 0; i < GRZ_VOTE_SLOTS; ++i) v += slots[i * GRZ_VOTE_STRIDE];
    *out = v;
    return GRZ_OK;
}

// digest of a CC/BFS result: out[0] = reached vertices (BFS: level set; CC: label == own id,
// i.e. components), out[1] = sum of out-degrees of the reached vertices (BFS), out[2] = an
// order-independent checksum of the labels and levels: sum over v of (value(v) + 1) * odd(v)
// mod 2^64, where value is the BFS level or the CC label (unreached = 2^32 - 1)
__global__ void __launch_bounds__(T) k_digest(const uint32_t* __restrict__ label, const uint32_t* __restrict__ level,
                                              const uint32_t* __restrict__ degree, uint64_t V, int bfs,
                                              unsigned long long* __restrict__ out)
{
    unsigned long long r = 0, e = 0, h = 0;
    for (uint64_t v = (uint64_t)blockIdx.x * T + threadIdx.x; v < V; v += (uint64_t)gridDim.x * T) {
        const uint32_t x = bfs ? level[v] : label[v];
        const bool reached = bfs ? x != INF : x == (uint32_t)v;
        if (reached) {
            r += 1;
            if (bfs) e += degree[v];
        }
        h += ((unsigned long long)x + 1ull) * ((v * 0x9E3779B97F4A7C15ull) | 1ull);
    }
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_down_sync(0xffffffffu, r, o);
        e += __shfl_down_sync(0xffffffffu, e, o);
        h += __shfl_down_sync(0xffffffffu, h, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out + 0, r);
        atomicAdd(out + 1, e);
        atomicAdd(out + 2, h);
    }
}

int grz_frontier_digest(grz_graph* g, uint64_t* out3)
{
    grz_frontier_state& f = g->fr;
    if (!grz_frontier_live(g)) return grz_set_error(g, GRZ_ERR_STATE, "no CC/BFS result for the loaded graph");
    int rc = grz_frontier_mail(g);
    if (rc) return rc;
    unsigned long long* d = nullptr;
    GRZ_CK(g, cudaMallocAsync((void**)&d, 3 * sizeof(unsigned long long), g->stream));
    cudaError_t e = cudaMemsetAsync(d, 0, 3 * sizeof(unsigned long long), g->stream);
    if (e == cudaSuccess && g->V) {
        const unsigned grid = (unsigned)std::min<uint64_t>(blocks_for(g->V), (uint64_t)g->num_sms * 8);
        k_digest<<<grid, T, 0, g->stream>>>(f.label, f.level, g->degree, g->V, f.app == GRZ_APP_BREADTH_FIRST_SEARCH, d); GRZ_COUNT_LAUNCH(g);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(f.mail, d, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, g->stream);
    cudaFreeAsync(d, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return grz_cuda_check(g, e, "digest");
    memcpy(out3, f.mail, 3 * sizeof(uint64_t));
    return GRZ_OK;
}

int grz_frontier_props(grz_graph* g)
{
    grz_frontier_state& f = g->fr;
    if (!grz_frontier_live(g)) return grz_set_error(g, GRZ_ERR_STATE, "no CC/BFS result for the loaded graph");
    k_u32_to_double<<<blocks_for(g->V), T, 0, g->stream>>>(f.label, g->V, g->prop, f.app == GRZ_APP_BREADTH_FIRST_SEARCH); GRZ_COUNT_LAUNCH(g);
    GRZ_CK(g, cudaGetLastError());
    return GRZ_OK;
}

void grz_frontier_park(grz_graph* g)
{
    grz_frontier_state& f = g->fr;
    // the captured run names the old lists
    if (f.run_exec) cudaGraphExecDestroy(f.run_exec);
    f.run_exec = nullptr;
    f.run_bm[0] = f.run_bm[1] = nullptr;
    f.lists_changed = 1;
}

void grz_frontier_free(grz_graph* g)
{
    grz_frontier_state& f = g->fr;
    void* ptrs[] = { f.label, f.level, f.has, f.has_next, f.wants, f.nonempty_push, f.nonempty_pull, f.unres, f.frontier, f.voff, f.vdelta, f.tile_first, f.chg, f.dev_err,
                     f.fr_part, f.touched, f.cand64, f.cand32,
                     f.counters, f.vote, f.sw_out, f.snap };
    for (void* p : ptrs) cudaFree(p);
    if (f.ev[0]) { cudaEventDestroy(f.ev[0]); cudaEventDestroy(f.ev[1]); }
    if (f.mail) cudaFreeHost(f.mail);
    if (f.run_exec) cudaGraphExecDestroy(f.run_exec);
    cudaFree(f.ctl);
    grz_mlp* keep_mlp = f.mlp;
    const int keep_policy = f.policy;
    memset(&f, 0, sizeof(f));
    f.mlp = keep_mlp;
    f.policy = keep_policy;
}

// ---------------------------------------------------------------------------------------------
// A whole CC/BFS run as one CUDA graph.
//
//   k_run_decide (initial: sets pull0/push0)  ->  WHILE (loop) {
//       IF (pull0) { pull edge phase, even roles }   IF (push0) { push edge phase, even roles }
//       k_run_decide (next HasInfo = B, clears A; sets pull1/push1, loop)
//       IF (pull1) { pull edge phase, odd roles }    IF (push1) { push edge phase, odd roles }
//       k_run_decide (next HasInfo = A, clears B; sets pull0/push0, loop)
//   }
//
// Even iterations read HasInfo from buffer A and write HasInfo* into B; odd ones the reverse,
// which is the reference's pointer swap (source/execution_cc.c:245-250) without a host step.
// The decision kernel sets the conditional handles, so the engine choice, the convergence test
// and the iteration count never leave the device: one launch, one read-back of the control
// block.  The iterations, engines and results are those of the host loop (grz_frontier_step).

static int capture_begin(grz_graph* g, cudaStream_t cs, cudaGraph_t graph, const cudaGraphNode_t* deps, size_t ndeps)
{
    GRZ_CK(g, cudaStreamBeginCaptureToGraph(cs, graph, deps, nullptr, ndeps, cudaStreamCaptureModeThreadLocal));
    return GRZ_OK;
}

// ends a capture into an existing graph; *sink = the captured work's last node
static int capture_end(grz_graph* g, cudaStream_t cs, cudaGraphNode_t* sink)
{
    cudaStreamCaptureStatus st;
    const cudaGraphNode_t* deps = nullptr;
    size_t n = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(cs, &st, nullptr, nullptr, &deps, nullptr, &n);
    cudaGraphNode_t last = (e == cudaSuccess && n == 1) ? deps[0] : nullptr;
    cudaGraph_t out = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(cs, &out);
    if (e != cudaSuccess) return grz_cuda_check(g, e, "capture info");
    if (e2 != cudaSuccess) return grz_cuda_check(g, e2, "end capture");
    if (sink) {
        if (!last) return grz_set_error(g, GRZ_ERR_STATE, "captured work does not end in one node");
        *sink = last;
    }
    return GRZ_OK;
}

static int add_conditional(grz_graph* g, cudaGraph_t graph, const cudaGraphNode_t* deps, size_t ndeps, cudaGraphConditionalHandle h,
                           cudaGraphConditionalNodeType type, cudaGraphNode_t* node, cudaGraph_t* body)
{
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = type;
    p.conditional.size = 1;
    GRZ_CK(g, cudaGraphAddNode(node, graph, deps, nullptr, ndeps, &p));
    *body = p.conditional.phGraph_out[0];
    return GRZ_OK;
}

static int build_run_graph(grz_graph* g)
{
    grz_frontier_state& f = g->fr;
    if (f.run_exec) {
        cudaGraphExecDestroy(f.run_exec);
        f.run_exec = nullptr;
    }
    unsigned long long* A = f.has;
    unsigned long long* B = f.has_next;
    cudaStream_t user = g->stream;
    cudaStream_t cs = nullptr;
    GRZ_CK(g, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t top = nullptr;
    int rc = grz_cuda_check(g, cudaGraphCreate(&top, 0), "graph create");
    // one handle per conditional node: the loop, and pull / push for the even and odd halves
    cudaGraphConditionalHandle hloop = 0, hpull[2] = { 0, 0 }, hpush[2] = { 0, 0 };
    if (!rc) rc = grz_cuda_check(g, cudaGraphConditionalHandleCreate(&hloop, top, 1, cudaGraphCondAssignDefault), "handle");
    for (int p = 0; p < 2 && !rc; ++p) {
        rc = grz_cuda_check(g, cudaGraphConditionalHandleCreate(&hpull[p], top, 0, cudaGraphCondAssignDefault), "handle");
        if (!rc) rc = grz_cuda_check(g, cudaGraphConditionalHandleCreate(&hpush[p], top, 0, cudaGraphCondAssignDefault), "handle");
    }
    g->stream = cs;
    f.level_dev = &f.ctl->level;
    cudaGraphNode_t n0 = nullptr, wnode = nullptr;
    cudaGraph_t body = nullptr;
    if (!rc) rc = capture_begin(g, cs, top, nullptr, 0);
    if (!rc) {
        rc = grz_switch_launch_run_decide(g, A, nullptr, 1, hloop, hpull[0], hpush[0]);
        const int rc2 = capture_end(g, cs, &n0);
        if (!rc) rc = rc2;
    }
    if (!rc) rc = add_conditional(g, top, &n0, 1, hloop, cudaGraphCondTypeWhile, &wnode, &body);
    cudaGraphNode_t prev = nullptr;
    for (int parity = 0; parity < 2 && !rc; ++parity) {
        f.has = parity ? B : A;
        f.has_next = parity ? A : B;
        cudaGraphNode_t npull = nullptr, npush = nullptr, ndec = nullptr;
        cudaGraph_t bpull = nullptr, bpush = nullptr;
        rc = add_conditional(g, body, prev ? &prev : nullptr, prev ? 1 : 0, hpull[parity], cudaGraphCondTypeIf, &npull, &bpull);
        if (!rc) rc = capture_begin(g, cs, bpull, nullptr, 0);
        if (!rc) {
            rc = edge_phase(g, 1, 0, g->pull.nvec);
            const int rc2 = capture_end(g, cs, nullptr);
            if (!rc) rc = rc2;
        }
        if (!rc) rc = add_conditional(g, body, &npull, 1, hpush[parity], cudaGraphCondTypeIf, &npush, &bpush);
        if (!rc) rc = capture_begin(g, cs, bpush, nullptr, 0);
        if (!rc) {
            rc = edge_phase(g, 0, 0, g->push.nvec);
            const int rc2 = capture_end(g, cs, nullptr);
            if (!rc) rc = rc2;
        }
        if (!rc) rc = capture_begin(g, cs, body, &npush, 1);
        if (!rc) {
            // decides the other half's engine
            rc = grz_switch_launch_run_decide(g, f.has_next, f.has, 0, hloop, hpull[1 - parity], hpush[1 - parity]);
            const int rc2 = capture_end(g, cs, &ndec);
            if (!rc) rc = rc2;
        }
        prev = ndec;
    }
    f.has = A;
    f.has_next = B;
    f.level_dev = nullptr;
    g->stream = user;
    if (!rc) rc = grz_cuda_check(g, cudaGraphInstantiate(&f.run_exec, top, 0), "graph instantiate");
    if (top) cudaGraphDestroy(top);
    cudaStreamDestroy(cs);
    if (rc) {
        f.run_exec = nullptr;
        return rc;
    }
    f.run_bm[0] = A;
    f.run_bm[1] = B;
    f.run_key[0] = f.app;
    f.run_key[1] = f.flags;
    f.run_tune = g->tune;
    f.run_seg = cc_use_segments(g) ? g->seg_nbr : nullptr;
    return GRZ_OK;
}

// Before grz_frontier_init: puts the HasInfo buffers back in the roles the cached graph has.
void grz_frontier_run_prepare(grz_graph* g)
{
    grz_frontier_state& f = g->fr;
    if (f.run_exec && f.has == f.run_bm[1] && f.has_next == f.run_bm[0]) {
        f.has = f.run_bm[0];
        f.has_next = f.run_bm[1];
    }
}

// Runs the initialised CC/BFS state to convergence with one graph launch.  *launches: kernels
// the graph ran.
int grz_frontier_run_graph(grz_graph* g, uint64_t* launches)
{
    grz_frontier_state& f = g->fr;
    if (!grz_frontier_live(g)) return grz_set_error(g, GRZ_ERR_STATE, "frontier state not initialised for the loaded graph");
    if (!g->pull.nbr || !g->push.nbr || !g->pull.nvec || !g->push.nvec)
        return grz_set_error(g, GRZ_ERR_STATE, "the graph run needs both edge lists");
    int rc = grz_frontier_mail(g);
    if (rc) return rc;
    if (!f.ctl) {
        GRZ_CK(g, cudaMalloc((void**)&f.ctl, sizeof(grz_runctl)));
    }
    rc = grz_switch_max_degree(g);
    if (rc) return rc;
    const bool same = f.run_exec && f.run_bm[0] == f.has && f.run_bm[1] == f.has_next && f.run_key[0] == f.app &&
                      f.run_key[1] == f.flags && !memcmp(&f.run_tune, &g->tune, sizeof(g->tune)) &&
                      f.run_seg == (cc_use_segments(g) ? g->seg_nbr : nullptr);
    if (!same) {
        int resident = 0;
        const size_t smem = sizeof(uint32_t) * std::min<uint32_t>(g->tune.cc_cache, g->pull.nhub);
        rc = g->tune.cc_threads == 256 ? cc_pull_config_any<256>(g, smem, &resident)
             : (g->tune.cc_threads == 1024 ? cc_pull_config_any<1024>(g, smem, &resident) : cc_pull_config_any<512>(g, smem, &resident));
        if (!rc) rc = build_run_graph(g);
        if (rc) return rc;
    }
    grz_runctl c;
    memset(&c, 0, sizeof(c));
    c.running = 1;
    c.level = f.iter + 1;
    c.last_engine = (uint32_t)f.last_engine;
    c.vote = f.vote_host;
    const uint64_t max_it = g->tune.run_max_iterations ? g->tune.run_max_iterations : std::min<uint64_t>(g->V + 2, 0xfffffff0ull);
    c.max_level = (uint32_t)std::min<uint64_t>(max_it + f.iter, 0xfffffff0ull);
    c.limit_ns = g->tune.run_limit_us ? (unsigned long long)g->tune.run_limit_us * 1000ull : 300ull * 1000000000ull;
    grz_switch_policy_ctl(g, &c);
    memcpy(f.mail, &c, sizeof(c));
    GRZ_CK(g, cudaMemcpyAsync(f.ctl, f.mail, sizeof(c), cudaMemcpyHostToDevice, g->stream));
    GRZ_CK(g, cudaMemsetAsync(f.vote, 0, sizeof(unsigned long long) * GRZ_VOTE_SLOTS * GRZ_VOTE_STRIDE, g->stream));
    GRZ_CK(g, cudaGraphLaunch(f.run_exec, g->stream));
    GRZ_CK(g, cudaMemcpyAsync(f.mail, f.ctl, sizeof(c), cudaMemcpyDeviceToHost, g->stream));
    GRZ_CK(g, cudaStreamSynchronize(g->stream));
    memcpy(&c, f.mail, sizeof(c));
    if (c.overrun) {
        // the loop stopped before convergence: the state is left as the last iteration made it
        // (a later grz_frontier_begin, grz_cc_run or grz_bfs_run starts over)
        f.iter += c.npull + c.npush;
        f.npull += c.npull;
        f.npush += c.npush;
        if ((c.npull + c.npush) % 2 == 0 && c.npull + c.npush > 0) {
            unsigned long long* t = f.has;
            f.has = f.has_next;
            f.has_next = t;
        }
        if (c.overrun == 1) return grz_set_error(g, GRZ_ERR_TIMEOUT, "no convergence within %u iterations", c.max_level);
        return grz_set_error(g, GRZ_ERR_TIMEOUT, "run stopped by its time bound (%llu us)", c.limit_ns / 1000ull);
    }
    const uint32_t n = c.npull + c.npush;
    f.iter += n;
    f.npull += c.npull;
    f.npush += c.npush;
    f.vote_host = c.vote;
    f.last_engine = (int)c.last_engine;
    f.next_pull = (int)c.engine;
    memcpy(f.last_features, c.features, sizeof(f.last_features));
    // iteration k (1-based within the launch) read HasInfo from A when k is odd
    if (n % 2 == 0 && n > 0) {
        unsigned long long* t = f.has;
        f.has = f.has_next;
        f.has_next = t;
    }
    const bool bfs = f.app == GRZ_APP_BREADTH_FIRST_SEARCH;
    // kernels of one pull iteration: BFS scan + visit, or (first pass,) compaction, expand, visit;
    // CC one pull launch, or one per source segment plus the whole-list one
    const uint64_t per_pull = bfs ? (g->tune.bfs_pull_scan ? 2 : (g->tune.bfs_pull_first ? 6 : 5))
                                  : (f.run_seg ? cc_segment_launches(g) + 1 : (g->tune.cc_pull_first == 2 ? 6 : (g->tune.cc_pull_first == 3 ? 7 : (g->tune.cc_pull_first == 4 ? 6 : (g->tune.cc_pull_first ? 2 : 1)))));
    const uint64_t per_push = bfs ? 5 : 4;
    uint64_t k = 1 + n + (uint64_t)c.npull * per_pull + (uint64_t)c.npush * per_push + (n % 2);
    g->nlaunch += k;
    if (launches) *launches = k;
    return GRZ_OK;
}
