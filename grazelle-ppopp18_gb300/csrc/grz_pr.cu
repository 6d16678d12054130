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
//   * Merge-path tiles (Merrill & Garland, SC'16) over the merged sequence of vectors and row
//     ends give every CTA the same work regardless of in-degree skew.  Each tile stages the
//     per-vector sums of its vectors in shared memory and walks its items.  A destination whose
//     vectors cross tiles is combined with exact u128 atomics; the last tile to arrive finalises
//     it.  No tile ever waits on another.  This replaces the reference's merge buffer
//     (source/phases.c:41-70).
//   * The fused iteration also applies the vertex phase to each destination as soon as its sum
//     is complete.  S_{k+1} = sum_u outdeg[u] * prop_{k+1}[u] is accumulated exactly during
//     iteration k; it equals iteration k+1's sum of accumulators.  So one pass per iteration is
//     enough, with the kernel boundary as the grid-wide barrier.
//   * The vertex formula uses a precomputed 1/deg' multiply instead of the division, at most one
//     rounding apart from the reference.
#include "grz_internal.cuh"

namespace {

constexpr int PR_THREADS = 256;
constexpr int PR_IPT = 8;
constexpr int PR_ITEMS = PR_THREADS * PR_IPT;  // merge items per tile
constexpr int PR_GB = 4;                        // vectors per thread per gather batch

struct PRArgs {
    const uint4* __restrict__ nbr;
    const uint32_t* __restrict__ rowptr;
    const uint2* __restrict__ tile_coord;
    const u128* __restrict__ src_fx;     // props being gathered
    u128* __restrict__ dst_fx;           // fused: next props
    const double* __restrict__ inv_deg;
    const uint32_t* __restrict__ degree;
    u128* __restrict__ split_acc;
    uint32_t* __restrict__ split_cnt;
    const u128* __restrict__ sum_in;     // fused: S_k (exact)
    u128* __restrict__ sum_out;          // fused: S_{k+1}; edge-only: sum of accumulators
    u128* __restrict__ sum_clear;        // fused: buffer to zero for the iteration after next
    double* __restrict__ accum;          // edge-only: reference accumulators (double)
    double* __restrict__ prop_out;       // fused: optional double props
    uint64_t V;
    uint64_t nvec;
    double num_vertices;
    double damping;
    double one_minus_d_by_v;
};

__device__ __forceinline__ u128 ld_fx(const u128* p, uint32_t i)
{
    const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(p) + i);
    u128 r;
    r.lo = v.x;
    r.hi = v.y;
    return r;
}

template <bool Fused>
struct Finalizer {
    const PRArgs& a;
    double G;
    u128 ssum;  // per-thread contribution to sum_out
    __device__ Finalizer(const PRArgs& a_, double G_) : a(a_), G(G_), ssum(u128_zero()) {}
    __device__ __forceinline__ void operator()(uint32_t row, u128 acc)
    {
        if (Fused) {
            const double s = fx_to_double(acc);
            double t = __dadd_rn(s, G);
            t = __dmul_rn(t, a.damping);
            t = __dadd_rn(t, a.one_minus_d_by_v);
            const double p = __dmul_rn(t, a.inv_deg[row]);
            const u128 pf = fx_from_double(p);
            reinterpret_cast<ulonglong2*>(a.dst_fx)[row] = make_ulonglong2(pf.lo, pf.hi);
            if (a.prop_out) a.prop_out[row] = p;
            ssum = u128_add(ssum, u128_mul32(pf, a.degree[row]));
        } else {
            a.accum[row] = fx_to_double(acc);
            ssum = u128_add(ssum, acc);
        }
    }
};

template <bool Fused>
__device__ __forceinline__ void split_contribute(const PRArgs& a, Finalizer<Fused>& fin, uint32_t row, u128 val)
{
    const uint64_t first_item = (uint64_t)a.rowptr[row] + row;
    const uint64_t last_item = (uint64_t)a.rowptr[row + 1] + row;
    const uint32_t ntiles = (uint32_t)(last_item / PR_ITEMS - first_item / PR_ITEMS + 1);
    u128_atomic_add(&a.split_acc[row], val);
    __threadfence();
    const uint32_t old = atomicAdd(&a.split_cnt[row], 1u);
    if (old == ntiles - 1) {
        __threadfence();
        u128 tot;
        tot.lo = atomicAdd(&a.split_acc[row].lo, 0ull);
        tot.hi = atomicAdd(&a.split_acc[row].hi, 0ull);
        a.split_acc[row] = u128_zero();
        a.split_cnt[row] = 0;
        fin(row, tot);
    }
}

template <bool Fused>
__global__ void __launch_bounds__(PR_THREADS) k_pr_pull(PRArgs a)
{
    __shared__ u128 vsum[PR_ITEMS];
    __shared__ uint32_t rend[PR_ITEMS];
    __shared__ uint32_t crow[PR_THREADS];
    __shared__ u128 cacc[PR_THREADS];
    __shared__ double sG;

    const int tid = threadIdx.x;
    const uint32_t tile = blockIdx.x;
    const uint2 c0 = a.tile_coord[tile];
    const uint2 c1 = a.tile_coord[tile + 1];
    const uint32_t r0 = c0.x, v0 = c0.y, r1 = c1.x, v1 = c1.y;
    const int R = (int)(r1 - r0);
    const int NV = (int)(v1 - v0);

    if (Fused && tid == 0) {
        const double S = fx_to_double(*a.sum_in);
        sG = (1.0 - S) / a.num_vertices;
        if (tile == 0 && a.sum_clear) *a.sum_clear = u128_zero();
    }
    for (int i = tid; i < R; i += PR_THREADS) rend[i] = a.rowptr[r0 + i + 1] - v0;

    // gather phase: per-vector exact sums into shared memory
    for (int base = 0; base < NV; base += PR_THREADS * PR_GB) {
        uint4 s[PR_GB];
#pragma unroll
        for (int k = 0; k < PR_GB; ++k) {
            const int j = base + k * PR_THREADS + tid;
            s[k] = (j < NV) ? __ldg(a.nbr + v0 + j) : make_uint4(GRZ_INVALID_ID, GRZ_INVALID_ID, GRZ_INVALID_ID, GRZ_INVALID_ID);
        }
        u128 g[PR_GB][4];
#pragma unroll
        for (int k = 0; k < PR_GB; ++k) {
            const uint32_t ids[4] = { s[k].x, s[k].y, s[k].z, s[k].w };
#pragma unroll
            for (int l = 0; l < 4; ++l) g[k][l] = (ids[l] != GRZ_INVALID_ID) ? ld_fx(a.src_fx, ids[l]) : u128_zero();
        }
#pragma unroll
        for (int k = 0; k < PR_GB; ++k) {
            const int j = base + k * PR_THREADS + tid;
            if (j < NV) vsum[j] = u128_add(u128_add(g[k][2], g[k][3]), u128_add(g[k][0], g[k][1]));
        }
    }
    __syncthreads();

    Finalizer<Fused> fin(a, Fused ? sG : 0.0);

    // walk phase: merge-path over (row ends, vectors) within the tile
    const int items = R + NV;
    const int dt0 = min(tid * PR_IPT, items);
    const int dt1 = min(dt0 + PR_IPT, items);
    int lo = max(0, dt0 - NV), hi = min(dt0, R);
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((int)rend[mid] <= dt0 - mid - 1) lo = mid + 1; else hi = mid;
    }
    int ri = lo, vj = dt0 - lo;
    const bool head_split = a.rowptr[r0] < v0;  // local row 0 started in an earlier tile
    const bool partial_first = (ri == 0) ? (a.rowptr[r0] < v0 + (uint32_t)vj) : ((int)rend[ri - 1] < vj);
    bool first = true, has_head = false;
    int head_row = 0;
    u128 head_acc = u128_zero();
    u128 acc = u128_zero();
    for (int d = dt0; d < dt1; ++d) {
        if (ri < R && (int)rend[ri] <= vj) {
            if (first && partial_first) {
                has_head = true;
                head_row = ri;
                head_acc = acc;
            } else {
                fin(r0 + ri, acc);
            }
            first = false;
            acc = u128_zero();
            ++ri;
        } else {
            acc = u128_add(acc, vsum[vj]);
            ++vj;
        }
    }
    crow[tid] = (uint32_t)ri;
    cacc[tid] = acc;
    __syncthreads();

    if (has_head) {
        u128 tot = head_acc;
        for (int t = tid - 1; t >= 0 && crow[t] == (uint32_t)head_row; --t) tot = u128_add(tot, cacc[t]);
        if (head_row == 0 && head_split) split_contribute<Fused>(a, fin, r0, tot);
        else fin(r0 + head_row, tot);
    }
    // the tile's trailing row continues into later tiles: contribute its in-tile part
    if (items > 0 && dt0 < dt1 && dt1 == items && r1 < a.V && a.rowptr[r1] < v1) {
        u128 tot = u128_zero();
        for (int t = tid; t >= 0 && crow[t] == (uint32_t)R; --t) tot = u128_add(tot, cacc[t]);
        split_contribute<Fused>(a, fin, r1, tot);
    }

    // block reduction of the sum contributions, one exact atomic per tile
    u128 s = fin.ssum;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
    __syncthreads();
    if ((tid & 31) == 0) cacc[tid >> 5] = s;
    __syncthreads();
    if (tid < 32) {
        s = (tid < PR_THREADS / 32) ? cacc[tid] : u128_zero();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
        if (tid == 0 && (s.lo | s.hi)) u128_atomic_add(a.sum_out, s);
    }
}

// perform_vertex_phase_pr over [first, first+count): double accumulators -> props (double and fixed)
__global__ void k_pr_vertex(const double* __restrict__ accum, const double* __restrict__ inv_deg,
                            const uint32_t* __restrict__ degree, double* __restrict__ prop, u128* __restrict__ prop_fx,
                            uint64_t first, uint64_t count, double G, double damping, double c, u128* __restrict__ sum_next)
{
    __shared__ u128 red[PR_THREADS / 32];
    const uint64_t i = (uint64_t)blockIdx.x * PR_THREADS + threadIdx.x;
    u128 s = u128_zero();
    if (i < count) {
        const uint64_t v = first + i;
        double t = __dadd_rn(accum[v], G);
        t = __dmul_rn(t, damping);
        t = __dadd_rn(t, c);
        const double p = __dmul_rn(t, inv_deg[v]);
        prop[v] = p;
        const u128 pf = fx_from_double(p);
        prop_fx[v] = pf;
        s = u128_mul32(pf, degree[v]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < PR_THREADS / 32) ? red[threadIdx.x] : u128_zero();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
        if (threadIdx.x == 0 && sum_next && (s.lo | s.hi)) u128_atomic_add(sum_next, s);
    }
}

// execution_initialize_vertex_prop_pr (source/execution_pr.c:85-88): (1/V) / deg'
__global__ void k_pr_init(const double* __restrict__ outdeg, const uint32_t* __restrict__ degree, uint64_t V,
                          double* __restrict__ prop, double* __restrict__ accum, u128* __restrict__ prop_fx,
                          u128* __restrict__ sum0)
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
        s = u128_mul32(pf, degree[v]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < PR_THREADS / 32) ? red[threadIdx.x] : u128_zero();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
        if (threadIdx.x == 0 && (s.lo | s.hi)) u128_atomic_add(sum0, s);
    }
}

__global__ void k_fx_to_double(const u128* __restrict__ fx, uint64_t V, double* __restrict__ out)
{
    const uint64_t v = (uint64_t)blockIdx.x * PR_THREADS + threadIdx.x;
    if (v < V) out[v] = fx_to_double(fx[v]);
}

PRArgs make_args(grz_graph* g)
{
    PRArgs a;
    a.nbr = g->pull.nbr;
    a.rowptr = g->pull.rowptr;
    a.tile_coord = g->pull.tile_coord;
    a.src_fx = g->pr_fx[g->pr_cur];
    a.dst_fx = g->pr_fx[g->pr_cur ^ 1];
    a.inv_deg = g->inv_deg;
    a.degree = g->degree;
    a.split_acc = g->pr_split_acc;
    a.split_cnt = g->pr_split_cnt;
    a.sum_in = nullptr;
    a.sum_out = nullptr;
    a.sum_clear = nullptr;
    a.accum = g->accum;
    a.prop_out = nullptr;
    a.V = g->V;
    a.nvec = g->pull.nvec;
    a.num_vertices = (double)g->V;
    a.damping = g->pr_damping;
    a.one_minus_d_by_v = (1.0 - g->pr_damping) / (double)g->V;
    return a;
}

unsigned blocks_for(uint64_t n) { return (unsigned)((n + PR_THREADS - 1) / PR_THREADS); }

}  // namespace

extern "C" int grz_pr_tile_items() { return PR_ITEMS; }

int grz_pr_prepare(grz_graph* g)
{
    if (g->pull.tile_coord == nullptr || g->pull.tile_items != (uint32_t)PR_ITEMS) {
        int rc = grz_build_pr_tiles(g, &g->pull, PR_ITEMS);
        if (rc) return rc;
    }
    const uint64_t V = g->V;
    if (!g->pr_fx[0]) {
        GRZ_CK(g, cudaMalloc((void**)&g->pr_fx[0], sizeof(u128) * (V + 1)));
        GRZ_CK(g, cudaMalloc((void**)&g->pr_fx[1], sizeof(u128) * (V + 1)));
        GRZ_CK(g, cudaMalloc((void**)&g->pr_sum, sizeof(u128) * 3));
        GRZ_CK(g, cudaMalloc((void**)&g->pr_split_acc, sizeof(u128) * (V + 1)));
        GRZ_CK(g, cudaMalloc((void**)&g->pr_split_cnt, sizeof(uint32_t) * (V + 1)));
        GRZ_CK(g, cudaMemsetAsync(g->pr_split_acc, 0, sizeof(u128) * (V + 1), g->stream));
        GRZ_CK(g, cudaMemsetAsync(g->pr_split_cnt, 0, sizeof(uint32_t) * (V + 1), g->stream));
    }
    return GRZ_OK;
}

// PageRank initial state (props, zero accumulators, S_0)
int grz_pr_init_state(grz_graph* g, double damping)
{
    int rc = grz_pr_prepare(g);
    if (rc) return rc;
    g->pr_damping = damping;
    g->pr_cur = 0;
    g->pr_sum_cur = 0;
    g->pr_iters_done = 0;
    GRZ_CK(g, cudaMemsetAsync(g->pr_sum, 0, sizeof(u128) * 3, g->stream));
    GRZ_CK(g, cudaMemsetAsync(g->accum, 0, sizeof(double) * (g->V + 8), g->stream));
    if (g->V) {
        k_pr_init<<<blocks_for(g->V), PR_THREADS, 0, g->stream>>>(g->outdeg, g->degree, g->V, g->prop, g->accum, g->pr_fx[0], g->pr_sum);
        GRZ_CK(g, cudaGetLastError());
    }
    return GRZ_OK;
}

// one fused PageRank iteration (edge-pull + vertex phase); launches one kernel
int grz_pr_fused_iteration(grz_graph* g, int write_double_props)
{
    if (g->V == 0) return GRZ_OK;
    PRArgs a = make_args(g);
    const int k = g->pr_sum_cur;
    a.sum_in = g->pr_sum + k;
    a.sum_out = g->pr_sum + (k + 1) % 3;
    a.sum_clear = g->pr_sum + (k + 2) % 3;
    a.prop_out = write_double_props ? g->prop : nullptr;
    k_pr_pull<true><<<g->pull.ntiles, PR_THREADS, 0, g->stream>>>(a);
    GRZ_CK(g, cudaGetLastError());
    g->pr_cur ^= 1;
    g->pr_sum_cur = (k + 1) % 3;
    g->pr_iters_done++;
    return GRZ_OK;
}

// edge-pull phase only: accumulators (double) and their exact sum into g->glob
int grz_pr_edge_pull(grz_graph* g)
{
    if (g->V == 0) return GRZ_OK;
    PRArgs a = make_args(g);
    a.sum_out = g->glob;
    k_pr_pull<false><<<g->pull.ntiles, PR_THREADS, 0, g->stream>>>(a);
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
    // the props being gathered are rewritten in place: the boundary path keeps one live copy
    k_pr_vertex<<<blocks_for(count), PR_THREADS, 0, g->stream>>>(g->accum, g->inv_deg, g->degree, g->prop, g->pr_fx[g->pr_cur],
                                                                 first, count, G, g->pr_damping, c, nullptr);
    GRZ_CK(g, cudaGetLastError());
    return GRZ_OK;
}

// reference-format props (double) from the current fixed-point props
int grz_pr_props_to_double(grz_graph* g)
{
    if (g->V == 0) return GRZ_OK;
    k_fx_to_double<<<blocks_for(g->V), PR_THREADS, 0, g->stream>>>(g->pr_fx[g->pr_cur], g->V, g->prop);
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
        if (threadIdx.x == 0 && (s.lo | s.hi)) u128_atomic_add(glob, s);
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
    // the split-row accumulators double as the push accumulators (zero between uses)
    k_pr_push<<<blocks_for(count), PR_THREADS, 0, g->stream>>>(g->push.nbr, g->push.shared, first_vec, count,
                                                               g->pr_fx[g->pr_cur], g->pr_split_acc, g->glob);
    GRZ_CK(g, cudaGetLastError());
    k_pr_push_accum_out<<<blocks_for(g->V), PR_THREADS, 0, g->stream>>>(g->pr_split_acc, g->accum, 0, g->V);
    GRZ_CK(g, cudaGetLastError());
    return GRZ_OK;
}
