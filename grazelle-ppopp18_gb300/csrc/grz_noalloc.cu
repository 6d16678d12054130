// grz_noalloc.cu -- one PageRank iteration that allocates no device memory.
//
// Some callers cannot call cudaMalloc from the code that runs an iteration.  Examples:
//   - a framework whose own pool owns all device memory;
//   - a latency-bound service loop, where cudaMalloc/cudaFree would synchronise the device;
//   - a sandbox that forbids allocation after start-up.
// For them, grz_pr_step_noalloc takes caller-owned device arrays and keeps its scratch in a
// fixed array compiled into this library.  The scratch is the exact per-destination
// accumulators and the per-block partial sums.  Every GPU that loads the library holds the
// array until the process exits.
//
// The iteration is the reference's perform_edge_pull_phase_pr + perform_vertex_phase_pr
// (source/phase_edge_pull_pr.asm, source/phase_vertex_pr.asm), read directly from the
// reference's 256-bit vectors.  Per-destination sums are exact (u128 fixed point, rounded once
// to double).  The vertex formula has the reference's operation order:
// ((acc + G)*d + (1-d)/V) / deg'.
#include <mutex>

#include "grz_internal.cuh"
#include "../../include/grazelle_gb300.h"

namespace {

constexpr int NA_T = 256;
constexpr unsigned NA_MAX_V = GRZ_NOALLOC_MAX_VERTICES;
constexpr unsigned NA_MAX_PARTS = NA_MAX_V / NA_T + 1;
constexpr int NA_MAX_DEVICES = 64;

// the scratch: u128 accumulator per vertex, u128 partial sum per block of 256 vertices
__device__ __align__(256) u128 g_na_acc[NA_MAX_V + 1];
__device__ __align__(256) u128 g_na_part[NA_MAX_PARTS];

std::mutex g_na_mutex;
u128* g_na_acc_ptr[NA_MAX_DEVICES];
u128* g_na_part_ptr[NA_MAX_DEVICES];

__device__ __forceinline__ u128 na_shfl_up(u128 v, int off)
{
    u128 r;
    r.lo = __shfl_up_sync(0xffffffffu, v.lo, off);
    r.hi = __shfl_up_sync(0xffffffffu, v.hi, off);
    return r;
}

// one thread per 256-bit vector: decode it (graphdata.c:114-120), sum the valid lanes' props
// exactly, sum per destination within the warp, add each warp's per-destination sum atomically
__global__ void __launch_bounds__(NA_T) k_na_gather(const ulonglong2* __restrict__ vecs, uint64_t nvec, uint32_t V,
                                                    const double* __restrict__ props, u128* __restrict__ acc)
{
    const uint64_t i = (uint64_t)blockIdx.x * NA_T + threadIdx.x;
    const int lane = threadIdx.x & 31;
    uint32_t key = 0xffffffffu;
    u128 val = u128_zero();
    if (i < nvec) {
        const ulonglong2 a = vecs[2 * i], b = vecs[2 * i + 1];
        const unsigned long long w[4] = { a.x, a.y, b.x, b.y };
        const unsigned long long d = ((w[0] & 0x7fff000000000000ull) >> 48) | ((w[1] & 0x7fff000000000000ull) >> 33) |
                                     ((w[2] & 0x7fff000000000000ull) >> 18) | ((w[3] & 0x0007000000000000ull) >> 3);
        if (d < V) {
            key = (uint32_t)d;
            u128 g[4];
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const unsigned long long s = w[l] & 0x0000ffffffffffffull;
                g[l] = ((w[l] >> 63) && s < V) ? fx_from_double(__ldg(props + s)) : u128_zero();
            }
            val = u128_add(u128_add(g[2], g[3]), u128_add(g[0], g[1]));
        }
    }
    const uint32_t prevkey = __shfl_up_sync(0xffffffffu, key, 1);
    const uint32_t nextkey = __shfl_down_sync(0xffffffffu, key, 1);
    const bool head = lane == 0 || key != prevkey;
    const bool tail = lane == 31 || key != nextkey;
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const int segstart = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
    for (int off = 1; off < 32; off <<= 1) {
        const u128 o = na_shfl_up(val, off);
        if (lane - off >= segstart) val = u128_add(val, o);
    }
    if (tail && key != 0xffffffffu && (val.lo | val.hi)) u128_atomic_add(acc + key, val);
}

// per-block partial sums of the accumulators (S = sum of all accumulators)
__global__ void __launch_bounds__(NA_T) k_na_partials(const u128* __restrict__ acc, uint32_t V, u128* __restrict__ part)
{
    __shared__ u128 red[NA_T / 32];
    const uint32_t v = blockIdx.x * NA_T + threadIdx.x;
    u128 s = v < V ? acc[v] : u128_zero();
    for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < NA_T / 32) ? red[threadIdx.x] : u128_zero();
        for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
        if (threadIdx.x == 0) part[blockIdx.x] = s;
    }
}

// vertex phase: G = (1 - S)/V; prop = ((acc + G)*d + (1-d)/V) / deg'
__global__ void __launch_bounds__(NA_T) k_na_apply(const u128* __restrict__ acc, uint32_t V, const u128* __restrict__ part,
                                                   uint32_t nparts, const double* __restrict__ outdeg, double damping,
                                                   double* __restrict__ props_out)
{
    __shared__ double sG;
    if (threadIdx.x < 32) {
        u128 s = u128_zero();
        for (uint32_t b = threadIdx.x; b < nparts; b += 32) s = u128_add(s, part[b]);
        for (int o = 16; o > 0; o >>= 1) s = u128_add(s, u128_shfl_down(s, o));
        if (threadIdx.x == 0) sG = (1.0 - fx_to_double(s)) / (double)V;
    }
    __syncthreads();
    const uint32_t v = blockIdx.x * NA_T + threadIdx.x;
    if (v >= V) return;
    const double dV = (double)V;
    const double c = (1.0 - damping) / dV;
    const double od = outdeg[v];
    double t = __dadd_rn(fx_to_double(acc[v]), sG);
    t = __dmul_rn(t, damping);
    t = __dadd_rn(t, c);
    props_out[v] = __ddiv_rn(t, od == 0.0 ? dV : od);
}

// Resolves the device addresses of the scratch arrays for the current device, once per device.
// The addresses are kept for the life of the process: a caller that resets the device
// (cudaDeviceReset) and then calls again is not supported.
int na_setup(int dev, u128** acc, u128** part)
{
    std::lock_guard<std::mutex> lk(g_na_mutex);
    if (!g_na_acc_ptr[dev]) {
        void* p = nullptr;
        void* q = nullptr;
        if (cudaGetSymbolAddress(&p, g_na_acc) != cudaSuccess || cudaGetSymbolAddress(&q, g_na_part) != cudaSuccess) {
            cudaGetLastError();
            return GRZ_ERR_CUDA;
        }
        g_na_acc_ptr[dev] = (u128*)p;
        g_na_part_ptr[dev] = (u128*)q;
    }
    *acc = g_na_acc_ptr[dev];
    *part = g_na_part_ptr[dev];
    return GRZ_OK;
}

}  // namespace

extern "C" int grz_pr_step_noalloc(const void* vectors, uint64_t num_vectors, uint64_t num_vertices, const double* props_in,
                                   const double* outdeg, double damping, double* props_out, void* stream)
{
    if (num_vertices == 0 || num_vertices > NA_MAX_V) return GRZ_ERR_RANGE;
    if (!vectors || num_vectors == 0 || num_vectors > 0xffffffffull || !props_in || !outdeg || !props_out) return GRZ_ERR_ARG;
    if (!(damping >= 0.0 && damping <= 1.0)) return GRZ_ERR_ARG;
    if (((uintptr_t)vectors & 31) != 0) return GRZ_ERR_ARG;
    // props_out is written while other blocks still gather props_in: the two ranges must not overlap
    const uintptr_t in0 = (uintptr_t)props_in, out0 = (uintptr_t)props_out, nb = (uintptr_t)(sizeof(double) * num_vertices);
    if (in0 < out0 + nb && out0 < in0 + nb) return GRZ_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) {
        cudaGetLastError();
        return GRZ_ERR_CUDA;
    }
    u128 *acc = nullptr, *part = nullptr;
    int rc = na_setup(dev, &acc, &part);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t V = (uint32_t)num_vertices;
    const uint32_t nparts = (V + NA_T - 1) / NA_T;
    // the accumulators must start at zero; the array keeps the last call's contents
    if (cudaMemsetAsync(acc, 0, sizeof(u128) * (V + 1), st) != cudaSuccess) {
        cudaGetLastError();
        return GRZ_ERR_CUDA;
    }
    k_na_gather<<<(unsigned)((num_vectors + NA_T - 1) / NA_T), NA_T, 0, st>>>((const ulonglong2*)vectors, num_vectors, V,
                                                                              props_in, acc);
    k_na_partials<<<nparts, NA_T, 0, st>>>(acc, V, part);
    k_na_apply<<<nparts, NA_T, 0, st>>>(acc, V, part, nparts, outdeg, damping, props_out);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GRZ_OK : GRZ_ERR_CUDA;
}

extern "C" uint64_t grz_pr_step_noalloc_max_vertices(void) { return NA_MAX_V; }
