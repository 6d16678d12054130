// grz_switch.cu -- the learned push/pull engine switch for CC and BFS.
//
// The reference picks the engine by a threshold on the vote: pull iff vote > E/5
// (source/execution_bfs.c:146-168, execution_cc.c:120-142).  That rule was tuned for CPUs.
// On a GB300 the push engine runs on a compacted frontier and the crossover lies elsewhere.
// Here a small MLP (GRZ_NFEAT -> 32 -> 32 -> 1, FP32) predicts, before each iteration, whether
// pull will be faster than push.  It learns from per-iteration timings of both engines, taken
// from the same state (snapshot / restore).  The threshold stays as the fallback and as the
// yardstick.  Results do not depend on the choice: CC labels and BFS levels are the same
// either way; only time changes.
//
// Kernels (all hand-written):
//   k_features_decide  grid-wide popcounts of HasInfo* and WantsInfo; the last block computes
//                      the features (those counts, the vote, degree statistics) and, in one
//                      warp, the MLP forward pass for that single sample -> the next engine
//   k_mlp_fwd_bwd      one thread per training sample: forward, weighted binary
//                      cross-entropy, backward; per-block gradient sums in shared memory
//   k_mlp_reduce_adam  sum of the per-block partials in block order, and an Adam step
#include <math.h>
#include <string.h>

#include <algorithm>

#include "grz_internal.cuh"
#include "../../include/grazelle_gb300.h"

#define NF GRZ_MLP_FEATURES
#define NH GRZ_MLP_HIDDEN

namespace {

constexpr int T = 256;
// parameter layout (floats): W1[NH][NF] b1[NH] W2[NH][NH] b2[NH] W3[NH] b3
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + NH * NF;
constexpr int OFF_W2 = OFF_B1 + NH;
constexpr int OFF_B2 = OFF_W2 + NH * NH;
constexpr int OFF_W3 = OFF_B2 + NH;
constexpr int OFF_B3 = OFF_W3 + NH;
constexpr int NP = OFF_B3 + 1;
static_assert(NP == GRZ_MLP_PARAMS, "parameter count");

__device__ __forceinline__ float relu(float x) { return x > 0.f ? x : 0.f; }

// forward of one sample: returns the logit (pull faster) and the hidden activations
__device__ __forceinline__ float mlp_forward(const float* p, const float* x, float* h1, float* h2)
{
    for (int j = 0; j < NH; ++j) {
        float s = p[OFF_B1 + j];
        for (int k = 0; k < NF; ++k) s = fmaf(p[OFF_W1 + j * NF + k], x[k], s);
        h1[j] = relu(s);
    }
    for (int j = 0; j < NH; ++j) {
        float s = p[OFF_B2 + j];
        for (int k = 0; k < NH; ++k) s = fmaf(p[OFF_W2 + j * NH + k], h1[k], s);
        h2[j] = relu(s);
    }
    float z = p[OFF_B3];
    for (int k = 0; k < NH; ++k) z = fmaf(p[OFF_W3 + k], h2[k], z);
    return z;
}

// features of the state the next iteration will start from (computed before the frontier swap:
// has_next is the next HasInfo)
struct FeatIn {
    const unsigned long long* frontier;
    unsigned long long vote_override;  // ~0: read the vote slots
    const unsigned long long* wants;
    const unsigned long long* vote_slots;
    uint64_t words;
    double V, E, max_degree;
    uint32_t iter;
    int app_bfs;
    int last_engine;
};

// sw_out layout (u64): [0] vote, [1] decision, [2] |frontier|, [3] |WantsInfo|, [4] block
// ticket, then NF floats.  Words 2-4 are zero between calls.
constexpr int SW_U64 = 5;

// MLP forward pass of one sample by one warp, lane j computing hidden unit j.  Same operation
// order as mlp_forward, so the logit equals grz_mlp_predict's.  f: NF features, h: NH scratch
// (both shared); every lane returns the logit.
// One warp, lane j = hidden unit j, the weights in registers: lane j loads its own rows of W1 and
// W2 straight from global memory (all loads issued together, one L2 round trip), and the hidden
// activations pass between lanes by shuffles.  The operation order is mlp_forward's, so the
// logit equals grz_mlp_predict's bit for bit.
__device__ float mlp_logit_warp(const float* __restrict__ params, const float* f, int lane)
{
    float w1[NF], w2[NH];
#pragma unroll
    for (int k = 0; k < NF; ++k) w1[k] = __ldg(params + OFF_W1 + lane * NF + k);
#pragma unroll
    for (int k = 0; k < NH; ++k) w2[k] = __ldg(params + OFF_W2 + lane * NH + k);
    const float b1 = __ldg(params + OFF_B1 + lane), b2 = __ldg(params + OFF_B2 + lane);
    const float w3 = __ldg(params + OFF_W3 + lane), b3 = __ldg(params + OFF_B3);
    float s = b1;
#pragma unroll
    for (int k = 0; k < NF; ++k) s = fmaf(w1[k], f[k], s);
    const float h1 = relu(s);
    s = b2;
#pragma unroll
    for (int k = 0; k < NH; ++k) s = fmaf(w2[k], __shfl_sync(0xffffffffu, h1, k), s);
    const float h2 = relu(s);
    float z = b3;
#pragma unroll
    for (int k = 0; k < NH; ++k) z = fmaf(__shfl_sync(0xffffffffu, w3, k), __shfl_sync(0xffffffffu, h2, k), z);
    return z;
}

// feature k of the state (lane k computes it)
__device__ float feature(int k, const FeatIn& in, float F, float U, float vote)
{
    const float V = (float)in.V, E = (float)in.E;
    switch (k) {
    case 0: return log2f(F + 1.f) / log2f(V + 1.f);
    case 1: return F / V;
    case 2: return vote / E;
    case 3: return log2f(vote + 1.f) / log2f(E + 1.f);
    case 4: return in.app_bfs ? U / V : 0.f;
    case 5: return (float)in.iter / 32.f;
    case 6: return log2f(E / V + 1.f) / 8.f;
    case 7: return log2f(V) / 32.f;
    case 8: return log2f((float)in.max_degree + 1.f) / log2f(E + 1.f);
    case 9: return in.app_bfs ? 1.f : 0.f;
    case 10: return in.last_engine ? 1.f : 0.f;
    default: return log2f(F + 1.f) / 32.f;
    }
}

// One launch: grid-wide popcounts of the frontier bitmap and (BFS) WantsInfo; the last block
// to finish then computes the features, the vote (sum of the vote slots) and, with one warp,
// the MLP forward pass for that sample (lane j = hidden unit j; the same operation order as
// mlp_forward, so the logit equals grz_mlp_predict's).  out[0] = vote, out[1] = decision
// (1 pull / 0 push), features after the SW_U64 words.  The last block re-zeroes words 2-4.
__global__ void __launch_bounds__(T) k_features_decide(FeatIn in, const float* __restrict__ params, int use_mlp,
                                                       double threshold, unsigned long long* __restrict__ out)
{
    __shared__ unsigned s_pf[T / 32], s_pw[T / 32];
    __shared__ bool s_last;
    __shared__ float f[NF];
    unsigned pf = 0, pw = 0;
    for (uint64_t w = (uint64_t)blockIdx.x * T + threadIdx.x; w < in.words; w += (uint64_t)gridDim.x * T) {
        pf += __popcll(in.frontier[w]);
        if (in.app_bfs) pw += __popcll(in.wants[w]);
    }
    pf = __reduce_add_sync(0xffffffffu, pf);
    pw = __reduce_add_sync(0xffffffffu, pw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { s_pf[warp] = pf; s_pw[warp] = pw; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long bf = 0, bw = 0;
        for (int i = 0; i < T / 32; ++i) { bf += s_pf[i]; bw += s_pw[i]; }
        if (bf) atomicAdd(out + 2, bf);
        if (bw) atomicAdd(out + 3, bw);
        __threadfence();
        s_last = atomicAdd(out + 4, 1ull) == (unsigned long long)(gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last || warp != 0) return;
    __threadfence();
    const unsigned long long F = *(volatile unsigned long long*)(out + 2);
    const unsigned long long U = *(volatile unsigned long long*)(out + 3);
    unsigned long long vote = in.vote_override;
    if (vote == ~0ull) {
        unsigned long long vs = in.vote_slots[lane * GRZ_VOTE_STRIDE] + in.vote_slots[(lane + 32) * GRZ_VOTE_STRIDE];
        for (int o = 16; o > 0; o >>= 1) vs += __shfl_down_sync(0xffffffffu, vs, o);
        vote = __shfl_sync(0xffffffffu, vs, 0);
    }
    if (lane < NF) f[lane] = feature(lane, in, (float)F, (float)U, (float)vote);
    __syncwarp();
    int pull;
    if (use_mlp) {
        pull = mlp_logit_warp(params, f, lane) > 0.f ? 1 : 0;
    } else {
        pull = (double)vote > threshold ? 1 : 0;
    }
    if (lane < NF) ((float*)(out + SW_U64))[lane] = f[lane];
    if (lane == 0) {
        out[0] = vote;
        out[1] = (unsigned long long)pull;
        out[2] = 0;
        out[3] = 0;
        out[4] = 0;
    }
}

// The decision at the end of an iteration of a CC/BFS run executed as one CUDA graph.
// Grid-wide: popcounts of the next frontier and WantsInfo; clears the old HasInfo (the
// reference's vertex phase after the pointer swap, source/phase_vertex_cc.asm:37-46).  The
// last block: the vote (sum of the slots, which it re-zeroes), convergence (vote 0), the
// iteration bound, the run statistics, the next engine (forced, threshold or MLP), and the
// graph's conditional handles: hpull / hpush select the next iteration's engine body, hloop
// keeps the WHILE node going.  `initial`: the decision before the first iteration, from the
// starting vote; no statistics, no clearing.
struct RunIn {
    FeatIn feat;                        // frontier = the next HasInfo
    unsigned long long* vote_slots;     // read and re-zeroed
    unsigned long long* clear_bm;       // old HasInfo (null when initial)
    int initial;
};

__global__ void __launch_bounds__(T) k_run_decide(RunIn in, grz_runctl* __restrict__ ctl, cudaGraphConditionalHandle hloop,
                                                  cudaGraphConditionalHandle hpull, cudaGraphConditionalHandle hpush)
{
    __shared__ unsigned s_pf[T / 32], s_pw[T / 32];
    __shared__ bool s_last;
    __shared__ float f[NF];
    if (!in.initial && !*(volatile uint32_t*)&ctl->running) return;
    const FeatIn& fi = in.feat;
    const float* params = ctl->params;
    unsigned pf = 0, pw = 0;
    for (uint64_t w = (uint64_t)blockIdx.x * T + threadIdx.x; w < fi.words; w += (uint64_t)gridDim.x * T) {
        pf += __popcll(fi.frontier[w]);
        if (fi.app_bfs) pw += __popcll(fi.wants[w]);
        if (in.clear_bm) in.clear_bm[w] = 0ull;
    }
    pf = __reduce_add_sync(0xffffffffu, pf);
    pw = __reduce_add_sync(0xffffffffu, pw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { s_pf[warp] = pf; s_pw[warp] = pw; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long bf = 0, bw = 0;
        for (int i = 0; i < T / 32; ++i) { bf += s_pf[i]; bw += s_pw[i]; }
        if (bf) atomicAdd(&ctl->cnt_f, bf);
        if (bw) atomicAdd(&ctl->cnt_u, bw);
        __threadfence();
        s_last = atomicAdd(&ctl->ticket, 1ull) == (unsigned long long)(gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last || warp != 0) return;
    __threadfence();
    const unsigned long long F = *(volatile unsigned long long*)&ctl->cnt_f;
    const unsigned long long U = *(volatile unsigned long long*)&ctl->cnt_u;
    unsigned long long vote = ctl->vote;  // initial: the starting vote, written by the host
    if (!in.initial) {
        unsigned long long* a = in.vote_slots + lane * GRZ_VOTE_STRIDE;
        unsigned long long* b = in.vote_slots + (lane + 32) * GRZ_VOTE_STRIDE;
        unsigned long long vs = *(volatile unsigned long long*)a + *(volatile unsigned long long*)b;
        *a = 0ull;
        *b = 0ull;
        for (int o = 16; o > 0; o >>= 1) vs += __shfl_down_sync(0xffffffffu, vs, o);
        vote = __shfl_sync(0xffffffffu, vs, 0);
    }
    uint32_t level = ctl->level;
    const uint32_t ran = ctl->engine;
    uint32_t last_engine = ctl->last_engine;
    uint32_t running = 1, overrun = 0;
    unsigned long long now;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
    if (!in.initial) {
        last_engine = ran;
        running = vote != 0ull;
        if (running) {
            ++level;
            if (level > ctl->max_level) { running = 0; overrun = 1; }
            if (now - ctl->t0_ns > ctl->limit_ns) { running = 0; overrun = 2; }
        }
    }
    FeatIn fe = fi;
    fe.iter = level;
    fe.last_engine = (int)last_engine;
    if (lane < NF) f[lane] = feature(lane, fe, (float)F, (float)U, (float)vote);
    __syncwarp();
    int pull;
    if (ctl->force >= 0) {
        pull = ctl->force;
    } else if (!running) {
        pull = 0;  // the loop stops: no next engine to choose
    } else if (params) {
        pull = mlp_logit_warp(params, f, lane) > 0.f ? 1 : 0;
    } else {
        pull = (double)vote > ctl->threshold ? 1 : 0;
    }
    if (lane < NF) ctl->features[lane] = f[lane];
    if (lane == 0) {
        if (!in.initial) {
            if (ran) ctl->npull += 1; else ctl->npush += 1;
        }
        if (in.initial) ctl->t0_ns = now;
        ctl->vote = vote;
        ctl->running = running;
        ctl->engine = (uint32_t)pull;
        ctl->level = level;
        ctl->last_engine = last_engine;
        ctl->overrun |= overrun;
        ctl->cnt_f = 0ull;
        ctl->cnt_u = 0ull;
        ctl->ticket = 0ull;
        cudaGraphSetConditional(hpull, running && pull ? 1u : 0u);
        cudaGraphSetConditional(hpush, running && !pull ? 1u : 0u);
        cudaGraphSetConditional(hloop, running);
    }
}

// Forward + backward of weighted binary cross-entropy on logits, one thread per sample.  Each
// block leaves its gradient sum (and loss sum) in part[block][0..NP] for a fixed-order reduction.
__global__ void __launch_bounds__(T) k_mlp_fwd_bwd(const float* __restrict__ params, const float* __restrict__ X,
                                                   const float* __restrict__ Y, const float* __restrict__ Wt, uint32_t n,
                                                   float* __restrict__ part, float* __restrict__ logits_out)
{
    __shared__ float sp[NP];
    __shared__ float sg[NP + 1];
    for (int i = threadIdx.x; i < NP; i += T) { sp[i] = params[i]; sg[i] = 0.f; }
    if (threadIdx.x == 0) sg[NP] = 0.f;
    __syncthreads();
    const uint32_t s = blockIdx.x * T + threadIdx.x;
    if (s < n) {
        float x[NF], h1[NH], h2[NH];
        for (int k = 0; k < NF; ++k) x[k] = X[(size_t)s * NF + k];
        const float z = mlp_forward(sp, x, h1, h2);
        if (logits_out) logits_out[s] = z;
        const float y = Y[s], w = Wt[s];
        // loss = w * (softplus(z) - y z); dL/dz = w * (sigmoid(z) - y)
        const float sig = 1.f / (1.f + expf(-z));
        const float sp_z = z > 0.f ? z + log1pf(expf(-z)) : log1pf(expf(z));
        atomicAdd(&sg[NP], w * (sp_z - y * z));
        const float dz = w * (sig - y);
        atomicAdd(&sg[OFF_B3], dz);
        float dh2[NH];
        for (int k = 0; k < NH; ++k) {
            atomicAdd(&sg[OFF_W3 + k], dz * h2[k]);
            dh2[k] = h2[k] > 0.f ? dz * sp[OFF_W3 + k] : 0.f;
        }
        float dh1[NH];
        for (int k = 0; k < NH; ++k) dh1[k] = 0.f;
        for (int j = 0; j < NH; ++j) {
            if (dh2[j] == 0.f) continue;
            atomicAdd(&sg[OFF_B2 + j], dh2[j]);
            for (int k = 0; k < NH; ++k) {
                atomicAdd(&sg[OFF_W2 + j * NH + k], dh2[j] * h1[k]);
                dh1[k] = fmaf(dh2[j], sp[OFF_W2 + j * NH + k], dh1[k]);
            }
        }
        for (int j = 0; j < NH; ++j) {
            if (!(h1[j] > 0.f) || dh1[j] == 0.f) continue;
            atomicAdd(&sg[OFF_B1 + j], dh1[j]);
            for (int k = 0; k < NF; ++k) atomicAdd(&sg[OFF_W1 + j * NF + k], dh1[j] * x[k]);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i <= NP; i += T) part[(size_t)blockIdx.x * (NP + 1) + i] = sg[i];
}

// grad[i] = sum over blocks in block order / n; loss likewise; then Adam
__global__ void k_mlp_reduce_adam(const float* __restrict__ part, uint32_t nblocks, uint32_t n, float* __restrict__ grad,
                                  float* __restrict__ params, float* __restrict__ m, float* __restrict__ v, float lr, int step,
                                  int apply)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > NP) return;
    float s = 0.f;
    for (uint32_t b = 0; b < nblocks; ++b) s += part[(size_t)b * (NP + 1) + i];
    s /= (float)n;
    grad[i] = s;
    if (!apply || i == NP) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    m[i] = b1 * m[i] + (1.f - b1) * s;
    v[i] = b2 * v[i] + (1.f - b2) * s * s;
    const float mh = m[i] / (1.f - powf(b1, (float)step));
    const float vh = v[i] / (1.f - powf(b2, (float)step));
    params[i] -= lr * mh / (sqrtf(vh) + eps);
}

}  // namespace

// ---------------------------------------------------------------------------------------------

struct grz_mlp {
    int device;
    float* params;   // device, NP
    float* m;
    float* v;
    float* grad;     // NP + 1 (last = loss)
    int step;
};

static int mlp_ck(cudaError_t e)
{
    if (e == cudaSuccess) return GRZ_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? GRZ_ERR_NOMEM : GRZ_ERR_CUDA;
}

extern "C" int grz_mlp_create(grz_mlp** out, int device, uint64_t seed)
{
    if (!out) return GRZ_ERR_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return GRZ_ERR_CUDA; }
    grz_mlp* n = (grz_mlp*)calloc(1, sizeof(grz_mlp));
    if (!n) return GRZ_ERR_NOMEM;
    n->device = device;
    int rc = mlp_ck(cudaMalloc((void**)&n->params, sizeof(float) * NP));
    if (!rc) rc = mlp_ck(cudaMalloc((void**)&n->m, sizeof(float) * NP));
    if (!rc) rc = mlp_ck(cudaMalloc((void**)&n->v, sizeof(float) * NP));
    if (!rc) rc = mlp_ck(cudaMalloc((void**)&n->grad, sizeof(float) * (NP + 1)));
    if (rc) { grz_mlp_destroy(n); return rc; }
    // He-uniform initialisation from a splitmix64 stream; zero biases
    float h[NP];
    uint64_t x = seed * 0x9E3779B97F4A7C15ull + 1;
    for (int i = 0; i < NP; ++i) {
        x += 0x9E3779B97F4A7C15ull;
        uint64_t z = x;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        const float u = (float)((z >> 40) * (1.0 / 16777216.0)) * 2.f - 1.f;
        const int fan_in = i < OFF_B1 ? NF : (i < OFF_W2 ? 0 : (i < OFF_B2 ? NH : (i < OFF_W3 ? 0 : (i < OFF_B3 ? NH : 0))));
        h[i] = fan_in ? u * sqrtf(6.f / (float)fan_in) : 0.f;
    }
    rc = mlp_ck(cudaMemcpy(n->params, h, sizeof(h), cudaMemcpyHostToDevice));
    if (!rc) rc = mlp_ck(cudaMemset(n->m, 0, sizeof(float) * NP));
    if (!rc) rc = mlp_ck(cudaMemset(n->v, 0, sizeof(float) * NP));
    if (rc) { grz_mlp_destroy(n); return rc; }
    *out = n;
    return GRZ_OK;
}

extern "C" void grz_mlp_destroy(grz_mlp* n)
{
    if (!n) return;
    cudaFree(n->params);
    cudaFree(n->m);
    cudaFree(n->v);
    cudaFree(n->grad);
    free(n);
}

extern "C" int grz_mlp_get_params(grz_mlp* n, float* host, uint64_t cap)
{
    if (!n || !host || cap < (uint64_t)NP) return GRZ_ERR_ARG;
    return mlp_ck(cudaMemcpy(host, n->params, sizeof(float) * NP, cudaMemcpyDeviceToHost));
}

extern "C" int grz_mlp_set_params(grz_mlp* n, const float* host, uint64_t count)
{
    if (!n || !host || count != (uint64_t)NP) return GRZ_ERR_ARG;
    n->step = 0;
    int rc = mlp_ck(cudaMemcpy(n->params, host, sizeof(float) * NP, cudaMemcpyHostToDevice));
    if (!rc) rc = mlp_ck(cudaMemset(n->m, 0, sizeof(float) * NP));
    if (!rc) rc = mlp_ck(cudaMemset(n->v, 0, sizeof(float) * NP));
    return rc;
}

// one pass over a host dataset: forward/backward, gradients (and loss) to host; optional Adam step
static int mlp_pass(grz_mlp* n, const float* X, const float* Y, const float* W, uint64_t count, float lr, int apply,
                    float* grads_out, float* loss_out, float* logits_out)
{
    if (!n || !X || !Y || !W || count == 0 || count > 0x7fffffffull) return GRZ_ERR_ARG;
    if (cudaSetDevice(n->device) != cudaSuccess) { cudaGetLastError(); return GRZ_ERR_CUDA; }
    const uint32_t nb = (uint32_t)((count + T - 1) / T);
    float *dX = nullptr, *dY = nullptr, *dW = nullptr, *dpart = nullptr, *dlog = nullptr;
    int rc = mlp_ck(cudaMalloc((void**)&dX, sizeof(float) * NF * count));
    if (!rc) rc = mlp_ck(cudaMalloc((void**)&dY, sizeof(float) * count));
    if (!rc) rc = mlp_ck(cudaMalloc((void**)&dW, sizeof(float) * count));
    if (!rc) rc = mlp_ck(cudaMalloc((void**)&dpart, sizeof(float) * (NP + 1) * nb));
    if (!rc && logits_out) rc = mlp_ck(cudaMalloc((void**)&dlog, sizeof(float) * count));
    if (!rc) rc = mlp_ck(cudaMemcpy(dX, X, sizeof(float) * NF * count, cudaMemcpyHostToDevice));
    if (!rc) rc = mlp_ck(cudaMemcpy(dY, Y, sizeof(float) * count, cudaMemcpyHostToDevice));
    if (!rc) rc = mlp_ck(cudaMemcpy(dW, W, sizeof(float) * count, cudaMemcpyHostToDevice));
    if (!rc) {
        if (apply) n->step++;
        k_mlp_fwd_bwd<<<nb, T>>>(n->params, dX, dY, dW, (uint32_t)count, dpart, dlog);
        k_mlp_reduce_adam<<<(NP + 1 + 127) / 128, 128>>>(dpart, nb, (uint32_t)count, n->grad, n->params, n->m, n->v, lr,
                                                         n->step, apply);
        rc = mlp_ck(cudaGetLastError());
    }
    float g[NP + 1];
    if (!rc) rc = mlp_ck(cudaMemcpy(g, n->grad, sizeof(g), cudaMemcpyDeviceToHost));
    if (!rc && grads_out) memcpy(grads_out, g, sizeof(float) * NP);
    if (!rc && loss_out) *loss_out = g[NP];
    if (!rc && logits_out) rc = mlp_ck(cudaMemcpy(logits_out, dlog, sizeof(float) * count, cudaMemcpyDeviceToHost));
    cudaFree(dX);
    cudaFree(dY);
    cudaFree(dW);
    cudaFree(dpart);
    cudaFree(dlog);
    return rc;
}

extern "C" int grz_mlp_gradients(grz_mlp* n, const float* X, const float* Y, const float* W, uint64_t count, float* grads,
                                 float* loss)
{
    return mlp_pass(n, X, Y, W, count, 0.f, 0, grads, loss, nullptr);
}

extern "C" int grz_mlp_predict(grz_mlp* n, const float* X, uint64_t count, float* logits)
{
    if (!X || !logits || count == 0) return GRZ_ERR_ARG;
    float* zeros = (float*)calloc(count, sizeof(float));
    if (!zeros) return GRZ_ERR_NOMEM;
    const int rc = mlp_pass(n, X, zeros, zeros, count, 0.f, 0, nullptr, nullptr, logits);
    free(zeros);
    return rc;
}

extern "C" int grz_mlp_train(grz_mlp* n, const float* X, const float* Y, const float* W, uint64_t count, uint32_t epochs,
                             float lr, float* final_loss)
{
    int rc = GRZ_OK;
    for (uint32_t e = 0; e < epochs && rc == GRZ_OK; ++e) rc = mlp_pass(n, X, Y, W, count, lr, 1, nullptr, final_loss, nullptr);
    return rc;
}

// ---------------------------------------------------------------------------------------------
// engine policy inside the CC/BFS step

__global__ void __launch_bounds__(T) k_max_u32(const uint32_t* __restrict__ a, uint64_t n, unsigned* __restrict__ out)
{
    unsigned m = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * T + threadIdx.x; i < n; i += (uint64_t)gridDim.x * T) m = max(m, a[i]);
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

// the largest degree (a feature), computed once per loaded graph
int grz_switch_max_degree(grz_graph* g)
{
    if (g->max_degree_known) return GRZ_OK;
    int rc = grz_frontier_mail(g);
    if (rc) return rc;
    unsigned* d = nullptr;
    GRZ_CK(g, cudaMallocAsync((void**)&d, sizeof(unsigned), g->stream));
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(unsigned), g->stream);
    if (e == cudaSuccess && g->V) {
        const unsigned grid = (unsigned)std::min<uint64_t>((g->V + T - 1) / T, (uint64_t)g->num_sms * 4);
        k_max_u32<<<grid, T, 0, g->stream>>>(g->degree, g->V, d); GRZ_COUNT_LAUNCH(g);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(g->fr.mail, d, sizeof(unsigned), cudaMemcpyDeviceToHost, g->stream);
    cudaFreeAsync(d, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return grz_cuda_check(g, e, "max degree");
    g->max_degree = *(const unsigned*)g->fr.mail;
    g->max_degree_known = 1;
    return GRZ_OK;
}

int grz_switch_decide(grz_graph* g, const unsigned long long* frontier, uint64_t vote_override, uint32_t iter,
                      uint64_t* vote, int* next_pull, float* features)
{
    grz_frontier_state& f = g->fr;
    if (!f.sw_out) {
        GRZ_CK(g, cudaMalloc((void**)&f.sw_out, sizeof(unsigned long long) * SW_U64 + sizeof(float) * NF));
        GRZ_CK(g, cudaMemsetAsync(f.sw_out, 0, sizeof(unsigned long long) * SW_U64, g->stream));
    }
    int rc = grz_frontier_mail(g);
    if (!rc) rc = grz_switch_max_degree(g);
    if (rc) return rc;
    FeatIn in;
    in.frontier = frontier;
    in.vote_override = vote_override;
    in.wants = f.wants;
    in.vote_slots = f.vote;
    in.words = (g->V >> 6) + 2;
    in.V = (double)(g->V ? g->V : 1);
    in.E = (double)(g->E ? g->E : 1);
    in.max_degree = (double)g->max_degree;
    in.iter = iter;
    in.app_bfs = f.app == GRZ_APP_BREADTH_FIRST_SEARCH;
    in.last_engine = f.last_engine;
    const int use_mlp = f.policy == GRZ_POLICY_LEARNED && f.mlp;
    const double thr = (f.flags & GRZ_FLAG_WITHOUT_OUTDEG) ? (double)(g->V / 2) : (double)(g->E / 5);
    unsigned long long* out = (unsigned long long*)f.sw_out;
    const unsigned grid = (unsigned)std::min<uint64_t>((in.words + T - 1) / T, (uint64_t)g->num_sms * 2);
    k_features_decide<<<grid, T, 0, g->stream>>>(in, use_mlp ? f.mlp->params : nullptr, use_mlp, thr, out); GRZ_COUNT_LAUNCH(g);
    GRZ_CK(g, cudaGetLastError());
    const size_t bytes = sizeof(unsigned long long) * SW_U64 + sizeof(float) * NF;
    GRZ_CK(g, cudaMemcpyAsync(f.mail, f.sw_out, bytes, cudaMemcpyDeviceToHost, g->stream));
    GRZ_CK(g, cudaStreamSynchronize(g->stream));
    const unsigned char* host = (const unsigned char*)f.mail;
    unsigned long long o[SW_U64];
    memcpy(o, host, sizeof(o));
    *vote = o[0];
    *next_pull = (int)o[1];
    if (features) memcpy(features, host + sizeof(o), sizeof(float) * NF);
    return GRZ_OK;
}

// Launches k_run_decide on the graph's stream (called while capturing the run graph).  The
// policy is not captured: the host writes it into the control block before each launch.
int grz_switch_launch_run_decide(grz_graph* g, const unsigned long long* next_frontier, unsigned long long* clear_bm, int initial,
                                 unsigned long long hloop, unsigned long long hpull, unsigned long long hpush)
{
    grz_frontier_state& f = g->fr;
    RunIn in;
    memset(&in, 0, sizeof(in));
    in.feat.frontier = next_frontier;
    in.feat.vote_override = 0;
    in.feat.wants = f.wants;
    in.feat.vote_slots = f.vote;
    in.feat.words = (g->V >> 6) + 2;
    in.feat.V = (double)(g->V ? g->V : 1);
    in.feat.E = (double)(g->E ? g->E : 1);
    in.feat.max_degree = (double)g->max_degree;
    in.feat.app_bfs = f.app == GRZ_APP_BREADTH_FIRST_SEARCH;
    in.vote_slots = f.vote;
    in.clear_bm = clear_bm;
    in.initial = initial;
    const unsigned grid = (unsigned)std::min<uint64_t>((in.feat.words + T - 1) / T, (uint64_t)g->num_sms * 2);
    k_run_decide<<<grid, T, 0, g->stream>>>(in, f.ctl, hloop, hpull, hpush);
    return grz_cuda_check(g, cudaGetLastError(), "run decision");
}

extern "C" int grz_frontier_set_policy(grz_graph* g, int policy, grz_mlp* mlp)
{
    if (!g || (policy != GRZ_POLICY_THRESHOLD && policy != GRZ_POLICY_LEARNED) || (policy == GRZ_POLICY_LEARNED && !mlp))
        return GRZ_ERR_ARG;
    g->fr.policy = policy;
    g->fr.mlp = mlp;
    return GRZ_OK;
}

extern "C" int grz_frontier_last_features(grz_graph* g, float* host, uint64_t cap)
{
    if (!g || !host || cap < (uint64_t)NF) return GRZ_ERR_ARG;
    memcpy(host, g->fr.last_features, sizeof(float) * NF);
    return GRZ_OK;
}

// features of the current state (the iteration about to run) and the current policy's choice
extern "C" int grz_frontier_features(grz_graph* g, float* host, uint64_t cap, int* policy_choice)
{
    if (!g || !host || cap < (uint64_t)NF) return GRZ_ERR_ARG;
    if (!grz_frontier_live(g)) return grz_set_error(g, GRZ_ERR_STATE, "grz_frontier_begin not called");
    uint64_t v = 0;
    int pull = 0;
    const int rc = grz_switch_decide(g, g->fr.has, g->fr.vote_host, g->fr.iter + 1, &v, &pull, host);
    if (rc) return rc;
    if (policy_choice) *policy_choice = pull;
    return GRZ_OK;
}

// snapshot / restore of the CC/BFS state, to time both engines from the same state
extern "C" int grz_frontier_snapshot(grz_graph* g)
{
    if (!g || !grz_frontier_live(g)) return GRZ_ERR_STATE;
    grz_frontier_state& f = g->fr;
    const uint64_t V = g->V, W = (V >> 6) + 2;
    const uint64_t need = sizeof(uint32_t) * (V + 1) * 2 + sizeof(unsigned long long) * W * 3;
    if (f.snap_bytes < need) {
        cudaFree(f.snap);
        f.snap = nullptr;
        f.snap_bytes = 0;
        GRZ_CK(g, cudaMalloc(&f.snap, need));
        f.snap_bytes = need;
    }
    char* p = (char*)f.snap;
    cudaStream_t st = g->stream;
    GRZ_CK(g, cudaMemcpyAsync(p, f.label, sizeof(uint32_t) * (V + 1), cudaMemcpyDeviceToDevice, st)); p += sizeof(uint32_t) * (V + 1);
    GRZ_CK(g, cudaMemcpyAsync(p, f.level, sizeof(uint32_t) * (V + 1), cudaMemcpyDeviceToDevice, st)); p += sizeof(uint32_t) * (V + 1);
    GRZ_CK(g, cudaMemcpyAsync(p, f.has, 8 * W, cudaMemcpyDeviceToDevice, st)); p += 8 * W;
    GRZ_CK(g, cudaMemcpyAsync(p, f.has_next, 8 * W, cudaMemcpyDeviceToDevice, st)); p += 8 * W;
    GRZ_CK(g, cudaMemcpyAsync(p, f.wants, 8 * W, cudaMemcpyDeviceToDevice, st));
    f.snap_scalars[0] = f.iter; f.snap_scalars[1] = f.npull; f.snap_scalars[2] = f.npush;
    f.snap_scalars[3] = f.vote_host; f.snap_scalars[4] = (uint64_t)f.last_engine; f.snap_scalars[5] = (uint64_t)f.next_pull;
    return GRZ_OK;
}

extern "C" int grz_frontier_restore(grz_graph* g)
{
    if (!g || !grz_frontier_live(g) || !g->fr.snap) return GRZ_ERR_STATE;
    grz_frontier_state& f = g->fr;
    const uint64_t V = g->V, W = (V >> 6) + 2;
    const char* p = (const char*)f.snap;
    cudaStream_t st = g->stream;
    GRZ_CK(g, cudaMemcpyAsync(f.label, p, sizeof(uint32_t) * (V + 1), cudaMemcpyDeviceToDevice, st)); p += sizeof(uint32_t) * (V + 1);
    GRZ_CK(g, cudaMemcpyAsync(f.level, p, sizeof(uint32_t) * (V + 1), cudaMemcpyDeviceToDevice, st)); p += sizeof(uint32_t) * (V + 1);
    GRZ_CK(g, cudaMemcpyAsync(f.has, p, 8 * W, cudaMemcpyDeviceToDevice, st)); p += 8 * W;
    GRZ_CK(g, cudaMemcpyAsync(f.has_next, p, 8 * W, cudaMemcpyDeviceToDevice, st)); p += 8 * W;
    GRZ_CK(g, cudaMemcpyAsync(f.wants, p, 8 * W, cudaMemcpyDeviceToDevice, st));
    f.iter = (uint32_t)f.snap_scalars[0]; f.npull = (uint32_t)f.snap_scalars[1]; f.npush = (uint32_t)f.snap_scalars[2];
    f.vote_host = f.snap_scalars[3]; f.last_engine = (int)f.snap_scalars[4]; f.next_pull = (int)f.snap_scalars[5];
    return GRZ_OK;
}

// one iteration with the edge phase timed by CUDA events (the per-iteration profile the
// learned switch trains on)
extern "C" int grz_frontier_next_timed(grz_graph* g, int engine, int* engine_used, uint64_t* vote, float* edge_ms)
{
    if (!g || !grz_frontier_live(g)) return GRZ_ERR_STATE;
    grz_frontier_state& f = g->fr;
    if (!f.ev[0]) {
        GRZ_CK(g, cudaEventCreate(&f.ev[0]));
        GRZ_CK(g, cudaEventCreate(&f.ev[1]));
    }
    f.time_edges = 1;
    const int rc = grz_frontier_step(g, engine, engine_used, vote);
    f.time_edges = 0;
    if (rc >= 0 && edge_ms) *edge_ms = f.last_edge_ms;
    return rc;
}

// the policy fields of the run control block for the current frontier state
void grz_switch_policy_ctl(grz_graph* g, grz_runctl* c)
{
    const grz_frontier_state& f = g->fr;
    c->force = (f.flags & GRZ_FLAG_FORCE_PULL) ? 1 : ((f.flags & GRZ_FLAG_FORCE_PUSH) ? 0 : -1);
    c->params = (f.policy == GRZ_POLICY_LEARNED && f.mlp) ? f.mlp->params : nullptr;
    c->threshold = (f.flags & GRZ_FLAG_WITHOUT_OUTDEG) ? (double)(g->V / 2) : (double)(g->E / 5);
}
