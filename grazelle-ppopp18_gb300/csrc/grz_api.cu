// grz_api.cu -- graph context, ingest, queries and the exported C ABI (include/grazelle_gb300.h).
#include <errno.h>
#include <fcntl.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <chrono>
#include <mutex>
#include <thread>
#include <vector>

#include "grz_internal.cuh"
#include "../../include/grazelle_gb300.h"

// grz_pr.cu
int grz_pr_init_state(grz_graph* g, double damping);
int grz_pr_fused_iteration(grz_graph* g, int write_double_props);
int grz_pr_use_persistent(const grz_graph* g);
int grz_pr_persistent_iterations(grz_graph* g, uint32_t iters);
int grz_pr_props_to_double(grz_graph* g);

int grz_set_error(grz_graph* g, int code, const char* fmt, ...)
{
    if (g) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(g->err, sizeof(g->err), fmt, ap);
        va_end(ap);
    }
    return code;
}

int grz_cuda_check(grz_graph* g, cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return GRZ_OK;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return grz_set_error(g, GRZ_ERR_NOMEM, "%s: %s", what, cudaGetErrorString(e));
    }
    return grz_set_error(g, GRZ_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

extern "C" const char* grz_error_string(int code)
{
    switch (code) {
        case GRZ_OK: return "ok";
        case GRZ_ERR_ARG: return "bad argument";
        case GRZ_ERR_CUDA: return "CUDA error";
        case GRZ_ERR_NOMEM: return "out of device memory";
        case GRZ_ERR_UNSORTED: return "edge list not grouped by its shared vertex in ascending order";
        case GRZ_ERR_RANGE: return "vertex ID or size out of range";
        case GRZ_ERR_STATE: return "call out of order";
        case GRZ_ERR_IO: return "file missing, truncated or inconsistent";
        case GRZ_ERR_TIMEOUT: return "bounded device wait timed out";
        default: return "unknown error";
    }
}

extern "C" const char* grz_graph_last_error(const grz_graph* g) { return g ? g->err : "no graph"; }

int grz_dev_alloc(grz_graph* g, void** p, size_t bytes)
{
    *p = nullptr;
    GRZ_CK(g, cudaMallocAsync(p, bytes ? bytes : 16, g->stream));
    return GRZ_OK;
}

void grz_dev_free(grz_graph* g, void* p)
{
    if (p) cudaFreeAsync(p, g->stream);
}

// keeps the memory freed into the device's default pool for reuse, once per device
static int pool_setup(int device)
{
    static std::mutex m;
    static bool done[64] = {};
    std::lock_guard<std::mutex> lk(m);
    if (device < 0 || device >= 64 || done[device]) return GRZ_OK;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) != cudaSuccess) { cudaGetLastError(); return GRZ_ERR_CUDA; }
    uint64_t thr = ~0ull;
    if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr) != cudaSuccess) { cudaGetLastError(); return GRZ_ERR_CUDA; }
    done[device] = true;
    return GRZ_OK;
}

static void free_list(grz_graph* g, grz_list* L)
{
    grz_dev_free(g, L->vs);
    grz_dev_free(g, L->vindex);
    grz_dev_free(g, L->nbr);
    grz_dev_free(g, L->shared);
    grz_dev_free(g, L->rowptr);
    grz_dev_free(g, L->hub_vid);
    memset(L, 0, sizeof(*L));
}

// next_V: the V of the graph about to be loaded; the CC/BFS buffers stay when it is the same
static void free_graph_data(grz_graph* g, uint64_t next_V = ~0ull)
{
    if (g->fr.label && g->fr.alloc_V == next_V)
        grz_frontier_park(g);
    else
        grz_frontier_free(g);
    free_list(g, &g->pull);
    free_list(g, &g->push);
    // pool: streamed per-vertex arrays; cudaMalloc: the PageRank props and sums, which the gather
    // reads at random (pool memory measured 12% slower for random gathers)
    void* pooled[] = { g->outdeg, g->degree, g->inv_deg, g->prop, g->accum, g->glob, g->scratch };
    for (void* p : pooled) grz_dev_free(g, p);
    if (g->pr_fx[0] && g->V == next_V) {
        // the PageRank arrays are sized by V alone: kept, and refilled at the next grz_pr_init
        g->pr_lists_changed = 1;
    } else {
        void* plain[] = { g->pr_fx[0], g->pr_fx[1], g->pr_sum, g->pr_K, g->pr_rowacc, g->pr_cut, g->pr_d[0], g->pr_d[1] };
        for (void* p : plain) cudaFree(p);
        g->pr_d[0] = g->pr_d[1] = nullptr;
        g->pr_fx[0] = g->pr_fx[1] = nullptr; g->pr_sum = nullptr; g->pr_K = nullptr; g->pr_rowacc = nullptr;
        g->pr_cut = nullptr;
    }
    grz_dev_free(g, g->seg_nbr);
    grz_dev_free(g, g->seg_dst);
    g->seg_nbr = nullptr;
    g->seg_dst = nullptr;
    g->seg_bits = 0;
    g->nseg = 0;
    g->pr_segmode = 0;
    g->pr_dmode = g->pr_fx_stale = g->pr_d_stale = 0;
    g->outdeg = nullptr; g->degree = nullptr; g->inv_deg = nullptr;
    g->pr_rowacc_stale = 0;
    g->prop = nullptr; g->accum = nullptr; g->glob = nullptr; g->scratch = nullptr;
    g->scratch_bytes = 0;
    g->max_degree_known = 0;
    g->V = g->E = 0;
}

int grz_scratch(grz_graph* g, size_t bytes, void** out)
{
    if (bytes > g->scratch_bytes) {
        grz_dev_free(g, g->scratch);
        g->scratch = nullptr;
        g->scratch_bytes = 0;
        int rc = grz_dev_alloc(g, &g->scratch, bytes);
        if (rc) return rc;
        g->scratch_bytes = bytes;
    }
    *out = g->scratch;
    return GRZ_OK;
}

extern "C" int grz_graph_create(grz_graph** out, int device, void* stream)
{
    if (!out) return GRZ_ERR_ARG;
    *out = nullptr;
    grz_graph* g = (grz_graph*)calloc(1, sizeof(grz_graph));
    if (!g) return GRZ_ERR_NOMEM;
    g->device = device;
    g->tune.hub_max = 0;      // measured: the label gathers are bound by the L1/L2 path of non-hub lanes
    g->tune.cc_cache = 16384;
    g->tune.cc_threads = 512;
    g->tune.cc_grid = 0;
    g->tune.pr_grid = 0;
    g->tune.pr_props = 0;
    g->tune.bfs_pull_first = 1;
    g->tune.cc_pull_first = 4;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g->l2_bytes, cudaDevAttrL2CacheSize, device);
    if (e == cudaSuccess && pool_setup(device) != GRZ_OK) e = cudaErrorUnknown;
    if (e != cudaSuccess) {
        free(g);
        cudaGetLastError();
        return GRZ_ERR_CUDA;
    }
    if (stream) {
        g->stream = (cudaStream_t)stream;
        g->own_stream = 0;
    } else {
        e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            free(g);
            cudaGetLastError();
            return GRZ_ERR_CUDA;
        }
        g->own_stream = 1;
    }
    *out = g;
    return GRZ_OK;
}

extern "C" int grz_graph_set_stream(grz_graph* g, void* stream)
{
    if (!g) return GRZ_ERR_ARG;
    cudaSetDevice(g->device);
    // the graph's pool allocations were ordered on the old stream: finish them before switching
    cudaStreamSynchronize(g->stream);
    if (g->own_stream) {
        cudaStreamDestroy(g->stream);
        g->own_stream = 0;
    }
    if (stream) {
        g->stream = (cudaStream_t)stream;
    } else {
        GRZ_CK(g, cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
        g->own_stream = 1;
    }
    return GRZ_OK;
}

// ---------------------------------------------------------------------------------------------
// kernel profiling

void grz_prof_begin(grz_graph* g, int kind)
{
    grz_prof* p = g->prof;
    if (!p || !p->on || p->n >= GRZ_PROF_MAX) return;
    if (p->n >= p->created) {
        cudaEventCreate(&p->ev[p->n][0]);
        cudaEventCreate(&p->ev[p->n][1]);
        p->created = p->n + 1;
    }
    p->kind[p->n] = kind;
    cudaEventRecord(p->ev[p->n][0], g->stream);
}

void grz_prof_end(grz_graph* g)
{
    grz_prof* p = g->prof;
    if (!p || !p->on || p->n >= GRZ_PROF_MAX) return;
    cudaEventRecord(p->ev[p->n][1], g->stream);
    p->direct_ms[p->n] = -1.0f;
    p->n++;
}

void grz_prof_direct(grz_graph* g, int kind, float ms)
{
    grz_prof* p = g->prof;
    if (!p || !p->on || p->n >= GRZ_PROF_MAX) return;
    p->kind[p->n] = kind;
    p->direct_ms[p->n] = ms;
    p->n++;
}

extern "C" int grz_profile_enable(grz_graph* g, int on)
{
    if (!g) return GRZ_ERR_ARG;
    if (!g->prof) {
        g->prof = (grz_prof*)calloc(1, sizeof(grz_prof));
        if (!g->prof) return GRZ_ERR_NOMEM;
    }
    g->prof->on = on;
    g->prof->n = 0;
    return GRZ_OK;
}

extern "C" int grz_profile_read(grz_graph* g, int* kinds, float* ms, int capacity)
{
    if (!g || (capacity > 0 && (!kinds || !ms))) return GRZ_ERR_ARG;
    grz_prof* p = g->prof;
    if (!p) return 0;
    GRZ_CK(g, cudaStreamSynchronize(g->stream));
    const int n = p->n < capacity ? p->n : capacity;
    for (int i = 0; i < n; ++i) {
        kinds[i] = p->kind[i];
        ms[i] = 0.0f;
        if (p->direct_ms[i] >= 0.0f) ms[i] = p->direct_ms[i];
        else cudaEventElapsedTime(&ms[i], p->ev[i][0], p->ev[i][1]);
    }
    p->n = 0;
    return n;
}

extern "C" int grz_profile_work(grz_graph* g, uint64_t* first_pull_vectors, uint64_t* later_pull_vectors)
{
    if (!g || !first_pull_vectors || !later_pull_vectors) return GRZ_ERR_ARG;
    unsigned long long h[2] = { 0, 0 };
    if (g->prof_work) {
        GRZ_CK(g, cudaMemcpyAsync(h, g->prof_work, sizeof(h), cudaMemcpyDeviceToHost, g->stream));
        GRZ_CK(g, cudaMemsetAsync(g->prof_work, 0, sizeof(h), g->stream));
        GRZ_CK(g, cudaStreamSynchronize(g->stream));
    }
    *first_pull_vectors = h[0];
    *later_pull_vectors = h[1];
    return GRZ_OK;
}

extern "C" const char* grz_profile_kind_name(int kind)
{
    static const char* names[] = { "none", "pr_gather", "pr_apply", "pr_push", "pr_vertex", "cc_pull", "cc_push",
                                   "bfs_pull", "bfs_push", "frontier", "vertex", "iteration", "mlp", "batch",
                                   "bfs_visit", "push_compact" };
    static_assert(sizeof(names) / sizeof(names[0]) == GRZ_PROF_KINDS, "kind names");
    return (kind > 0 && kind < GRZ_PROF_KINDS) ? names[kind] : "none";
}

extern "C" void grz_graph_destroy(grz_graph* g)
{
    if (!g) return;
    cudaSetDevice(g->device);
    cudaStreamSynchronize(g->stream);
    if (g->prof) {
        for (int i = 0; i < g->prof->created; ++i) { cudaEventDestroy(g->prof->ev[i][0]); cudaEventDestroy(g->prof->ev[i][1]); }
        free(g->prof);
    }
    free_graph_data(g);
    cudaStreamSynchronize(g->stream);
    if (g->stats_dev) cudaFree(g->stats_dev);
    if (g->prof_work) cudaFree(g->prof_work);
    if (g->pr_bar) cudaFree(g->pr_bar);
    if (g->pr_bar_host) cudaFreeHost(g->pr_bar_host);
    if (g->copy_stream) {
        cudaStreamDestroy(g->copy_stream);
        cudaEventDestroy(g->copy_ev[0]);
        cudaEventDestroy(g->copy_ev[1]);
    }
    if (g->own_stream) cudaStreamDestroy(g->stream);
    free(g);
}

extern "C" int grz_sync(grz_graph* g)
{
    if (!g) return GRZ_ERR_ARG;
    GRZ_CK(g, cudaStreamSynchronize(g->stream));
    return GRZ_OK;
}

static bool is_device_ptr(const void* p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// the device's address of page-locked host memory, or null for any other pointer
static const void* pinned_device_view(const void* p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

static int load_pairs(grz_graph* g, uint64_t V, uint64_t E, const uint64_t* pull_pairs, const uint64_t* push_pairs,
                      int flags);

// the graph's second stream for host-to-device copies, and its two events, made on first use
cudaError_t grz_copy_stream(grz_graph* g)
{
    if (g->copy_stream) return cudaSuccess;
    cudaError_t e = cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->copy_ev[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->copy_ev[1], cudaEventDisableTiming);
    return e;
}
static int finish_load(grz_graph* g, int rc);

extern "C" int grz_graph_load_pairs(grz_graph* g, uint64_t V, uint64_t E, const uint64_t* pull_pairs,
                                    const uint64_t* push_pairs)
{
    return load_pairs(g, V, E, pull_pairs, push_pairs, 0);
}

extern "C" int grz_graph_load_pairs_ex(grz_graph* g, uint64_t V, uint64_t E, const uint64_t* pull_pairs,
                                       const uint64_t* push_pairs, int flags)
{
    if (flags & ~GRZ_LOAD_DERIVE_PUSH) return GRZ_ERR_ARG;
    if ((flags & GRZ_LOAD_DERIVE_PUSH) && push_pairs) return grz_set_error(g, GRZ_ERR_ARG, "push pairs given and asked to derive them");
    return load_pairs(g, V, E, pull_pairs, push_pairs, flags);
}

static int load_pairs(grz_graph* g, uint64_t V, uint64_t E, const uint64_t* pull_pairs, const uint64_t* push_pairs,
                      int flags)
{
    if (!g || (E > 0 && !pull_pairs)) return GRZ_ERR_ARG;
    if (V >= 0xffffffffull) return grz_set_error(g, GRZ_ERR_RANGE, "V = %llu exceeds the 32-bit device ID limit", (unsigned long long)V);
    GRZ_CK(g, cudaSetDevice(g->device));
    free_graph_data(g, V);
    g->V = V;
    g->E = E;
    cudaStream_t st = g->stream;
    const size_t pbytes = sizeof(uint64_t) * 2 * E;
    int rc = GRZ_OK;
    if ((flags & GRZ_LOAD_DERIVE_PUSH) && !push_pairs && E > 0) {
        // Pull-only ingest: pinned host pairs cross the link chunk by chunk while the chunks already
        // in are processed; device pairs are read where they are.  Pageable host memory is first
        // copied into a device buffer.
        const void* view = is_device_ptr(pull_pairs) ? (const void*)pull_pairs : pinned_device_view(pull_pairs);
        void* dbuf = nullptr;
        if (!view) {
            rc = grz_dev_alloc(g, &dbuf, pbytes);
            if (rc == GRZ_OK) rc = grz_cuda_check(g, cudaMemcpyAsync(dbuf, pull_pairs, pbytes, cudaMemcpyHostToDevice, st), "H2D pull pairs");
            view = dbuf;
        }
        if (rc == GRZ_OK) rc = grz_ingest_pull_derive(g, (const uint64_t*)view, E, dbuf || is_device_ptr(pull_pairs) ? nullptr : pull_pairs);
        if (rc == GRZ_OK) rc = grz_build_hubs(g, &g->pull, g->tune.hub_max);
        if (rc == GRZ_OK) rc = grz_cuda_check(g, cudaStreamSynchronize(st), "layout build");
        grz_dev_free(g, dbuf);
        return finish_load(g, rc);
    }
    // Host lists are copied into device buffers.  The -push copy runs on a second stream after the
    // -pull copy, so it overlaps the -pull list's build instead of following it.
    const uint64_t* dsrc[2] = { pull_pairs, push_pairs };
    void* dbuf[2] = { nullptr, nullptr };
    for (int which = 0; which < 2 && rc == GRZ_OK && E > 0; ++which) {
        if (!dsrc[which] || is_device_ptr(dsrc[which])) continue;
        rc = grz_dev_alloc(g, &dbuf[which], pbytes);
    }
    if (rc == GRZ_OK && E > 0 && dbuf[0]) {
        cudaError_t e = cudaMemcpyAsync(dbuf[0], pull_pairs, pbytes, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) rc = grz_cuda_check(g, e, "H2D pull pairs");
        else dsrc[0] = (const uint64_t*)dbuf[0];
    }
    bool push_on_copy_stream = false;
    if (rc == GRZ_OK && E > 0 && dbuf[1]) {
        cudaError_t e = grz_copy_stream(g);
        if (e == cudaSuccess) e = cudaEventRecord(g->copy_ev[0], st);  // after the -pull copy (and the allocations)
        if (e == cudaSuccess) e = cudaStreamWaitEvent(g->copy_stream, g->copy_ev[0], 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dbuf[1], push_pairs, pbytes, cudaMemcpyHostToDevice, g->copy_stream);
        if (e == cudaSuccess) e = cudaEventRecord(g->copy_ev[1], g->copy_stream);
        if (e != cudaSuccess) rc = grz_cuda_check(g, e, "H2D push pairs");
        else { dsrc[1] = (const uint64_t*)dbuf[1]; push_on_copy_stream = true; }
    }
    for (int which = 0; which < 2 && rc == GRZ_OK; ++which) {
        if (which == 1 && !push_pairs) break;
        if (which == 1 && push_on_copy_stream) {
            cudaError_t e = cudaStreamWaitEvent(st, g->copy_ev[1], 0);
            if (e != cudaSuccess) { rc = grz_cuda_check(g, e, "wait for push pairs"); break; }
        }
        // outdegrees credit the sources of the -pull pairs (graphdata.c:792-821)
        rc = grz_build_list(g, which == 0 ? &g->pull : &g->push, dsrc[which], E, which == 0 ? 1 : 0);
        if (rc == GRZ_OK && which == 0) rc = grz_build_outdegrees(g, dsrc[0], E);
        if (rc == GRZ_OK && which == 0) rc = grz_build_hubs(g, &g->pull, g->tune.hub_max);
        if (rc == GRZ_OK) rc = grz_cuda_check(g, cudaStreamSynchronize(st), "layout build");
    }
    if (push_on_copy_stream && rc != GRZ_OK) cudaStreamSynchronize(g->copy_stream);
    for (void* p : dbuf) grz_dev_free(g, p);
    return finish_load(g, rc);
}

// per-vertex state of a loaded graph (or, on a failed load, nothing)
static int finish_load(grz_graph* g, int rc)
{
    const uint64_t V = g->V;
    cudaStream_t st = g->stream;
    if (rc == GRZ_OK) {
        if ((rc = grz_dev_alloc(g, (void**)&g->prop, sizeof(double) * (V + 8))) == GRZ_OK &&
            (rc = grz_dev_alloc(g, (void**)&g->accum, sizeof(double) * (V + 8))) == GRZ_OK &&
            (rc = grz_dev_alloc(g, (void**)&g->glob, sizeof(u128) * GRZ_SUM_SLOTS)) == GRZ_OK) {
            cudaMemsetAsync(g->prop, 0, sizeof(double) * (V + 8), st);
            cudaMemsetAsync(g->accum, 0, sizeof(double) * (V + 8), st);
            cudaMemsetAsync(g->glob, 0, sizeof(u128) * GRZ_SUM_SLOTS, st);
            rc = grz_cuda_check(g, cudaStreamSynchronize(st), "state init");
        }
    }
    if (rc != GRZ_OK) free_graph_data(g);
    return rc;
}

// ---------------------------------------------------------------------------------------------
// File ingest (source/graphdata.c:957-1049): each list file is a {V, E} header and E (src, dst)
// uint64 pairs.  The pairs are streamed into a device buffer: reader threads fill one pinned
// staging buffer with pread while the previous one is copied to the device, so the disk (or page
// cache) and the host link work at the same time.  Sort order and ID range are checked on the
// device by the layout builder.

namespace {

constexpr size_t STAGE_BYTES = 64u << 20;  // per staging buffer
constexpr int STAGE_READERS = 4;           // pread threads per chunk

struct ListFile {
    int fd = -1;
    uint64_t V = 0, E = 0;
};

int open_list(grz_graph* g, const char* path, ListFile* lf, bool optional, bool* missing)
{
    if (missing) *missing = false;
    lf->fd = open(path, O_RDONLY);
    if (lf->fd < 0) {
        if (optional && errno == ENOENT) {
            if (missing) *missing = true;
            return GRZ_OK;
        }
        return grz_set_error(g, GRZ_ERR_IO, "unable to read file \"%s\"", path);
    }
    uint64_t hdr[2];
    if (pread(lf->fd, hdr, sizeof(hdr), 0) != (ssize_t)sizeof(hdr))
        return grz_set_error(g, GRZ_ERR_IO, "\"%s\": missing {V, E} header", path);
    if (hdr[1] > (1ull << 40))
        return grz_set_error(g, GRZ_ERR_IO, "\"%s\": implausible edge count %llu", path, (unsigned long long)hdr[1]);
    struct stat st;
    if (fstat(lf->fd, &st) == 0 && (uint64_t)st.st_size < sizeof(hdr) + 16 * hdr[1])
        return grz_set_error(g, GRZ_ERR_IO, "\"%s\": truncated (header says %llu edges)", path, (unsigned long long)hdr[1]);
    lf->V = hdr[0];
    lf->E = hdr[1];
    return GRZ_OK;
}

// reads [off, off + n) of fd into buf completely; false on an error or a short file
bool pread_all(int fd, char* buf, size_t n, uint64_t off)
{
    while (n > 0) {
        const ssize_t r = pread(fd, buf, n, (off_t)off);
        if (r < 0 && errno == EINTR) continue;
        if (r <= 0) return false;
        buf += r;
        off += (uint64_t)r;
        n -= (size_t)r;
    }
    return true;
}

int stream_to_device(grz_graph* g, const ListFile& lf, const char* path, char* dst)
{
    const uint64_t bytes = 16 * lf.E;
    if (bytes == 0) return GRZ_OK;
    char* stage[2] = { nullptr, nullptr };
    cudaEvent_t ev[2] = { nullptr, nullptr };
    int rc = GRZ_OK;
    for (int i = 0; i < 2 && rc == GRZ_OK; ++i) {
        cudaError_t e = cudaMallocHost((void**)&stage[i], STAGE_BYTES);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
        if (e != cudaSuccess) rc = grz_cuda_check(g, e, "staging buffers");
    }
    for (uint64_t off = 0, k = 0; off < bytes && rc == GRZ_OK; off += STAGE_BYTES, ++k) {
        const int b = (int)(k & 1);
        const size_t n = (size_t)std::min<uint64_t>(STAGE_BYTES, bytes - off);
        cudaError_t e = cudaEventSynchronize(ev[b]);  // the copy out of this buffer two chunks ago
        if (e != cudaSuccess) { rc = grz_cuda_check(g, e, "staging copy"); break; }
        bool ok[STAGE_READERS];
        std::vector<std::thread> th;
        const size_t part = (n + STAGE_READERS - 1) / STAGE_READERS;
        for (int t = 0; t < STAGE_READERS; ++t) {
            const size_t lo = std::min(n, t * part), hi = std::min(n, lo + part);
            ok[t] = true;
            if (hi > lo)
                th.emplace_back([&, t, lo, hi] { ok[t] = pread_all(lf.fd, stage[b] + lo, hi - lo, 16 + off + lo); });
        }
        for (auto& x : th) x.join();
        for (int t = 0; t < STAGE_READERS; ++t)
            if (!ok[t]) rc = grz_set_error(g, GRZ_ERR_IO, "\"%s\": read failed at byte %llu", path, (unsigned long long)(16 + off));
        if (rc) break;
        e = cudaMemcpyAsync(dst + off, stage[b], n, cudaMemcpyHostToDevice, g->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ev[b], g->stream);
        if (e != cudaSuccess) rc = grz_cuda_check(g, e, "H2D pairs");
    }
    cudaStreamSynchronize(g->stream);
    for (int i = 0; i < 2; ++i) {
        if (stage[i]) cudaFreeHost(stage[i]);
        if (ev[i]) cudaEventDestroy(ev[i]);
    }
    return rc;
}

}  // namespace

extern "C" int grz_graph_load_files_ex(grz_graph* g, const char* base, int flags)
{
    if (!g || !base) return GRZ_ERR_ARG;
    if (flags & ~GRZ_LOAD_DERIVE_PUSH) return GRZ_ERR_ARG;
    GRZ_CK(g, cudaSetDevice(g->device));
    char path[2][4096];
    snprintf(path[0], sizeof(path[0]), "%s-pull", base);
    snprintf(path[1], sizeof(path[1]), "%s-push", base);
    const bool derive = (flags & GRZ_LOAD_DERIVE_PUSH) != 0;
    ListFile lf[2];
    bool push_missing = derive;
    int rc = open_list(g, path[0], &lf[0], false, nullptr);
    if (rc == GRZ_OK && !derive) rc = open_list(g, path[1], &lf[1], true, &push_missing);  // the push list is optional
    if (rc == GRZ_OK && !push_missing && (lf[1].V != lf[0].V || lf[1].E != lf[0].E))
        rc = grz_set_error(g, GRZ_ERR_IO, "\"%s\": header {V, E} differs from the -pull file", path[1]);
    void* dbuf[2] = { nullptr, nullptr };
    if (rc == GRZ_OK) {
        free_graph_data(g, lf[0].V);  // the old graph's memory back to the pool before the new pairs take it
        const uint64_t E = lf[0].E;
        for (int i = 0; i < 2 && rc == GRZ_OK; ++i) {
            if (i == 1 && push_missing) break;
            if (E > 0) rc = grz_dev_alloc(g, &dbuf[i], 16 * E);
            if (rc == GRZ_OK) rc = stream_to_device(g, lf[i], path[i], (char*)dbuf[i]);
        }
        if (rc == GRZ_OK)
            rc = load_pairs(g, lf[0].V, E, (const uint64_t*)dbuf[0], (const uint64_t*)dbuf[1],
                            derive && E > 0 ? GRZ_LOAD_DERIVE_PUSH : 0);
    }
    for (int i = 0; i < 2; ++i) {
        if (lf[i].fd >= 0) close(lf[i].fd);
        grz_dev_free(g, dbuf[i]);
    }
    return rc;
}

extern "C" int grz_graph_load_files(grz_graph* g, const char* base)
{
    return grz_graph_load_files_ex(g, base, 0);
}

extern "C" int grz_graph_get_info(const grz_graph* gc, grz_graph_info_t* out)
{
    if (!gc || !out) return GRZ_ERR_ARG;
    memset(out, 0, sizeof(*out));
    // the reference-format lists whose device pointers the info hands out are a cache built on
    // first request; the graph is otherwise unchanged
    grz_graph* g = const_cast<grz_graph*>(gc);
    if (g->V || g->E) {
        GRZ_CK(g, cudaSetDevice(g->device));
        int rc = grz_list_reference(g, &g->pull);
        if (rc == GRZ_OK) rc = grz_list_reference(g, &g->push);
        if (rc != GRZ_OK) return rc;
    }
    out->num_vertices = g->V;
    out->num_edges = g->E;
    out->pull_vectors = g->pull.nvec;
    out->push_vectors = g->push.nvec;
    out->pull_index_start = g->pull.vindex_start;
    out->pull_index_end = g->pull.vindex_end;
    out->push_index_start = g->push.vindex_start;
    out->push_index_end = g->push.vindex_end;
    out->pull_list_device = g->pull.vs;
    out->push_list_device = g->push.vs;
    uint64_t b = 0;
    const grz_list* Ls[2] = { &g->pull, &g->push };
    for (const grz_list* L : Ls)
        if (L->nbr) b += L->nvec * ((L->vs ? 32 : 0) + 16 + 4) + (g->V + 64) * 8 + (g->V + 1) * 4;
    b += (g->V + 8) * 8 * 3 + g->V * 12;
    if (g->pr_fx[0]) b += g->V * (16 * 3 + 4);
    if (g->pr_d[0]) b += g->V * 16;
    out->device_bytes = b;
    return GRZ_OK;
}

static const grz_list* list_of(const grz_graph* g, int list) { return list == GRZ_LIST_PUSH ? &g->push : &g->pull; }

extern "C" int grz_graph_copy_list(grz_graph* g, int list, uint64_t* host, uint64_t cap)
{
    if (!g || !host) return GRZ_ERR_ARG;
    grz_list* L = list == GRZ_LIST_PUSH ? &g->push : &g->pull;
    if (!L->nbr) return grz_set_error(g, GRZ_ERR_STATE, "list not built");
    GRZ_CK(g, cudaSetDevice(g->device));
    int rc = grz_list_reference(g, L);
    if (rc) return rc;
    if (cap < L->nvec) return grz_set_error(g, GRZ_ERR_ARG, "capacity %llu < %llu vectors", (unsigned long long)cap, (unsigned long long)L->nvec);
    GRZ_CK(g, cudaMemcpyAsync(host, L->vs, sizeof(uint64_t) * 4 * L->nvec, cudaMemcpyDeviceToHost, g->stream));
    GRZ_CK(g, cudaStreamSynchronize(g->stream));
    return GRZ_OK;
}

extern "C" int grz_graph_copy_vertex_index(grz_graph* g, int list, uint64_t* host, uint64_t cap)
{
    if (!g || !host) return GRZ_ERR_ARG;
    const grz_list* L = list_of(g, list);
    if (!L->vindex) return grz_set_error(g, GRZ_ERR_STATE, "list not built");
    if (cap < g->V + 64) return grz_set_error(g, GRZ_ERR_ARG, "capacity below V + 64");
    GRZ_CK(g, cudaMemcpyAsync(host, L->vindex, sizeof(uint64_t) * (g->V + 64), cudaMemcpyDeviceToHost, g->stream));
    GRZ_CK(g, cudaStreamSynchronize(g->stream));
    return GRZ_OK;
}

extern "C" int grz_graph_copy_outdegrees(grz_graph* g, double* host, uint64_t cap)
{
    if (!g || !host) return GRZ_ERR_ARG;
    if (!g->outdeg) return grz_set_error(g, GRZ_ERR_STATE, "no graph loaded");
    if (cap < g->V) return grz_set_error(g, GRZ_ERR_ARG, "capacity below V");
    GRZ_CK(g, cudaMemcpyAsync(host, g->outdeg, sizeof(double) * g->V, cudaMemcpyDeviceToHost, g->stream));
    GRZ_CK(g, cudaStreamSynchronize(g->stream));
    return GRZ_OK;
}

// ---------------------------------------------------------------------------------------------
// PageRank

extern "C" int grz_pr_init(grz_graph* g, double damping)
{
    if (!g) return GRZ_ERR_ARG;
    if (!g->outdeg) return grz_set_error(g, GRZ_ERR_STATE, "no graph loaded");
    if (!(damping >= 0.0 && damping <= 1.0)) return grz_set_error(g, GRZ_ERR_ARG, "damping must be in [0, 1]");
    GRZ_CK(g, cudaSetDevice(g->device));
    g->app = GRZ_APP_PAGERANK;
    return grz_pr_init_state(g, damping);
}

extern "C" int grz_pr_iterate(grz_graph* g, uint32_t iterations)
{
    if (!g) return GRZ_ERR_ARG;
    if (!grz_pr_live(g)) return grz_set_error(g, GRZ_ERR_STATE, "grz_pr_init not called since the graph was loaded");
    GRZ_CK(g, cudaSetDevice(g->device));
    if (grz_pr_use_persistent(g)) return grz_pr_persistent_iterations(g, iterations);
    for (uint32_t i = 0; i < iterations; ++i) {
        int rc = grz_pr_fused_iteration(g, 0);
        if (rc) return rc;
    }
    return GRZ_OK;
}

extern "C" int grz_pr_time_iterations(grz_graph* g, uint32_t iterations, float* ms_out)
{
    if (!g || !ms_out) return GRZ_ERR_ARG;
    if (!grz_pr_live(g)) return grz_set_error(g, GRZ_ERR_STATE, "grz_pr_init not called since the graph was loaded");
    cudaEvent_t e0, e1;
    GRZ_CK(g, cudaEventCreate(&e0));
    GRZ_CK(g, cudaEventCreate(&e1));
    int rc = GRZ_OK;
    cudaEventRecord(e0, g->stream);
    if (grz_pr_use_persistent(g)) rc = grz_pr_persistent_iterations(g, iterations);
    else
        for (uint32_t i = 0; i < iterations && rc == GRZ_OK; ++i) rc = grz_pr_fused_iteration(g, 0);
    cudaEventRecord(e1, g->stream);
    if (rc == GRZ_OK) rc = grz_cuda_check(g, cudaEventSynchronize(e1), "event sync");
    if (rc == GRZ_OK) cudaEventElapsedTime(ms_out, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

extern "C" int grz_read_props(grz_graph* g, double* host, uint64_t cap)
{
    if (!g || !host) return GRZ_ERR_ARG;
    if (cap < g->V) return grz_set_error(g, GRZ_ERR_ARG, "capacity below V");
    GRZ_CK(g, cudaSetDevice(g->device));
    if (g->app == GRZ_APP_PAGERANK && g->pr_fx[0]) {
        if (g->pr_lists_changed) return grz_set_error(g, GRZ_ERR_STATE, "grz_pr_init not called since the graph was loaded");
        int rc = grz_pr_props_to_double(g);
        if (rc) return rc;
    } else if (g->app != GRZ_APP_PAGERANK) {
        int rc = grz_frontier_props(g);
        if (rc) return rc;
    }
    GRZ_CK(g, cudaMemcpyAsync(host, g->prop, sizeof(double) * g->V, cudaMemcpyDeviceToHost, g->stream));
    GRZ_CK(g, cudaStreamSynchronize(g->stream));
    return GRZ_OK;
}

// ---------------------------------------------------------------------------------------------
// Connected Components and BFS

// One CC/BFS run to convergence.  By default the whole loop is one CUDA graph launch
// (grz_frontier_run_graph); GRZ_FLAG_HOST_LOOP, profiling, or a graph without both lists run
// it with one host round trip per iteration (grz_frontier_step).  Both give the same
// iterations, engines and results.
static int frontier_run(grz_graph* g, int app, uint32_t root, int flags, grz_run_stats_t* stats)
{
    if (!g) return GRZ_ERR_ARG;
    GRZ_CK(g, cudaSetDevice(g->device));
    g->app = app;
    // the counting of kernel profiling and iteration stats happens on the host loop
    const bool profiling = g->prof && g->prof->on;
    const bool graph = !(flags & GRZ_FLAG_HOST_LOOP) && !profiling && !g->stats_on && g->pull.nvec && g->push.nvec;
    if (graph) grz_frontier_run_prepare(g);
    int rc = grz_frontier_init(g, app, flags, root);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    GRZ_CK(g, cudaEventCreate(&e0));
    GRZ_CK(g, cudaEventCreate(&e1));
    cudaEventRecord(e0, g->stream);
    if (graph) {
        rc = grz_frontier_run_graph(g, nullptr);
    } else {
        // the same bounds as the graph run's decision kernel, checked between iterations
        const uint64_t max_it = g->tune.run_max_iterations ? g->tune.run_max_iterations : g->V + 2;
        const double limit_s = g->tune.run_limit_us ? g->tune.run_limit_us * 1e-6 : 300.0;
        const auto t0 = std::chrono::steady_clock::now();
        for (;;) {
            int engine = -1;
            uint64_t vote = 0;
            rc = grz_frontier_step(g, -1, &engine, &vote);
            if (rc <= 0) break;
            if (g->fr.iter >= max_it) {
                rc = grz_set_error(g, GRZ_ERR_TIMEOUT, "no convergence within %llu iterations", (unsigned long long)max_it);
                break;
            }
            if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > limit_s) {
                rc = grz_set_error(g, GRZ_ERR_TIMEOUT, "run stopped by its time bound (%.0f ms)", limit_s * 1e3);
                break;
            }
        }
    }
    cudaEventRecord(e1, g->stream);
    if (rc == 0) rc = grz_cuda_check(g, cudaEventSynchronize(e1), "run");
    if (rc == 0 && g->tune.pull_staging) rc = grz_frontier_check_waits(g);
    if (rc == 0 && stats) {
        memset(stats, 0, sizeof(*stats));
        stats->iterations = g->fr.iter;
        stats->pull_iterations = g->fr.npull;
        stats->push_iterations = g->fr.npush;
        cudaEventElapsedTime(&stats->ms, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

extern "C" int grz_cc_run(grz_graph* g, int flags, grz_run_stats_t* stats)
{
    return frontier_run(g, GRZ_APP_CONNECTED_COMPONENTS, 0, flags, stats);
}

extern "C" int grz_bfs_run(grz_graph* g, uint32_t root, int flags, grz_run_stats_t* stats)
{
    return frontier_run(g, GRZ_APP_BREADTH_FIRST_SEARCH, root, flags, stats);
}

extern "C" int grz_frontier_begin(grz_graph* g, int app, uint32_t root, int flags)
{
    if (!g || (app != GRZ_APP_CONNECTED_COMPONENTS && app != GRZ_APP_BREADTH_FIRST_SEARCH)) return GRZ_ERR_ARG;
    GRZ_CK(g, cudaSetDevice(g->device));
    g->app = app;
    return grz_frontier_init(g, app, flags, root);
}

extern "C" int grz_frontier_next(grz_graph* g, int engine, int* engine_used, uint64_t* vote)
{
    if (!g) return GRZ_ERR_ARG;
    if (!grz_frontier_live(g)) return grz_set_error(g, GRZ_ERR_STATE, "grz_frontier_begin not called since the graph was loaded");
    return grz_frontier_step(g, engine, engine_used, vote);
}

extern "C" int grz_frontier_current_vote(grz_graph* g, uint64_t* vote, int* threshold_engine)
{
    if (!g || !vote) return GRZ_ERR_ARG;
    *vote = g->fr.vote_host;
    if (threshold_engine) *threshold_engine = grz_engine_threshold(g, g->fr.vote_host);
    return GRZ_OK;
}

extern "C" int grz_read_levels(grz_graph* g, int64_t* host, uint64_t cap)
{
    if (!g || !host) return GRZ_ERR_ARG;
    if (cap < g->V) return grz_set_error(g, GRZ_ERR_ARG, "capacity below V");
    if (!grz_frontier_live(g) || g->fr.app != GRZ_APP_BREADTH_FIRST_SEARCH) return grz_set_error(g, GRZ_ERR_STATE, "no BFS result");
    uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * (g->V ? g->V : 1));
    if (!tmp) return GRZ_ERR_NOMEM;
    cudaError_t e = cudaMemcpyAsync(tmp, g->fr.level, sizeof(uint32_t) * g->V, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess)
        for (uint64_t v = 0; v < g->V; ++v) host[v] = tmp[v] == 0xffffffffu ? -1 : (int64_t)tmp[v];
    free(tmp);
    return grz_cuda_check(g, e, "read levels");
}

extern "C" int grz_result_digest(grz_graph* g, uint64_t* out3)
{
    if (!g || !out3) return GRZ_ERR_ARG;
    return grz_frontier_digest(g, out3);
}

extern "C" int grz_tune_set(grz_graph* g, int param, int64_t value)
{
    if (!g || value < 0) return GRZ_ERR_ARG;
    switch (param) {
    case GRZ_TUNE_HUBS:
        if (value > (int64_t)GRZ_HUB_MAX) return grz_set_error(g, GRZ_ERR_RANGE, "at most %u hubs", GRZ_HUB_MAX);
        g->tune.hub_max = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_CC_CACHE:
        if (value > (int64_t)GRZ_HUB_MAX) return grz_set_error(g, GRZ_ERR_RANGE, "at most %u cached hubs", GRZ_HUB_MAX);
        g->tune.cc_cache = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_CC_THREADS:
        if (value != 256 && value != 512 && value != 1024) return grz_set_error(g, GRZ_ERR_ARG, "threads must be 256, 512 or 1024");
        g->tune.cc_threads = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_CC_GRID:
        if (value > (1 << 20)) return GRZ_ERR_RANGE;
        g->tune.cc_grid = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_PR_GRID:
        if (value > (1 << 20)) return GRZ_ERR_RANGE;
        g->tune.pr_grid = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_BFS_PULL_SCAN:
        if (value > 1) return grz_set_error(g, GRZ_ERR_ARG, "BFS pull mode must be 0 or 1");
        g->tune.bfs_pull_scan = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_PR_PROPS:
        if (value > 2) return grz_set_error(g, GRZ_ERR_ARG, "PageRank gathered props must be 0 (by size), 1 (fixed point) or 2 (doubles)");
        g->tune.pr_props = (uint32_t)value;  // from the next grz_pr_init
        return GRZ_OK;
    case GRZ_TUNE_INGEST_CHUNKS:
        if (value > GRZ_INGEST_MAX_CHUNKS) return grz_set_error(g, GRZ_ERR_RANGE, "at most %d ingest chunks", GRZ_INGEST_MAX_CHUNKS);
        g->tune.ingest_chunks = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_PR_PERSISTENT:
        if (value > 3) return grz_set_error(g, GRZ_ERR_ARG, "PageRank iteration form must be 0 (default), 1 (two kernels), 2 or 3 (persistent, 6 or 8 blocks per SM)");
        g->tune.pr_persistent = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_PR_WAIT_LIMIT_US:
        if (value > 60000000) return grz_set_error(g, GRZ_ERR_RANGE, "barrier wait limit above 60 s");
        g->tune.pr_wait_limit_us = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_PR_WITHHOLD:
        if (value > (1 << 20)) return GRZ_ERR_RANGE;
        g->tune.pr_withhold = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_RUN_MAX_ITERATIONS:
        if (value > 0xfffffff0ll) return GRZ_ERR_RANGE;
        g->tune.run_max_iterations = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_PULL_STAGING:
        if (value > 1) return grz_set_error(g, GRZ_ERR_ARG, "pull staging must be 0 (loads) or 1 (bulk copies)");
        g->tune.pull_staging = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_CC_PULL_FIRST:
        if (value > 4) return grz_set_error(g, GRZ_ERR_ARG, "CC pull form must be 0..4");
        g->tune.cc_pull_first = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_BFS_PULL_FIRST:
        if (value > 64) return grz_set_error(g, GRZ_ERR_ARG, "BFS pull first pass must read 0..64 vectors");
        g->tune.bfs_pull_first = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_CC_SEGMENTS:
        if (value > 2) return grz_set_error(g, GRZ_ERR_ARG, "CC segments must be 0 (when built), 1 (never) or 2 (build them)");
        g->tune.cc_segments = (uint32_t)value;
        return GRZ_OK;
    case GRZ_TUNE_PR_SEGMENT_BITS:
        if (value > 31 || (value > 1 && value < 8))
            return grz_set_error(g, GRZ_ERR_ARG, "PageRank segment bits must be 0 (by size), 1 (none) or 8..31");
        g->tune.pr_segment_bits = (uint32_t)value;  // from the next grz_pr_init
        return GRZ_OK;
    case GRZ_TUNE_RUN_LIMIT_US:
        if (value > 3600000000ll) return grz_set_error(g, GRZ_ERR_RANGE, "run time bound above one hour");
        g->tune.run_limit_us = (uint32_t)value;
        return GRZ_OK;
    default:
        return grz_set_error(g, GRZ_ERR_ARG, "unknown tuning parameter %d", param);
    }
}

extern "C" int grz_tune_get(const grz_graph* g, int param, int64_t* value)
{
    if (!g || !value) return GRZ_ERR_ARG;
    switch (param) {
    case GRZ_TUNE_HUBS: *value = g->tune.hub_max; return GRZ_OK;
    case GRZ_TUNE_CC_CACHE: *value = g->tune.cc_cache; return GRZ_OK;
    case GRZ_TUNE_CC_THREADS: *value = g->tune.cc_threads; return GRZ_OK;
    case GRZ_TUNE_CC_GRID: *value = g->tune.cc_grid; return GRZ_OK;
    case GRZ_TUNE_PR_GRID: *value = g->tune.pr_grid; return GRZ_OK;
    case GRZ_TUNE_BFS_PULL_SCAN: *value = g->tune.bfs_pull_scan; return GRZ_OK;
    case GRZ_TUNE_PR_PROPS: *value = g->tune.pr_props; return GRZ_OK;
    case GRZ_TUNE_INGEST_CHUNKS: *value = g->tune.ingest_chunks; return GRZ_OK;
    case GRZ_TUNE_PR_PERSISTENT: *value = g->tune.pr_persistent; return GRZ_OK;
    case GRZ_TUNE_PR_WAIT_LIMIT_US: *value = g->tune.pr_wait_limit_us; return GRZ_OK;
    case GRZ_TUNE_PR_WITHHOLD: *value = g->tune.pr_withhold; return GRZ_OK;
    case GRZ_TUNE_RUN_MAX_ITERATIONS: *value = g->tune.run_max_iterations; return GRZ_OK;
    case GRZ_TUNE_RUN_LIMIT_US: *value = g->tune.run_limit_us; return GRZ_OK;
    case GRZ_TUNE_PULL_STAGING: *value = g->tune.pull_staging; return GRZ_OK;
    case GRZ_TUNE_PR_SEGMENT_BITS: *value = g->tune.pr_segment_bits; return GRZ_OK;
    case GRZ_TUNE_CC_SEGMENTS: *value = g->tune.cc_segments; return GRZ_OK;
    case GRZ_TUNE_BFS_PULL_FIRST: *value = g->tune.bfs_pull_first; return GRZ_OK;
    case GRZ_TUNE_CC_PULL_FIRST: *value = g->tune.cc_pull_first; return GRZ_OK;
    case GRZ_TUNE_HUBS_LOADED: *value = g->pull.nhub; return GRZ_OK;
    default: return GRZ_ERR_ARG;
    }
}

extern "C" unsigned long long grz_launch_count(const grz_graph* g) { return g ? g->nlaunch : 0ull; }

// ---------------------------------------------------------------------------------------------
// host-side diagnostics of the 4.124 fixed-point arithmetic the PageRank kernels use

extern "C" int grz_fixed_point_roundtrip(double x, double* out)
{
    if (!out || !(x >= 0.0) || !(x < 16.0)) return GRZ_ERR_ARG;
    *out = fx_to_double(fx_from_double(x));
    return GRZ_OK;
}

extern "C" int grz_fixed_point_sum(const double* xs, uint64_t n, double* out)
{
    if (!out || (n && !xs)) return GRZ_ERR_ARG;
    u128 s = u128_zero();
    for (uint64_t i = 0; i < n; ++i) {
        if (!(xs[i] >= 0.0) || !(xs[i] < 16.0)) return GRZ_ERR_RANGE;
        const u128 t = u128_add(s, fx_from_double(xs[i]));
        if (t.hi < s.hi) return GRZ_ERR_RANGE;  // carry out of bit 127: the sum reached 16
        s = t;
    }
    *out = fx_to_double(s);
    return GRZ_OK;
}
