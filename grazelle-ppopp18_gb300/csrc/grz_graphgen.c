/*
 * grz_graphgen.c -- fast seeded R-MAT / Erdős–Rényi edge draws (host, OpenMP).
 *
 * Draw-for-draw the same as grazelle/graphgen.py: edge i at bit level l uses
 * splitmix64(i*64 + key + l) against 64-bit thresholds, so both produce
 * identical graphs.  The C version exists only for speed; deduplication and
 * sorting stay in the caller.
 */
#include <stdint.h>

static inline uint64_t splitmix64(uint64_t x)
{
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* raw R-MAT draws: src[i], dst[i] for i in [0, m); thresholds ta <= tb <= tc (a, a+b, a+b+c as 64-bit) */
void grz_gen_rmat_raw(int scale, uint64_t m, uint64_t key, uint64_t ta, uint64_t tb, uint64_t tc, uint64_t* src,
                      uint64_t* dst)
{
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)m; ++ii) {
        const uint64_t i = (uint64_t)ii;
        const uint64_t base = i * 64ull + key;
        uint64_t s = 0, d = 0;
        for (int l = 0; l < scale; ++l) {
            const uint64_t u = splitmix64(base + (uint64_t)l);
            const uint64_t bit = 1ull << (scale - 1 - l);
            if (u >= ta && u < tb) d |= bit;
            else if (u >= tb && u < tc) s |= bit;
            else if (u >= tc) { s |= bit; d |= bit; }
        }
        src[i] = s;
        dst[i] = d;
    }
}

/* raw uniform draws for G(n, m) */
void grz_gen_er_raw(uint64_t n, uint64_t m, uint64_t key, uint64_t* src, uint64_t* dst)
{
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)m; ++ii) {
        const uint64_t i = (uint64_t)ii;
        const uint64_t u = splitmix64(i * 2ull + key);
        const uint64_t w = splitmix64(i * 2ull + 1ull + key);
        src[i] = ((u >> 32) * n) >> 32;
        dst[i] = ((w >> 32) * n) >> 32;
    }
}

/* LSD radix sort of 64-bit keys using `tmp` (same length); `bits` = significant key bits */
void grz_radix_sort_u64(uint64_t* keys, uint64_t* tmp, uint64_t n, int bits)
{
    uint64_t* a = keys;
    uint64_t* b = tmp;
    for (int shift = 0; shift < bits; shift += 16) {
        static uint64_t cnt[65536];
        for (int i = 0; i < 65536; ++i) cnt[i] = 0;
        for (uint64_t i = 0; i < n; ++i) cnt[(a[i] >> shift) & 0xffff]++;
        uint64_t run = 0;
        for (int i = 0; i < 65536; ++i) { const uint64_t c = cnt[i]; cnt[i] = run; run += c; }
        for (uint64_t i = 0; i < n; ++i) b[cnt[(a[i] >> shift) & 0xffff]++] = a[i];
        uint64_t* t = a; a = b; b = t;
    }
    if (a != keys)
        for (uint64_t i = 0; i < n; ++i) keys[i] = a[i];
}

/* removes adjacent duplicates and keys whose two 32-bit halves are equal (self-loops) from a
 * sorted key array; returns the new length */
uint64_t grz_unique_no_loops(uint64_t* keys, uint64_t n)
{
    uint64_t w = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t k = keys[i];
        if ((k >> 32) == (k & 0xffffffffull)) continue;
        if (w > 0 && keys[w - 1] == k) continue;
        keys[w++] = k;
    }
    return w;
}

/* Parallel LSD radix sort of 64-bit keys (16-bit digits, OpenMP): per-thread histograms of a
 * contiguous chunk, a column-major prefix over (digit, thread), then a stable scatter. */
#ifdef _OPENMP
#include <omp.h>
#endif
#include <stdlib.h>

void grz_radix_sort_u64_mt(uint64_t* keys, uint64_t* tmp, uint64_t n, int bits)
{
#ifdef _OPENMP
    const int nt = omp_get_max_threads();
#else
    const int nt = 1;
#endif
    const int B = 65536;
    uint64_t* hist = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)B * (size_t)nt);
    uint64_t* a = keys;
    uint64_t* b = tmp;
    for (int shift = 0; shift < bits; shift += 16) {
#pragma omp parallel num_threads(nt)
        {
#ifdef _OPENMP
            const int t = omp_get_thread_num();
#else
            const int t = 0;
#endif
            uint64_t* h = hist + (size_t)t * B;
            for (int i = 0; i < B; ++i) h[i] = 0;
            const uint64_t lo = n * (uint64_t)t / (uint64_t)nt, hi = n * (uint64_t)(t + 1) / (uint64_t)nt;
            for (uint64_t i = lo; i < hi; ++i) h[(a[i] >> shift) & 0xffff]++;
#pragma omp barrier
#pragma omp single
            {
                uint64_t run = 0;
                for (int d = 0; d < B; ++d)
                    for (int k = 0; k < nt; ++k) {
                        const uint64_t c = hist[(size_t)k * B + d];
                        hist[(size_t)k * B + d] = run;
                        run += c;
                    }
            }
            for (uint64_t i = lo; i < hi; ++i) b[h[(a[i] >> shift) & 0xffff]++] = a[i];
        }
        uint64_t* t2 = a; a = b; b = t2;
    }
    if (a != keys) {
#pragma omp parallel for
        for (int64_t i = 0; i < (int64_t)n; ++i) keys[i] = a[i];
    }
    free(hist);
}

/* key = (src << 32) | dst for both directions of each draw (symmetrised raw edge keys) */
void grz_sym_keys(const uint64_t* src, const uint64_t* dst, uint64_t m, uint64_t* keys)
{
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)m; ++i) {
        keys[2 * i] = (src[i] << 32) | dst[i];
        keys[2 * i + 1] = (dst[i] << 32) | src[i];
    }
}

/* interleaved (src, dst) pairs from sorted keys; swap = 1 if the key is (dst << 32) | src */
void grz_keys_to_pairs(const uint64_t* keys, uint64_t n, int swap, uint64_t* pairs)
{
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const uint64_t hi = keys[i] >> 32, lo = keys[i] & 0xffffffffull;
        pairs[2 * i] = swap ? lo : hi;
        pairs[2 * i + 1] = swap ? hi : lo;
    }
}
