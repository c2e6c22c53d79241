/*
 * scdgen — seeded synthetic graph generators for the SCD engine's parity tests
 * and benchmarks (planted partition, R-MAT, Chung-Lu with planted communities).
 *
 * The reference measures on SNAP graphs that are not available offline; these
 * generators produce graphs of the same shapes.  Every generator returns the
 * undirected edge list as sorted, de-duplicated, self-loop-free pairs (u < v),
 * which is the canonical text order the `convert` tool reads (first-appearance
 * renumbering in the reference, src/convert.cpp:141-170, is then deterministic).
 *
 * Determinism: every random draw is a pure function of (seed, stream, index)
 * (a splitmix64-style hash), all floating point is IEEE basic arithmetic
 * (+ - * / only; log/exp are computed here from series), and the build uses
 * -ffp-contract=off, so x86-64 and aarch64 hosts produce identical graphs at
 * any OpenMP thread count.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

/* ------------------------------------------------------------------------ */
/* counter-based randomness                                                  */

static inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline uint64_t rnd(uint64_t seed, uint64_t stream, uint64_t i) {
    return mix64(mix64(seed * 0xD1B54A32D192ED03ull + stream) ^ (i * 0xAEF17502108EF2D9ull));
}

/* uniform double in [0,1) from the top 53 bits */
static inline double unif(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

/* uniform integer in [0, k) (k >= 1) by 128-bit multiply-high */
static inline uint64_t below(uint64_t h, uint64_t k) {
    return (uint64_t)(((unsigned __int128)h * k) >> 64);
}

/* ------------------------------------------------------------------------ */
/* deterministic log / exp from basic operations                             */

static double det_log(double x) {
    /* x > 0: x = f * 2^e with f in [sqrt(1/2), sqrt(2)), ln f by atanh series */
    int e = 0;
    while (x >= 1.4142135623730951) { x *= 0.5; e++; }
    while (x < 0.7071067811865476) { x *= 2.0; e--; }
    double s = (x - 1.0) / (x + 1.0), s2 = s * s, term = s, sum = 0.0;
    for (int k = 1; k < 60; k += 2) { sum += term / k; term *= s2; }
    return 2.0 * sum + e * 0.6931471805599453;
}

static double det_exp(double x) {
    /* x = k ln2 + r, |r| <= ln2/2, e^r by Taylor series */
    double kf = x / 0.6931471805599453;
    long k = (long)(kf >= 0 ? kf + 0.5 : kf - 0.5);
    double r = x - k * 0.6931471805599453, term = 1.0, sum = 1.0;
    for (int i = 1; i < 30; i++) { term *= r / i; sum += term; }
    while (k > 0) { sum *= 2.0; k--; }
    while (k < 0) { sum *= 0.5; k++; }
    return sum;
}

static double det_pow(double x, double y) { return det_exp(y * det_log(x)); }

/* ------------------------------------------------------------------------ */
/* parallel LSD radix sort of 64-bit keys + dedup                            */

static void radix_sort_u64(uint64_t *keys, int64_t n) {
    if (n < 2) return;
    uint64_t *tmp = (uint64_t *)malloc((size_t)n * sizeof(uint64_t));
    uint64_t mx = 0;
#pragma omp parallel for reduction(| : mx)
    for (int64_t i = 0; i < n; i++) mx |= keys[i];
    int nt = omp_get_max_threads();
    int64_t *hist = (int64_t *)calloc((size_t)nt * 256, sizeof(int64_t));
    uint64_t *src = keys, *dst = tmp;
    for (int shift = 0; shift < 64 && (mx >> shift); shift += 8) {
        memset(hist, 0, (size_t)nt * 256 * sizeof(int64_t));
#pragma omp parallel num_threads(nt)
        {
            int t = omp_get_thread_num();
            int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
            int64_t *h = hist + (size_t)t * 256;
            for (int64_t i = lo; i < hi; i++) h[(src[i] >> shift) & 255]++;
#pragma omp barrier
#pragma omp single
            {
                int64_t run = 0;
                for (int d = 0; d < 256; d++)
                    for (int u = 0; u < nt; u++) {
                        int64_t c = hist[(size_t)u * 256 + d];
                        hist[(size_t)u * 256 + d] = run;
                        run += c;
                    }
            }
            for (int64_t i = lo; i < hi; i++) dst[h[(src[i] >> shift) & 255]++] = src[i];
        }
        uint64_t *s = src; src = dst; dst = s;
    }
    if (src != keys) memcpy(keys, src, (size_t)n * sizeof(uint64_t));
    free(hist);
    free(tmp);
}

/* sorts keys (u<<32|v, u<v), drops duplicates, returns the pair array */
static int64_t finish_edges(uint64_t *keys, int64_t n, uint32_t **out) {
    radix_sort_u64(keys, n);
    int64_t w = 0;
    for (int64_t i = 0; i < n; i++)
        if (w == 0 || keys[i] != keys[w - 1]) keys[w++] = keys[i];
    uint32_t *pairs = (uint32_t *)malloc((size_t)(w ? w : 1) * 2 * sizeof(uint32_t));
#pragma omp parallel for
    for (int64_t i = 0; i < w; i++) {
        pairs[2 * i] = (uint32_t)(keys[i] >> 32);
        pairs[2 * i + 1] = (uint32_t)keys[i];
    }
    free(keys);
    *out = pairs;
    return w;
}

static inline uint64_t edge_key(uint32_t a, uint32_t b) {
    return a < b ? ((uint64_t)a << 32) | b : ((uint64_t)b << 32) | a;
}

/* random permutation of [0,n) (Fisher-Yates, sequential, deterministic) */
static uint32_t *random_perm(uint32_t n, uint64_t seed, uint64_t stream) {
    uint32_t *p = (uint32_t *)malloc((size_t)(n ? n : 1) * sizeof(uint32_t));
    for (uint32_t i = 0; i < n; i++) p[i] = i;
    for (uint32_t i = n; i > 1; i--) {
        uint32_t j = (uint32_t)below(rnd(seed, stream, i), i);
        uint32_t t = p[i - 1]; p[i - 1] = p[j]; p[j] = t;
    }
    return p;
}

/* community sizes with P(s) ∝ 1/s on [smin, smax]; the last one is truncated to fit n */
static uint32_t community_sizes(uint32_t n, uint32_t smin, uint32_t smax, uint64_t seed,
                                uint32_t **starts_out) {
    uint32_t ns = smax - smin + 1;
    double *cdf = (double *)malloc(ns * sizeof(double));
    double acc = 0.0;
    for (uint32_t i = 0; i < ns; i++) { acc += 1.0 / (double)(smin + i); cdf[i] = acc; }
    uint32_t cap = n / smin + 2, k = 0;
    uint32_t *starts = (uint32_t *)malloc((size_t)(cap + 1) * sizeof(uint32_t));
    uint32_t total = 0;
    while (total < n) {
        double u = unif(rnd(seed, 11, k)) * acc;
        uint32_t lo = 0, hi = ns - 1;
        while (lo < hi) { uint32_t mid = (lo + hi) / 2; if (cdf[mid] > u) hi = mid; else lo = mid + 1; }
        uint32_t s = smin + lo;
        if (s > n - total) s = n - total;
        starts[k++] = total;
        total += s;
    }
    starts[k] = n;
    free(cdf);
    *starts_out = starts;
    return k;
}

/* ------------------------------------------------------------------------ */
/* planted partition                                                         */

/*
 * n vertices in communities of size P(s) ∝ 1/s on [smin, smax].  Inside a
 * community of size s, round(s*min(k_in, s-1)/2) distinct pairs are chosen
 * uniformly without replacement (mean internal degree k_in, capped at s-1).
 * round(n*k_in*mu/(1-mu)/2) external edges join uniform random vertex pairs.
 * Vertex ids are a seeded random permutation of the community layout.
 */
int64_t scdgen_planted(uint32_t n, double k_in, double mu, uint32_t smin, uint32_t smax,
                       uint64_t seed, uint32_t **out) {
    uint32_t *starts;
    uint32_t nc = community_sizes(n, smin, smax, seed, &starts);
    uint32_t *perm = random_perm(n, seed, 12);
    int64_t *off = (int64_t *)malloc((size_t)(nc + 1) * sizeof(int64_t));
    off[0] = 0;
    for (uint32_t c = 0; c < nc; c++) {
        uint32_t s = starts[c + 1] - starts[c];
        double k = k_in < (double)(s - 1) ? k_in : (double)(s - 1);
        double t = (double)s * k / 2.0;
        int64_t target = (int64_t)(t + 0.5);
        int64_t pairs = (int64_t)s * (s - 1) / 2;
        if (target > pairs) target = pairs;
        off[c + 1] = off[c] + target;
    }
    int64_t m_int = off[nc];
    int64_t m_ext = mu > 0.0 ? (int64_t)((double)n * k_in * mu / (1.0 - mu) / 2.0 + 0.5) : 0;
    uint64_t *keys = (uint64_t *)malloc((size_t)(m_int + m_ext + 1) * sizeof(uint64_t));

#pragma omp parallel
    {
        uint32_t *pool = NULL;
        int64_t pool_cap = 0;
#pragma omp for schedule(dynamic, 16)
        for (uint32_t c = 0; c < nc; c++) {
            uint32_t base = starts[c], s = starts[c + 1] - starts[c];
            int64_t pairs = (int64_t)s * (s - 1) / 2, target = off[c + 1] - off[c];
            if (pairs > pool_cap) { free(pool); pool_cap = pairs; pool = (uint32_t *)malloc((size_t)pairs * 4); }
            for (int64_t i = 0; i < pairs; i++) pool[i] = (uint32_t)i;
            for (int64_t i = 0; i < target; i++) {   /* partial Fisher-Yates over pair indices */
                int64_t j = i + (int64_t)below(rnd(seed, 13 + ((uint64_t)c << 8), (uint64_t)i), (uint64_t)(pairs - i));
                uint32_t t = pool[i]; pool[i] = pool[j]; pool[j] = t;
                /* pair index -> (a, b), a < b, row-major over the upper triangle */
                uint32_t idx = pool[i], a = 0, row = s - 1;
                while (idx >= row) { idx -= row; a++; row--; }
                uint32_t b = a + 1 + idx;
                keys[off[c] + i] = edge_key(perm[base + a], perm[base + b]);
            }
        }
        free(pool);
    }
    int64_t w = m_int;
    for (int64_t i = 0; i < m_ext; i++) {
        uint32_t a = (uint32_t)below(rnd(seed, 14, (uint64_t)i), n);
        uint32_t b = (uint32_t)below(rnd(seed, 15, (uint64_t)i), n);
        if (a != b) keys[w++] = edge_key(a, b);
    }
    free(off); free(perm); free(starts);
    return finish_edges(keys, w, out);
}

/* ------------------------------------------------------------------------ */
/* R-MAT                                                                     */

/*
 * 2^scale * edge_factor samples; each level picks a quadrant with
 * probabilities a, b, c, d = 1-a-b-c by comparing 32-bit uniforms against
 * integer thresholds.  Symmetrised (u,v)->(min,max), self-loops dropped, deduplicated.
 */
int64_t scdgen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed,
                    uint32_t **out) {
    int64_t samples = ((int64_t)1 << scale) * edge_factor;
    uint64_t ta = (uint64_t)(a * 4294967296.0);
    uint64_t tb = (uint64_t)((a + b) * 4294967296.0);
    uint64_t tc = (uint64_t)((a + b + c) * 4294967296.0);
    uint64_t *keys = (uint64_t *)malloc((size_t)samples * sizeof(uint64_t));
    uint8_t *keep = (uint8_t *)malloc((size_t)samples);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < samples; i++) {
        uint32_t u = 0, v = 0;
        uint64_t h = 0;
        for (int l = 0; l < scale; l++) {
            if ((l & 1) == 0) h = rnd(seed, 21 + (uint64_t)(l >> 1), (uint64_t)i);
            uint64_t r = (l & 1) ? (h >> 32) : (h & 0xffffffffull);
            uint32_t ub = r >= tb, vb = (r >= ta && r < tb) || r >= tc;
            u = (u << 1) | ub;
            v = (v << 1) | vb;
        }
        keep[i] = u != v;
        keys[i] = edge_key(u, v);
    }
    int64_t w = 0;
    for (int64_t i = 0; i < samples; i++)
        if (keep[i]) keys[w++] = keys[i];
    free(keep);
    return finish_edges(keys, w, out);
}

/* ------------------------------------------------------------------------ */
/* Chung-Lu with planted communities                                         */

static uint32_t pick_cdf(const double *cdf, uint32_t lo, uint32_t hi, double u) {
    /* first index i in [lo, hi) with cdf[i] > u (clamped to hi-1) */
    uint32_t end = hi;
    while (lo < hi) { uint32_t mid = lo + (hi - lo) / 2; if (cdf[mid] > u) hi = mid; else lo = mid + 1; }
    return lo < end ? lo : end - 1;
}

/*
 * n vertices with expected degrees w ~ power law (exponent gamma) truncated to
 * [wmin, wmax], grouped into communities of size P(s) ∝ 1/s on [smin, smax].
 * w_in = min((1-mu) w, s-1) of each vertex's weight is sampled inside its community
 * (round(sum w_in / 2) pairs, endpoints ∝ w_in); the rest, w - w_in, is global
 * Chung-Lu (round(sum w_out / 2) pairs, endpoints ∝ w_out).  Ids are permuted.
 */
int64_t scdgen_chunglu(uint32_t n, double gamma, double wmin, double wmax, double mu,
                       uint32_t smin, uint32_t smax, uint64_t seed, uint32_t **out) {
    uint32_t *starts;
    uint32_t nc = community_sizes(n, smin, smax, seed, &starts);
    uint32_t *perm = random_perm(n, seed, 31);
    double g1 = gamma - 1.0;
    double lo_t = det_pow(wmin, -g1), hi_t = det_pow(wmax, -g1);
    double *cin = (double *)malloc((size_t)n * sizeof(double));
    double *cout = (double *)malloc((size_t)n * sizeof(double));
    uint32_t *comm = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    for (uint32_t c = 0; c < nc; c++)
        for (uint32_t v = starts[c]; v < starts[c + 1]; v++) comm[v] = c;
#pragma omp parallel for schedule(static)
    for (uint32_t v = 0; v < n; v++) {
        double u = unif(rnd(seed, 32, v));
        double w = det_pow(lo_t + u * (hi_t - lo_t), -1.0 / g1);
        uint32_t s = starts[comm[v] + 1] - starts[comm[v]];
        double wi = (1.0 - mu) * w;
        if (wi > (double)(s - 1)) wi = (double)(s - 1);
        cin[v] = wi;
        cout[v] = w - wi;
    }
    /* per-community and global prefix sums (sequential: deterministic order) */
    double acc_out = 0.0;
    int64_t *coff = (int64_t *)malloc((size_t)(nc + 1) * sizeof(int64_t));
    coff[0] = 0;
    for (uint32_t c = 0; c < nc; c++) {
        double acc = 0.0;
        for (uint32_t v = starts[c]; v < starts[c + 1]; v++) { acc += cin[v]; cin[v] = acc; }
        coff[c + 1] = coff[c] + (int64_t)(acc / 2.0 + 0.5);
    }
    for (uint32_t v = 0; v < n; v++) { acc_out += cout[v]; cout[v] = acc_out; }
    int64_t m_int = coff[nc], m_ext = (int64_t)(acc_out / 2.0 + 0.5);
    uint64_t *keys = (uint64_t *)malloc((size_t)(m_int + m_ext + 1) * sizeof(uint64_t));
    uint8_t *keep = (uint8_t *)malloc((size_t)(m_int + m_ext + 1));
#pragma omp parallel for schedule(dynamic, 64)
    for (uint32_t c = 0; c < nc; c++) {
        uint32_t b0 = starts[c], b1 = starts[c + 1];
        double tot = cin[b1 - 1];
        for (int64_t i = coff[c]; i < coff[c + 1]; i++) {
            uint32_t a = pick_cdf(cin, b0, b1, unif(rnd(seed, 33, (uint64_t)i)) * tot);
            uint32_t b = pick_cdf(cin, b0, b1, unif(rnd(seed, 34, (uint64_t)i)) * tot);
            keep[i] = a != b;
            keys[i] = edge_key(perm[a], perm[b]);
        }
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m_ext; i++) {
        uint32_t a = pick_cdf(cout, 0, n, unif(rnd(seed, 35, (uint64_t)i)) * acc_out);
        uint32_t b = pick_cdf(cout, 0, n, unif(rnd(seed, 36, (uint64_t)i)) * acc_out);
        keep[m_int + i] = a != b;
        keys[m_int + i] = edge_key(perm[a], perm[b]);
    }
    int64_t w = 0;
    for (int64_t i = 0; i < m_int + m_ext; i++)
        if (keep[i]) keys[w++] = keys[i];
    free(keep); free(cin); free(cout); free(comm); free(coff); free(perm); free(starts);
    return finish_edges(keys, w, out);
}

/* ------------------------------------------------------------------------ */

void scdgen_free(void *p) { free(p); }

/* writes "u v\n" lines (the text format `convert` reads) */
int scdgen_write_text(const char *path, const uint32_t *pairs, int64_t count) {
    FILE *f = fopen(path, "w");
    if (!f) return -1;
    char buf[32];
    for (int64_t i = 0; i < count; i++) {
        int len = snprintf(buf, sizeof buf, "%u %u\n", pairs[2 * i], pairs[2 * i + 1]);
        if (fwrite(buf, 1, (size_t)len, f) != (size_t)len) { fclose(f); return -1; }
    }
    return fclose(f) == 0 ? 0 : -1;
}
