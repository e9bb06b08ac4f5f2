/*
 * phylo_oracle.c -- CPU oracle for the composition-vector (CV) path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (rocket_gb300/) links,
 * loads or calls this file.  It is used by tests/, by __graft_entry__.smoke()
 * as the checker, and by bench.py's CPU-baseline / reference arm.
 *
 * What it restates (paths are relative to the Rocket project root):
 *
 *   1. The GPU key rule of phylogenetics/src/main/cpp/native.cu
 *      - digit mapping            native.cu:50-141
 *      - K/K-1/K-2 window counts  native.cu:220-256 (count_kmers)
 *      - totals n0/n1/n2          native.cu:317-345
 *      - Markov alpha per slot    native.cu:350-400 (double, exact op order,
 *                                 float result, float bits != 0 keeps a slot)
 *      - nnz / sorted selection   native.cu:402-412, 449-458
 *      Two formulations are provided: the literal loop over every dense slot
 *      (oracle_cv_slots, small K) and a loop over (K-1)-prefix candidates
 *      (oracle_cv_candidates).  Tests check that they agree.
 *
 *   2. The Java CPU path, CompositionVectorKernels.java
 *      - buildCPU    :91-145 (float probabilities, keeps alpha == 0,
 *                     Kahan-compensated double norm as DoubleStream.sum)
 *      - compareCPU  :147-168 (float products, recursive pairwise double sum
 *                     sumFloats :211-222)
 *      This is the timed CPU baseline ("port").
 *
 *   3. java.util.Random (48-bit LCG, published algorithm) and the input
 *      generators of BindingsTest.java (generateInput :29-46,
 *      testCompareVector :159-202), so the reference's test sweeps can be
 *      reproduced exactly.
 *
 * Parity status: the reference's CPU path is Java (no JVM here) and its GPU
 * path cannot run on this machine (no GPU) nor be rebuilt on the Arm GPU host
 * (its sources stay out of this repository); the reference tests hold no
 * golden vectors.  Parity against reference OUTPUTS is therefore unpinned;
 * this oracle is pinned by hand-derived known answers of the reference's
 * formula and by the reference tests' own input procedures.
 *
 * Build: see oracle/Makefile (gcc -O2 -ffp-contract=off, no fast-math: the
 * double arithmetic of the alpha rule must round exactly like the GPU's).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* alphabets (native.cu:50-141; CompositionVectorKernels.java:97-101)  */
/* ------------------------------------------------------------------ */

static const uint8_t PROTEIN_MAP[26] = {
    /*A*/0, /*B*/255, /*C*/1, /*D*/2, /*E*/3, /*F*/4, /*G*/5, /*H*/6, /*I*/7,
    /*J*/255, /*K*/8, /*L*/9, /*M*/10, /*N*/11, /*O*/255, /*P*/12, /*Q*/13,
    /*R*/14, /*S*/15, /*T*/16, /*U*/255, /*V*/17, /*W*/18, /*X*/20, /*Y*/19,
    /*Z*/255};
static const uint8_t DNA_MAP[26] = {
    /*A*/0, 255, /*C*/1, 255, 255, 255, /*G*/2, 255, 255, 255, 255, 255, 255,
    255, 255, 255, 255, 255, 255, /*T*/3, 255, 255, 255, 255, 255, 255};

/* alphabet id: 0 = protein (21 symbols), 1 = DNA (4 symbols) */
static inline uint8_t digit_of(int alpha, uint8_t c) {
    if (c >= 'A' && c <= 'Z') return alpha ? DNA_MAP[c - 'A'] : PROTEIN_MAP[c - 'A'];
    return 0xff;
}
static inline uint64_t nsym(int alpha) { return alpha ? 4u : 21u; }

static uint64_t ipow(uint64_t a, int b) {
    uint64_t r = 1;
    while (b-- > 0) r *= a;
    return r;
}

/* ------------------------------------------------------------------ */
/* native-rule counting (native.cu:220-256, 317-345)                   */
/* ------------------------------------------------------------------ */

typedef struct {
    uint32_t *k1, *k2;      /* dense (K-1)- and (K-2)-mer counts */
    uint32_t *k0_codes;     /* sorted distinct K-mer codes */
    uint32_t *k0_counts;    /* their counts */
    uint64_t k0_n;          /* number of distinct K-mers */
    uint32_t n0, n1, n2;    /* totals (uint32 like the reference) */
} counts_t;

static int cmp_u32(const void *a, const void *b) {
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return (x > y) - (x < y);
}

static int count_windows(int alpha, int k, const uint8_t *s, uint64_t len, counts_t *c) {
    const uint64_t A = nsym(alpha);
    const uint64_t t1 = ipow(A, k - 1), t2 = ipow(A, k - 2);
    memset(c, 0, sizeof(*c));
    c->k1 = (uint32_t *)calloc(t1, sizeof(uint32_t));
    c->k2 = (uint32_t *)calloc(t2, sizeof(uint32_t));
    uint32_t *codes = (uint32_t *)malloc((len ? len : 1) * sizeof(uint32_t));
    if (!c->k1 || !c->k2 || !codes) return -1;
    uint64_t nk0 = 0;
    for (uint64_t i = 0; i < len; i++) {
        uint64_t w = 0;
        int j;
        for (j = 0; j <= k; j++) {
            if (j == k - 2) { c->k2[w]++; c->n2++; }
            if (j == k - 1) { c->k1[w]++; c->n1++; }
            if (j == k) { codes[nk0++] = (uint32_t)w; c->n0++; break; }
            if (i + j >= len) break;
            uint8_t d = digit_of(alpha, s[i + j]);
            if (d == 0xff) break;
            w = w * A + d;
        }
    }
    qsort(codes, nk0, sizeof(uint32_t), cmp_u32);
    c->k0_codes = (uint32_t *)malloc((nk0 ? nk0 : 1) * sizeof(uint32_t));
    c->k0_counts = (uint32_t *)malloc((nk0 ? nk0 : 1) * sizeof(uint32_t));
    uint64_t u = 0;
    for (uint64_t i = 0; i < nk0; i++) {
        if (u > 0 && c->k0_codes[u - 1] == codes[i]) c->k0_counts[u - 1]++;
        else { c->k0_codes[u] = codes[i]; c->k0_counts[u] = 1; u++; }
    }
    c->k0_n = u;
    free(codes);
    return 0;
}

static void free_counts(counts_t *c) {
    free(c->k1); free(c->k2); free(c->k0_codes); free(c->k0_counts);
}

static uint32_t k0_lookup(const counts_t *c, uint32_t code) {
    uint64_t lo = 0, hi = c->k0_n;
    while (lo < hi) {
        uint64_t mid = (lo + hi) / 2;
        if (c->k0_codes[mid] < code) lo = mid + 1; else hi = mid;
    }
    return (lo < c->k0_n && c->k0_codes[lo] == code) ? c->k0_counts[lo] : 0;
}

/* Markov alpha, native.cu:387-394, with the reference's operation order. */
static inline float markov_alpha(uint32_t full, uint32_t prefix, uint32_t suffix,
                                 uint32_t middle, uint32_t n0, uint32_t n1, uint32_t n2) {
    double p = (double)full / n0;
    double p0 = (((double)prefix / n1) * ((double)suffix / n1)) / ((double)middle / n2);
    return (float)((p - p0) / p0);
}

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/*
 * Output arrays (capacity cap): keys, alpha bits, and per-key counts
 * (full, prefix, suffix, middle).  Any count pointer may be NULL.
 * Returns nnz (may exceed cap: then only cap entries are written), or
 * -1 on allocation failure, -2 on bad arguments.
 * totals[3] (may be NULL) receives n0, n1, n2.
 */
typedef struct {
    uint32_t *keys, *alpha_bits, *c0, *c1p, *c1s, *c2m;
    int64_t cap;
} cv_out_t;

static int64_t emit(cv_out_t *o, int64_t n, uint32_t key, uint32_t bits, uint32_t c0,
                    uint32_t c1p, uint32_t c1s, uint32_t c2m) {
    if (n < o->cap) {
        o->keys[n] = key;
        o->alpha_bits[n] = bits;
        if (o->c0) o->c0[n] = c0;
        if (o->c1p) o->c1p[n] = c1p;
        if (o->c1s) o->c1s[n] = c1s;
        if (o->c2m) o->c2m[n] = c2m;
    }
    return n + 1;
}

static int check_args(int alpha, int k) {
    if (alpha != 0 && alpha != 1) return -2;
    if (k < 3 || k > 10) return -2;
    if (ipow(nsym(alpha), k) > (1ull << 32)) return -2;  /* keys must fit uint32 */
    return 0;
}

/* Literal restatement: loop over every dense slot (native.cu:350-400). */
int64_t oracle_cv_slots(int alpha, int k, const uint8_t *s, uint64_t len,
                        uint32_t *keys, uint32_t *alpha_bits, uint32_t *c0, uint32_t *c1p,
                        uint32_t *c1s, uint32_t *c2m, int64_t cap, uint32_t *totals) {
    if (check_args(alpha, k)) return -2;
    counts_t c;
    if (count_windows(alpha, k, s, len, &c)) { free_counts(&c); return -1; }
    const uint64_t A = nsym(alpha), t0 = ipow(A, k), t1 = ipow(A, k - 1);
    cv_out_t o = {keys, alpha_bits, c0, c1p, c1s, c2m, cap};
    int64_t n = 0;
    for (uint64_t i = 0; i < t0; i++) {
        uint64_t full = i, prefix = full / A, suffix = full % t1, middle = suffix / A;
        float a = 0.0f;
        uint32_t mc = c.k2[middle], pc = 0, sc = 0, fc = 0;
        do {
            if (mc == 0) break;
            pc = c.k1[prefix];
            if (pc == 0) break;
            sc = c.k1[suffix];
            if (sc == 0) break;
            fc = k0_lookup(&c, (uint32_t)full);
            a = markov_alpha(fc, pc, sc, mc, c.n0, c.n1, c.n2);
        } while (0);
        uint32_t bits = f2u(a);
        if (bits != 0) n = emit(&o, n, (uint32_t)full, bits, fc, pc, sc, mc);
    }
    if (totals) { totals[0] = c.n0; totals[1] = c.n1; totals[2] = c.n2; }
    free_counts(&c);
    return n;
}

/* Candidate formulation: only slots whose prefix and suffix (K-1)-mers were seen. */
int64_t oracle_cv_candidates(int alpha, int k, const uint8_t *s, uint64_t len,
                             uint32_t *keys, uint32_t *alpha_bits, uint32_t *c0, uint32_t *c1p,
                             uint32_t *c1s, uint32_t *c2m, int64_t cap, uint32_t *totals,
                             int64_t *n_candidates) {
    if (check_args(alpha, k)) return -2;
    counts_t c;
    if (count_windows(alpha, k, s, len, &c)) { free_counts(&c); return -1; }
    const uint64_t A = nsym(alpha), t1 = ipow(A, k - 1), t2 = ipow(A, k - 2);
    cv_out_t o = {keys, alpha_bits, c0, c1p, c1s, c2m, cap};
    int64_t n = 0, cand = 0;
    for (uint64_t q = 0; q < t1; q++) {
        uint32_t pc = c.k1[q];
        if (pc == 0) continue;
        uint64_t m = q % t2;
        uint32_t mc = c.k2[m];
        for (uint64_t b = 0; b < A; b++) {
            uint32_t sc = c.k1[m * A + b];
            if (sc == 0) continue;
            cand++;
            uint32_t key = (uint32_t)(q * A + b);
            uint32_t fc = k0_lookup(&c, key);
            float a = markov_alpha(fc, pc, sc, mc, c.n0, c.n1, c.n2);
            uint32_t bits = f2u(a);
            if (bits != 0) n = emit(&o, n, key, bits, fc, pc, sc, mc);
        }
    }
    if (totals) { totals[0] = c.n0; totals[1] = c.n1; totals[2] = c.n2; }
    if (n_candidates) *n_candidates = cand;
    free_counts(&c);
    return n;
}

/* Dense count tables only (for count-parity tests). */
int oracle_count_tables(int alpha, int k, const uint8_t *s, uint64_t len,
                        uint32_t *k1_out, uint32_t *k2_out, uint32_t *totals) {
    if (check_args(alpha, k)) return -2;
    counts_t c;
    if (count_windows(alpha, k, s, len, &c)) { free_counts(&c); return -1; }
    const uint64_t A = nsym(alpha);
    memcpy(k1_out, c.k1, ipow(A, k - 1) * sizeof(uint32_t));
    memcpy(k2_out, c.k2, ipow(A, k - 2) * sizeof(uint32_t));
    totals[0] = c.n0; totals[1] = c.n1; totals[2] = c.n2;
    free_counts(&c);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Java CPU path port (CompositionVectorKernels.java:91-222)           */
/* ------------------------------------------------------------------ */

/* open-addressing map uint32 code -> uint32 count */
typedef struct { uint32_t *key; uint32_t *val; uint64_t mask; } hmap_t;
#define HEMPTY 0xffffffffu

static int hmap_init(hmap_t *h, uint64_t expect) {
    uint64_t cap = 16;
    while (cap < expect * 2 + 16) cap <<= 1;
    h->key = (uint32_t *)malloc(cap * sizeof(uint32_t));
    h->val = (uint32_t *)calloc(cap, sizeof(uint32_t));
    h->mask = cap - 1;
    if (!h->key || !h->val) return -1;
    memset(h->key, 0xff, cap * sizeof(uint32_t));
    return 0;
}
static inline uint64_t hslot(uint32_t k) { return (uint64_t)(k * 0x9E3779B1u) ^ (k >> 15); }
static void hmap_add(hmap_t *h, uint32_t k) {
    uint64_t i = hslot(k) & h->mask;
    while (h->key[i] != HEMPTY && h->key[i] != k) i = (i + 1) & h->mask;
    h->key[i] = k;
    h->val[i]++;
}
static uint32_t hmap_get(const hmap_t *h, uint32_t k) {
    uint64_t i = hslot(k) & h->mask;
    while (h->key[i] != HEMPTY) {
        if (h->key[i] == k) return h->val[i];
        i = (i + 1) & h->mask;
    }
    return 0;
}
static void hmap_free(hmap_t *h) { free(h->key); free(h->val); }

/* countKmers (:170-199): windows of length k made only of alphabet letters. */
static int java_count(int alpha, int k, const uint8_t *s, uint64_t len, hmap_t *h, uint32_t *n) {
    const uint64_t A = nsym(alpha);
    if (hmap_init(h, len / 2 + 16)) return -1;
    *n = 0;
    if (len < (uint64_t)k) return 0;
    for (uint64_t i = 0; i + k <= len; i++) {
        uint64_t w = 0;
        int ok = 1;
        for (int j = 0; j < k; j++) {
            uint8_t d = digit_of(alpha, s[i + j]);
            if (d == 0xff) { ok = 0; break; }
            w = w * A + d;
        }
        if (ok) { hmap_add(h, (uint32_t)w); (*n)++; }
    }
    return 0;
}

typedef struct { uint32_t key; float val; } kv_t;
static int cmp_kv(const void *a, const void *b) {
    uint32_t x = ((const kv_t *)a)->key, y = ((const kv_t *)b)->key;
    return (x > y) - (x < y);
}

/*
 * buildCPU (:91-145).  Probabilities are float (count / (float) n); for every
 * observed (K-2)-mer "middle" and every (before, after) letter pair,
 * p0 = P(suffix) * P(prefix) / P(middle) in float; kept when p0 != 0.
 * norm = DoubleStream.sum of float squares (Kahan-compensated);
 * value = alpha / (float) sqrt(norm).  Output sorted by key.
 * Returns nnz (entries beyond cap are not written) or < 0 on error.
 */
int64_t java_build_cpu(int alpha, int k, const uint8_t *s, uint64_t len,
                       uint32_t *keys, float *values, int64_t cap) {
    if (check_args(alpha, k)) return -2;
    const uint64_t A = nsym(alpha);
    hmap_t h0, h1, h2;
    uint32_t n0, n1, n2;
    if (java_count(alpha, k, s, len, &h0, &n0) || java_count(alpha, k - 1, s, len, &h1, &n1) ||
        java_count(alpha, k - 2, s, len, &h2, &n2))
        return -1;
    const float fn0 = (float)n0, fn1 = (float)n1, fn2 = (float)n2;
    const uint64_t t2 = ipow(A, k - 2);
    uint64_t cap_res = 1024, nres = 0;
    kv_t *res = (kv_t *)malloc(cap_res * sizeof(kv_t));
    double sum = 0.0, comp = 0.0;  /* Kahan, as DoubleStream.sum */
    for (uint64_t slot = 0; slot <= h2.mask; slot++) {
        uint32_t middle = h2.key[slot];
        if (middle == HEMPTY) continue;
        float pm = (float)h2.val[slot] / fn2;
        for (uint64_t before = 0; before < A; before++) {
            uint32_t prefix = (uint32_t)(before * t2 + middle);
            uint32_t cp = hmap_get(&h1, prefix);
            float pp = cp ? (float)cp / fn1 : 0.0f;
            for (uint64_t after = 0; after < A; after++) {
                uint32_t suffix = (uint32_t)(middle * A + after);
                uint32_t cs = hmap_get(&h1, suffix);
                float ps = cs ? (float)cs / fn1 : 0.0f;
                float p0 = ps * pp / pm;
                uint32_t key = (uint32_t)((before * t2 + middle) * A + after);
                uint32_t cf = hmap_get(&h0, key);
                float p = cf ? (float)cf / fn0 : 0.0f;
                if (p0 != 0.0f) {
                    float a = (p - p0) / p0;
                    if (nres == cap_res) {
                        cap_res *= 2;
                        res = (kv_t *)realloc(res, cap_res * sizeof(kv_t));
                    }
                    res[nres].key = key;
                    res[nres].val = a;
                    nres++;
                    double y = (double)(a * a) - comp;
                    double t = sum + y;
                    comp = (t - sum) - y;
                    sum = t;
                }
            }
        }
    }
    float denom = (float)sqrt(sum);
    qsort(res, nres, sizeof(kv_t), cmp_kv);
    for (uint64_t i = 0; i < nres && (int64_t)i < cap; i++) {
        keys[i] = res[i].key;
        values[i] = res[i].val / denom;
    }
    free(res);
    hmap_free(&h0); hmap_free(&h1); hmap_free(&h2);
    return (int64_t)nres;
}

/* sumFloats (:211-222): recursive pairwise sum in double. */
static double sum_floats(const float *l, int64_t n) {
    if (n == 0) return 0.0;
    if (n == 1) return (double)l[0];
    int64_t mid = n / 2;
    return sum_floats(l, mid) + sum_floats(l + mid, n - mid);
}

/* compareCPU (:147-168).  Keys compared as Java int (signed). */
double java_compare_cpu(const int32_t *lk, const float *lv, int64_t nl,
                        const int32_t *rk, const float *rv, int64_t nr) {
    int64_t cap = (nl < nr ? nl : nr) + 1;
    float *ab = (float *)malloc(cap * sizeof(float));
    int64_t m = 0, i = 0, j = 0;
    while (i < nl && j < nr) {
        if (lk[i] == rk[j]) { ab[m++] = lv[i] * rv[j]; i++; }
        else if (lk[i] < rk[j]) i++;
        else j++;
    }
    double r = sum_floats(ab, m);
    free(ab);
    return r;
}

/* ------------------------------------------------------------------ */
/* FP64 compare: exact products, double-double accumulation            */
/* ------------------------------------------------------------------ */
double oracle_compare_fp64(const uint32_t *lk, const float *lv, int64_t nl,
                           const uint32_t *rk, const float *rv, int64_t nr) {
    double s = 0.0, e = 0.0;
    int64_t i = 0, j = 0;
    while (i < nl && j < nr) {
        if (lk[i] == rk[j]) {
            double p = (double)lv[i] * (double)rv[j]; /* exact: 24+24 bits */
            double t = s + p, z = t - s;
            e += (s - (t - z)) + (p - z);
            s = t;
            i++; j++;
        } else if (lk[i] < rk[j]) i++;
        else j++;
    }
    return s + e;
}

/* ------------------------------------------------------------------ */
/* CPU baseline drivers (OpenMP): Java-path build of many proteomes,  */
/* Java-path compare of many pairs.                                     */
/* ------------------------------------------------------------------ */

/* Builds each proteome with java_build_cpu; returns total nnz. */
int64_t java_build_many(int alpha, int k, int n, const uint8_t *const *seqs, const uint64_t *lens,
                        uint32_t **keys, float **values, const int64_t *caps, int64_t *nnz,
                        int threads) {
    int64_t total = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
    for (int i = 0; i < n; i++) {
        nnz[i] = java_build_cpu(alpha, k, seqs[i], lens[i], keys[i], values[i], caps[i]);
        total += nnz[i];
    }
    return total;
}

/* compareCPU over a list of pairs (indices into key/value arrays). */
void java_compare_pairs(int npairs, const int32_t *pi, const int32_t *pj,
                        const int32_t *const *keys, const float *const *values, const int64_t *sizes,
                        double *out, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for schedule(dynamic, 4)
    for (int p = 0; p < npairs; p++) {
        int a = pi[p], b = pj[p];
        out[p] = java_compare_cpu(keys[a], values[a], sizes[a], keys[b], values[b], sizes[b]);
    }
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* java.util.Random (published 48-bit LCG) and BindingsTest generators */
/* ------------------------------------------------------------------ */

typedef struct { uint64_t seed; } jrand_t;
#define JMULT 0x5DEECE66DULL
#define JMASK ((1ULL << 48) - 1)

static void jr_init(jrand_t *r, int64_t seed) { r->seed = ((uint64_t)seed ^ JMULT) & JMASK; }
static int32_t jr_next(jrand_t *r, int bits) {
    r->seed = (r->seed * JMULT + 0xBULL) & JMASK;
    return (int32_t)(int64_t)(r->seed >> (48 - bits));
}
static int32_t jr_next_int(jrand_t *r) { return jr_next(r, 32); }
static int32_t jr_next_int_bound(jrand_t *r, int32_t bound) {
    if ((bound & -bound) == bound) return (int32_t)(((int64_t)bound * (int64_t)jr_next(r, 31)) >> 31);
    int32_t bits, val;
    do {
        bits = jr_next(r, 31);
        val = bits % bound;
    } while ((int32_t)((uint32_t)bits - (uint32_t)val + (uint32_t)(bound - 1)) < 0);
    return val;
}
static float jr_next_float(jrand_t *r) { return (float)jr_next(r, 24) / (float)(1 << 24); }

/* exported thin wrappers for testing the clone itself */
int32_t jrandom_ints(int64_t seed, int n, int32_t bound, int32_t *out) {
    jrand_t r;
    jr_init(&r, seed);
    for (int i = 0; i < n; i++) out[i] = bound > 0 ? jr_next_int_bound(&r, bound) : jr_next_int(&r);
    return 0;
}
int32_t jrandom_floats(int64_t seed, int n, float *out) {
    jrand_t r;
    jr_init(&r, seed);
    for (int i = 0; i < n; i++) out[i] = jr_next_float(&r);
    return 0;
}

/*
 * BindingsTest.generateInput(seed, n, alphabet) (:29-46).  Note that
 * StringBuilder.append((byte) '\n') appends the decimal text "10" (append(int)),
 * so proteins are separated by the two characters '1','0'.
 * Returns the length written (cap must be >= n + 512).
 */
int64_t bindings_generate_input(int64_t seed, int64_t n, int alpha, uint8_t *out, int64_t cap) {
    const char *letters = alpha ? "ACGT" : "ACDEFGHIKLMNPQRSTVWYX";
    const int32_t nl = (int32_t)strlen(letters);
    jrand_t r;
    jr_init(&r, seed);
    int64_t len = 0;
    while (len < n) {
        for (int32_t i = jr_next_int_bound(&r, 500); i > 0; i--) {
            if (len >= cap) return -1;
            out[len++] = (uint8_t)letters[jr_next_int_bound(&r, nl)];
        }
        if (len + 2 > cap) return -1;
        out[len++] = '1';
        out[len++] = '0';
    }
    return len;
}

static int cmp_i32(const void *a, const void *b) {
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* key set for generateKey (:162-167): open addressing on int32 */
typedef struct { int32_t *k; uint8_t *used; uint64_t mask; } iset_t;
static int iset_add(iset_t *s, int32_t key) {
    uint64_t i = ((uint64_t)(uint32_t)key * 0x9E3779B97F4A7C15ULL >> 20) & s->mask;
    while (s->used[i]) {
        if (s->k[i] == key) return 0;
        i = (i + 1) & s->mask;
    }
    s->used[i] = 1;
    s->k[i] = key;
    return 1;
}

/*
 * BindingsTest.testCompareVector(seed, n, overlapRatio) input generation
 * (:159-196).  Writes sizes to sizes[2]; arrays must hold 2n entries each.
 * Keys are sorted as Java int (signed); values keep their generation order.
 * Returns 0, or 1 if a key equals Integer.MIN_VALUE (Math.abs overflow),
 * whose signed order differs from the unsigned order used on the device.
 */
int bindings_compare_case(int64_t seed, int32_t n, double overlap, int32_t *lk, float *lv,
                          int32_t *rk, float *rv, int32_t *sizes) {
    jrand_t r;
    jr_init(&r, seed);
    iset_t set;
    uint64_t cap = 16;
    while (cap < (uint64_t)n * 16 + 64) cap <<= 1;
    set.k = (int32_t *)malloc(cap * sizeof(int32_t));
    set.used = (uint8_t *)calloc(cap, 1);
    set.mask = cap - 1;
    int minval = 0;
#define GENKEY(dst)                                               \
    do {                                                          \
        int32_t _k;                                               \
        for (;;) {                                                \
            int32_t _x = jr_next_int(&r);                         \
            _k = (_x == INT32_MIN) ? INT32_MIN : (_x < 0 ? -_x : _x); \
            if (iset_add(&set, _k)) break;                        \
        }                                                         \
        if (_k == INT32_MIN) minval = 1;                          \
        dst = _k;                                                 \
    } while (0)
    int32_t ls = jr_next_int_bound(&r, n) + n;
    int32_t rs = jr_next_int_bound(&r, n) + n;
    for (int32_t i = 0; i < ls; i++) { GENKEY(lk[i]); lv[i] = jr_next_float(&r); }
    for (int32_t i = 0; i < rs; i++) { GENKEY(rk[i]); rv[i] = jr_next_float(&r); }
    for (int32_t i = 0; i < overlap * n; i++) {
        int32_t kk;
        GENKEY(kk);
        lk[i] = kk;
        rk[i] = kk;
    }
#undef GENKEY
    qsort(lk, ls, sizeof(int32_t), cmp_i32);
    qsort(rk, rs, sizeof(int32_t), cmp_i32);
    sizes[0] = ls;
    sizes[1] = rs;
    free(set.k);
    free(set.used);
    return minval;
}
