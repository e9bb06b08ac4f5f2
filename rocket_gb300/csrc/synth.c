/*
 * synth.c -- seeded synthetic proteomes for the all-pair workloads.
 *
 * Stand-in for real proteome files (no dataset is available): a root
 * proteome of protein sequences drawn i.i.d. from a fixed 20-letter amino-acid
 * background, evolved down a random binary tree.  Every branch substitutes each
 * site independently with probability `rate` (drawn per branch, uniform in
 * [rate_lo, rate_hi]); the new residue is drawn from the background (it may
 * equal the old one).  No insertions or deletions.  Leaf i keeps the first
 * counts[i] proteins of the root's list, so proteomes of very different sizes
 * stay related.
 *
 * Root protein lengths are lognormal (median, sigma).  Normal deviates use the
 * Irwin-Hall sum of 12 uniforms, and exp() is computed here from its Taylor
 * series after range reduction, with FP contraction disabled, so the same seed
 * gives the same bytes on x86-64 and aarch64.
 *
 * Output: each leaf as ReadFasta would produce it -- for every protein one
 * '\n' (its header line) followed by the residues.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* amino-acid background, per mille (sums to 1000) */
static const char AA[20] = {'A', 'R', 'N', 'D', 'C', 'Q', 'E', 'G', 'H', 'I',
                            'L', 'K', 'M', 'F', 'P', 'S', 'T', 'W', 'Y', 'V'};
static const int AA_PERMILLE[20] = {83, 55, 41, 55, 14, 39, 67, 71, 23, 59,
                                    99, 58, 24, 39, 47, 65, 53, 11, 29, 68};

static uint32_t g_cum[20]; /* cumulative thresholds on a 32-bit uniform */

static void init_tables(void) {
    uint64_t acc = 0;
    for (int i = 0; i < 20; i++) {
        acc += (uint64_t)AA_PERMILLE[i];
        g_cum[i] = (uint32_t)((acc * 4294967296ull) / 1000ull - (acc == 1000 ? 1 : 0));
    }
}

static inline uint64_t splitmix64(uint64_t *s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* xoshiro128++ style fast generator per node (seeded from splitmix64) */
typedef struct { uint64_t a, b; } rng_t;
static inline uint64_t rng_next(rng_t *r) { /* xorshift128+ */
    uint64_t s1 = r->a;
    const uint64_t s0 = r->b;
    r->a = s0;
    s1 ^= s1 << 23;
    r->b = s1 ^ s0 ^ (s1 >> 17) ^ (s0 >> 26);
    return r->b + s0;
}
static void rng_seed(rng_t *r, uint64_t seed) {
    uint64_t s = seed;
    r->a = splitmix64(&s);
    r->b = splitmix64(&s);
    if (!r->a && !r->b) r->a = 1;
}
static inline double rng_unit(rng_t *r) { /* [0, 1) with 53 bits */
    return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0);
}

static inline uint8_t draw_residue(uint32_t u) {
    int i = 0;
    while (i < 19 && u > g_cum[i]) i++;
    return (uint8_t)AA[i];
}

/* exp(x): x = k ln2 + r, |r| <= ln2/2, Taylor series of e^r, scaled by 2^k. */
static double my_exp(double x) {
    const double LN2_HI = 6.93147180369123816490e-01, LN2_LO = 1.90821492927058770002e-10;
    double kf = x * 1.44269504088896338700e+00;
    long k = (long)(kf < 0 ? kf - 0.5 : kf + 0.5);
    double r = (x - (double)k * LN2_HI) - (double)k * LN2_LO;
    double term = 1.0, sum = 1.0;
    for (int n = 1; n < 24; n++) {
        term = term * r / (double)n;
        sum = sum + term;
    }
    /* scale by 2^k exactly */
    while (k > 0) { sum *= 2.0; k--; }
    while (k < 0) { sum *= 0.5; k++; }
    return sum;
}

static double normal_ih(rng_t *r) { /* Irwin-Hall: sum of 12 uniforms - 6 */
    double s = 0.0;
    for (int i = 0; i < 12; i++) s = s + rng_unit(r);
    return s - 6.0;
}

/* lognormal integer >= 1 with the given median and sigma */
static int64_t lognormal_int(rng_t *r, double median, double sigma) {
    double v = median * my_exp(sigma * normal_ih(r));
    int64_t n = (int64_t)(v + 0.5);
    return n < 1 ? 1 : n;
}

/* Exported: lognormal integers clipped to [lo, hi] (used for protein counts). */
void synth_lognormal_counts(uint64_t seed, int n, double median, double sigma, int64_t lo,
                            int64_t hi, int64_t *out) {
    rng_t r;
    rng_seed(&r, seed ^ 0x1234567ull);
    for (int i = 0; i < n; i++) {
        int64_t v = lognormal_int(&r, median, sigma);
        out[i] = v < lo ? lo : (v > hi ? hi : v);
    }
}

typedef struct {
    int n_leaves;
    const int64_t *counts;    /* proteins kept by each leaf */
    const int64_t *plen;      /* root protein lengths */
    const int64_t *pstart;    /* start of protein p in a node buffer (no separators) */
    double rate_lo, rate_hi;
    uint64_t seed;
    uint8_t **level_buf;      /* one residue buffer per tree depth */
    uint8_t *out;
    const int64_t *leaf_off;  /* output offset of each leaf */
} ctx_t;

static int64_t max_count(const ctx_t *c, int lo, int hi) {
    int64_t m = 0;
    for (int i = lo; i < hi; i++) if (c->counts[i] > m) m = c->counts[i];
    return m;
}

/* node covers leaves [lo, hi); buf holds its residues for the first `need` proteins */
static void descend(ctx_t *c, int lo, int hi, int depth, uint64_t node_id, int64_t need) {
    const uint8_t *buf = c->level_buf[depth];
    if (hi - lo == 1) {
        uint8_t *o = c->out + c->leaf_off[lo];
        const int64_t np = c->counts[lo];
        for (int64_t p = 0; p < np; p++) {
            *o++ = '\n';
            memcpy(o, buf + c->pstart[p], (size_t)c->plen[p]);
            o += c->plen[p];
        }
        return;
    }
    rng_t r;
    rng_seed(&r, c->seed * 0x9E3779B97F4A7C15ull + node_id * 0xD1B54A32D192ED03ull + 7);
    const int mid = lo + 1 + (int)(rng_next(&r) % (uint64_t)(hi - lo - 1));
    const int child_lo[2] = {lo, mid}, child_hi[2] = {mid, hi};
    for (int ch = 0; ch < 2; ch++) {
        rng_t br;
        rng_seed(&br, c->seed ^ (node_id * 2 + 1 + ch) * 0xA24BAED4963EE407ull);
        const double rate = c->rate_lo + (c->rate_hi - c->rate_lo) * rng_unit(&br);
        const uint32_t thr = (uint32_t)(rate * 4294967295.0);
        const int64_t cneed = max_count(c, child_lo[ch], child_hi[ch]);
        const int64_t nres = c->pstart[cneed];
        uint8_t *dst = c->level_buf[depth + 1];
        for (int64_t i = 0; i < nres; i++) {
            uint64_t u = rng_next(&br);
            uint8_t x = buf[i];
            if ((uint32_t)u < thr) x = draw_residue((uint32_t)(u >> 32));
            dst[i] = x;
        }
        descend(c, child_lo[ch], child_hi[ch], depth + 1, node_id * 2 + 1 + ch, cneed);
    }
    (void)need;
}

static int tree_depth(uint64_t seed, int lo, int hi, uint64_t node_id) {
    if (hi - lo == 1) return 0;
    rng_t r;
    rng_seed(&r, seed * 0x9E3779B97F4A7C15ull + node_id * 0xD1B54A32D192ED03ull + 7);
    const int mid = lo + 1 + (int)(rng_next(&r) % (uint64_t)(hi - lo - 1));
    int a = tree_depth(seed, lo, mid, node_id * 2 + 1);
    int b = tree_depth(seed, mid, hi, node_id * 2 + 2);
    return 1 + (a > b ? a : b);
}

/*
 * Protein lengths of the root (first max_proteins proteins).
 */
void synth_protein_lengths(uint64_t seed, int64_t max_proteins, double median, double sigma,
                           int64_t *out) {
    rng_t r;
    rng_seed(&r, seed ^ 0xABCDEF12345ull);
    for (int64_t p = 0; p < max_proteins; p++) out[p] = lognormal_int(&r, median, sigma);
}

/*
 * Sizes: leaf_bytes[i] = counts[i] + sum of the first counts[i] lengths.
 * Fill: writes all leaves into out at leaf_off (exclusive prefix of leaf_bytes).
 * Returns 0, or -1 on allocation failure.
 */
int synth_proteomes(uint64_t seed, int n_leaves, const int64_t *counts, const int64_t *plen,
                    int64_t max_proteins, double rate_lo, double rate_hi, uint8_t *out,
                    const int64_t *leaf_off) {
    init_tables();
    int64_t *pstart = (int64_t *)malloc(sizeof(int64_t) * (size_t)(max_proteins + 1));
    if (!pstart) return -1;
    pstart[0] = 0;
    for (int64_t p = 0; p < max_proteins; p++) pstart[p + 1] = pstart[p] + plen[p];
    ctx_t c;
    c.n_leaves = n_leaves;
    c.counts = counts;
    c.plen = plen;
    c.pstart = pstart;
    c.rate_lo = rate_lo;
    c.rate_hi = rate_hi;
    c.seed = seed;
    c.out = out;
    c.leaf_off = leaf_off;
    const int depth = tree_depth(seed, 0, n_leaves, 0);
    const int64_t need = max_count(&c, 0, n_leaves);
    const int64_t nres = pstart[need];
    c.level_buf = (uint8_t **)calloc((size_t)depth + 2, sizeof(uint8_t *));
    for (int d = 0; d <= depth + 1; d++) {
        c.level_buf[d] = (uint8_t *)malloc((size_t)(nres ? nres : 1));
        if (!c.level_buf[d]) return -1;
    }
    /* root residues */
    rng_t r;
    rng_seed(&r, seed ^ 0x5EEDull);
    for (int64_t i = 0; i < nres; i++) c.level_buf[0][i] = draw_residue((uint32_t)(rng_next(&r) >> 32));
    descend(&c, 0, n_leaves, 0, 0, need);
    for (int d = 0; d <= depth + 1; d++) free(c.level_buf[d]);
    free(c.level_buf);
    free(pstart);
    return 0;
}
