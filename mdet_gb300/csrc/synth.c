/*
 * synth.c -- seeded synthetic metagenome assemblies (FASTA) for the TNF path.
 *
 * The reference is measured on real assemblies that are not available here;
 * this generator stands in for them with the shapes the workloads call for:
 *   - G genomes, each an order-3 Markov chain (64 contexts x 4 next-base
 *     probabilities) with GC fraction ~ U(0.30, 0.70) and log-normal
 *     per-context perturbations; genome g of a set seeded `seed` uses the
 *     stream seeded seed*1e6+g;
 *   - contig lengths log-normal(ln median, sigma), clamped into
 *     [min_len, max_len] (clamping, not resampling: the lower bound collects
 *     the left tail);
 *   - each contig drawn afresh from a uniformly chosen genome, 0.5% of its
 *     positions replaced by 'N';
 *   - written as FASTA with 60-column lines and LF endings, the layout the
 *     reference's own printFasta writes (cuda/Cuda2.cu:456-480).
 *
 * Everything is integer arithmetic or IEEE +,-,*,/,sqrt (this file must be
 * compiled with -ffp-contract=off), so the same seed gives the same bytes on
 * x86-64 and aarch64.  Contigs are independent streams, so the output does
 * not depend on the thread count.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#define LINE_WIDTH 60

static uint64_t splitmix64(uint64_t* s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct {
    uint64_t s[4];
} xoshiro;

static void xo_seed(xoshiro* x, uint64_t seed) {
    uint64_t sm = seed;
    for (int i = 0; i < 4; ++i) x->s[i] = splitmix64(&sm);
}

static inline uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }

/* xoshiro256** */
static inline uint64_t xo_next(xoshiro* x) {
    uint64_t* s = x->s;
    uint64_t r = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
}

static double xo_unif(xoshiro* x) { return (double)(xo_next(x) >> 11) * (1.0 / 9007199254740992.0); }

/* exp and log from their series, with exact argument reduction steps
 * (ldexp/frexp are exact), so results are identical on every IEEE machine. */
static double det_exp(double x) {
    const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10;
    double kf = floor(x / 0.69314718055994530942 + 0.5);
    double r = (x - kf * ln2_hi) - kf * ln2_lo;
    double term = 1.0, sum = 1.0;
    for (int i = 1; i <= 16; ++i) {
        term = term * r / (double)i;
        sum = sum + term;
    }
    return ldexp(sum, (int)kf);
}

static double det_log(double x) {
    int e;
    double m = frexp(x, &e); /* x = m * 2^e, m in [0.5,1) */
    if (m < 0.70710678118654752440) {
        m = m * 2.0;
        e -= 1;
    }
    double s = (m - 1.0) / (m + 1.0), s2 = s * s, term = s, sum = 0.0;
    for (int k = 1; k <= 41; k += 2) {
        sum = sum + term / (double)k;
        term = term * s2;
    }
    return (double)e * 0.69314718055994530942 + 2.0 * sum;
}

/* Marsaglia's polar method. */
static double det_normal(xoshiro* x) {
    for (;;) {
        double u = 2.0 * xo_unif(x) - 1.0, v = 2.0 * xo_unif(x) - 1.0;
        double s = u * u + v * v;
        if (s >= 1.0 || s == 0.0) continue;
        return u * sqrt(-2.0 * det_log(s) / s);
    }
}

typedef struct {
    uint32_t thr[64][3]; /* cumulative next-base thresholds, base order A,C,G,T */
} genome_model;

static const char kBase[4] = {'A', 'C', 'G', 'T'};

static void build_genome(uint64_t seed, genome_model* g) {
    xoshiro x;
    xo_seed(&x, seed);
    double gc = 0.30 + 0.40 * xo_unif(&x);
    double base_p[4] = {(1.0 - gc) / 2.0, gc / 2.0, gc / 2.0, (1.0 - gc) / 2.0};
    for (int ctx = 0; ctx < 64; ++ctx) {
        double w[4], tot = 0.0;
        for (int b = 0; b < 4; ++b) {
            w[b] = base_p[b] * det_exp(0.25 * det_normal(&x));
            tot = tot + w[b];
        }
        double cum = 0.0;
        for (int b = 0; b < 3; ++b) {
            cum = cum + w[b] / tot;
            double t = cum * 4294967296.0;
            g->thr[ctx][b] = t >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t;
        }
    }
}

static uint32_t header_len(uint64_t k) {
    uint32_t digits = 1;
    while (k >= 10) {
        k /= 10;
        ++digits;
    }
    return 4 + digits + 1; /* ">ctg" + digits + '\n' */
}

static uint64_t record_bytes(uint64_t k, uint32_t L) {
    return (uint64_t)header_len(k) + L + (L + LINE_WIDTH - 1) / LINE_WIDTH;
}

/* Lengths, genome ids and FASTA byte offsets of every record; returns the
 * total FASTA size in bytes. */
uint64_t mdet_synth_plan(uint64_t seed, uint64_t n, uint32_t genomes, uint32_t min_len, uint32_t max_len,
                         double median, double sigma, uint32_t* len, uint32_t* genome, uint64_t* rec_off) {
    xoshiro x;
    xo_seed(&x, seed ^ 0x5EEDC0DEULL);
    double mu = det_log(median);
    uint64_t pos = 0;
    for (uint64_t k = 0; k < n; ++k) {
        double l = det_exp(mu + sigma * det_normal(&x));
        uint32_t L;
        if (l <= (double)min_len)
            L = min_len;
        else if (l >= (double)max_len)
            L = max_len;
        else
            L = (uint32_t)floor(l + 0.5);
        len[k] = L;
        genome[k] = (uint32_t)(((xo_next(&x) >> 32) * (uint64_t)genomes) >> 32);
        rec_off[k] = pos;
        pos += record_bytes(k, L);
    }
    return pos;
}

typedef struct {
    uint64_t seed, n, k0, k1;
    uint32_t genomes;
    const uint32_t* len;
    const uint32_t* genome;
    const uint64_t* rec_off;
    const genome_model* models;
    char* buf;
    uint64_t* seq_off;
    uint64_t* seq_len;
} job;

static void write_contig(const job* jb, uint64_t k) {
    char* p = jb->buf + jb->rec_off[k];
    int h = sprintf(p, ">ctg%llu\n", (unsigned long long)k);
    p += h;
    uint32_t L = jb->len[k];
    jb->seq_off[k] = jb->rec_off[k] + (uint64_t)h;
    jb->seq_len[k] = (uint64_t)L + (L + LINE_WIDTH - 1) / LINE_WIDTH - 1;
    const genome_model* g = &jb->models[jb->genome[k]];
    xoshiro x;
    xo_seed(&x, (jb->seed * 0x100000001B3ULL) ^ (k * 0x9E3779B97F4A7C15ULL + 0x1234567ULL));
    uint32_t ctx = (uint32_t)(xo_next(&x) & 63);
    const uint32_t n_thr = (uint32_t)(0.005 * 4294967296.0);
    uint32_t col = 0;
    for (uint32_t i = 0; i < L; ++i) {
        uint64_t r = xo_next(&x);
        uint32_t rb = (uint32_t)r, rn = (uint32_t)(r >> 32);
        const uint32_t* t = g->thr[ctx];
        uint32_t b = (rb >= t[0]) + (rb >= t[1]) + (rb >= t[2]);
        ctx = ((ctx << 2) | b) & 63;
        *p++ = rn < n_thr ? 'N' : kBase[b];
        if (++col == LINE_WIDTH || i + 1 == L) {
            *p++ = '\n';
            col = 0;
        }
    }
}

static void* run_job(void* arg) {
    const job* jb = (const job*)arg;
    for (uint64_t k = jb->k0; k < jb->k1; ++k) write_contig(jb, k);
    return NULL;
}

/* Writes the FASTA text of every record into buf (size from
 * mdet_synth_plan) and each contig's sequence view: seq_off[k] is the first
 * byte after the header line, seq_len[k] spans the sequence lines including
 * their inner newlines but not the record's final newline -- the view the
 * reference's reader builds (cuda/Cuda2.cu:1521-1530). Returns 0 on success. */
int mdet_synth_write(uint64_t seed, uint64_t n, uint32_t genomes, const uint32_t* len, const uint32_t* genome,
                     const uint64_t* rec_off, char* buf, uint64_t* seq_off, uint64_t* seq_len, int threads) {
    genome_model* models = (genome_model*)malloc(sizeof(genome_model) * (genomes ? genomes : 1));
    if (!models) return 1;
    for (uint32_t g = 0; g < genomes; ++g) build_genome(seed * 1000000ULL + g, &models[g]);
    if (threads <= 0) threads = 1;
    if ((uint64_t)threads > n) threads = n ? (int)n : 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * threads);
    job* jobs = (job*)malloc(sizeof(job) * threads);
    /* byte-balanced split */
    uint64_t total = n ? rec_off[n - 1] + record_bytes(n - 1, len[n - 1]) : 0;
    uint64_t k = 0;
    for (int t = 0; t < threads; ++t) {
        uint64_t target = total / threads * (t + 1);
        uint64_t k1 = k;
        if (t == threads - 1)
            k1 = n;
        else
            while (k1 < n && rec_off[k1] < target) ++k1;
        job jb = {seed, n, k, k1, genomes, len, genome, rec_off, models, buf, seq_off, seq_len};
        jobs[t] = jb;
        k = k1;
    }
    int rc = 0;
    char* created = (char*)calloc(threads, 1);
    for (int t = 0; t < threads; ++t) {
        if (pthread_create(&th[t], NULL, run_job, &jobs[t]) == 0)
            created[t] = 1;
        else
            run_job(&jobs[t]);
    }
    for (int t = 0; t < threads; ++t)
        if (created[t]) pthread_join(th[t], NULL);
    free(created);
    free(jobs);
    free(th);
    free(models);
    return rc;
}
