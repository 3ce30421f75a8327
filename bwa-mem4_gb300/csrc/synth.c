/*
 * synth.c -- seeded synthetic job generators for the benchmark workloads.
 *
 * Host-only C (built into libbwasynth.so by build.py).  Every random draw comes
 * from an integer-only counter-based generator keyed by (seed, job/read index,
 * stream), so the same jobs come out on x86 and aarch64 and for any thread
 * count.  Two passes: *_sizes fills the per-job lengths / h0 / w, the caller
 * lays out the sequence buffer, *_fill writes the bases.
 *
 * Workloads (codes 0=A 1=C 2=G 3=T 4=N, bwa's default scoring):
 *   ext1  20,000-job style: target uniform ACGT with N at 0.1%, tlen = qlen+100,
 *         qlen ~ U[1,120]; query = target prefix with 1% substitutions and 0.1%
 *         1-3 bp indel events; h0 ~ U[19,60].
 *   ext2  left/right extension pairs of 2x150 reads: a seed of length U[19,60]
 *         splits the read (qlen per side 0..131), tlen = qlen + w (w = 100),
 *         0.1% SNV / 0.01% indel divergence, 2% of jobs with a 5%-error tail.
 *         Left h0 = seed length, right h0 = seed length + left query length.
 *   ext3  as ext2 with reads 30% 100 / 50% 150 / 20% 250 bp, w per job in
 *         {50, 100, 200}, h0 capped at 250.
 *   res4  mate rescue: 150 bp query (0.5% substitutions) against a 750 bp
 *         window holding the true mate at a near-Gaussian offset (mean 300,
 *         sd ~50); 10% of jobs get an unrelated random window.
 */
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct { uint64_t s; } rng_t;

static inline rng_t rng_for(uint64_t seed, uint64_t idx, uint64_t stream)
{
    rng_t r;
    r.s = mix64(seed ^ mix64(idx * 0xD1B54A32D192ED03ull + stream));
    return r;
}

static inline uint64_t rnext(rng_t *r)
{
    r->s += 0x9E3779B97F4A7C15ull;
    return mix64(r->s);
}

/* uniform in [0, n) */
static inline uint32_t runder(rng_t *r, uint32_t n) { return (uint32_t)(((rnext(r) >> 32) * (uint64_t)n) >> 32); }
/* true with probability num / 1e6 */
static inline int rppm(rng_t *r, uint32_t num) { return runder(r, 1000000u) < num; }

static inline uint8_t rbase(rng_t *r) { return (uint8_t)runder(r, 4); }

/* ------------------------------------------------------------------ ext1 */

void synth_ext1_sizes(uint64_t seed, int64_t n, int32_t *qlen, int32_t *tlen, int32_t *h0, int32_t *w)
{
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        rng_t r = rng_for(seed, (uint64_t)k, 0);
        qlen[k] = 1 + (int32_t)runder(&r, 120);
        tlen[k] = qlen[k] + 100;
        h0[k] = 19 + (int32_t)runder(&r, 42);
        w[k] = 100;
    }
}

void synth_ext1_fill(uint64_t seed, int64_t n, const int64_t *q_off, const int64_t *t_off,
                     const int32_t *qlen, const int32_t *tlen, uint8_t *seq)
{
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        rng_t r = rng_for(seed, (uint64_t)k, 1);
        uint8_t *t = seq + t_off[k], *q = seq + q_off[k];
        for (int i = 0; i < tlen[k]; ++i) t[i] = rppm(&r, 1000) ? 4 : rbase(&r);
        int qi = 0, ti = 0;
        while (qi < qlen[k]) {
            if (rppm(&r, 1000)) { /* 1-3 bp indel event */
                int len = 1 + (int)runder(&r, 3);
                if (runder(&r, 2)) { /* insertion in the query */
                    for (int u = 0; u < len && qi < qlen[k]; ++u) q[qi++] = rbase(&r);
                } else { /* deletion: skip target bases */
                    ti += len;
                }
                continue;
            }
            uint8_t b = ti < tlen[k] ? t[ti] : rbase(&r);
            ++ti;
            if (rppm(&r, 10000)) b = (uint8_t)((b + 1 + runder(&r, 3)) & 3);
            q[qi++] = b;
        }
    }
}

/* ------------------------------------------------------------------ ext2 / ext3 */

/* Per read: geometry shared by its left (job 2r) and right (job 2r+1) extension. */
typedef struct { int rl, L, s0, w; } read_geom;

static read_geom read_geometry(uint64_t seed, int64_t rd, int mixed)
{
    rng_t r = rng_for(seed, (uint64_t)rd, 0);
    read_geom g;
    if (mixed) {
        uint32_t p = runder(&r, 100);
        g.rl = p < 30 ? 100 : (p < 80 ? 150 : 250);
        uint32_t wq = runder(&r, 3);
        g.w = wq == 0 ? 50 : (wq == 1 ? 100 : 200);
    } else {
        g.rl = 150;
        g.w = 100;
    }
    g.L = 19 + (int)runder(&r, 42);
    g.s0 = (int)runder(&r, (uint32_t)(g.rl - g.L + 1));
    return g;
}

void synth_ext2_sizes(uint64_t seed, int64_t n, int mixed, int32_t *qlen, int32_t *tlen, int32_t *h0,
                      int32_t *w)
{
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        read_geom g = read_geometry(seed, k / 2, mixed);
        int left = (k & 1) == 0;
        int ql = left ? g.s0 : g.rl - g.s0 - g.L;
        qlen[k] = ql;
        tlen[k] = ql + g.w;
        int hv = left ? g.L : g.L + g.s0;
        if (mixed && hv > 250) hv = 250;
        h0[k] = hv;
        w[k] = g.w;
    }
}

void synth_ext2_fill(uint64_t seed, int64_t n, int mixed, const int64_t *q_off, const int64_t *t_off,
                     const int32_t *qlen, const int32_t *tlen, uint8_t *seq)
{
    const int64_t nreads = (n + 1) / 2;
#pragma omp parallel for schedule(static)
    for (int64_t rd = 0; rd < nreads; ++rd) {
        read_geom g = read_geometry(seed, rd, mixed);
        rng_t r = rng_for(seed, (uint64_t)rd, 1);
        /* reference window: w bases | read span (rl + slack) | w bases */
        uint8_t ref[250 + 2 * 200 + 64];
        uint8_t rdq[250];
        const int reflen = g.rl + 2 * g.w + 32;
        for (int i = 0; i < reflen; ++i) ref[i] = rbase(&r);
        /* read = ref[w ..] with 0.1% SNV and 0.01% 1-3 bp indels */
        int qi = 0, ti = g.w;
        while (qi < g.rl) {
            if (rppm(&r, 100)) {
                int len = 1 + (int)runder(&r, 3);
                if (runder(&r, 2)) {
                    for (int u = 0; u < len && qi < g.rl; ++u) rdq[qi++] = rbase(&r);
                } else if (ti + len < reflen) {
                    ti += len;
                }
                continue;
            }
            uint8_t b = ti < reflen ? ref[ti] : rbase(&r);
            ++ti;
            if (rppm(&r, 1000)) b = (uint8_t)((b + 1 + runder(&r, 3)) & 3);
            rdq[qi++] = b;
        }
        for (int side = 0; side < 2; ++side) {
            int64_t k = rd * 2 + side;
            if (k >= n) break;
            uint8_t *q = seq + q_off[k], *t = seq + t_off[k];
            const int ql = qlen[k], tl = tlen[k];
            if (side == 0) { /* leftward: reversed read prefix vs reversed ref ending at the seed */
                for (int j = 0; j < ql; ++j) q[j] = rdq[g.s0 - 1 - j];
                for (int i = 0; i < tl; ++i) t[i] = ref[g.w + g.s0 - 1 - i];
            } else {
                const int qs = g.s0 + g.L, ts = g.w + g.s0 + g.L;
                for (int j = 0; j < ql; ++j) q[j] = rdq[qs + j];
                for (int i = 0; i < tl; ++i) t[i] = ts + i < reflen ? ref[ts + i] : 0;
            }
            /* 2% of jobs: a 5%-error tail over the second half of the query */
            rng_t rt = rng_for(seed, (uint64_t)k, 2);
            if (ql > 1 && runder(&rt, 100) < 2)
                for (int j = ql / 2; j < ql; ++j)
                    if (rppm(&rt, 50000)) q[j] = (uint8_t)((q[j] + 1 + runder(&rt, 3)) & 3);
        }
    }
}

/* ------------------------------------------------------------------ res4 */

void synth_res4_sizes(uint64_t seed, int64_t n, int32_t *qlen, int32_t *tlen)
{
    (void)seed;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        qlen[k] = 150;
        tlen[k] = 400 + 4 * 50 + 150;
    }
}

void synth_res4_fill(uint64_t seed, int64_t n, const int64_t *q_off, const int64_t *t_off,
                     const int32_t *qlen, const int32_t *tlen, uint8_t *seq)
{
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        rng_t r = rng_for(seed, (uint64_t)k, 1);
        uint8_t *q = seq + q_off[k], *t = seq + t_off[k];
        const int ql = qlen[k], tl = tlen[k];
        for (int i = 0; i < tl; ++i) t[i] = rbase(&r);
        if (runder(&r, 100) < 10) { /* no true mate */
            for (int j = 0; j < ql; ++j) q[j] = rbase(&r);
            continue;
        }
        /* offset: mean (tl-ql)/2, four-uniform sum (sd ~50), clamped into the window */
        int off = (tl - ql) / 2;
        for (int u = 0; u < 4; ++u) off += (int)runder(&r, 87) - 43;
        if (off < 0) off = 0;
        if (off > tl - ql) off = tl - ql;
        for (int j = 0; j < ql; ++j) {
            uint8_t b = t[off + j];
            if (rppm(&r, 5000)) b = (uint8_t)((b + 1 + runder(&r, 3)) & 3);
            q[j] = b;
        }
    }
}

/* ------------------------------------------------------------------ glb5 */
/*
 * CIGAR stage (ksw_global2 as crates/bwa-mem/src/cigar.rs:400-447 calls it):
 * a read of 100 / 150 / 250 bp (30 / 50 / 20%) against the reference interval
 * it aligned to: 1% substitutions and 0.05%-per-base indel events of 1-3 bp,
 * band w from the caller's rule at bwa's default scoring
 *   max_gap = max(((l+1)/2 - 6) / 1 + 1, 1), w = min((max_gap + |rlen - l| + 1) / 2, 100),
 *   w = max(w, |rlen - l| + 3).
 * The geometry (read length, indel events) comes from stream 1, so the sizes
 * pass and the fill pass walk the same events; bases come from stream 2.
 */

static int glb5_read_len(rng_t *g)
{
    const uint32_t u = runder(g, 10);
    return u < 3 ? 100 : (u < 8 ? 150 : 250);
}

/* One step of the edit walk at query position p: 0 = aligned base,
 * 1 = deletion of *len target bases, 2 = insertion of *len query bases. */
static int glb5_event(rng_t *g, int *len)
{
    if (!rppm(g, 500)) return 0;
    *len = 1 + (int)runder(g, 3);
    return runder(g, 2) ? 1 : 2;
}

void synth_glb5_sizes(uint64_t seed, int64_t n, int32_t *qlen, int32_t *tlen, int32_t *w)
{
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        rng_t g = rng_for(seed, (uint64_t)k, 1);
        const int l = glb5_read_len(&g);
        int rlen = 0;
        for (int p = 0; p < l;) {
            int len = 0;
            const int ev = glb5_event(&g, &len);
            if (ev == 1) rlen += len;
            else if (ev == 2) p += len;
            else { rlen += 1; p += 1; }
        }
        int max_gap = ((l + 1) / 2 - 6) / 1 + 1;
        if (max_gap < 1) max_gap = 1;
        const int diff = rlen > l ? rlen - l : l - rlen;
        int ww = (max_gap + diff + 1) >> 1;
        if (ww > 100) ww = 100;
        if (ww < diff + 3) ww = diff + 3;
        qlen[k] = l;
        tlen[k] = rlen;
        w[k] = ww;
    }
}

void synth_glb5_fill(uint64_t seed, int64_t n, const int64_t *q_off, const int64_t *t_off,
                     const int32_t *qlen, const int32_t *tlen, uint8_t *seq)
{
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        rng_t g = rng_for(seed, (uint64_t)k, 1);
        rng_t r = rng_for(seed, (uint64_t)k, 2);
        uint8_t *q = seq + q_off[k], *t = seq + t_off[k];
        const int l = glb5_read_len(&g);
        int tp = 0;
        for (int p = 0; p < l;) {
            int len = 0;
            const int ev = glb5_event(&g, &len);
            if (ev == 1) {
                for (int x = 0; x < len; ++x) t[tp++] = rbase(&r);
            } else if (ev == 2) {
                for (int x = 0; x < len && p < l; ++x) q[p++] = rbase(&r);
            } else {
                const uint8_t b = rbase(&r);
                t[tp++] = b;
                q[p++] = rppm(&r, 10000) ? (uint8_t)((b + 1 + runder(&r, 3)) & 3) : b;
            }
        }
        (void)qlen;
        (void)tlen;
    }
}
