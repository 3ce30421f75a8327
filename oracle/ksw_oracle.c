/*
 * ksw_oracle.c -- CPU restatement of bwa-mem4's banded seed extension
 * (ksw_extend2) and mate-rescue local Smith-Waterman (ksw_local_fwd /
 * ksw_align2 / batched_ksw_align2).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA kernels.  Nothing in the
 * product library calls into this file.
 *
 * Written from the reference's documented semantics; each function cites the
 * file:line of the reference code it restates.  Integer behaviour (tie-breaks,
 * the zero sentinel, the f64 band clamp, the stale-state adaptive band) is kept
 * exactly; the code layout is not the reference's.
 */
#include "ksw_oracle.h"

#include <limits.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Rust's `f64 as i32`: truncate toward zero, saturate, NaN -> 0 (the band
 * clamp relies on truncation toward zero, crates/bwa-extend/src/sw.rs:296-308). */
static int trunc_sat(double x)
{
    if (x != x) return 0;
    if (x >= 2147483647.0) return INT_MAX;
    if (x <= -2147483648.0) return INT_MIN;
    return (int)x;
}

/* Largest entry of the m*m matrix (sw.rs:292, batched.rs:965). */
static int mat_max(int m, const int8_t *mat)
{
    int mx = 0;
    for (int k = 0; k < m * m; ++k)
        if (k == 0 || mat[k] > mx) mx = mat[k];
    return mx;
}

static inline int imax2(int a, int b) { return a > b ? a : b; }

void ko_fill_scmat(int a, int b, int8_t mat[25])
{
    /* crates/bwa-core/src/opt.rs:445-482: +a on the diagonal, -b off it, -1 on the N row/col. */
    for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c)
            mat[r * 5 + c] = (r == 4 || c == 4) ? (int8_t)-1
                                                : (r == c ? (int8_t)a : (int8_t)(-(int8_t)b));
}

int ko_clamp_band(int w, int qlen, int max_sc, int end_bonus, int o_ins, int e_ins,
                  int o_del, int e_del)
{
    /* crates/bwa-neon/src/batched.rs:1305-1329 (== sw.rs:296-308): the widest gap that can
     * still pay for itself, computed in double and truncated toward zero, floored at 1. */
    int max_ins = trunc_sat(((double)qlen * max_sc + end_bonus - o_ins) / e_ins + 1.0);
    if (max_ins < 1) max_ins = 1;
    if (w > max_ins) w = max_ins;
    int max_del = trunc_sat(((double)qlen * max_sc + end_bonus - o_del) / e_del + 1.0);
    if (max_del < 1) max_del = 1;
    if (w > max_del) w = max_del;
    return w;
}

/* ------------------------------------------------------------------------- */
/* Banded seed extension                                                      */
/* ------------------------------------------------------------------------- */

ko_ext_result ko_extend2(const uint8_t *q, int qlen, const uint8_t *t, int tlen,
                         int m, const int8_t *mat, int o_del, int e_del,
                         int o_ins, int e_ins, int w, int end_bonus, int zdrop,
                         int h0, uint64_t *cells)
{
    /* crates/bwa-extend/src/sw.rs:203-493.  hrow[j] holds H(i-1, j-1) on entry to column j
     * and H(i, j-1) after it; erow[j] holds E(i, j).  Both persist across rows: cells
     * outside the live window keep whatever an earlier row (or the row -1 init) left. */
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;
    int32_t *hrow = (int32_t *)calloc((size_t)qlen + 2, sizeof(int32_t));
    int32_t *erow = (int32_t *)calloc((size_t)qlen + 2, sizeof(int32_t));

    /* Row -1: h0 at column -1, then an insertion chain that stops while still > e_ins
     * (sw.rs:269-279).  The qlen >= 1 guard is the lockstep path's (batched.rs:1025-1031). */
    hrow[0] = h0;
    if (qlen >= 1) hrow[1] = h0 > oe_ins ? h0 - oe_ins : 0;
    for (int j = 2; j <= qlen && hrow[j - 1] > e_ins; ++j) hrow[j] = hrow[j - 1] - e_ins;

    if (w < 0) w = 0; /* negative bands are rejected at the C ABI; never exercised */
    w = ko_clamp_band(w, qlen, mat_max(m, mat), end_bonus, o_ins, e_ins, o_del, e_del);

    int best = h0, best_i = -1, best_j = -1, best_ie = -1, gscore = -1, max_off = 0;
    int beg = 0, end = qlen;
    uint64_t nc = 0;
    for (int i = 0; i < tlen; ++i) {
        const int8_t *srow = mat + (size_t)t[i] * m;
        /* band intersection (sw.rs:342-351): beg only grows, end only shrinks */
        if (beg < i - w) beg = i - w;
        if (end > i + w + 1) end = i + w + 1;
        if (end > qlen) end = qlen;
        /* H(i, beg-1): reachable by a deletion from the origin only while beg == 0 (sw.rs:355-360) */
        int h1 = beg == 0 ? imax2(h0 - (o_del + e_del * (i + 1)), 0) : 0;
        int f = 0, rmax = 0, mj = -1, j;
        for (j = beg; j < end; ++j) {
            int hd = hrow[j], e = erow[j];
            hrow[j] = h1;
            int M = hd != 0 ? hd + srow[q[j]] : 0; /* zero diagonal is never extended (sw.rs:377-381) */
            int h = M > e ? M : e;
            h = h > f ? h : f;
            h1 = h;
            if (!(rmax > h)) { mj = j; rmax = h; } /* ties move to the later column (sw.rs:390-391) */
            /* gaps open from M (sw.rs:402-413) */
            int open = imax2(M - oe_del, 0);
            e -= e_del;
            erow[j] = e > open ? e : open;
            open = imax2(M - oe_ins, 0);
            f -= e_ins;
            f = f > open ? f : open;
        }
        if (end > beg) nc += (uint64_t)(end - beg);
        hrow[end] = h1; /* sentinel column (sw.rs:418-419) */
        erow[end] = 0;
        if (j == qlen && gscore <= h1) { best_ie = i; gscore = h1; } /* later row wins (sw.rs:424-427) */
        if (rmax == 0) break;
        if (rmax > best) {
            best = rmax; best_i = i; best_j = mj;
            int off = mj > i ? mj - i : i - mj;
            if (off > max_off) max_off = off;
        } else if (zdrop > 0) { /* sw.rs:440-456 */
            if (i - best_i > mj - best_j) {
                if (best - rmax - ((i - best_i) - (mj - best_j)) * e_del > zdrop) break;
            } else if (best - rmax - ((mj - best_j) - (i - best_i)) * e_ins > zdrop) {
                break;
            }
        }
        /* adaptive band (sw.rs:465-482): trim dead columns; end may grow by up to two */
        int lo = beg;
        while (lo < end && hrow[lo] == 0 && erow[lo] == 0) ++lo;
        beg = lo;
        int hi = end;
        while (hi >= beg && hrow[hi] == 0 && erow[hi] == 0) --hi;
        end = hi + 2 < qlen ? hi + 2 : qlen;
    }
    free(hrow);
    free(erow);
    if (cells) *cells = nc;
    ko_ext_result r = {best, best_j + 1, best_i + 1, best_ie + 1, gscore, max_off};
    return r;
}

void ko_extend_lockstep(int n, const uint8_t *const *qs, const int *qlens,
                        const uint8_t *const *ts, const int *tlens, const int *h0s,
                        int m, const int8_t *mat, int o_del, int e_del, int o_ins,
                        int e_ins, int w0, int end_bonus, int zdrop, int lanes,
                        ko_ext_result *out)
{
    /* crates/bwa-neon/src/batched.rs:947-1251: `lanes` jobs advance one shared row counter;
     * each keeps its own band, trackers and a private row buffer (lane-major here). */
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;
    const int max_sc = mat_max(m, mat);
    if (lanes < 1) lanes = 1;
    int *qlen = malloc(sizeof(int) * lanes), *tlen = malloc(sizeof(int) * lanes);
    int *h0 = malloc(sizeof(int) * lanes), *w = malloc(sizeof(int) * lanes);
    int *beg = malloc(sizeof(int) * lanes), *end = malloc(sizeof(int) * lanes);
    int *best = malloc(sizeof(int) * lanes), *bi = malloc(sizeof(int) * lanes);
    int *bj = malloc(sizeof(int) * lanes), *bie = malloc(sizeof(int) * lanes);
    int *gs = malloc(sizeof(int) * lanes), *moff = malloc(sizeof(int) * lanes);
    int *done = malloc(sizeof(int) * lanes), *act = malloc(sizeof(int) * lanes);
    int *h1 = malloc(sizeof(int) * lanes), *f = malloc(sizeof(int) * lanes);
    int *rmax = malloc(sizeof(int) * lanes), *mj = malloc(sizeof(int) * lanes);
    for (int c0 = 0; c0 < n; c0 += lanes) {
        int nl = n - c0 < lanes ? n - c0 : lanes;
        int maxq = 0, maxt = 0;
        for (int l = 0; l < nl; ++l) {
            qlen[l] = qlens[c0 + l]; tlen[l] = tlens[c0 + l]; h0[l] = h0s[c0 + l];
            w[l] = ko_clamp_band(w0, qlen[l], max_sc, end_bonus, o_ins, e_ins, o_del, e_del);
            if (qlen[l] > maxq) maxq = qlen[l];
            if (tlen[l] > maxt) maxt = tlen[l];
        }
        const int stride = maxq + 1;
        int32_t *H = calloc((size_t)lanes * stride, sizeof(int32_t));
        int32_t *E = calloc((size_t)lanes * stride, sizeof(int32_t));
        for (int l = 0; l < nl; ++l) {
            int32_t *hr = H + (size_t)l * stride;
            hr[0] = h0[l];
            if (qlen[l] >= 1) hr[1] = h0[l] > oe_ins ? h0[l] - oe_ins : 0;
            for (int j = 2; j <= qlen[l] && hr[j - 1] > e_ins; ++j) hr[j] = hr[j - 1] - e_ins;
            best[l] = h0[l]; bi[l] = -1; bj[l] = -1; bie[l] = -1; gs[l] = -1; moff[l] = 0;
            beg[l] = 0; end[l] = qlen[l]; done[l] = 0;
        }
        for (int i = 0; i < maxt; ++i) {
            int gb = INT_MAX, ge = 0;
            for (int l = 0; l < nl; ++l) {
                act[l] = !done[l] && i < tlen[l];
                if (!act[l]) continue;
                if (beg[l] < i - w[l]) beg[l] = i - w[l];
                if (end[l] > i + w[l] + 1) end[l] = i + w[l] + 1;
                if (end[l] > qlen[l]) end[l] = qlen[l];
                h1[l] = beg[l] == 0 ? imax2(h0[l] - (o_del + e_del * (i + 1)), 0) : 0;
                f[l] = 0; rmax[l] = 0; mj[l] = -1;
                if (beg[l] < gb) gb = beg[l];
                if (end[l] > ge) ge = end[l];
            }
            for (int j = gb; j < ge; ++j) {
                for (int l = 0; l < nl; ++l) {
                    if (!act[l] || j < beg[l] || j >= end[l]) continue;
                    int32_t *hr = H + (size_t)l * stride, *er = E + (size_t)l * stride;
                    int M = hr[j], e = er[j];
                    hr[j] = h1[l];
                    int sc = mat[(size_t)ts[c0 + l][i] * m + qs[c0 + l][j]];
                    M = M != 0 ? M + sc : 0;
                    int h = imax2(imax2(M, e), f[l]);
                    h1[l] = h;
                    if (rmax[l] <= h) { mj[l] = j; rmax[l] = h; }
                    er[j] = imax2(e - e_del, imax2(M - oe_del, 0));
                    f[l] = imax2(f[l] - e_ins, imax2(M - oe_ins, 0));
                }
            }
            for (int l = 0; l < nl; ++l) {
                if (!act[l]) continue;
                int32_t *hr = H + (size_t)l * stride, *er = E + (size_t)l * stride;
                hr[end[l]] = h1[l];
                er[end[l]] = 0;
                if (end[l] == qlen[l] && gs[l] <= h1[l]) { bie[l] = i; gs[l] = h1[l]; }
                if (rmax[l] == 0) { done[l] = 1; continue; }
                if (rmax[l] > best[l]) {
                    best[l] = rmax[l]; bi[l] = i; bj[l] = mj[l];
                    int off = mj[l] > i ? mj[l] - i : i - mj[l];
                    if (off > moff[l]) moff[l] = off;
                } else if (zdrop > 0) {
                    int drop = (i - bi[l] > mj[l] - bj[l])
                                   ? best[l] - rmax[l] - ((i - bi[l]) - (mj[l] - bj[l])) * e_del
                                   : best[l] - rmax[l] - ((mj[l] - bj[l]) - (i - bi[l])) * e_ins;
                    if (drop > zdrop) { done[l] = 1; continue; }
                }
                int lo = beg[l];
                while (lo < end[l] && hr[lo] == 0 && er[lo] == 0) ++lo;
                beg[l] = lo;
                int hi = end[l];
                while (hi >= beg[l] && hr[hi] == 0 && er[hi] == 0) --hi;
                end[l] = hi + 2 < qlen[l] ? hi + 2 : qlen[l];
            }
        }
        for (int l = 0; l < nl; ++l) {
            ko_ext_result r = {best[l], bj[l] + 1, bi[l] + 1, bie[l] + 1, gs[l], moff[l]};
            out[c0 + l] = r;
        }
        free(H);
        free(E);
    }
    free(qlen); free(tlen); free(h0); free(w); free(beg); free(end); free(best); free(bi);
    free(bj); free(bie); free(gs); free(moff); free(done); free(act); free(h1); free(f);
    free(rmax); free(mj);
}

int ko_ref_extend(const uint8_t *q, int qlen, const uint8_t *t, int tlen, int m,
                  const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins, int h0)
{
    /* crates/bwa-extend/src/sw.rs:1255-1310: the same recurrence with no band, no z-drop
     * and no zero-row break; only the best local score. */
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;
    int32_t *H = calloc((size_t)qlen + 2, sizeof(int32_t));
    int32_t *E = calloc((size_t)qlen + 2, sizeof(int32_t));
    H[0] = h0;
    if (qlen >= 1) H[1] = h0 > oe_ins ? h0 - oe_ins : 0;
    for (int j = 2; j <= qlen && H[j - 1] > e_ins; ++j) H[j] = H[j - 1] - e_ins;
    int best = h0;
    for (int i = 0; i < tlen; ++i) {
        int f = 0, h1 = imax2(h0 - (o_del + e_del * (i + 1)), 0);
        for (int j = 0; j < qlen; ++j) {
            int M = H[j], e = E[j];
            H[j] = h1;
            M = M != 0 ? M + mat[(size_t)t[i] * m + q[j]] : 0;
            int h = imax2(imax2(M, e), f);
            h1 = h;
            if (h > best) best = h;
            E[j] = imax2(e - e_del, imax2(M - oe_del, 0));
            f = imax2(f - e_ins, imax2(M - oe_ins, 0));
        }
        H[qlen] = h1;
        E[qlen] = 0;
    }
    free(H);
    free(E);
    return best;
}

int ko_x_threshold(int a, int b, int o_del, int e_del, int o_ins, int e_ins)
{
    /* crates/bwa-neon/src/batched.rs:756-764: the ungapped walk is provably optimal while
     * X*(a+b) < o_min + e_min. */
    int o_min = o_del < o_ins ? o_del : o_ins, e_min = e_del < e_ins ? e_del : e_ins;
    int denom = a + b;
    return denom > 0 ? (o_min + e_min - 1) / denom : -1;
}

int ko_ungapped_hit(const uint8_t *q, int qlen, const uint8_t *t, int tlen, int h0,
                    int a, int b, int x_threshold, int zdrop, ko_ext_result *out)
{
    /* crates/bwa-neon/src/batched.rs:602-697. */
    if (qlen == 0 || h0 <= 0 || tlen < qlen || x_threshold < 0) return 0;
    int nmis = 0;
    for (int c = 0; c < qlen; ++c) {
        if (q[c] >= 4 || t[c] >= 4) return 0;
        if (q[c] != t[c]) {
            if (++nmis > x_threshold) return 0;
            if (c >= 128) return 0; /* the reference's mismatch bitmap holds 128 columns */
        }
    }
    if (nmis == 0) {
        int s = h0 + qlen * a;
        ko_ext_result r = {s, qlen, qlen, qlen, s, 0};
        *out = r;
        return 1;
    }
    if (qlen > 128) return 0;
    int run = h0, bs = h0, be = 0;
    for (int c = 0; c < qlen; ++c) {
        if (run == 0) continue;
        if (q[c] == t[c]) run += a;
        else { run -= b; if (run < 0) run = 0; }
        if (run > bs) { bs = run; be = c + 1; }
        else if (zdrop > 0 && bs - run > zdrop) return 0;
    }
    if (run == 0) return 0;
    ko_ext_result r = {bs, be, be, qlen, run, 0};
    *out = r;
    return 1;
}

static int is_uniform_dna(int m, const int8_t *mat)
{
    /* crates/bwa-neon/src/batched.rs:480-515 */
    if (m < 2) return 0;
    int a = mat[0], mm = mat[1], npen = mat[m - 1];
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) {
            int want = (i == m - 1 || j == m - 1) ? npen : (i == j ? a : mm);
            if (mat[i * m + j] != want) return 0;
        }
    return 1;
}

int ko_ext_bin(int qlen, int tlen, int h0, int m, const int8_t *mat)
{
    /* crates/bwa-neon/src/batched.rs:817-865 (non-uniform matrices never reach the bins and
     * run the scalar path, batched.rs:730-735). */
    if (!is_uniform_dna(m, mat)) return 2;
    int max_sc = mat_max(m, mat);
    int head = imax2(imax2(-(int)mat[1], -(int)mat[m - 1]), 0) + max_sc;
    int bound = h0 + (qlen < tlen ? qlen : tlen) * imax2(max_sc, 0);
    if (qlen < 256 && tlen < 256 && bound + head < 256) return 0;
    if (qlen < 32768 && tlen < 32768 && bound + head < 32768) return 1;
    return 2;
}

/* ------------------------------------------------------------------------- */
/* Mate rescue                                                                */
/* ------------------------------------------------------------------------- */

int ko_padded_qlen(int qlen, int max_sc)
{
    /* crates/bwa-neon/src/matesw.rs:676-686: bwa's l_ms * a < 250 picks the 16-wide profile. */
    int lanes = qlen * max_sc < 250 ? 16 : 8;
    return (qlen + lanes - 1) / lanes * lanes;
}

static int mat_is_standard(int m, const int8_t *mat)
{
    /* crates/bwa-neon/src/matesw.rs:895-915 */
    if (m != 5) return 0;
    int mt = mat[0], mis = mat[1];
    for (int i = 0; i < 4; ++i) {
        for (int j = 0; j < 4; ++j)
            if (mat[i * 5 + j] != (i == j ? mt : mis)) return 0;
        if (mat[i * 5 + 4] != -1 || mat[20 + i] != -1) return 0;
    }
    return mat[24] == -1;
}

int ko_rescue_width(int n, const int *qlens, const int *tlens, int m, const int8_t *mat,
                    int max_sc)
{
    /* crates/bwa-neon/src/matesw.rs:780-795: the whole batch takes one width. */
    if (!mat_is_standard(m, mat)) return 2;
    int u8ok = 1, i16ok = 1;
    for (int k = 0; k < n; ++k) {
        int ceil = (qlens[k] < tlens[k] ? qlens[k] : tlens[k]) * max_sc;
        if (!(ceil < 250 && qlens[k] < 250)) u8ok = 0;
        if (!(ceil < 30000 && tlens[k] < 30000)) i16ok = 0;
    }
    return u8ok ? 0 : (i16ok ? 1 : 2);
}

typedef struct { int32_t score, row; } sub_entry;
typedef struct { sub_entry *v; int n, cap; } sub_tracker;

static void tracker_push(sub_tracker *b, int row, int row_max, int minsc)
{
    /* crates/bwa-extend/src/sw.rs:806-829: a row directly after the last entry's row merges,
     * and the stored row advances only when the score improves. */
    if (row_max < minsc) return;
    if (b->n > 0 && b->v[b->n - 1].row + 1 == row) {
        if (b->v[b->n - 1].score < row_max) { b->v[b->n - 1].score = row_max; b->v[b->n - 1].row = row; }
        return;
    }
    if (b->n == b->cap) {
        b->cap = b->cap ? 2 * b->cap : 16;
        b->v = realloc(b->v, sizeof(sub_entry) * (size_t)b->cap);
    }
    b->v[b->n].score = row_max;
    b->v[b->n].row = row;
    b->n++;
}

static void tracker_finish(const sub_tracker *b, int gmax, int te, int max_sc, int *s2, int *t2)
{
    /* crates/bwa-extend/src/sw.rs:831-851: best entry outside |row - te| <= ceil(gmax/max_sc);
     * the first entry wins ties; -1/-1 when nothing qualifies. */
    int score2 = -1, te2 = -1;
    if (gmax > 0 && b->n > 0) {
        int hw = (gmax + max_sc - 1) / max_sc;
        int lo = te - hw, hi = te + hw;
        for (int k = 0; k < b->n; ++k)
            if ((b->v[k].row < lo || b->v[k].row > hi) && b->v[k].score > score2) {
                score2 = b->v[k].score;
                te2 = b->v[k].row;
            }
    }
    *s2 = score2;
    *t2 = te2;
}

ko_fwd_result ko_local_fwd(const uint8_t *q, int qlen_real, const uint8_t *t, int tlen,
                           int m, const int8_t *mat, int o_del, int e_del, int o_ins,
                           int e_ins, int minsc, int endsc, int max_sc, int lanes)
{
    /* crates/bwa-extend/src/sw.rs:921-1075.  Full rectangle, gaps open from H, the query
     * padded to a multiple of `lanes` with score-0 columns that carry the diagonal. */
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;
    const int qlen = (qlen_real + lanes - 1) / lanes * lanes;
    int32_t *hp = calloc((size_t)qlen + 1, sizeof(int32_t));
    int32_t *hc = calloc((size_t)qlen + 1, sizeof(int32_t));
    int32_t *E = calloc((size_t)qlen + 1, sizeof(int32_t));
    int32_t *hbest = calloc((size_t)qlen + 1, sizeof(int32_t));
    sub_tracker b = {0, 0, 0};
    int gmax = 0, te = -1;
    for (int i = 0; i < tlen; ++i) {
        const int8_t *srow = mat + (size_t)t[i] * m;
        int f = 0, hd = 0, rmax = 0;
        for (int j = 0; j < qlen; ++j) {
            int sc = j < qlen_real ? srow[q[j]] : 0;
            int h = hd + sc;
            if (h < 0) h = 0;
            if (E[j] > h) h = E[j];
            if (f > h) h = f;
            if (h > rmax) rmax = h;
            hc[j] = h;
            int en = E[j] - e_del, od = h - oe_del; /* E and F open from H (sw.rs:1007-1029) */
            if (od > en) en = od;
            E[j] = en > 0 ? en : 0;
            int fn = f - e_ins, oi = h - oe_ins;
            if (oi > fn) fn = oi;
            f = fn > 0 ? fn : 0;
            hd = hp[j];
        }
        tracker_push(&b, i, rmax, minsc);
        if (rmax > gmax) { /* first row reaching the max keeps te (sw.rs:1035-1044) */
            gmax = rmax;
            te = i;
            memcpy(hbest, hc, sizeof(int32_t) * (size_t)qlen);
            if (gmax >= endsc) break;
        }
        int32_t *tmp = hp; hp = hc; hc = tmp;
    }
    /* qe: smallest column attaining the max in row te (sw.rs:1050-1070; the striped scan
     * order of the reference is irrelevant because ties take the smaller column). */
    int qe = -1;
    if (te >= 0) {
        int bh = -1;
        for (int j = 0; j < qlen; ++j)
            if (hbest[j] > bh) { bh = hbest[j]; qe = j; }
    }
    ko_fwd_result r;
    r.score = gmax; r.te = te; r.qe = qe;
    tracker_finish(&b, gmax, te, max_sc, &r.score2, &r.te2);
    free(b.v); free(hp); free(hc); free(E); free(hbest);
    return r;
}

ko_aln_result ko_align2_scalar(const uint8_t *q, int qlen, const uint8_t *t, int tlen,
                               int m, const int8_t *mat, int o_del, int e_del,
                               int o_ins, int e_ins, int minsc, int max_sc, int lanes)
{
    /* crates/bwa-extend/src/sw.rs:1108-1185 */
    ko_fwd_result fw = ko_local_fwd(q, qlen, t, tlen, m, mat, o_del, e_del, o_ins, e_ins,
                                    minsc, INT_MAX, max_sc, lanes);
    ko_aln_result r = {fw.score, -1, fw.qe, -1, fw.te, fw.score2, fw.te2};
    if (fw.score < minsc || fw.qe < 0) return r;
    uint8_t *qr = malloc((size_t)fw.qe + 1), *tr = malloc((size_t)tlen);
    for (int k = 0; k <= fw.qe; ++k) qr[k] = q[fw.qe - k];
    memcpy(tr, t, (size_t)tlen);
    for (int k = 0; k <= fw.te; ++k) tr[k] = t[fw.te - k]; /* only the prefix is reversed */
    ko_fwd_result rv = ko_local_fwd(qr, fw.qe + 1, tr, tlen, m, mat, o_del, e_del, o_ins,
                                    e_ins, INT_MAX, fw.score, max_sc, lanes);
    if (rv.score == fw.score) { r.tb = fw.te - rv.te; r.qb = fw.qe - rv.qe; }
    free(qr);
    free(tr);
    return r;
}

ko_aln_result ko_align2_batched(const uint8_t *q, int qlen, const uint8_t *t, int tlen,
                                int m, const int8_t *mat, int o_del, int e_del,
                                int o_ins, int e_ins, int minsc, int max_sc)
{
    /* crates/bwa-neon/src/matesw.rs:299-497: the forward pass pads from qlen; the reverse
     * pass runs on the truncated reversed prefixes and pads from qe + 1. */
    int lanes = qlen * max_sc < 250 ? 16 : 8;
    ko_fwd_result fw = ko_local_fwd(q, qlen, t, tlen, m, mat, o_del, e_del, o_ins, e_ins,
                                    minsc, INT_MAX, max_sc, lanes);
    ko_aln_result r = {fw.score, -1, fw.qe, -1, fw.te, fw.score2, fw.te2};
    if (!(fw.score >= minsc && fw.qe >= 0)) return r;
    int rq = fw.qe + 1, rt = fw.te + 1;
    uint8_t *qr = malloc((size_t)rq), *tr = malloc((size_t)rt);
    for (int k = 0; k < rq; ++k) qr[k] = q[fw.qe - k];
    for (int k = 0; k < rt; ++k) tr[k] = t[fw.te - k];
    int rl = rq * max_sc < 250 ? 16 : 8;
    ko_fwd_result rv = ko_local_fwd(qr, rq, tr, rt, m, mat, o_del, e_del, o_ins, e_ins,
                                    INT_MAX, fw.score, max_sc, rl);
    if (rv.score == fw.score) { r.tb = fw.te - rv.te; r.qb = fw.qe - rv.qe; }
    free(qr);
    free(tr);
    return r;
}

/* ------------------------------------------------------------------------- */
/* Flat batch drivers                                                         */
/* ------------------------------------------------------------------------- */

static int pick_threads(int nthreads)
{
#ifdef _OPENMP
    return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

void ko_extend_batch(const uint8_t *seq, int64_t n, const int64_t *q_off,
                     const int64_t *t_off, const int32_t *qlen, const int32_t *tlen,
                     const int32_t *h0, const int32_t *w, int m, const int8_t *mat,
                     int o_del, int e_del, int o_ins, int e_ins, int end_bonus,
                     int zdrop, int nthreads, ko_ext_result *out, uint64_t *cells_out)
{
    uint64_t total = 0;
    int nt = pick_threads(nthreads);
    (void)nt;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : total) num_threads(nt)
    for (int64_t k = 0; k < n; ++k) {
        uint64_t c = 0;
        out[k] = ko_extend2(seq + q_off[k], qlen[k], seq + t_off[k], tlen[k], m, mat, o_del,
                            e_del, o_ins, e_ins, w[k], end_bonus, zdrop, h0[k], &c);
        total += c;
    }
    if (cells_out) *cells_out = total;
}

void ko_extend_batch_dispatch(const uint8_t *seq, int64_t n, const int64_t *q_off,
                              const int64_t *t_off, const int32_t *qlen, const int32_t *tlen,
                              const int32_t *h0, const int32_t *w, int m, const int8_t *mat,
                              int o_del, int e_del, int o_ins, int e_ins, int end_bonus,
                              int zdrop, int nthreads, ko_ext_result *out, uint64_t *settled_out,
                              uint64_t *cells_out)
{
    /* The reference's production flow for an extension batch, crates/bwa-neon/src/batched.rs:716-775:
     * with a uniform DNA matrix, every job first tries the ungapped closed form (:773,
     * ungapped_hit :602-697, threshold :756-764); the jobs it declines run the DP.  The
     * reference's DP runs lane-parallel bins (:817-925, NEON / AVX2); this restatement runs the
     * scalar ksw_extend2 per job, whose results the bins equal.  *cells_out counts the DP cells
     * actually evaluated, *settled_out the jobs the closed form settled. */
    uint64_t total = 0, settled = 0;
    int nt = pick_threads(nthreads);
    (void)nt;
    const int uniform = m == 5 && is_uniform_dna(m, mat);
    const int a = mat[0], b = -(int)mat[1];
    const int x = uniform ? ko_x_threshold(a, b, o_del, e_del, o_ins, e_ins) : -1;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : total, settled) num_threads(nt)
    for (int64_t k = 0; k < n; ++k) {
        const uint8_t *q = seq + q_off[k], *t = seq + t_off[k];
        if (x >= 0 && ko_ungapped_hit(q, qlen[k], t, tlen[k], h0[k], a, b, x, zdrop, &out[k])) {
            ++settled;
            continue;
        }
        uint64_t c = 0;
        out[k] = ko_extend2(q, qlen[k], t, tlen[k], m, mat, o_del, e_del, o_ins, e_ins, w[k], end_bonus, zdrop,
                            h0[k], &c);
        total += c;
    }
    if (cells_out) *cells_out = total;
    if (settled_out) *settled_out = settled;
}

void ko_align2_batch(const uint8_t *seq, int64_t n, const int64_t *q_off,
                     const int64_t *t_off, const int32_t *qlen, const int32_t *tlen,
                     int m, const int8_t *mat, int o_del, int e_del, int o_ins,
                     int e_ins, int minsc, int max_sc, int mode, int lanes,
                     int nthreads, ko_aln_result *out, uint64_t *cells_out)
{
    uint64_t total = 0;
    int nt = pick_threads(nthreads);
    (void)nt;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total) num_threads(nt)
    for (int64_t k = 0; k < n; ++k) {
        const uint8_t *q = seq + q_off[k], *t = seq + t_off[k];
        if (mode == 0) {
            out[k] = ko_align2_batched(q, qlen[k], t, tlen[k], m, mat, o_del, e_del, o_ins,
                                       e_ins, minsc, max_sc);
        } else {
            int l = lanes > 0 ? lanes : (qlen[k] * max_sc < 250 ? 16 : 8);
            out[k] = ko_align2_scalar(q, qlen[k], t, tlen[k], m, mat, o_del, e_del, o_ins,
                                      e_ins, minsc, max_sc, l);
        }
        total += (uint64_t)qlen[k] * (uint64_t)tlen[k];
    }
    if (cells_out) *cells_out = total;
}

void ko_local_fwd_batch(const uint8_t *seq, int64_t n, const int64_t *q_off,
                        const int64_t *t_off, const int32_t *qlen, const int32_t *tlen,
                        const int32_t *minsc, const int32_t *endsc, int m,
                        const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins,
                        int max_sc, int lanes, int nthreads, ko_fwd_result *out)
{
    int nt = pick_threads(nthreads);
    (void)nt;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
    for (int64_t k = 0; k < n; ++k) {
        int l = lanes > 0 ? lanes : (qlen[k] * max_sc < 250 ? 16 : 8);
        out[k] = ko_local_fwd(seq + q_off[k], qlen[k], seq + t_off[k], tlen[k], m, mat, o_del,
                              e_del, o_ins, e_ins, minsc[k], endsc[k], max_sc, l);
    }
}

/* ------------------------------------------------------------------------- */
/* Banded global alignment with traceback                                     */
/* ------------------------------------------------------------------------- */

#define KO_MINUS_INF (-0x40000000)

static void cigar_push(uint32_t *cig, int *n, uint32_t op, uint32_t len)
{
    /* crates/bwa-extend/src/sw.rs:516-524: a repeated op extends the previous run */
    if (*n > 0 && (cig[*n - 1] & 0xfu) == op) {
        cig[*n - 1] += len << 4;
        return;
    }
    cig[(*n)++] = (len << 4) | op;
}

int ko_global2(const uint8_t *q, int qlen, const uint8_t *t, int tlen, int m, const int8_t *mat,
               int o_del, int e_del, int o_ins, int e_ins, int w, int32_t *score, uint32_t *cigar,
               int *n_cigar)
{
    /* crates/bwa-extend/src/sw.rs:561-740.  cigar must hold qlen + tlen + 1 words.  Returns 0, or
     * -1 where the reference's traceback index goes out of range (it panics there); its caller,
     * crates/bwa-mem/src/cigar.rs:420-447, sizes w >= |tlen - qlen| + 3, which keeps the path in
     * the band. */
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;
    if (w < 0) w = 0;
    const int n_col = qlen < 2 * w + 1 ? qlen : 2 * w + 1;
    uint8_t *z = malloc((size_t)(n_col > 0 ? n_col : 1) * (size_t)(tlen > 0 ? tlen : 1));
    int32_t *eh_h = malloc(sizeof(int32_t) * (size_t)(qlen + 1));
    int32_t *eh_e = malloc(sizeof(int32_t) * (size_t)(qlen + 1));
    for (int j = 0; j <= qlen; ++j) { eh_h[j] = KO_MINUS_INF; eh_e[j] = KO_MINUS_INF; }
    eh_h[0] = 0;
    for (int j = 1; j <= (qlen < w ? qlen : w); ++j) eh_h[j] = -(o_ins + e_ins * j);
    for (int i = 0; i < tlen; ++i) {
        int32_t f = KO_MINUS_INF;
        const int beg = i > w ? i - w : 0;
        const int end = i + w + 1 < qlen ? i + w + 1 : qlen;
        int32_t h1 = beg == 0 ? -(o_del + e_del * (i + 1)) : KO_MINUS_INF;
        const int8_t *row = mat + t[i] * m;
        uint8_t *zr = z + (size_t)i * (size_t)n_col;
        for (int j = beg; j < end; ++j) {
            int32_t mm = eh_h[j], e = eh_e[j];
            eh_h[j] = h1;
            mm += row[q[j]];
            uint8_t d = mm < e ? 1 : 0;
            int32_t h = mm >= e ? mm : e;
            if (!(h >= f)) { d = 2; h = f; }
            h1 = h;
            int32_t tt = mm - oe_del;
            e -= e_del;
            if (e > tt) d |= 1 << 2;
            else e = tt;
            eh_e[j] = e;
            tt = mm - oe_ins;
            f -= e_ins;
            if (f > tt) d |= 2 << 4;
            else f = tt;
            zr[j - beg] = d;
        }
        eh_h[end] = h1;
        eh_e[end] = KO_MINUS_INF;
    }
    *score = eh_h[qlen];
    /* traceback from the band's last cell of the last row (sw.rs:684-737) */
    int n = 0, rc = 0;
    long i = (long)tlen - 1;
    long k = ((long)tlen - 1 + w + 1 < qlen ? (long)tlen - 1 + w + 1 : qlen) - 1;
    int which = 0;
    while (i >= 0 && k >= 0) {
        const long beg = i > w ? i - w : 0;
        /* the reference indexes the flat matrix: an offset past the row reads the next row's
         * byte; below the row's start, or past the matrix, it stops with an index error */
        const long flat = i * (long)n_col + (k - beg);
        if (k < beg || flat >= (long)n_col * tlen) { rc = -1; break; }
        const uint8_t d = z[flat];
        which = (d >> (which << 1)) & 3;
        if (which == 0) { cigar_push(cigar, &n, 0, 1); --i; --k; }
        else if (which == 1) { cigar_push(cigar, &n, 2, 1); --i; }
        else { cigar_push(cigar, &n, 1, 1); --k; }
    }
    if (rc == 0) {
        if (i >= 0) cigar_push(cigar, &n, 2, (uint32_t)(i + 1));
        if (k >= 0) cigar_push(cigar, &n, 1, (uint32_t)(k + 1));
        for (int a = 0, b = n - 1; a < b; ++a, --b) { uint32_t x = cigar[a]; cigar[a] = cigar[b]; cigar[b] = x; }
    }
    *n_cigar = rc == 0 ? n : 0;
    free(z); free(eh_h); free(eh_e);
    return rc;
}

int ko_global2_batch(const uint8_t *seq, int64_t n, const int64_t *q_off, const int64_t *t_off,
                     const int32_t *qlen, const int32_t *tlen, const int32_t *w, int m,
                     const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins, int nthreads,
                     int32_t *score, const int64_t *cig_off, uint32_t *cigar, int32_t *n_cigar)
{
    /* cigar[cig_off[k] ..] holds job k's runs (room for qlen + tlen + 1 words each). */
    int nt = pick_threads(nthreads), bad = 0;
    (void)nt;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt) reduction(| : bad)
    for (int64_t k = 0; k < n; ++k) {
        int nc = 0;
        bad |= ko_global2(seq + q_off[k], qlen[k], seq + t_off[k], tlen[k], m, mat, o_del, e_del, o_ins,
                          e_ins, w[k], &score[k], cigar + cig_off[k], &nc) != 0;
        n_cigar[k] = nc;
    }
    return bad ? -1 : 0;
}

/* ------------------------------------------------------------------------- */
/* Mate-rescue windows                                                        */
/* ------------------------------------------------------------------------- */

uint8_t ko_ref_base(const uint8_t *pac, int64_t l_pac, int64_t pos)
{
    /* crates/bwa-index/src/fmindex.rs:173-185: forward unpack, most significant pair first;
     * the reverse half is the complement of the mirrored forward base */
    int rc = pos >= l_pac;
    int64_t f = rc ? 2 * l_pac - 1 - pos : pos;
    uint8_t b = (uint8_t)((pac[f >> 2] >> ((3 - (int)(f & 3)) << 1)) & 3);
    return rc ? (uint8_t)(3 - b) : b;
}

static int32_t ko_pos2rid(const int64_t *off, int32_t n, int64_t l_pac, int64_t pos_f)
{
    /* crates/bwa-index/src/bntseq.rs:337-365, including its "last probe" return */
    if (pos_f >= l_pac) return -1;
    int32_t left = 0, mid = 0, right = n;
    while (left < right) {
        mid = (left + right) >> 1;
        if (pos_f >= off[mid]) {
            if (mid == n - 1) break;
            if (pos_f < off[mid + 1]) break;
            left = mid + 1;
        } else {
            right = mid;
        }
    }
    return mid;
}

int ko_rescue_window(const uint8_t *pac, int64_t l_pac, const int64_t *off, const int32_t *len, int32_t n,
                     int64_t anchor_rb, int32_t anchor_rid, int orient, int low, int high, int l_ms,
                     int min_seed_len, int64_t *rb_out, int64_t *re_out, int32_t *rid_out)
{
    /* matesw_collect's window for one orientation (crates/bwa-mem/src/pe.rs:631-674) and
     * bns_fetch_seq's contig clamp (pe.rs:232-270).  Returns 1 when the window is accepted.
     * (pac is unused: the window depends only on the contig table.) */
    (void)pac;
    int is_rev = (orient >> 1) != (orient & 1);
    int is_larger = (orient >> 1) == 0;
    int64_t lo = low, hi = high, rb, re;
    if (!is_rev) {
        rb = is_larger ? anchor_rb + lo : anchor_rb - hi;
        re = (is_larger ? anchor_rb + hi : anchor_rb - lo) + l_ms;
    } else {
        rb = (is_larger ? anchor_rb + lo : anchor_rb - hi) - l_ms;
        re = is_larger ? anchor_rb + hi : anchor_rb - lo;
    }
    if (rb < 0) rb = 0;
    if (re > (l_pac << 1)) re = l_pac << 1;
    *rb_out = rb;
    *re_out = re;
    *rid_out = -1;
    if (!(rb < re)) return 0;
    int64_t mid = (rb + re) >> 1;
    int mrev = mid >= l_pac;
    int64_t mid_f = mrev ? (l_pac << 1) - 1 - mid : mid;
    int32_t rid = ko_pos2rid(off, n, l_pac, mid_f);
    int64_t fb = 0, fe = l_pac << 1;
    if (rid >= 0) {
        fb = off[rid];
        fe = off[rid] + (int64_t)len[rid];
        if (mrev) {
            int64_t t = fb;
            fb = (l_pac << 1) - fe;
            fe = (l_pac << 1) - t;
        }
    }
    if (rb < fb) rb = fb;
    if (re > fe) re = fe;
    *rb_out = rb;
    *re_out = re;
    *rid_out = rid;
    return rid == anchor_rid && re - rb >= min_seed_len;
}
