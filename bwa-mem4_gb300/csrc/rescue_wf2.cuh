// rescue_wf2.cuh -- the mate-rescue register wavefront (rescue_wf.cuh) with two jobs per lane
// group: job A in the low 16-bit lane of every register, job B in the high one, so each DPX
// instruction (__viaddmax_s16x2_relu, __vimax_s16x2_relu, __vimax3_u16x2) updates one cell
// of each job.  The recurrences, tie rules and the suboptimal tracker are those of the 32-bit
// wavefront (ksw_local_fwd, crates/bwa-extend/src/sw.rs:921-1075; start recovery of
// batched_ksw_align2 / ksw_align2), cell for cell.
//
// A job qualifies when every value fits a byte: min(qlen, tlen) * max_sc <= 255 (a local score
// gains at most max_sc per diagonal step, gaps never add), and its padded query (forward and
// reverse) fits 256 columns -- the reference's own 8-bit rescue class (min(q, t) * a < 250 and
// q < 250, crates/bwa-neon/src/matesw.rs:780-795) lies inside it.  Then the row-maximum key
// of a job is 16 bits, (H << 8) | (255 - column): the largest H, and among equal H the smallest
// column, as the reference's qe rule wants.
//
// Scores.  Each lane holds, per column and job, the column's query-profile word: byte t is
// mat[t][q_j] for target codes 0..3 (ksw's padding columns: 0; an N column: the N score).  One
// prmt with a per-row selector picks (mat[tA][qA_j], mat[tB][qB_j]) sign-extended into the two
// lanes.  A target N row (code 4) scores the N value on every real column, so the matrix's N row
// and column must be one value (bwa's matrix is); such rows take a second prmt per column, on a
// warp-uniform branch.
//
// Columns past the padded query do not exist for the job; they are computed with score -128.
// Their H then never exceeds the row's largest real H (a diagonal step from a real cell loses
// 128 >= o_del + e_del, at least the E step below that real cell loses; E and F only decay), and
// their key's column byte is below every real column's, so they are never a row maximum.
//
// Per column and row: the score prmt, M0 = max(Hd + s, E, 0), H = max(M0, F), the key prmt and
// half a 3-way key maximum, and E, F: with o_del + e_del == o_ins + e_ins both open from the
// shared H - (o + e) (F opening from H equals F opening from M0 for o >= 0), 7.5 instructions
// for two cells; otherwise F opens from M0 - (o_ins + e_ins), 8.5.  M0 of the next column is
// computed before H of this one, so the previous row's H is overwritten in place.
//
// The group's last lane stores each row's two keys (2 bytes a job and row, in the job's tracker
// scratch) and keeps max(rmax << 20 | (2^20 - 1 - row)) -- score and first row -- per job; after
// the forward pass the suboptimal-score rule runs over the stored keys (peaks_scan), and qe is
// read from the key of row te.
#pragma once
#include <cuda_runtime.h>

#include <climits>

#include "common.cuh"
#include "kernels.h"

namespace bwacuda {
namespace wf2 {

constexpr uint32_t MIN2 = 0x80008000u;   // (-32768, -32768)
constexpr uint32_t NOCOL = 0x80808080u;  // score -128 for every target code: a column past the query
constexpr int ROW_BITS = 20;             // rows of a target (rescue_pair_job_ok keeps tlen below 2^20)
constexpr uint32_t ROW_MASK = (1u << ROW_BITS) - 1u;

__host__ __device__ inline int ceil_to(int x, int m) { return (x + m - 1) / m * m; }

__host__ __device__ inline bool job_ok(int qlen, int tlen, int max_sc, int lanes_fixed, int cols)
{
    return rescue_pair_job_ok(qlen, tlen, max_sc, lanes_fixed, cols);
}

constexpr int WF2_THREADS = 64;  // threads a block: two warps

template <int L, int C>
struct Lane2 {
    int k;                    // lane index within the group
    uint32_t nf;              // 0 in the group's first lane, 1 elsewhere (zeroes the values it receives)
    uint2 *qw;                // the lane's query-profile words of jobs A and B in shared memory, column c
                              // at qw[c * WF2_THREADS] (read once per row; registers hold the DP state)
    uint32_t cw[(C + 3) / 4]; // key column bytes 255 - j, four columns a word
};

// Gap constants, each 16-bit value in both lanes.
struct Gap2 {
    uint32_t noe_del, noe_ins, ne_del, ne_ins;
};

__device__ __forceinline__ Gap2 gap2(const Scoring &sc)
{
    Gap2 g;
    g.noe_del = (uint32_t)(-(sc.o_del + sc.e_del) & 0xffff) * 0x10001u;
    g.noe_ins = (uint32_t)(-(sc.o_ins + sc.e_ins) & 0xffff) * 0x10001u;
    g.ne_del = (uint32_t)(-sc.e_del & 0xffff) * 0x10001u;
    g.ne_ins = (uint32_t)(-sc.e_ins & 0xffff) * 0x10001u;
    return g;
}

// Query-profile words in shared memory: qp[q] for query codes 0..3 holds mat[t][q] in byte t,
// qp[4] the N score in every byte, qp[5..7] 0 (codes the matrix does not have; flagged).
__device__ __forceinline__ void build_qprof(uint32_t *qp, const Scoring &sc, int npen)
{
    const int q = threadIdx.x;
    if (q < 4) {
        uint32_t w = 0u;
#pragma unroll
        for (int t = 0; t < 4; ++t) w |= ((sc.prof[t][0] >> (8 * q)) & 0xffu) << (8 * t);
        qp[q] = w;
    } else if (q < 8) {
        qp[q] = q == 4 ? ((uint32_t)npen & 0xffu) * 0x01010101u : 0u;
    }
}

// Loads the lane's columns of job h (0: A, the low 16-bit lanes; 1: B, the high ones): forward
// (query[j]) or the reversed prefix (query[qe0 - j]); columns [qlen, qpad) are ksw padding
// (score 0, part of the row maxima), columns >= qpad do not exist (score -128, never a row
// maximum).  Job A's call also writes the key column bytes.
template <int L, int C>
__device__ __forceinline__ void load_query2_half(Lane2<L, C> &W, const uint32_t *qp, const uint8_t *q, int ql, int qpd,
                                                 bool rev, int qe0, int h, int m, bool &bad)
{
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const int j = W.k * C + c;
        if (h == 0) {
            if ((c & 3) == 0) W.cw[c >> 2] = 0u;
            W.cw[c >> 2] |= ((uint32_t)(255 - j) & 0xffu) << (8 * (c & 3));
        }
        uint32_t w = j < qpd ? 0u : NOCOL;
        if (j < ql) {
            const uint32_t code = rev ? q[qe0 - j] : q[j];
            bad |= code >= (uint32_t)m;
            w = qp[code & 7u];
        }
        if (h == 0) W.qw[c * WF2_THREADS].x = w;
        else W.qw[c * WF2_THREADS].y = w;
    }
}

struct Out2 {
    int score[2], te[2], qe[2];
};

// Score of column c for both jobs.  SLOW: some row of the warp is a target N (or a code outside
// 0..3): selN keeps a job's profile score (0x10 / 0x3200) or takes its N-row score from nz, which
// is the N value on real columns, 0 on padding and -128 past the padded query.
template <bool SLOW>
__device__ __forceinline__ uint32_t score2(uint2 q, uint32_t selT, int c, uint32_t selN, int ra, int pa, int rb,
                                           int pb, uint32_t npa, uint32_t npb)
{
    const uint32_t s = prmt(q.x, q.y, selT);
    if constexpr (!SLOW) {
        return s;
    } else {
        const uint32_t za = c < ra ? npa : (c < pa ? 0u : 0xff80u);
        const uint32_t zb = c < rb ? npb : (c < pb ? 0u : 0xff800000u);
        return prmt(s, za | zb, selN);
    }
}

// One row of the lane's C columns for both jobs.  hd: H of row i-1 at the column left of the
// lane's first; f, key: F and the row key entering from the left; on return f, key leave to the
// right and Hp holds row i.
template <int C, bool SYM, bool SLOW>
__device__ __forceinline__ void row2(const uint2 *qw, const uint32_t *cw, uint32_t (&Hp)[C], uint32_t (&E)[C],
                                     uint32_t &f, uint32_t &key, uint32_t hd, uint32_t selT, const Gap2 &g,
                                     uint32_t selN, int ra, int pa, int rb, int pb, uint32_t npa, uint32_t npb)
{
    uint32_t m0 = __viaddmax_s16x2_relu(hd, score2<SLOW>(qw[0], selT, 0, selN, ra, pa, rb, pb, npa, npb), E[0]);
    uint32_t kprev = 0u;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        // M0 of the next column first: it is the last reader of this column's previous-row H,
        // which H of this row then replaces in the same register
        uint32_t m0n = 0u;
        if (c + 1 < C)
            m0n = __viaddmax_s16x2_relu(
                Hp[c], score2<SLOW>(qw[(c + 1) * WF2_THREADS], selT, c + 1, selN, ra, pa, rb, pb, npa, npb), E[c + 1]);
        const uint32_t h = __vimax_s16x2_relu(m0, f);  // H = max(M0, F)
        // row-maximum key per job: (H << 8) | (255 - column); selector bytes: column, H_A, column, H_B
        const uint32_t kk = prmt(h, cw[c >> 2], (uint32_t)((4 + (c & 3)) * 0x101 + 0x2000));
        if (c & 1) key = __vimax3_u16x2(key, kprev, kk);
        else kprev = kk;
        if constexpr (SYM) {
            const uint32_t t = __viaddmax_s16x2(h, g.noe_del, MIN2);  // H - (o + e), both gaps open from it
            E[c] = __viaddmax_s16x2_relu(E[c], g.ne_del, t);
            f = __viaddmax_s16x2_relu(f, g.ne_ins, t);
        } else {
            const uint32_t ti = __viaddmax_s16x2(m0, g.noe_ins, MIN2);  // F opens from M0
            const uint32_t td = __viaddmax_s16x2(h, g.noe_del, MIN2);   // E opens from H
            E[c] = __viaddmax_s16x2_relu(E[c], g.ne_del, td);
            f = __viaddmax_s16x2_relu(f, g.ne_ins, ti);
        }
        Hp[c] = h;
        m0 = m0n;
    }
    if (C & 1) key = __vimax3_u16x2(key, kprev, kprev);
}

// One local-SW pass of both jobs of every group in the warp, in lockstep.  tlen[h] = 0 makes half
// h inactive.  TMAP: the reverse pass's target mapping (row r reads t[te0 - r] while r <= te0,
// t[r] after).  stop: half h stops at its first row whose maximum reaches endsc[h] (at least 1).
// The last lane stores every computed row's key to rk[h][row].  ql / qp: the pass's query length
// and padded length per job.  Returns the results in every lane.
template <int L, int C, bool SYM, bool TMAP>
__device__ Out2 pass2(const Lane2<L, C> &W, const uint8_t *const t[2], const int tlen[2], const int te0[2],
                      const Gap2 &g, int npen, int m, bool stop, const int endsc[2], uint16_t *const rk[2],
                      const int ql[2], const int qp[2], bool &bad)
{
    const int k = W.k;
    uint32_t Hp[C], E[C];
#pragma unroll
    for (int c = 0; c < C; ++c) { Hp[c] = 0u; E[c] = 0u; }
    const int tl_max = tlen[0] > tlen[1] ? tlen[0] : tlen[1];
    int steps = tl_max > 0 ? tl_max + L - 1 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) steps = max(steps, __shfl_xor_sync(0xffffffffu, steps, o));
    // slow-row parameters: the lane's real / padded column counts per job, the N value per lane
    const int ra = ql[0] - k * C, pa = qp[0] - k * C, rb = ql[1] - k * C, pb = qp[1] - k * C;
    const uint32_t npa = (uint32_t)npen & 0xffffu, npb = (uint32_t)npen << 16;
    const uint32_t thr = (uint32_t)(m < 4 ? m : 4);  // codes from thr on take the slow rows
    const int end_a = endsc[0] > 1 ? endsc[0] : 1, end_b = endsc[1] > 1 ? endsc[1] : 1;

    uint32_t ga = 0u, gb = 0u;  // (rmax << 20) | (2^20 - 1 - row), best so far
    bool done_a = tlen[0] <= 0, done_b = tlen[1] <= 0;
    uint32_t send_h = 0u, send_f = 0u, send_key = 0u;
    uint32_t hprev = 0u;  // (H_A, H_B) of row i-1 at the column left of this lane's first
    // target codes of rows i + 1 and i + 2: each load is issued two rows before its use, so a
    // miss on a new target sector has two steps of the warp's work to arrive
    uint32_t tn[2] = {0u, 0u}, tn2[2] = {0u, 0u};
    {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i0 = -k, i1 = 1 - k;
            if (i0 >= 0 && i0 < tlen[h]) tn[h] = (TMAP && i0 <= te0[h]) ? t[h][te0[h] - i0] : t[h][i0];
            if (i1 >= 0 && i1 < tlen[h]) tn2[h] = (TMAP && i1 <= te0[h]) ? t[h][te0[h] - i1] : t[h][i1];
        }
    }
    for (int s = 0; s < steps; ++s) {
        const uint32_t rh = __shfl_up_sync(0xffffffffu, send_h, 1, L) * W.nf;
        uint32_t f = __shfl_up_sync(0xffffffffu, send_f, 1, L) * W.nf;
        uint32_t key = __shfl_up_sync(0xffffffffu, send_key, 1, L) * W.nf;
        const int i = s - k;
        const uint32_t tca = tn[0], tcb = tn[1];
        if ((s & 15) == 0 && k == 0) {  // every 16 rows, the group's first lane pulls row i + 64 into L2
            const int ip = i + 64;
#pragma unroll
            for (int h = 0; h < 2; ++h)
                if ((unsigned)ip < (unsigned)tlen[h])
                    prefetch_l2(t[h] + ((TMAP && ip <= te0[h]) ? te0[h] - ip : ip));
        }
        {
            const int in = i + 2;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                tn[h] = tn2[h];
                if ((unsigned)in < (unsigned)tlen[h]) tn2[h] = (TMAP && in <= te0[h]) ? t[h][te0[h] - in] : t[h][in];
            }
        }
        const bool live_a = !done_a && (unsigned)i < (unsigned)tlen[0];
        const bool live_b = !done_b && (unsigned)i < (unsigned)tlen[1];
        // the vote runs in every lane of the warp, before the branch on this lane's rows
        const bool any_slow = __any_sync(0xffffffffu, (live_a && tca >= thr) || (live_b && tcb >= thr));
        if (live_a || live_b) {
            const uint32_t ta = tca & 3u, tb = tcb & 3u;
            // selector bytes: A's score and its sign from word A, B's score and its sign from word B
            const uint32_t selT = ta * 0x11u + 0x80u + tb * 0x1100u + 0xC400u;
            if (any_slow) {
                if (live_a) bad |= tca >= (uint32_t)m;
                if (live_b) bad |= tcb >= (uint32_t)m;
                const uint32_t selN = (live_a && tca >= 4u ? 0x54u : 0x10u) | (live_b && tcb >= 4u ? 0x7600u : 0x3200u);
                row2<C, SYM, true>(W.qw, W.cw, Hp, E, f, key, hprev, selT, g, selN, ra, pa, rb, pb, npa, npb);
            } else {
                row2<C, SYM, false>(W.qw, W.cw, Hp, E, f, key, hprev, selT, g, 0u, 0, 0, 0, 0, 0u, 0u);
            }
            send_h = Hp[C - 1];
            send_f = f;
            send_key = key;
            if (k == L - 1) {  // row i of both jobs is complete in this lane
                const uint32_t rowinv = ROW_MASK - (uint32_t)i;
                const uint32_t rma = (key >> 8) & 0xffu, rmb = key >> 24;
                if (live_a) {
                    ga = max(ga, (rma << ROW_BITS) | rowinv);
                    rk[0][i] = (uint16_t)key;
                }
                if (live_b) {
                    gb = max(gb, (rmb << ROW_BITS) | rowinv);
                    rk[1][i] = (uint16_t)(key >> 16);
                }
                if (stop) {
                    done_a = done_a || (live_a && (int)rma >= end_a);
                    done_b = done_b || (live_b && (int)rmb >= end_b);
                }
            }
        }
        hprev = rh;
        if (stop) {  // warp-uniform early stop; the last lane tells its group
            done_a = __shfl_sync(0xffffffffu, done_a, L - 1, L);
            done_b = __shfl_sync(0xffffffffu, done_b, L - 1, L);
            if (__all_sync(0xffffffffu, done_a && done_b)) break;
        }
    }
    Out2 r;
    const uint32_t gg[2] = {ga, gb};
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
        const int sc = (int)(gg[hh] >> ROW_BITS);
        const int te = sc > 0 ? (int)(ROW_MASK - (gg[hh] & ROW_MASK)) : -1;
        // qe: the key column of row te (the last lane wrote it)
        const int qe = (k == L - 1 && te >= 0) ? 255 - (int)(rk[hh][te] & 0xffu) : -1;
        r.score[hh] = __shfl_sync(0xffffffffu, sc, L - 1, L);
        r.te[hh] = __shfl_sync(0xffffffffu, te, L - 1, L);
        r.qe[hh] = __shfl_sync(0xffffffffu, qe, L - 1, L);
    }
    return r;
}

// bwa's second-best rule (the peak list of ksw_align2's tracker, as the 32-bit wavefront's
// tracker builds it) over the row maxima a forward pass recorded: rows reaching minsc open a
// peak, the row right after a peak's row replaces it only when strictly higher; the best peak
// lying more than ceil(score / max_sc) rows from te wins, the earlier one on ties.  Peaks are
// judged as they close, so no list is kept.  rk is 8-byte aligned; rows are read four at a time.
__device__ inline void peaks_scan(const uint16_t *rk, int nrows, int minsc, int score, int te, int max_sc,
                                  int &score2, int &te2)
{
    score2 = -1;
    te2 = -1;
    if (score <= 0) return;
    const int hw = (score + max_sc - 1) / max_sc, lo = te - hw, hi = te + hw;
    bool has = false;
    int ls = 0, lr = 0;
    // words of four rows, four words in flight (the scan is one lane's serial walk: its loads,
    // not its arithmetic, set its time); a word whose four maxima are all below minsc is skipped
    const uint2 *p = reinterpret_cast<const uint2 *>(rk);
    const int nw = (nrows + 3) >> 2;
    const uint2 z = make_uint2(0u, 0u);
    uint2 b0 = nw > 0 ? p[0] : z, b1 = nw > 1 ? p[1] : z, b2 = nw > 2 ? p[2] : z, b3 = nw > 3 ? p[3] : z;
    const uint32_t kmin = (uint32_t)(minsc > 0 ? minsc : 0) << 8;
    for (int wi = 0; wi < nw; ++wi) {
        const uint2 v4 = b0;
        b0 = b1;
        b1 = b2;
        b2 = b3;
        b3 = wi + 4 < nw ? p[wi + 4] : z;
        const uint32_t mx = __vimax3_u16x2(v4.x, v4.y, 0u);
        if (max(mx & 0xffffu, mx >> 16) < kmin && minsc > 0) continue;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int r = 4 * wi + u;
            const uint32_t w = u < 2 ? v4.x : v4.y;
            const int v = (int)((w >> (16 * (u & 1) + 8)) & 0xffu);
            if (r >= nrows || v < minsc) continue;
            const bool cont = has && lr + 1 == r;
            if (has && !cont && (lr < lo || lr > hi) && ls > score2) { score2 = ls; te2 = lr; }
            if (!cont || ls < v) { ls = v; lr = r; }
            has = true;
        }
    }
    if (has && (lr < lo || lr > hi) && ls > score2) { score2 = ls; te2 = lr; }
}

// One job's fields as a phase of the kernel uses them; inactive: an empty job.
struct JobView {
    const uint8_t *q, *t;
    int qlen, tlen, qpad, minsc, endsc;
    uint16_t *rk;  // row-maximum keys, 2 bytes a row, in the job's tracker scratch (4 * tlen + 16 bytes)
};

__device__ __forceinline__ JobView job_view(const volatile bwacuda_dev_rescue_job *jobs, uint32_t jid, bool act,
                                            const uint8_t *seq, uint2 *scratch, const uint64_t *scratch_off, int mode,
                                            int minsc_all, int lanes_fixed, int max_sc)
{
    JobView v;
    uint64_t q_off = 0, t_off = 0, s_off = 0;
    int qlen = 0, tlen = 0, jminsc = 0, jendsc = 0;
    if (act) {
        const volatile bwacuda_dev_rescue_job &J = jobs[jid];
        q_off = J.q_off;
        t_off = J.t_off;
        qlen = J.qlen;
        tlen = J.tlen;
        jminsc = J.minsc;
        jendsc = J.endsc;
        s_off = scratch_off[jid];
    }
    v.q = seq + q_off;
    v.t = seq + t_off;
    v.qlen = qlen;
    v.tlen = tlen;
    const int ln = lanes_fixed ? lanes_fixed : (qlen * max_sc < 250 ? 16 : 8);
    v.qpad = act ? ceil_to(qlen, ln) : 0;
    v.minsc = mode == 2 ? jminsc : minsc_all;
    v.endsc = mode == 2 ? jendsc : 0x7fffffff;
    v.rk = reinterpret_cast<uint16_t *>(scratch + s_off);
    return v;
}

// One group of L lanes (4, 8 or 16) per pair of jobs (positions 2p and 2p+1 of the launch); a half whose job
// does not qualify (job_ok) stays idle and is left to the other rescue kernels.
// Blocks per SM the register budget aims at (two warps a block): 8 (128 registers, four warps a
// scheduler) up to 12 columns a lane, 6 (168 registers, three) up to 24, and no cap above, where
// a cap would spill (40 columns a lane at 247 registers and two warps a scheduler: 2761 GCUPS on
// the rescue windows, against 2316 capped at 168 with spills and 2564 for 20 columns at 168).
template <int C>
constexpr int wf2_min_blocks() { return C <= 12 ? 8 : (C <= 24 ? 6 : 1); }

template <int L, int C, bool SYM>
__global__ void __launch_bounds__(WF2_THREADS, wf2_min_blocks<C>())
rescue_wf2_kernel(const uint8_t *__restrict__ seq, const bwacuda_dev_rescue_job *__restrict__ jobs,
                  const uint32_t *__restrict__ order, uint32_t n, const __grid_constant__ Scoring sc, int mode,
                  int lanes_fixed, int minsc_all, int npen, uint2 *__restrict__ scratch,
                  const uint64_t *__restrict__ scratch_off, bwacuda_rescue_result *__restrict__ out_aln,
                  bwacuda_fwd_result *__restrict__ out_fwd, uint32_t *__restrict__ err)
{
    __shared__ uint32_t qp_s[8];
    __shared__ uint2 qw_s[C * WF2_THREADS];
    build_qprof(qp_s, sc, npen);
    __syncthreads();
    const uint32_t pair = (blockIdx.x * blockDim.x + threadIdx.x) / L;
    Lane2<L, C> W;
    W.k = threadIdx.x % L;
    W.qw = qw_s + threadIdx.x;
    W.nf = W.k != 0 ? 1u : 0u;
    const bool last = W.k == L - 1;
    bool act[2];
    uint32_t jid[2] = {0u, 0u};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint32_t pos = 2 * pair + h;
        act[h] = pos < n;
        if (act[h]) {
            jid[h] = order ? order[pos] : pos;
            const bwacuda_dev_rescue_job &J = jobs[jid[h]];
            act[h] = job_ok(J.qlen, J.tlen, sc.max_sc, lanes_fixed, L * C);
        }
    }
    // The job records are read again for each phase (volatile reads, cached in L2) instead of
    // being held in registers across the forward pass: the pass's register budget sets how many
    // warps an SM holds.
    const volatile bwacuda_dev_rescue_job *vjobs = jobs;
    bool bad = false;
    const Gap2 g = gap2(sc);
    Out2 fw;
    int score2[2] = {-1, -1}, te2[2] = {-1, -1};
    {
        const uint8_t *t[2];
        int qlen[2], tlen[2], qpad[2], endsc[2];
        uint16_t *rk[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const JobView v = job_view(vjobs, jid[h], act[h], seq, scratch, scratch_off, mode, minsc_all, lanes_fixed,
                                       sc.max_sc);
            load_query2_half<L, C>(W, qp_s, v.q, v.qlen, v.qpad, false, 0, h, sc.m, bad);
            t[h] = v.t;
            qlen[h] = v.qlen;
            tlen[h] = v.tlen;
            qpad[h] = v.qpad;
            endsc[h] = v.endsc;
            rk[h] = v.rk;
        }
        const int te0z[2] = {0, 0};
        fw = pass2<L, C, SYM, false>(W, t, tlen, te0z, g, npen, sc.m, mode == 2, endsc, rk, qlen, qpad, bad);
    }
    __syncwarp();  // the last lane's key stores before the scans of lanes L - 1 (job A) and L - 2 (job B)
    {
        // lane L - 1 scans job A, lane L - 2 job B (selects, not a dynamic index, keep this in registers)
        const bool b = !last;
        const bool a_h = b ? act[1] : act[0];
        const int sc_h = b ? fw.score[1] : fw.score[0], te_h = b ? fw.te[1] : fw.te[0];
        int s2 = -1, t2 = -1;
        if ((last || W.k == L - 2) && a_h) {
            const JobView v = job_view(vjobs, b ? jid[1] : jid[0], true, seq, scratch, scratch_off, mode, minsc_all,
                                       lanes_fixed, sc.max_sc);
            // a forward pass that stopped (mode 2, score reached endsc) recorded rows up to te
            const int nrows = mode == 2 && sc_h >= (v.endsc > 1 ? v.endsc : 1) ? te_h + 1 : v.tlen;
            peaks_scan(v.rk, nrows, v.minsc, sc_h, te_h, sc.max_sc, s2, t2);
        }
        // job B's result to the last lane, which writes both
        score2[0] = s2;
        te2[0] = t2;
        score2[1] = __shfl_sync(0xffffffffu, s2, L - 2, L);
        te2[1] = __shfl_sync(0xffffffffu, t2, L - 2, L);
    }
    if (mode == 2) {
        if (last) {
#pragma unroll
            for (int h = 0; h < 2; ++h)
                if (act[h]) {
                    bwacuda_fwd_result r;
                    r.score = fw.score[h]; r.te = fw.te[h]; r.qe = fw.qe[h]; r.score2 = score2[h]; r.te2 = te2[h];
                    out_fwd[jid[h]] = r;
                }
        }
    } else {
        bool rev[2];
        const uint8_t *t[2];
        int rq[2], rqpad[2], rt[2], te0[2], stopsc[2];
        uint16_t *rk[2];
        __syncwarp();  // the scans' reads of the keys before the reverse pass rewrites them
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const JobView v = job_view(vjobs, jid[h], act[h], seq, scratch, scratch_off, mode, minsc_all, lanes_fixed,
                                       sc.max_sc);
            rev[h] = act[h] && fw.score[h] >= v.minsc && fw.qe[h] >= 0 && fw.qe[h] < v.qlen;
            rq[h] = rev[h] ? fw.qe[h] + 1 : 0;
            // reverse-pass padding: batched_ksw_align2 recomputes the width from qe + 1, the
            // scalar form keeps the forward one
            const int ln = lanes_fixed ? lanes_fixed : (v.qlen * sc.max_sc < 250 ? 16 : 8);
            const int rl = mode == 0 ? (rq[h] * sc.max_sc < 250 ? 16 : 8) : ln;
            rqpad[h] = rev[h] ? ceil_to(rq[h], rl) : 0;
            rt[h] = rev[h] ? (mode == 0 ? fw.te[h] + 1 : v.tlen) : 0;
            te0[h] = fw.te[h];
            stopsc[h] = fw.score[h];
            t[h] = v.t;
            rk[h] = v.rk;
            load_query2_half<L, C>(W, qp_s, v.q, rq[h], rqpad[h], true, fw.qe[h], h, sc.m, bad);
        }
        const Out2 rv = pass2<L, C, SYM, true>(W, t, rt, te0, g, npen, sc.m, true, stopsc, rk, rq, rqpad, bad);
        if (last) {
#pragma unroll
            for (int h = 0; h < 2; ++h)
                if (act[h]) {
                    bwacuda_rescue_result r;
                    r.score = fw.score[h]; r.qb = -1; r.qe = fw.qe[h]; r.tb = -1; r.te = fw.te[h];
                    r.score2 = score2[h]; r.te2 = te2[h];
                    if (rev[h] && rv.score[h] == fw.score[h]) {
                        r.tb = fw.te[h] - rv.te[h];
                        r.qb = fw.qe[h] - rv.qe[h];
                    }
                    out_aln[jid[h]] = r;
                }
        }
    }
    if (bad) atomicOr(err, ERR_BASE);
}

template <int L, int C, bool SYM>
cudaError_t launch_wf2(const RescueLaunch &Lr, int npen)
{
    // two-warp blocks: residency is register-bound, and small blocks let an SM hold every warp its
    // register file fits
    const uint32_t threads = WF2_THREADS;
    const uint64_t total = (uint64_t)((Lr.n + 1) / 2) * L;
    const uint32_t grid = (uint32_t)((total + threads - 1) / threads);
    if (grid == 0) return cudaSuccess;
    rescue_wf2_kernel<L, C, SYM><<<grid, threads, 0, Lr.stream>>>(Lr.seq, Lr.jobs, Lr.order, (uint32_t)Lr.n, Lr.sc,
                                                                  Lr.mode, Lr.lanes, Lr.minsc, npen, Lr.scratch,
                                                                  Lr.scratch_off, Lr.out_aln, Lr.out_fwd, Lr.err);
    return cudaGetLastError();
}

// Column counts built per lane count (L * C covers queries padded to 256 columns; 4-lane
// groups to 192: their 48 columns a lane already hold every register).
constexpr int C4[] = {8, 16, 24, 32, 40, 48};
constexpr int C8[] = {4, 8, 12, 16, 20, 24, 32};
constexpr int C16[] = {4, 6, 8, 10, 12, 16};

template <bool SYM>
cudaError_t launch_shape(const RescueLaunch &Lr, int lanes, int c, int npen)
{
    if (lanes == 4) {
        switch (c) {
        case 8: return launch_wf2<4, 8, SYM>(Lr, npen);
        case 16: return launch_wf2<4, 16, SYM>(Lr, npen);
        case 24: return launch_wf2<4, 24, SYM>(Lr, npen);
        case 32: return launch_wf2<4, 32, SYM>(Lr, npen);
        case 40: return launch_wf2<4, 40, SYM>(Lr, npen);
        case 48: return launch_wf2<4, 48, SYM>(Lr, npen);
        default: return cudaErrorInvalidValue;
        }
    }
    if (lanes == 16) {
        switch (c) {
        case 4: return launch_wf2<16, 4, SYM>(Lr, npen);
        case 6: return launch_wf2<16, 6, SYM>(Lr, npen);
        case 8: return launch_wf2<16, 8, SYM>(Lr, npen);
        case 10: return launch_wf2<16, 10, SYM>(Lr, npen);
        case 12: return launch_wf2<16, 12, SYM>(Lr, npen);
        case 16: return launch_wf2<16, 16, SYM>(Lr, npen);
        default: return cudaErrorInvalidValue;
        }
    }
    switch (c) {
    case 4: return launch_wf2<8, 4, SYM>(Lr, npen);
    case 8: return launch_wf2<8, 8, SYM>(Lr, npen);
    case 12: return launch_wf2<8, 12, SYM>(Lr, npen);
    case 16: return launch_wf2<8, 16, SYM>(Lr, npen);
    case 20: return launch_wf2<8, 20, SYM>(Lr, npen);
    case 24: return launch_wf2<8, 24, SYM>(Lr, npen);
    case 32: return launch_wf2<8, 32, SYM>(Lr, npen);
    default: return cudaErrorInvalidValue;
    }
}

// The launches of one gap class, each in its own translation unit (rescue_wf2.cu:
// o_del + e_del == o_ins + e_ins; rescue_wf2a.cu: the rest).
cudaError_t launch_sym(const RescueLaunch &Lr, int lanes, int c, int npen);
cudaError_t launch_asym(const RescueLaunch &Lr, int lanes, int c, int npen);

}  // namespace wf2
}  // namespace bwacuda
