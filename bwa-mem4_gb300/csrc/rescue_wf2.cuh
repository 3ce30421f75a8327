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
// Scores.  A target row's four scores for query codes 0..3 are one 32-bit profile word, so one
// prmt picks (mat[tA][qA], mat[tB][qB]) sign-extended into the two lanes.  Query columns that
// are N (code 4), ksw padding (score 0) or invalid (score 0, flagged) are patched by a second
// prmt against a word holding the N penalty and zeros; this needs the N column of the matrix to
// be one value (mat[t][4] equal for every t, as bwa's matrix has), which the host checks.
//
// Per column and row: two prmt for the scores, M0 = max(Hd + s, E, 0), H = max(M0, F), the key
// prmt and half a 3-way key maximum, and two fused add-max each for E and F -- 9.5 instructions
// for two cells.  M0 of the next column is computed before H of this one, so the previous
// row's H is overwritten in place (no register copies per step).
#pragma once
#include <cuda_runtime.h>

#include <climits>

#include "common.cuh"
#include "kernels.h"
#include "rescue_wf.cuh"

namespace bwacuda {
namespace wf2 {

constexpr uint32_t MIN2 = 0x80008000u;  // (-32768, -32768)

__host__ __device__ inline int ceil_to(int x, int m) { return (x + m - 1) / m * m; }

__host__ __device__ inline bool job_ok(int qlen, int tlen, int max_sc, int lanes_fixed, int cols)
{
    return rescue_pair_job_ok(qlen, tlen, max_sc, lanes_fixed, cols);
}

template <int L, int C>
struct Lane2 {
    int k;
    uint32_t sel[C];          // prmt selectors: low half picks job A's byte from word A, high half job B's from word B
    uint32_t sf[C];           // prmt selectors patching the score: keep it, the N penalty, or 0
    uint32_t ks[C];           // row-key selectors: (H << 8) | column byte, or 0 for a column past the padded query
    uint32_t cw[(C + 3) / 4]; // key column bytes 255 - j, four columns a word
};

// Loads the lane's columns of both jobs: forward (query[j]) or the reversed prefix
// (query[qe0 - j]); columns [qlen, qpad) are ksw padding (score 0, part of the row maxima),
// columns >= qpad do not exist: their cells are computed but their row keys are 0, so they are
// never a row maximum (they lie right of every real column and feed no real cell).
template <int L, int C>
__device__ __forceinline__ void load_query2(Lane2<L, C> &W, const uint8_t *qa, int qla, int qpa, const uint8_t *qb,
                                            int qlb, int qpb, bool rev, int qea, int qeb, int m, bool &bad)
{
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const int j = W.k * C + c;
        const uint32_t b = 4u + (uint32_t)(c & 3);  // this column's byte of cw[c / 4] as a prmt source
        // key bytes: the column byte, H; past the padded query two zero bytes (H's high bytes)
        W.ks[c] = (j < qpa ? b : 0x11u) | (j < qpb ? ((b << 8) | 0x2000u) : 0x3300u);
        if ((c & 3) == 0) W.cw[c >> 2] = 0u;
        W.cw[c >> 2] |= ((uint32_t)(255 - j) & 0xffu) << (8 * (c & 3));
        uint32_t ca = 7u, cb = 7u;
        if (j < qla) {
            ca = rev ? qa[qea - j] : qa[j];
            bad |= ca >= (uint32_t)m;
            ca = ca < (uint32_t)m ? ca : 7u;
        }
        if (j < qlb) {
            cb = rev ? qb[qeb - j] : qb[j];
            bad |= cb >= (uint32_t)m;
            cb = cb < (uint32_t)m ? cb : 7u;
        }
        const bool sa = ca >= 4u, sb = cb >= 4u;  // N, padding or invalid
        const uint32_t ba = sa ? 0u : ca, bb = sb ? 4u : 4u + cb;
        W.sel[c] = ba | ((ba | 8u) << 4) | (bb << 8) | ((bb | 8u) << 12);
        // patch selectors over (score, Z): Z = (N penalty, 0) as bytes 4-7
        W.sf[c] = (ca < 4u ? 0x10u : (ca == 4u ? 0x54u : 0x76u)) | (cb < 4u ? 0x3200u : (cb == 4u ? 0x5400u : 0x7600u));
    }
}

struct Out2 {
    int score[2], te[2], qe[2];
};

// One local-SW pass of both jobs of every group in the warp, in lockstep.  tlen[h] = 0 makes half
// h inactive; tmap / te0 select the reverse pass's target mapping (rows <= te0 read reversed).
// stop[h]: the half stops once its score reaches endsc[h].  REC: the group's last lane stores
// every computed row's maximum key to rk[h][row] (the suboptimal-score scan reads them after the
// pass).  Returns the results in every lane.
template <int L, int C, bool REC>
__device__ Out2 pass2(const Lane2<L, C> &W, const uint32_t *prof_s, uint32_t zw, const uint8_t *const t[2],
                      const int tlen[2], int tmap, const int te0[2], const Scoring &sc, const int endsc[2],
                      bool stop_enabled, uint16_t *const rk[2], bool &bad)
{
    const int k = W.k;
    const uint32_t noe_del2 = (uint32_t)(-(sc.o_del + sc.e_del) & 0xffff) * 0x10001u;
    const uint32_t noe_ins2 = (uint32_t)(-(sc.o_ins + sc.e_ins) & 0xffff) * 0x10001u;
    const uint32_t ne_del2 = (uint32_t)(-sc.e_del & 0xffff) * 0x10001u;
    const uint32_t ne_ins2 = (uint32_t)(-sc.e_ins & 0xffff) * 0x10001u;
    uint32_t Hp[C], E[C];
#pragma unroll
    for (int c = 0; c < C; ++c) { Hp[c] = 0u; E[c] = 0u; }
    const int tl_max = tlen[0] > tlen[1] ? tlen[0] : tlen[1];
    int steps = tl_max > 0 ? tl_max + L - 1 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) steps = max(steps, __shfl_xor_sync(0xffffffffu, steps, o));

    int gmax[2] = {0, 0}, te[2] = {-1, -1}, qe[2] = {-1, -1};
    bool done[2] = {tlen[0] <= 0, tlen[1] <= 0};
    uint32_t send_hf = 0u;   // bytes H_A, F_A, H_B, F_B of this lane's last column
    uint32_t send_key = 0u;
    uint32_t hprev_in = 0u;  // (H_A, H_B) of row i-1 at the column left of this lane's first
    uint32_t tn[2] = {0u, 0u};
    {
        const int i0 = -k;
#pragma unroll
        for (int h = 0; h < 2; ++h)
            if (i0 >= 0 && i0 < tlen[h]) tn[h] = (tmap && i0 <= te0[h]) ? t[h][te0[h] - i0] : t[h][i0];
    }
    for (int s = 0; s < steps; ++s) {
        const uint32_t rhf = __shfl_up_sync(0xffffffffu, send_hf, 1, L);
        const uint32_t rkey = __shfl_up_sync(0xffffffffu, send_key, 1, L);
        const int i = s - k;
        const uint32_t tca = tn[0], tcb = tn[1];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int in = i + 1;
            if (in >= 0 && in < tlen[h] && !done[h]) tn[h] = (tmap && in <= te0[h]) ? t[h][te0[h] - in] : t[h][in];
        }
        const uint32_t h_in = k == 0 ? 0u : prmt(rhf, 0u, 0x4240u);
        uint32_t f = k == 0 ? 0u : prmt(rhf, 0u, 0x4341u);
        uint32_t key = k == 0 ? 0u : rkey;
        const bool live_a = !done[0] && i >= 0 && i < tlen[0];
        const bool live_b = !done[1] && i >= 0 && i < tlen[1];
        if (live_a || live_b) {
            if (live_a) bad |= tca >= (uint32_t)sc.m;
            if (live_b) bad |= tcb >= (uint32_t)sc.m;
            const uint32_t wa = prof_s[2 * (tca & 7u)], wb = prof_s[2 * (tcb & 7u)];
            uint32_t m0 = __viaddmax_s16x2_relu(hprev_in, prmt(prmt(wa, wb, W.sel[0]), zw, W.sf[0]), E[0]);
            uint32_t kprev = 0u;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                // M0 of the next column first: it is the last reader of this column's previous-row H,
                // which H of this row then replaces in the same register
                uint32_t m0n = 0u;
                if (c + 1 < C)
                    m0n = __viaddmax_s16x2_relu(Hp[c], prmt(prmt(wa, wb, W.sel[c + 1]), zw, W.sf[c + 1]), E[c + 1]);
                const uint32_t h = __vimax_s16x2_relu(m0, f);                 // H = max(M0, F)
                const uint32_t ti = __viaddmax_s16x2(m0, noe_ins2, MIN2);     // M0 - oe_ins
                // row-maximum key per job: (H << 8) | (255 - column), two columns per 3-way max
                const uint32_t kk = prmt(h, W.cw[c >> 2], W.ks[c]);
                if (c & 1) key = __vimax3_u16x2(key, kprev, kk);
                else kprev = kk;
                E[c] = __viaddmax_s16x2_relu(E[c], ne_del2, __viaddmax_s16x2(h, noe_del2, MIN2));  // E opens from H
                f = __viaddmax_s16x2_relu(f, ne_ins2, ti);                    // F opens from M0
                Hp[c] = h;
                m0 = m0n;
            }
            if (C & 1) key = __vimax3_u16x2(key, kprev, kprev);
            send_hf = prmt(Hp[C - 1], f, 0x6240u);
            send_key = key;
            if (k == L - 1) {  // row i of both jobs is complete in this lane
                // predicated updates: the branch-free form keeps the warp's common path short
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const bool live = hh == 0 ? live_a : live_b;
                    const uint32_t kh = hh == 0 ? (key & 0xffffu) : (key >> 16);
                    const int rmax = (int)(kh >> 8);
                    const bool up = live && rmax > gmax[hh];  // first row reaching the maximum keeps te
                    gmax[hh] = up ? rmax : gmax[hh];
                    te[hh] = up ? i : te[hh];
                    qe[hh] = up ? 255 - (int)(kh & 0xffu) : qe[hh];
                    done[hh] = done[hh] || (up && rmax >= endsc[hh]);
                    if (REC && live) rk[hh][i] = (uint16_t)kh;
                }
            }
        }
        hprev_in = h_in;
        if (stop_enabled) {  // warp-uniform early stop; the last lane tells its group
            done[0] = __shfl_sync(0xffffffffu, done[0], L - 1, L);
            done[1] = __shfl_sync(0xffffffffu, done[1], L - 1, L);
            if (__all_sync(0xffffffffu, done[0] && done[1])) break;
        }
    }
    Out2 r;
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
        r.score[hh] = __shfl_sync(0xffffffffu, gmax[hh], L - 1, L);
        r.te[hh] = __shfl_sync(0xffffffffu, te[hh], L - 1, L);
        r.qe[hh] = __shfl_sync(0xffffffffu, qe[hh], L - 1, L);
        if (r.te[hh] < 0) r.qe[hh] = -1;
    }
    return r;
}

// bwa's second-best rule (the peak list of ksw_align2's tracker, as wf::WfTracker builds it) over
// the row maxima a forward pass recorded: rows reaching minsc open a peak, the row right after a
// peak's row replaces it only when strictly higher; the best peak lying more than
// ceil(score / max_sc) rows from te wins, the earlier one on ties.  Peaks are judged as they
// close, so no list is kept.  rk is 8-byte aligned; rows are read four at a time.
__device__ inline void peaks_scan(const uint16_t *rk, int nrows, int minsc, int score, int te, int max_sc,
                                  int &score2, int &te2)
{
    score2 = -1;
    te2 = -1;
    if (score <= 0) return;
    const int hw = (score + max_sc - 1) / max_sc, lo = te - hw, hi = te + hw;
    bool has = false;
    int ls = 0, lr = 0;
    const uint2 *p = reinterpret_cast<const uint2 *>(rk);
    for (int r0 = 0; r0 < nrows; r0 += 4) {
        const uint2 v4 = p[r0 >> 2];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int r = r0 + u;
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

// One group of L lanes per pair of jobs (positions 2p and 2p+1 of the launch); a half whose job
// does not qualify (job_ok) stays idle and is left to the other rescue kernels.
template <int L, int C>
__global__ void __launch_bounds__(128)
rescue_wf2_kernel(const uint8_t *__restrict__ seq, const bwacuda_dev_rescue_job *__restrict__ jobs,
                  const uint32_t *__restrict__ order, uint32_t n, const __grid_constant__ Scoring sc, int mode,
                  int lanes_fixed, int minsc_all, int npen, uint2 *__restrict__ scratch,
                  const uint64_t *__restrict__ scratch_off, bwacuda_rescue_result *__restrict__ out_aln,
                  bwacuda_fwd_result *__restrict__ out_fwd, uint32_t *__restrict__ err)
{
    __shared__ uint32_t prof_s[16];
    if (threadIdx.x < 16) prof_s[threadIdx.x] = sc.prof[threadIdx.x >> 1][threadIdx.x & 1];
    __syncthreads();
    const uint32_t pair = (blockIdx.x * blockDim.x + threadIdx.x) / L;
    Lane2<L, C> W;
    W.k = threadIdx.x % L;
    const bool last = W.k == L - 1;
    bool act[2];
    uint32_t jid[2] = {0u, 0u};
    bwacuda_dev_rescue_job J[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint32_t pos = 2 * pair + h;
        act[h] = pos < n;
        J[h].q_off = 0; J[h].t_off = 0; J[h].qlen = 0; J[h].tlen = 0; J[h].minsc = 0; J[h].endsc = 0;
        if (act[h]) {
            jid[h] = order ? order[pos] : pos;
            J[h] = jobs[jid[h]];
            act[h] = job_ok(J[h].qlen, J[h].tlen, sc.max_sc, lanes_fixed, L * C);
        }
    }
    const uint8_t *q[2], *t[2];
    int qlen[2], tlen[2], qpad[2], minsc[2], endsc[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        q[h] = seq + J[h].q_off;
        t[h] = seq + J[h].t_off;
        qlen[h] = act[h] ? J[h].qlen : 0;
        tlen[h] = act[h] ? J[h].tlen : 0;
        const int ln = lanes_fixed ? lanes_fixed : (J[h].qlen * sc.max_sc < 250 ? 16 : 8);
        qpad[h] = act[h] ? ceil_to(J[h].qlen, ln) : 0;
        minsc[h] = mode == 2 ? J[h].minsc : minsc_all;
        endsc[h] = mode == 2 ? J[h].endsc : 0x7fffffff;
    }
    bool bad = false;
    // row-maximum keys, 2 bytes a row, in the job's tracker scratch (4 * tlen + 16 bytes)
    uint16_t *rk[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) rk[h] = reinterpret_cast<uint16_t *>(scratch + (act[h] ? scratch_off[jid[h]] : 0));
    const uint32_t zw = (uint32_t)npen & 0xffffu;  // patch word: bytes N penalty (16-bit), 0, 0
    load_query2<L, C>(W, q[0], qlen[0], qpad[0], q[1], qlen[1], qpad[1], false, 0, 0, sc.m, bad);
    const int te0z[2] = {0, 0};
    const Out2 fw = pass2<L, C, true>(W, prof_s, zw, t, tlen, 0, te0z, sc, endsc, mode == 2, rk, bad);
    __syncwarp();  // the last lane's key stores before the scans of lanes L - 1 (job A) and L - 2 (job B)
    int score2[2] = {-1, -1}, te2[2] = {-1, -1};
    {
        // lane L - 1 scans job A, lane L - 2 job B (selects, not a dynamic index, keep this in registers)
        const bool b = !last;
        const bool a_h = b ? act[1] : act[0];
        const int sc_h = b ? fw.score[1] : fw.score[0], te_h = b ? fw.te[1] : fw.te[0];
        const int end_h = b ? endsc[1] : endsc[0];
        int s2 = -1, t2 = -1;
        if ((last || W.k == L - 2) && a_h) {
            // a forward pass that stopped (mode 2, score reached endsc) recorded rows up to te
            const int nrows = mode == 2 && sc_h >= end_h ? te_h + 1 : (b ? tlen[1] : tlen[0]);
            peaks_scan(b ? rk[1] : rk[0], nrows, b ? minsc[1] : minsc[0], sc_h, te_h, sc.max_sc, s2, t2);
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
        int rq[2], rqpad[2], rt[2], te0[2], stopsc[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            rev[h] = act[h] && fw.score[h] >= minsc[h] && fw.qe[h] >= 0 && fw.qe[h] < J[h].qlen;
            rq[h] = rev[h] ? fw.qe[h] + 1 : 0;
            // reverse-pass padding: batched_ksw_align2 recomputes the width from qe + 1, the
            // scalar form keeps the forward one
            const int ln = lanes_fixed ? lanes_fixed : (J[h].qlen * sc.max_sc < 250 ? 16 : 8);
            const int rl = mode == 0 ? (rq[h] * sc.max_sc < 250 ? 16 : 8) : ln;
            rqpad[h] = rev[h] ? ceil_to(rq[h], rl) : 0;
            rt[h] = rev[h] ? (mode == 0 ? fw.te[h] + 1 : J[h].tlen) : 0;
            te0[h] = fw.te[h];
            stopsc[h] = fw.score[h];
        }
        load_query2<L, C>(W, q[0], rq[0], rqpad[0], q[1], rq[1], rqpad[1], true, fw.qe[0], fw.qe[1], sc.m, bad);
        const Out2 rv = pass2<L, C, false>(W, prof_s, zw, t, rt, 1, te0, sc, stopsc, true, rk, bad);
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

template <int L, int C>
cudaError_t launch_wf2(const RescueLaunch &Lr, int npen)
{
    // two-warp blocks: residency is register-bound (about 190 registers at 20 columns a lane), and
    // small blocks let an SM hold every warp its register file fits
    const uint32_t threads = 64;
    const uint64_t total = (uint64_t)((Lr.n + 1) / 2) * L;
    const uint32_t grid = (uint32_t)((total + threads - 1) / threads);
    if (grid == 0) return cudaSuccess;
    rescue_wf2_kernel<L, C><<<grid, threads, 0, Lr.stream>>>(Lr.seq, Lr.jobs, Lr.order, (uint32_t)Lr.n, Lr.sc,
                                                             Lr.mode, Lr.lanes, Lr.minsc, npen, Lr.scratch,
                                                             Lr.scratch_off, Lr.out_aln, Lr.out_fwd, Lr.err);
    return cudaGetLastError();
}

}  // namespace wf2
}  // namespace bwacuda
