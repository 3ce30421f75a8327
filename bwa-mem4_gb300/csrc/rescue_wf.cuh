// rescue_wf.cuh -- mate-rescue local Smith-Waterman as a register-resident
// anti-diagonal wavefront: one group of L lanes per job, lane k owning query
// columns [k*C, (k+1)*C) in registers.  At step s lane k computes row s - k of
// its columns and hands H and F of its last column, plus the running row-max
// key, to lane k+1 with one shuffle each; the last lane of the group holds the
// finished row maximum and does the per-row bookkeeping (te / qe / the
// suboptimal tracker).  No shared memory holds DP state, so occupancy is set by
// registers alone.
//
// Semantics are those of rescue_tpj.cu (ksw_local_fwd, crates/bwa-extend/src/
// sw.rs:921-1075; start recovery of batched_ksw_align2 / ksw_align2).  One
// rearrangement keeps the horizontal dependency to a single op per cell:
//   F(i, j+1) = max(0, F(i,j) - e_ins, H(i,j) - oe_ins) with H = max(M0, F)
//             = max(0, F(i,j) - e_ins, M0(i,j) - oe_ins)   because o_ins >= 0
// (the F-derived part of H never beats extending F); o_ins >= 0 is validated
// on the host.  E still opens from the full H.
//
// The templates below are instantiated per group width L by rescue_wf.cu
// (16 lanes), rescue_wf8.cu and rescue_wf32.cu (separate translation units so
// they compile in parallel); the autotuner picks L per batch.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"

namespace bwacuda {
namespace wf {

__device__ __forceinline__ int relu_addmax(int a, int b, int c)
{
    // max(a + b, c, 0)
    return __viaddmax_s32_relu(a, b, c);
}

// Suboptimal tracker (crates/bwa-extend/src/sw.rs:789-852), finalised entries
// in device scratch; used by the last lane of a group only.
struct WfTracker {
    uint2 *slot;
    int cap, nb, ls, lr;
    bool has, overflow;
    __device__ void init(uint2 *s, int c) { slot = s; cap = c; nb = 0; ls = 0; lr = 0; has = false; overflow = false; }
    __device__ __forceinline__ void push(int row, int rmax, int minsc)
    {
        if (rmax < minsc) return;
        if (has && lr + 1 == row) {
            if (ls < rmax) { ls = rmax; lr = row; }
            return;
        }
        if (has) {
            if (nb < cap) slot[nb] = make_uint2((uint32_t)ls, (uint32_t)lr);
            else overflow = true;
            ++nb;
        }
        ls = rmax; lr = row; has = true;
    }
    __device__ void finish(int gmax, int te, int max_sc, int &score2, int &te2) const
    {
        score2 = -1; te2 = -1;
        if (gmax > 0 && has) {
            const int hw = (gmax + max_sc - 1) / max_sc;
            const int lo = te - hw, hi = te + hw;
            const int nc = nb < cap ? nb : cap;
            for (int k = 0; k < nc; ++k) {
                const uint2 v = slot[k];
                const int r = (int)v.y, s = (int)v.x;
                if ((r < lo || r > hi) && s > score2) { score2 = s; te2 = r; }
            }
            if ((lr < lo || lr > hi) && ls > score2) { score2 = ls; te2 = lr; }
        }
    }
};

template <int L, int C>
struct WfLane {
    int k;           // lane index within the group
    uint32_t qsel[C];  // prmt selectors of this lane's query columns
    int kcol[C];       // row-max key column part; sign bit set past the padded query
};

// Loads the lane's selectors: forward (query[j]) or reversed prefix (query[qe0 - j]),
// columns [qlen, qpad) are ksw padding (score 0), columns >= qpad do not exist.
template <int L, int C>
__device__ __forceinline__ void wf_load_query(WfLane<L, C> &W, const uint8_t *q, int qlen, int qpad, bool rev,
                                              int qe0, int m, bool &bad)
{
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const int j = W.k * C + c;
        uint32_t code = (uint32_t)PAD_CODE;
        if (j < qlen) {
            code = rev ? q[qe0 - j] : q[j];
            bad |= code >= (uint32_t)m;
            code = code < (uint32_t)m ? code : (uint32_t)PAD_CODE;
        }
        W.qsel[c] = code * 0x1111u | 0x8880u;
        W.kcol[c] = j < qpad ? (0xffff - j) : (int)0x80000000;
    }
}

struct WfOut {
    int score, te, qe;
};

// One forward local-SW pass of every group in the warp, in lockstep.
// Returns the result in every lane of the group.
template <int L, int C>
__device__ WfOut wf_pass(const WfLane<L, C> &W, const uint32_t *prof_s, const uint8_t *t, int tlen, int tmap,
                         int te0, const Scoring &sc, int minsc, int endsc, bool stop_enabled, WfTracker *trk,
                         bool active_job, bool &bad)
{
    const int k = W.k;
    const int oe_del = sc.o_del + sc.e_del, oe_ins = sc.o_ins + sc.e_ins;
    const int e_del = sc.e_del, e_ins = sc.e_ins;
    int Hp[C], E[C];
#pragma unroll
    for (int c = 0; c < C; ++c) { Hp[c] = 0; E[c] = 0; }
    int steps = active_job ? tlen + L - 1 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) steps = max(steps, __shfl_xor_sync(0xffffffffu, steps, o));

    int gmax = 0, te = -1, qe = -1;
    bool done = !active_job;
    uint32_t send_hf = 0;  // H(i, last column) | F(i, next column) << 16
    int send_key = 0;
    int hprev_in = 0;      // H(i-1, first column - 1): the diagonal of this lane's first cell
    // target base of this lane's next row (prefetched one step ahead)
    int i0 = -k;
    uint32_t tnext = 0;
    if (i0 >= 0 && i0 < tlen) tnext = (tmap && i0 <= te0) ? t[te0 - i0] : t[i0];
    for (int s = 0; s < steps; ++s) {
        const uint32_t rhf = __shfl_up_sync(0xffffffffu, send_hf, 1, L);
        const int rkey = __shfl_up_sync(0xffffffffu, send_key, 1, L);
        const int i = s - k;
        const uint32_t tc_raw = tnext;
        {
            const int in = i + 1;
            if (in >= 0 && in < tlen && !done) tnext = (tmap && in <= te0) ? t[te0 - in] : t[in];
        }
        const int h_in = k == 0 ? 0 : (int)(rhf & 0xffffu);
        int f = k == 0 ? 0 : (int)(rhf >> 16);
        int key = k == 0 ? 0 : rkey;
        if (!done && i >= 0 && i < tlen) {
            bad |= tc_raw >= (uint32_t)sc.m;
            const uint32_t tc = tc_raw & 7u;
            const uint32_t plo = prof_s[2 * tc], phi = prof_s[2 * tc + 1];
            int hd = hprev_in;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const int sc_c = (int)prmt(plo, phi, W.qsel[c]);
                const int m0 = relu_addmax(hd, sc_c, E[c]);  // max(H(i-1,j-1)+s, E, 0)
                const int h = m0 > f ? m0 : f;
                const int kk = h * 65536 + W.kcol[c];       // largest h, then smallest column
                key = key > kk ? key : kk;
                E[c] = relu_addmax(E[c], -e_del, h - oe_del);  // E opens from H
                f = relu_addmax(f, -e_ins, m0 - oe_ins);       // see the header: exact for o_ins >= 0
                hd = Hp[c];
                Hp[c] = h;
            }
            send_hf = (uint32_t)(Hp[C - 1] & 0xffff) | ((uint32_t)f << 16);
            send_key = key;
            if (k == L - 1) {  // row i is complete in this lane
                const int rmax = key >> 16;
                if (trk) trk->push(i, rmax, minsc);
                if (rmax > gmax) {
                    gmax = rmax;
                    te = i;
                    qe = 0xffff - (key & 0xffff);
                    if (gmax >= endsc) done = true;
                }
            }
        }
        hprev_in = h_in;
        if (stop_enabled) {  // warp-uniform: early stop, the last lane tells its group
            done = __shfl_sync(0xffffffffu, done, L - 1, L);
            const bool all_done = __all_sync(0xffffffffu, done);
            if (all_done) break;
        }
    }
    WfOut r;
    r.score = __shfl_sync(0xffffffffu, gmax, L - 1, L);
    r.te = __shfl_sync(0xffffffffu, te, L - 1, L);
    r.qe = __shfl_sync(0xffffffffu, qe, L - 1, L);
    if (r.te < 0) r.qe = -1;
    return r;
}

template <int L, int C>
__global__ void __launch_bounds__(128)
rescue_wf_kernel(const uint8_t *__restrict__ seq, const bwacuda_dev_rescue_job *__restrict__ jobs,
                 const uint32_t *__restrict__ order, uint32_t n, const __grid_constant__ Scoring sc, int mode,
                 int lanes_fixed, int minsc_all, int pair_cols, uint2 *__restrict__ scratch,
                 const uint64_t *__restrict__ scratch_off, bwacuda_rescue_result *__restrict__ out_aln,
                 bwacuda_fwd_result *__restrict__ out_fwd, uint32_t *__restrict__ err)
{
    __shared__ uint32_t prof_s[16];
    if (threadIdx.x < 16) prof_s[threadIdx.x] = sc.prof[threadIdx.x >> 1][threadIdx.x & 1];
    __syncthreads();
    const uint32_t gid = (blockIdx.x * blockDim.x + threadIdx.x) / L;
    WfLane<L, C> W;
    W.k = threadIdx.x % L;
    bool active = gid < n;
    const uint32_t jid = active ? (order ? order[gid] : gid) : 0u;
    bwacuda_dev_rescue_job J;
    J.qlen = 0; J.tlen = 0; J.q_off = 0; J.t_off = 0; J.minsc = 0; J.endsc = 0;
    if (active) J = jobs[jid];
    const int lanes = lanes_fixed ? lanes_fixed : (J.qlen * sc.max_sc < 250 ? 16 : 8);
    const int qpad = (J.qlen + lanes - 1) / lanes * lanes;
    // jobs whose scores need int32 cells go to the wide shared-memory launch; jobs the paired
    // wavefront took are done
    if (active && (long long)min(J.qlen, J.tlen) * sc.max_sc >= 32768) active = false;
    if (active && rescue_pair_job_ok(J.qlen, J.tlen, sc.max_sc, lanes_fixed, pair_cols)) active = false;
    if (active && qpad > L * C) {
        if (W.k == 0) atomicOr(err, ERR_RANGE);  // the host sizes C from the batch
        active = false;
    }
    const uint8_t *q = seq + J.q_off;
    const uint8_t *t = seq + J.t_off;
    const int minsc = mode == 2 ? J.minsc : minsc_all;
    const int endsc = mode == 2 ? J.endsc : 0x7fffffff;
    bool bad = false;
    WfTracker trk;
    trk.init(active ? scratch + scratch_off[jid] : nullptr, active ? (int)rescue_scratch_entries(J.tlen) : 0);
    const bool last = W.k == L - 1;
    wf_load_query<L, C>(W, q, active ? J.qlen : 0, qpad, false, 0, sc.m, bad);
    // endsc is per job in mode 2 (the pass then stops group by group); the
    // forward pass of modes 0 and 1 never stops early.
    const WfOut fw = wf_pass<L, C>(W, prof_s, t, active ? J.tlen : 0, 0, 0, sc, minsc, endsc, mode == 2,
                                   (active && last) ? &trk : nullptr, active, bad);
    int score2 = -1, te2 = -1;
    if (last && active) {
        trk.finish(fw.score, fw.te, sc.max_sc, score2, te2);
        if (trk.overflow) atomicOr(err, ERR_SCRATCH);
    }
    if (mode == 2) {
        if (last && active) {
            bwacuda_fwd_result r;
            r.score = fw.score; r.te = fw.te; r.qe = fw.qe; r.score2 = score2; r.te2 = te2;
            out_fwd[jid] = r;
        }
    } else {
        const bool rev = active && fw.score >= minsc && fw.qe >= 0 && fw.qe < J.qlen;
        const int rq = fw.qe + 1;
        const int rl = mode == 0 ? (rq * sc.max_sc < 250 ? 16 : 8) : lanes;
        const int rqpad = rev ? (rq + rl - 1) / rl * rl : 0;
        const int rt = mode == 0 ? fw.te + 1 : J.tlen;
        bool rev_ok = rev && rqpad <= L * C;
        wf_load_query<L, C>(W, q, rev_ok ? rq : 0, rqpad, true, fw.qe, sc.m, bad);
        const WfOut rv = wf_pass<L, C>(W, prof_s, t, rev_ok ? rt : 0, 1, fw.te, sc, 0x7fffffff, fw.score, true,
                                       nullptr, rev_ok, bad);
        if (last && active) {
            bwacuda_rescue_result r;
            r.score = fw.score; r.qb = -1; r.qe = fw.qe; r.tb = -1; r.te = fw.te; r.score2 = score2; r.te2 = te2;
            if (rev && !rev_ok) atomicOr(err, ERR_RANGE);
            if (rev_ok && rv.score == fw.score) {
                r.tb = fw.te - rv.te;
                r.qb = fw.qe - rv.qe;
            }
            out_aln[jid] = r;
        }
    }
    if (bad) atomicOr(err, ERR_BASE);
}

template <int L, int C>
cudaError_t launch_wf(const RescueLaunch &Lr)
{
    const uint32_t threads = 128;
    const uint64_t total = (uint64_t)Lr.n * L;
    const uint32_t grid = (uint32_t)((total + threads - 1) / threads);
    if (grid == 0) return cudaSuccess;
    rescue_wf_kernel<L, C><<<grid, threads, 0, Lr.stream>>>(Lr.seq, Lr.jobs, Lr.order, (uint32_t)Lr.n, Lr.sc, Lr.mode,
                                                            Lr.lanes, Lr.minsc, Lr.pair_cols, Lr.scratch,
                                                            Lr.scratch_off, Lr.out_aln, Lr.out_fwd, Lr.err);
    return cudaGetLastError();
}


// Columns per lane C for a group of L lanes and a padded query of qcap columns:
// the smallest listed C with L * C >= qcap.
template <int L>
cudaError_t launch_for_qcap(const RescueLaunch &Lr, int qcap);

}  // namespace wf
}  // namespace bwacuda
