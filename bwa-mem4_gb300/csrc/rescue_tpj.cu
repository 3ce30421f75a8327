// rescue_tpj.cu -- mate-rescue local Smith-Waterman, one thread per job.
//
// Semantics:
//   forward pass      ksw_local_fwd, crates/bwa-extend/src/sw.rs:921-1075
//   suboptimal list   SuboptimalTracker, crates/bwa-extend/src/sw.rs:789-852
//   start recovery    mode 0: batched_ksw_align2's truncated reverse pass,
//                             crates/bwa-neon/src/matesw.rs:299-497
//                     mode 1: ksw_align2's untruncated reverse pass,
//                             crates/bwa-extend/src/sw.rs:1108-1185
//                     mode 2: forward pass only (per-job minsc / endsc)
//   query padding     crates/bwa-neon/src/matesw.rs:676-686 (16 or 8 wide,
//                     padded columns score 0 and carry the diagonal)
//
// Both passes of a job run back to back in the same thread, so the reverse pass
// needs no second launch and no host round trip.  The DP row (H(i-1, j) and
// E(i, j) for the padded query) lives in shared memory, column j at
// cell[j * T].  Row maxima that clear minsc feed the suboptimal tracker; its
// finalised entries go to a per-job slice of device scratch memory (at most
// tlen/2 + 2 entries, since consecutive entries are two or more rows apart),
// the still-open last entry stays in registers.
//
// Work unit (cells): qlen * tlen of the forward pass, the reference's own
// convention (crates/bwa-neon/src/matesw.rs:151-155).
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"

namespace bwacuda {

namespace {

template <bool WIDE>
struct ResCell;

template <>
struct ResCell<false> {
    using T = uint32_t;
    using Key = int32_t;
    __device__ static __forceinline__ T pack(int h, int e) { return __byte_perm((uint32_t)h, (uint32_t)e, 0x5410); }
    __device__ static __forceinline__ int h(T c) { return (int)(c & 0xffffu); }
    __device__ static __forceinline__ int e(T c) { return (int)(c >> 16); }
    // max key -> largest h, then smallest column (strict `>` keeps the first)
    __device__ static __forceinline__ Key key(int h, int j) { return (h << 16) | (0xffff - j); }
    __device__ static __forceinline__ int key_h(Key k) { return k >> 16; }
    __device__ static __forceinline__ int key_j(Key k) { return 0xffff - (k & 0xffff); }
};

template <>
struct ResCell<true> {
    using T = int2;
    using Key = long long;
    __device__ static __forceinline__ T pack(int h, int e) { return make_int2(h, e); }
    __device__ static __forceinline__ int h(T c) { return c.x; }
    __device__ static __forceinline__ int e(T c) { return c.y; }
    __device__ static __forceinline__ Key key(int h, int j) { return ((long long)h << 32) | (unsigned)(0x7fffffff - j); }
    __device__ static __forceinline__ int key_h(Key k) { return (int)(k >> 32); }
    __device__ static __forceinline__ int key_j(Key k) { return 0x7fffffff - (int)(k & 0xffffffffLL); }
};

__device__ __forceinline__ int pad_lanes(int qlen, int max_sc) { return qlen * max_sc < 250 ? 16 : 8; }

__device__ __forceinline__ bool res_fits_narrow(int qlen, int tlen, int max_sc)
{
    long long mn = qlen < tlen ? qlen : tlen;
    return mn * (long long)(max_sc > 0 ? max_sc : 0) < 32768 && qlen + 32 < 65536;
}

struct FwdOut {
    int score, te, qe;
};

// Suboptimal tracker with its finalised entries in device scratch.
struct Tracker {
    uint2 *slot;
    int cap, nb;
    int ls, lr;
    bool has, overflow;
    __device__ void init(uint2 *s, int c)
    {
        slot = s; cap = c; nb = 0; ls = 0; lr = 0; has = false; overflow = false;
    }
    // crates/bwa-extend/src/sw.rs:806-829
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
    // crates/bwa-extend/src/sw.rs:831-851
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

// One forward local-SW pass (sw.rs:921-1075) over a logical query/target.
// Query codes are already in shared memory (qw), padded columns carry PAD_CODE.
// tmap: 0 = target as is, 1 = reversed prefix t[te0-i] for i <= te0 then t[i]
// (untruncated reverse), the truncated reverse uses tmap 1 with tlen = te0+1.
template <bool WIDE, int TB>
__device__ FwdOut local_pass(typename ResCell<WIDE>::T *cell, const uint32_t *qw, int qpad,
                             const uint8_t *t, int tlen, int tmap, int te0, const Scoring &sc,
                             int minsc, int endsc, Tracker *trk, bool &bad)
{
    using C = ResCell<WIDE>;
    const int oe_del = sc.o_del + sc.e_del, oe_ins = sc.o_ins + sc.e_ins;
    const int e_del = sc.e_del, e_ins = sc.e_ins;
    for (int j = 0; j < qpad; ++j) cell[(size_t)j * TB] = C::pack(0, 0);
    int gmax = 0, te = -1, qe = -1;
    for (int i = 0; i < tlen; ++i) {
        uint32_t tc = (tmap && i <= te0) ? t[te0 - i] : t[i];
        bad |= tc >= (uint32_t)sc.m;
        tc &= 7u;
        const uint32_t plo = sc.prof[tc][0], phi = sc.prof[tc][1];
        int f = 0, hd = 0;
        typename C::Key rowkey = 0;
        for (int j = 0; j < qpad; ++j) {
            const typename C::T c = cell[(size_t)j * TB];
            const int hp = C::h(c);
            const int e = C::e(c);
            const uint32_t qc = (qw[(j >> 2) * TB] >> ((j & 3) * 8)) & 0xffu;
            int h = hd + prof_score(plo, phi, qc);
            h = h > 0 ? h : 0;
            h = h > e ? h : e;
            h = h > f ? h : f;
            const typename C::Key kk = C::key(h, j);
            rowkey = rowkey > kk ? rowkey : kk;
            int en = e - e_del, od = h - oe_del;  // gaps open from H (sw.rs:1007-1029)
            en = en > od ? en : od;
            en = en > 0 ? en : 0;
            int fn = f - e_ins, oi = h - oe_ins;
            fn = fn > oi ? fn : oi;
            f = fn > 0 ? fn : 0;
            cell[(size_t)j * TB] = C::pack(h, en);
            hd = hp;
        }
        const int rmax = C::key_h(rowkey);
        if (trk) trk->push(i, rmax, minsc);
        if (rmax > gmax) {  // first row reaching the max keeps te
            gmax = rmax;
            te = i;
            qe = C::key_j(rowkey);
            if (gmax >= endsc) break;
        }
    }
    FwdOut r;
    r.score = gmax;
    r.te = te;
    r.qe = te >= 0 ? qe : -1;
    return r;
}

template <int TB>
__device__ void load_query(uint32_t *qw, const uint8_t *q, int qlen, int qpad, bool reverse, int qe0,
                           int m, bool &bad)
{
    for (int jw = 0; jw * 4 < qpad; ++jw) {
        uint32_t v = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = jw * 4 + u;
            uint32_t c = (uint32_t)PAD_CODE;
            if (j < qlen) {
                c = reverse ? q[qe0 - j] : q[j];
                bad |= c >= (uint32_t)m;
                c = c < (uint32_t)m ? c : (uint32_t)PAD_CODE;  // keep invalid codes off the profile
            }
            v |= c << (8 * u);
        }
        qw[jw * TB] = v;
    }
}

template <bool WIDE, int TB>
__global__ void __launch_bounds__(TB)
rescue_tpj_kernel(const uint8_t *__restrict__ seq, const bwacuda_dev_rescue_job *__restrict__ jobs,
                  const uint32_t *__restrict__ order, const uint32_t *__restrict__ count_ptr,
                  uint32_t n, const __grid_constant__ Scoring sc, int mode, int lanes_fixed, int minsc_all, int qcap,
                  int only_wide, uint2 *__restrict__ scratch, const uint64_t *__restrict__ scratch_off,
                  bwacuda_rescue_result *__restrict__ out_aln, bwacuda_fwd_result *__restrict__ out_fwd,
                  uint32_t *__restrict__ err)
{
    using C = ResCell<WIDE>;
    using CellT = typename C::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    CellT *cell = reinterpret_cast<CellT *>(smem_raw) + tid;
    uint32_t *qw = reinterpret_cast<uint32_t *>(reinterpret_cast<CellT *>(smem_raw) + (size_t)qcap * TB) + tid;

    const uint32_t lim = count_ptr ? min(*count_ptr, n) : n;  // a device count never exceeds the launch's n
    const uint32_t k = blockIdx.x * TB + tid;
    if (k >= lim) return;
    const uint32_t jid = order ? order[k] : k;
    const bwacuda_dev_rescue_job J = jobs[jid];
    const int qlen = J.qlen, tlen = J.tlen;
    if (!WIDE && !res_fits_narrow(qlen, tlen, sc.max_sc)) {  // left to the wide launch
        if (only_wide == 2) atomicOr(err, ERR_RANGE);          // ... unless none follows
        return;
    }
    if (WIDE && only_wide && res_fits_narrow(qlen, tlen, sc.max_sc)) return;
    const int lanes = lanes_fixed ? lanes_fixed : pad_lanes(qlen, sc.max_sc);
    const int qpad = (qlen + lanes - 1) / lanes * lanes;
    if (qpad + 16 > qcap) { atomicOr(err, ERR_RANGE); return; }
    const uint8_t *q = seq + J.q_off;
    const uint8_t *t = seq + J.t_off;
    const int minsc = mode == 2 ? J.minsc : minsc_all;
    const int endsc = mode == 2 ? J.endsc : 0x7fffffff;
    bool bad = false;

    Tracker trk;
    trk.init(scratch + scratch_off[jid], (int)rescue_scratch_entries(tlen));
    load_query<TB>(qw, q, qlen, qpad, false, 0, sc.m, bad);
    const FwdOut fw = local_pass<WIDE, TB>(cell, qw, qpad, t, tlen, 0, 0, sc, minsc, endsc, &trk, bad);
    int score2, te2;
    trk.finish(fw.score, fw.te, sc.max_sc, score2, te2);
    if (trk.overflow) atomicOr(err, ERR_SCRATCH);

    if (mode == 2) {
        bwacuda_fwd_result r;
        r.score = fw.score; r.te = fw.te; r.qe = fw.qe; r.score2 = score2; r.te2 = te2;
        out_fwd[jid] = r;
    } else {
        bwacuda_rescue_result r;
        r.score = fw.score; r.qb = -1; r.qe = fw.qe; r.tb = -1; r.te = fw.te;
        r.score2 = score2; r.te2 = te2;
        if (fw.score >= minsc && fw.qe >= 0) {
            // start recovery: reversed query prefix, reversed target prefix
            const int rq = fw.qe + 1;
            const int rl = mode == 0 ? pad_lanes(rq, sc.max_sc) : lanes;
            const int rqpad = (rq + rl - 1) / rl * rl;
            const int rt = mode == 0 ? fw.te + 1 : tlen;
            // qe lies inside the real query whenever gap opens cost >= 0 (validated
            // on the host); guard the reversed read regardless.
            if (rq > qlen || rqpad > qcap) {
                atomicOr(err, ERR_RANGE);
                return;
            }
            load_query<TB>(qw, q, rq, rqpad, true, fw.qe, sc.m, bad);
            const FwdOut rv = local_pass<WIDE, TB>(cell, qw, rqpad, t, rt, 1, fw.te, sc, 0x7fffffff,
                                                   fw.score, nullptr, bad);
            if (rv.score == fw.score) {
                r.tb = fw.te - rv.te;
                r.qb = fw.qe - rv.qe;
            }
        }
        out_aln[jid] = r;
    }
    if (bad) atomicOr(err, ERR_BASE);
}

constexpr size_t SMEM_MAX = 227u * 1024u;

template <bool WIDE>
size_t res_smem_bytes(int qcap, int tb)
{
    size_t cellsz = WIDE ? 8 : 4;
    size_t qwords = (size_t)(qcap + 3) / 4;
    return (size_t)qcap * tb * cellsz + qwords * tb * 4;
}

template <bool WIDE, int TB>
cudaError_t launch_res_tb(const RescueLaunch &L)
{
    size_t smem = res_smem_bytes<WIDE>(L.qcap, TB);
    // process-wide per kernel: always the ceiling (concurrent contexts must not shrink it)
    cudaError_t e = cudaFuncSetAttribute(rescue_tpj_kernel<WIDE, TB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_MAX);
    if (e != cudaSuccess) return e;
    uint32_t grid = (uint32_t)((L.n + TB - 1) / TB);
    if (grid == 0) return cudaSuccess;
    rescue_tpj_kernel<WIDE, TB><<<grid, TB, smem, L.stream>>>(
        L.seq, L.jobs, L.order, L.count_ptr, (uint32_t)L.n, L.sc, L.mode, L.lanes, L.minsc,
        L.qcap, L.only_wide, L.scratch, L.scratch_off, L.out_aln, L.out_fwd, L.err);
    return cudaGetLastError();
}

template <bool WIDE>
cudaError_t launch_res(const RescueLaunch &L)
{
    if (res_smem_bytes<WIDE>(L.qcap, 128) <= SMEM_MAX) return launch_res_tb<WIDE, 128>(L);
    if (res_smem_bytes<WIDE>(L.qcap, 64) <= SMEM_MAX) return launch_res_tb<WIDE, 64>(L);
    if (res_smem_bytes<WIDE>(L.qcap, 32) <= SMEM_MAX) return launch_res_tb<WIDE, 32>(L);
    return cudaErrorInvalidValue;
}

// Exclusive scan of per-job tracker capacities (three small kernels).
constexpr int SCAN_B = 1024;

__global__ void scan_block_kernel(const bwacuda_dev_rescue_job *__restrict__ jobs, uint32_t n,
                                  uint64_t *__restrict__ off, uint64_t *__restrict__ block_sum)
{
    __shared__ uint64_t s[SCAN_B];
    const uint32_t i = blockIdx.x * SCAN_B + threadIdx.x;
    uint64_t v = i < n ? rescue_scratch_entries(jobs[i].tlen) : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int d = 1; d < SCAN_B; d <<= 1) {  // Hillis-Steele inclusive scan
        uint64_t add = threadIdx.x >= (unsigned)d ? s[threadIdx.x - d] : 0;
        __syncthreads();
        s[threadIdx.x] += add;
        __syncthreads();
    }
    if (i < n) off[i] = s[threadIdx.x] - v;
    if (threadIdx.x == SCAN_B - 1) block_sum[blockIdx.x] = s[SCAN_B - 1];
}

__global__ void scan_sums_kernel(uint64_t *__restrict__ block_sum, uint32_t nb)
{
    // one block: exclusive scan of the block sums in chunks, carrying the total
    __shared__ uint64_t s[SCAN_B];
    uint64_t carry = 0;
    for (uint32_t base = 0; base < nb; base += SCAN_B) {
        const uint32_t i = base + threadIdx.x;
        uint64_t v = i < nb ? block_sum[i] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int d = 1; d < SCAN_B; d <<= 1) {
            uint64_t add = threadIdx.x >= (unsigned)d ? s[threadIdx.x - d] : 0;
            __syncthreads();
            s[threadIdx.x] += add;
            __syncthreads();
        }
        if (i < nb) block_sum[i] = carry + s[threadIdx.x] - v;
        const uint64_t tot = s[SCAN_B - 1];
        __syncthreads();
        carry += tot;
    }
}

__global__ void scan_add_kernel(uint64_t *__restrict__ off, uint32_t n, const uint64_t *__restrict__ block_sum)
{
    const uint32_t i = blockIdx.x * SCAN_B + threadIdx.x;
    if (i < n) off[i] += block_sum[blockIdx.x];
}

}  // namespace

size_t rescue_tpj_smem_limit_qcap(bool wide)
{
    size_t q = SMEM_MAX / ((wide ? 8 : 4) * 32 + 32);
    while (q > 0 && (wide ? res_smem_bytes<true>((int)q, 32) : res_smem_bytes<false>((int)q, 32)) > SMEM_MAX) --q;
    return q;
}

cudaError_t rescue_tpj_launch(const RescueLaunch &L, bool wide)
{
    return wide ? launch_res<true>(L) : launch_res<false>(L);
}

// tmp must hold ceil(n / 1024) uint64 block sums.
cudaError_t rescue_scratch_offsets(const bwacuda_dev_rescue_job *jobs, size_t n, uint64_t *off,
                                   void *tmp, size_t tmp_bytes, size_t *tmp_needed, cudaStream_t s)
{
    const uint32_t nb = (uint32_t)((n + SCAN_B - 1) / SCAN_B);
    if (tmp_needed) *tmp_needed = (size_t)(nb ? nb : 1) * sizeof(uint64_t);
    if (n == 0 || tmp == nullptr) return cudaSuccess;
    if (tmp_bytes < (size_t)nb * sizeof(uint64_t)) return cudaErrorInvalidValue;
    uint64_t *bs = static_cast<uint64_t *>(tmp);
    scan_block_kernel<<<nb, SCAN_B, 0, s>>>(jobs, (uint32_t)n, off, bs);
    scan_sums_kernel<<<1, SCAN_B, 0, s>>>(bs, nb);
    scan_add_kernel<<<nb, SCAN_B, 0, s>>>(off, (uint32_t)n, bs);
    return cudaGetLastError();
}

}  // namespace bwacuda
