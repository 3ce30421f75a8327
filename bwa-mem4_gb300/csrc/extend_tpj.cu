// extend_tpj.cu -- banded seed extension (ksw_extend2), one thread per job.
//
// Semantics: crates/bwa-extend/src/sw.rs:203-493, integer for integer, with the
// qlen == 0 convention of the production lockstep path
// (crates/bwa-neon/src/batched.rs:1025-1039).
//
// Layout.  Each thread owns one job.  Its persistent DP row (H(i-1, j-1) and
// E(i, j) for j = 0..qlen) lives in shared memory, column j at word
// cell[j * T] (T = threads per block), so a warp touching any mix of columns
// hits 32 distinct banks.  Cells outside the live window [beg, end) are never
// written, so they keep the stale values of earlier rows exactly as the scalar
// code does (sw.rs:465-482 can grow `end` by two and read them back).
// Narrow cells pack H (low 16 bits) and E (high 16 bits): legal whenever
// h0 + min(qlen, tlen) * max_sc < 32768, which covers the reference's 8-bit and
// 16-bit bins (crates/bwa-neon/src/batched.rs:817-865).  Wide cells hold two
// int32 and serve the reference's scalar bin.
// The query codes sit in shared memory too, four per word (word jw of the
// thread at qw[jw * T]).
//
// Work unit (cells): one iteration of the inner column loop, i.e. the sum over
// processed rows of (end - beg), the same count the oracle reports.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"

namespace bwacuda {

namespace {

template <bool WIDE>
struct ExtCell;

template <>
struct ExtCell<false> {
    using T = uint32_t;
    using Key = int32_t;
    __device__ static __forceinline__ T pack(int h, int e) { return __byte_perm((uint32_t)h, (uint32_t)e, 0x5410); }
    __device__ static __forceinline__ int h(T c) { return (int)(c & 0xffffu); }
    __device__ static __forceinline__ int e(T c) { return (int)(c >> 16); }
    __device__ static __forceinline__ bool dead(T c) { return c == 0u; }
    __device__ static __forceinline__ Key key(int h, int j) { return (h << 16) | j; }
    __device__ static __forceinline__ int key_h(Key k) { return k >> 16; }
    __device__ static __forceinline__ int key_j(Key k) { return k & 0xffff; }
};

template <>
struct ExtCell<true> {
    using T = int2;
    using Key = long long;
    __device__ static __forceinline__ T pack(int h, int e) { return make_int2(h, e); }
    __device__ static __forceinline__ int h(T c) { return c.x; }
    __device__ static __forceinline__ int e(T c) { return c.y; }
    __device__ static __forceinline__ bool dead(T c) { return c.x == 0 && c.y == 0; }
    __device__ static __forceinline__ Key key(int h, int j) { return ((long long)h << 32) | (unsigned)j; }
    __device__ static __forceinline__ int key_h(Key k) { return (int)(k >> 32); }
    __device__ static __forceinline__ int key_j(Key k) { return (int)(k & 0xffffffffLL); }
};

// Narrow storage is legal for this job (all H, E, F values < 32768).
__device__ __forceinline__ bool ext_fits_narrow(const bwacuda_dev_ext_job &J, int max_sc)
{
    long long mn = J.qlen < J.tlen ? J.qlen : J.tlen;
    long long bound = (long long)J.h0 + mn * (max_sc > 0 ? max_sc : 0);
    return bound < 32768;
}

template <bool WIDE, int TB>
__global__ void __launch_bounds__(TB)
ext_tpj_kernel(const uint8_t *__restrict__ seq, const bwacuda_dev_ext_job *__restrict__ jobs,
               const uint32_t *__restrict__ order, const uint32_t *__restrict__ count_ptr,
               uint32_t n, const __grid_constant__ ExtParams P, int qcap, int only_wide, bwacuda_ext_result *__restrict__ out,
               uint32_t *__restrict__ err, unsigned long long *__restrict__ cells_total)
{
    using C = ExtCell<WIDE>;
    using CellT = typename C::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    CellT *cell = reinterpret_cast<CellT *>(smem_raw) + tid;                         // column j: cell[j*TB]
    uint32_t *qw = reinterpret_cast<uint32_t *>(reinterpret_cast<CellT *>(smem_raw) + (size_t)qcap * TB) + tid;

    const uint32_t lim = count_ptr ? *count_ptr : n;
    const uint32_t k = blockIdx.x * TB + tid;
    bool active = k < lim;
    const uint32_t jid = active ? (order ? order[k] : k) : 0u;
    bwacuda_dev_ext_job J;
    if (active) J = jobs[jid];
    // The narrow launch leaves wide jobs to the wide launch; a wide launch with
    // only_wide set skips the jobs the narrow launch handles.
    // For the narrow launch, only_wide == 2 means no wide launch follows: a wide
    // job is then reported as unsupported instead of being left without output.
    if (active && !WIDE && !ext_fits_narrow(J, P.sc.max_sc)) {
        if (only_wide == 2) atomicOr(err, ERR_RANGE);
        active = false;
    }
    if (active && WIDE && only_wide && ext_fits_narrow(J, P.sc.max_sc)) active = false;
    if (active && J.qlen + 1 > qcap) { atomicOr(err, ERR_RANGE); active = false; }

    unsigned long long ncells = 0;
    if (active) {
        const int qlen = J.qlen, tlen = J.tlen, h0 = J.h0, m = P.sc.m;
        const uint8_t *q = seq + J.q_off;
        const uint8_t *t = seq + J.t_off;
        const int o_del = P.sc.o_del, e_del = P.sc.e_del, o_ins = P.sc.o_ins, e_ins = P.sc.e_ins;
        const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;
        bool bad = false;

        // Query codes, four per shared word.
        for (int jw = 0; jw * 4 < qlen; ++jw) {
            uint32_t v = 0;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                int j = jw * 4 + u;
                uint32_t c = j < qlen ? (uint32_t)q[j] : 0u;
                bad |= c >= (uint32_t)m;
                v |= (c & 7u) << (8 * u);
            }
            qw[jw * TB] = v;
        }
        // Row -1 (sw.rs:269-279): h0, then the insertion chain while > e_ins; E = 0.
        {
            int hv = h0;
            cell[0] = C::pack(h0, 0);
            if (qlen >= 1) {
                hv = h0 > oe_ins ? h0 - oe_ins : 0;
                cell[TB] = C::pack(hv, 0);
            }
            for (int j = 2; j <= qlen; ++j) {
                hv = hv > e_ins ? hv - e_ins : 0;
                cell[(size_t)j * TB] = C::pack(hv, 0);
            }
        }
        const int w = clamp_band(J.w < 0 ? 0 : J.w, qlen, P.sc.max_sc, P.end_bonus, o_ins, e_ins,
                                 o_del, e_del);
        int best = h0, best_i = -1, best_j = -1, best_ie = -1, gscore = -1, max_off = 0;
        int beg = 0, end = qlen;
        for (int i = 0; i < tlen; ++i) {
            uint32_t tc = t[i];
            bad |= tc >= (uint32_t)m;
            tc &= 7u;
            const uint32_t plo = P.sc.prof[tc][0], phi = P.sc.prof[tc][1];
            if (beg < i - w) beg = i - w;
            if (end > i + w + 1) end = i + w + 1;
            if (end > qlen) end = qlen;
            int h1 = 0;
            if (beg == 0) {
                h1 = h0 - (o_del + e_del * (i + 1));
                h1 = h1 > 0 ? h1 : 0;
            }
            int f = 0;
            typename C::Key rowkey = 0;
            for (int j = beg; j < end; ++j) {
                const CellT c = cell[(size_t)j * TB];
                const int hd = C::h(c);
                const int e = C::e(c);
                const uint32_t qc = (qw[(j >> 2) * TB] >> ((j & 3) * 8)) & 0xffu;
                const int s = prof_score(plo, phi, qc);
                const int M = hd != 0 ? hd + s : 0;  // zero diagonal is never extended
                int h = M > e ? M : e;
                h = h > f ? h : f;
                int od = M - oe_del;
                od = od > 0 ? od : 0;
                int en = e - e_del;
                en = en > od ? en : od;
                cell[(size_t)j * TB] = C::pack(h1, en);  // H(i, j-1) for the next row, E(i+1, j)
                h1 = h;
                const typename C::Key kk = C::key(h, j);  // ties -> later column
                rowkey = rowkey > kk ? rowkey : kk;
                int oi = M - oe_ins;
                oi = oi > 0 ? oi : 0;
                f -= e_ins;
                f = f > oi ? f : oi;
            }
            if (end > beg) ncells += (unsigned long long)(end - beg);
            cell[(size_t)end * TB] = C::pack(h1, 0);
            const int jf = end > beg ? end : beg;
            if (jf == qlen && gscore <= h1) {
                best_ie = i;
                gscore = h1;
            }
            const int rmax = C::key_h(rowkey);
            const int mj = C::key_j(rowkey);
            if (rmax == 0) break;
            if (rmax > best) {
                best = rmax;
                best_i = i;
                best_j = mj;
                const int off = mj > i ? mj - i : i - mj;
                if (off > max_off) max_off = off;
            } else if (P.zdrop > 0) {
                if (i - best_i > mj - best_j) {
                    if (best - rmax - ((i - best_i) - (mj - best_j)) * e_del > P.zdrop) break;
                } else if (best - rmax - ((mj - best_j) - (i - best_i)) * e_ins > P.zdrop) {
                    break;
                }
            }
            int lo = beg;
            while (lo < end && C::dead(cell[(size_t)lo * TB])) ++lo;
            beg = lo;
            int hi = end;
            while (hi >= beg && C::dead(cell[(size_t)hi * TB])) --hi;
            end = hi + 2 < qlen ? hi + 2 : qlen;
        }
        if (bad) atomicOr(err, ERR_BASE);
        bwacuda_ext_result r;
        r.score = best;
        r.qle = best_j + 1;
        r.tle = best_i + 1;
        r.gtle = best_ie + 1;
        r.gscore = gscore;
        r.max_off = max_off;
        out[jid] = r;
    }
    // one 64-bit atomic per warp for the cell counter
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ncells += __shfl_xor_sync(0xffffffffu, ncells, o);
    if ((tid & 31) == 0 && ncells) atomicAdd(cells_total, ncells);
}

constexpr size_t SMEM_MAX = 227u * 1024u;

template <bool WIDE>
size_t ext_smem_bytes(int qcap, int tb)
{
    size_t cellsz = WIDE ? 8 : 4;
    size_t qwords = (size_t)(qcap + 3) / 4;
    return (size_t)qcap * tb * cellsz + qwords * tb * 4;
}

template <bool WIDE, int TB>
cudaError_t launch_ext_tb(const ExtLaunch &L)
{
    size_t smem = ext_smem_bytes<WIDE>(L.qcap, TB);
    cudaError_t e = cudaFuncSetAttribute(ext_tpj_kernel<WIDE, TB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    uint32_t grid = (uint32_t)((L.n + TB - 1) / TB);
    if (grid == 0) return cudaSuccess;
    ext_tpj_kernel<WIDE, TB><<<grid, TB, smem, L.stream>>>(L.seq, L.jobs, L.order, L.count_ptr,
                                                         (uint32_t)L.n, L.P, L.qcap, L.only_wide, L.out,
                                                         L.err, L.cells);
    return cudaGetLastError();
}

// Largest block (128, 64 or 32 threads) whose shared memory fits.
template <bool WIDE>
cudaError_t launch_ext(const ExtLaunch &L)
{
    if (ext_smem_bytes<WIDE>(L.qcap, 128) <= SMEM_MAX) return launch_ext_tb<WIDE, 128>(L);
    if (ext_smem_bytes<WIDE>(L.qcap, 64) <= SMEM_MAX) return launch_ext_tb<WIDE, 64>(L);
    if (ext_smem_bytes<WIDE>(L.qcap, 32) <= SMEM_MAX) return launch_ext_tb<WIDE, 32>(L);
    return cudaErrorInvalidValue;
}

}  // namespace

size_t ext_tpj_smem_limit_qcap(bool wide)
{
    // largest qcap whose 32-thread block fits in shared memory
    size_t q = SMEM_MAX / ((wide ? 8 : 4) * 32 + 32);
    while (q > 0 && (wide ? ext_smem_bytes<true>((int)q, 32) : ext_smem_bytes<false>((int)q, 32)) > SMEM_MAX) --q;
    return q;
}

cudaError_t ext_tpj_launch(const ExtLaunch &L, bool wide)
{
    return wide ? launch_ext<true>(L) : launch_ext<false>(L);
}

}  // namespace bwacuda
