// ext_slide.cu -- banded seed extension (ksw_extend2, crates/bwa-extend/src/sw.rs:203-493) of
// queries longer than a thread's shared-memory row holds, one thread per job.
//
// The cell update is the thread-per-job 16-bit pair form (ext_job.cuh, ext_run_job_i16p): two
// columns per DPX instruction, H and E in 16-bit lanes, F through the lanes, row maxima as
// (H << 16) | column keys.  What changes is where the row lives.  The full-row kernels hold
// qlen + 1 columns per thread; here a thread holds a window of wc columns [base, base + wc)
// (wc / 2 + 2 pair words and wc / 4 + 3 query words, so ~1.4 KB a job for bands up to 101),
// and before row i, if i - w - 1 - base >= SLIDE_K, the window moves right by SLIDE_K columns:
// the kept pair and query words are copied down and the new ones filled.
//
// Why the results equal the full row's (w the clamped band).  Row i touches columns
// [beg - 1, end + 3] at most (the odd first column's pair word, the look-ahead pair and query
// word, the sentinel column end and the live-cell scans) with beg >= i - w and
// end <= i + w + 1.  The move rule keeps base <= i - w - 1 < base + SLIDE_K once the window has
// moved (base = 0 before), so every touched column lies in [base, base + 2w + 5 + SLIDE_K)
// (slide_fits in ext_long.cuh); a query of qlen + 4 <= wc columns lies in the window whatever
// base is.  Columns left of the window are never touched again (beg never decreases).  A column
// entering on the right lies beyond every column written so far (earlier rows wrote inside the
// old window), so it enters with what the reference's row holds for a never-written column:
// its row -1 value (sw.rs:269-279) and E = 0.  The row-maximum key carries the column relative
// to base (below 2^16 for any window) and is decoded back within the row.  A row with an empty
// band ends the job (its maximum is 0, sw.rs:436-438) before anything reads its sentinel, which
// may lie left of the window and is not written.
//
// Work split.  The batched path's open-ended buckets (the queries the full-row kernels cannot
// hold) run this kernel ahead of the group-per-job kernel (ext_long.cuh); both evaluate
// slide_takes on every job, so each job runs in exactly one of them.  The window kernel takes a
// bucket only when it holds at least slide_min jobs (a thread per job needs many jobs to fill
// the GPU); the sort orders these buckets by target length, longest first.
#include <cuda_runtime.h>

#include <algorithm>

#include "ext_long.cuh"
#include "kernels.h"

namespace bwacuda {
namespace slide {

using xl::FULL;
using xl::SLIDE_K;

constexpr int TB = 32;  // one warp per block: the finest step of the shared-memory footprint

__host__ __device__ inline int win_pairs(int wc) { return wc / 2 + 2; }
__host__ __device__ inline int win_qwords(int wc) { return wc / 4 + 3; }
__host__ __device__ inline size_t job_bytes(int wc) { return (size_t)win_pairs(wc) * 8 + (size_t)win_qwords(wc) * 4; }

// Query selector word of columns c .. c + 3: bytes 0x80 | code * 0x11 (the prmt selector of the
// pair form), code 0 past the query.
__device__ __forceinline__ uint32_t query_word(const uint8_t *__restrict__ q, int qlen, int c)
{
    uint32_t v = 0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int j = c + u;
        const uint32_t code = j < qlen ? (uint32_t)q[j] : 0u;
        v |= (0x80u | (code & 7u) * 0x11u) << (8 * u);
    }
    return v;
}

// Row -1 pair word of columns c, c + 1 (c even): H = the row -1 value up to column qlen, E = 0.
__device__ __forceinline__ uint2 row_minus1_pair(int c, int qlen, int h0, int oe_ins, int e_ins)
{
    const int a = c <= qlen ? xl::row_minus1(c, h0, oe_ins, e_ins) : 0;
    const int b = c + 1 <= qlen ? xl::row_minus1(c + 1, h0, oe_ins, e_ins) : 0;
    return make_uint2((uint32_t)a | ((uint32_t)b << 16), 0u);
}

template <bool SYM>
__device__ __forceinline__ bwacuda_ext_result slide_job(uint2 *__restrict__ cell2, uint32_t *__restrict__ qw, int wc,
                                                        const uint8_t *__restrict__ seq, const bwacuda_dev_ext_job &J,
                                                        int w, const ExtParams &P, bool &bad,
                                                        unsigned long long &ncells)
{
    const int qlen = J.qlen, tlen = J.tlen, h0 = J.h0, m = P.sc.m;
    const uint8_t *q = seq + J.q_off;
    const uint8_t *t = seq + J.t_off;
    const int o_del = P.sc.o_del, e_del = P.sc.e_del, o_ins = P.sc.o_ins, e_ins = P.sc.e_ins;
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;
    const int np = win_pairs(wc), nq = win_qwords(wc);
    constexpr int KP = SLIDE_K / 2, KQ = SLIDE_K / 4;

    // every query code is checked, as the full-row kernels check the staged query
    for (int j = 0; j < qlen; ++j) bad |= q[j] >= (uint32_t)m;
    for (int p = 0; p < np; ++p) cell2[p * TB] = row_minus1_pair(2 * p, qlen, h0, oe_ins, e_ins);
    for (int x = 0; x < nq; ++x) qw[x * TB] = query_word(q, qlen, 4 * x);
    const bool moves = (long long)qlen + 4 > wc;
    int base = 0;  // first column of the window, a multiple of SLIDE_K

    int best = h0, best_i = -1, best_j = -1, best_ie = -1, gscore = -1, max_off = 0;
    int beg = 0, end = qlen;
    uint32_t tnext = tlen > 0 ? t[0] : 0u;
    const uint32_t noe_ins2 = (uint32_t)(-oe_ins & 0xffff) * 0x10001u;
    const uint32_t noe_del2 = (uint32_t)(-oe_del & 0xffff) * 0x10001u;
    const uint32_t ne_del2 = (uint32_t)(-e_del & 0xffff) * 0x10001u;
    const uint32_t ne_ins2 = (uint32_t)(-e_ins & 0xffff) * 0x10001u;
    const uint32_t fsel2 = 0x8000u | ((uint32_t)(-e_ins & 0xffff) << 16);
    for (int i = 0; i < tlen; ++i) {
        if (moves && i - w - 1 - base >= SLIDE_K) {
            for (int p = 0; p < np - KP; ++p) cell2[p * TB] = cell2[(p + KP) * TB];
            for (int p = np - KP; p < np; ++p)
                cell2[p * TB] = row_minus1_pair(base + SLIDE_K + 2 * p, qlen, h0, oe_ins, e_ins);
            for (int x = 0; x < nq - KQ; ++x) qw[x * TB] = qw[(x + KQ) * TB];
            for (int x = nq - KQ; x < nq; ++x) qw[x * TB] = query_word(q, qlen, base + SLIDE_K + 4 * x);
            base += SLIDE_K;
        }
        uint32_t tc = tnext;
        if (i + 1 < tlen) tnext = t[i + 1];
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
        int32_t rowkey = 0;
        if (beg < end) {
            // columns relative to the window (base is a multiple of 4: same parity and
            // position in a query word)
            const int rend = end - base;
            int j = beg - base;
            if (j & 1) {  // odd first column: the high lanes of its pair
                const uint2 wv = cell2[(j >> 1) * TB];
                const uint32_t qc = (qw[(j >> 2) * TB] >> ((j & 3) * 8)) & 7u;
                int h, en;
                ext_cell((int)(wv.x >> 16), (int)(wv.y >> 16), qc, plo, phi, oe_del, e_del, oe_ins, e_ins, f, h, en);
                cell2[(j >> 1) * TB] =
                    make_uint2((wv.x & 0xffffu) | ((uint32_t)h1 << 16), (wv.y & 0xffffu) | ((uint32_t)en << 16));
                h1 = h;
                const int32_t kk = (h << 16) | j;
                rowkey = rowkey > kk ? rowkey : kk;
                ++j;
            }
            uint2 wn = cell2[(j >> 1) * TB];
            uint32_t fv = (uint32_t)f << 16, h1v = (uint32_t)h1 << 16;
            // cw: the pair word of the current pair (running pointer: constant offsets, no
            // per-pair index arithmetic)
            uint2 *cw = cell2 + (j >> 1) * TB;
            // columns jj, jj + 1 from their pair word wv (read before it is stored at cw[off])
            auto cell_pair = [&](uint2 wv, uint32_t sel, int off, int jj) {
                const uint32_t s2 = prmt(plo, phi, sel);
                const uint32_t hd2 = wv.x, e2 = wv.y;
                const uint32_t g2 = __viaddmin_u16x2(hd2, 0u, 0x00010001u) * 0x7fffu;
                const uint32_t M2 = __viaddmin_s16x2(hd2, s2, g2);
                const uint32_t ti2 = __viaddmax_s16x2_relu(M2, noe_ins2, 0u);
                const uint32_t td2 = SYM ? ti2 : __viaddmax_s16x2_relu(M2, noe_del2, 0u);
                const uint32_t en2 = __viaddmax_s16x2(e2, ne_del2, td2);
                const uint32_t f2 = f_pair(fv, ti2, fsel2, ne_ins2);
                const uint32_t h2 = __vimax3_s16x2(M2, e2, f2);
                cw[off] = make_uint2(prmt(h1v, h2, 0x5432u), en2);
                h1v = h2;
                rowkey = pair_rowkey(rowkey, h2, jj);
            };
            auto pair_at = [&](int off, uint32_t sel, int jj) {
                const uint2 wv = wn;
                wn = cw[off + TB];  // the window's spare pairs keep this inside
                cell_pair(wv, sel, off, jj);
            };
            if ((j & 2) && j + 1 < rend) {
                pair_at(0, qw[(j >> 2) * TB] >> 16, j);
                j += 2;
                cw += TB;
            }
            // Sixteen columns a step, their eight pair words and four query words loaded
            // together: a thread is often alone on its scheduler here, and only F and the row
            // key carry from pair to pair, so the pairs' other work overlaps.
            if (j + 15 < rend) {
                const uint32_t *qp = qw + (j >> 2) * TB;
                for (; j + 15 < rend; j += 16) {
                    uint2 wv[8];
                    uint32_t qv[4];
#pragma unroll
                    for (int u = 0; u < 8; ++u) wv[u] = cw[u * TB];
#pragma unroll
                    for (int u = 0; u < 4; ++u) qv[u] = qp[u * TB];
                    // phase by phase over the eight pairs (the same operations per pair as
                    // cell_pair): a warp alone on its scheduler issues in order, so independent
                    // instructions go back to back and only F chains from pair to pair
                    uint32_t M2[8], ti2[8], en2[8], f2[8], h2[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const uint32_t s2 = prmt(plo, phi, qv[u >> 1] >> ((u & 1) * 16));
                        const uint32_t g2 = __viaddmin_u16x2(wv[u].x, 0u, 0x00010001u) * 0x7fffu;
                        M2[u] = __viaddmin_s16x2(wv[u].x, s2, g2);
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) ti2[u] = __viaddmax_s16x2_relu(M2[u], noe_ins2, 0u);
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const uint32_t td2 = SYM ? ti2[u] : __viaddmax_s16x2_relu(M2[u], noe_del2, 0u);
                        en2[u] = __viaddmax_s16x2(wv[u].y, ne_del2, td2);
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) f2[u] = f_pair(fv, ti2[u], fsel2, ne_ins2);
#pragma unroll
                    for (int u = 0; u < 8; ++u) h2[u] = __vimax3_s16x2(M2[u], wv[u].y, f2[u]);
#pragma unroll
                    for (int u = 0; u < 8; ++u) cw[u * TB] = make_uint2(prmt(u == 0 ? h1v : h2[u - 1], h2[u], 0x5432u), en2[u]);
                    h1v = h2[7];
#pragma unroll
                    for (int u = 0; u < 8; ++u) rowkey = pair_rowkey(rowkey, h2[u], j + 2 * u);
                    cw += 8 * TB;
                    qp += 4 * TB;
                }
                wn = cw[0];  // j <= rend: inside the window
            }
            if (j + 3 < rend) {
                const uint32_t *qp = qw + (j >> 2) * TB;
                uint32_t qn = qp[0];
                for (; j + 3 < rend; j += 4) {
                    const uint32_t qv = qn;
                    qp += TB;
                    qn = qp[0];  // the window's spare words keep this inside
                    pair_at(0, qv, j);
                    pair_at(TB, qv >> 16, j + 2);
                    cw += 2 * TB;
                }
            }
            if (j + 1 < rend) {
                pair_at(0, qw[(j >> 2) * TB] >> ((j & 2) * 8), j);
                j += 2;
            }
            f = (int)(fv >> 16);
            h1 = (int)(h1v >> 16);
            if (j < rend) {  // even last column: the low lanes of its pair
                const uint2 wv = wn;
                const uint32_t qc = (qw[(j >> 2) * TB] >> ((j & 3) * 8)) & 7u;
                int h, en;
                ext_cell((int)(wv.x & 0xffffu), (int)(wv.y & 0xffffu), qc, plo, phi, oe_del, e_del, oe_ins, e_ins, f,
                         h, en);
                cell2[(j >> 1) * TB] = make_uint2((wv.x & 0xffff0000u) | (uint32_t)h1, (wv.y & 0xffff0000u) | (uint32_t)en);
                h1 = h;
                const int32_t kk = (h << 16) | j;
                rowkey = rowkey > kk ? rowkey : kk;
            }
            ncells += (unsigned long long)(end - beg);
            // sentinel column end (sw.rs:418-419): H = h1, E = 0
            const uint2 sv = cell2[(rend >> 1) * TB];
            cell2[(rend >> 1) * TB] = (rend & 1) ? make_uint2((sv.x & 0xffffu) | ((uint32_t)h1 << 16), sv.y & 0xffffu)
                                                 : make_uint2((sv.x & 0xffff0000u) | (uint32_t)h1, sv.y & 0xffff0000u);
        }
        const int jf = end > beg ? end : beg;
        if (jf == qlen && gscore <= h1) {
            best_ie = i;
            gscore = h1;
        }
        const int rmax = rowkey >> 16;
        const int mj = (rowkey & 0xffff) + base;
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
        // adaptive band (sw.rs:465-482) over this row's cells [beg, end]
        const int rb = beg - base, re = end - base;
        int lo = rb;
        while (lo < re && i16p_dead<TB>(cell2, lo)) ++lo;
        beg = lo + base;
        int hi = re;
        while (hi >= lo && i16p_dead<TB>(cell2, hi)) --hi;
        hi += base;
        end = hi + 2 < qlen ? hi + 2 : qlen;
    }
    bwacuda_ext_result r;
    r.score = best;
    r.qle = best_j + 1;
    r.tle = best_i + 1;
    r.gtle = best_ie + 1;
    r.gscore = gscore;
    r.max_off = max_off;
    return r;
}

// Jobs from order[bounds[0] .. bounds[1]) (order nullptr: the identity), 32 per warp grab from
// *counter; a job is this kernel's when it is a 16-bit job of qlen >= min_qlen that slide_takes
// gives to it (the group kernel leaves exactly those).
__global__ void __launch_bounds__(TB)
ext_slide_kernel(const uint8_t *__restrict__ seq, const bwacuda_dev_ext_job *__restrict__ jobs,
                 const uint32_t *__restrict__ order, const uint32_t *__restrict__ bounds,
                 uint32_t *__restrict__ counter, uint32_t njobs, int min_qlen, int wc, uint32_t slide_min,
                 const __grid_constant__ ExtParams P, bwacuda_ext_result *__restrict__ out,
                 uint32_t *__restrict__ err, unsigned long long *__restrict__ cells_total)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x;
    uint2 *cell2 = reinterpret_cast<uint2 *>(smem_raw) + lane;
    uint32_t *qw = reinterpret_cast<uint32_t *>(reinterpret_cast<uint2 *>(smem_raw) + (size_t)win_pairs(wc) * TB) + lane;
    uint32_t start = 0, stop = njobs;
    if (bounds) {
        // device-written bounds, clamped to the launch's job count
        stop = min(bounds[1], njobs);
        start = min(bounds[0], stop);
    }
    const uint32_t count = stop - start;
    if (wc <= 0 || count < slide_min) return;  // the group kernel runs this bucket
    const bool sym = P.sc.o_del + P.sc.e_del == P.sc.o_ins + P.sc.e_ins;
    unsigned long long ncells = 0;
    for (;;) {
        uint32_t b0 = 0;
        if (lane == 0) b0 = atomicAdd(counter, 32u);
        b0 = __shfl_sync(FULL, b0, 0);
        if (b0 >= count) break;
        const uint32_t pos = start + b0 + (uint32_t)lane;
        if (pos < stop) {
            const uint32_t jid = order ? order[pos] : pos;
            if (jid < njobs) {  // the group kernel flags an index past the jobs
                const bwacuda_dev_ext_job J = jobs[jid];
                if (J.qlen >= 0 && J.tlen >= 0 && J.qlen >= min_qlen &&
                    ext_fits_i16(J.qlen, J.tlen, J.h0, P.sc.max_sc)) {
                    const int w = clamp_band(J.w < 0 ? 0 : J.w, J.qlen, P.sc.max_sc, P.end_bonus, P.sc.o_ins,
                                             P.sc.e_ins, P.sc.o_del, P.sc.e_del);
                    if (xl::slide_takes(J.qlen, w, wc, count, slide_min)) {
                        bool bad = false;
                        const bwacuda_ext_result r = sym ? slide_job<true>(cell2, qw, wc, seq, J, w, P, bad, ncells)
                                                         : slide_job<false>(cell2, qw, wc, seq, J, w, P, bad, ncells);
                        if (bad) atomicOr(err, ERR_BASE);
                        out[jid] = r;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ncells += __shfl_xor_sync(FULL, ncells, o);
    if (lane == 0 && ncells) atomicAdd(cells_total, ncells);
}

}  // namespace slide

int ext_slide_window_for_band(int w)
{
    const long long need = 2LL * (w < 0 ? 0 : w) + 5 + xl::SLIDE_K;
    return (int)((need + 7) & ~7LL);
}

cudaError_t ext_slide_launch(const ExtLongLaunch &X, int nsm)
{
    using namespace slide;
    const int wc = X.slide_wc;
    const size_t smem = job_bytes(wc) * TB;
    if (wc <= 0 || wc % 8 != 0 || smem > EXT_SMEM_BLOCK_MAX) return cudaErrorInvalidValue;
    auto kern = ext_slide_kernel;
    // process-wide per kernel: always the ceiling (see the persistent kernels)
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)EXT_SMEM_BLOCK_MAX);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TB, smem)) != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidValue;
    if (X.reserve_regs > 0 || X.reserve_threads > 0) {
        cudaFuncAttributes fa;
        if ((e = cudaFuncGetAttributes(&fa, kern)) != cudaSuccess) return e;
        const int regs_block = ((fa.numRegs * 32 + 255) / 256) * 256;
        const int cap_r = regs_block > 0 ? (X.sm_regs - X.reserve_regs) / regs_block : per_sm;
        const int cap_t = (X.sm_threads - X.reserve_threads) / TB;
        per_sm = std::max(1, std::min(per_sm, std::min(cap_r, cap_t)));
    }
    kern<<<per_sm * nsm, TB, smem, X.stream>>>(X.seq, X.jobs, X.order, X.bounds, X.slide_counter, X.njobs,
                                              X.min_qlen, wc, X.slide_min, X.P, X.out, X.err, X.cells);
    return cudaGetLastError();
}

}  // namespace bwacuda
