// ext_long.cuh -- banded seed extension (ksw_extend2, crates/bwa-extend/src/sw.rs:203-493)
// for queries of any length: one group of L lanes per job (L = 8, 16 or 32), each DP row
// processed in parallel across the group, the row's state in a shared-memory ring.
//
// Parallel form.  Row i's window [beg, end) is cut into chunks of L*C columns; lane k owns
// columns cb + k*C .. cb + k*C + C-1 of a chunk.  Every cell except the horizontal gap F
// depends on the previous row only, so a lane computes M, the vertical gap E and the gap
// opens of its C columns from the ring, then F comes from one max-scan over the group:
//   F(j) = max(F(cb), max_{cb <= k' < j} G(k')) - (j - cb) * e_ins,
//   G(k') = max(M(k') - oe_ins, 0) + (k' - cb + 1) * e_ins,
// which unrolls the reference's f = max(f - e_ins, max(M - oe_ins, 0)) (f = 0 at beg).
// The row maximum (later column on ties), the first and last live cells (the adaptive band,
// sw.rs:465-482) are group reductions; the per-row bookkeeping (z-drop, gscore, band) runs
// redundantly in every lane of the group.
//
// Row storage.  The reference keeps qlen + 1 cells per job and reads stale cells left by
// earlier rows (the band end grows by up to two columns per row).  Every cell a row touches
// lies in [beg, end] with i - w <= beg and end <= i + w + 1 (w the clamped band), and beg
// never decreases, so a ring of R >= 2w + 3 columns (slot = column mod R) returns for every
// read the value the full row would hold: a column c that is still needed and a column
// c +- R can never both lie in one row's window, so neither overwrites the other.  The ring
// starts with row -1 (sw.rs:269-279) for columns 0 .. R-1; after a row whose sentinel column
// is the largest column written so far, the next column (the only never-written column the
// next row can read) is set to its row -1 value, overwriting a column left of the band.  A
// job with qlen + 1 <= R indexes the ring directly.  Memory per job is O(band), not O(query).
//
// Jobs whose band needs a larger ring than the launch's are appended to a deferred list and
// run by a second launch with the largest ring (RING_MAX_*); beyond that the call fails with
// BWACUDA_EUNSUPPORTED (bands over 16382 columns on 16-bit jobs of more than 32767 query
// bases, or over 8190 on 32-bit jobs of more than 16383).
#pragma once
#include <cuda_runtime.h>

#include <climits>

#include "common.cuh"
#include "ext_job.cuh"

namespace bwacuda {
namespace xl {

constexpr unsigned FULL = 0xffffffffu;
constexpr int RING_MAX_16 = 32768;  // 16-bit cells: H | E << 16, 4 bytes a column
constexpr int RING_MAX_32 = 16384;  // 32-bit cells: H and E arrays, 8 bytes a column

// Shared-memory words of one ring (bank-skewed: one spare word per 32 slots).
__host__ __device__ inline int ring_words(int R, bool w32) { return (R + R / 32) * (w32 ? 2 : 1); }

// Slot s at word s + s / 32: the C consecutive columns of consecutive lanes fall in
// different banks.
__device__ __forceinline__ int ring_phys(int slot) { return slot + (slot >> 5); }

template <bool W32>
struct Ring;

template <>
struct Ring<false> {
    uint32_t *c;
    int mask;
    __device__ __forceinline__ void init(uint32_t *base, int R) { c = base; mask = R - 1; }
    __device__ __forceinline__ void get(int col, int &h, int &e) const
    {
        const uint32_t v = c[ring_phys(col & mask)];
        h = (int)(v & 0xffffu);
        e = (int)(v >> 16);
    }
    __device__ __forceinline__ void put(int col, int h, int e) const
    {
        c[ring_phys(col & mask)] = (uint32_t)h | ((uint32_t)e << 16);
    }
};

template <>
struct Ring<true> {
    int *H, *E;
    int mask;
    __device__ __forceinline__ void init(uint32_t *base, int R)
    {
        H = reinterpret_cast<int *>(base);
        E = H + (R + R / 32);
        mask = R - 1;
    }
    __device__ __forceinline__ void get(int col, int &h, int &e) const
    {
        const int p = ring_phys(col & mask);
        h = H[p];
        e = E[p];
    }
    __device__ __forceinline__ void put(int col, int h, int e) const
    {
        const int p = ring_phys(col & mask);
        H[p] = h;
        E[p] = e;
    }
};

// H of row -1 at column col (sw.rs:269-279): h0, then h0 - oe_ins, decreasing by e_ins
// until it would reach 0, then 0.
__device__ __forceinline__ int row_minus1(int col, int h0, int oe_ins, int e_ins)
{
    if (col == 0) return h0;
    const long long v = (long long)h0 - oe_ins - (long long)(col - 1) * e_ins;
    return v > 0 ? (int)v : 0;
}

// Whether a ring of R columns holds a job of qlen columns at clamped band w.
__host__ __device__ inline bool ring_fits(int qlen, int w, int R)
{
    return (long long)qlen + 1 <= R || 2LL * w + 3 <= R;
}

// The thread-per-job window kernel (ext_slide.cu): a job's row lives in a window of wc
// columns that moves right SLIDE_K columns at a time.  A row touches at most columns
// [i - w - 1, i + w + 4], and the window starts at most SLIDE_K - 1 columns left of i - w - 1,
// so it holds every band of 2w + 5 + SLIDE_K <= wc columns, and every query of qlen + 4 <= wc
// columns without moving.
constexpr int SLIDE_K = 64;

__host__ __device__ inline bool slide_fits(int qlen, int w, int wc)
{
    return (long long)qlen + 4 <= wc || 2LL * w + 5 + SLIDE_K <= wc;
}

// Whether the window kernel takes a 16-bit job of a bucket of `count` jobs: it is enabled for
// the launch (wc > 0), the bucket holds at least slide_min jobs and the job's band fits.  The
// group-per-job kernel leaves exactly these jobs to it.
__host__ __device__ inline bool slide_takes(int qlen, int w, int wc, uint32_t count, uint32_t slide_min)
{
    return wc > 0 && count >= slide_min && slide_fits(qlen, w, wc);
}

template <int L>
__device__ __forceinline__ int group_max(int v)
{
    if constexpr (L == 32) {
        return __reduce_max_sync(FULL, v);
    } else {
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(FULL, v, o, L));
        return v;
    }
}

template <int L>
__device__ __forceinline__ int group_min(int v)
{
    if constexpr (L == 32) {
        return __reduce_min_sync(FULL, v);
    } else {
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(FULL, v, o, L));
        return v;
    }
}

// Jobs come from order[bounds[0] .. bounds[1]) (order nullptr: the identity; bounds nullptr:
// [0, njobs)), taken G = 32 / L at a time per warp from *counter.  A job is this launch's if
// its cell class is W32's, qlen >= min_qlen and the window kernel does not take it
// (slide_takes with slide_wc, slide_min); one whose band needs a larger ring than ring_cols
// goes to defer[] (count in *defer_count), or fails the call when defer is nullptr.
template <bool W32, int L, int C>
__global__ void __launch_bounds__(128)
ext_long_kernel(const uint8_t *__restrict__ seq, const bwacuda_dev_ext_job *__restrict__ jobs,
                const uint32_t *__restrict__ order, const uint32_t *__restrict__ bounds,
                uint32_t *__restrict__ counter, uint32_t njobs, int min_qlen, int ring_cols,
                uint32_t *__restrict__ defer, uint32_t *__restrict__ defer_count, int slide_wc,
                uint32_t slide_min, const __grid_constant__ ExtParams P, bwacuda_ext_result *__restrict__ out,
                uint32_t *__restrict__ err, unsigned long long *__restrict__ cells_total)
{
    constexpr int G = 32 / L;  // jobs per warp
    constexpr int W = L * C;   // columns per chunk
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, k = lane % L, grp = lane / L;
    const int gid = (threadIdx.x >> 5) * G + grp;
    Ring<W32> ring;
    ring.init(reinterpret_cast<uint32_t *>(smem_raw) + (size_t)gid * ring_words(ring_cols, W32), ring_cols);
    uint32_t start = 0, stop = njobs;
    if (bounds) {
        // device-written bounds, clamped to the launch's job count
        stop = min(bounds[1], njobs);
        start = min(bounds[0], stop);
    }
    const int m = P.sc.m;
    const int o_del = P.sc.o_del, e_del = P.sc.e_del, o_ins = P.sc.o_ins, e_ins = P.sc.e_ins;
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;
    unsigned long long ncells = 0;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(counter, (uint32_t)G);
        base = __shfl_sync(FULL, base, 0);
        if (base >= stop - start) break;
        const uint32_t pos = start + base + (uint32_t)grp;
        bool active = pos < stop;
        uint32_t jid = 0;
        bwacuda_dev_ext_job J;
        J.q_off = 0; J.t_off = 0; J.qlen = 0; J.tlen = 0; J.h0 = 1; J.w = 0;
        if (active) {
            jid = order ? order[pos] : pos;
            if (jid >= njobs) {
                if (k == 0) atomicOr(err, ERR_RANGE);
                active = false;
            } else {
                J = jobs[jid];
            }
        }
        if (active && (J.qlen < 0 || J.tlen < 0)) {
            if (k == 0) atomicOr(err, ERR_RANGE);
            active = false;
        }
        if (active && (J.qlen < min_qlen || ext_fits_i16(J.qlen, J.tlen, J.h0, P.sc.max_sc) == W32))
            active = false;  // another launch's job
        // value bound: with gap extends capped at it (exact, see below) every F term stays in int
        long long vb = active ? ext_value_bound(J.qlen, J.tlen, J.h0, P.sc.max_sc) : 1;
        if (vb < 1) vb = 1;
        if (active && vb * (W + 1) >= (1LL << 31)) {
            if (k == 0) atomicOr(err, ERR_RANGE);
            active = false;
        }
        int w = 0;
        if (active) {
            w = clamp_band(J.w < 0 ? 0 : J.w, J.qlen, P.sc.max_sc, P.end_bonus, o_ins, e_ins, o_del, e_del);
            if (!W32 && slide_takes(J.qlen, w, slide_wc, stop - start, slide_min)) active = false;
        }
        if (active) {
            if (!ring_fits(J.qlen, w, ring_cols)) {
                if (k == 0) {
                    if (defer) {
                        const uint32_t d = atomicAdd(defer_count, 1u);
                        if (d < njobs) defer[d] = jid;
                        else atomicOr(err, ERR_RANGE);
                    } else {
                        atomicOr(err, ERR_RANGE);
                    }
                }
                active = false;
            }
        }
        const int qlen = active ? J.qlen : 0, tlen = active ? J.tlen : 0, h0 = J.h0;
        const uint8_t *q = seq + J.q_off;
        const uint8_t *t = seq + J.t_off;
        bool bad = false;
        if (active) {
            // every query code is checked, as the thread-per-job kernels check the staged query
            for (int j = k; j < qlen; j += L) bad |= q[j] >= (uint32_t)m;
            const int lim = qlen < ring_cols - 1 ? qlen : ring_cols - 1;
            for (int j = k; j <= lim; j += L) ring.put(j, row_minus1(j, h0, oe_ins, e_ins), 0);
        }
        __syncwarp();
        // Extends capped at the value bound: a term that extends a gap by one or more columns
        // at cost >= vb is <= 0 <= F with either cost, so F is unchanged.
        const int ec = (int)((long long)e_ins < vb ? (long long)e_ins : vb);
        int beg = 0, end = qlen, best = h0, best_i = -1, best_j = -1, best_ie = -1, gscore = -1, max_off = 0;
        int maxw = -1;
        bool done = !active;
        for (int i = 0;; ++i) {
            if (i >= tlen) done = true;
            if (__all_sync(FULL, done)) break;
            const bool run = !done;
            uint32_t tc = 0;
            if (run) {
                tc = t[i];
                bad |= tc >= (uint32_t)m;
            }
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
            const int ncol = run && beg < end ? end - beg : 0;
            const int nch = (ncol + W - 1) / W;
            const int nch_w = __reduce_max_sync(FULL, nch);
            int fcarry = 0, hcarry = h1;
            int kh = -1, kj = -1;                   // the lane's row maximum, later column on ties
            int first_live = INT_MAX, last_live = -1;
            int hlast_lane = h1;                    // H(i, end - 1) in the lane that holds it
            for (int ch = 0; ch < nch_w; ++ch) {
                const int c0 = beg + ch * W + k * C;
                int Mv[C], Ev[C], Gv[C], Hv[C], ENv[C];
                int gl = INT_MIN / 2;
#pragma unroll
                for (int u = 0; u < C; ++u) {
                    const int col = c0 + u;
                    const bool v = ch < nch && col < end;
                    int hd = 0, e = 0;
                    uint32_t qc = 0;
                    if (v) {
                        ring.get(col, hd, e);
                        qc = q[col];
                    }
                    const int s = prof_score(plo, phi, qc & 7u);
                    const int M = hd != 0 ? hd + s : 0;  // a zero diagonal is never extended
                    int oi = M - oe_ins;
                    oi = oi > 0 ? oi : 0;
                    int od = M - oe_del;
                    od = od > 0 ? od : 0;
                    int en = e - e_del;
                    ENv[u] = en > od ? en : od;         // E(i+1, col)
                    Mv[u] = M;
                    Ev[u] = e;
                    Gv[u] = oi + (k * C + u + 1) * ec;
                    gl = gl > Gv[u] ? gl : Gv[u];
                }
                // exclusive max-scan of the lanes' G maxima
                int sc = gl;
#pragma unroll
                for (int o = 1; o < L; o <<= 1) {
                    const int x = __shfl_up_sync(FULL, sc, o, L);
                    if (k >= o) sc = sc > x ? sc : x;
                }
                int ex = __shfl_up_sync(FULL, sc, 1, L);
                if (k == 0) ex = INT_MIN / 2;
                const int tot = __shfl_sync(FULL, sc, L - 1, L);
                int runf = fcarry > ex ? fcarry : ex;
#pragma unroll
                for (int u = 0; u < C; ++u) {
                    const int F = runf - (k * C + u) * ec;  // F(i, col)
                    runf = runf > Gv[u] ? runf : Gv[u];
                    int h = Mv[u] > Ev[u] ? Mv[u] : Ev[u];
                    Hv[u] = h > F ? h : F;
                }
                int hp = __shfl_up_sync(FULL, Hv[C - 1], 1, L);
                if (k == 0) hp = hcarry;
#pragma unroll
                for (int u = 0; u < C; ++u) {
                    const int col = c0 + u;
                    if (ch < nch && col < end) {
                        const int sh = u == 0 ? hp : Hv[u - 1];  // stored: H(i, col - 1), E(i+1, col)
                        ring.put(col, sh, ENv[u]);
                        if (sh != 0 || ENv[u] != 0) {
                            first_live = first_live < col ? first_live : col;
                            last_live = col;
                        }
                        if (Hv[u] >= kh) {
                            kh = Hv[u];
                            kj = col;
                        }
                        if (col == end - 1) hlast_lane = Hv[u];
                    }
                }
                fcarry = (fcarry > tot ? fcarry : tot) - W * ec;  // F at the next chunk's first column
                hcarry = __shfl_sync(FULL, Hv[C - 1], L - 1, L);
            }
            int hlast = h1;
            if (nch_w > 0) {
                const int owner = ncol > 0 ? (end - 1 - (beg + (nch - 1) * W)) / C : 0;
                const int hv = __shfl_sync(FULL, hlast_lane, owner, L);
                if (ncol > 0) hlast = hv;
            }
            const int rmax_raw = group_max<L>(kh);
            const int mj = group_max<L>(kh == rmax_raw ? kj : -1);
            const int lo = group_min<L>(first_live);
            const int hi_live = group_max<L>(last_live);
            if (run) {
                if (k == 0) {
                    ring.put(end, hlast, 0);  // sentinel column (sw.rs:418-419)
                    ncells += (unsigned long long)ncol;
                }
                const int jf = end > beg ? end : beg;
                if (jf == qlen && gscore <= hlast) {  // later row wins ties (sw.rs:424-427)
                    best_ie = i;
                    gscore = hlast;
                }
                const int rmax = rmax_raw > 0 ? rmax_raw : 0;
                if (rmax == 0) {
                    done = true;
                } else {
                    if (rmax > best) {
                        best = rmax;
                        best_i = i;
                        best_j = mj;
                        const int off = mj > i ? mj - i : i - mj;
                        if (off > max_off) max_off = off;
                    } else if (P.zdrop > 0) {  // sw.rs:440-456
                        if (i - best_i > mj - best_j) {
                            if (best - rmax - ((i - best_i) - (mj - best_j)) * e_del > P.zdrop) done = true;
                        } else if (best - rmax - ((mj - best_j) - (i - best_i)) * e_ins > P.zdrop) {
                            done = true;
                        }
                    }
                    if (!done) {  // adaptive band (sw.rs:465-482)
                        const int e_row = end;
                        beg = lo != INT_MAX ? lo : end;
                        const int hi = hlast != 0 ? end : (hi_live >= beg ? hi_live : beg - 1);
                        end = hi + 2 < qlen ? hi + 2 : qlen;
                        if (e_row > maxw) maxw = e_row;
                        if (e_row == maxw && e_row + 1 <= qlen && k == 0)
                            ring.put(e_row + 1, row_minus1(e_row + 1, h0, oe_ins, e_ins), 0);
                    }
                }
            }
            __syncwarp();
        }
        const bool gbad = group_max<L>(bad ? 1 : 0) != 0;
        if (active) {
            if (k == 0) {
                if (gbad) atomicOr(err, ERR_BASE);
                bwacuda_ext_result r;
                r.score = best;
                r.qle = best_j + 1;
                r.tle = best_i + 1;
                r.gtle = best_ie + 1;
                r.gscore = gscore;
                r.max_off = max_off;
                out[jid] = r;
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ncells += __shfl_xor_sync(FULL, ncells, o);
    if (lane == 0 && ncells) atomicAdd(cells_total, ncells);
}

}  // namespace xl
}  // namespace bwacuda
