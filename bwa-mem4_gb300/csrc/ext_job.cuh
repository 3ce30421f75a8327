// ext_job.cuh -- one banded seed extension (ksw_extend2) run by one thread,
// shared by the plain launch (extend_tpj.cu) and the persistent bucketed
// launch (ext_persist.cu).
//
// Semantics: crates/bwa-extend/src/sw.rs:203-493 integer for integer, with the
// qlen == 0 convention of crates/bwa-neon/src/batched.rs:1025-1039.
//
// The thread's persistent DP row lives in shared memory: column j (H(i-1, j-1)
// and E(i, j), j = 0..qlen) at cell[j * TB], so any mix of columns across a
// warp hits distinct banks.  Cells outside the live window [beg, end) are never
// written and keep the stale values of earlier rows exactly as the scalar code
// does (sw.rs:465-482 can grow `end` by two and read them back).  Query codes
// are four per shared word at qw[(j / 4) * TB].
#pragma once
#include "common.cuh"

namespace bwacuda {

// H (low 16 bits) and E (high 16 bits): exact whenever every DP value < 32768.
struct FmtI16 {
    using T = uint32_t;
    using Key = int32_t;
    static constexpr int bytes = 4;
    __device__ static __forceinline__ T pack(int h, int e) { return __byte_perm((uint32_t)h, (uint32_t)e, 0x5410); }
    __device__ static __forceinline__ int h(T c) { return (int)(c & 0xffffu); }
    __device__ static __forceinline__ int e(T c) { return (int)(c >> 16); }
    __device__ static __forceinline__ bool dead(T c) { return c == 0u; }
    // row max with ties going to the later column: max of (h << 16 | j)
    __device__ static __forceinline__ Key key(int h, int j) { return (h << 16) | j; }
    __device__ static __forceinline__ int key_h(Key k) { return k >> 16; }
    __device__ static __forceinline__ int key_j(Key k) { return k & 0xffff; }
};

// Two int32: the reference's scalar bin (values >= 32768).
struct FmtI32 {
    using T = int2;
    using Key = long long;
    static constexpr int bytes = 8;
    __device__ static __forceinline__ T pack(int h, int e) { return make_int2(h, e); }
    __device__ static __forceinline__ int h(T c) { return c.x; }
    __device__ static __forceinline__ int e(T c) { return c.y; }
    __device__ static __forceinline__ bool dead(T c) { return c.x == 0 && c.y == 0; }
    __device__ static __forceinline__ Key key(int h, int j) { return ((long long)h << 32) | (unsigned)j; }
    __device__ static __forceinline__ int key_h(Key k) { return (int)(k >> 32); }
    __device__ static __forceinline__ int key_j(Key k) { return (int)(k & 0xffffffffLL); }
};

// Upper bound of every H, E, F value of a job: a path gains at most max_sc per
// diagonal step and gaps never add (opens and extends are validated >= 0).
__host__ __device__ inline long long ext_value_bound(int qlen, int tlen, int h0, int max_sc)
{
    long long mn = qlen < tlen ? qlen : tlen;
    return (long long)h0 + mn * (max_sc > 0 ? max_sc : 0);
}

__host__ __device__ inline bool ext_fits_i16(int qlen, int tlen, int h0, int max_sc)
{
    return ext_value_bound(qlen, tlen, h0, max_sc) < 32768 && qlen < 65535;
}

// The pair kernels (8- and 16-bit pair cells) subtract gap costs in signed 16-bit
// lanes; costs up to 16384 keep every lane difference inside the lane.  Larger
// costs send every narrow job to the one-column-per-cell 16-bit kernel.
__host__ __device__ inline bool ext_pair_lanes_ok(int o_del, int e_del, int o_ins, int e_ins)
{
    return (long long)o_del + e_del <= 16384 && (long long)o_ins + e_ins <= 16384;
}

// Target bases of a job read as aligned 32-bit words, the next word loaded a word
// ahead (four to seven rows of prefetch for the row loop).  A word is read only
// when it holds at least one byte of the target, so it lies in mapped memory.
struct TargetStream {
    const uint32_t *w;
    uint32_t cur, nxt;
    int b, end;  // byte index of the current row from w, and one past the last
    __device__ __forceinline__ void init(const uint8_t *t, int tlen)
    {
        const uintptr_t a = reinterpret_cast<uintptr_t>(t);
        w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
        b = (int)(a & 3);
        end = b + tlen;
        cur = tlen > 0 ? w[0] : 0u;
        nxt = end > 4 ? w[1] : 0u;
    }
    __device__ __forceinline__ uint32_t next()
    {
        const uint32_t c = (cur >> ((b & 3) * 8)) & 0xffu;
        ++b;
        if ((b & 3) == 0) {
            cur = nxt;
            const int k = (b >> 2) + 1;
            if (k * 4 < end) nxt = w[k];
        }
        return c;
    }
};

// Runs job J; returns the ExtendResult, adds the inner-loop iterations to ncells.
template <class F, int TB>
__device__ __forceinline__ bwacuda_ext_result ext_run_job(typename F::T *__restrict__ cell,
                                                          uint32_t *__restrict__ qw,
                                                          const uint8_t *__restrict__ seq,
                                                          const bwacuda_dev_ext_job &J, const ExtParams &P,
                                                          bool &bad, unsigned long long &ncells)
{
    using CellT = typename F::T;
    const int qlen = J.qlen, tlen = J.tlen, h0 = J.h0, m = P.sc.m;
    const uint8_t *q = seq + J.q_off;
    const uint8_t *t = seq + J.t_off;
    const int o_del = P.sc.o_del, e_del = P.sc.e_del, o_ins = P.sc.o_ins, e_ins = P.sc.e_ins;
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;

    // Query codes, four per shared word (one word past the end stays readable).
    for (int jw = 0; jw * 4 <= qlen; ++jw) {
        uint32_t v = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = jw * 4 + u;
            uint32_t c = j < qlen ? (uint32_t)q[j] : 0u;
            bad |= c >= (uint32_t)m;
            v |= (c & 7u) << (8 * u);
        }
        qw[jw * TB] = v;
    }
    // Row -1 (sw.rs:269-279): h0, then the insertion chain while > e_ins; E = 0.
    {
        int hv = h0;
        cell[0] = F::pack(h0, 0);
        if (qlen >= 1) {
            hv = h0 > oe_ins ? h0 - oe_ins : 0;
            cell[TB] = F::pack(hv, 0);
        }
        for (int j = 2; j <= qlen; ++j) {
            hv = hv > e_ins ? hv - e_ins : 0;
            cell[(size_t)j * TB] = F::pack(hv, 0);
        }
    }
    const int w = clamp_band(J.w < 0 ? 0 : J.w, qlen, P.sc.max_sc, P.end_bonus, o_ins, e_ins, o_del, e_del);
    int best = h0, best_i = -1, best_j = -1, best_ie = -1, gscore = -1, max_off = 0;
    int beg = 0, end = qlen;
    TargetStream ts;
    ts.init(t, tlen);
    for (int i = 0; i < tlen; ++i) {
        uint32_t tc = ts.next();
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
        typename F::Key rowkey = 0;
        if (beg < end) {
            // Software pipelined: the cell and query word for column j+1 are loaded
            // while column j computes.  cell[end] (end <= qlen) and the query word
            // holding column end are always allocated, so the look-ahead is in bounds.
            int j = beg;
            CellT cn = cell[(size_t)j * TB];
            uint32_t qn = qw[(j >> 2) * TB] >> ((j & 3) * 8);
            for (; j < end; ++j) {
                const CellT c = cn;
                cn = cell[(size_t)(j + 1) * TB];
                const uint32_t qc = qn & 0xffu;
                qn = ((j & 3) == 3) ? qw[((j >> 2) + 1) * TB] : (qn >> 8);
                const int hd = F::h(c);
                const int e = F::e(c);
                const int s = prof_score(plo, phi, qc);
                const int M = hd != 0 ? hd + s : 0;  // a zero diagonal is never extended
                int h = M > e ? M : e;
                h = h > f ? h : f;
                int od = M - oe_del;
                od = od > 0 ? od : 0;
                int en = e - e_del;
                en = en > od ? en : od;
                cell[(size_t)j * TB] = F::pack(h1, en);  // H(i, j-1) for the next row, E(i+1, j)
                h1 = h;
                const typename F::Key kk = F::key(h, j);  // ties -> later column
                rowkey = rowkey > kk ? rowkey : kk;
                int oi = M - oe_ins;
                oi = oi > 0 ? oi : 0;
                f -= e_ins;
                f = f > oi ? f : oi;
            }
            ncells += (unsigned long long)(end - beg);
        }
        cell[(size_t)end * TB] = F::pack(h1, 0);  // sentinel column (sw.rs:418-419)
        const int jf = end > beg ? end : beg;
        if (jf == qlen && gscore <= h1) {  // later row wins ties (sw.rs:424-427)
            best_ie = i;
            gscore = h1;
        }
        const int rmax = F::key_h(rowkey);
        const int mj = F::key_j(rowkey);
        if (rmax == 0) break;
        if (rmax > best) {
            best = rmax;
            best_i = i;
            best_j = mj;
            const int off = mj > i ? mj - i : i - mj;
            if (off > max_off) max_off = off;
        } else if (P.zdrop > 0) {  // sw.rs:440-456
            if (i - best_i > mj - best_j) {
                if (best - rmax - ((i - best_i) - (mj - best_j)) * e_del > P.zdrop) break;
            } else if (best - rmax - ((mj - best_j) - (i - best_i)) * e_ins > P.zdrop) {
                break;
            }
        }
        // adaptive band (sw.rs:465-482)
        int lo = beg;
        while (lo < end && F::dead(cell[(size_t)lo * TB])) ++lo;
        beg = lo;
        int hi = end;
        while (hi >= beg && F::dead(cell[(size_t)hi * TB])) --hi;
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

// Shared-memory bytes of a block: TB threads, qcap cell columns each, plus the
// query words (one spare word for the look-ahead).
__host__ __device__ inline size_t ext_block_smem(int qcap, int tb, int cell_bytes)
{
    size_t qwords = (size_t)qcap / 4 + 1;
    return (size_t)qcap * tb * cell_bytes + qwords * tb * 4;
}

// ---------------------------------------------------------------------------
// 8-bit pair cells: word k of a thread holds columns 2k and 2k+1 as the bytes
// (H_2k, E_2k, H_2k+1, E_2k+1).  Exact whenever every DP value < 256, i.e. for
// the jobs the reference routes to its 8-bit kernels
// (crates/bwa-neon/src/batched.rs:850-864).  Half the row footprint of FmtI16,
// so twice the jobs per SM; each word access serves two columns.
// ---------------------------------------------------------------------------

__host__ __device__ inline bool ext_fits_u8(int qlen, int tlen, int h0, int max_sc)
{
    return ext_value_bound(qlen, tlen, h0, max_sc) < 256;
}

// Cell words of a block for the pair format (one spare word for the look-ahead).
__host__ __device__ inline size_t ext_block_smem_u8p(int qcap, int tb)
{
    size_t cwords = (size_t)qcap / 2 + 2;
    size_t qwords = (size_t)qcap / 4 + 1;
    return (cwords + qwords) * tb * 4;
}

// One extension cell (sw.rs:363-414): in hd = H(i-1, j-1), e = E(i, j) and the
// carried f = F(i, j); out h = H(i, j), en = E(i+1, j), f = F(i, j+1).
__device__ __forceinline__ void ext_cell(int hd, int e, uint32_t qc, uint32_t plo, uint32_t phi, int oe_del,
                                         int e_del, int oe_ins, int e_ins, int &f, int &h, int &en)
{
    const int s = prof_score(plo, phi, qc);
    const int M = hd != 0 ? hd + s : 0;  // a zero diagonal is never extended
    h = M > e ? M : e;
    h = h > f ? h : f;
    int od = M - oe_del;
    od = od > 0 ? od : 0;
    en = e - e_del;
    en = en > od ? en : od;
    int oi = M - oe_ins;
    oi = oi > 0 ? oi : 0;
    f -= e_ins;
    f = f > oi ? f : oi;
}

// F through one column pair in 16x2 lanes.  In: fv's high half = F(i, j), ti2 =
// (max(M_j - oe_ins, 0), max(M_j+1 - oe_ins, 0)); fsel2 = (-32768, -e_ins) and
// ne_ins2 = (-e_ins, -e_ins).  Returns (F(i, j), F(i, j+1)) and leaves F(i, j+2) in
// fv's high half.  The low lane of the first step is max(fv.lo - 32768, F(i, j)) =
// F(i, j) because fv's low half always lies in [0, 32768).
__device__ __forceinline__ uint32_t f_pair(uint32_t &fv, uint32_t ti2, uint32_t fsel2, uint32_t ne_ins2)
{
    const uint32_t d2 = prmt(fv, ti2, 0x5432u);           // (F(i,j), ti_j)
    const uint32_t f2 = __viaddmax_s16x2(fv, fsel2, d2);  // (F(i,j), max(F(i,j) - e_ins, ti_j))
    fv = __viaddmax_s16x2(f2, ne_ins2, ti2);              // high: max(F(i,j+1) - e_ins, ti_j+1)
    return f2;
}

// Row-maximum key over a column pair (H(i,jj), H(i,jj+1)) in h2: max of
// (H << 16) | column, so ties go to the later column.  H < 32768 keeps keys positive.
__device__ __forceinline__ int32_t pair_rowkey(int32_t rowkey, uint32_t h2, int jj)
{
    const int32_t ka = (int32_t)prmt((uint32_t)jj, h2, 0x5410u);  // (H_jj << 16) | jj
    const int32_t kb = (int32_t)((h2 & 0xffff0000u) | (uint32_t)(jj + 1));
    return __vimax3_s32(rowkey, ka, kb);
}

template <int TB>
__device__ __forceinline__ bool u8p_dead(const uint32_t *cellw, int x)
{
    return ((cellw[(x >> 1) * TB] >> ((x & 1) * 16)) & 0xffffu) == 0u;
}

// Row-maximum keys of the 8-bit pair kernel.  K16 (rows of at most 512 columns):
// two 16-bit lanes, lane 0 over even columns 2k and lane 1 over odd columns 2k+1,
// each the max of (H << 8) | k (H < 256, k < 256), so a lane keeps its latest
// column among equal H; the lanes are merged once per row.  Otherwise the 32-bit
// key (H << 16) | column.
template <bool K16>
struct U8Keys {
    uint32_t v = 0;
    __device__ __forceinline__ void one(int h, int j)
    {
        if (K16) {
            const uint32_t k = (((uint32_t)h << 8) | (uint32_t)(j >> 1)) << ((j & 1) * 16);
            v = __vimax3_u16x2(v, k, k);
        } else {
            const int32_t kk = (h << 16) | j;
            v = (uint32_t)((int32_t)v > kk ? (int32_t)v : kk);
        }
    }
    __device__ __forceinline__ void pair(uint32_t h2, int jj)
    {
        if (K16) {
            const uint32_t k = prmt((uint32_t)(jj >> 1), h2, 0x6040u);  // ((H_jj << 8) | k, (H_jj+1 << 8) | k)
            v = __vimax3_u16x2(v, k, k);
        } else {
            v = (uint32_t)pair_rowkey((int32_t)v, h2, jj);
        }
    }
    // quad with its key bytes given (kk = bytes k, k + 1 with k = jj / 2)
    __device__ __forceinline__ void quad_kk(uint32_t h2a, uint32_t h2b, uint32_t kk, int jj)
    {
        if (K16) {
            v = __vimax3_u16x2(v, prmt(kk, h2a, 0x6040u), prmt(kk, h2b, 0x6141u));
        } else {
            v = (uint32_t)pair_rowkey((int32_t)v, h2a, jj);
            v = (uint32_t)pair_rowkey((int32_t)v, h2b, jj + 2);
        }
    }
    // two consecutive pairs at columns jj..jj+3 (jj even)
    __device__ __forceinline__ void quad(uint32_t h2a, uint32_t h2b, int jj)
    {
        if (K16) {
            const uint32_t kk = (uint32_t)(jj >> 1) * 0x0101u + 0x0100u;  // bytes k, k + 1
            v = __vimax3_u16x2(v, prmt(kk, h2a, 0x6040u), prmt(kk, h2b, 0x6141u));
        } else {
            v = (uint32_t)pair_rowkey((int32_t)v, h2a, jj);
            v = (uint32_t)pair_rowkey((int32_t)v, h2b, jj + 2);
        }
    }
    __device__ __forceinline__ void decode(int &rmax, int &mj) const
    {
        if (K16) {
            const int hlo = (int)((v >> 8) & 0xffu), hhi = (int)(v >> 24);
            const int jlo = 2 * (int)(v & 0xffu), jhi = 2 * (int)((v >> 16) & 0xffu) + 1;
            const bool hi = hhi > hlo || (hhi == hlo && jhi > jlo);  // ties -> later column
            rmax = hi ? hhi : hlo;
            mj = hi ? jhi : jlo;
        } else {
            rmax = (int)v >> 16;
            mj = (int)(v & 0xffffu);
        }
    }
};

// SYM: o_del + e_del == o_ins + e_ins, so the deletion-open lane equals the
// insertion-open lane and is not computed twice.
template <int TB, bool K16, bool SYM>
__device__ __forceinline__ bwacuda_ext_result ext_run_job_u8p(uint32_t *__restrict__ cellw, uint32_t *__restrict__ qw,
                                                              const uint8_t *__restrict__ seq,
                                                              const bwacuda_dev_ext_job &J, const ExtParams &P,
                                                              bool &bad, unsigned long long &ncells)
{
    const int qlen = J.qlen, tlen = J.tlen, h0 = J.h0, m = P.sc.m;
    const uint8_t *q = seq + J.q_off;
    const uint8_t *t = seq + J.t_off;
    const int o_del = P.sc.o_del, e_del = P.sc.e_del, o_ins = P.sc.o_ins, e_ins = P.sc.e_ins;
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;

    // Query codes as prmt selector bytes 0x80 | c * 0x11 (nibbles c, c|8): two
    // consecutive bytes select two sign-extended 16-bit scores in one prmt.
    for (int jw = 0; jw * 4 <= qlen; ++jw) {
        uint32_t v = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = jw * 4 + u;
            uint32_t c = j < qlen ? (uint32_t)q[j] : 0u;
            bad |= c >= (uint32_t)m;
            v |= (0x80u | (c & 7u) * 0x11u) << (8 * u);
        }
        qw[jw * TB] = v;
    }
    // Row -1 (sw.rs:269-279): H(-1, j-1) = h0, h0 - oe_ins, then - e_ins while > e_ins; E = 0.
    {
        int hv = h0;
        for (int k = 0; 2 * k <= qlen; ++k) {
            const int a = hv;  // column 2k
            if (2 * k == 0) hv = h0 > oe_ins ? h0 - oe_ins : 0;
            else hv = hv > e_ins ? hv - e_ins : 0;
            const int b = 2 * k + 1 <= qlen ? hv : 0;  // column 2k+1
            if (2 * k + 1 <= qlen) hv = hv > e_ins ? hv - e_ins : 0;
            cellw[k * TB] = (uint32_t)a | ((uint32_t)b << 16);
        }
    }
    const int w = clamp_band(J.w < 0 ? 0 : J.w, qlen, P.sc.max_sc, P.end_bonus, o_ins, e_ins, o_del, e_del);
    int best = h0, best_i = -1, best_j = -1, best_ie = -1, gscore = -1, max_off = 0;
    int beg = 0, end = qlen;
    TargetStream ts;
    ts.init(t, tlen);
    // 16x2 broadcasts of the negated gap costs
    const uint32_t noe_ins2 = (uint32_t)(-oe_ins & 0xffff) * 0x10001u;
    const uint32_t noe_del2 = (uint32_t)(-oe_del & 0xffff) * 0x10001u;
    const uint32_t ne_del2 = (uint32_t)(-e_del & 0xffff) * 0x10001u;
    const uint32_t ne_ins2 = (uint32_t)(-e_ins & 0xffff) * 0x10001u;
    const uint32_t fsel2 = 0x8000u | ((uint32_t)(-e_ins & 0xffff) << 16);
    for (int i = 0; i < tlen; ++i) {
        uint32_t tc = ts.next();
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
        U8Keys<K16> rowkey;
        if (beg < end) {
            int j = beg;
            if (j & 1) {  // odd first column: the high half of its word
                uint32_t wv = cellw[(j >> 1) * TB];
                const uint32_t qc = (qw[(j >> 2) * TB] >> ((j & 3) * 8)) & 7u;
                int h, en;
                ext_cell((int)((wv >> 16) & 0xffu), (int)(wv >> 24), qc, plo, phi, oe_del, e_del, oe_ins, e_ins, f, h,
                         en);
                cellw[(j >> 1) * TB] = (wv & 0xffffu) | ((uint32_t)h1 << 16) | ((uint32_t)en << 24);
                h1 = h;
                rowkey.one(h, j);
                ++j;
            }
            uint32_t wn = cellw[(j >> 1) * TB];  // j <= end <= qlen: allocated
            // columns j, j+1 of one word as 16x2 lanes.  F runs through the lanes too:
            // fv holds F(i, j) in its high half, h1v holds H(i, j-1) in its high half.
            uint32_t fv = (uint32_t)f << 16, h1v = (uint32_t)h1 << 16;
            // cw: the cell word of the current pair (running pointer: constant offsets, no
            // per-pair index arithmetic)
            uint32_t *cw = cellw + (j >> 1) * TB;
            auto pair_at = [&](int off, uint32_t sel) {
                const uint32_t wv = wn;
                wn = cw[off + TB];  // spare word keeps this in bounds
                const uint32_t s2 = prmt(plo, phi, sel);   // (s_j, s_j+1)
                const uint32_t hd2 = prmt(wv, 0u, 0x4240u);  // (H(i-1,j-1), H(i-1,j))
                const uint32_t e2 = prmt(wv, 0u, 0x4341u);   // (E(i,j), E(i,j+1))
                // M = hd ? hd + s : 0, as min(hd + s, 128 hd): hd <= 255 and s >= -128, so
                // the minimum is hd + s whenever hd >= 1 and <= 0 when hd == 0, and a
                // non-positive M acts as 0 below (E, F >= 0)
                const uint32_t M2 = __viaddmin_s16x2(hd2, s2, hd2 << 7);
                const uint32_t ti2 = __viaddmax_s16x2_relu(M2, noe_ins2, 0u);  // max(M - oe_ins, 0)
                const uint32_t td2 = SYM ? ti2 : __viaddmax_s16x2_relu(M2, noe_del2, 0u);  // max(M - oe_del, 0)
                const uint32_t en2 = __viaddmax_s16x2(e2, ne_del2, td2);       // E(i+1, .)
                const uint32_t f2 = f_pair(fv, ti2, fsel2, ne_ins2);            // (F(i,j), F(i,j+1))
                const uint32_t h2 = __vimax3_s16x2(M2, e2, f2);  // (H(i,j), H(i,j+1))
                // stored bytes: H(i,j-1), E(i+1,j), H(i,j), E(i+1,j+1)
                cw[off] = prmt(prmt(h1v, h2, 0x0042u), en2, 0x6140u);
                h1v = h2;
                return h2;
            };
            // one pair to reach a query-word boundary, then whole words (four columns) with
            // the next word loaded one step ahead, then a last pair
            if ((j & 2) && j + 1 < end) {
                rowkey.pair(pair_at(0, qw[(j >> 2) * TB] >> 16), j);
                j += 2;
                cw += TB;
            }
            if (j + 3 < end) {
                const uint32_t *qp = qw + (j >> 2) * TB;
                uint32_t qn = qp[0];
                uint32_t kk = (uint32_t)(j >> 1) * 0x0101u + 0x0100u;  // key column bytes of the quad
                for (; j + 3 < end; j += 4) {
                    const uint32_t qv = qn;
                    qp += TB;
                    qn = qp[0];  // j + 4 <= qlen < qcap: inside the query words
                    const uint32_t h2a = pair_at(0, qv);
                    const uint32_t h2b = pair_at(TB, qv >> 16);
                    cw += 2 * TB;
                    rowkey.quad_kk(h2a, h2b, kk, j);
                    kk += 0x0202u;
                }
            }
            if (j + 1 < end) {
                rowkey.pair(pair_at(0, qw[(j >> 2) * TB] >> ((j & 2) * 8)), j);
                j += 2;
            }
            f = (int)(fv >> 16);
            h1 = (int)(h1v >> 16);
            if (j < end) {  // even last column: the low half of its word
                const uint32_t wv = wn;
                const uint32_t qc = (qw[(j >> 2) * TB] >> ((j & 3) * 8)) & 7u;
                int h, en;
                ext_cell((int)(wv & 0xffu), (int)((wv >> 8) & 0xffu), qc, plo, phi, oe_del, e_del, oe_ins, e_ins, f,
                         h, en);
                cellw[(j >> 1) * TB] = (wv & 0xffff0000u) | (uint32_t)h1 | ((uint32_t)en << 8);
                h1 = h;
                rowkey.one(h, j);
            }
            ncells += (unsigned long long)(end - beg);
        }
        {   // sentinel column end (sw.rs:418-419): H = h1, E = 0
            const uint32_t wv = cellw[(end >> 1) * TB];
            cellw[(end >> 1) * TB] =
                (end & 1) ? ((wv & 0xffffu) | ((uint32_t)h1 << 16)) : ((wv & 0xffff0000u) | (uint32_t)h1);
        }
        const int jf = end > beg ? end : beg;
        if (jf == qlen && gscore <= h1) {
            best_ie = i;
            gscore = h1;
        }
        int rmax, mj;
        rowkey.decode(rmax, mj);
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
        while (lo < end && u8p_dead<TB>(cellw, lo)) ++lo;
        beg = lo;
        int hi = end;
        while (hi >= beg && u8p_dead<TB>(cellw, hi)) --hi;
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

// ---------------------------------------------------------------------------
// 16-bit pair cells: pair word k of a thread (8 bytes) holds columns 2k and
// 2k+1 as .x = (H_2k, H_2k+1) and .y = (E_2k, E_2k+1), 16 bits each.  Exact
// whenever every DP value < 32768 (the reference's 16-bit bin).  The same
// footprint per column as FmtI16, but every lane operation serves two columns
// and H and E arrive already split into lanes.
// ---------------------------------------------------------------------------

// Shared-memory bytes of a block for 16-bit pair cells (one spare pair word for
// the look-ahead, one for the sentinel) plus the query words.
__host__ __device__ inline size_t ext_block_smem_i16p(int qcap, int tb)
{
    size_t cpairs = (size_t)qcap / 2 + 2;
    size_t qwords = (size_t)qcap / 4 + 1;
    return (cpairs * 8 + qwords * 4) * tb;
}

template <int TB>
__device__ __forceinline__ bool i16p_dead(const uint2 *cell2, int x)
{
    const uint2 c = cell2[(x >> 1) * TB];
    return (((c.x | c.y) >> ((x & 1) * 16)) & 0xffffu) == 0u;
}

template <int TB, bool SYM>
__device__ __forceinline__ bwacuda_ext_result ext_run_job_i16p(uint2 *__restrict__ cell2, uint32_t *__restrict__ qw,
                                                               const uint8_t *__restrict__ seq,
                                                               const bwacuda_dev_ext_job &J, const ExtParams &P,
                                                               bool &bad, unsigned long long &ncells)
{
    const int qlen = J.qlen, tlen = J.tlen, h0 = J.h0, m = P.sc.m;
    const uint8_t *q = seq + J.q_off;
    const uint8_t *t = seq + J.t_off;
    const int o_del = P.sc.o_del, e_del = P.sc.e_del, o_ins = P.sc.o_ins, e_ins = P.sc.e_ins;
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;

    // Query codes as prmt selector bytes, as in the 8-bit pair form.
    for (int jw = 0; jw * 4 <= qlen; ++jw) {
        uint32_t v = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = jw * 4 + u;
            uint32_t c = j < qlen ? (uint32_t)q[j] : 0u;
            bad |= c >= (uint32_t)m;
            v |= (0x80u | (c & 7u) * 0x11u) << (8 * u);
        }
        qw[jw * TB] = v;
    }
    // Row -1 (sw.rs:269-279), E = 0.
    {
        int hv = h0;
        for (int k = 0; 2 * k <= qlen; ++k) {
            const int a = hv;  // column 2k
            if (2 * k == 0) hv = h0 > oe_ins ? h0 - oe_ins : 0;
            else hv = hv > e_ins ? hv - e_ins : 0;
            const int b = 2 * k + 1 <= qlen ? hv : 0;  // column 2k+1
            if (2 * k + 1 <= qlen) hv = hv > e_ins ? hv - e_ins : 0;
            cell2[k * TB] = make_uint2((uint32_t)a | ((uint32_t)b << 16), 0u);
        }
    }
    const int w = clamp_band(J.w < 0 ? 0 : J.w, qlen, P.sc.max_sc, P.end_bonus, o_ins, e_ins, o_del, e_del);
    int best = h0, best_i = -1, best_j = -1, best_ie = -1, gscore = -1, max_off = 0;
    int beg = 0, end = qlen;
    uint32_t tnext = tlen > 0 ? t[0] : 0u;
    const uint32_t noe_ins2 = (uint32_t)(-oe_ins & 0xffff) * 0x10001u;
    const uint32_t noe_del2 = (uint32_t)(-oe_del & 0xffff) * 0x10001u;
    const uint32_t ne_del2 = (uint32_t)(-e_del & 0xffff) * 0x10001u;
    const uint32_t ne_ins2 = (uint32_t)(-e_ins & 0xffff) * 0x10001u;
    const uint32_t fsel2 = 0x8000u | ((uint32_t)(-e_ins & 0xffff) << 16);
    for (int i = 0; i < tlen; ++i) {
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
            int j = beg;
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
            uint2 wn = cell2[(j >> 1) * TB];  // j <= end <= qlen: allocated
            uint32_t fv = (uint32_t)f << 16, h1v = (uint32_t)h1 << 16;
            // cw: the pair word of the current pair (running pointer, as in the 8-bit form)
            uint2 *cw = cell2 + (j >> 1) * TB;
            auto pair_at = [&](int off, uint32_t sel, int jj) {
                const uint2 wv = wn;
                wn = cw[off + TB];  // spare pair keeps this in bounds
                const uint32_t s2 = prmt(plo, phi, sel);  // (s_j, s_j+1)
                const uint32_t hd2 = wv.x, e2 = wv.y;
                // M = hd ? hd + s : 0, as min(hd + s, 32767 * min(hd, 1)): every path score
                // is < 32768 here, and a non-positive M acts as 0 below (E, F >= 0)
                const uint32_t g2 = __viaddmin_u16x2(hd2, 0u, 0x00010001u) * 0x7fffu;
                const uint32_t M2 = __viaddmin_s16x2(hd2, s2, g2);
                const uint32_t ti2 = __viaddmax_s16x2_relu(M2, noe_ins2, 0u);
                const uint32_t td2 = SYM ? ti2 : __viaddmax_s16x2_relu(M2, noe_del2, 0u);
                const uint32_t en2 = __viaddmax_s16x2(e2, ne_del2, td2);
                const uint32_t f2 = f_pair(fv, ti2, fsel2, ne_ins2);
                const uint32_t h2 = __vimax3_s16x2(M2, e2, f2);
                // stored: H(i,j-1), H(i,j) and E(i+1,j), E(i+1,j+1)
                cw[off] = make_uint2(prmt(h1v, h2, 0x5432u), en2);
                h1v = h2;
                rowkey = pair_rowkey(rowkey, h2, jj);
            };
            if ((j & 2) && j + 1 < end) {
                pair_at(0, qw[(j >> 2) * TB] >> 16, j);
                j += 2;
                cw += TB;
            }
            if (j + 3 < end) {
                const uint32_t *qp = qw + (j >> 2) * TB;
                uint32_t qn = qp[0];
                for (; j + 3 < end; j += 4) {
                    const uint32_t qv = qn;
                    qp += TB;
                    qn = qp[0];  // j + 4 <= qlen < qcap: inside the query words
                    pair_at(0, qv, j);
                    pair_at(TB, qv >> 16, j + 2);
                    cw += 2 * TB;
                }
            }
            if (j + 1 < end) {
                pair_at(0, qw[(j >> 2) * TB] >> ((j & 2) * 8), j);
                j += 2;
            }
            f = (int)(fv >> 16);
            h1 = (int)(h1v >> 16);
            if (j < end) {  // even last column: the low lanes of its pair
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
        }
        {   // sentinel column end (sw.rs:418-419): H = h1, E = 0
            const uint2 wv = cell2[(end >> 1) * TB];
            cell2[(end >> 1) * TB] = (end & 1) ? make_uint2((wv.x & 0xffffu) | ((uint32_t)h1 << 16), wv.y & 0xffffu)
                                               : make_uint2((wv.x & 0xffff0000u) | (uint32_t)h1, wv.y & 0xffff0000u);
        }
        const int jf = end > beg ? end : beg;
        if (jf == qlen && gscore <= h1) {
            best_ie = i;
            gscore = h1;
        }
        const int rmax = rowkey >> 16;
        const int mj = rowkey & 0xffff;
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
        while (lo < end && i16p_dead<TB>(cell2, lo)) ++lo;
        beg = lo;
        int hi = end;
        while (hi >= beg && i16p_dead<TB>(cell2, hi)) --hi;
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

}  // namespace bwacuda
