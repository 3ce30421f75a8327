// global.cu -- banded global alignment with traceback (ksw_global2,
// crates/bwa-extend/src/sw.rs:561-740), batched on the GPU.
//
// One thread per alignment.  The DP row pair (H and E of the previous row)
// lives in shared memory, interleaved across the block (slot x of thread t at
// x * TB + t), with the query codes beside it.  Only the band is kept: row i
// reads and writes columns [i - w, i + w + 1] and every column it reads was
// written by the previous row (or by the row -1 initialisation), so the row is
// a circular buffer of B = min(2w + 2, qlen + 1) slots, column j in slot j % B.
// The traceback byte of every band cell (f << 4 | e << 2 | h, the reference's
// encoding) goes to HBM, each alignment's matrix contiguous with rows padded to
// 16 bytes and written 16 cells per store.  The traceback then walks only its
// path's cells and writes the CIGAR runs (len << 4 | op), merged and reversed
// as the reference does.
//
// On the device route the alignments are radix-sorted by (query-length bucket,
// query length, target length) and each bucket is launched with the shared
// memory its own longest query and widest band need, so warps hold alignments
// of one read length and short reads are not held to the long reads' footprint.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "kernels.h"
#include "runtime.h"

namespace bwacuda {

namespace {

constexpr int MINUS_INF = -0x40000000;
constexpr size_t SMEM_LIMIT = 227u * 1024u;

// One alignment as the kernel sees it (bases addressed from the chunk's base buffer).
struct GlobalDevJob {
    uint64_t q_off, t_off;
    uint64_t z_off;    // byte offset of this job's traceback matrix (tlen rows of zrow bytes)
    uint64_t cig_off;  // word offset of this job's CIGAR scratch (qlen + tlen + 1 words)
    int32_t qlen, tlen, w;
    int32_t zrow;      // traceback bytes per row: the band width rounded up to 16
};
static_assert(sizeof(GlobalDevJob) == 48, "descriptor layout");

// Shared memory of a block: bcap band slots of {H, E} (two int32, or two int16 for
// narrow jobs) and qcap + 1 query codes per thread (one spare for the look-ahead).
__host__ __device__ inline size_t global_smem(int bcap, int qcap, int tb, bool narrow = false)
{
    return (size_t)tb * ((size_t)bcap * (narrow ? 4 : 8) + (size_t)qcap + 1);
}

// 16-bit cells.  Every value of ksw_global2's DP is either reachable (a path score)
// or derived from the MINUS_INF sentinel by adding scores and gap costs.  Path
// scores of a job lie in [-D, D] and sentinel-derived values in MINUS_INF + [-D, D],
// with D = (qlen + tlen) * max(o + e of either gap, -min score, max score) +
// o_del + o_ins + o_del + e_del + o_ins + e_ins.  When D <= GLB_NARROW_D the int16
// cells hold path scores as they are and sentinel-derived values as
// GLB_NEG16 + (v - MINUS_INF): every sum, maximum and comparison of the recurrence
// gives the same result in both forms (the two ranges stay apart and inside int16),
// so traceback bytes and scores are identical.
constexpr int GLB_NEG16 = -24576;
// what a DP kernel leaves in ncig[k] for the traceback kernel: the direction-byte layout
constexpr int GLB_TB_ROWS = -1;   // a row's bytes from column beg (32-bit cell kernel)
constexpr int GLB_TB_PAIRS = -2;  // from column beg & ~1 (pair kernel)
constexpr int GLB_TB_AHEAD = 4;     // traceback cells loaded together down the diagonal
constexpr int GLB_SIDE_STREAMS = 2;  // streams beside the context's for the bucket DP launches
constexpr int GLB_NARROW_D = 8000;
struct GlbNarrowRule {
    int cost;  // max(o_del + e_del, o_ins + e_ins, -min score, max score)
    int base;  // o_del + o_ins + o_del + e_del + o_ins + e_ins
};
__host__ __device__ inline bool global_narrow(int qlen, int tlen, const GlbNarrowRule &r)
{
    // two steps of margin: the pair kernel also forms F and E one column / row past the matrix
    return (long long)(qlen + (long long)tlen + 2) * r.cost + r.base <= GLB_NARROW_D;
}

// Traceback bytes per row: the band's columns plus one (the pair kernel keeps a row's
// bytes at column - (beg & ~1), so column pairs sit at even offsets), rounded up to 16.
__host__ __device__ inline int global_zrow(int qlen, int w)
{
    if (w < 0) w = 0;
    const long long nc = qlen < 2LL * w + 1 ? qlen : 2LL * w + 1;
    return (int)((nc + 1 + 15) & ~15LL);
}

// Query-length buckets of the device route (upper bounds, inclusive).
constexpr int GLB_NBUCKETS = 8;
__host__ __device__ inline int global_bucket(int qlen)
{
    return qlen <= 64 ? 0 : qlen <= 128 ? 1 : qlen <= 192 ? 2 : qlen <= 256 ? 3 : qlen <= 320 ? 4 : qlen <= 448 ? 5
           : qlen <= 640 ? 6 : 7;
}

// Band slots a job needs.
__host__ __device__ inline int global_band_slots(int qlen, int w)
{
    if (w < 0) w = 0;
    const long long b = 2LL * w + 2;
    return (int)(b < (long long)qlen + 1 ? b : (long long)qlen + 1);
}

__device__ __forceinline__ void cigar_push(uint32_t *cig, int &n, uint32_t op, uint32_t len)
{
    if (n > 0 && (cig[n - 1] & 0xfu) == op) {
        cig[n - 1] += len << 4;
        return;
    }
    cig[n++] = (len << 4) | op;
}

// The reference's traceback (sw.rs:700-738) from the band's last cell of the last row over a
// job's direction bytes; the CIGAR runs, reversed, into cg.  Returns the run count, or -1
// where the reference's flat index leaves the matrix (its panic).  PAIR: the pair kernel's
// row layout, a row's bytes starting at column beg & ~1.
template <bool PAIR>
__device__ int global_traceback(const uint8_t *zj, size_t zrow, int n_col, int qlen, int tlen, int w, uint32_t *cg)
{
    int nc = 0;
    long i = (long)tlen - 1;
    long kk = ((long)tlen - 1 + w + 1 < qlen ? (long)tlen - 1 + w + 1 : (long)qlen) - 1;
    uint32_t which = 0;
    const long total = (long)n_col * tlen;
    while (i >= 0 && kk >= 0) {
        // In state M the walk usually stays on the diagonal: the next GLB_TB_AHEAD cells down it
        // are loaded together (independent loads, their latencies overlap), then consumed while
        // every step is diagonal; a step off the diagonal, or state E / F, loads afresh.
        const int ahead = which == 0 ? GLB_TB_AHEAD : 1;
        uint32_t dv[GLB_TB_AHEAD];
        bool okv[GLB_TB_AHEAD];
#pragma unroll
        for (int t = 0; t < GLB_TB_AHEAD; ++t) {
            const long ii = i - t, kt = kk - t;
            dv[t] = 0;
            okv[t] = false;
            if (t < ahead && ii >= 0 && kt >= 0) {
                const long beg = ii > w ? ii - w : 0;
                // the reference reads the flat row-major matrix: an offset past the row lands in a
                // later row; one before the band or past the matrix is its panic
                const long flat = ii * (long)n_col + (kt - beg);
                if (kt >= beg && flat < total) {
                    long row = ii, col = kt - beg;
                    if (col >= n_col) {
                        row = flat / n_col;
                        col = flat - row * n_col;
                    }
                    const long shift = PAIR ? ((row > w ? row - w : 0) & 1) : 0;
                    dv[t] = zj[(size_t)row * zrow + (size_t)(col + shift)];
                    okv[t] = true;
                }
            }
        }
#pragma unroll
        for (int t = 0; t < GLB_TB_AHEAD; ++t) {
            // (i, kk) is cell t down the diagonal from where the loads started
            if (t >= ahead || i < 0 || kk < 0) break;
            if (!okv[t]) return -1;
            which = (dv[t] >> (which << 1)) & 3u;
            if (which == 0) {
                cigar_push(cg, nc, 0, 1);
                --i;
                --kk;
                continue;
            }
            if (which == 1) { cigar_push(cg, nc, 2, 1); --i; }
            else { cigar_push(cg, nc, 1, 1); --kk; }
            break;
        }
    }
    if (i >= 0) cigar_push(cg, nc, 2, (uint32_t)(i + 1));
    if (kk >= 0) cigar_push(cg, nc, 1, (uint32_t)(kk + 1));
    for (int a = 0, b = nc - 1; a < b; ++a, --b) {
        const uint32_t x = cg[a];
        cg[a] = cg[b];
        cg[b] = x;
    }
    return nc;
}

template <bool NARROW>
struct GlbCell {
    using T = int2;
    static constexpr int NEG = MINUS_INF;
    __device__ static __forceinline__ T pack(int h, int e) { return make_int2(h, e); }
    __device__ static __forceinline__ int h(T c) { return c.x; }
    __device__ static __forceinline__ int e(T c) { return c.y; }
    __device__ static __forceinline__ int score32(int v) { return v; }
};
template <>
struct GlbCell<true> {
    using T = uint32_t;
    static constexpr int NEG = GLB_NEG16;
    __device__ static __forceinline__ T pack(int h, int e) { return ((uint32_t)h & 0xffffu) | ((uint32_t)e << 16); }
    __device__ static __forceinline__ int h(T c) { return (int)(int16_t)(c & 0xffffu); }
    __device__ static __forceinline__ int e(T c) { return (int)c >> 16; }
    // sentinel-derived values sit below -16384, path scores above
    __device__ static __forceinline__ int score32(int v) { return v < -16384 ? MINUS_INF + (v - GLB_NEG16) : v; }
};

template <int TB, bool NARROW>
__global__ void __launch_bounds__(TB)
global_tpj_kernel(const uint8_t *__restrict__ seq, const GlobalDevJob *__restrict__ jobs,
                  const uint32_t *__restrict__ order, uint32_t base, uint32_t count,
                  const __grid_constant__ Scoring sc, int bcap, int qcap, uint8_t *__restrict__ z,
                  uint32_t *__restrict__ cig, int32_t *__restrict__ score_out, int32_t *__restrict__ ncig_out,
                  uint32_t *__restrict__ err, unsigned long long *__restrict__ cells_total)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    const uint32_t t = blockIdx.x * TB + tid;
    unsigned long long ncells = 0;
    if (t >= count) return;
    const uint32_t k = order ? order[base + t] : base + t;
    using C = GlbCell<NARROW>;
    using CellT = typename C::T;
    constexpr int NEG = C::NEG;  // MINUS_INF in this cell form
    CellT *cell = reinterpret_cast<CellT *>(smem_raw) + tid;       // cell[x * TB]: {H, E} of band slot x
    uint8_t *qs = smem_raw + (size_t)bcap * sizeof(CellT) * TB + tid;  // qs[j * TB]: query code
    const GlobalDevJob J = jobs[k];
    const int qlen = J.qlen, tlen = J.tlen;
    const int w = J.w < 0 ? 0 : J.w;
    const int n_col = qlen < 2 * w + 1 ? qlen : 2 * w + 1;
    const int B = global_band_slots(qlen, w);
    const int oe_del = sc.o_del + sc.e_del, oe_ins = sc.o_ins + sc.e_ins;
    const uint8_t *q = seq + J.q_off;
    const uint8_t *tg = seq + J.t_off;
    uint8_t *zj = z + J.z_off;
    const size_t zrow = (size_t)J.zrow;
    bool bad = false;
    if (B > bcap || qlen > qcap) {  // the host sizes bcap / qcap from the launch's jobs
        atomicOr(err, ERR_RANGE);
        ncig_out[k] = 0;
        return;
    }
    for (int j = 0; j < qlen; ++j) {
        uint32_t c = q[j];
        bad |= c >= (uint32_t)sc.m;
        qs[(size_t)j * TB] = (uint8_t)(c < (uint32_t)sc.m ? c : PAD_CODE);
    }
    // row -1: the origin, a leading insertion over columns 1..w, unreachable beyond
    // (slots 0..B-1 hold columns 0..B-1, which covers every column row 0 reads)
    for (int j = 0; j < B; ++j) {
        int h = NEG;
        if (j == 0) h = 0;
        else if (j <= w) h = -(sc.o_ins + sc.e_ins * j);
        cell[(size_t)j * TB] = C::pack(h, NEG);
    }
    for (int i = 0; i < tlen; ++i) {
        int f = NEG;
        const int beg = i > w ? i - w : 0;
        const int end = i + w + 1 < qlen ? i + w + 1 : qlen;
        int h1 = beg == 0 ? -(sc.o_del + sc.e_del * (i + 1)) : NEG;
        uint32_t tc = tg[i];
        bad |= tc >= (uint32_t)sc.m;
        tc = tc < (uint32_t)sc.m ? tc : (uint32_t)PAD_CODE;
        const uint32_t plo = sc.prof[tc & 7u][0], phi = sc.prof[tc & 7u][1];
        uint4 *zr = reinterpret_cast<uint4 *>(zj + (size_t)i * zrow);
        // direction bytes: four columns gather in acc, four words make a 16-column store
        uint32_t acc = 0, zw0 = 0, zw1 = 0, zw2 = 0, zw3 = 0;
        int x = beg % (B > 0 ? B : 1);  // slot of column j
        // Software pipelined: column j+1's slot and query code load while column j computes.
        // A row's columns occupy distinct slots (end - beg < B), so the look-ahead reads the
        // previous row's value of that slot, as the in-order read would.
        CellT cn = cell[(size_t)x * TB];
        uint32_t qn = qs[(size_t)beg * TB];  // beg <= qlen: inside the qcap + 1 codes
        for (int j = beg; j < end; ++j) {
            CellT *cp = cell + (size_t)x * TB;
            const CellT he = cn;
            const uint32_t qc = qn;
            if (++x == B) x = 0;
            cn = cell[(size_t)x * TB];
            qn = qs[(size_t)(j + 1) * TB];  // j + 1 <= qlen
            int mm = C::h(he), e = C::e(he);
            mm += prof_score(plo, phi, qc);
            uint32_t d = mm < e ? 1u : 0u;
            int h = mm >= e ? mm : e;
            if (!(h >= f)) { d = 2u; h = f; }
            int tt = mm - oe_del;
            e -= sc.e_del;
            if (e > tt) d |= 1u << 2;
            else e = tt;
            *cp = C::pack(h1, e);  // H(i, j-1) for the next row's diagonal; E(i+1, j)
            h1 = h;
            tt = mm - oe_ins;
            f -= sc.e_ins;
            if (f > tt) d |= 2u << 4;
            else f = tt;
            const int jj = j - beg;
            acc |= d << (8 * (jj & 3));
            const bool last = j == end - 1;
            if ((jj & 3) == 3 || last) {
                const int g = (jj >> 2) & 3;
                zw0 = g == 0 ? acc : zw0;
                zw1 = g == 1 ? acc : zw1;
                zw2 = g == 2 ? acc : zw2;
                zw3 = g == 3 ? acc : zw3;
                acc = 0;
                if (g == 3 || last) {
                    zr[jj >> 4] = make_uint4(zw0, zw1, zw2, zw3);
                    zw0 = zw1 = zw2 = zw3 = 0;
                }
            }
        }
        if (B > 0) cell[(size_t)(end % B) * TB] = C::pack(h1, NEG);
        // band cells this row did not reach read as 0, as in the reference's zeroed matrix
        for (int ci = end > beg ? (end - beg + 15) >> 4 : 0; ci < (n_col + 15) >> 4; ++ci)
            zr[ci] = make_uint4(0u, 0u, 0u, 0u);
        ncells += (unsigned long long)(end > beg ? end - beg : 0);
    }
    // eh_h[qlen] after the last row: written by that row's epilogue when its band reaches the last
    // column, else still its row -1 value (the bands' ends never decrease)
    const int end_last = tlen > 0 ? (tlen + w < qlen ? tlen + w : qlen) : -1;
    int score;
    if (end_last == qlen) score = C::score32(C::h(cell[(size_t)(qlen % B) * TB]));
    else score = qlen == 0 ? 0 : (qlen <= w ? -(sc.o_ins + sc.e_ins * qlen) : MINUS_INF);
    score_out[k] = score;
    ncig_out[k] = GLB_TB_ROWS;  // glb_traceback_kernel follows (this layout)
    if (bad) atomicOr(err, ERR_BASE);
    atomicAdd(cells_total, ncells);
}

// Shared memory of a block for the pair kernel: the band slots as 8-byte pair words (bcap
// rounded up to even) and the query per column pair (one spare pair for the look-ahead) as a
// 16-bit prmt selector, or (q4) as two 4-bit codes.
__host__ __device__ inline size_t global_smem_pair(int bcap, int qcap, int tb, bool q4 = false)
{
    return (size_t)tb * ((size_t)((bcap + 1) / 2) * 8 + (size_t)((qcap + 2) / 2 + 1) * (q4 ? 1 : 2));
}

// A column pair's codes c0 | c1 << 4 as the prmt selector (0x80 | c0 * 0x11) | (0x80 | c1 * 0x11) << 8:
// c0 | c1 << 8 by one mask and one multiply-add, then * 0x11 + 0x8080 (c <= 7: no carries).
__device__ __forceinline__ uint32_t glb_q4_sel(uint32_t b)
{
    return (b + (b & 0xf0u) * 15u) * 0x11u + 0x8080u;
}

// One column of the recurrence in 32-bit registers (the head / tail columns of a row in the pair
// kernel), the scalar kernel's cell: in hd = H(i-1, j-1), e = E(i, j), f = F(i, j); out h, e =
// E(i+1, j), f = F(i, j+1) and the direction byte.
__device__ __forceinline__ uint32_t glb_cell(int hd, int &e, int &f, int s, int oe_del, int e_del, int oe_ins,
                                             int e_ins, int &h)
{
    const int mm = hd + s;
    uint32_t d = mm < e ? 1u : 0u;
    h = mm >= e ? mm : e;
    if (!(h >= f)) { d = 2u; h = f; }
    int tt = mm - oe_del;
    e -= e_del;
    if (e > tt) d |= 1u << 2;
    else e = tt;
    tt = mm - oe_ins;
    f -= e_ins;
    if (f > tt) d |= 2u << 4;
    else f = tt;
    return d;
}

// ksw_global2 on 16-bit pair cells (jobs that pass global_narrow): two columns per lane
// operation, direction bits from the DPX max-with-predicate instructions.  Slot x of the
// band (x = column mod B2, B2 the band slots rounded up to even) is lane x & 1 of pair word
// x / 2: .x = (H, H), .y = (E, E).  Sentinel-derived values are kept as in GlbCell<true>.
// All lane sums stay inside int16: values lie in [GLB_NEG16 - D, D] with D <= GLB_NARROW_D.
// Q4: the query as 4-bit code pairs (half the query's shared memory, more jobs resident, one
// ALU and two multiply-add instructions per column pair to rebuild the selector).
template <int TB, bool Q4>
__global__ void __launch_bounds__(TB)
global_pair_kernel(const uint8_t *__restrict__ seq, const GlobalDevJob *__restrict__ jobs,
                   const uint32_t *__restrict__ order, uint32_t base, uint32_t count,
                   const __grid_constant__ Scoring sc, int bcap, int qcap, uint8_t *__restrict__ z,
                   uint32_t *__restrict__ cig, int32_t *__restrict__ score_out, int32_t *__restrict__ ncig_out,
                   uint32_t *__restrict__ err, unsigned long long *__restrict__ cells_total)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using C = GlbCell<true>;
    constexpr int NEG = GLB_NEG16;
    const int tid = threadIdx.x;
    const uint32_t t = blockIdx.x * TB + tid;
    unsigned long long ncells = 0;
    if (t >= count) return;
    const uint32_t k = order ? order[base + t] : base + t;
    const int bpairs = (bcap + 1) / 2;
    uint2 *cell2 = reinterpret_cast<uint2 *>(smem_raw) + tid;                          // cell2[p * TB]
    // query word of column pair jp at [jp * TB]
    uint16_t *qs2 = reinterpret_cast<uint16_t *>(smem_raw + (size_t)bpairs * 8 * TB) + tid;
    uint8_t *qs1 = smem_raw + (size_t)bpairs * 8 * TB + tid;
    auto qsel = [&](int jp) -> uint32_t {
        return Q4 ? glb_q4_sel(qs1[(size_t)jp * TB]) : (uint32_t)qs2[(size_t)jp * TB];
    };
    const GlobalDevJob J = jobs[k];
    const int qlen = J.qlen, tlen = J.tlen;
    const int w = J.w < 0 ? 0 : J.w;
    const int n_col = qlen < 2 * w + 1 ? qlen : 2 * w + 1;
    const int B = global_band_slots(qlen, w);
    const int B2 = B + (B & 1), P2 = B2 / 2;
    const int oe_del = sc.o_del + sc.e_del, oe_ins = sc.o_ins + sc.e_ins;
    const uint8_t *q = seq + J.q_off;
    const uint8_t *tg = seq + J.t_off;
    uint8_t *zj = z + J.z_off;
    const size_t zrow = (size_t)J.zrow;
    bool bad = false;
    if (P2 > bpairs || qlen > qcap) {  // the host sizes bcap / qcap from the launch's jobs
        atomicOr(err, ERR_RANGE);
        ncig_out[k] = 0;
        return;
    }
    // query codes as prmt selector bytes 0x80 | c * 0x11 (two sign-extended 16-bit scores per
    // prmt), two columns per 16-bit word, or as two 4-bit codes per byte; columns >= qlen are
    // padding
    for (int jp = 0; 2 * jp <= qlen; ++jp) {
        uint32_t v = 0, v4 = 0;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int j = 2 * jp + u;
            uint32_t c = j < qlen ? (uint32_t)q[j] : (uint32_t)PAD_CODE;
            if (j < qlen) bad |= c >= (uint32_t)sc.m;
            c = c < (uint32_t)sc.m || j >= qlen ? c : (uint32_t)PAD_CODE;
            v |= (0x80u | (c & 7u) * 0x11u) << (8 * u);
            v4 |= (c & 7u) << (4 * u);
        }
        if (Q4) qs1[(size_t)jp * TB] = (uint8_t)v4;
        else qs2[(size_t)jp * TB] = (uint16_t)v;
    }
    // row -1 (as the scalar kernel): slot x holds column x
    for (int p = 0; p < P2; ++p) {
        uint32_t hx = 0;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int j = 2 * p + u;
            const int h = j == 0 ? 0 : (j <= w ? -(sc.o_ins + sc.e_ins * j) : NEG);
            hx |= ((uint32_t)h & 0xffffu) << (16 * u);
        }
        cell2[(size_t)p * TB] = make_uint2(hx, ((uint32_t)NEG & 0xffffu) * 0x10001u);
    }
    const uint32_t MIN2 = 0x80008000u;
    const uint32_t noe_ins2 = ((uint32_t)(-oe_ins) & 0xffffu) * 0x10001u;
    const uint32_t noe_del2 = ((uint32_t)(-oe_del) & 0xffffu) * 0x10001u;
    const uint32_t ne_ins2 = ((uint32_t)(-sc.e_ins) & 0xffffu) * 0x10001u;
    const uint32_t ne_del2 = ((uint32_t)(-sc.e_del) & 0xffffu) * 0x10001u;
    const int ngroups = (n_col + 1 + 15) >> 4;
    // slots of columns beg and end, advanced with the band (each moves by at most one a row)
    int xbeg = 0, xend = (w + 1 < qlen ? w + 1 : qlen) % B2, prev_end = w + 1 < qlen ? w + 1 : qlen;
    uint32_t tnext = tlen > 0 ? tg[0] : 0u;
    for (int i = 0; i < tlen; ++i) {
        const int beg = i > w ? i - w : 0;
        const int end = i + w + 1 < qlen ? i + w + 1 : qlen;
        if (i > w && ++xbeg == B2) xbeg = 0;
        if (end > prev_end && ++xend == B2) xend = 0;
        prev_end = end;
        int h1 = beg == 0 ? -(sc.o_del + sc.e_del * (i + 1)) : NEG;  // H(i, beg-1)
        int f = NEG;                                                   // F(i, beg)
        uint32_t tc = tnext;
        if (i + 1 < tlen) tnext = tg[i + 1];
        bad |= tc >= (uint32_t)sc.m;
        tc = tc < (uint32_t)sc.m ? tc : (uint32_t)PAD_CODE;
        const uint32_t plo = sc.prof[tc & 7u][0], phi = sc.prof[tc & 7u][1];
        // Direction bytes of the row at offset column - (beg & ~1): 4-byte words from word 0,
        // kept as a group of four (g0..g3, the newest in g3) and stored 16 bytes at a time.
        uint4 *zr = reinterpret_cast<uint4 *>(zj + (size_t)i * zrow);
        uint32_t g0 = 0, g1 = 0, g2 = 0, g3 = 0;
        int nw = 0;  // words emitted so far
        auto emit = [&](uint32_t word) {
            g0 = g1;
            g1 = g2;
            g2 = g3;
            g3 = word;
            if ((nw & 3) == 3) zr[nw >> 2] = make_uint4(g0, g1, g2, g3);
            ++nw;
        };
        uint32_t part = 0;  // the open word: its low half (or the odd first column's byte 1)
        bool open = false;
        int j = beg;
        int xj = xbeg;  // slot of column j
        if (j < end && (j & 1)) {  // odd first column (offset 1): the high lanes of its pair
            const int x = xj;
            uint2 cw = cell2[(size_t)(x >> 1) * TB];
            int e = (int)cw.y >> 16, h;
            const uint32_t sel = qsel(j >> 1) >> 8;
            const uint32_t d = glb_cell((int)cw.x >> 16, e, f, (int)prmt(plo, phi, (sel & 0xffu) * 0x101u | 0x8800u),
                                        oe_del, sc.e_del, oe_ins, sc.e_ins, h);
            cw.x = (cw.x & 0xffffu) | ((uint32_t)h1 << 16);
            cw.y = (cw.y & 0xffffu) | ((uint32_t)e << 16);
            cell2[(size_t)(x >> 1) * TB] = cw;
            h1 = h;
            part = d << 8;
            open = true;
            ++j;
            if (++xj == B2) xj = 0;
        }
        const int npairs = j < end ? (end - j) >> 1 : 0;
        if (npairs > 0) {
            // F(i, j) in fv's high lane, H(i, j-1) in h1v's high lane
            uint32_t fv = (uint32_t)f << 16, h1v = (uint32_t)h1 << 16;
            const int p0 = xj >> 1;
            // one column pair: cp its pair word (read, then overwritten), sel its selector;
            // returns the two direction bytes
            auto pair_dir = [&](uint2 *cp, uint32_t sel) -> uint32_t {
                const uint2 cw = *cp;
                const uint32_t s2 = prmt(plo, phi, sel);  // (s_j, s_j+1)
                const uint32_t M2 = __viaddmax_s16x2(cw.x, s2, MIN2);  // H(i-1, .-1) + s
                bool pm_hi, pm_lo, ph_hi, ph_lo, pf_hi, pf_lo, pe_hi, pe_lo;
                const uint32_t ME2 = __vibmax_s16x2(M2, cw.y, &pm_hi, &pm_lo);      // M >= E
                const uint32_t tti2 = __viaddmax_s16x2(M2, noe_ins2, MIN2);         // M - oe_ins
                // (F(i, j), F(i, j+1)): lane lo passes F(i, j) through, lane hi updates it
                const uint32_t X = prmt(fv, tti2, 0x5432u);                         // (F(i,j), tti_j)
                const uint32_t fvm = __viaddmax_s16x2(fv, ne_ins2, MIN2);           // hi: F(i,j) - e_ins
                const uint32_t A2 = prmt(MIN2, fvm, 0x7610u);                       // (MIN, F(i,j) - e_ins)
                const uint32_t F2 = __viaddmax_s16x2(X, 0u, A2);                     // max(X, A2)
                const uint32_t H2 = __vibmax_s16x2(ME2, F2, &ph_hi, &ph_lo);        // max(M, E) >= F
                const uint32_t F2m = __viaddmax_s16x2(F2, ne_ins2, MIN2);
                fv = __vibmax_s16x2(tti2, F2m, &pf_hi, &pf_lo);                     // open >= extend
                const uint32_t ttd2 = __viaddmax_s16x2(M2, noe_del2, MIN2);         // M - oe_del
                const uint32_t E2m = __viaddmax_s16x2(cw.y, ne_del2, MIN2);
                const uint32_t En2 = __vibmax_s16x2(ttd2, E2m, &pe_hi, &pe_lo);     // open >= extend
                *cp = make_uint2(prmt(h1v, H2, 0x5432u), En2);
                h1v = H2;
                const uint32_t dlo = (ph_lo ? (pm_lo ? 0u : 1u) : 2u) | (pe_lo ? 0u : 4u) | (pf_lo ? 0u : 32u);
                const uint32_t dhi = (ph_hi ? (pm_hi ? 0u : 1u) : 2u) | (pe_hi ? 0u : 4u) | (pf_hi ? 0u : 32u);
                return dlo | (dhi << 8);
            };
            // two consecutive column pairs (pair words pa, pb; selectors sa, sb) with the same
            // operations as pair_dir, ordered so both pairs' independent work comes first and
            // only F chains from a to b; returns the four direction bytes
            auto pair2_dir = [&](uint2 *pa, uint2 *pb, uint32_t sa, uint32_t sb) -> uint32_t {
                const uint2 ca = *pa, cb = *pb;
                const uint32_t M2a = __viaddmax_s16x2(ca.x, prmt(plo, phi, sa), MIN2);
                const uint32_t M2b = __viaddmax_s16x2(cb.x, prmt(plo, phi, sb), MIN2);
                const uint32_t tti2a = __viaddmax_s16x2(M2a, noe_ins2, MIN2);
                const uint32_t tti2b = __viaddmax_s16x2(M2b, noe_ins2, MIN2);
                const uint32_t ttd2a = __viaddmax_s16x2(M2a, noe_del2, MIN2);
                const uint32_t ttd2b = __viaddmax_s16x2(M2b, noe_del2, MIN2);
                const uint32_t E2ma = __viaddmax_s16x2(ca.y, ne_del2, MIN2);
                const uint32_t E2mb = __viaddmax_s16x2(cb.y, ne_del2, MIN2);
                uint32_t v = 0;
                uint32_t H2a;
                {
                    bool pm_hi, pm_lo, ph_hi, ph_lo, pf_hi, pf_lo, pe_hi, pe_lo;
                    const uint32_t ME2 = __vibmax_s16x2(M2a, ca.y, &pm_hi, &pm_lo);
                    const uint32_t En2 = __vibmax_s16x2(ttd2a, E2ma, &pe_hi, &pe_lo);
                    const uint32_t X = prmt(fv, tti2a, 0x5432u);
                    const uint32_t fvm = __viaddmax_s16x2(fv, ne_ins2, MIN2);
                    const uint32_t F2 = __viaddmax_s16x2(X, 0u, prmt(MIN2, fvm, 0x7610u));
                    H2a = __vibmax_s16x2(ME2, F2, &ph_hi, &ph_lo);
                    fv = __vibmax_s16x2(tti2a, __viaddmax_s16x2(F2, ne_ins2, MIN2), &pf_hi, &pf_lo);
                    *pa = make_uint2(prmt(h1v, H2a, 0x5432u), En2);
                    const uint32_t dlo = (ph_lo ? (pm_lo ? 0u : 1u) : 2u) | (pe_lo ? 0u : 4u) | (pf_lo ? 0u : 32u);
                    const uint32_t dhi = (ph_hi ? (pm_hi ? 0u : 1u) : 2u) | (pe_hi ? 0u : 4u) | (pf_hi ? 0u : 32u);
                    v = dlo | (dhi << 8);
                }
                {
                    bool pm_hi, pm_lo, ph_hi, ph_lo, pf_hi, pf_lo, pe_hi, pe_lo;
                    const uint32_t ME2 = __vibmax_s16x2(M2b, cb.y, &pm_hi, &pm_lo);
                    const uint32_t En2 = __vibmax_s16x2(ttd2b, E2mb, &pe_hi, &pe_lo);
                    const uint32_t X = prmt(fv, tti2b, 0x5432u);
                    const uint32_t fvm = __viaddmax_s16x2(fv, ne_ins2, MIN2);
                    const uint32_t F2 = __viaddmax_s16x2(X, 0u, prmt(MIN2, fvm, 0x7610u));
                    const uint32_t H2b = __vibmax_s16x2(ME2, F2, &ph_hi, &ph_lo);
                    fv = __vibmax_s16x2(tti2b, __viaddmax_s16x2(F2, ne_ins2, MIN2), &pf_hi, &pf_lo);
                    *pb = make_uint2(prmt(H2a, H2b, 0x5432u), En2);
                    h1v = H2b;
                    const uint32_t dlo = (ph_lo ? (pm_lo ? 0u : 1u) : 2u) | (pe_lo ? 0u : 4u) | (pf_lo ? 0u : 32u);
                    const uint32_t dhi = (ph_hi ? (pm_hi ? 0u : 1u) : 2u) | (pe_hi ? 0u : 4u) | (pf_hi ? 0u : 32u);
                    v |= (dlo | (dhi << 8)) << 16;
                }
                return v;
            };
            // the row's pairs k = 0 .. npairs-1 take slots p0 + k, wrapping once at P2 (kw pairs
            // before the wrap): straight runs of running pointers, no per-pair wrap test
            const int kw = P2 - p0 < npairs ? P2 - p0 : npairs;
            uint2 *cp = cell2 + (size_t)p0 * TB;
            int k = 0;
            const uint8_t *q1p = qs1 + (size_t)(j >> 1) * TB;
            const uint16_t *q2p = qs2 + (size_t)(j >> 1) * TB;
            auto next_sel = [&]() -> uint32_t {
                uint32_t s;
                if (Q4) {
                    s = glb_q4_sel(*q1p);
                    q1p += TB;
                } else {
                    s = *q2p;
                    q2p += TB;
                }
                return s;
            };
            auto advance = [&]() {
                cp += TB;
                if (++k == kw) cp = cell2;
            };
            if (open) {  // a pair at offset 2 closes word 0
                const uint32_t v = pair_dir(cp, next_sel());
                emit(part | (v << 16));
                part = 0;
                open = false;
                advance();
            }
            // word-aligned pairs two at a time; the pair pointers of a step that straddles the
            // wrap come apart
            while (k + 2 <= npairs) {
                const int run = (k < kw ? kw : npairs) - k;  // pairs before the wrap or the end
                if (run >= 2) {
                    const int steps = run >> 1;
                    for (int s = 0; s < steps; ++s) {
                        const uint32_t sa = next_sel();
                        const uint32_t sb = next_sel();
                        emit(pair2_dir(cp, cp + TB, sa, sb));
                        cp += 2 * TB;
                    }
                    k += 2 * steps;
                    if (k == kw) cp = cell2;
                } else {  // one pair left before the wrap: its partner is slot 0
                    const uint32_t va = pair_dir(cp, next_sel());
                    const uint32_t vb = pair_dir(cell2, next_sel());
                    emit(va | (vb << 16));
                    k += 2;
                    cp = cell2 + TB;
                }
            }
            if (k < npairs) {  // a last pair: the low half of an open word
                part = pair_dir(cp, next_sel());
                open = true;
                advance();
            }
            j += 2 * npairs;
            const int pe = p0 + npairs;
            xj = 2 * (pe >= P2 ? pe - P2 : pe);
            f = (int)fv >> 16;
            h1 = (int)h1v >> 16;
        }
        if (j < end) {  // even last column: the low lanes of its pair
            const int x = xj;
            uint2 cw = cell2[(size_t)(x >> 1) * TB];
            int e = (int)(int16_t)(cw.y & 0xffffu), h;
            const uint32_t sel = qsel(j >> 1);
            const uint32_t d = glb_cell((int)(int16_t)(cw.x & 0xffffu), e, f,
                                        (int)prmt(plo, phi, (sel & 0xffu) * 0x101u | 0x8800u), oe_del, sc.e_del,
                                        oe_ins, sc.e_ins, h);
            cw.x = (cw.x & 0xffff0000u) | ((uint32_t)h1 & 0xffffu);
            cw.y = (cw.y & 0xffff0000u) | ((uint32_t)e & 0xffffu);
            cell2[(size_t)(x >> 1) * TB] = cw;
            h1 = h;
            part |= open ? d << 16 : d;  // offset even: byte 2 after an open pair, else byte 0
            open = true;
            ++j;
        }
        {   // sentinel slot of column end: H(i, end-1), E unreachable
            const int x = xend;
            uint2 cw = cell2[(size_t)(x >> 1) * TB];
            if (x & 1) cw = make_uint2((cw.x & 0xffffu) | ((uint32_t)h1 << 16), (cw.y & 0xffffu) | ((uint32_t)NEG << 16));
            else cw = make_uint2((cw.x & 0xffff0000u) | ((uint32_t)h1 & 0xffffu),
                                 (cw.y & 0xffff0000u) | ((uint32_t)NEG & 0xffffu));
            cell2[(size_t)(x >> 1) * TB] = cw;
        }
        // the open word, the rest of its group as zeros, then zero groups up to ngroups
        if (open) emit(part);
        while (nw & 3) emit(0u);
        for (int g = nw >> 2; g < ngroups; ++g) zr[g] = make_uint4(0u, 0u, 0u, 0u);
        ncells += (unsigned long long)(end > beg ? end - beg : 0);
    }
    const int end_last = tlen > 0 ? (tlen + w < qlen ? tlen + w : qlen) : -1;
    int score;
    if (end_last == qlen) {
        const int x = qlen % B2;
        const uint32_t hx = cell2[(size_t)(x >> 1) * TB].x;
        score = C::score32((x & 1) ? (int)hx >> 16 : (int)(int16_t)(hx & 0xffffu));
    } else {
        score = qlen == 0 ? 0 : (qlen <= w ? -(sc.o_ins + sc.e_ins * qlen) : MINUS_INF);
    }
    score_out[k] = score;
    ncig_out[k] = GLB_TB_PAIRS;  // glb_traceback_kernel follows (the column-pair layout)
    if (bad) atomicOr(err, ERR_BASE);
    atomicAdd(cells_total, ncells);
}

// The traceback of jobs order[base .. base + count) (base .. base + count without an order)
// whose DP ran: one thread per job, no shared memory, so its warps fit beside the
// shared-memory-bound DP kernel of another bucket and the walk's dependent HBM reads overlap
// that kernel's ALU work.  ncig[k] carries the layout the DP kernel wrote the direction bytes in
// (0: the job was rejected, no walk) and leaves with the run count.
__global__ void __launch_bounds__(256) glb_traceback_kernel(const GlobalDevJob *__restrict__ jobs,
                                                            const uint32_t *__restrict__ order, uint32_t base,
                                                            uint32_t count, const uint8_t *__restrict__ z,
                                                            uint32_t *__restrict__ cig, int32_t *__restrict__ ncig,
                                                            uint32_t *__restrict__ err)
{
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
        const uint32_t k = order ? order[base + t] : base + t;
        const int layout = ncig[k];
        if (layout != GLB_TB_ROWS && layout != GLB_TB_PAIRS) continue;
        const GlobalDevJob J = jobs[k];
        const int w = J.w < 0 ? 0 : J.w;
        const int n_col = J.qlen < 2 * w + 1 ? J.qlen : 2 * w + 1;
        const uint8_t *zj = z + J.z_off;
        const int nc = layout == GLB_TB_PAIRS
                           ? global_traceback<true>(zj, (size_t)J.zrow, n_col, J.qlen, J.tlen, w, cig + J.cig_off)
                           : global_traceback<false>(zj, (size_t)J.zrow, n_col, J.qlen, J.tlen, w, cig + J.cig_off);
        if (nc < 0) atomicOr(err, ERR_RANGE);
        ncig[k] = nc < 0 ? 0 : nc;
    }
}

// dense[doff[k] ..] = cig[cig_off[k] .. + ncig[k]]: one warp per job.
__global__ void global_compact_kernel(const GlobalDevJob *__restrict__ jobs, uint32_t n,
                                      const uint32_t *__restrict__ cig, const int32_t *__restrict__ ncig,
                                      const uint64_t *__restrict__ doff, uint32_t *__restrict__ dense)
{
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n; k += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t *src = cig + jobs[k].cig_off;
        uint32_t *dst = dense + doff[k];
        for (int x = (int)lane; x < ncig[k]; x += 32) dst[x] = src[x];
    }
}

// ---- device-side planning and gather for host-buffer calls (pageable host memory)

__device__ __forceinline__ bool gjob_ok(const bwacuda_global_job &J)
{
    return J.qlen >= 0 && J.tlen >= 0 && (J.qlen == 0 || J.query != nullptr) && (J.tlen == 0 || J.target != nullptr);
}

// Per job: base reserve, CIGAR capacity, traceback bytes and the sort key
// (bucket, query length descending, target length descending); per bucket the
// widest band (slots) and longest query, reduced over the lanes that share a
// bucket.  flags[0]: input error bits.  bstat[2b], bstat[2b+1]: bucket b's max
// band slots and max query length.
__global__ void glb_plan_kernel(const bwacuda_global_job *__restrict__ hj, uint32_t n, int qlim,
                                GlbNarrowRule nr, uint64_t *__restrict__ seq_sz, uint64_t *__restrict__ cig_sz,
                                uint64_t *__restrict__ z_sz, uint32_t *__restrict__ keys, uint32_t *__restrict__ idx,
                                uint32_t *__restrict__ flags, uint32_t *__restrict__ bstat, uint32_t *__restrict__ bwide)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t k0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); k0 < n; k0 += stride) {
        const uint32_t k = k0 + (threadIdx.x & 31u);
        int ql = 0, tl = 0, bs = 0, bucket = 0;
        bool bad = false, wide = false;
        if (k < n) {
            const bwacuda_global_job J = hj[k];
            const bool ok = gjob_ok(J);
            bad = !ok || J.qlen > qlim;
            ql = ok ? J.qlen : 0;
            tl = ok ? J.tlen : 0;
            seq_sz[k] = ok ? 16ull * (slice_words(J.query, ql) + slice_words(J.target, tl)) : 0u;
            cig_sz[k] = (uint64_t)ql + (uint64_t)tl + 1u;
            z_sz[k] = (uint64_t)tl * (uint64_t)global_zrow(ql, J.w);
            bs = global_band_slots(ql, J.w);
            bucket = global_bucket(ql);
            wide = !global_narrow(ql, tl, nr);
            const uint32_t qk = ql > 1023 ? 0u : 1023u - (uint32_t)ql;
            const uint32_t tk = tl > 4095 ? 0u : 4095u - (uint32_t)tl;
            keys[k] = ((uint32_t)bucket << 22) | (qk << 12) | tk;
            idx[k] = k;
        }
        const unsigned live = __ballot_sync(0xffffffffu, k < n);
        if (__reduce_or_sync(0xffffffffu, bad ? 1u : 0u) && (threadIdx.x & 31u) == 0) atomicOr(flags, 1u);
        // lanes of one bucket reduce together; their lowest lane updates the bucket's maxima
        const unsigned grp = __match_any_sync(0xffffffffu, bucket) & live;
        if (k < n) {
            const unsigned bmax = __reduce_max_sync(grp, (unsigned)bs);
            const unsigned qmax = __reduce_max_sync(grp, (unsigned)ql);
            const unsigned anyw = __reduce_or_sync(grp, wide ? 1u : 0u);
            if ((int)(threadIdx.x & 31u) == __ffs(grp) - 1) {
                atomicMax(bstat + 2 * bucket, bmax);
                atomicMax(bstat + 2 * bucket + 1, qmax);
                if (anyw) atomicOr(bwide + bucket, 1u);
            }
        }
    }
}

// [start, end) of each bucket in the sorted keys.
__global__ void glb_bucket_bounds_kernel(const uint32_t *__restrict__ keys, uint32_t n, uint32_t *__restrict__ bounds)
{
    const int b = threadIdx.x;
    if (b >= GLB_NBUCKETS) return;
    for (int side = 0; side < 2; ++side) {
        const uint32_t v = (uint32_t)(b + side) << 22;
        uint32_t lo = 0, hi = n;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (keys[mid] < v) lo = mid + 1;
            else hi = mid;
        }
        bounds[2 * b + side] = lo;
    }
}

// One warp per 32 jobs: lane l writes its job's descriptor, then the warp copies the
// 32 jobs' slices as aligned 16-byte words (warp_gather_slices).
__global__ void __launch_bounds__(256) glb_gather_kernel(const bwacuda_global_job *__restrict__ hj, uint32_t n,
                                                         const uint64_t *__restrict__ seq_off,
                                                         const uint64_t *__restrict__ cig_off,
                                                         const uint64_t *__restrict__ z_off,
                                                         uint8_t *__restrict__ seq, GlobalDevJob *__restrict__ dj)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t ngroups = (n + 31) / 32;
    for (uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < ngroups; g += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t k = g * 32 + lane;
        uint64_t qa = 0, ta = 0, base = 0;
        uint32_t qw = 0, tw = 0;
        if (k < n) {
            const bwacuda_global_job J = hj[k];
            const bool ok = gjob_ok(J);
            const int ql = ok ? J.qlen : 0, tl = ok ? J.tlen : 0;
            base = seq_off[k];
            qa = reinterpret_cast<uint64_t>(J.query);
            ta = reinterpret_cast<uint64_t>(J.target);
            qw = slice_words(J.query, ql);
            tw = slice_words(J.target, tl);
            GlobalDevJob D;
            D.q_off = base + (qa & 15);
            D.t_off = base + 16ull * qw + (ta & 15);
            D.z_off = z_off[k];
            D.cig_off = cig_off[k];
            D.qlen = ql;
            D.tlen = tl;
            D.w = J.w;
            D.zrow = global_zrow(ql, J.w);
            dj[k] = D;
        }
        warp_gather_slices(qa & ~15ull, ta & ~15ull, base, qw, tw, seq);
    }
}

// Results straight into the caller's arrays: score[k], cigar_off[k + 1] = base + doff[k + 1],
// and (when the chunk's runs fit the caller's capacity) the runs themselves.  One thread per
// job: consecutive jobs' scores, offsets and runs lie at consecutive host addresses, so a
// warp's stores coalesce.
__global__ void glb_store_kernel(const GlobalDevJob *__restrict__ dj, uint32_t n, const int32_t *__restrict__ dscore,
                                 const uint32_t *__restrict__ cig, const int32_t *__restrict__ ncig,
                                 const uint64_t *__restrict__ doff, uint64_t out_base, size_t cap,
                                 int32_t *__restrict__ hscore, uint64_t *__restrict__ hoff, uint32_t *__restrict__ hcig)
{
    const bool fits = hcig != nullptr && out_base + doff[n] <= cap;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        hscore[k] = dscore[k];
        hoff[k + 1] = out_base + doff[k + 1];
        if (fits) {
            const uint32_t *src = cig + dj[k].cig_off;
            uint32_t *dst = hcig + out_base + doff[k];
            const int nk = ncig[k];
            for (int x = 0; x < nk; ++x) dst[x] = src[x];
        }
    }
}

template <int TB, bool NARROW, bool Q4 = false>
cudaError_t launch_global_tb(const uint8_t *seq, const GlobalDevJob *jobs, const uint32_t *order, uint32_t base,
                             uint32_t count, const Scoring &sc, int bcap, int qcap, uint8_t *z, uint32_t *cig,
                             int32_t *score, int32_t *ncig, uint32_t *err, unsigned long long *cells, cudaStream_t s)
{
    // narrow jobs: the 16x2 pair kernel; wide jobs: 32-bit cells, one column at a time
    const size_t smem = NARROW ? global_smem_pair(bcap, qcap, TB, Q4) : global_smem(bcap, qcap, TB, false);
    auto kern = NARROW ? global_pair_kernel<TB, Q4> : global_tpj_kernel<TB, false>;
    // process-wide per kernel: always the ceiling (concurrent contexts must not shrink it)
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LIMIT);
    if (e != cudaSuccess) return e;
    kern<<<(count + TB - 1) / TB, TB, smem, s>>>(seq, jobs, order, base, count, sc, bcap, qcap, z, cig, score, ncig,
                                                 err, cells);
    return cudaGetLastError();
}

template <bool NARROW>
cudaError_t launch_global_form(const uint8_t *seq, const GlobalDevJob *jobs, const uint32_t *order, uint32_t base,
                               uint32_t count, const Scoring &sc, int bcap, int qcap, uint8_t *z, uint32_t *cig,
                               int32_t *score, int32_t *ncig, uint32_t *err, unsigned long long *cells, cudaStream_t s)
{
    // the block size that keeps the most warps resident (shared memory bounds this kernel;
    // 228 KB per SM, 1 KB of it reserved per block), larger blocks on ties
    auto resident = [&](bool q4, int &best_tb) {
        int best_warps = 0;
        best_tb = 32;
        for (int tb = 128; tb >= 32; tb >>= 1) {
            const size_t sm = NARROW ? global_smem_pair(bcap, qcap, tb, q4) : global_smem(bcap, qcap, tb, false);
            if (sm > SMEM_LIMIT) continue;
            const int blocks = std::min<int>(32, (int)((228u * 1024u) / (sm + 1024u)));
            const int warps = std::min(64, blocks * tb / 32);
            if (warps > best_warps) {
                best_warps = warps;
                best_tb = tb;
            }
        }
        return best_warps;
    };
    int best_tb = 32, tb4 = 32;
    const int warps = resident(false, best_tb);
    // 4-bit query codes wherever they keep more warps resident (measured on the CIGAR-stage
    // buckets: the extra instructions cost less than the added warps bring, also in the
    // ALU-bound 100 and 150 bp buckets)
    if (NARROW && resident(true, tb4) > warps) {
        if (tb4 == 128)
            return launch_global_tb<128, NARROW, true>(seq, jobs, order, base, count, sc, bcap, qcap, z, cig, score,
                                                       ncig, err, cells, s);
        if (tb4 == 64)
            return launch_global_tb<64, NARROW, true>(seq, jobs, order, base, count, sc, bcap, qcap, z, cig, score,
                                                      ncig, err, cells, s);
        return launch_global_tb<32, NARROW, true>(seq, jobs, order, base, count, sc, bcap, qcap, z, cig, score, ncig,
                                                  err, cells, s);
    }
    if (best_tb == 128)
        return launch_global_tb<128, NARROW>(seq, jobs, order, base, count, sc, bcap, qcap, z, cig, score, ncig, err,
                                             cells, s);
    if (best_tb == 64)
        return launch_global_tb<64, NARROW>(seq, jobs, order, base, count, sc, bcap, qcap, z, cig, score, ncig, err,
                                            cells, s);
    return launch_global_tb<32, NARROW>(seq, jobs, order, base, count, sc, bcap, qcap, z, cig, score, ncig, err,
                                        cells, s);
}

// Jobs order[base .. base + count) (or base .. base + count without an order); bcap / qcap:
// their largest band-slot count and query length; narrow: every one of them fits the
// 16-bit cells (global_narrow).
cudaError_t launch_global(const uint8_t *seq, const GlobalDevJob *jobs, const uint32_t *order, uint32_t base,
                          uint32_t count, const Scoring &sc, int bcap, int qcap, bool narrow, uint8_t *z, uint32_t *cig,
                          int32_t *score, int32_t *ncig, uint32_t *err, unsigned long long *cells, cudaStream_t s)
{
    if (count == 0) return cudaSuccess;
    if (bcap < 1) bcap = 1;
    if (narrow)
        return launch_global_form<true>(seq, jobs, order, base, count, sc, bcap, qcap, z, cig, score, ncig, err,
                                        cells, s);
    return launch_global_form<false>(seq, jobs, order, base, count, sc, bcap, qcap, z, cig, score, ncig, err, cells,
                                     s);
}

// The traceback of jobs order[base .. base + count), after their DP launches.
cudaError_t launch_global_traceback(const GlobalDevJob *jobs, const uint32_t *order, uint32_t base, uint32_t count,
                                    const uint8_t *z, uint32_t *cig, int32_t *ncig, uint32_t *err, int nsm,
                                    cudaStream_t s)
{
    if (count == 0) return cudaSuccess;
    const uint32_t grid = (uint32_t)std::min<size_t>((count + 255) / 256, (size_t)nsm * 8);
    glb_traceback_kernel<<<grid, 256, 0, s>>>(jobs, order, base, count, z, cig, ncig, err);
    return cudaGetLastError();
}

GlbNarrowRule global_narrow_rule(const Scoring &sc, int m, const int8_t *mat)
{
    int mn = 0, mx = 0;
    for (int i = 0; i < m * m; ++i) {
        mn = std::min(mn, (int)mat[i]);
        mx = std::max(mx, (int)mat[i]);
    }
    GlbNarrowRule r;
    r.cost = std::max(std::max(sc.o_del + sc.e_del, sc.o_ins + sc.e_ins), std::max(-mn, mx));
    r.base = sc.o_del + sc.o_ins + sc.o_del + sc.e_del + sc.o_ins + sc.e_ins;
    return r;
}

// Longest query a 32-thread block holds (its band slots are at most qlen + 1).
int global_max_qlen()
{
    int q = (int)(SMEM_LIMIT / (32 * 9));
    while (q > 0 && global_smem(q + 1, q, 32) > SMEM_LIMIT) --q;
    return q;
}

struct GlobalBufs {
    HostBuf h_seq, h_jobs, h_res;
    DevBuf d_seq, d_jobs, d_z, d_cig, d_res, d_doff, d_dense, d_tmp;
    // device-gather route
    DevBuf d_sz, d_flags;
    HostBuf h_tot;
};

}  // namespace

struct GlobalState {
    GlobalBufs b;
    static constexpr int NSIDE = GLB_SIDE_STREAMS;
    cudaStream_t side[NSIDE] = {};  // bucket DP launches beside the context's stream
    cudaEvent_t ready = nullptr, done[NSIDE] = {};
    cudaError_t init_streams()
    {
        cudaError_t e = cudaSuccess;
        if (!ready) e = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
        for (int x = 0; x < NSIDE && e == cudaSuccess; ++x) {
            if (!side[x]) e = cudaStreamCreateWithFlags(&side[x], cudaStreamNonBlocking);
            if (e == cudaSuccess && !done[x]) e = cudaEventCreateWithFlags(&done[x], cudaEventDisableTiming);
        }
        return e;
    }
};

void global_release(bwacuda_ctx *c)
{
    if (!c->global) return;
    GlobalBufs &b = c->global->b;
    b.h_seq.release(); b.h_jobs.release(); b.h_res.release();
    b.d_seq.release(); b.d_jobs.release(); b.d_z.release(); b.d_cig.release(); b.d_res.release();
    b.d_doff.release(); b.d_dense.release(); b.d_tmp.release();
    b.d_sz.release(); b.d_flags.release(); b.h_tot.release();
    for (int x = 0; x < GlobalState::NSIDE; ++x) {
        if (c->global->side[x]) {
            cudaStreamSynchronize(c->global->side[x]);
            cudaStreamDestroy(c->global->side[x]);
        }
        if (c->global->done[x]) cudaEventDestroy(c->global->done[x]);
    }
    if (c->global->ready) cudaEventDestroy(c->global->ready);
    delete c->global;
    c->global = nullptr;
}

}  // namespace bwacuda

using namespace bwacuda;

namespace {

// The device-gather route: planning, gather, DP, compaction and the result stores
// run as kernels that read and write the caller's host arrays through the host
// page tables; the host launches and reads back four words per chunk.
int global_batch_device(bwacuda_ctx *c, const bwacuda_global_job *jobs, size_t n, const Scoring &sc,
                        const GlbNarrowRule &nrule, int32_t *score, uint64_t *cigar_off, uint32_t *cigar,
                        size_t cigar_cap)
{
    GlobalState &G = *c->global;
    GlobalBufs &b = G.b;
    cudaStream_t s = c->stream;
    if (cudaError_t e0 = G.init_streams()) return cuda_status(e0);
    uint32_t *d_err = static_cast<uint32_t *>(c->d_misc.p);
    unsigned long long *d_cells = reinterpret_cast<unsigned long long *>((char *)c->d_misc.p + 8);
    // chunks of 4 x BWACUDA_OPT_CHUNK_JOBS jobs, at most 1M (several waves of the longest
    // bucket per launch), halved while a chunk's traceback matrices would exceed 16 GiB of HBM
    const size_t kMaxZBytes = size_t(16) << 30;
    size_t chunk = std::min(size_t(1) << 20, std::max<size_t>(c->chunk_jobs, 1) * 4);
    const int qlim = global_max_qlen();
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || nsm < 1) nsm = 1;
    uint64_t out_base = 0;
    bool short_buf = false;
    int rc = BWACUDA_OK;
    cudaError_t e = cudaSuccess;
    if ((e = b.d_flags.ensure(256)) != cudaSuccess) return cuda_status(e);
    if ((e = b.h_tot.ensure(512)) != cudaSuccess) return cuda_status(e);
    uint64_t *ht = static_cast<uint64_t *>(b.h_tot.p);
    for (size_t c0 = 0, cn = 0; c0 < n && rc == BWACUDA_OK; c0 += cn) {
        cn = std::min(chunk, n - c0);
        const bwacuda_global_job *hj = jobs + c0;
        // planning arrays: seq / cig / z sizes and offsets (cn + 1 each), keys and indices (two
        // copies each for the sort)
        const size_t n1 = cn + 1;
        if ((e = b.d_sz.ensure(n1 * 6 * 8 + n1 * 4 * 4 + 256)) != cudaSuccess) break;
        uint64_t *seq_sz = static_cast<uint64_t *>(b.d_sz.p), *seq_off = seq_sz + n1;
        uint64_t *cig_sz = seq_off + n1, *cig_off = cig_sz + n1;
        uint64_t *z_sz = cig_off + n1, *z_off = z_sz + n1;
        uint32_t *keys = reinterpret_cast<uint32_t *>(z_off + n1), *keys2 = keys + n1;
        uint32_t *idx = keys2 + n1, *order = idx + n1;
        // [0] errors, [16..31] bucket stats, [32..47] bounds, [48..55] bucket holds a job too wide for 16-bit cells
        uint32_t *flags = static_cast<uint32_t *>(b.d_flags.p);
        uint32_t *bstat = flags + 16, *bounds = flags + 32, *bwide = flags + 48;
        size_t t1 = 0, t2 = 0, t3 = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, t1, (const uint64_t *)nullptr, (uint64_t *)nullptr, (int)cn + 1);
        cub::DeviceScan::ExclusiveSum(nullptr, t2, (const int32_t *)nullptr, (uint64_t *)nullptr, (int)cn + 1);
        cub::DeviceRadixSort::SortPairs(nullptr, t3, (const uint32_t *)nullptr, (uint32_t *)nullptr,
                                        (const uint32_t *)nullptr, (uint32_t *)nullptr, (int)cn, 0, 25);
        if ((e = b.d_tmp.ensure(std::max(std::max(t1, t2), t3) + 64)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(flags, 0, 256, s)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(seq_sz + cn, 0, 8, s)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(cig_sz + cn, 0, 8, s)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(z_sz + cn, 0, 8, s)) != cudaSuccess) break;
        uint32_t grid = (uint32_t)std::min<size_t>((cn + 255) / 256, (size_t)nsm * 8);
        glb_plan_kernel<<<grid, 256, 0, s>>>(hj, (uint32_t)cn, qlim, nrule, seq_sz, cig_sz, z_sz, keys, idx, flags,
                                             bstat, bwide);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cub::DeviceScan::ExclusiveSum(b.d_tmp.p, t1, seq_sz, seq_off, (int)cn + 1, s)) != cudaSuccess) break;
        if ((e = cub::DeviceScan::ExclusiveSum(b.d_tmp.p, t1, cig_sz, cig_off, (int)cn + 1, s)) != cudaSuccess) break;
        if ((e = cub::DeviceScan::ExclusiveSum(b.d_tmp.p, t1, z_sz, z_off, (int)cn + 1, s)) != cudaSuccess) break;
        if ((e = cub::DeviceRadixSort::SortPairs(b.d_tmp.p, t3, keys, keys2, idx, order, (int)cn, 0, 25, s)) != cudaSuccess)
            break;
        glb_bucket_bounds_kernel<<<1, 32, 0, s>>>(keys2, (uint32_t)cn, bounds);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(ht + 0, seq_off + cn, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(ht + 1, cig_off + cn, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(ht + 2, z_off + cn, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(ht + 3, flags, 256, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
        const uint32_t *hf = reinterpret_cast<const uint32_t *>(ht + 3);
        if (hf[0] & 1u) {
            // an invalid job, or a query longer than the kernel takes: find which on the host
            rc = BWACUDA_EINVAL;
            for (size_t k = 0; k < cn; ++k)
                if (hj[k].qlen > qlim && hj[k].qlen >= 0 && hj[k].tlen >= 0) rc = BWACUDA_EUNSUPPORTED;
            break;
        }
        if (ht[2] > kMaxZBytes && cn > 1024) {  // plan this range again in halves
            chunk = cn / 2;
            cn = 0;
            continue;
        }
        if ((e = b.d_seq.ensure(ht[0] + 16)) != cudaSuccess) break;
        if ((e = b.d_cig.ensure(ht[1] * 4 + 16)) != cudaSuccess) break;
        if ((e = b.d_z.ensure(ht[2] + 16)) != cudaSuccess) break;
        if ((e = b.d_jobs.ensure(cn * sizeof(GlobalDevJob))) != cudaSuccess) break;
        if ((e = b.d_res.ensure((cn + 1) * 8 + 16)) != cudaSuccess) break;
        if ((e = b.d_doff.ensure((cn + 1) * 8)) != cudaSuccess) break;
        GlobalDevJob *dj = static_cast<GlobalDevJob *>(b.d_jobs.p);
        glb_gather_kernel<<<grid, 256, 0, s>>>(hj, (uint32_t)cn, seq_off, cig_off, z_off,
                                              static_cast<uint8_t *>(b.d_seq.p), dj);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        int32_t *d_score = static_cast<int32_t *>(b.d_res.p);
        int32_t *d_ncig = d_score + cn + 1;
        uint64_t *d_doff = static_cast<uint64_t *>(b.d_doff.p);
        if ((e = cudaMemsetAsync(d_ncig + cn, 0, 4, s)) != cudaSuccess) break;
        // one DP launch per non-empty length bucket, sized by the bucket's own maxima, longest
        // queries first, round-robin over the context's stream and the side streams so a
        // bucket's blocks fill the last partial wave of the ones before it; the tracebacks
        // follow all of them
        const uint32_t *hb = hf + 16, *hbd = hf + 32, *hbw = hf + 48;
        if ((e = cudaEventRecord(G.ready, s)) != cudaSuccess) break;
        for (int x = 0; x < GlobalState::NSIDE && e == cudaSuccess; ++x) e = cudaStreamWaitEvent(G.side[x], G.ready, 0);
        if (e != cudaSuccess) break;
        int nl = 0;
        for (int bk = GLB_NBUCKETS - 1; bk >= 0 && e == cudaSuccess; --bk) {
            const uint32_t b0 = hbd[2 * bk], b1 = hbd[2 * bk + 1];
            if (b1 <= b0) continue;
            e = launch_global(static_cast<const uint8_t *>(b.d_seq.p), dj, order, b0, b1 - b0, sc, (int)hb[2 * bk],
                              (int)hb[2 * bk + 1], hbw[bk] == 0u, static_cast<uint8_t *>(b.d_z.p),
                              static_cast<uint32_t *>(b.d_cig.p), d_score, d_ncig, d_err, d_cells,
                              nl % (GlobalState::NSIDE + 1) ? G.side[nl % (GlobalState::NSIDE + 1) - 1] : s);
            ++nl;
            c->stats.kernel_launches += 1;
        }
        for (int x = 0; x < GlobalState::NSIDE && e == cudaSuccess; ++x) {
            e = cudaEventRecord(G.done[x], G.side[x]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(s, G.done[x], 0);
        }
        if (e != cudaSuccess) {
            for (int x = 0; x < GlobalState::NSIDE; ++x) cudaStreamSynchronize(G.side[x]);  // nothing runs on
            break;
        }
        if ((e = launch_global_traceback(dj, nullptr, 0, (uint32_t)cn, static_cast<const uint8_t *>(b.d_z.p),
                                         static_cast<uint32_t *>(b.d_cig.p), d_ncig, d_err, nsm, s)) != cudaSuccess)
            break;
        if ((e = cub::DeviceScan::ExclusiveSum(b.d_tmp.p, t2, d_ncig, d_doff, (int)cn + 1, s)) != cudaSuccess) break;
        grid = (uint32_t)std::min<size_t>((cn + 255) / 256, (size_t)nsm * 8);
        glb_store_kernel<<<grid, 256, 0, s>>>(dj, (uint32_t)cn, d_score, static_cast<const uint32_t *>(b.d_cig.p), d_ncig,
                                             d_doff, out_base, cigar ? cigar_cap : 0, score + c0, cigar_off + c0, cigar);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(ht + 40, d_doff + cn, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
        if (!cigar || out_base + ht[40] > cigar_cap) short_buf = true;
        out_base += ht[40];
        c->stats.kernel_launches += 11;
    }
    if (e != cudaSuccess) return cuda_status(e);
    if (rc) {
        uint64_t dummy;
        collect_device_status(c, s, &dummy);
        return rc;
    }
    uint64_t cells = 0;
    if ((rc = collect_device_status(c, s, &cells)) != BWACUDA_OK) return rc;
    c->stats.global_jobs += n;
    c->stats.global_cells += cells;
    return short_buf ? BWACUDA_ESHORT : BWACUDA_OK;
}

}  // namespace

extern "C" int bwacuda_ksw_global2_batch(bwacuda_ctx *c, const bwacuda_global_job *jobs, size_t n, int m,
                                         const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins,
                                         int32_t *score, uint64_t *cigar_off, uint32_t *cigar, size_t cigar_cap)
{
    if (!c) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    int rc = validate_scoring(m, mat, o_del, e_del, o_ins, e_ins);
    if (rc) return rc;
    if (n && (!jobs || !score || !cigar_off)) return BWACUDA_EINVAL;
    if (cigar_off) cigar_off[0] = 0;
    if (n == 0) return BWACUDA_OK;
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    if (!c->global) {
        c->global = new (std::nothrow) GlobalState();
        if (!c->global) return BWACUDA_ENOMEM;
    }
    const bool device_gather = c->host_gather == BWACUDA_GATHER_DEVICE ||
                               (c->host_gather == BWACUDA_GATHER_AUTO && c->pageable_access);
    if (device_gather) {
        if (!c->pageable_access) return BWACUDA_EUNSUPPORTED;
        const Scoring scd = make_scoring(m, mat, o_del, e_del, o_ins, e_ins);
        return global_batch_device(c, jobs, n, scd, global_narrow_rule(scd, m, mat), score, cigar_off, cigar,
                                   cigar_cap);
    }
    const int qlim = global_max_qlen();
    for (size_t k = 0; k < n; ++k) {
        const bwacuda_global_job &J = jobs[k];
        if (J.qlen < 0 || J.tlen < 0 || (J.qlen && !J.query) || (J.tlen && !J.target)) return BWACUDA_EINVAL;
        if (J.qlen > qlim) return BWACUDA_EUNSUPPORTED;
    }
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    if (!c->global) {
        c->global = new (std::nothrow) GlobalState();
        if (!c->global) return BWACUDA_ENOMEM;
    }
    GlobalBufs &b = c->global->b;
    const Scoring sc = make_scoring(m, mat, o_del, e_del, o_ins, e_ins);
    const GlbNarrowRule nrule = global_narrow_rule(sc, m, mat);
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || nsm < 1) nsm = 1;
    cudaStream_t s = c->stream;
    uint32_t *d_err = static_cast<uint32_t *>(c->d_misc.p);
    // chunks bounded in jobs and in traceback bytes
    const size_t kMaxJobs = 262144, kMaxZBytes = (size_t)1 << 31;  // 2 GiB of traceback per chunk
    uint64_t out_base = 0;
    bool short_buf = false;
    cudaError_t e = cudaSuccess;
    size_t c0 = 0;
    while (c0 < n && rc == BWACUDA_OK && e == cudaSuccess) {
        size_t cn = 0;
        uint64_t zbytes = 0, cigw = 0, bytes = 0;
        int qmax = 0, bmax = 1;
        bool narrow = true;
        while (c0 + cn < n && cn < kMaxJobs) {
            const bwacuda_global_job &J = jobs[c0 + cn];
            narrow = narrow && global_narrow(J.qlen, J.tlen, nrule);
            const uint64_t jz = (uint64_t)J.tlen * (uint64_t)global_zrow(J.qlen, J.w);
            if (cn > 0 && zbytes + jz > kMaxZBytes) break;
            zbytes += jz;
            bytes += (uint64_t)J.qlen + (uint64_t)J.tlen;
            cigw += (uint64_t)J.qlen + (uint64_t)J.tlen + 1;
            qmax = std::max(qmax, J.qlen);
            bmax = std::max(bmax, global_band_slots(J.qlen, J.w));
            ++cn;
        }
        // pack: bases and descriptors (each job's traceback matrix contiguous)
        if ((e = b.h_seq.ensure(bytes + 16)) != cudaSuccess) break;
        if ((e = b.h_jobs.ensure(cn * sizeof(GlobalDevJob))) != cudaSuccess) break;
        if ((e = b.h_res.ensure(cn * 8 + 16)) != cudaSuccess) break;
        uint8_t *hs = static_cast<uint8_t *>(b.h_seq.p);
        GlobalDevJob *hj = static_cast<GlobalDevJob *>(b.h_jobs.p);
        uint64_t so = 0, zo = 0, co = 0;
        for (size_t k = 0; k < cn; ++k) {
            const bwacuda_global_job &J = jobs[c0 + k];
            GlobalDevJob D;
            D.q_off = so;
            if (J.qlen) memcpy(hs + so, J.query, (size_t)J.qlen);
            so += (uint64_t)J.qlen;
            D.t_off = so;
            if (J.tlen) memcpy(hs + so, J.target, (size_t)J.tlen);
            so += (uint64_t)J.tlen;
            D.z_off = zo;
            D.zrow = global_zrow(J.qlen, J.w);
            zo += (uint64_t)J.tlen * (uint64_t)D.zrow;
            D.cig_off = co;
            co += (uint64_t)J.qlen + (uint64_t)J.tlen + 1;
            D.qlen = J.qlen;
            D.tlen = J.tlen;
            D.w = J.w;
            hj[k] = D;
        }
        size_t scan_bytes = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (const int32_t *)nullptr, (uint64_t *)nullptr, (int)cn + 1);
        if ((e = b.d_seq.ensure(bytes + 16)) != cudaSuccess) break;
        if ((e = b.d_jobs.ensure(cn * sizeof(GlobalDevJob))) != cudaSuccess) break;
        if ((e = b.d_z.ensure(zbytes + 16)) != cudaSuccess) break;
        if ((e = b.d_cig.ensure(cigw * 4 + 16)) != cudaSuccess) break;
        if ((e = b.d_res.ensure((cn + 1) * 8 + 16)) != cudaSuccess) break;
        if ((e = b.d_doff.ensure((cn + 1) * 8)) != cudaSuccess) break;
        if ((e = b.d_tmp.ensure(scan_bytes + 16)) != cudaSuccess) break;
        int32_t *d_score = static_cast<int32_t *>(b.d_res.p);
        int32_t *d_ncig = d_score + cn + 1;  // one spare slot: the scan's n+1-th input is zero
        uint64_t *d_doff = static_cast<uint64_t *>(b.d_doff.p);
        if (bytes && (e = cudaMemcpyAsync(b.d_seq.p, hs, bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(b.d_jobs.p, hj, cn * sizeof(GlobalDevJob), cudaMemcpyHostToDevice, s)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(d_ncig + cn, 0, 4, s)) != cudaSuccess) break;
        c->stats.h2d_bytes += bytes + cn * sizeof(GlobalDevJob);
        e = launch_global(static_cast<const uint8_t *>(b.d_seq.p), static_cast<const GlobalDevJob *>(b.d_jobs.p),
                          nullptr, 0, (uint32_t)cn, sc, bmax, qmax, narrow, static_cast<uint8_t *>(b.d_z.p),
                          static_cast<uint32_t *>(b.d_cig.p), d_score, d_ncig, d_err,
                          reinterpret_cast<unsigned long long *>((char *)c->d_misc.p + 8), s);
        if (e != cudaSuccess) break;
        if ((e = launch_global_traceback(static_cast<const GlobalDevJob *>(b.d_jobs.p), nullptr, 0, (uint32_t)cn,
                                         static_cast<const uint8_t *>(b.d_z.p), static_cast<uint32_t *>(b.d_cig.p),
                                         d_ncig, d_err, nsm, s)) != cudaSuccess)
            break;
        if ((e = cub::DeviceScan::ExclusiveSum(b.d_tmp.p, scan_bytes, d_ncig, d_doff, (int)cn + 1, s)) != cudaSuccess) break;
        // scores and run counts back; the host derives the offsets the device scan also made
        int32_t *hr = static_cast<int32_t *>(b.h_res.p);
        if ((e = cudaMemcpyAsync(hr, d_score, cn * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(hr + cn, d_ncig, cn * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
        uint64_t tot = 0;
        for (size_t k = 0; k < cn; ++k) {
            score[c0 + k] = hr[k];
            tot += (uint64_t)hr[cn + k];
            cigar_off[c0 + k + 1] = out_base + tot;
        }
        if (cigar && out_base + tot <= cigar_cap && tot) {
            if ((e = b.d_dense.ensure(tot * 4 + 16)) != cudaSuccess) break;
            const uint32_t grid = (uint32_t)std::min<size_t>((cn * 32 + 255) / 256, 4096);
            global_compact_kernel<<<grid, 256, 0, s>>>(static_cast<const GlobalDevJob *>(b.d_jobs.p), (uint32_t)cn,
                                                       static_cast<const uint32_t *>(b.d_cig.p), d_ncig, d_doff,
                                                       static_cast<uint32_t *>(b.d_dense.p));
            if ((e = cudaGetLastError()) != cudaSuccess) break;
            if ((e = cudaMemcpyAsync(cigar + out_base, b.d_dense.p, tot * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
            if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
            c->stats.d2h_bytes += tot * 4;
        } else if (out_base + tot > cigar_cap || !cigar) {
            short_buf = true;
        }
        c->stats.d2h_bytes += cn * 8;
        c->stats.kernel_launches += 4;
        out_base += tot;
        c0 += cn;
    }
    if (e != cudaSuccess) return cuda_status(e);
    uint64_t cells = 0;
    rc = collect_device_status(c, s, &cells);
    if (rc) return rc;
    c->stats.global_jobs += n;
    c->stats.global_cells += cells;
    return short_buf ? BWACUDA_ESHORT : BWACUDA_OK;
}
