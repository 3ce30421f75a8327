// common.cuh -- shared device-side definitions of the bwa-cuda engine.
//
// Score lookup.  Every kernel scores a cell with one byte permute: for target
// code tc the 8-byte "profile row" holds mat[tc*m + qc] in byte qc (qc < m) and
// 0 in the unused bytes, so a query column whose code is PAD_CODE (7) scores 0.
// That zero column is exactly ksw's query-profile padding
// (crates/bwa-neon/src/matesw.rs:591-607, ksw_qinit's `k >= qlen ? 0`).
#pragma once
#include <cstdint>

#include "../../include/bwacuda.h"

namespace bwacuda {

constexpr int PAD_CODE = 7;

// Per-launch scoring parameters, passed by value (kernel parameter space).
struct Scoring {
    int32_t m;
    int32_t o_del, e_del, o_ins, e_ins;
    int32_t max_sc;     // largest matrix entry (band clamp, score2 window)
    uint32_t prof[8][2]; // profile rows, see above; rows >= m unused
};

// The ungapped-diagonal fast path of the reference's batched extension
// (crates/bwa-neon/src/batched.rs:602-697, gated at :721-775): enabled only for a
// uniform matrix; a = match score, b = mismatch penalty magnitude, x = the most
// mismatches a diagonal may carry and still be provably optimal.
struct UngappedRule {
    int32_t enabled, a, b, x;
};

struct ExtParams {
    Scoring sc;
    int32_t end_bonus, zdrop;
    UngappedRule ug;
};

// Device error flags (OR-ed into ctx->d_err).
constexpr uint32_t ERR_BASE = 1u;      // a base code >= m
constexpr uint32_t ERR_RANGE = 2u;     // a score left the kernel's storage range
constexpr uint32_t ERR_SCRATCH = 4u;   // tracker scratch overflow (never expected)

__host__ __device__ inline uint32_t prof_lo(const Scoring &s, int tc) { return s.prof[tc][0]; }
__host__ __device__ inline uint32_t prof_hi(const Scoring &s, int tc) { return s.prof[tc][1]; }

// Pulls the 32-byte sector holding p into L2 (no register result, no wait).
__device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// PTX prmt in its generic mode: a selector nibble with bit 3 set replicates the
// sign of the selected byte (the __byte_perm intrinsic ignores that bit).
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel)
{
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(sel));
    return r;
}

// Sign-extended byte `qc` of the 8-byte profile row {lo, hi}.
__device__ __forceinline__ int prof_score(uint32_t lo, uint32_t hi, uint32_t qc)
{
    // selector nibbles: byte 0 <- qc, bytes 1..3 <- sign of byte qc
    return (int)prmt(lo, hi, qc * 0x1111u | 0x8880u);
}

// Band clamp, crates/bwa-neon/src/batched.rs:1305-1329: double division, then a
// truncating (toward zero, saturating) conversion exactly like `f64 as i32`.
__host__ __device__ inline int clamp_band(int w, int qlen, int max_sc, int end_bonus, int o_ins,
                                          int e_ins, int o_del, int e_del)
{
    double di = ((double)qlen * max_sc + end_bonus - o_ins) / e_ins + 1.0;
    double dd = ((double)qlen * max_sc + end_bonus - o_del) / e_del + 1.0;
#ifdef __CUDA_ARCH__
    int max_ins = __double2int_rz(di);
    int max_del = __double2int_rz(dd);
#else
    int max_ins = di != di ? 0 : (di >= 2147483647.0 ? 2147483647 : (di <= -2147483648.0 ? (-2147483647 - 1) : (int)di));
    int max_del = dd != dd ? 0 : (dd >= 2147483647.0 ? 2147483647 : (dd <= -2147483648.0 ? (-2147483647 - 1) : (int)dd));
#endif
    if (max_ins < 1) max_ins = 1;
    if (max_del < 1) max_del = 1;
    if (w > max_ins) w = max_ins;
    if (w > max_del) w = max_del;
    return w;
}

// Aligned 16-byte words covering a slice of len bytes at address src.  A
// device gather copies slices as whole words and places each one at a 16-byte
// aligned base plus (src & 15); the widened reads stay in the slice's own pages
// (a 16-byte word never straddles a page).
__host__ __device__ inline uint32_t slice_words(const uint8_t *src, int len)
{
    const uint64_t a = reinterpret_cast<uint64_t>(src);
    return len > 0 ? (uint32_t)(((a + (uint64_t)len - 1) >> 4) - (a >> 4) + 1) : 0u;
}

#ifdef __CUDACC__
// Copy the slices of the warp's 32 jobs (lane l's job: qw words at qa, then tw
// words at ta, both 16-byte aligned addresses) as one flat list of words over
// the whole warp: word x belongs to the lane whose exclusive prefix of word
// counts is the largest one <= x (a 5-step shuffle search), and every lane keeps
// eight independent 16-byte loads in flight before storing (the kernel is bound
// by host-memory latency, and beside the persistent DP kernels it gets few warps
// per SM).  The destinations are consecutive: lane l's job lands at
// seq + base_l with base_l = base_0 + 16 * (words of lanes < l) -- the layout an
// exclusive scan of 16 * (qw + tw) over consecutive jobs gives -- so flat word x
// is stored at seq + base_0 + 16 x.  All 32 lanes must call it, and lane 0 must
// carry a job (possibly empty).
__device__ __forceinline__ void warp_gather_slices(uint64_t qa, uint64_t ta, uint64_t base, uint32_t qw, uint32_t tw,
                                                   uint8_t *seq)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t wc = qw + tw;
    uint32_t pre = wc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, pre, o);
        if (lane >= (uint32_t)o) pre += v;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, pre, 31);
    pre -= wc;
    uint4 *dst = reinterpret_cast<uint4 *>(seq + __shfl_sync(0xffffffffu, base, 0));
    constexpr int U = 8;
    for (uint32_t x0 = 0; x0 < total; x0 += 32u * U) {
        uint4 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t x = x0 + (uint32_t)u * 32u + lane;
            int j = 0;
#pragma unroll
            for (int st = 16; st > 0; st >>= 1) {
                const uint32_t pj = __shfl_sync(0xffffffffu, pre, j + st);
                if (x >= pj) j += st;
            }
            const uint32_t pre_j = __shfl_sync(0xffffffffu, pre, j);
            const uint32_t qw_j = __shfl_sync(0xffffffffu, qw, j);
            const uint64_t qa_j = __shfl_sync(0xffffffffu, qa, j);
            const uint64_t ta_j = __shfl_sync(0xffffffffu, ta, j);
            const uint32_t wi = x - pre_j;
            if (x < total)
                v[u] = wi < qw_j ? reinterpret_cast<const uint4 *>(qa_j)[wi]
                                 : reinterpret_cast<const uint4 *>(ta_j)[wi - qw_j];
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t x = x0 + (uint32_t)u * 32u + lane;
            if (x < total) dst[x] = v[u];
        }
    }
}
#endif

// bwa-mem's 8/16-bit bin label of an extension job, the rule of
// crates/bwa-neon/src/batched.rs:817-865 split in two: bin_rule() summarises
// the matrix once per call, bin_label() classifies one job (statistics only).
struct BinRule {
    int32_t uniform;  // matrix is match / mismatch / N-penalty shaped
    int32_t mx;       // largest entry
    int32_t head;     // max(-mismatch, -N penalty, 0) + mx
};

inline BinRule bin_rule(int m, const int8_t *mat)
{
    BinRule r;
    const int a = mat[0], mm = mat[1], npen = mat[m - 1];
    bool uniform = m >= 2;
    for (int i = 0; i < m && uniform; ++i)
        for (int j = 0; j < m; ++j) {
            int want = (i == m - 1 || j == m - 1) ? npen : (i == j ? a : mm);
            if (mat[i * m + j] != want) { uniform = false; break; }
        }
    int mx = mat[0];
    for (int k = 0; k < m * m; ++k) mx = mat[k] > mx ? mat[k] : mx;
    int head = -(int)mat[1];
    if (-(int)mat[m - 1] > head) head = -(int)mat[m - 1];
    if (head < 0) head = 0;
    r.uniform = uniform;
    r.mx = mx;
    r.head = head + mx;
    return r;
}

__host__ __device__ inline int bin_label(const BinRule &r, int qlen, int tlen, int h0)
{
    if (!r.uniform) return 2;
    const int mn = qlen < tlen ? qlen : tlen;
    const long long bound = (long long)h0 + (long long)mn * (r.mx > 0 ? r.mx : 0);
    if (qlen < 256 && tlen < 256 && bound + r.head < 256) return 0;
    if (qlen < 32768 && tlen < 32768 && bound + r.head < 32768) return 1;
    return 2;
}

}  // namespace bwacuda
