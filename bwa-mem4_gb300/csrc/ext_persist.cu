// ext_persist.cu -- the batched extension path: jobs are length-sorted on the
// device, cut into buckets by query length and cell width, and each bucket is
// run by a persistent kernel sized to fill the GPU at that bucket's shared
// memory footprint.  Warps pull 32 consecutive sorted jobs at a time from the
// bucket's work counter, so the jobs that share a warp have near-equal row
// counts and window widths (the SIMT analogue of the reference's length-sorted
// lane groups, crates/bwa-neon/src/matesw.rs:176-183).  Bucket kernels go out
// on several streams so one bucket's tail overlaps the next bucket's start.
// The whole sequence (keys, sort, bucket bounds, launches) depends only on
// device data, so it can be captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>

#include "common.cuh"
#include "ext_job.cuh"
#include "kernels.h"
#include "persist.h"

namespace bwacuda {

namespace {

// Cell class of a job: 0 = 8-bit pairs, 1 = 16-bit, 2 = 32-bit cells.
__device__ __forceinline__ uint32_t ext_cell_class(const bwacuda_dev_ext_job &J, int max_sc)
{
    if (ext_fits_u8(J.qlen, J.tlen, J.h0, max_sc)) return 0u;
    return ext_fits_i16(J.qlen, J.tlen, J.h0, max_sc) ? 1u : 2u;
}

// 16-bit sort key: cell class (at least min_cls), query length descending
// (clamped at 1023), target length descending in 32-row steps (1024-row steps for the
// queries of 1023 bases or more, whose rows the open-ended buckets' kernels run longest
// first).  Within a bucket the order sets only which jobs run together, never a result.
__device__ __forceinline__ uint16_t ext_sort_key(const bwacuda_dev_ext_job &J, int max_sc, uint32_t min_cls)
{
    uint32_t cls = ext_cell_class(J, max_sc);
    cls = cls > min_cls ? cls : min_cls;
    const uint32_t ql = J.qlen < 0 ? 0u : (J.qlen > 1023 ? 1023u : (uint32_t)J.qlen);
    const uint32_t tsh = ql == 1023u ? 10u : 5u;
    const uint32_t tb = J.tlen < 0 ? 0u : ((uint32_t)J.tlen >> tsh > 15u ? 15u : (uint32_t)J.tlen >> tsh);
    return (uint16_t)((cls << 14) | ((1023u - ql) << 4) | (15u - tb));
}

// ungapped_hit (crates/bwa-neon/src/batched.rs:602-697): the result of a job whose
// diagonal carries at most x mismatches, no N and no z-drop, or false ("run the DP").
__device__ bool ungapped_hit(const uint8_t *q, int qlen, const uint8_t *t, int tlen, int h0, const UngappedRule &u,
                             int zdrop, bwacuda_ext_result &r)
{
    if (qlen == 0 || h0 <= 0 || tlen < qlen || u.x < 0) return false;
    // mismatch columns; only the first 128 are representable (the reference's u128 bitmap)
    uint32_t mis[4] = {0u, 0u, 0u, 0u};
    int nmis = 0;
    for (int c = 0; c < qlen; ++c) {
        const uint32_t qb = q[c], tb = t[c];
        if (qb >= 4u || tb >= 4u) return false;
        if (qb != tb) {
            if (++nmis > u.x) return false;
            if (c >= 128) return false;
            mis[c >> 5] |= 1u << (c & 31);
        }
    }
    if (nmis == 0) {
        const int s = h0 + qlen * u.a;
        r.score = s; r.qle = qlen; r.tle = qlen; r.gtle = qlen; r.gscore = s; r.max_off = 0;
        return true;
    }
    if (qlen > 128) return false;
    int run = h0, best = h0, best_end = 0;
    for (int c = 0; c < qlen; ++c) {
        if (run == 0) continue;
        if (((mis[c >> 5] >> (c & 31)) & 1u) == 0u) run += u.a;
        else {
            run -= u.b;
            if (run < 0) run = 0;
        }
        if (run > best) { best = run; best_end = c + 1; }
        else if (zdrop > 0 && best - run > zdrop) return false;
    }
    if (run == 0) return false;
    r.score = best; r.qle = best_end; r.tle = best_end; r.gtle = qlen; r.gscore = run; r.max_off = 0;
    return true;
}

// Sort keys; with the ungapped rule on, jobs it settles get their result here
// and key class 3, which no bucket covers.
__global__ void ext_keys_kernel(const bwacuda_dev_ext_job *__restrict__ jobs, uint32_t n, int max_sc,
                                uint32_t min_cls, const uint8_t *__restrict__ seq, const UngappedRule ug, int zdrop,
                                bwacuda_ext_result *__restrict__ out, uint16_t *__restrict__ keys,
                                uint32_t *__restrict__ idx)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const bwacuda_dev_ext_job J = jobs[k];
        uint16_t key = ext_sort_key(J, max_sc, min_cls);
        if (ug.enabled) {
            bwacuda_ext_result r;
            if (ungapped_hit(seq + J.q_off, J.qlen, seq + J.t_off, J.tlen, J.h0, ug, zdrop, r)) {
                out[k] = r;
                key = (uint16_t)(3u << 14);
            }
        }
        keys[k] = key;
        idx[k] = k;
    }
}

__device__ __forceinline__ uint32_t lower_bound16(const uint16_t *a, uint32_t n, uint32_t v)
{
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Bucket b covers sorted keys [key_lo, key_hi]; writes its [start, end) and
// clears its work counter.  This kernel is the only writer of the bounds, and a lower bound over
// the n sorted keys lies in [0, n], so no persistent kernel reading them (in a stream launch or a
// graph replay, whose capture is keyed on the same n) can index past the order and job arrays.
__global__ void ext_bucket_bounds_kernel(const uint16_t *__restrict__ keys, uint32_t n,
                                         const ExtBucketDef *__restrict__ defs, int nb,
                                         uint32_t *__restrict__ table)
{
    const int b = threadIdx.x;
    if (b >= nb) return;
    const ExtBucketDef d = defs[b];
    const uint32_t ql_hi = d.qhi > 1023 ? 1023u : (uint32_t)d.qhi;
    const uint32_t ql_lo = d.qlo > 1023 ? 1023u : (uint32_t)d.qlo;
    const uint32_t key_lo = ((uint32_t)d.cls << 14) | ((1023u - ql_hi) << 4);
    const uint32_t key_hi = ((uint32_t)d.cls << 14) | ((1023u - ql_lo) << 4) | 15u;
    table[b * 4 + 0] = lower_bound16(keys, n, key_lo);
    table[b * 4 + 1] = lower_bound16(keys, n, key_hi + 1);
    table[b * 4 + 2] = 0;  // work counter
    table[b * 4 + 3] = 0;  // work counter of the window kernel (open-ended buckets)
}

}  // namespace

// Query-length buckets of each cell class.  Below 257 columns the caps step by
// `step` (16, 32 or 64: the autotuner's bucket granularity); longer queries
// (16/32-bit cells only: an 8-bit job has h0 + min(qlen, tlen) * max_sc < 256)
// take fixed caps; the last bucket of a class is open-ended.
static const int kQcapLong[] = {385, 513, 769, 1023};

static int max_qcap_of_class(int cls)
{
    if (cls == 0) return 257;  // bound < 256 forces min(qlen, tlen) < 256; longer queries meet short targets
    return (int)ext_tpj_smem_limit_qcap(cls == 2);
}

int ext_bucket_defs(ExtBucketDef *defs, int max_defs, int step, int long_qlo)
{
    if (step != 16 && step != 32 && step != 64) step = 32;
    int nb = 0;
    for (int cls = 0; cls < 3; ++cls) {
        int caps[32], nc = 0;
        for (int c = step + 1; c <= 257; c += step) caps[nc++] = c;
        const int nlong = cls == 0 ? 0 : (cls == 1 ? 4 : 3);  // 32-bit cells: up to 769 columns in one block
        for (int k = 0; k < nlong; ++k) caps[nc++] = kQcapLong[k];
        int lo = 0;
        for (int c = 0; c < nc && nb < max_defs; ++c) {
            ExtBucketDef d;
            d.cls = cls;
            d.qlo = lo;
            d.qhi = caps[c] - 1;
            d.qcap = caps[c];
            d.kernel = d.qhi >= long_qlo ? 1 : 0;  // the bucket holds queries of long_qlo or more
            defs[nb++] = d;
            lo = caps[c];
        }
        // the open-ended last class: every longer query up to the class's limit
        if (nb < max_defs) {
            ExtBucketDef d;
            d.cls = cls;
            d.qlo = lo;
            d.qhi = EXT_QHI_OPEN;
            d.qcap = cls == 0 ? (int)ext_tpj_smem_limit_qcap(false) : max_qcap_of_class(cls);
            d.kernel = 1;  // any query length
            defs[nb++] = d;
        }
    }
    return nb;
}

cudaError_t ext_sort_prefer_shared()
{
    // The bucket-bound kernel (one block, no shared memory) prefers the bucket kernels'
    // maximum shared-memory carveout.  The key kernel keeps the default: its blocks live for
    // one pass only, and with the ungapped rule it reads every job's bases through L1.
    return cudaFuncSetAttribute(ext_bucket_bounds_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                cudaSharedmemCarveoutMaxShared);
}

size_t ext_sort_temp_bytes(size_t n)
{
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, (const uint16_t *)nullptr, (uint16_t *)nullptr,
                                    (const uint32_t *)nullptr, (uint32_t *)nullptr, (int)n, 0, 16);
    return bytes;
}

cudaError_t ext_sort_and_bucket(const bwacuda_dev_ext_job *jobs, size_t n, int max_sc, bool pair_lanes,
                                const uint8_t *seq, const UngappedRule &ug, int zdrop, bwacuda_ext_result *out, uint16_t *keys_in,
                                uint16_t *keys_out, uint32_t *idx_in, uint32_t *idx_out, void *tmp,
                                size_t tmp_bytes, const ExtBucketDef *d_defs, int nb, uint32_t *d_table,
                                cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    uint32_t grid = (uint32_t)((n + 255) / 256);
    if (grid > 8192) grid = 8192;
    ext_keys_kernel<<<grid, 256, 0, s>>>(jobs, (uint32_t)n, max_sc, pair_lanes ? 0u : 1u, seq, ug, zdrop, out,
                                         keys_in, idx_in);
    cudaError_t e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys_in, keys_out, idx_in, idx_out, (int)n, 0,
                                                    16, s);
    if (e != cudaSuccess) return e;
    ext_bucket_bounds_kernel<<<1, EXT_MAX_BUCKETS, 0, s>>>(keys_out, (uint32_t)n, d_defs, nb, d_table);
    return cudaGetLastError();
}

cudaError_t ext_persist_launch(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *d_bucket_table, int nsm,
                               int tb)
{
    if (L.grab == 4) return ext_persist_launch_g4(L, d, d_bucket_table, nsm, tb);
    if (L.grab == 2) return ext_persist_launch_g2(L, d, d_bucket_table, nsm, tb);
    return ext_persist_launch_g1(L, d, d_bucket_table, nsm, tb);
}

}  // namespace bwacuda
