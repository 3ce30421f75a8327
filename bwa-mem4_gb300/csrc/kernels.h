// kernels.h -- host-side launch interface of the device kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "common.cuh"

namespace bwacuda {

// Largest shared memory of one extension block.  An SM holds 228 KB and reserves 1 KB per
// resident block, so a block of at most 225 KB still lets one small block (a gather, a
// length pass, another stream's kernel) run beside it; a 227 KB block would hold its SM
// alone, and a bucket launch of such blocks waits for every other kernel to leave an SM.
constexpr size_t EXT_SMEM_BLOCK_MAX = 225u * 1024u;

struct ExtLaunch {
    const uint8_t *seq;
    const bwacuda_dev_ext_job *jobs;
    const uint32_t *order;      // job index list, or nullptr for 0..n-1
    const uint32_t *count_ptr;  // device count overriding n, or nullptr
    size_t n;
    ExtParams P;
    int qcap;                   // >= max qlen + 1 over the launch
    int only_wide;              // wide launch: 1 = skip jobs that fit narrow cells;
                                // narrow launch: 2 = report wide jobs (no wide launch follows)
    int long_follows = 0;       // 1: jobs with qlen + 1 > qcap are left to a group-per-job launch
    bwacuda_ext_result *out;
    uint32_t *err;
    unsigned long long *cells;
    cudaStream_t stream;
};

cudaError_t ext_tpj_launch(const ExtLaunch &L, bool wide);
size_t ext_tpj_smem_limit_qcap(bool wide);

// Group-per-job extension of any query length (ext_long.cu, ext_long.cuh).  Every call site
// owns XL_WORK_WORDS device words, zeroed before its launches, and a deferred-job list of
// njobs entries.
constexpr int XL_WORK_DCOUNT = 1;                              // [0] stays 0, [1] deferred jobs
constexpr int XL_WORK_DCOUNTER16 = 2, XL_WORK_DCOUNTER32 = 3;  // work counters of the deferred launches
constexpr int XL_WORK_COUNTER16 = 4, XL_WORK_COUNTER32 = 5;    // work counters of unbucketed first launches
constexpr int XL_WORK_WORDS = 8;
constexpr int XL_RING_MIN = 256, XL_RING_FIRST_MAX = 4096;
constexpr int XL_RING_DEFAULT = 512;  // first-launch ring when the bands are not known on the host

struct ExtLongLaunch {
    const uint8_t *seq;
    const bwacuda_dev_ext_job *jobs;
    const uint32_t *order;   // job index list (nullptr: the identity)
    const uint32_t *bounds;  // [start, stop) of positions in order, device words (nullptr: [0, njobs))
    uint32_t *counter;       // zeroed work counter of the first launch
    uint32_t njobs;          // jobs of the call: bounds every position and job index
    int min_qlen;            // shorter jobs belong to another launch
    int lanes;               // lanes per job: 8, 16 or 32
    int ring_cols;           // first launch's ring columns per job (a power of two)
    ExtParams P;
    bwacuda_ext_result *out;
    uint32_t *err;
    unsigned long long *cells;
    uint32_t *defer;         // njobs entries: jobs set aside for the deferred launch
    uint32_t *defer_count;   // work + XL_WORK_DCOUNT
    // thread-per-job window kernel (ext_slide.cu) ahead of the group kernel on 16-bit jobs:
    // window columns (0: off), the fewest jobs [start, stop) must hold for it to run, and its
    // zeroed work counter
    int slide_wc = 0;
    uint32_t slide_min = 0;
    uint32_t *slide_counter = nullptr;
    int reserve_regs = 0, reserve_threads = 0, sm_regs = 65536, sm_threads = 2048;
    cudaStream_t stream;
};

cudaError_t ext_long_launch(const ExtLongLaunch &X, bool w32, int nsm);
// The window kernel alone (ext_long_launch runs it ahead of the group kernel when slide_wc > 0).
cudaError_t ext_slide_launch(const ExtLongLaunch &X, int nsm);
// Window columns for clamped bands up to w.
int ext_slide_window_for_band(int w);
cudaError_t ext_long_deferred_launch(const ExtLongLaunch &X, bool w32, uint32_t *work, int nsm);
// First-launch ring for bands up to w (XL_RING_MIN .. XL_RING_FIRST_MAX columns).
int ext_long_ring_for_band(int w);

// Rescue (ksw_local_fwd / ksw_align2).  mode: 0 = batched_ksw_align2,
// 1 = scalar ksw_align2, 2 = forward pass only (per-job minsc / endsc).
struct RescueLaunch {
    const uint8_t *seq;
    const bwacuda_dev_rescue_job *jobs;
    const uint32_t *order;
    const uint32_t *count_ptr;
    size_t n;
    Scoring sc;
    int mode;
    int lanes;        // 0 = bwa's rule per job, else 16 or 8
    int minsc;        // modes 0 and 1
    int qcap;         // >= padded query length + 16
    int only_wide;    // as ExtLaunch::only_wide
    int pair_cols = 0;  // 32-bit wavefront: skip the jobs the paired wavefront of this many columns took
    uint2 *scratch;   // suboptimal-tracker entries
    const uint64_t *scratch_off;  // per job entry offset into scratch
    bwacuda_rescue_result *out_aln;
    bwacuda_fwd_result *out_fwd;
    uint32_t *err;
    cudaStream_t stream;
};

// Whether a rescue job runs in the two-jobs-per-group wavefront of `cols` columns
// (rescue_wf2.cuh): every value fits a byte (min(qlen, tlen) * max_sc <= 255) and the padded
// query of both passes (bwa's width rule, or lanes_fixed; the reverse pass may pad to 16) fits
// min(cols, 256) columns; the target has fewer than 2^20 rows (the kernel's row field).
__host__ __device__ inline bool rescue_pair_job_ok(int qlen, int tlen, int max_sc, int lanes_fixed, int cols)
{
    if (qlen < 0 || tlen < 0 || tlen >= (1 << 20) || max_sc < 1 || cols <= 0) return false;
    const long long mn = qlen < tlen ? qlen : tlen;
    if (mn * max_sc > 255) return false;
    const int ln = lanes_fixed ? lanes_fixed : ((long long)qlen * max_sc < 250 ? 16 : 8);
    const int p1 = (qlen + ln - 1) / ln * ln, p16 = (qlen + 15) / 16 * 16;
    const int need = p1 > p16 ? p1 : p16;
    return need <= (cols < 256 ? cols : 256);
}

cudaError_t rescue_tpj_launch(const RescueLaunch &L, bool wide);
cudaError_t rescue_wf_launch(const RescueLaunch &L, int qcap, int lanes);  // lanes per job: 8, 16 or 32
// The paired wavefront (two jobs per group of 4, 8 or 16 lanes) over the jobs rescue_pair_job_ok
// admits at its column count; *cols receives that count (0: no launch, the matrix or the
// queries do not suit it).
cudaError_t rescue_wf2_launch(const RescueLaunch &L, int qcap, int lanes, int *cols);
int rescue_wf_max_qpad();
size_t rescue_tpj_smem_limit_qcap(bool wide);
// Entries the suboptimal tracker may need for a target of tlen rows.
__host__ __device__ inline uint64_t rescue_scratch_entries(int tlen) { return (uint64_t)(tlen / 2 + 2); }
cudaError_t rescue_scratch_offsets(const bwacuda_dev_rescue_job *jobs, size_t n, uint64_t *off,
                                   void *tmp, size_t tmp_bytes, size_t *tmp_needed,
                                   cudaStream_t s);

}  // namespace bwacuda
