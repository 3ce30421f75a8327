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
    bwacuda_ext_result *out;
    uint32_t *err;
    unsigned long long *cells;
    cudaStream_t stream;
};

cudaError_t ext_tpj_launch(const ExtLaunch &L, bool wide);
size_t ext_tpj_smem_limit_qcap(bool wide);

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
    uint2 *scratch;   // suboptimal-tracker entries
    const uint64_t *scratch_off;  // per job entry offset into scratch
    bwacuda_rescue_result *out_aln;
    bwacuda_fwd_result *out_fwd;
    uint32_t *err;
    cudaStream_t stream;
};

cudaError_t rescue_tpj_launch(const RescueLaunch &L, bool wide);
cudaError_t rescue_wf_launch(const RescueLaunch &L, int qcap, int lanes);  // lanes per job: 8, 16 or 32
int rescue_wf_max_qpad();
size_t rescue_tpj_smem_limit_qcap(bool wide);
// Entries the suboptimal tracker may need for a target of tlen rows.
__host__ __device__ inline uint64_t rescue_scratch_entries(int tlen) { return (uint64_t)(tlen / 2 + 2); }
cudaError_t rescue_scratch_offsets(const bwacuda_dev_rescue_job *jobs, size_t n, uint64_t *off,
                                   void *tmp, size_t tmp_bytes, size_t *tmp_needed,
                                   cudaStream_t s);

}  // namespace bwacuda
