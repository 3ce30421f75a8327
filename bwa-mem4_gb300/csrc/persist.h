// persist.h -- interface of the batched (sorted, bucketed, persistent) extension path.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "common.cuh"

namespace bwacuda {

// One bucket: jobs of cell class `cls` (0 = 8-bit pairs, 1 = 16-bit, 2 = 32-bit)
// with qlen in [qlo, qhi], run with qcap cell columns per thread (kernel 0) or by the
// group-per-job kernel (kernel 1: the open-ended buckets, whose queries may exceed any
// thread's shared-memory row, and the buckets from the tuned query length up).
struct ExtBucketDef {
    int32_t cls;
    int32_t qlo, qhi;
    int32_t qcap;
    int32_t kernel;
};

constexpr int EXT_MAX_BUCKETS = 64;  // one thread each in the bucket-bounds kernel
constexpr int32_t EXT_QHI_OPEN = 1 << 30;  // qhi of a class's open-ended last bucket

struct PersistLaunch {
    const uint8_t *seq;
    const bwacuda_dev_ext_job *jobs;
    const uint32_t *order;  // sorted job indices
    ExtParams P;
    bwacuda_ext_result *out;
    uint32_t *err;
    unsigned long long *cells;
    int grab;  // 32-job rounds a warp takes per work-counter grab
    cudaStream_t stream;
    // registers and threads per SM the persistent blocks leave free for kernels
    // that run beside them (0: fill the SM); sm_regs / sm_threads are the SM's
    int reserve_regs = 0, reserve_threads = 0;
    int sm_regs = 65536, sm_threads = 2048;
};

// long_qlo: buckets holding queries of this length or longer use the group-per-job kernel
// (INT_MAX: only the open-ended ones).
int ext_bucket_defs(ExtBucketDef *defs, int max_defs, int step, int long_qlo);
size_t ext_sort_temp_bytes(size_t n);
// the sort's own kernels prefer the maximum shared-memory carveout (once per device)
cudaError_t ext_sort_prefer_shared();
// keys + radix sort + bucket bounds; d_table holds 4 words per bucket
// (start, end, work counter, spare).
// With P.ug enabled the key kernel also settles ungapped hits (results written to out).
// pair_lanes false (gap costs too large for 16-bit lanes) keeps every job out of
// the 8-bit class.
cudaError_t ext_sort_and_bucket(const bwacuda_dev_ext_job *jobs, size_t n, int max_sc, bool pair_lanes,
                                const uint8_t *seq,
                                const UngappedRule &ug, int zdrop, bwacuda_ext_result *out, uint16_t *keys_in,
                                uint16_t *keys_out, uint32_t *idx_in, uint32_t *idx_out, void *tmp,
                                size_t tmp_bytes, const ExtBucketDef *d_defs, int nb, uint32_t *d_table,
                                cudaStream_t s);
// per-grab instantiations (ext_persist_g1.cu, _g2.cu, _g4.cu)
cudaError_t ext_persist_launch_g1(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *table, int nsm, int tb);
cudaError_t ext_persist_launch_g2(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *table, int nsm, int tb);
cudaError_t ext_persist_launch_g4(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *table, int nsm, int tb);
cudaError_t ext_persist_launch(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *d_bucket_table, int nsm,
                               int tb);

}  // namespace bwacuda
