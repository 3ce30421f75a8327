// ext_long.cu -- launches of the group-per-job extension kernel (ext_long.cuh): the query
// lengths the thread-per-job kernels cannot hold (their DP row lives in shared memory per
// thread), and, where the autotuner measures it faster, the longer buckets of the batched path.
//
// A call makes up to two launches per cell class: the first with the caller's ring size
// (enough for bands up to (R - 3) / 2 columns, or any band on queries of fewer than R
// columns), and a deferred launch over the jobs the first one set aside, one 32-lane group
// per block with the largest ring that fits a block's shared memory.
#include <cuda_runtime.h>

#include <algorithm>

#include "ext_long.cuh"
#include "kernels.h"

namespace bwacuda {

namespace {

constexpr int XL_C = 8;          // columns per lane per chunk
constexpr int XL_BLOCK = 128;    // threads per block of the first launch

template <bool W32, int L>
cudaError_t launch_first(const ExtLongLaunch &X, int nsm)
{
    auto kern = xl::ext_long_kernel<W32, L, XL_C>;
    const int groups = XL_BLOCK / L;
    // the largest ring up to the requested one whose block fits (jobs needing more are deferred)
    int ring = X.ring_cols;
    while (ring > XL_RING_MIN && (size_t)groups * xl::ring_words(ring, W32) * 4 > EXT_SMEM_BLOCK_MAX) ring >>= 1;
    const size_t smem = (size_t)groups * xl::ring_words(ring, W32) * 4;
    if (smem > EXT_SMEM_BLOCK_MAX) return cudaErrorInvalidValue;
    // process-wide per kernel: always the ceiling (see the persistent kernels)
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)EXT_SMEM_BLOCK_MAX);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, XL_BLOCK, smem)) != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidValue;
    if (X.reserve_regs > 0 || X.reserve_threads > 0) {
        cudaFuncAttributes fa;
        if ((e = cudaFuncGetAttributes(&fa, kern)) != cudaSuccess) return e;
        const int regs_block = ((fa.numRegs * 32 + 255) / 256) * 256 * (XL_BLOCK / 32);
        const int cap_r = regs_block > 0 ? (X.sm_regs - X.reserve_regs) / regs_block : per_sm;
        const int cap_t = (X.sm_threads - X.reserve_threads) / XL_BLOCK;
        per_sm = std::max(1, std::min(per_sm, std::min(cap_r, cap_t)));
    }
    kern<<<per_sm * nsm, XL_BLOCK, smem, X.stream>>>(X.seq, X.jobs, X.order, X.bounds, X.counter, X.njobs,
                                                    X.min_qlen, ring, X.defer, X.defer_count, W32 ? 0 : X.slide_wc,
                                                    X.slide_min, X.P, X.out, X.err, X.cells);
    return cudaGetLastError();
}

template <bool W32>
cudaError_t launch_first_lanes(const ExtLongLaunch &X, int nsm)
{
    if (X.lanes == 8) return launch_first<W32, 8>(X, nsm);
    if (X.lanes == 16) return launch_first<W32, 16>(X, nsm);
    return launch_first<W32, 32>(X, nsm);
}

template <bool W32>
cudaError_t launch_deferred(const ExtLongLaunch &X, const uint32_t *dbounds, uint32_t *dcounter, int nsm)
{
    constexpr int R = W32 ? xl::RING_MAX_32 : xl::RING_MAX_16;
    auto kern = xl::ext_long_kernel<W32, 32, XL_C>;
    const size_t smem = (size_t)xl::ring_words(R, W32) * 4;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)EXT_SMEM_BLOCK_MAX);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32, smem)) != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidValue;
    kern<<<per_sm * nsm, 32, smem, X.stream>>>(X.seq, X.jobs, X.defer, dbounds, dcounter, X.njobs, 0, R, nullptr,
                                              nullptr, 0, 0u, X.P, X.out, X.err, X.cells);
    return cudaGetLastError();
}

}  // namespace

cudaError_t ext_long_launch(const ExtLongLaunch &X, bool w32, int nsm)
{
    if (w32) return launch_first_lanes<true>(X, nsm);
    // the window kernel first (it exits at once when the bucket is below slide_min jobs); the
    // group kernel then runs the jobs it left
    if (X.slide_wc > 0) {
        const cudaError_t e = ext_slide_launch(X, nsm);
        if (e != cudaSuccess) return e;
    }
    return launch_first_lanes<false>(X, nsm);
}

cudaError_t ext_long_deferred_launch(const ExtLongLaunch &X, bool w32, uint32_t *work, int nsm)
{
    // work[0] = 0 and work[1] = the deferred count are the deferred launch's [start, stop)
    return w32 ? launch_deferred<true>(X, work, work + XL_WORK_DCOUNTER32, nsm)
               : launch_deferred<false>(X, work, work + XL_WORK_DCOUNTER16, nsm);
}

int ext_long_ring_for_band(int w)
{
    long long need = 2LL * (w < 0 ? 0 : w) + 3;
    int r = XL_RING_MIN;
    while (r < need && r < XL_RING_FIRST_MAX) r <<= 1;
    return r;
}

}  // namespace bwacuda
