// ext_persist.cuh -- the persistent bucket kernels of the batched extension
// path (ext_persist.cu has the sort, the buckets and the overview).  Warps pull
// 32 * GRAB consecutive sorted jobs per grab from the bucket's work counter;
// GRAB (1, 2 or 4, picked by the autotuner) is a template parameter so each
// value compiles to its own straight-line loop; ext_persist_g{1,2,4}.cu
// instantiate one value each (separate translation units build in parallel).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "ext_job.cuh"
#include "kernels.h"
#include "persist.h"

namespace bwacuda {
namespace persist {

template <class F, int TB, int GRAB>
__global__ void __launch_bounds__(TB)
ext_persist_kernel(const uint8_t *__restrict__ seq, const bwacuda_dev_ext_job *__restrict__ jobs,
                   const uint32_t *__restrict__ order, uint32_t *__restrict__ table,
                   const __grid_constant__ ExtParams P, int qcap, bwacuda_ext_result *__restrict__ out,
                   uint32_t *__restrict__ err, unsigned long long *__restrict__ cells_total)
{
    using CellT = typename F::T;
    constexpr bool WIDE = sizeof(CellT) == 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x, lane = tid & 31;
    CellT *cell = reinterpret_cast<CellT *>(smem_raw) + tid;
    uint32_t *qw = reinterpret_cast<uint32_t *>(reinterpret_cast<CellT *>(smem_raw) + (size_t)qcap * TB) + tid;
    const uint32_t start = table[0], stop = table[1];
    uint32_t *counter = table + 2;
    unsigned long long ncells = 0;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(counter, 32u * (uint32_t)GRAB);
        base = __shfl_sync(0xffffffffu, base, 0) + start;
        if (base >= stop) break;
#pragma unroll
        for (int g = 0; g < GRAB; ++g) {
        const uint32_t k = base + 32u * (uint32_t)g + lane;
        if (k < stop) {
            const uint32_t jid = order[k];
            const bwacuda_dev_ext_job J = jobs[jid];
            const bool fits = WIDE || ext_fits_i16(J.qlen, J.tlen, J.h0, P.sc.max_sc);
            if (J.qlen < 0 || J.qlen + 1 > qcap || !fits) {
                atomicOr(err, ERR_RANGE);
            } else {
                bool bad = false;
                const bwacuda_ext_result r = ext_run_job<F, TB>(cell, qw, seq, J, P, bad, ncells);
                if (bad) atomicOr(err, ERR_BASE);
                out[jid] = r;
            }
        }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ncells += __shfl_xor_sync(0xffffffffu, ncells, o);
    if (lane == 0 && ncells) atomicAdd(cells_total, ncells);
}

// The same persistent loop over pair cells: 8-bit (W16 false, jobs of the 8-bit
// class) or 16-bit (W16 true, jobs of the 16-bit class).
template <int TB, int GRAB, bool W16>
__global__ void __launch_bounds__(TB)
ext_persist_pair_kernel(const uint8_t *__restrict__ seq, const bwacuda_dev_ext_job *__restrict__ jobs,
                        const uint32_t *__restrict__ order, uint32_t *__restrict__ table,
                        const __grid_constant__ ExtParams P, int qcap, bwacuda_ext_result *__restrict__ out,
                        uint32_t *__restrict__ err, unsigned long long *__restrict__ cells_total)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x, lane = tid & 31;
    const size_t cpairs = (size_t)qcap / 2 + 2;
    uint32_t *cellw = reinterpret_cast<uint32_t *>(smem_raw) + tid;
    uint2 *cell2 = reinterpret_cast<uint2 *>(smem_raw) + tid;
    uint32_t *qw = reinterpret_cast<uint32_t *>(smem_raw) + cpairs * (W16 ? 2 : 1) * TB + tid;
    const uint32_t start = table[0], stop = table[1];
    uint32_t *counter = table + 2;
    const bool sym = P.sc.o_del + P.sc.e_del == P.sc.o_ins + P.sc.e_ins;
    unsigned long long ncells = 0;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(counter, 32u * (uint32_t)GRAB);
        base = __shfl_sync(0xffffffffu, base, 0) + start;
        if (base >= stop) break;
#pragma unroll
        for (int g = 0; g < GRAB; ++g) {
        const uint32_t k = base + 32u * (uint32_t)g + lane;
        if (k < stop) {
            const uint32_t jid = order[k];
            const bwacuda_dev_ext_job J = jobs[jid];
            const bool fits = W16 ? ext_fits_i16(J.qlen, J.tlen, J.h0, P.sc.max_sc)
                                  : ext_fits_u8(J.qlen, J.tlen, J.h0, P.sc.max_sc);
            if (J.qlen < 0 || J.qlen + 1 > qcap || !fits) {
                atomicOr(err, ERR_RANGE);
            } else {
                bool bad = false;
                // 8-bit rows of at most 512 columns keep their row maxima in 16-bit lanes;
                // equal open+extend costs share one gap-open lane
                bwacuda_ext_result r;
                if (W16)
                    r = sym ? ext_run_job_i16p<TB, true>(cell2, qw, seq, J, P, bad, ncells)
                            : ext_run_job_i16p<TB, false>(cell2, qw, seq, J, P, bad, ncells);
                else if (qcap <= 513)
                    r = sym ? ext_run_job_u8p<TB, true, true>(cellw, qw, seq, J, P, bad, ncells)
                            : ext_run_job_u8p<TB, true, false>(cellw, qw, seq, J, P, bad, ncells);
                else
                    r = sym ? ext_run_job_u8p<TB, false, true>(cellw, qw, seq, J, P, bad, ncells)
                            : ext_run_job_u8p<TB, false, false>(cellw, qw, seq, J, P, bad, ncells);
                if (bad) atomicOr(err, ERR_BASE);
                out[jid] = r;
            }
        }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ncells += __shfl_xor_sync(0xffffffffu, ncells, o);
    if (lane == 0 && ncells) atomicAdd(cells_total, ncells);
}

constexpr size_t SMEM_MAX = EXT_SMEM_BLOCK_MAX;

// Resident blocks per SM of a persistent launch: the occupancy limit, lowered so
// that L.reserve_regs registers and L.reserve_threads threads stay free (at least
// one block).  Registers are allocated per warp in steps of 256.
template <class K>
cudaError_t persist_blocks_per_sm(K kern, int tb, size_t smem, const PersistLaunch &L, int &per_sm)
{
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, tb, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidValue;
    if (L.reserve_regs > 0 || L.reserve_threads > 0) {
        cudaFuncAttributes fa;
        if ((e = cudaFuncGetAttributes(&fa, kern)) != cudaSuccess) return e;
        const int regs_block = ((fa.numRegs * 32 + 255) / 256) * 256 * (tb / 32);
        const int cap_r = regs_block > 0 ? (L.sm_regs - L.reserve_regs) / regs_block : per_sm;
        const int cap_t = (L.sm_threads - L.reserve_threads) / tb;
        per_sm = std::max(1, std::min(per_sm, std::min(cap_r, cap_t)));
    }
    return cudaSuccess;
}

template <class F, int TB, int GRAB>
cudaError_t launch_persist_tb(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *table, int nsm)
{
    const size_t smem = ext_block_smem(d.qcap, TB, sizeof(typename F::T));
    if (smem > SMEM_MAX) return cudaErrorInvalidValue;
    auto kern = ext_persist_kernel<F, TB, GRAB>;
    // process-wide per kernel: always the ceiling, so a launch on another context (another
    // host thread) never shrinks it under this one
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_MAX);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    if ((e = persist_blocks_per_sm(kern, TB, smem, L, per_sm)) != cudaSuccess) return e;
    const int grid = per_sm * nsm;
    kern<<<grid, TB, smem, L.stream>>>(L.seq, L.jobs, L.order, table, L.P, d.qcap, L.out, L.err, L.cells);
    return cudaGetLastError();
}

__host__ __device__ inline size_t pair_block_smem(int qcap, int tb, bool w16)
{
    return w16 ? ext_block_smem_i16p(qcap, tb) : ext_block_smem_u8p(qcap, tb);
}

template <int TB, int GRAB, bool W16>
cudaError_t launch_persist_pair_tb(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *table, int nsm)
{
    const size_t smem = pair_block_smem(d.qcap, TB, W16);
    if (smem > SMEM_MAX) return cudaErrorInvalidValue;
    auto kern = ext_persist_pair_kernel<TB, GRAB, W16>;
    // process-wide per kernel: always the ceiling, so a launch on another context (another
    // host thread) never shrinks it under this one
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_MAX);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    if ((e = persist_blocks_per_sm(kern, TB, smem, L, per_sm)) != cudaSuccess) return e;
    kern<<<per_sm * nsm, TB, smem, L.stream>>>(L.seq, L.jobs, L.order, table, L.P, d.qcap, L.out, L.err, L.cells);
    return cudaGetLastError();
}

template <int GRAB, bool W16>
cudaError_t launch_persist_pair(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *table, int nsm, int tb)
{
    if (tb >= 256 && pair_block_smem(d.qcap, 256, W16) <= SMEM_MAX)
        return launch_persist_pair_tb<256, GRAB, W16>(L, d, table, nsm);
    if (tb >= 128 && pair_block_smem(d.qcap, 128, W16) <= SMEM_MAX)
        return launch_persist_pair_tb<128, GRAB, W16>(L, d, table, nsm);
    if (tb >= 64 && pair_block_smem(d.qcap, 64, W16) <= SMEM_MAX)
        return launch_persist_pair_tb<64, GRAB, W16>(L, d, table, nsm);
    return launch_persist_pair_tb<32, GRAB, W16>(L, d, table, nsm);
}

template <class F, int GRAB>
cudaError_t launch_persist(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *table, int nsm, int tb)
{
    const int cb = sizeof(typename F::T);
    // requested block size if it fits, else the largest that does
    if (tb >= 256 && ext_block_smem(d.qcap, 256, cb) <= SMEM_MAX) return launch_persist_tb<F, 256, GRAB>(L, d, table, nsm);
    if (tb >= 128 && ext_block_smem(d.qcap, 128, cb) <= SMEM_MAX) return launch_persist_tb<F, 128, GRAB>(L, d, table, nsm);
    if (tb >= 64 && ext_block_smem(d.qcap, 64, cb) <= SMEM_MAX) return launch_persist_tb<F, 64, GRAB>(L, d, table, nsm);
    return launch_persist_tb<F, 32, GRAB>(L, d, table, nsm);
}

// One bucket's persistent launch with GRAB 32-job rounds per work grab.
template <int GRAB>
cudaError_t ext_persist_launch_grab(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *table, int nsm, int tb)
{
    // the sort keeps the 8-bit class empty when the gap costs do not fit 16-bit lanes
    const bool lanes = ext_pair_lanes_ok(L.P.sc.o_del, L.P.sc.e_del, L.P.sc.o_ins, L.P.sc.e_ins);
    if (d.cls == 0) return launch_persist_pair<GRAB, false>(L, d, table, nsm, tb);
    if (d.cls == 2) return launch_persist<FmtI32, GRAB>(L, d, table, nsm, tb);
    // 16-bit pair cells where one warp's rows fit, else one column per cell
    if (lanes && pair_block_smem(d.qcap, 32, true) <= SMEM_MAX)
        return launch_persist_pair<GRAB, true>(L, d, table, nsm, tb);
    return launch_persist<FmtI16, GRAB>(L, d, table, nsm, tb);
}


}  // namespace persist
}  // namespace bwacuda
