// extend_tpj.cu -- the plain extension launch: one thread per job, jobs in
// caller order, one launch per chunk.  The per-job routine is ext_run_job
// (ext_job.cuh); the persistent bucketed launch in ext_persist.cu shares it.
//
// Work unit (cells): one iteration of the inner column loop, i.e. the sum over
// processed rows of (end - beg), the same count the oracle reports.
#include <cuda_runtime.h>

#include "common.cuh"
#include "ext_job.cuh"
#include "kernels.h"

namespace bwacuda {

namespace {

template <class F, int TB>
__global__ void __launch_bounds__(TB)
ext_tpj_kernel(const uint8_t *__restrict__ seq, const bwacuda_dev_ext_job *__restrict__ jobs,
               const uint32_t *__restrict__ order, const uint32_t *__restrict__ count_ptr, uint32_t n,
               const __grid_constant__ ExtParams P, int qcap, int only_wide, int long_follows,
               bwacuda_ext_result *__restrict__ out, uint32_t *__restrict__ err,
               unsigned long long *__restrict__ cells_total)
{
    constexpr bool WIDE = sizeof(typename F::T) == 8;
    using CellT = typename F::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    CellT *cell = reinterpret_cast<CellT *>(smem_raw) + tid;
    uint32_t *qw = reinterpret_cast<uint32_t *>(reinterpret_cast<CellT *>(smem_raw) + (size_t)qcap * TB) + tid;

    const uint32_t lim = count_ptr ? min(*count_ptr, n) : n;  // a device count never exceeds the launch's n
    const uint32_t k = blockIdx.x * TB + tid;
    bool active = k < lim;
    const uint32_t jid = active ? (order ? order[k] : k) : 0u;
    bwacuda_dev_ext_job J;
    if (active) J = jobs[jid];
    // The narrow launch leaves wide jobs to a wide launch (only_wide == 2: none
    // follows, so they are reported as unsupported); a wide launch with
    // only_wide == 1 skips the jobs the narrow launch handles.
    if (active) {
        const bool narrow = ext_fits_i16(J.qlen, J.tlen, J.h0, P.sc.max_sc);
        if (!WIDE && !narrow) {
            if (only_wide == 2) atomicOr(err, ERR_RANGE);
            active = false;
        } else if (WIDE && only_wide == 1 && narrow) {
            active = false;
        }
    }
    if (active && J.qlen + 1 > qcap && J.qlen >= 0 && long_follows) {
        active = false;  // the group-per-job launch that follows takes it
    } else if (active && (J.qlen < 0 || J.qlen + 1 > qcap)) {
        atomicOr(err, ERR_RANGE);
        active = false;
    }
    unsigned long long ncells = 0;
    if (active) {
        bool bad = false;
        const bwacuda_ext_result r = ext_run_job<F, TB>(cell, qw, seq, J, P, bad, ncells);
        if (bad) atomicOr(err, ERR_BASE);
        out[jid] = r;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ncells += __shfl_xor_sync(0xffffffffu, ncells, o);
    if ((tid & 31) == 0 && ncells) atomicAdd(cells_total, ncells);
}

constexpr size_t SMEM_MAX = EXT_SMEM_BLOCK_MAX;

template <class F, int TB>
cudaError_t launch_ext_tb(const ExtLaunch &L)
{
    const size_t smem = ext_block_smem(L.qcap, TB, sizeof(typename F::T));
    // the attribute is process-wide per kernel: always its ceiling, so calls on other
    // contexts (other host threads) never shrink it under this launch
    cudaError_t e = cudaFuncSetAttribute(ext_tpj_kernel<F, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)SMEM_MAX);
    if (e != cudaSuccess) return e;
    const uint32_t grid = (uint32_t)((L.n + TB - 1) / TB);
    if (grid == 0) return cudaSuccess;
    ext_tpj_kernel<F, TB><<<grid, TB, smem, L.stream>>>(L.seq, L.jobs, L.order, L.count_ptr, (uint32_t)L.n,
                                                       L.P, L.qcap, L.only_wide, L.long_follows, L.out, L.err,
                                                       L.cells);
    return cudaGetLastError();
}

// Largest block (128, 64 or 32 threads) whose shared memory fits.
template <class F>
cudaError_t launch_ext(const ExtLaunch &L)
{
    const int cb = sizeof(typename F::T);
    if (ext_block_smem(L.qcap, 128, cb) <= SMEM_MAX) return launch_ext_tb<F, 128>(L);
    if (ext_block_smem(L.qcap, 64, cb) <= SMEM_MAX) return launch_ext_tb<F, 64>(L);
    if (ext_block_smem(L.qcap, 32, cb) <= SMEM_MAX) return launch_ext_tb<F, 32>(L);
    return cudaErrorInvalidValue;
}

}  // namespace

size_t ext_tpj_smem_limit_qcap(bool wide)
{
    const int cb = wide ? 8 : 4;
    size_t q = SMEM_MAX / (cb * 32 + 8);
    while (q > 0 && ext_block_smem((int)q, 32, cb) > SMEM_MAX) --q;
    return q;
}

cudaError_t ext_tpj_launch(const ExtLaunch &L, bool wide)
{
    return wide ? launch_ext<FmtI32>(L) : launch_ext<FmtI16>(L);
}

}  // namespace bwacuda
