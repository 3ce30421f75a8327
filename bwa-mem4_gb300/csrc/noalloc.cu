// noalloc.cu -- bwacuda_ksw_align2_device_noalloc: the device-resident mate
// rescue for callers that must not allocate GPU memory.
//
// Some callers cannot call cudaMalloc: a process whose device memory is owned
// by a pool allocator that reserved the whole budget up front, or a loop on a
// latency-critical stream where cudaMalloc / cudaFree would synchronise the
// device and stall other work.  This entry point runs the same kernels as
// bwacuda_ksw_align2_device, but the one piece of scratch memory they need (the
// suboptimal-tracker entries of every job, and the per-job offsets into them)
// lives in a statically sized __device__ array defined in this file.  Every GPU
// that loads the library holds that array until the process exits.
//
// Limits: NOALLOC_ENTRIES tracker entries of 8 bytes (128 MiB) and
// NOALLOC_JOBS jobs (4 MiB of offsets) per call.  A call needs
// n * (max_tlen / 2 + 2) entries; larger calls are rejected with
// BWACUDA_EUNSUPPORTED before anything is launched.
//
// The array is shared by all calls on a device, and it keeps the previous call's
// contents.  The error word and the length maxima are cleared at the start of
// every call; tracker entries are always written before they are read.  A call
// returns only after its kernels finish, and calls from several host threads
// (on one context or several) take a process-wide lock for their whole length,
// so they never overlap on the array.
//
// The first call on a device looks the array up with cudaGetSymbolAddress,
// which needs that device to be current; make that first call before any
// stream capture.  Every call synchronises its stream before it returns, on
// error paths too once a kernel may have been launched.
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"

namespace bwacuda {

namespace {

constexpr size_t NOALLOC_ENTRIES = (size_t)16 << 20;  // 16 Mi entries x 8 B = 128 MiB
constexpr size_t NOALLOC_JOBS = (size_t)512 << 10;    // 512 Ki jobs x 8 B offsets = 4 MiB
constexpr int NOALLOC_MAX_DEVICES = 64;

// [0] error flags, [1] max qlen, [2] max tlen, [3] count of jobs with a negative length
struct NoallocStatus {
    uint32_t err;
    int32_t max_qlen, max_tlen;
    uint32_t bad_len;
};

static __device__ __align__(256) uint2 g_noalloc_entries[NOALLOC_ENTRIES];
static __device__ __align__(256) uint64_t g_noalloc_offsets[NOALLOC_JOBS];
static __device__ __align__(256) NoallocStatus g_noalloc_status;

struct NoallocPtrs {
    bool ready = false;
    uint2 *entries = nullptr;
    uint64_t *offsets = nullptr;
    NoallocStatus *status = nullptr;
};

std::mutex g_noalloc_mu;
NoallocPtrs g_noalloc_ptrs[NOALLOC_MAX_DEVICES];

// Device addresses of the static arrays on `device` (which must be current).
int noalloc_setup(int device, NoallocPtrs *out)
{
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) return BWACUDA_EUNSUPPORTED;
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    NoallocPtrs &p = g_noalloc_ptrs[device];
    if (!p.ready) {
        cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void **>(&p.entries), g_noalloc_entries);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(reinterpret_cast<void **>(&p.offsets), g_noalloc_offsets);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(reinterpret_cast<void **>(&p.status), g_noalloc_status);
        if (e != cudaSuccess) return cuda_status(e);
        p.ready = true;
    }
    *out = p;
    return BWACUDA_OK;
}

__global__ void noalloc_scan_kernel(const bwacuda_dev_rescue_job *__restrict__ jobs, uint32_t n,
                                    NoallocStatus *__restrict__ st)
{
    int mq = 0, mt = 0;
    uint32_t bad = 0;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int q = jobs[k].qlen, t = jobs[k].tlen;
        bad += (q < 0 || t < 0);
        mq = max(mq, q);
        mt = max(mt, t);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mq = max(mq, __shfl_xor_sync(0xffffffffu, mq, o));
        mt = max(mt, __shfl_xor_sync(0xffffffffu, mt, o));
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&st->max_qlen, mq);
        atomicMax(&st->max_tlen, mt);
        if (bad) atomicAdd(&st->bad_len, bad);
    }
}

// Every job gets a fixed stride of tracker entries, sized for the longest target.
__global__ void noalloc_offsets_kernel(uint64_t *__restrict__ off, uint32_t n, uint64_t stride)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        off[k] = (uint64_t)k * stride;
}

int read_status(const NoallocPtrs &p, cudaStream_t s, NoallocStatus *h)
{
    cudaError_t e = cudaMemcpyAsync(h, p.status, sizeof(NoallocStatus), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return cuda_status(e);
}

// Waits for the call's stream on every return once a kernel may be in flight, so no kernel of
// this call still writes the static arrays after the process-wide lock is released.
struct StreamDrain {
    cudaStream_t s;
    bool armed = false;
    ~StreamDrain()
    {
        if (armed) cudaStreamSynchronize(s);
    }
};

}  // namespace

}  // namespace bwacuda

using namespace bwacuda;

extern "C" int bwacuda_ksw_align2_device_noalloc(bwacuda_ctx *c, const uint8_t *d_seq,
                                                 const bwacuda_dev_rescue_job *d_jobs, size_t n,
                                                 const bwacuda_scoring *scp, int minsc, int max_sc, int mode,
                                                 int lanes, bwacuda_rescue_result *d_out, void *stream)
{
    if (!c || !scp) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    static std::mutex array_mu;  // the static arrays are shared by every context of the process
    std::lock_guard<std::mutex> ga(array_mu);
    int rc = validate_scoring(scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
    if (rc) return rc;
    if (max_sc < 1 || (mode != 0 && mode != 1) || (lanes != 0 && lanes != 8 && lanes != 16)) return BWACUDA_EINVAL;
    if (n == 0) return BWACUDA_OK;
    if (!d_seq || !d_jobs || !d_out) return BWACUDA_EINVAL;
    if (n > NOALLOC_JOBS) return BWACUDA_EUNSUPPORTED;
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    NoallocPtrs p;
    if ((rc = noalloc_setup(c->device, &p)) != BWACUDA_OK) return rc;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    StreamDrain drain{s};  // declared after the locks: runs before they are released

    // clear the status block, then find the longest query and target
    cudaError_t e = cudaMemsetAsync(p.status, 0, sizeof(NoallocStatus), s);
    if (e != cudaSuccess) return cuda_status(e);
    drain.armed = true;
    uint32_t grid = (uint32_t)((n + 255) / 256);
    if (grid > 1024) grid = 1024;
    noalloc_scan_kernel<<<grid, 256, 0, s>>>(d_jobs, (uint32_t)n, p.status);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
    NoallocStatus h;
    if ((rc = read_status(p, s, &h)) != BWACUDA_OK) return rc;
    if (h.bad_len) return BWACUDA_EINVAL;
    const uint64_t stride = rescue_scratch_entries(h.max_tlen);
    if ((uint64_t)n * stride > NOALLOC_ENTRIES) return BWACUDA_EUNSUPPORTED;
    const int qcap = (h.max_qlen + 15) / 16 * 16 + 16;
    const bool wide_fits = (size_t)qcap <= rescue_tpj_smem_limit_qcap(true);
    if ((size_t)qcap > rescue_tpj_smem_limit_qcap(false)) return BWACUDA_EUNSUPPORTED;

    noalloc_offsets_kernel<<<grid, 256, 0, s>>>(p.offsets, (uint32_t)n, stride);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);

    RescueLaunch L;
    L.seq = d_seq;
    L.jobs = d_jobs;
    L.order = nullptr;
    L.count_ptr = nullptr;
    L.n = n;
    L.sc = make_scoring(scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
    L.sc.max_sc = max_sc;
    L.mode = mode;
    L.lanes = lanes;
    L.minsc = minsc;
    L.qcap = qcap;
    L.only_wide = wide_fits ? 0 : 2;
    L.scratch = p.entries;
    L.scratch_off = p.offsets;
    L.out_aln = d_out;
    L.out_fwd = nullptr;
    L.err = &p.status->err;
    L.stream = s;
    if ((e = rescue_narrow_launch(c, L)) != cudaSuccess) return cuda_status(e);
    c->stats.kernel_launches += 3;
    if (wide_fits) {
        L.only_wide = 1;
        if ((e = rescue_tpj_launch(L, true)) != cudaSuccess) return cuda_status(e);
        c->stats.kernel_launches += 1;
    }
    c->stats.rescue_jobs += n;
    if ((rc = read_status(p, s, &h)) != BWACUDA_OK) return rc;
    if (h.err & ERR_BASE) return BWACUDA_EBASE;
    if (h.err & (ERR_RANGE | ERR_SCRATCH)) return BWACUDA_EUNSUPPORTED;
    return BWACUDA_OK;
}
