// ats.cu -- host-buffer extension batches gathered by the GPU itself.
//
// On Grace-Blackwell the GPU reads and writes pageable host memory through the
// host's page tables (cudaDevAttrPageableMemoryAccess), over NVLink-C2C.  So
// bwacuda_extend_batch hands the caller's job array to the device as it is:
//   1. a length kernel reads the jobs, validates them and writes per-job sizes
//      (and counts the bwa-mem bin labels for the statistics);
//   2. a device scan turns sizes into HBM offsets;
//   3. a gather kernel copies every query and target slice from host memory
//      into one HBM buffer and writes the device descriptors;
//   4. the batched extension runs (sort, buckets, persistent kernels);
//   5. a scatter kernel stores the results straight into the caller's out[].
// The host only launches.  Chunks alternate between two streams, so the gather
// of chunk k+1 overlaps the extension of chunk k; one 8-byte readback per chunk
// (the byte total) sizes the sequence buffer.
//
// A job is validated before any of its slices is read: a negative length,
// h0 <= 0, or a null pointer with a non-zero length makes the call return
// BWACUDA_EINVAL, and such a job's pointers are never dereferenced.  Pointers
// that are neither null nor valid are the caller's contract, exactly as for the
// host-packing path (which would read them with memcpy).
#include <cuda_runtime.h>

#include <algorithm>
#include <new>

#include <cub/device/device_scan.cuh>

#include "kernels.h"
#include "runtime.h"

namespace bwacuda {

namespace {

constexpr uint32_t ERR_INPUT = 8u;
constexpr size_t ATS_MAX_CHUNK = size_t(1) << 24;  // 32-bit word indexing in the scatter
constexpr int ATS_FLAG_BYTES = 32;                 // u32 input flag, pad, u64 bins[3]
// Blocks per SM of the pipeline's length / gather / scatter launches.  They run
// beside the previous chunk's persistent DP kernels; a full-occupancy grid would
// crowd those off the SMs, while two blocks per SM with eight 16-byte loads in
// flight per lane already keep several MB of host reads outstanding.
constexpr int ATS_BLOCKS_PER_SM = 2;

__device__ __forceinline__ bool job_ok(const bwacuda_ext_job &J)
{
    return J.qlen >= 0 && J.tlen >= 0 && J.h0 > 0 && (J.qlen == 0 || J.query != nullptr) &&
           (J.tlen == 0 || J.target != nullptr);
}

// Slices are copied as whole aligned 16-byte words (slice_words, common.cuh):
// a slice of len bytes at host address src covers words [src >> 4,
// (src + len - 1) >> 4] and lands at a 16-byte aligned HBM base plus
// (src & 15), so every word maps to one aligned word of HBM.  The bytes of a
// covering word outside the slice lie in the same page as bytes of the slice,
// so the widened reads touch only mapped memory; in HBM they land in the
// slice's own reserve.
__global__ void ats_lengths_kernel(const bwacuda_ext_job *__restrict__ hjobs, uint32_t n, BinRule br,
                                   uint64_t *__restrict__ sizes, uint32_t *__restrict__ flags)
{
    uint32_t bad = 0, bins[3] = {0, 0, 0};
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const bwacuda_ext_job J = hjobs[k];
        const bool ok = job_ok(J);
        bad |= !ok;
        if (ok) bins[bin_label(br, J.qlen, J.tlen, J.h0)]++;
        // reserve, in bytes (a multiple of 16, so every job's base stays aligned)
        sizes[k] = ok ? 16ull * (slice_words(J.query, J.qlen) + slice_words(J.target, J.tlen)) : 0u;
    }
    // every thread of the warp reaches this point
    bad = __reduce_or_sync(0xffffffffu, bad);
    const uint32_t b0 = __reduce_add_sync(0xffffffffu, bins[0]);
    const uint32_t b1 = __reduce_add_sync(0xffffffffu, bins[1]);
    const uint32_t b2 = __reduce_add_sync(0xffffffffu, bins[2]);
    if ((threadIdx.x & 31) == 0) {
        if (bad) atomicOr(flags, ERR_INPUT);
        unsigned long long *cnt = reinterpret_cast<unsigned long long *>(flags + 2);
        if (b0) atomicAdd(cnt + 0, (unsigned long long)b0);
        if (b1) atomicAdd(cnt + 1, (unsigned long long)b1);
        if (b2) atomicAdd(cnt + 2, (unsigned long long)b2);
    }
}

// A warp takes 32 consecutive jobs: lane i loads job i's descriptor (one
// coalesced read of the caller's array) and writes its device descriptor; then
// the warp copies all 32 jobs' words as one flat list (warp_gather_slices).  An
// invalid job becomes an empty one (qlen = tlen = 0, h0 = 1); the call then fails.
__global__ void __launch_bounds__(256) ats_gather_kernel(const bwacuda_ext_job *__restrict__ hjobs, uint32_t n,
                                                         const uint64_t *__restrict__ offs, int w,
                                                         uint8_t *__restrict__ seq,
                                                         bwacuda_dev_ext_job *__restrict__ djobs)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t k0 = warp * 32; k0 < n; k0 += nwarps * 32) {
        const uint32_t k = k0 + lane;
        uint64_t qa = 0, ta = 0, base = 0;
        uint32_t qw = 0, tw = 0;
        if (k < n) {
            const bwacuda_ext_job J = hjobs[k];
            const bool ok = job_ok(J);
            base = offs[k];
            qa = reinterpret_cast<uint64_t>(J.query);
            ta = reinterpret_cast<uint64_t>(J.target);
            qw = ok ? slice_words(J.query, J.qlen) : 0u;
            tw = ok ? slice_words(J.target, J.tlen) : 0u;
            bwacuda_dev_ext_job D;
            D.q_off = base + (qa & 15);
            D.t_off = base + 16ull * qw + (ta & 15);
            D.qlen = ok ? J.qlen : 0;
            D.tlen = ok ? J.tlen : 0;
            D.h0 = ok ? J.h0 : 1;
            D.w = w;
            djobs[k] = D;
        }
        warp_gather_slices(qa & ~15ull, ta & ~15ull, base, qw, tw, seq);
    }
}

// Results to the caller's array, word by word so consecutive threads write
// consecutive host addresses.
__global__ void ats_scatter_kernel(const uint32_t *__restrict__ src, uint32_t words, uint32_t *__restrict__ dst)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < words; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

struct AtsSlot {
    DevBuf sizes, offs, scan_tmp, seq, djobs, dout, flags;
    HostBuf h_total, h_flags;
    cudaEvent_t gathered = nullptr;  // this slot's last gather finished
    bool busy = false;
};

}  // namespace

struct AtsState {
    AtsSlot slot[2];
};

void ats_release(bwacuda_ctx *c)
{
    if (!c->ats) return;
    for (auto &s : c->ats->slot) {
        s.sizes.release(); s.offs.release(); s.scan_tmp.release(); s.seq.release();
        s.djobs.release(); s.dout.release(); s.flags.release();
        s.h_total.release(); s.h_flags.release();
        if (s.gathered) cudaEventDestroy(s.gathered);
    }
    delete c->ats;
    c->ats = nullptr;
}

namespace {

// Wait for a slot's chunk and fold its input flag and bin counts in.
int ats_drain(bwacuda_ctx *c, int si, uint32_t *input_flags)
{
    AtsSlot &S = c->ats->slot[si];
    if (!S.busy) return BWACUDA_OK;
    S.busy = false;
    cudaError_t e = cudaStreamSynchronize(c->slot[si].stream);
    if (e != cudaSuccess) return cuda_status(e);
    const uint32_t *f = static_cast<const uint32_t *>(S.h_flags.p);
    const uint64_t *bins = reinterpret_cast<const uint64_t *>(f + 2);
    *input_flags |= f[0];
    c->stats.ext_bin_u8 += bins[0];
    c->stats.ext_bin_i16 += bins[1];
    c->stats.ext_bin_i32 += bins[2];
    return BWACUDA_OK;
}

cudaError_t ats_enqueue_chunk(bwacuda_ctx *c, int si, const bwacuda_ext_job *hj, size_t cn, const BinRule &br,
                              const ExtParams &P, int w, bwacuda_ext_result *hout)
{
    AtsSlot &S = c->ats->slot[si];
    cudaStream_t s = c->slot[si].stream;
    cudaError_t e;
    size_t scan_bytes = 0;
    if ((e = cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (const uint64_t *)nullptr, (uint64_t *)nullptr,
                                           (int)cn + 1)) != cudaSuccess)
        return e;
    if ((e = S.sizes.ensure((cn + 1) * 8)) != cudaSuccess) return e;
    if ((e = S.offs.ensure((cn + 1) * 8)) != cudaSuccess) return e;
    if ((e = S.scan_tmp.ensure(scan_bytes + 16)) != cudaSuccess) return e;
    if ((e = S.djobs.ensure(cn * sizeof(bwacuda_dev_ext_job))) != cudaSuccess) return e;
    if ((e = S.dout.ensure(cn * sizeof(bwacuda_ext_result))) != cudaSuccess) return e;
    if ((e = S.flags.ensure(ATS_FLAG_BYTES)) != cudaSuccess) return e;
    if ((e = S.h_total.ensure(16)) != cudaSuccess) return e;
    if ((e = S.h_flags.ensure(ATS_FLAG_BYTES)) != cudaSuccess) return e;
    uint64_t *sizes = static_cast<uint64_t *>(S.sizes.p), *offs = static_cast<uint64_t *>(S.offs.p);
    uint32_t *flags = static_cast<uint32_t *>(S.flags.p);
    if (!S.gathered && (e = cudaEventCreateWithFlags(&S.gathered, cudaEventDisableTiming)) != cudaSuccess) return e;
    // One chunk reads host memory at a time: the host-memory link is the shared resource,
    // and the chunk whose DP runs next gets all of it.
    AtsSlot &O = c->ats->slot[si ^ 1];
    if (O.busy && O.gathered && (e = cudaStreamWaitEvent(s, O.gathered, 0)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(flags, 0, ATS_FLAG_BYTES, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(sizes + cn, 0, 8, s)) != cudaSuccess) return e;
    const int nsm = batched_nsm(c);
    uint32_t grid = (uint32_t)std::min<size_t>((cn + 255) / 256, (size_t)nsm * ATS_BLOCKS_PER_SM);
    ats_lengths_kernel<<<grid, 256, 0, s>>>(hj, (uint32_t)cn, br, sizes, flags);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cub::DeviceScan::ExclusiveSum(S.scan_tmp.p, scan_bytes, sizes, offs, (int)cn + 1, s)) != cudaSuccess)
        return e;
    // the chunk's byte total sizes the sequence buffer
    if ((e = cudaMemcpyAsync(S.h_total.p, offs + cn, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    const uint64_t total = *static_cast<const uint64_t *>(S.h_total.p);
    if ((e = S.seq.ensure(total + 16)) != cudaSuccess) return e;
    grid = (uint32_t)std::min<size_t>((cn + 255) / 256, (size_t)nsm * ATS_BLOCKS_PER_SM);
    ats_gather_kernel<<<grid, 256, 0, s>>>(hj, (uint32_t)cn, offs, w, static_cast<uint8_t *>(S.seq.p),
                                          static_cast<bwacuda_dev_ext_job *>(S.djobs.p));
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaEventRecord(S.gathered, s)) != cudaSuccess) return e;
    e = batched_enqueue(c, batched_slot_bufs(c, si), static_cast<const uint8_t *>(S.seq.p),
                        static_cast<const bwacuda_dev_ext_job *>(S.djobs.p), cn, P,
                        static_cast<bwacuda_ext_result *>(S.dout.p), s, nullptr, nullptr);
    if (e != cudaSuccess) return e;
    const uint32_t words = (uint32_t)(cn * (sizeof(bwacuda_ext_result) / 4));
    grid = (uint32_t)std::min<size_t>((words + 255) / 256, (size_t)nsm * ATS_BLOCKS_PER_SM);
    ats_scatter_kernel<<<grid, 256, 0, s>>>(static_cast<const uint32_t *>(S.dout.p), words,
                                           reinterpret_cast<uint32_t *>(hout));
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(S.h_flags.p, flags, ATS_FLAG_BYTES, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    S.busy = true;
    c->stats.kernel_launches += 4 + 3 + (uint64_t)batched_bucket_count(c);
    return cudaSuccess;
}

}  // namespace

// Gather n host jobs (caller's array, caller's slices) into seq / djobs on stream s,
// every job with band w; synchronous up to the gather launch.  EINVAL if a job is
// invalid (nothing of it is read).
int ats_gather_ext(bwacuda_ctx *c, const bwacuda_ext_job *hj, size_t n, int w, DevBuf &seq, DevBuf &djobs,
                   DevBuf &tmp, HostBuf &htmp, cudaStream_t s)
{
    if (!c->pageable_access) return BWACUDA_EUNSUPPORTED;
    if (n > ATS_MAX_CHUNK * 16) return BWACUDA_EUNSUPPORTED;
    int rc = batched_prepare(c);
    if (rc) return rc;
    size_t scan_bytes = 0;
    cudaError_t e = cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (const uint64_t *)nullptr, (uint64_t *)nullptr,
                                                  (int)n + 1);
    const size_t flag_at = ((n + 1) * 16 + 255) & ~(size_t)255, scan_at = flag_at + 256;
    if (e == cudaSuccess) e = tmp.ensure(scan_at + scan_bytes + 16);
    if (e == cudaSuccess) e = htmp.ensure(64);
    if (e == cudaSuccess) e = djobs.ensure(n * sizeof(bwacuda_dev_ext_job));
    if (e != cudaSuccess) return cuda_status(e);
    uint64_t *sizes = static_cast<uint64_t *>(tmp.p), *offs = sizes + n + 1;
    uint32_t *flags = reinterpret_cast<uint32_t *>(static_cast<char *>(tmp.p) + flag_at);
    void *scan_tmp = static_cast<char *>(tmp.p) + scan_at;
    if ((e = cudaMemsetAsync(flags, 0, ATS_FLAG_BYTES, s)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaMemsetAsync(sizes + n, 0, 8, s)) != cudaSuccess) return cuda_status(e);
    const int nsm = batched_nsm(c);
    const uint32_t grid = (uint32_t)std::min<size_t>((n + 255) / 256, (size_t)nsm * 8);
    BinRule br{0, 0, 0};
    ats_lengths_kernel<<<grid, 256, 0, s>>>(hj, (uint32_t)n, br, sizes, flags);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
    if ((e = cub::DeviceScan::ExclusiveSum(scan_tmp, scan_bytes, sizes, offs, (int)n + 1, s)) != cudaSuccess)
        return cuda_status(e);
    uint64_t *h = static_cast<uint64_t *>(htmp.p);
    if ((e = cudaMemcpyAsync(h, offs + n, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaMemcpyAsync(h + 1, flags, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e);
    if (static_cast<uint32_t>(h[1]) & ERR_INPUT) return BWACUDA_EINVAL;
    if ((e = seq.ensure(h[0] + 16)) != cudaSuccess) return cuda_status(e);
    ats_gather_kernel<<<grid, 256, 0, s>>>(hj, (uint32_t)n, offs, w, static_cast<uint8_t *>(seq.p),
                                          static_cast<bwacuda_dev_ext_job *>(djobs.p));
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
    c->stats.kernel_launches += 4;
    return BWACUDA_OK;
}

// extend_batch with the device doing the gather; validated arguments, n > 0.
int extend_batch_ats(bwacuda_ctx *c, const bwacuda_ext_job *jobs, size_t n, int m, const int8_t *mat,
                     const ExtParams &P, int w, bwacuda_ext_result *out)
{
    if (!c->pageable_access) return BWACUDA_EUNSUPPORTED;
    int rc = batched_prepare(c);
    if (rc) return rc;
    if (!c->ats) {
        c->ats = new (std::nothrow) AtsState();
        if (!c->ats) return BWACUDA_ENOMEM;
    }
    const BinRule br = bin_rule(m, mat);
    const size_t CH = std::min(c->chunk_jobs, ATS_MAX_CHUNK);
    uint32_t input_flags = 0;
    int si = 0;
    for (size_t c0 = 0, cn = 0; c0 < n && rc == BWACUDA_OK; c0 += cn) {
        // a short first chunk: the DP starts after a short gather, later gathers hide behind it
        cn = std::min(c0 == 0 ? std::max(CH / 8, std::min(CH, (size_t)65536)) : CH, n - c0);
        if ((rc = ats_drain(c, si, &input_flags)) != BWACUDA_OK) break;
        cudaError_t e = ats_enqueue_chunk(c, si, jobs + c0, cn, br, P, w, out + c0);
        if (e != cudaSuccess) rc = cuda_status(e);
        si ^= 1;
    }
    const int rc0 = ats_drain(c, 0, &input_flags);
    const int rc1 = ats_drain(c, 1, &input_flags);
    if (!rc) rc = rc0 ? rc0 : rc1;
    uint64_t cells = 0;
    const int st = collect_device_status(c, c->slot[0].stream, &cells);
    if (!rc && (input_flags & ERR_INPUT)) rc = BWACUDA_EINVAL;
    if (!rc) rc = st;
    c->stats.ext_jobs += n;
    c->stats.ext_cells += cells;
    return rc;
}

}  // namespace bwacuda
