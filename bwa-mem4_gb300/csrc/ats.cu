// ats.cu -- host-buffer extension batches gathered by the GPU itself.
//
// On Grace-Blackwell the GPU reads and writes pageable host memory through the
// host's page tables (cudaDevAttrPageableMemoryAccess), over NVLink-C2C.  So
// bwacuda_extend_batch hands the caller's job array to the device as it is:
//   1. a length kernel reads the jobs (the only read of the job array), validates
//      them, writes per-job sizes and leaves each job in its device descriptor
//      (and counts the bwa-mem bin labels for the statistics);
//   2. a device scan turns sizes into HBM offsets;
//   3. a gather kernel copies every query and target slice from host memory
//      into one HBM buffer and completes the device descriptors;
//   4. the batched extension runs (sort, buckets, persistent kernels);
//   5. a scatter kernel stores the results straight into the caller's out[].
// The host only launches.  Steps 1-2 of chunk k+1 run on a plan stream while
// chunk k's gather (step 3) runs on the high-priority gather stream, so the
// gathers follow one another on the host link (the shared resource); steps 4-5
// run on two alternating extension streams, each chunk's extension waiting only
// for its own gather.  A ring of ATS_RING chunk
// buffers lets the gathers run ahead of the extensions; one 8-byte readback per
// chunk (its byte total) sizes the chunk's sequence buffer.  While a chunk is in
// flight the persistent bucket kernels leave one small block's worth of registers
// and threads free on every SM, so the next chunk's length and gather blocks
// start at once instead of waiting for a bucket to drain.
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
// Blocks per SM (of ATS_THREADS threads) of the pipeline's length / gather /
// scatter launches.  They run beside the persistent DP kernels, in the room
// those leave free (ATS_RESERVE_*): one block per SM with eight 16-byte loads in
// flight per lane keeps about 2.4 MB of host reads outstanding, and a second one
// would take room from the extension.
constexpr int ATS_BLOCKS_PER_SM = 1;
constexpr int ATS_THREADS = 128;
// What the persistent kernels leave free per SM while the pipeline runs: one
// ATS_THREADS block at the gather kernel's register bound (64 per thread).
constexpr int ATS_RESERVE_REGS = ATS_THREADS * 64;
constexpr int ATS_RESERVE_THREADS = ATS_THREADS;
constexpr int ATS_RING = 4;  // chunk buffers in flight

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
// The lengths kernel is the only reader of the caller's job array: it leaves each job's fields in
// its device descriptor (the slice addresses, for now, in q_off / t_off; an invalid job empty)
// for the gather, so the array crosses the host link once.
__global__ void __launch_bounds__(ATS_THREADS) ats_lengths_kernel(const bwacuda_ext_job *__restrict__ hjobs,
                                                                  uint32_t n, BinRule br,
                                   uint64_t *__restrict__ sizes, uint32_t *__restrict__ flags,
                                   bwacuda_dev_ext_job *__restrict__ djobs)
{
    uint32_t bad = 0, bins[3] = {0, 0, 0};
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const bwacuda_ext_job J = hjobs[k];
        const bool ok = job_ok(J);
        bad |= !ok;
        if (ok) bins[bin_label(br, J.qlen, J.tlen, J.h0)]++;
        // reserve, in bytes (a multiple of 16, so every job's base stays aligned)
        sizes[k] = ok ? 16ull * (slice_words(J.query, J.qlen) + slice_words(J.target, J.tlen)) : 0u;
        bwacuda_dev_ext_job D;
        D.q_off = reinterpret_cast<uint64_t>(J.query);
        D.t_off = reinterpret_cast<uint64_t>(J.target);
        D.qlen = ok ? J.qlen : 0;
        D.tlen = ok ? J.tlen : 0;
        D.h0 = ok ? J.h0 : 1;
        D.w = 0;
        djobs[k] = D;
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

// A warp takes 32 consecutive jobs: lane i reads job i's fields from the descriptor the lengths
// kernel left (HBM) and completes it with the job's offsets in the sequence buffer; then the warp
// copies all 32 jobs' words as one flat list (warp_gather_slices).  An invalid job is an empty one
// (qlen = tlen = 0, h0 = 1); the call then fails.
__global__ void __launch_bounds__(ATS_THREADS, 8) ats_gather_kernel(uint32_t n, const uint64_t *__restrict__ offs,
                                                                    int w, uint8_t *__restrict__ seq,
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
            bwacuda_dev_ext_job D = djobs[k];
            base = offs[k];
            qa = D.q_off;  // the slice addresses, as the lengths kernel left them
            ta = D.t_off;
            qw = slice_words(reinterpret_cast<const uint8_t *>(qa), D.qlen);
            tw = slice_words(reinterpret_cast<const uint8_t *>(ta), D.tlen);
            D.q_off = base + (qa & 15);
            D.t_off = base + 16ull * qw + (ta & 15);
            D.w = w;
            djobs[k] = D;
        }
        warp_gather_slices(qa & ~15ull, ta & ~15ull, base, qw, tw, seq);
    }
}

// Results to the caller's array, word by word so consecutive threads write
// consecutive host addresses.
__global__ void __launch_bounds__(ATS_THREADS) ats_scatter_kernel(const uint32_t *__restrict__ src, uint32_t words,
                                                                  uint32_t *__restrict__ dst)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < words; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

struct AtsChunk {
    DevBuf sizes, offs, scan_tmp, seq, djobs, dout, flags;
    HostBuf h_total, h_flags;
    cudaEvent_t planned = nullptr;   // lengths, offsets and the byte total are in (plan stream)
    cudaEvent_t gathered = nullptr;  // sequence buffer and descriptors are in HBM
    cudaEvent_t done = nullptr;      // results stored, flags read back
    bool busy = false;
};

}  // namespace

struct AtsState {
    AtsChunk ring[ATS_RING];
    cudaStream_t gstream = nullptr;  // gathers (highest priority)
    cudaStream_t pstream = nullptr;  // the next chunk's lengths and offsets, beside the current gather
};

void ats_release(bwacuda_ctx *c)
{
    if (!c->ats) return;
    if (c->ats->gstream) cudaStreamSynchronize(c->ats->gstream);
    if (c->ats->pstream) cudaStreamSynchronize(c->ats->pstream);
    for (auto &r : c->ats->ring) {
        if (r.done) cudaEventSynchronize(r.done);
        r.sizes.release(); r.offs.release(); r.scan_tmp.release(); r.seq.release();
        r.djobs.release(); r.dout.release(); r.flags.release();
        r.h_total.release(); r.h_flags.release();
        if (r.planned) cudaEventDestroy(r.planned);
        if (r.gathered) cudaEventDestroy(r.gathered);
        if (r.done) cudaEventDestroy(r.done);
    }
    if (c->ats->gstream) cudaStreamDestroy(c->ats->gstream);
    if (c->ats->pstream) cudaStreamDestroy(c->ats->pstream);
    delete c->ats;
    c->ats = nullptr;
}

namespace {

int ats_init(bwacuda_ctx *c)
{
    if (c->ats) return BWACUDA_OK;
    AtsState *A = new (std::nothrow) AtsState();
    if (!A) return BWACUDA_ENOMEM;
    int lo_prio = 0, hi_prio = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&A->gstream, cudaStreamNonBlocking, hi_prio);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&A->pstream, cudaStreamNonBlocking, hi_prio);
    for (auto &r : A->ring) {
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r.planned, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r.gathered, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r.done, cudaEventDisableTiming);
    }
    // These kernels use no shared memory, but an SM takes the shared-memory carveout of the
    // first kernel placed on it while empty: with the default (small shared memory) an SM
    // that one gather block lands on cannot take the bucket kernels' blocks until it leaves.
    if (e == cudaSuccess) e = cudaFuncSetAttribute(ats_lengths_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                   cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(ats_gather_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                   cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(ats_scatter_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                   cudaSharedmemCarveoutMaxShared);
    c->ats = A;
    if (e != cudaSuccess) {
        ats_release(c);
        return cuda_status(e);
    }
    return BWACUDA_OK;
}

// Wait for a ring entry's chunk and fold its input flag and bin counts in.
int ats_retire(bwacuda_ctx *c, AtsChunk &R, uint32_t *input_flags)
{
    if (!R.busy) return BWACUDA_OK;
    R.busy = false;
    cudaError_t e = cudaEventSynchronize(R.done);
    if (e != cudaSuccess) return cuda_status(e);
    const uint32_t *f = static_cast<const uint32_t *>(R.h_flags.p);
    const uint64_t *bins = reinterpret_cast<const uint64_t *>(f + 2);
    *input_flags |= f[0];
    c->stats.ext_bin_u8 += bins[0];
    c->stats.ext_bin_i16 += bins[1];
    c->stats.ext_bin_i32 += bins[2];
    return BWACUDA_OK;
}

// Steps 1-2 of a chunk on the plan stream: lengths and validation (the only read of the
// caller's job array: each job lands in its device descriptor), the offset scan, the byte total
// back to the host.  Enqueued while the previous chunk's gather runs.
cudaError_t ats_plan_chunk(bwacuda_ctx *c, AtsChunk &R, const bwacuda_ext_job *hj, size_t cn, const BinRule &br)
{
    cudaStream_t p = c->ats->pstream;
    cudaError_t e;
    size_t scan_bytes = 0;
    if ((e = cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (const uint64_t *)nullptr, (uint64_t *)nullptr,
                                           (int)cn + 1)) != cudaSuccess)
        return e;
    if ((e = R.sizes.ensure((cn + 1) * 8)) != cudaSuccess) return e;
    if ((e = R.offs.ensure((cn + 1) * 8)) != cudaSuccess) return e;
    if ((e = R.scan_tmp.ensure(scan_bytes + 16)) != cudaSuccess) return e;
    if ((e = R.djobs.ensure(cn * sizeof(bwacuda_dev_ext_job))) != cudaSuccess) return e;
    if ((e = R.dout.ensure(cn * sizeof(bwacuda_ext_result))) != cudaSuccess) return e;
    if ((e = R.flags.ensure(ATS_FLAG_BYTES)) != cudaSuccess) return e;
    if ((e = R.h_total.ensure(16)) != cudaSuccess) return e;
    if ((e = R.h_flags.ensure(ATS_FLAG_BYTES)) != cudaSuccess) return e;
    uint64_t *sizes = static_cast<uint64_t *>(R.sizes.p), *offs = static_cast<uint64_t *>(R.offs.p);
    uint32_t *flags = static_cast<uint32_t *>(R.flags.p);
    if ((e = cudaMemsetAsync(flags, 0, ATS_FLAG_BYTES, p)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(sizes + cn, 0, 8, p)) != cudaSuccess) return e;
    const uint32_t grid = (uint32_t)std::min<size_t>((cn + ATS_THREADS - 1) / ATS_THREADS,
                                                     (size_t)batched_nsm(c) * ATS_BLOCKS_PER_SM);
    ats_lengths_kernel<<<grid, ATS_THREADS, 0, p>>>(hj, (uint32_t)cn, br, sizes, flags,
                                                    static_cast<bwacuda_dev_ext_job *>(R.djobs.p));
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cub::DeviceScan::ExclusiveSum(R.scan_tmp.p, scan_bytes, sizes, offs, (int)cn + 1, p)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(R.h_total.p, offs + cn, 8, cudaMemcpyDeviceToHost, p)) != cudaSuccess) return e;
    return cudaEventRecord(R.planned, p);
}

// Step 3 on the gather stream, once the chunk is planned: the host reads the byte total (it
// sizes the sequence buffer), then the gather.
cudaError_t ats_gather_chunk(bwacuda_ctx *c, AtsChunk &R, size_t cn, int w)
{
    cudaStream_t g = c->ats->gstream;
    cudaError_t e;
    if ((e = cudaEventSynchronize(R.planned)) != cudaSuccess) return e;
    const uint64_t total = *static_cast<const uint64_t *>(R.h_total.p);
    if ((e = R.seq.ensure(total + 16)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(g, R.planned, 0)) != cudaSuccess) return e;
    const uint32_t grid = (uint32_t)std::min<size_t>((cn + ATS_THREADS - 1) / ATS_THREADS,
                                                     (size_t)batched_nsm(c) * ATS_BLOCKS_PER_SM);
    ats_gather_kernel<<<grid, ATS_THREADS, 0, g>>>((uint32_t)cn, static_cast<const uint64_t *>(R.offs.p), w,
                                                   static_cast<uint8_t *>(R.seq.p),
                                                   static_cast<bwacuda_dev_ext_job *>(R.djobs.p));
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return cudaEventRecord(R.gathered, g);
}

// Steps 4-5 on extension stream s: the batched extension once the gather is in,
// then the results into the caller's out[] and the flags back to the host.
cudaError_t ats_extend_chunk(bwacuda_ctx *c, AtsChunk &R, int si, size_t cn, const ExtParams &P,
                             bwacuda_ext_result *hout)
{
    cudaStream_t s = c->slot[si].stream;
    cudaError_t e;
    if ((e = cudaStreamWaitEvent(s, R.gathered, 0)) != cudaSuccess) return e;
    BatchBufs *bb = batched_slot_bufs(c, si);
    batched_set_reserve(bb, ATS_RESERVE_REGS, ATS_RESERVE_THREADS);
    e = batched_enqueue(c, bb, static_cast<const uint8_t *>(R.seq.p), static_cast<const bwacuda_dev_ext_job *>(R.djobs.p),
                        cn, P, static_cast<bwacuda_ext_result *>(R.dout.p), s, nullptr, nullptr);
    batched_set_reserve(bb, 0, 0);
    if (e != cudaSuccess) return e;
    const uint32_t words = (uint32_t)(cn * (sizeof(bwacuda_ext_result) / 4));
    const uint32_t grid = (uint32_t)std::min<size_t>((words + ATS_THREADS - 1) / ATS_THREADS,
                                                     (size_t)batched_nsm(c) * ATS_BLOCKS_PER_SM);
    ats_scatter_kernel<<<grid, ATS_THREADS, 0, s>>>(static_cast<const uint32_t *>(R.dout.p), words,
                                                    reinterpret_cast<uint32_t *>(hout));
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(R.h_flags.p, R.flags.p, ATS_FLAG_BYTES, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return e;
    return cudaEventRecord(R.done, s);
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
    const uint32_t grid = (uint32_t)std::min<size_t>((n + ATS_THREADS - 1) / ATS_THREADS, (size_t)nsm * 16);
    BinRule br{0, 0, 0};
    ats_lengths_kernel<<<grid, ATS_THREADS, 0, s>>>(hj, (uint32_t)n, br, sizes, flags,
                                                    static_cast<bwacuda_dev_ext_job *>(djobs.p));
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
    if ((e = cub::DeviceScan::ExclusiveSum(scan_tmp, scan_bytes, sizes, offs, (int)n + 1, s)) != cudaSuccess)
        return cuda_status(e);
    uint64_t *h = static_cast<uint64_t *>(htmp.p);
    if ((e = cudaMemcpyAsync(h, offs + n, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaMemcpyAsync(h + 1, flags, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e);
    if (static_cast<uint32_t>(h[1]) & ERR_INPUT) return BWACUDA_EINVAL;
    if ((e = seq.ensure(h[0] + 16)) != cudaSuccess) return cuda_status(e);
    ats_gather_kernel<<<grid, ATS_THREADS, 0, s>>>((uint32_t)n, offs, w, static_cast<uint8_t *>(seq.p),
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
    if ((rc = ats_init(c)) != BWACUDA_OK) return rc;
    const BinRule br = bin_rule(m, mat);
    const size_t CH = std::min(c->chunk_jobs, ATS_MAX_CHUNK);
    uint32_t input_flags = 0;
    // chunks ramp up from 64k jobs, doubling: the extension starts after a short gather, and each
    // gather (about 2.5x faster than the extension of as many jobs) ends before the extension of
    // the chunks ahead of it.  Chunk k+1 is planned (its lengths and offsets) while chunk k is
    // gathered, so the gathers follow one another on the host link.
    auto chunk_len = [&](size_t k, size_t c0) {
        return std::min(std::min(CH, (size_t)65536 << (k < 16 ? k : 16)), n - c0);
    };
    {
        AtsChunk &R0 = c->ats->ring[0];
        if ((rc = ats_retire(c, R0, &input_flags)) == BWACUDA_OK) {
            const cudaError_t e = ats_plan_chunk(c, R0, jobs, chunk_len(0, 0), br);
            if (e != cudaSuccess) rc = cuda_status(e);
        }
    }
    size_t k = 0;
    for (size_t c0 = 0, cn = 0; c0 < n && rc == BWACUDA_OK; c0 += cn, ++k) {
        cn = chunk_len(k, c0);
        AtsChunk &R = c->ats->ring[k % ATS_RING];
        cudaError_t e = ats_gather_chunk(c, R, cn, w);
        if (e == cudaSuccess) e = ats_extend_chunk(c, R, (int)(k & 1), cn, P, out + c0);
        if (e != cudaSuccess) {
            rc = cuda_status(e);
            break;
        }
        R.busy = true;
        c->stats.kernel_launches += 3 + 3 + (uint64_t)batched_bucket_count(c);
        const size_t c1 = c0 + cn;
        if (c1 < n) {
            AtsChunk &R1 = c->ats->ring[(k + 1) % ATS_RING];
            if ((rc = ats_retire(c, R1, &input_flags)) != BWACUDA_OK) break;
            if ((e = ats_plan_chunk(c, R1, jobs + c1, chunk_len(k + 1, c1), br)) != cudaSuccess) {
                rc = cuda_status(e);
                break;
            }
        }
    }
    for (auto &R : c->ats->ring) {
        const int r2 = ats_retire(c, R, &input_flags);
        if (!rc) rc = r2;
    }
    if (rc != BWACUDA_OK) {  // a failed enqueue may leave work behind on the streams
        cudaStreamSynchronize(c->ats->pstream);
        cudaStreamSynchronize(c->ats->gstream);
        cudaStreamSynchronize(c->slot[0].stream);
        cudaStreamSynchronize(c->slot[1].stream);
    }
    uint64_t cells = 0;
    const int st = collect_device_status(c, c->slot[0].stream, &cells);
    if (!rc && (input_flags & ERR_INPUT)) rc = BWACUDA_EINVAL;
    if (!rc) rc = st;
    c->stats.ext_jobs += n;
    c->stats.ext_cells += cells;
    return rc;
}

}  // namespace bwacuda
