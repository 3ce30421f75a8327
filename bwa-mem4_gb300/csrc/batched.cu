// batched.cu -- host orchestration of the batched extension path: buffers,
// the bucket fan-out over several streams, CUDA-graph capture and replay of the
// whole device sequence, and the host-buffer pipeline that feeds it.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "ext_job.cuh"
#include "kernels.h"
#include "persist.h"
#include "runtime.h"

namespace bwacuda {

constexpr int FAN = 4;  // bucket streams

// Device work buffers of one in-flight batch.
struct BatchBufs {
    DevBuf keys_in, keys_out, idx_in, idx_out, tmp, table;
    DevBuf xl;  // group-per-job buckets: work words and the deferred-job list
    cudaStream_t fan[FAN] = {};
    cudaEvent_t fork = nullptr, join[FAN] = {};
    // graph cache for device-resident replays
    cudaGraphExec_t graph = nullptr;
    const void *g_seq = nullptr, *g_jobs = nullptr, *g_out = nullptr;
    const void *g_bufs[6] = {};  // work buffers the graph was captured with
    uint64_t g_gen = 0;          // tuning generation the graph was captured with
    size_t g_n = 0;
    cudaStream_t g_stream = nullptr;
    ExtParams g_P{};
    // per-SM room the bucket kernels leave for kernels running beside them
    int reserve_regs = 0, reserve_threads = 0;
    size_t jobs_cap = 0;  // jobs the work buffers are sized for (batched_enqueue, batched_reserve)
};

// Jobs to size a reused slot's work buffers for, n or more: they grow at least twofold (every
// regrowth frees a buffer, and cudaFree waits for the whole device, stalling the work of the
// other streams, e.g. the serving loop's other waves).
static size_t batched_grow_jobs(BatchBufs &bb, size_t n)
{
    if (n > bb.jobs_cap) bb.jobs_cap = std::max(n, bb.jobs_cap * 2);
    return bb.jobs_cap;
}

struct BatchedState {
    int nsm = 0;
    int sm_regs = 65536, sm_threads = 2048;
    int nb = 0;
    // tuning (set by bwacuda_autotune_extend or the options); gen changes with every setting
    int tb = 128;    // threads per block of the persistent kernels
    int grab = 1;    // 32-job rounds per work-counter grab
    int step = 32;   // query-length bucket width below 257 columns
    int long_qlo = INT_MAX;  // buckets from this query length up use the group-per-job kernel
    uint64_t gen = 1;
    ExtBucketDef defs[EXT_MAX_BUCKETS];
    DevBuf d_defs;
    BatchBufs bufs[3];  // [0], [1]: host-pipeline slots; [2]: device-resident calls
};

static int batched_init(bwacuda_ctx *c)
{
    if (c->batched) return BWACUDA_OK;
    BatchedState *B = new (std::nothrow) BatchedState();
    if (!B) return BWACUDA_ENOMEM;
    cudaError_t e = cudaDeviceGetAttribute(&B->nsm, cudaDevAttrMultiProcessorCount, c->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&B->sm_regs, cudaDevAttrMaxRegistersPerMultiprocessor, c->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&B->sm_threads, cudaDevAttrMaxThreadsPerMultiProcessor, c->device);
    if (e == cudaSuccess) e = ext_sort_prefer_shared();
    if (e != cudaSuccess) { delete B; return cuda_status(e); }
    B->nb = ext_bucket_defs(B->defs, EXT_MAX_BUCKETS, B->step, B->long_qlo);
    if ((e = B->d_defs.ensure(sizeof(B->defs))) != cudaSuccess) { delete B; return cuda_status(e); }
    if ((e = cudaMemcpy(B->d_defs.p, B->defs, sizeof(ExtBucketDef) * B->nb, cudaMemcpyHostToDevice)) != cudaSuccess) {
        delete B;
        return cuda_status(e);
    }
    for (auto &bb : B->bufs) {
        for (int f = 0; f < FAN; ++f) {
            if ((e = cudaStreamCreateWithFlags(&bb.fan[f], cudaStreamNonBlocking)) != cudaSuccess) break;
            if ((e = cudaEventCreateWithFlags(&bb.join[f], cudaEventDisableTiming)) != cudaSuccess) break;
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bb.fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = bb.table.ensure(EXT_MAX_BUCKETS * 4 * sizeof(uint32_t));
        if (e != cudaSuccess) break;
    }
    c->batched = B;
    return cuda_status(e);
}

void batched_release(bwacuda_ctx *c)
{
    BatchedState *B = c->batched;
    if (!B) return;
    for (auto &bb : B->bufs) {
        if (bb.graph) cudaGraphExecDestroy(bb.graph);
        for (int f = 0; f < FAN; ++f) {
            if (bb.fan[f]) cudaStreamSynchronize(bb.fan[f]);
        }
        for (int f = 0; f < FAN; ++f) {
            if (bb.fan[f]) cudaStreamDestroy(bb.fan[f]);
            if (bb.join[f]) cudaEventDestroy(bb.join[f]);
        }
        if (bb.fork) cudaEventDestroy(bb.fork);
        bb.keys_in.release(); bb.keys_out.release(); bb.idx_in.release(); bb.idx_out.release();
        bb.tmp.release(); bb.table.release(); bb.xl.release();
    }
    B->d_defs.release();
    delete B;
    c->batched = nullptr;
}

int batched_set_block(bwacuda_ctx *c, int tb)
{
    int rc = batched_init(c);
    if (rc) return rc;
    c->batched->tb = tb;
    c->batched->gen++;
    return BWACUDA_OK;
}

int batched_set_grab(bwacuda_ctx *c, int grab)
{
    int rc = batched_init(c);
    if (rc) return rc;
    c->batched->grab = grab;
    c->batched->gen++;
    return BWACUDA_OK;
}

// New bucket boundaries; waits for in-flight batches (they read the old table).
int batched_set_bucket_step(bwacuda_ctx *c, int step)
{
    int rc = batched_init(c);
    if (rc) return rc;
    BatchedState *B = c->batched;
    if (B->step == step) return BWACUDA_OK;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_status(e);
    B->step = step;
    B->nb = ext_bucket_defs(B->defs, EXT_MAX_BUCKETS, step, B->long_qlo);
    if ((e = cudaMemcpy(B->d_defs.p, B->defs, sizeof(ExtBucketDef) * B->nb, cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_status(e);
    B->gen++;
    return BWACUDA_OK;
}

// Query length from which the buckets use the group-per-job kernel (INT_MAX: only the
// open-ended buckets); waits for in-flight batches like batched_set_bucket_step.
int batched_set_long(bwacuda_ctx *c, int long_qlo)
{
    int rc = batched_init(c);
    if (rc) return rc;
    BatchedState *B = c->batched;
    if (B->long_qlo == long_qlo) return BWACUDA_OK;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_status(e);
    B->long_qlo = long_qlo;
    B->nb = ext_bucket_defs(B->defs, EXT_MAX_BUCKETS, B->step, long_qlo);
    if ((e = cudaMemcpy(B->d_defs.p, B->defs, sizeof(ExtBucketDef) * B->nb, cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_status(e);
    B->gen++;
    return BWACUDA_OK;
}

int batched_get_long(bwacuda_ctx *c) { return c->batched ? c->batched->long_qlo : INT_MAX; }

// Lanes per job of the group-per-job kernel; a new value invalidates captured graphs.
int batched_set_long_lanes(bwacuda_ctx *c, int lanes)
{
    int rc = batched_init(c);
    if (rc) return rc;
    if (c->long_lanes != lanes) {
        c->long_lanes = lanes;
        c->batched->gen++;
    }
    return BWACUDA_OK;
}

// Window kernel on the open-ended buckets: 0 off, 1 on buckets of a warp of jobs per SM or
// more, 2 always; a new value invalidates captured graphs.
int batched_set_long_slide(bwacuda_ctx *c, int mode)
{
    int rc = batched_init(c);
    if (rc) return rc;
    if (c->long_slide != mode) {
        c->long_slide = mode;
        c->batched->gen++;
    }
    return BWACUDA_OK;
}

void batched_get_tuning(bwacuda_ctx *c, int *tb, int *grab, int *step)
{
    BatchedState *B = c->batched;
    *tb = B ? B->tb : 128;
    *grab = B ? B->grab : 1;
    *step = B ? B->step : 32;
}

static cudaError_t ensure_bufs(BatchBufs &bb, size_t n)
{
    cudaError_t e;
    if ((e = bb.keys_in.ensure(n * 2 + 16)) != cudaSuccess) return e;
    if ((e = bb.keys_out.ensure(n * 2 + 16)) != cudaSuccess) return e;
    if ((e = bb.idx_in.ensure(n * 4 + 16)) != cudaSuccess) return e;
    if ((e = bb.idx_out.ensure(n * 4 + 16)) != cudaSuccess) return e;
    if ((e = bb.xl.ensure(((size_t)XL_WORK_WORDS + n) * 4 + 16)) != cudaSuccess) return e;
    return bb.tmp.ensure(ext_sort_temp_bytes(n) + 256);
}

// Enqueue the batched sequence for n device-resident jobs on stream s.
static cudaError_t enqueue_batched(bwacuda_ctx *c, BatchBufs &bb, const uint8_t *d_seq,
                                   const bwacuda_dev_ext_job *d_jobs, size_t n, const ExtParams &P,
                                   bwacuda_ext_result *d_out, cudaStream_t s, uint32_t *err = nullptr,
                                   unsigned long long *cells = nullptr)
{
    BatchedState *B = c->batched;
    const bool lanes = ext_pair_lanes_ok(P.sc.o_del, P.sc.e_del, P.sc.o_ins, P.sc.e_ins);
    cudaError_t e = ext_sort_and_bucket(d_jobs, n, P.sc.max_sc, lanes, d_seq, P.ug, P.zdrop, d_out,
                                        static_cast<uint16_t *>(bb.keys_in.p),
                                        static_cast<uint16_t *>(bb.keys_out.p), static_cast<uint32_t *>(bb.idx_in.p),
                                        static_cast<uint32_t *>(bb.idx_out.p), bb.tmp.p, bb.tmp.cap,
                                        static_cast<const ExtBucketDef *>(B->d_defs.p), B->nb,
                                        static_cast<uint32_t *>(bb.table.p), s);
    if (e != cudaSuccess) return e;
    uint32_t *work = static_cast<uint32_t *>(bb.xl.p);
    if ((e = cudaMemsetAsync(work, 0, XL_WORK_WORDS * 4, s)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(bb.fork, s)) != cudaSuccess) return e;
    for (int f = 0; f < FAN; ++f)
        if ((e = cudaStreamWaitEvent(bb.fan[f], bb.fork, 0)) != cudaSuccess) return e;
    // Group-per-job buckets (the open-ended ones take queries of any length) one after
    // another on the first stream, then the deferred launches over the jobs whose bands
    // needed a larger ring; empty buckets exit at once.
    ExtLongLaunch X;
    X.seq = d_seq;
    X.jobs = d_jobs;
    X.order = static_cast<const uint32_t *>(bb.idx_out.p);
    X.njobs = (uint32_t)n;
    X.min_qlen = 0;
    X.lanes = c->long_lanes;
    X.ring_cols = XL_RING_DEFAULT;
    X.P = P;
    X.out = d_out;
    X.err = err ? err : reinterpret_cast<uint32_t *>(c->d_misc.p);
    X.cells = cells ? cells : reinterpret_cast<unsigned long long *>((char *)c->d_misc.p + 8);
    X.defer = work + XL_WORK_WORDS;
    X.defer_count = work + XL_WORK_DCOUNT;
    X.reserve_regs = bb.reserve_regs;
    X.reserve_threads = bb.reserve_threads;
    X.sm_regs = B->sm_regs;
    X.sm_threads = B->sm_threads;
    X.stream = bb.fan[0];
    // the open-ended buckets of the 8- and 16-bit classes run the thread-per-job window kernel
    // first (bands up to bwa-mem's default 100; wider ones stay with the group kernel), on
    // buckets of at least a warp of jobs per SM unless BWACUDA_OPT_LONG_SLIDE forces it
    const int slide_wc = c->long_slide && lanes ? ext_slide_window_for_band(100) : 0;
    X.slide_min = c->long_slide == 2 ? 0u : (uint32_t)B->nsm * 32u;
    bool long16 = false, long32 = false;
    for (int b = B->nb - 1; b >= 0; --b) {
        if (B->defs[b].kernel != 1) continue;
        uint32_t *tab = static_cast<uint32_t *>(bb.table.p) + 4 * b;
        X.bounds = tab;
        X.counter = tab + 2;
        X.slide_counter = tab + 3;
        X.slide_wc = B->defs[b].qhi == EXT_QHI_OPEN ? slide_wc : 0;
        const bool w32 = B->defs[b].cls == 2;
        if ((e = ext_long_launch(X, w32, B->nsm)) != cudaSuccess) return e;
        long16 |= !w32;
        long32 |= w32;
    }
    if (long16 && (e = ext_long_deferred_launch(X, false, work, B->nsm)) != cudaSuccess) return e;
    if (long32 && (e = ext_long_deferred_launch(X, true, work, B->nsm)) != cudaSuccess) return e;
    PersistLaunch L;
    L.seq = d_seq;
    L.jobs = d_jobs;
    L.order = static_cast<const uint32_t *>(bb.idx_out.p);
    L.P = P;
    L.out = d_out;
    L.err = err ? err : reinterpret_cast<uint32_t *>(c->d_misc.p);
    L.cells = cells ? cells : reinterpret_cast<unsigned long long *>((char *)c->d_misc.p + 8);
    L.grab = B->grab;
    L.reserve_regs = bb.reserve_regs;
    L.reserve_threads = bb.reserve_threads;
    L.sm_regs = B->sm_regs;
    L.sm_threads = B->sm_threads;
    // thread-per-job buckets, largest first: they hold the long jobs
    for (int b = B->nb - 1, k = 1; b >= 0; --b) {
        if (B->defs[b].kernel == 1) continue;
        L.stream = bb.fan[k++ % FAN];
        uint32_t *tab = static_cast<uint32_t *>(bb.table.p) + 4 * b;
        if ((e = ext_persist_launch(L, B->defs[b], tab, B->nsm, B->tb)) != cudaSuccess) return e;
    }
    for (int f = 0; f < FAN; ++f) {
        if ((e = cudaEventRecord(bb.join[f], bb.fan[f])) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(s, bb.join[f], 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

int extend_device_batched(bwacuda_ctx *c, const uint8_t *d_seq, const bwacuda_dev_ext_job *d_jobs, size_t n,
                          const ExtParams &P, bwacuda_ext_result *d_out, cudaStream_t s)
{
    int rc = batched_init(c);
    if (rc) return rc;
    BatchBufs &bb = c->batched->bufs[2];
    cudaError_t e = ensure_bufs(bb, n);
    if (e != cudaSuccess) return cuda_status(e);
    // Replay a captured graph when the same batch comes back (same buffers, size,
    // scoring and stream); otherwise capture a new one.
    const void *bufs[6] = {bb.keys_in.p, bb.keys_out.p, bb.idx_in.p, bb.idx_out.p, bb.tmp.p, bb.table.p};
    const bool same = bb.graph && bb.g_seq == d_seq && bb.g_jobs == d_jobs && bb.g_out == d_out && bb.g_n == n &&
                      bb.g_stream == s && bb.g_gen == c->batched->gen && memcmp(bb.g_bufs, bufs, sizeof(bufs)) == 0 &&
                      memcmp(&bb.g_P, &P, sizeof(P)) == 0;
    if (!same && c->use_graphs) {
        if (bb.graph) {
            cudaGraphExecDestroy(bb.graph);
            bb.graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return cuda_status(e);
        cudaError_t e2 = enqueue_batched(c, bb, d_seq, d_jobs, n, P, d_out, s);
        e = cudaStreamEndCapture(s, &g);
        if (e2 != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_status(e2); }
        if (e != cudaSuccess) return cuda_status(e);
        e = cudaGraphInstantiate(&bb.graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { bb.graph = nullptr; return cuda_status(e); }
        bb.g_seq = d_seq; bb.g_jobs = d_jobs; bb.g_out = d_out; bb.g_n = n; bb.g_stream = s; bb.g_P = P;
        bb.g_gen = c->batched->gen;
        memcpy(bb.g_bufs, bufs, sizeof(bufs));
    }
    if (c->use_graphs) {
        if ((e = cudaGraphLaunch(bb.graph, s)) != cudaSuccess) return cuda_status(e);
    } else if ((e = enqueue_batched(c, bb, d_seq, d_jobs, n, P, d_out, s)) != cudaSuccess) {
        return cuda_status(e);
    }
    c->stats.kernel_launches += 3 + (uint64_t)batched_bucket_count(c);
    c->stats.ext_jobs += n;
    c->dev_pending_stream = s;
    return BWACUDA_OK;
}

int batched_prepare(bwacuda_ctx *c) { return batched_init(c); }
void batched_set_reserve(BatchBufs *bb, int regs, int threads)
{
    bb->reserve_regs = regs;
    bb->reserve_threads = threads;
}
BatchBufs *batched_slot_bufs(bwacuda_ctx *c, int slot) { return &c->batched->bufs[slot & 1]; }
int batched_nsm(bwacuda_ctx *c) { return c->batched->nsm; }
// Launches of the bucket stage: one per bucket and the two deferred group-per-job launches.
int batched_bucket_count(bwacuda_ctx *c) { return c->batched->nb + 2 + (c->long_slide ? 2 : 0); }

static cudaError_t bufs_streams(BatchBufs &bb)
{
    cudaError_t e = cudaSuccess;
    for (int f = 0; f < FAN && e == cudaSuccess; ++f) {
        e = cudaStreamCreateWithFlags(&bb.fan[f], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bb.join[f], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bb.fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = bb.table.ensure(EXT_MAX_BUCKETS * 4 * sizeof(uint32_t));
    return e;
}

BatchBufs *batchbufs_create()
{
    BatchBufs *bb = new (std::nothrow) BatchBufs();
    if (!bb) return nullptr;
    if (bufs_streams(*bb) != cudaSuccess) {
        batchbufs_destroy(bb);
        return nullptr;
    }
    return bb;
}

void batchbufs_destroy(BatchBufs *bb)
{
    if (!bb) return;
    for (int f = 0; f < FAN; ++f) {
        if (bb->fan[f]) cudaStreamSynchronize(bb->fan[f]);
        if (bb->fan[f]) cudaStreamDestroy(bb->fan[f]);
        if (bb->join[f]) cudaEventDestroy(bb->join[f]);
    }
    if (bb->fork) cudaEventDestroy(bb->fork);
    if (bb->graph) cudaGraphExecDestroy(bb->graph);
    bb->keys_in.release(); bb->keys_out.release(); bb->idx_in.release(); bb->idx_out.release();
    bb->tmp.release(); bb->table.release(); bb->xl.release();
    delete bb;
}

// The batched sequence on the caller's buffers (batched_prepare must have run).
cudaError_t batched_enqueue(bwacuda_ctx *c, BatchBufs *bb, const uint8_t *d_seq, const bwacuda_dev_ext_job *d_jobs,
                            size_t n, const ExtParams &P, bwacuda_ext_result *d_out, cudaStream_t s, uint32_t *err,
                            unsigned long long *cells)
{
    cudaError_t e = ensure_bufs(*bb, batched_grow_jobs(*bb, n));
    if (e != cudaSuccess) return e;
    return enqueue_batched(c, *bb, d_seq, d_jobs, n, P, d_out, s, err, cells);
}

// Work buffers of a slot for n jobs ahead of its first batch (the serving loop's wave slots).
cudaError_t batched_reserve(BatchBufs *bb, size_t n)
{
    cudaError_t e = ensure_bufs(*bb, n);
    if (e == cudaSuccess) bb->jobs_cap = std::max(bb->jobs_cap, n);
    return e;
}

// Host-buffer form: the plain path's packing pipeline, each chunk run batched.
int extend_batch_host_batched(bwacuda_ctx *c, const bwacuda_ext_job *jobs, size_t n, int m, const int8_t *mat,
                              const ExtParams &P, int w, bwacuda_ext_result *out)
{
    int rc = batched_init(c);
    if (rc) return rc;
    return extend_host_pipeline(c, jobs, n, m, mat, P, w, out, [c](int slot, const ExtChunkInfo &I, cudaStream_t s) {
        BatchBufs &bb = c->batched->bufs[slot];
        cudaError_t e = ensure_bufs(bb, I.n);
        if (e == cudaSuccess) e = enqueue_batched(c, bb, I.d_seq, I.d_jobs, I.n, I.P, I.d_out, s);
        c->stats.kernel_launches += 3 + (uint64_t)batched_bucket_count(c);
        return cuda_status(e);
    });
}


}  // namespace bwacuda
