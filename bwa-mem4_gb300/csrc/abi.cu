// abi.cu -- the C ABI (include/bwacuda.h): context, pinned staging, job packing,
// validation, the chunked host-buffer pipeline and the device-resident entry points.
//
// Host-buffer calls (bwacuda_extend_batch, bwacuda_ksw_align2_batch, ...) mirror
// the reference's borrowed-slice interfaces: the caller's per-job pointers are
// gathered into pinned staging (in parallel on the host cores), copied to HBM,
// run, and the results copied back into the caller's array before returning.
// Large batches are cut into chunks that alternate between two staging slots
// and two streams, so packing chunk k+1 overlaps the GPU work of chunk k.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"

using namespace bwacuda;

// ------------------------------------------------------------------ helpers

namespace bwacuda {

int cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return BWACUDA_OK;
    if (e == cudaErrorMemoryAllocation) return BWACUDA_ENOMEM;
    return BWACUDA_ECUDA;
}

cudaError_t DevBuf::ensure(size_t bytes)
{
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 4 + 256;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
}

void DevBuf::release()
{
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
}

cudaError_t HostBuf::ensure(size_t bytes)
{
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 4 + 256;
    cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
    if (e == cudaSuccess) cap = want;
    return e;
}

void HostBuf::release()
{
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
}

// Persistent worker pool for host-side packing.
WorkerPool::WorkerPool(int n)
{
    if (n < 1) n = 1;
    for (int i = 0; i < n - 1; ++i) threads_.emplace_back([this, i] { loop(i + 1); });
    nthreads_ = n;
}

WorkerPool::~WorkerPool()
{
    {
        std::lock_guard<std::mutex> g(mu_);
        stop_ = true;
        ++gen_;
    }
    cv_.notify_all();
    for (auto &t : threads_) t.join();
}

void WorkerPool::loop(int id)
{
    uint64_t seen = 0;
    for (;;) {
        std::function<void(int)> *fn;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [&] { return gen_ != seen; });
            seen = gen_;
            if (stop_) return;
            fn = fn_;
        }
        (*fn)(id);
        {
            std::lock_guard<std::mutex> g(mu_);
            if (--pending_ == 0) done_cv_.notify_all();
        }
    }
}

void WorkerPool::run(const std::function<void(int)> &fn)
{
    if (nthreads_ == 1) {
        fn(0);
        return;
    }
    std::function<void(int)> copy = fn;
    {
        std::lock_guard<std::mutex> g(mu_);
        fn_ = &copy;
        pending_ = nthreads_ - 1;
        ++gen_;
    }
    cv_.notify_all();
    copy(0);
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return pending_ == 0; });
}

Scoring make_scoring(int m, const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins)
{
    Scoring s;
    memset(&s, 0, sizeof(s));
    s.m = m;
    s.o_del = o_del; s.e_del = e_del; s.o_ins = o_ins; s.e_ins = e_ins;
    int mx = mat[0];
    for (int k = 0; k < m * m; ++k) mx = mat[k] > mx ? mat[k] : mx;
    s.max_sc = mx;
    for (int tc = 0; tc < 8; ++tc) {
        uint8_t b[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (tc < m)
            for (int qc = 0; qc < m; ++qc) b[qc] = (uint8_t)mat[tc * m + qc];
        s.prof[tc][0] = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
        s.prof[tc][1] = (uint32_t)b[4] | ((uint32_t)b[5] << 8) | ((uint32_t)b[6] << 16) | ((uint32_t)b[7] << 24);
    }
    return s;
}

int validate_scoring(int m, const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins)
{
    // Extends divide in the band clamp (>= 1); opens must not reward a gap, which
    // is what bounds every DP value by h0 + min(qlen, tlen) * max_sc.
    if (!mat || m < 1 || m > BWACUDA_MAX_M) return BWACUDA_EINVAL;
    if (e_del < 1 || e_ins < 1 || o_del < 0 || o_ins < 0) return BWACUDA_EINVAL;
    return BWACUDA_OK;
}

// The ungapped fast path's gate and threshold, crates/bwa-neon/src/batched.rs:721-765:
// uniform matrix only (and bwa's 5-letter alphabet, where code 4 = N declines the
// fast path and codes >= 5 reach the DP, which reports them);
// x = (o_min + e_min - 1) / (a + b), the most mismatches a diagonal may carry
// while every gapped alternative scores strictly less.
UngappedRule ungapped_rule(const bwacuda_ctx *c, int m, const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins)
{
    UngappedRule u{0, 0, 0, -1};
    if (!c->ungapped || m != 5 || !bin_rule(m, mat).uniform) return u;
    u.enabled = 1;
    u.a = mat[0];
    u.b = -(int)mat[1];
    const int o_min = std::min(o_del, o_ins), e_min = std::min(e_del, e_ins);
    const int denom = u.a + u.b;
    u.x = denom > 0 ? (o_min + e_min - 1) / denom : -1;
    return u;
}

// bwa-mem's 8/16-bit bin label, crates/bwa-neon/src/batched.rs:817-865 (statistics only).
int ext_bin_label(int qlen, int tlen, int h0, int m, const int8_t *mat)
{
    return bin_label(bin_rule(m, mat), qlen, tlen, h0);
}

}  // namespace bwacuda

// ------------------------------------------------------------------ context

bwacuda_ctx::bwacuda_ctx(int dev) : device(dev), pool((int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), 32u)) {}

static int ctx_init(bwacuda_ctx *c)
{
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_status(e);
    for (int s = 0; s < 2; ++s) {
        // The pipeline slots carry the short gather / sort / scatter kernels and run at the
        // device's highest stream priority: their blocks then take the SM room that the
        // persistent bucket kernels (default priority, shared-memory bound) leave free
        // instead of queueing behind bucket launches that cannot be placed yet.
        int lo_prio = 0, hi_prio = 0;
        if ((e = cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio)) != cudaSuccess) return cuda_status(e);
        if ((e = cudaStreamCreateWithPriority(&c->slot[s].stream, cudaStreamNonBlocking, hi_prio)) != cudaSuccess)
            return cuda_status(e);
        if ((e = cudaEventCreateWithFlags(&c->slot[s].done, cudaEventDisableTiming)) != cudaSuccess) return cuda_status(e);
    }
    c->stream = c->slot[0].stream;
    int pageable = 0;
    if ((e = cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, c->device)) != cudaSuccess) return cuda_status(e);
    c->pageable_access = pageable != 0;
    if ((e = c->d_misc.ensure(4096)) != cudaSuccess) return cuda_status(e);
    if ((e = c->h_misc.ensure(4096)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaMemset(c->d_misc.p, 0, 4096)) != cudaSuccess) return cuda_status(e);
    return BWACUDA_OK;
}

extern "C" int bwacuda_ctx_create(int device, bwacuda_ctx **out)
{
    if (!out) return BWACUDA_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return BWACUDA_ECUDA;
    bwacuda_ctx *c = new (std::nothrow) bwacuda_ctx(device);
    if (!c) return BWACUDA_ENOMEM;
    int rc = ctx_init(c);
    if (rc != BWACUDA_OK) {
        bwacuda_ctx_destroy(c);
        return rc;
    }
    *out = c;
    return BWACUDA_OK;
}

extern "C" void bwacuda_ctx_destroy(bwacuda_ctx *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    server_shutdown(c);
    for (int s = 0; s < 2; ++s) {
        if (c->slot[s].stream) cudaStreamSynchronize(c->slot[s].stream);
    }
    for (int s = 0; s < 2; ++s) {
        Slot &sl = c->slot[s];
        sl.h_seq.release(); sl.h_jobs.release(); sl.h_out.release(); sl.h_aux.release();
        sl.d_seq.release(); sl.d_jobs.release(); sl.d_out.release(); sl.d_aux.release();
        sl.d_scratch.release();
        sl.d_xl.release();
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    c->d_misc.release();
    c->h_misc.release();
    c->d_dev_aux.release();
    c->d_dev_scratch.release();
    c->d_dev_xl.release();
    ats_release(c);
    global_release(c);
    retry_release(c);
    ref_release(c);
    batched_release(c);
    delete c;
}

extern "C" int bwacuda_set_option(bwacuda_ctx *c, int option, int64_t value)
{
    if (!c) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    switch (option) {
    case BWACUDA_OPT_EXT_PATH:
        if (value != BWACUDA_PATH_PLAIN && value != BWACUDA_PATH_BATCHED) return BWACUDA_EINVAL;
        c->ext_path = (int)value;
        return BWACUDA_OK;
    case BWACUDA_OPT_CHUNK_JOBS:
        if (value < 1) return BWACUDA_EINVAL;
        c->chunk_jobs = (size_t)value;
        return BWACUDA_OK;
    case BWACUDA_OPT_RESCUE_KERNEL:
        if (value != BWACUDA_RESCUE_AUTO && value != BWACUDA_RESCUE_TPJ) return BWACUDA_EINVAL;
        c->rescue_kernel = (int)value;
        return BWACUDA_OK;
    case BWACUDA_OPT_GRAPHS:
        c->use_graphs = value != 0;
        return BWACUDA_OK;
    case BWACUDA_OPT_HOST_GATHER:
        if (value != BWACUDA_GATHER_AUTO && value != BWACUDA_GATHER_HOST && value != BWACUDA_GATHER_DEVICE)
            return BWACUDA_EINVAL;
        c->host_gather = (int)value;
        return BWACUDA_OK;
    case BWACUDA_OPT_PERSIST_BLOCK:
        if (value != 32 && value != 64 && value != 128 && value != 256) return BWACUDA_EINVAL;
        return batched_set_block(c, (int)value);
    case BWACUDA_OPT_GRAB:
        if (value != 1 && value != 2 && value != 4) return BWACUDA_EINVAL;
        return batched_set_grab(c, (int)value);
    case BWACUDA_OPT_BUCKET_STEP:
        if (value != 16 && value != 32 && value != 64) return BWACUDA_EINVAL;
        if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
        return batched_set_bucket_step(c, (int)value);
    case BWACUDA_OPT_UNGAPPED:
        if (value != 0 && value != 1) return BWACUDA_EINVAL;
        c->ungapped = value != 0;
        return BWACUDA_OK;
    case BWACUDA_OPT_RESCUE_LANES:
        if (value != 8 && value != 16 && value != 32) return BWACUDA_EINVAL;
        c->rescue_lanes = (int)value;
        return BWACUDA_OK;
    case BWACUDA_OPT_RESCUE_PAIR:
        if (value != 0 && value != 1 && value != 4 && value != 8 && value != 16) return BWACUDA_EINVAL;
        c->rescue_pair = value == 1 ? 4 : (int)value;
        return BWACUDA_OK;
    case BWACUDA_OPT_LONG_QLEN:
        if (value < 0 || value > (1 << 30)) return BWACUDA_EINVAL;
        if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
        return batched_set_long(c, value == 0 ? INT_MAX : (int)value);
    case BWACUDA_OPT_LONG_LANES:
        if (value != 8 && value != 16 && value != 32) return BWACUDA_EINVAL;
        return batched_set_long_lanes(c, (int)value);
    case BWACUDA_OPT_LONG_SLIDE:
        if (value < 0 || value > 2) return BWACUDA_EINVAL;
        return batched_set_long_slide(c, (int)value);
    case BWACUDA_OPT_DEVICE_PIECE:
        if (value < 1 || value > ((int64_t)1 << 30)) return BWACUDA_EINVAL;
        c->dev_piece = (size_t)value;
        return BWACUDA_OK;
    default:
        return BWACUDA_EINVAL;
    }
}

extern "C" const char *bwacuda_strerror(int code)
{
    switch (code) {
    case BWACUDA_OK: return "ok";
    case BWACUDA_EINVAL: return "invalid argument";
    case BWACUDA_EBASE: return "base code out of range (>= m)";
    case BWACUDA_ENOMEM: return "out of memory";
    case BWACUDA_ECUDA: return "CUDA runtime error";
    case BWACUDA_ETIMEOUT: return "bounded device wait timed out";
    case BWACUDA_ESHORT: return "output buffer too small (required sizes written)";
    case BWACUDA_EUNSUPPORTED: return "input beyond the kernels' limits";
    case BWACUDA_EBUSY: return "serving queue full";
    case BWACUDA_EAGAIN: return "request not finished";
    default: return "unknown error";
    }
}

extern "C" const char *bwacuda_backend_name(void) { return "cuda"; }

extern "C" int bwacuda_get_stats(bwacuda_ctx *c, bwacuda_stats *out)
{
    if (!c || !out) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    *out = c->stats;
    return BWACUDA_OK;
}

extern "C" int bwacuda_reset_stats(bwacuda_ctx *c)
{
    if (!c) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    memset(&c->stats, 0, sizeof(c->stats));
    return BWACUDA_OK;
}

// ------------------------------------------------------------------ misc device words
// d_misc layout: [0] err flags (u32), [8] ext cells (u64), [16] wide count (u32)

static uint32_t *d_err(bwacuda_ctx *c) { return reinterpret_cast<uint32_t *>(c->d_misc.p); }
static unsigned long long *d_cells(bwacuda_ctx *c) { return reinterpret_cast<unsigned long long *>((char *)c->d_misc.p + 8); }

namespace bwacuda {

// Read back and clear the error word and the cell counter (synchronous).
int collect_device_status(bwacuda_ctx *c, cudaStream_t s, uint64_t *cells)
{
    cudaError_t e = cudaMemcpyAsync(c->h_misc.p, c->d_misc.p, 16, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_misc.p, 0, 16, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e);
    uint32_t flags = *reinterpret_cast<uint32_t *>(c->h_misc.p);
    if (cells) *cells = *reinterpret_cast<uint64_t *>((char *)c->h_misc.p + 8);
    if (flags & ERR_BASE) return BWACUDA_EBASE;
    if (flags & (ERR_RANGE | ERR_SCRATCH)) return BWACUDA_EUNSUPPORTED;
    return BWACUDA_OK;
}

}  // namespace bwacuda

// ------------------------------------------------------------------ extension

namespace {

struct ExtChunk {
    size_t c0, cn;      // job range
    uint64_t bytes;     // sequence bytes
    int qmax;
    uint32_t nwide;
    int w;              // the call's band
};

// Gather jobs [c0, c0+cn) into the slot's pinned buffers.  Returns the chunk summary.
ExtChunk pack_ext_chunk(bwacuda_ctx *c, Slot &sl, const bwacuda_ext_job *jobs, size_t c0, size_t cn,
                        int w, int max_sc, int m, const int8_t *mat, int *rc)
{
    ExtChunk ch{c0, cn, 0, 0, 0, w};
    *rc = BWACUDA_OK;
    const int P = c->pool.size();
    std::vector<uint64_t> part_bytes(P, 0);
    std::vector<int> part_qmax(P, 0), part_bad(P, 0);
    std::vector<std::vector<uint32_t>> part_wide(P);
    std::vector<uint64_t> part_bins((size_t)P * 3, 0);
    const BinRule br = bin_rule(m, mat);
    auto range = [&](int id, size_t &b, size_t &e) {
        b = cn * (size_t)id / P;
        e = cn * (size_t)(id + 1) / P;
    };
    c->pool.run([&](int id) {
        size_t b, e;
        range(id, b, e);
        uint64_t sum = 0;
        int qm = 0;
        for (size_t k = b; k < e; ++k) {
            const bwacuda_ext_job &J = jobs[c0 + k];
            if (J.qlen < 0 || J.tlen < 0 || J.h0 <= 0 || (J.qlen > 0 && !J.query) ||
                (J.tlen > 0 && !J.target)) {
                part_bad[id] = 1;
                continue;
            }
            sum += (uint64_t)J.qlen + (uint64_t)J.tlen;
            qm = std::max(qm, J.qlen);
            long long bound = (long long)J.h0 + (long long)std::min(J.qlen, J.tlen) * std::max(max_sc, 0);
            if (bound >= 32768) part_wide[id].push_back((uint32_t)k);
            part_bins[(size_t)id * 3 + bin_label(br, J.qlen, J.tlen, J.h0)]++;
        }
        part_bytes[id] = sum;
        part_qmax[id] = qm;
    });
    for (int id = 0; id < P; ++id) {
        if (part_bad[id]) { *rc = BWACUDA_EINVAL; return ch; }
        ch.bytes += part_bytes[id];
        ch.qmax = std::max(ch.qmax, part_qmax[id]);
        ch.nwide += (uint32_t)part_wide[id].size();
        c->stats.ext_bin_u8 += part_bins[(size_t)id * 3 + 0];
        c->stats.ext_bin_i16 += part_bins[(size_t)id * 3 + 1];
        c->stats.ext_bin_i32 += part_bins[(size_t)id * 3 + 2];
    }
    cudaError_t e;
    if ((e = sl.h_seq.ensure(ch.bytes + 16)) != cudaSuccess ||
        (e = sl.h_jobs.ensure(cn * sizeof(bwacuda_dev_ext_job) + (size_t)ch.nwide * 4 + 16)) != cudaSuccess) {
        *rc = cuda_status(e);
        return ch;
    }
    // byte offsets per part, then parallel gather
    std::vector<uint64_t> part_base(P, 0);
    for (int id = 1; id < P; ++id) part_base[id] = part_base[id - 1] + part_bytes[id - 1];
    uint8_t *hs = static_cast<uint8_t *>(sl.h_seq.p);
    bwacuda_dev_ext_job *hj = static_cast<bwacuda_dev_ext_job *>(sl.h_jobs.p);
    c->pool.run([&](int id) {
        size_t b, e2;
        range(id, b, e2);
        uint64_t off = part_base[id];
        for (size_t k = b; k < e2; ++k) {
            const bwacuda_ext_job &J = jobs[c0 + k];
            bwacuda_dev_ext_job D;
            D.q_off = off;
            if (J.qlen) memcpy(hs + off, J.query, (size_t)J.qlen);
            off += (uint64_t)J.qlen;
            D.t_off = off;
            if (J.tlen) memcpy(hs + off, J.target, (size_t)J.tlen);
            off += (uint64_t)J.tlen;
            D.qlen = J.qlen;
            D.tlen = J.tlen;
            D.h0 = J.h0;
            D.w = w;
            hj[k] = D;
        }
    });
    uint32_t *widx = reinterpret_cast<uint32_t *>(hj + cn);
    size_t wpos = 0;
    for (int id = 0; id < P; ++id)
        for (uint32_t v : part_wide[id]) widx[wpos++] = v;
    return ch;
}

int run_ext_chunk(bwacuda_ctx *c, int slot_i, const ExtChunk &ch, const ExtParams &P, const ExtRunner &run)
{
    Slot &sl = c->slot[slot_i];
    cudaError_t e;
    const size_t jb = ch.cn * sizeof(bwacuda_dev_ext_job);
    if ((e = sl.d_seq.ensure(ch.bytes + 16)) != cudaSuccess) return cuda_status(e);
    if ((e = sl.d_jobs.ensure(jb + (size_t)ch.nwide * 4 + 16)) != cudaSuccess) return cuda_status(e);
    if ((e = sl.d_out.ensure(ch.cn * sizeof(bwacuda_ext_result))) != cudaSuccess) return cuda_status(e);
    if ((e = sl.h_out.ensure(ch.cn * sizeof(bwacuda_ext_result))) != cudaSuccess) return cuda_status(e);
    cudaStream_t s = sl.stream;
    if (ch.bytes && (e = cudaMemcpyAsync(sl.d_seq.p, sl.h_seq.p, ch.bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaMemcpyAsync(sl.d_jobs.p, sl.h_jobs.p, jb + (size_t)ch.nwide * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess) return cuda_status(e);
    c->stats.h2d_bytes += ch.bytes + jb + (size_t)ch.nwide * 4;
    ExtChunkInfo info;
    info.d_seq = static_cast<const uint8_t *>(sl.d_seq.p);
    info.d_jobs = static_cast<const bwacuda_dev_ext_job *>(sl.d_jobs.p);
    info.d_wide = reinterpret_cast<const uint32_t *>(info.d_jobs + ch.cn);
    info.n = ch.cn;
    info.nwide = ch.nwide;
    info.qmax = ch.qmax;
    info.w = ch.w;
    info.P = P;
    info.d_out = static_cast<bwacuda_ext_result *>(sl.d_out.p);
    int rc = run(slot_i, info, s);
    if (rc) return rc;
    if ((e = cudaMemcpyAsync(sl.h_out.p, sl.d_out.p, ch.cn * sizeof(bwacuda_ext_result), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_status(e);
    c->stats.d2h_bytes += ch.cn * sizeof(bwacuda_ext_result);
    if ((e = cudaEventRecord(sl.done, s)) != cudaSuccess) return cuda_status(e);
    return BWACUDA_OK;
}

// The plain path: narrow launch over the chunk in caller order, wide jobs from
// the host-built list; queries too long for a thread's shared-memory row go to the
// group-per-job kernel.
int run_plain(bwacuda_ctx *c, int slot_i, const ExtChunkInfo &I, cudaStream_t s)
{
    const int lim16 = (int)ext_tpj_smem_limit_qcap(false), lim32 = (int)ext_tpj_smem_limit_qcap(true);
    const bool long16 = I.qmax + 1 > lim16, long32 = I.nwide > 0 && I.qmax + 1 > lim32;
    ExtLaunch L;
    L.seq = I.d_seq;
    L.jobs = I.d_jobs;
    L.order = nullptr;
    L.count_ptr = nullptr;
    L.n = I.n;
    L.P = I.P;
    L.qcap = std::min(I.qmax + 1, lim16);
    L.only_wide = 0;
    L.long_follows = long16;
    L.out = I.d_out;
    L.err = d_err(c);
    L.cells = d_cells(c);
    L.stream = s;
    cudaError_t e;
    if (I.n > I.nwide) {
        if ((e = ext_tpj_launch(L, false)) != cudaSuccess) return cuda_status(e);
        c->stats.kernel_launches++;
    }
    if (I.nwide) {
        L.order = I.d_wide;
        L.n = I.nwide;
        L.qcap = std::min(I.qmax + 1, lim32);
        L.long_follows = long32;
        if ((e = ext_tpj_launch(L, true)) != cudaSuccess) return cuda_status(e);
        c->stats.kernel_launches++;
    }
    if (long16 || long32)
        return launch_long_unbucketed(c, c->slot[slot_i].d_xl, I.d_seq, I.d_jobs, I.n, I.P, I.d_out,
                                      long16 ? lim16 : INT_MAX, long32 ? lim32 : INT_MAX, ext_long_ring_for_band(I.w),
                                      s);
    return BWACUDA_OK;
}

}  // namespace

namespace bwacuda {

int extend_host_pipeline(bwacuda_ctx *c, const bwacuda_ext_job *jobs, size_t n, int m, const int8_t *mat,
                         const ExtParams &P, int w, bwacuda_ext_result *out, const ExtRunner &run)
{
    const size_t CH = c->chunk_jobs;
    ExtChunk pend[2] = {};
    bool busy[2] = {false, false};
    int slot_i = 0;
    int rc = BWACUDA_OK;
    auto drain = [&](int s) -> int {
        if (!busy[s]) return BWACUDA_OK;
        busy[s] = false;
        cudaError_t e = cudaEventSynchronize(c->slot[s].done);
        if (e != cudaSuccess) return cuda_status(e);
        memcpy(out + pend[s].c0, c->slot[s].h_out.p, pend[s].cn * sizeof(bwacuda_ext_result));
        return BWACUDA_OK;
    };
    for (size_t c0 = 0; c0 < n && rc == BWACUDA_OK; c0 += CH) {
        const size_t cn = std::min(CH, n - c0);
        Slot &sl = c->slot[slot_i];
        if ((rc = drain(slot_i)) != BWACUDA_OK) break;
        int prc;
        ExtChunk ch = pack_ext_chunk(c, sl, jobs, c0, cn, w, P.sc.max_sc, m, mat, &prc);
        if (prc) { rc = prc; break; }
        if ((rc = run_ext_chunk(c, slot_i, ch, P, run)) != BWACUDA_OK) break;
        pend[slot_i] = ch;
        busy[slot_i] = true;
        slot_i ^= 1;
    }
    int rc2 = drain(0);
    int rc3 = drain(1);
    if (!rc) rc = rc2 ? rc2 : rc3;
    uint64_t cells = 0;
    int st = collect_device_status(c, c->slot[0].stream, &cells);
    if (!rc) rc = st;
    c->stats.ext_jobs += n;
    c->stats.ext_cells += cells;
    return rc;
}

int extend_batch_host(bwacuda_ctx *c, const bwacuda_ext_job *jobs, size_t n, int m, const int8_t *mat,
                      int o_del, int e_del, int o_ins, int e_ins, int w, int end_bonus, int zdrop,
                      bwacuda_ext_result *out)
{
    int rc = validate_scoring(m, mat, o_del, e_del, o_ins, e_ins);
    if (rc) return rc;
    if (w < 0 || (n && (!jobs || !out))) return BWACUDA_EINVAL;
    if (n == 0) return BWACUDA_OK;
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    ExtParams P;
    P.sc = make_scoring(m, mat, o_del, e_del, o_ins, e_ins);
    P.end_bonus = end_bonus;
    P.zdrop = zdrop;
    P.ug = ungapped_rule(c, m, mat, o_del, e_del, o_ins, e_ins);
    if (c->ext_path == BWACUDA_PATH_BATCHED) {
        const bool device_gather = c->host_gather == BWACUDA_GATHER_DEVICE ||
                                   (c->host_gather == BWACUDA_GATHER_AUTO && c->pageable_access);
        if (device_gather) return extend_batch_ats(c, jobs, n, m, mat, P, w, out);
        return extend_batch_host_batched(c, jobs, n, m, mat, P, w, out);
    }
    return extend_host_pipeline(c, jobs, n, m, mat, P, w, out,
                                [c](int slot, const ExtChunkInfo &I, cudaStream_t s) { return run_plain(c, slot, I, s); });
}

}  // namespace bwacuda

extern "C" int bwacuda_extend_batch(bwacuda_ctx *c, const bwacuda_ext_job *jobs, size_t n, int m,
                                    const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins,
                                    int w, int end_bonus, int zdrop, bwacuda_ext_result *out)
{
    if (!c) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    return extend_batch_host(c, jobs, n, m, mat, o_del, e_del, o_ins, e_ins, w, end_bonus, zdrop, out);
}

extern "C" int bwacuda_extend(bwacuda_ctx *c, const uint8_t *query, int32_t qlen, const uint8_t *target,
                              int32_t tlen, int m, const int8_t *mat, int o_del, int e_del, int o_ins,
                              int e_ins, int w, int end_bonus, int zdrop, int h0, bwacuda_ext_result *out)
{
    bwacuda_ext_job J;
    J.query = query;
    J.target = target;
    J.qlen = qlen;
    J.tlen = tlen;
    J.h0 = h0;
    return bwacuda_extend_batch(c, &J, 1, m, mat, o_del, e_del, o_ins, e_ins, w, end_bonus, zdrop, out);
}

// ------------------------------------------------------------------ long queries

namespace bwacuda {

int launch_long_unbucketed(bwacuda_ctx *c, DevBuf &xl, const uint8_t *seq, const bwacuda_dev_ext_job *jobs, size_t n,
                           const ExtParams &P, bwacuda_ext_result *out, int min16, int min32, int ring, cudaStream_t s)
{
    int rc = batched_prepare(c);  // the SM count
    if (rc) return rc;
    cudaError_t e;
    if ((e = xl.ensure(((size_t)XL_WORK_WORDS + n) * 4)) != cudaSuccess) return cuda_status(e);
    uint32_t *work = static_cast<uint32_t *>(xl.p);
    if ((e = cudaMemsetAsync(work, 0, XL_WORK_WORDS * 4, s)) != cudaSuccess) return cuda_status(e);
    ExtLongLaunch X;
    X.seq = seq;
    X.jobs = jobs;
    X.order = nullptr;
    X.bounds = nullptr;
    X.njobs = (uint32_t)n;
    X.lanes = c->long_lanes;
    X.ring_cols = ring;
    X.P = P;
    X.out = out;
    X.err = d_err(c);
    X.cells = d_cells(c);
    X.defer = work + XL_WORK_WORDS;
    X.defer_count = work + XL_WORK_DCOUNT;
    X.stream = s;
    const int nsm = batched_nsm(c);
    for (int w32 = 0; w32 < 2; ++w32) {
        const int mq = w32 ? min32 : min16;
        if (mq == INT_MAX) continue;
        X.min_qlen = mq;
        X.counter = work + (w32 ? XL_WORK_COUNTER32 : XL_WORK_COUNTER16);
        if ((e = ext_long_launch(X, w32 != 0, nsm)) != cudaSuccess) return cuda_status(e);
        c->stats.kernel_launches++;
    }
    for (int w32 = 0; w32 < 2; ++w32) {
        if ((w32 ? min32 : min16) == INT_MAX) continue;
        if ((e = ext_long_deferred_launch(X, w32 != 0, work, nsm)) != cudaSuccess) return cuda_status(e);
        c->stats.kernel_launches++;
    }
    return BWACUDA_OK;
}

}  // namespace bwacuda

// ------------------------------------------------------------------ rescue

namespace bwacuda {

// Narrow-cell rescue jobs: the register wavefront when the padded query fits
// 16 lanes x 32 columns (and the kernel choice allows it), else the
// shared-memory thread-per-job kernel.  Wide jobs always go to the latter.
cudaError_t rescue_narrow_launch(bwacuda_ctx *c, const RescueLaunch &L)
{
    if (c->rescue_kernel == BWACUDA_RESCUE_AUTO && L.qcap <= rescue_wf_max_qpad() && L.only_wide != 2) {
        if (!c->rescue_pair) return rescue_wf_launch(L, L.qcap, c->rescue_lanes);
        // jobs whose values fit a byte: two per group; the rest in the 32-bit wavefront
        int cols = 0;
        cudaError_t e = rescue_wf2_launch(L, L.qcap, c->rescue_pair, &cols);
        if (e != cudaSuccess) return e;
        RescueLaunch R = L;
        R.pair_cols = cols;
        return rescue_wf_launch(R, R.qcap, c->rescue_lanes);
    }
    return rescue_tpj_launch(L, false);
}

}  // namespace bwacuda

namespace {

struct ResChunk {
    size_t c0, cn;
    uint64_t bytes;
    uint64_t scratch_entries;
    int qcap;
    uint32_t nwide;
    uint64_t cells;
};

template <typename JobT>
ResChunk pack_res_chunk(bwacuda_ctx *c, Slot &sl, const JobT *jobs, size_t c0, size_t cn, int max_sc,
                        int lanes, bool per_job_sc, int *rc)
{
    ResChunk ch{c0, cn, 0, 0, 0, 0, 0};
    *rc = BWACUDA_OK;
    const int P = c->pool.size();
    std::vector<uint64_t> part_bytes(P, 0), part_scr(P, 0), part_cells(P, 0);
    std::vector<int> part_q(P, 0), part_bad(P, 0);
    std::vector<std::vector<uint32_t>> part_wide(P);
    auto range = [&](int id, size_t &b, size_t &e) {
        b = cn * (size_t)id / P;
        e = cn * (size_t)(id + 1) / P;
    };
    c->pool.run([&](int id) {
        size_t b, e;
        range(id, b, e);
        uint64_t sum = 0, scr = 0, cells = 0;
        int qc = 0;
        for (size_t k = b; k < e; ++k) {
            const JobT &J = jobs[c0 + k];
            if (J.qlen < 0 || J.tlen < 0 || (J.qlen > 0 && !J.query) || (J.tlen > 0 && !J.target) ||
                J.qlen > 65000) {
                part_bad[id] = 1;
                continue;
            }
            sum += (uint64_t)J.qlen + (uint64_t)J.tlen;
            scr += rescue_scratch_entries(J.tlen);
            cells += (uint64_t)J.qlen * (uint64_t)J.tlen;
            // room for the padded forward query and the reverse pass's padding
            int q16 = (J.qlen + 15) / 16 * 16;
            int ln = lanes ? lanes : (J.qlen * max_sc < 250 ? 16 : 8);
            int qp = (J.qlen + ln - 1) / ln * ln;
            qc = std::max(qc, std::max(q16, qp) + 16);
            long long mn = std::min(J.qlen, J.tlen);
            if (!(mn * (long long)std::max(max_sc, 0) < 32768 && J.qlen + 32 < 65536))
                part_wide[id].push_back((uint32_t)k);
        }
        part_bytes[id] = sum;
        part_scr[id] = scr;
        part_q[id] = qc;
        part_cells[id] = cells;
    });
    for (int id = 0; id < P; ++id) {
        if (part_bad[id]) { *rc = BWACUDA_EINVAL; return ch; }
        ch.bytes += part_bytes[id];
        ch.scratch_entries += part_scr[id];
        ch.qcap = std::max(ch.qcap, part_q[id]);
        ch.nwide += (uint32_t)part_wide[id].size();
        ch.cells += part_cells[id];
    }
    cudaError_t e;
    const size_t jb = cn * sizeof(bwacuda_dev_rescue_job);
    if ((e = sl.h_seq.ensure(ch.bytes + 16)) != cudaSuccess ||
        (e = sl.h_jobs.ensure(jb + cn * 8 + (size_t)ch.nwide * 4 + 16)) != cudaSuccess) {
        *rc = cuda_status(e);
        return ch;
    }
    std::vector<uint64_t> part_base(P, 0), part_sbase(P, 0);
    for (int id = 1; id < P; ++id) {
        part_base[id] = part_base[id - 1] + part_bytes[id - 1];
        part_sbase[id] = part_sbase[id - 1] + part_scr[id - 1];
    }
    uint8_t *hs = static_cast<uint8_t *>(sl.h_seq.p);
    bwacuda_dev_rescue_job *hj = static_cast<bwacuda_dev_rescue_job *>(sl.h_jobs.p);
    uint64_t *hoff = reinterpret_cast<uint64_t *>(hj + cn);
    c->pool.run([&](int id) {
        size_t b, e2;
        range(id, b, e2);
        uint64_t off = part_base[id], soff = part_sbase[id];
        for (size_t k = b; k < e2; ++k) {
            const JobT &J = jobs[c0 + k];
            bwacuda_dev_rescue_job D;
            D.q_off = off;
            if (J.qlen) memcpy(hs + off, J.query, (size_t)J.qlen);
            off += (uint64_t)J.qlen;
            D.t_off = off;
            if (J.tlen) memcpy(hs + off, J.target, (size_t)J.tlen);
            off += (uint64_t)J.tlen;
            D.qlen = J.qlen;
            D.tlen = J.tlen;
            if constexpr (sizeof(JobT) == sizeof(bwacuda_fwd_job)) {
                if (per_job_sc) {
                    const bwacuda_fwd_job &F = reinterpret_cast<const bwacuda_fwd_job &>(J);
                    D.minsc = F.minsc;
                    D.endsc = F.endsc;
                } else {
                    D.minsc = 0; D.endsc = 0;
                }
            } else {
                D.minsc = 0;
                D.endsc = 0;
            }
            hj[k] = D;
            hoff[k] = soff;
            soff += rescue_scratch_entries(J.tlen);
        }
    });
    uint32_t *widx = reinterpret_cast<uint32_t *>(hoff + cn);
    size_t wpos = 0;
    for (int id = 0; id < P; ++id)
        for (uint32_t v : part_wide[id]) widx[wpos++] = v;
    return ch;
}

int run_res_chunk(bwacuda_ctx *c, Slot &sl, const ResChunk &ch, const Scoring &sc, int mode, int lanes,
                  int minsc)
{
    cudaError_t e;
    const size_t jb = ch.cn * sizeof(bwacuda_dev_rescue_job);
    const size_t aux = jb + ch.cn * 8 + (size_t)ch.nwide * 4;
    const size_t osz = mode == 2 ? sizeof(bwacuda_fwd_result) : sizeof(bwacuda_rescue_result);
    if ((e = sl.d_seq.ensure(ch.bytes + 16)) != cudaSuccess) return cuda_status(e);
    if ((e = sl.d_jobs.ensure(aux + 16)) != cudaSuccess) return cuda_status(e);
    if ((e = sl.d_out.ensure(ch.cn * osz)) != cudaSuccess) return cuda_status(e);
    if ((e = sl.h_out.ensure(ch.cn * osz)) != cudaSuccess) return cuda_status(e);
    if ((e = sl.d_scratch.ensure(ch.scratch_entries * sizeof(uint2) + 16)) != cudaSuccess) return cuda_status(e);
    cudaStream_t s = sl.stream;
    if (ch.bytes && (e = cudaMemcpyAsync(sl.d_seq.p, sl.h_seq.p, ch.bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaMemcpyAsync(sl.d_jobs.p, sl.h_jobs.p, aux, cudaMemcpyHostToDevice, s)) != cudaSuccess) return cuda_status(e);
    c->stats.h2d_bytes += ch.bytes + aux;
    RescueLaunch L;
    const bwacuda_dev_rescue_job *dj = static_cast<const bwacuda_dev_rescue_job *>(sl.d_jobs.p);
    L.seq = static_cast<const uint8_t *>(sl.d_seq.p);
    L.jobs = dj;
    L.order = nullptr;
    L.count_ptr = nullptr;
    L.n = ch.cn;
    L.sc = sc;
    L.mode = mode;
    L.lanes = lanes;
    L.minsc = minsc;
    L.qcap = ch.qcap;
    L.only_wide = 0;
    L.scratch = static_cast<uint2 *>(sl.d_scratch.p);
    L.scratch_off = reinterpret_cast<const uint64_t *>(dj + ch.cn);
    L.out_aln = mode == 2 ? nullptr : static_cast<bwacuda_rescue_result *>(sl.d_out.p);
    L.out_fwd = mode == 2 ? static_cast<bwacuda_fwd_result *>(sl.d_out.p) : nullptr;
    L.err = d_err(c);
    L.stream = s;
    if (ch.cn > ch.nwide) {
        if ((e = rescue_narrow_launch(c, L)) != cudaSuccess) return cuda_status(e);
        c->stats.kernel_launches++;
    }
    if (ch.nwide) {
        L.order = reinterpret_cast<const uint32_t *>(L.scratch_off + ch.cn);
        L.n = ch.nwide;
        if ((e = rescue_tpj_launch(L, true)) != cudaSuccess) return cuda_status(e);
        c->stats.kernel_launches++;
    }
    if ((e = cudaMemcpyAsync(sl.h_out.p, sl.d_out.p, ch.cn * osz, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_status(e);
    c->stats.d2h_bytes += ch.cn * osz;
    if ((e = cudaEventRecord(sl.done, s)) != cudaSuccess) return cuda_status(e);
    return BWACUDA_OK;
}

template <typename JobT>
int rescue_host(bwacuda_ctx *c, const JobT *jobs, size_t n, int m, const int8_t *mat, int o_del, int e_del,
                int o_ins, int e_ins, int minsc, int max_sc, int mode, int lanes, void *out)
{
    int rc = validate_scoring(m, mat, o_del, e_del, o_ins, e_ins);
    if (rc) return rc;
    if (max_sc < 1 || (lanes != 0 && lanes != 8 && lanes != 16) || (n && (!jobs || !out))) return BWACUDA_EINVAL;
    if (n == 0) return BWACUDA_OK;
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    Scoring sc = make_scoring(m, mat, o_del, e_del, o_ins, e_ins);
    sc.max_sc = max_sc;  // the caller's max_sc sizes the padding rule and the score2 window
    const size_t osz = mode == 2 ? sizeof(bwacuda_fwd_result) : sizeof(bwacuda_rescue_result);
    {   // reference batch-width label (statistics only)
        std::vector<int> ql(n), tl(n);
        bool u8ok = true, i16ok = true;
        bool standard = m == 5;
        for (int i = 0; i < 4 && standard; ++i) {
            for (int j = 0; j < 4; ++j)
                if (mat[i * 5 + j] != (i == j ? mat[0] : mat[1])) standard = false;
            if (mat[i * 5 + 4] != -1 || mat[20 + i] != -1) standard = false;
        }
        if (standard && mat[24] != -1) standard = false;
        for (size_t k = 0; k < n; ++k) {
            long long ceil = (long long)std::min(jobs[k].qlen, jobs[k].tlen) * max_sc;
            if (!(ceil < 250 && jobs[k].qlen < 250)) u8ok = false;
            if (!(ceil < 30000 && jobs[k].tlen < 30000)) i16ok = false;
        }
        if (!standard) c->stats.rescue_width_i32++;
        else if (u8ok) c->stats.rescue_width_u8++;
        else if (i16ok) c->stats.rescue_width_i16++;
        else c->stats.rescue_width_i32++;
    }
    const size_t CH = c->chunk_jobs;
    ResChunk pend[2] = {};
    bool busy[2] = {false, false};
    int slot_i = 0;
    uint64_t cells = 0;
    auto drain = [&](int s) -> int {
        if (!busy[s]) return BWACUDA_OK;
        busy[s] = false;
        cudaError_t e = cudaEventSynchronize(c->slot[s].done);
        if (e != cudaSuccess) return cuda_status(e);
        memcpy(static_cast<char *>(out) + pend[s].c0 * osz, c->slot[s].h_out.p, pend[s].cn * osz);
        return BWACUDA_OK;
    };
    for (size_t c0 = 0; c0 < n && rc == BWACUDA_OK; c0 += CH) {
        const size_t cn = std::min(CH, n - c0);
        Slot &sl = c->slot[slot_i];
        if ((rc = drain(slot_i)) != BWACUDA_OK) break;
        int prc;
        ResChunk ch = pack_res_chunk<JobT>(c, sl, jobs, c0, cn, max_sc, lanes, mode == 2, &prc);
        if (prc) { rc = prc; break; }
        if ((size_t)ch.qcap > rescue_tpj_smem_limit_qcap(ch.nwide > 0)) { rc = BWACUDA_EUNSUPPORTED; break; }
        cells += ch.cells;
        if ((rc = run_res_chunk(c, sl, ch, sc, mode, lanes, minsc)) != BWACUDA_OK) break;
        pend[slot_i] = ch;
        busy[slot_i] = true;
        slot_i ^= 1;
    }
    int rc2 = drain(0);
    int rc3 = drain(1);
    if (!rc) rc = rc2 ? rc2 : rc3;
    int st = collect_device_status(c, c->slot[0].stream, nullptr);
    if (!rc) rc = st;
    c->stats.rescue_jobs += n;
    c->stats.rescue_cells += cells;
    return rc;
}

}  // namespace

extern "C" int bwacuda_ksw_align2_batch(bwacuda_ctx *c, const bwacuda_rescue_job *jobs, size_t n, int m,
                                        const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins,
                                        int minsc, int max_sc, bwacuda_rescue_result *out)
{
    if (!c) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    return rescue_host(c, jobs, n, m, mat, o_del, e_del, o_ins, e_ins, minsc, max_sc, 0, 0, out);
}

extern "C" int bwacuda_ksw_align2_scalar_batch(bwacuda_ctx *c, const bwacuda_rescue_job *jobs, size_t n,
                                               int m, const int8_t *mat, int o_del, int e_del, int o_ins,
                                               int e_ins, int minsc, int max_sc, int lanes,
                                               bwacuda_rescue_result *out)
{
    if (!c) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    return rescue_host(c, jobs, n, m, mat, o_del, e_del, o_ins, e_ins, minsc, max_sc, 1, lanes, out);
}

extern "C" int bwacuda_ksw_local_fwd_batch(bwacuda_ctx *c, const bwacuda_fwd_job *jobs, size_t n, int m,
                                           const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins,
                                           int max_sc, int lanes, bwacuda_fwd_result *out)
{
    if (!c) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    return rescue_host(c, jobs, n, m, mat, o_del, e_del, o_ins, e_ins, 0, max_sc, 2, lanes, out);
}

// ------------------------------------------------------------------ device-resident

namespace {

// Max query length over device jobs (synchronous: sizes the shared memory), and whether any
// job carries a negative length (out[1] != 0).
template <typename J>
__global__ void qmax_kernel(const J *__restrict__ jobs, uint32_t n, int *__restrict__ out)
{
    int mx = 0, neg = 0;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        mx = max(mx, jobs[k].qlen);
        neg |= jobs[k].qlen < 0 || jobs[k].tlen < 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        neg |= __shfl_xor_sync(0xffffffffu, neg, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, mx);
        if (neg) atomicOr(out + 1, 1);
    }
}

template <typename J>
int device_qmax(bwacuda_ctx *c, const J *jobs, size_t n, cudaStream_t s, int *qmax, bool *negative = nullptr)
{
    int *d = reinterpret_cast<int *>((char *)c->d_misc.p + 32);
    cudaError_t e = cudaMemsetAsync(d, 0, 8, s);
    if (e != cudaSuccess) return cuda_status(e);
    uint32_t grid = (uint32_t)std::min<size_t>((n + 255) / 256, 1024);
    if (grid) qmax_kernel<J><<<grid, 256, 0, s>>>(jobs, (uint32_t)n, d);
    if ((e = cudaMemcpyAsync((char *)c->h_misc.p + 32, d, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e);
    *qmax = *reinterpret_cast<int *>((char *)c->h_misc.p + 32);
    if (negative) *negative = *reinterpret_cast<int *>((char *)c->h_misc.p + 36) != 0;
    return BWACUDA_OK;
}

// The plain path over n device-resident jobs (n <= the context's piece size).
int extend_device_plain(bwacuda_ctx *c, const uint8_t *d_seq, const bwacuda_dev_ext_job *d_jobs, size_t n,
                        const ExtParams &P, bwacuda_ext_result *d_out, cudaStream_t s)
{
    int rc;
    int qmax = 0;
    if ((rc = device_qmax(c, d_jobs, n, s, &qmax)) != BWACUDA_OK) return rc;
    const int lim16 = (int)ext_tpj_smem_limit_qcap(false), lim32 = (int)ext_tpj_smem_limit_qcap(true);
    const bool long16 = qmax + 1 > lim16, long32 = qmax + 1 > lim32;
    cudaError_t e;
    ExtLaunch L;
    L.seq = d_seq;
    L.jobs = d_jobs;
    L.order = nullptr;
    L.count_ptr = nullptr;
    L.n = n;
    L.P = P;
    L.qcap = std::min(qmax + 1, lim16);
    L.long_follows = long16;
    L.out = d_out;
    L.err = d_err(c);
    L.cells = d_cells(c);
    L.stream = s;
    // narrow launch, then the wide one over the jobs needing 32-bit cells; queries too long for
    // either go to the group-per-job kernel
    L.only_wide = 0;
    if ((e = ext_tpj_launch(L, false)) != cudaSuccess) return cuda_status(e);
    L.only_wide = 1;
    L.qcap = std::min(qmax + 1, lim32);
    L.long_follows = long32;
    if ((e = ext_tpj_launch(L, true)) != cudaSuccess) return cuda_status(e);
    c->stats.kernel_launches += 3;
    if (long16 || long32) {
        rc = launch_long_unbucketed(c, c->d_dev_xl, d_seq, d_jobs, n, P, d_out, long16 ? lim16 : INT_MAX,
                                    long32 ? lim32 : INT_MAX, XL_RING_DEFAULT, s);
        if (rc) return rc;
    }
    c->stats.ext_jobs += n;
    c->dev_pending_stream = s;
    return BWACUDA_OK;
}

}  // namespace

extern "C" int bwacuda_extend_device(bwacuda_ctx *c, const uint8_t *d_seq, const bwacuda_dev_ext_job *d_jobs,
                                     size_t n, const bwacuda_scoring *scp, int end_bonus, int zdrop, int path,
                                     bwacuda_ext_result *d_out, void *stream)
{
    if (!c || !scp) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    int rc = validate_scoring(scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
    if (rc) return rc;
    if (n == 0) return BWACUDA_OK;
    if (!d_seq || !d_jobs || !d_out) return BWACUDA_EINVAL;
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    ExtParams P;
    P.sc = make_scoring(scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
    P.end_bonus = end_bonus;
    P.zdrop = zdrop;
    P.ug = ungapped_rule(c, scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
    // consecutive pieces on the stream: the sort, scans and kernels index a piece in 32 bits
    for (size_t off = 0; off < n; off += c->dev_piece) {
        const size_t m = std::min(c->dev_piece, n - off);
        rc = path == BWACUDA_PATH_BATCHED ? extend_device_batched(c, d_seq, d_jobs + off, m, P, d_out + off, s)
                                          : extend_device_plain(c, d_seq, d_jobs + off, m, P, d_out + off, s);
        if (rc) return rc;
    }
    return BWACUDA_OK;
}

extern "C" int bwacuda_ksw_align2_device(bwacuda_ctx *c, const uint8_t *d_seq,
                                         const bwacuda_dev_rescue_job *d_jobs, size_t n,
                                         const bwacuda_scoring *scp, int minsc, int max_sc, int mode,
                                         int lanes, bwacuda_rescue_result *d_out, void *stream)
{
    if (!c || !scp) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    return bwacuda::ksw_align2_device_locked(c, d_seq, d_jobs, n, scp, minsc, max_sc, mode, lanes, d_out, stream);
}

namespace bwacuda {

// One piece of a device-resident rescue call (n <= the context's piece size).
static int ksw_align2_device_piece(bwacuda_ctx *c, const uint8_t *d_seq, const bwacuda_dev_rescue_job *d_jobs, size_t n,
                                   const Scoring &sc, int minsc, int mode, int lanes, bwacuda_rescue_result *d_out,
                                   cudaStream_t s)
{
    int rc;
    int qmax = 0;
    bool negative = false;
    if ((rc = device_qmax(c, d_jobs, n, s, &qmax, &negative)) != BWACUDA_OK) return rc;
    if (negative) return BWACUDA_EINVAL;  // a negative length would size the tracker scratch wrongly
    const int qcap = (qmax + 15) / 16 * 16 + 16;
    if ((size_t)qcap > rescue_tpj_smem_limit_qcap(false)) return BWACUDA_EUNSUPPORTED;
    // tracker scratch: exclusive scan of per-job capacities, total read back to size the pool
    cudaError_t e;
    size_t tmp_need = 0;
    rescue_scratch_offsets(d_jobs, n, nullptr, nullptr, 0, &tmp_need, s);
    if ((e = c->d_dev_aux.ensure(n * 8 + tmp_need + 64)) != cudaSuccess) return cuda_status(e);
    uint64_t *off = static_cast<uint64_t *>(c->d_dev_aux.p);
    void *tmp = static_cast<char *>(c->d_dev_aux.p) + n * 8;
    if ((e = rescue_scratch_offsets(d_jobs, n, off, tmp, tmp_need, nullptr, s)) != cudaSuccess) return cuda_status(e);
    // total = off[n-1] + cap(n-1): read the last job's offset and tlen
    uint64_t last_off = 0;
    bwacuda_dev_rescue_job last;
    if ((e = cudaMemcpyAsync(&last_off, off + n - 1, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaMemcpyAsync(&last, d_jobs + n - 1, sizeof(last), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e);
    const uint64_t total = last_off + rescue_scratch_entries(last.tlen);
    if ((e = c->d_dev_scratch.ensure(total * sizeof(uint2) + 16)) != cudaSuccess) return cuda_status(e);
    RescueLaunch L;
    L.seq = d_seq;
    L.jobs = d_jobs;
    L.order = nullptr;
    L.count_ptr = nullptr;
    L.n = n;
    L.sc = sc;
    L.mode = mode;
    L.lanes = lanes;
    L.minsc = minsc;
    L.qcap = qcap;
    L.only_wide = 0;
    L.scratch = static_cast<uint2 *>(c->d_dev_scratch.p);
    L.scratch_off = off;
    L.out_aln = d_out;
    L.out_fwd = nullptr;
    L.err = d_err(c);
    L.stream = s;
    const bool wide_fits = (size_t)qcap <= rescue_tpj_smem_limit_qcap(true);
    L.only_wide = wide_fits ? 0 : 2;
    if ((e = rescue_narrow_launch(c, L)) != cudaSuccess) return cuda_status(e);
    if (wide_fits) {
        L.only_wide = 1;
        if ((e = rescue_tpj_launch(L, true)) != cudaSuccess) return cuda_status(e);
        c->stats.kernel_launches += 1;
    }
    c->stats.kernel_launches += 4;
    c->stats.rescue_jobs += n;
    c->dev_pending_stream = s;
    return BWACUDA_OK;
}

// bwacuda_ksw_align2_device with the context lock already held.
int ksw_align2_device_locked(bwacuda_ctx *c, const uint8_t *d_seq, const bwacuda_dev_rescue_job *d_jobs, size_t n,
                             const bwacuda_scoring *scp, int minsc, int max_sc, int mode, int lanes,
                             bwacuda_rescue_result *d_out, void *stream)
{
    int rc = validate_scoring(scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
    if (rc) return rc;
    if (max_sc < 1 || (mode != 0 && mode != 1) || (lanes != 0 && lanes != 8 && lanes != 16)) return BWACUDA_EINVAL;
    if (n == 0) return BWACUDA_OK;
    if (!d_seq || !d_jobs || !d_out) return BWACUDA_EINVAL;
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    Scoring sc = make_scoring(scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
    sc.max_sc = max_sc;
    // consecutive pieces on the stream: the scans and kernels index a piece in 32 bits
    for (size_t off = 0; off < n; off += c->dev_piece) {
        const size_t m = std::min(c->dev_piece, n - off);
        if ((rc = ksw_align2_device_piece(c, d_seq, d_jobs + off, m, sc, minsc, mode, lanes, d_out + off, s)))
            return rc;
    }
    return BWACUDA_OK;
}

}  // namespace bwacuda

extern "C" int bwacuda_ctx_sync(bwacuda_ctx *c)
{
    if (!c) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    cudaStream_t s = c->dev_pending_stream ? c->dev_pending_stream : c->stream;
    uint64_t cells = 0;
    int rc = collect_device_status(c, s, &cells);
    c->stats.ext_cells += cells;
    return rc;
}
