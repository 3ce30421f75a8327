// server.cu -- the serving loop: requests of extension or rescue jobs arrive at
// any time, are admitted to the GPU as HBM (within a fixed budget) frees up,
// and are run in "waves": every admitted request that shares a scoring joins
// the next wave, so requests that arrive while earlier waves run are batched
// together (continuous batching) and several waves overlap on the device.
// Inputs, queues of descriptors and results stay on the GPU; a client's
// bwacuda_server_wait copies its results out and releases its memory.
//
// Memory: one device arena of `hbm_budget_bytes`; a request occupies one
// contiguous range of it: [descriptors | (rescue) tracker offsets | results |
// bases | (rescue) tracker entries].  Descriptor offsets address the arena base,
// so a wave's jobs from many requests run in one launch.
//
// Admission: where the device reads pageable host memory (Grace-Blackwell), a
// gather kernel on a high-priority copy stream reads the caller's job array and
// slices straight into the request's range and checks the base codes; otherwise
// worker threads pack into a pinned mirror of the arena and the copy engines
// move it.  Scheduling is a host thread that admits, settles gathered requests
// (a bad base fails its request alone), launches waves, and retires waves by
// polling their completion events; every wait is bounded by the caller's timeout.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "kernels.h"
#include "runtime.h"

namespace bwacuda {

namespace {

using Clock = std::chrono::steady_clock;

// First-fit allocator over [0, cap), 256-byte granules.
class ArenaAlloc {
public:
    explicit ArenaAlloc(size_t cap) { free_[0] = cap; }
    bool alloc(size_t n, size_t *off)
    {
        n = (n + 255) & ~(size_t)255;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                *off = it->first;
                const size_t rest = it->second - n, at = it->first + n;
                free_.erase(it);
                if (rest) free_[at] = rest;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t n)
    {
        n = (n + 255) & ~(size_t)255;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }

private:
    std::map<size_t, size_t> free_;
};

enum ReqState { PENDING, ADMITTED, LAUNCHED, DONE };

struct Request {
    uint64_t id = 0;
    int kind = 0;  // 0 extension, 1 rescue
    const bwacuda_ext_job *ejobs = nullptr;
    const bwacuda_rescue_job *rjobs = nullptr;
    size_t n = 0;
    ExtParams P{};   // extension: scoring, end bonus, zdrop
    Scoring sc{};    // rescue scoring
    int w = 0, minsc = 0, max_sc = 1;
    // arena placement (bytes from the arena base)
    size_t off = 0, bytes = 0;
    size_t desc_at = 0, soff_at = 0, res_at = 0, seq_at = 0, scr_at = 0;
    uint64_t seq_bytes = 0, scr_entries = 0;
    int qmax = 0;
    bool wide = false;  // rescue: needs 32-bit cells
    ReqState state = PENDING;
    int rc = BWACUDA_OK;
    Clock::time_point t_submit, t_done;
    cudaEvent_t h2d = nullptr;
    // device-gather admission: per-job base and tracker offsets inside the request's
    // range, and the status word the gather kernel sets when a base code is >= m
    bool dev = false;
    bool ready = true;  // device-gather admissions: false until settled
    std::vector<uint64_t> goff, gsoff;
    volatile uint32_t status = 0;
};

struct WaveSlot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    DevBuf desc, out, soff;   // combined per-wave arrays
    BatchBufs *bb = nullptr;  // sort buffers of the batched extension path
    DevBuf flags;             // err word + cell counter of this wave
    HostBuf h_flags;
    std::vector<Request *> reqs;
    bool busy = false;
};

}  // namespace

struct ServerState {
    bwacuda_ctx *c = nullptr;
    size_t budget = 0;
    uint8_t *d_arena = nullptr, *h_arena = nullptr;
    ArenaAlloc *alloc = nullptr;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread thread;
    bool stop = false;
    uint64_t next_id = 1;
    size_t max_requests = 4096;
    std::deque<Request *> pending;
    std::vector<Request *> admitted;
    std::unordered_map<uint64_t, Request *> reqs;
    // mixed requests: id -> (extension part, rescue part), both in reqs
    std::unordered_map<uint64_t, std::pair<uint64_t, uint64_t>> mixed;
    std::vector<WaveSlot> slots;
    cudaStream_t copy_stream = nullptr, read_stream = nullptr;
    WorkerPool *pool = nullptr;
    uint64_t served_jobs = 0, served_ext_cells = 0, served_rescue_cells = 0, waves = 0;
    bool dev = false;  // admission by device gather (the device reads pageable host memory)
};

namespace {

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Device-gather admission of one request: one warp per 32 jobs writes their
// descriptors (absolute arena offsets) and, for rescue, their tracker offsets,
// copies the slices from the caller's host memory into the arena as aligned
// 16-byte words, then scans the copied bases and sets *status if any code is
// >= m (the request then fails alone instead of failing its wave).  Both job
// structs begin with query, target, qlen, tlen.
constexpr int SRV_GATHER_THREADS = 128;

template <int KIND>
__global__ void __launch_bounds__(SRV_GATHER_THREADS, 8) srv_gather_kernel(const void *__restrict__ hjobs, uint32_t n,
                                                         const uint64_t *__restrict__ goff,
                                                         const uint64_t *__restrict__ gsoff, uint8_t *__restrict__ arena,
                                                         uint64_t desc_abs, uint64_t soff_abs, uint64_t seq_abs,
                                                         uint64_t scr_base, int w, int m, volatile uint32_t *status)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t ngroups = (n + 31) / 32;
    for (uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < ngroups; g += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t k = g * 32 + lane;
        uint64_t qa = 0, ta = 0, base = 0, qo = 0, to = 0;
        uint32_t qw = 0, tw = 0;
        int ql = 0, tl = 0;
        if (k < n) {
            const uint8_t *q, *t;
            if (KIND == 0) {
                const bwacuda_ext_job J = static_cast<const bwacuda_ext_job *>(hjobs)[k];
                q = J.query; t = J.target; ql = J.qlen; tl = J.tlen;
                base = seq_abs + goff[k];
                qa = reinterpret_cast<uint64_t>(q);
                ta = reinterpret_cast<uint64_t>(t);
                qw = slice_words(q, ql);
                tw = slice_words(t, tl);
                bwacuda_dev_ext_job D;
                D.q_off = qo = base + (qa & 15);
                D.t_off = to = base + 16ull * qw + (ta & 15);
                D.qlen = ql; D.tlen = tl; D.h0 = J.h0; D.w = w;
                reinterpret_cast<bwacuda_dev_ext_job *>(arena + desc_abs)[k] = D;
            } else {
                const bwacuda_rescue_job J = static_cast<const bwacuda_rescue_job *>(hjobs)[k];
                q = J.query; t = J.target; ql = J.qlen; tl = J.tlen;
                base = seq_abs + goff[k];
                qa = reinterpret_cast<uint64_t>(q);
                ta = reinterpret_cast<uint64_t>(t);
                qw = slice_words(q, ql);
                tw = slice_words(t, tl);
                bwacuda_dev_rescue_job D;
                D.q_off = qo = base + (qa & 15);
                D.t_off = to = base + 16ull * qw + (ta & 15);
                D.qlen = ql; D.tlen = tl; D.minsc = 0; D.endsc = 0;
                reinterpret_cast<bwacuda_dev_rescue_job *>(arena + desc_abs)[k] = D;
                reinterpret_cast<uint64_t *>(arena + soff_abs)[k] = scr_base + gsoff[k];
            }
        }
        warp_gather_slices(qa & ~15ull, ta & ~15ull, base, qw, tw, arena);
        __syncwarp();
        bool bad = false;
        const uint32_t cnt = min(32u, n - g * 32);
        for (uint32_t j = 0; j < cnt; ++j) {
            const uint64_t jq = __shfl_sync(0xffffffffu, qo, j), jt = __shfl_sync(0xffffffffu, to, j);
            const int jql = __shfl_sync(0xffffffffu, ql, j), jtl = __shfl_sync(0xffffffffu, tl, j);
            for (int x = (int)lane; x < jql; x += 32) bad |= arena[jq + x] >= (uint32_t)m;
            for (int x = (int)lane; x < jtl; x += 32) bad |= arena[jt + x] >= (uint32_t)m;
        }
        if (__any_sync(0xffffffffu, bad) && lane == 0) *status = 1u;
    }
}

// Lays out a request's range and checks its inputs on the host.
int plan_request(Request *r, int m)
{
    uint64_t seq = 0, scr = 0;
    int qmax = 0;
    bool wide = false;
    if (r->dev) {
        r->goff.resize(r->n);
        if (r->kind == 1) r->gsoff.resize(r->n);
    }
    for (size_t k = 0; k < r->n; ++k) {
        const int32_t ql = r->kind == 0 ? r->ejobs[k].qlen : r->rjobs[k].qlen;
        const int32_t tl = r->kind == 0 ? r->ejobs[k].tlen : r->rjobs[k].tlen;
        const uint8_t *q = r->kind == 0 ? r->ejobs[k].query : r->rjobs[k].query;
        const uint8_t *t = r->kind == 0 ? r->ejobs[k].target : r->rjobs[k].target;
        if (ql < 0 || tl < 0 || (ql && !q) || (tl && !t)) return BWACUDA_EINVAL;
        if (r->kind == 0 && r->ejobs[k].h0 <= 0) return BWACUDA_EINVAL;
        if (r->dev) {
            // slices travel as the aligned 16-byte words that cover them
            r->goff[k] = seq;
            seq += 16ull * (slice_words(q, ql) + slice_words(t, tl));
        } else {
            seq += (uint64_t)ql + (uint64_t)tl;
        }
        qmax = std::max(qmax, ql);
        if (r->kind == 1) {
            if (r->dev) r->gsoff[k] = scr;
            scr += rescue_scratch_entries(tl);
            if ((long long)std::min(ql, tl) * std::max(r->max_sc, 0) >= 32768) wide = true;
        }
    }
    (void)m;
    r->qmax = qmax;
    r->wide = wide;
    r->seq_bytes = seq;
    r->scr_entries = scr;
    const size_t rsz = r->kind == 0 ? sizeof(bwacuda_ext_result) : sizeof(bwacuda_rescue_result);
    size_t at = 0;
    r->desc_at = at;
    at = align256(at + r->n * 32);
    if (r->kind == 1) {
        r->soff_at = at;
        at = align256(at + r->n * 8);
    }
    r->res_at = at;
    at = align256(at + r->n * rsz);
    r->seq_at = at;
    at = align256(at + seq);
    r->scr_at = at;
    at = align256(at + scr * 8);
    r->bytes = at;
    // the rescue kernels' per-launch limit (extension takes any query length)
    if (r->kind == 1 && (size_t)((qmax + 15) / 16 * 16 + 16) > rescue_tpj_smem_limit_qcap(wide)) return BWACUDA_EUNSUPPORTED;
    return BWACUDA_OK;
}

// Packs the request into the pinned host arena at its offset (absolute
// offsets in the descriptors), validating base codes.
int pack_request(ServerState *S, Request *r, int m)
{
    uint8_t *H = S->h_arena + r->off;
    const uint64_t base = r->off + r->seq_at;
    const int P = S->pool->size();
    std::vector<uint64_t> part_bytes(P, 0), part_scr(P, 0);
    std::vector<int> bad(P, 0);
    auto range = [&](int id, size_t &b, size_t &e) {
        b = r->n * (size_t)id / P;
        e = r->n * (size_t)(id + 1) / P;
    };
    S->pool->run([&](int id) {
        size_t b, e;
        range(id, b, e);
        uint64_t sum = 0, scr = 0;
        for (size_t k = b; k < e; ++k) {
            const int32_t ql = r->kind == 0 ? r->ejobs[k].qlen : r->rjobs[k].qlen;
            const int32_t tl = r->kind == 0 ? r->ejobs[k].tlen : r->rjobs[k].tlen;
            sum += (uint64_t)ql + (uint64_t)tl;
            if (r->kind == 1) scr += rescue_scratch_entries(tl);
        }
        part_bytes[id] = sum;
        part_scr[id] = scr;
    });
    std::vector<uint64_t> pb(P, 0), ps(P, 0);
    for (int id = 1; id < P; ++id) {
        pb[id] = pb[id - 1] + part_bytes[id - 1];
        ps[id] = ps[id - 1] + part_scr[id - 1];
    }
    const uint64_t scr_base = (r->off + r->scr_at) / 8;  // uint2 index from the arena base
    S->pool->run([&](int id) {
        size_t b, e;
        range(id, b, e);
        uint64_t off = pb[id], soff = ps[id];
        for (size_t k = b; k < e; ++k) {
            const uint8_t *q = r->kind == 0 ? r->ejobs[k].query : r->rjobs[k].query;
            const uint8_t *t = r->kind == 0 ? r->ejobs[k].target : r->rjobs[k].target;
            const int32_t ql = r->kind == 0 ? r->ejobs[k].qlen : r->rjobs[k].qlen;
            const int32_t tl = r->kind == 0 ? r->ejobs[k].tlen : r->rjobs[k].tlen;
            uint8_t *dq = H + r->seq_at + off;
            int acc = 0;
            for (int32_t x = 0; x < ql; ++x) { dq[x] = q[x]; acc |= q[x] >= (unsigned)m; }
            uint8_t *dt = dq + ql;
            for (int32_t x = 0; x < tl; ++x) { dt[x] = t[x]; acc |= t[x] >= (unsigned)m; }
            if (acc) bad[id] = 1;
            if (r->kind == 0) {
                bwacuda_dev_ext_job D;
                D.q_off = base + off;
                D.t_off = base + off + (uint64_t)ql;
                D.qlen = ql;
                D.tlen = tl;
                D.h0 = r->ejobs[k].h0;
                D.w = r->w;
                memcpy(H + r->desc_at + k * 32, &D, 32);
            } else {
                bwacuda_dev_rescue_job D;
                D.q_off = base + off;
                D.t_off = base + off + (uint64_t)ql;
                D.qlen = ql;
                D.tlen = tl;
                D.minsc = 0;
                D.endsc = 0;
                memcpy(H + r->desc_at + k * 32, &D, 32);
                const uint64_t so = scr_base + soff;
                memcpy(H + r->soff_at + k * 8, &so, 8);
                soff += rescue_scratch_entries(tl);
            }
            off += (uint64_t)ql + (uint64_t)tl;
        }
    });
    for (int id = 0; id < P; ++id)
        if (bad[id]) return BWACUDA_EBASE;
    return BWACUDA_OK;
}

bool same_group(const Request *a, const Request *b)
{
    if (a->kind != b->kind) return false;
    if (a->kind == 0) return memcmp(&a->P, &b->P, sizeof(ExtParams)) == 0;
    return a->minsc == b->minsc && a->max_sc == b->max_sc && memcmp(&a->sc, &b->sc, sizeof(Scoring)) == 0;
}

void finish(ServerState *S, Request *r, int rc)
{
    r->rc = rc;
    r->state = DONE;
    r->t_done = Clock::now();
    (void)S;
}

// Admit pending requests in arrival order while their range fits the arena.
void admit(ServerState *S)
{
    while (!S->pending.empty()) {
        Request *r = S->pending.front();
        size_t off;
        if (!S->alloc->alloc(r->bytes, &off)) break;
        S->pending.pop_front();
        r->off = off;
        const int mm = r->kind == 0 ? r->P.sc.m : r->sc.m;
        cudaError_t e = cudaSuccess;
        if (r->dev) {
            r->ready = false;
            // the device reads the caller's jobs and slices; the request is usable
            // once its event fires and its status word is still 0
            int nsm = 0;
            if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, S->c->device) != cudaSuccess || nsm < 1) nsm = 1;
            // one block per SM, in the room the waves' bucket kernels leave free
            const uint32_t grid =
                (uint32_t)std::min<size_t>((r->n * 32 + SRV_GATHER_THREADS - 1) / SRV_GATHER_THREADS, (size_t)nsm);
            const uint64_t scr_base = (r->off + r->scr_at) / 8;  // uint2 index from the arena base
            if (r->kind == 0)
                srv_gather_kernel<0><<<grid, SRV_GATHER_THREADS, 0, S->copy_stream>>>(r->ejobs, (uint32_t)r->n, r->goff.data(), nullptr,
                                                                      S->d_arena, r->off + r->desc_at, 0,
                                                                      r->off + r->seq_at, 0, r->w, mm, &r->status);
            else
                srv_gather_kernel<1><<<grid, SRV_GATHER_THREADS, 0, S->copy_stream>>>(r->rjobs, (uint32_t)r->n, r->goff.data(),
                                                                      r->gsoff.data(), S->d_arena, r->off + r->desc_at,
                                                                      r->off + r->soff_at, r->off + r->seq_at, scr_base,
                                                                      0, mm, &r->status);
            e = cudaGetLastError();
        } else {
            int rc = pack_request(S, r, mm);
            if (rc != BWACUDA_OK) {
                S->alloc->release(r->off, r->bytes);
                r->bytes = 0;
                finish(S, r, rc);
                continue;
            }
            // copy in: descriptors (+ tracker offsets) and bases
            const size_t head = r->kind == 1 ? r->res_at : r->n * 32;
            e = cudaMemcpyAsync(S->d_arena + r->off, S->h_arena + r->off, head, cudaMemcpyHostToDevice, S->copy_stream);
            if (e == cudaSuccess && r->seq_bytes)
                e = cudaMemcpyAsync(S->d_arena + r->off + r->seq_at, S->h_arena + r->off + r->seq_at, r->seq_bytes,
                                    cudaMemcpyHostToDevice, S->copy_stream);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->h2d, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(r->h2d, S->copy_stream);
        if (e != cudaSuccess) {
            finish(S, r, cuda_status(e));
            continue;
        }
        r->state = ADMITTED;
        S->admitted.push_back(r);
    }
}

// Device-gather admissions whose copy has landed: a request with a bad base code
// fails alone; the rest may join a wave.  Returns true when anything changed.
bool settle_admitted(ServerState *S)
{
    bool any = false;
    std::vector<Request *> keep;
    keep.reserve(S->admitted.size());
    for (Request *r : S->admitted) {
        if (!r->dev) { keep.push_back(r); continue; }
        const cudaError_t q = cudaEventQuery(r->h2d);
        if (q == cudaErrorNotReady) { keep.push_back(r); continue; }
        if (q != cudaSuccess || r->status != 0u) {
            S->alloc->release(r->off, r->bytes);
            r->bytes = 0;
            finish(S, r, q != cudaSuccess ? cuda_status(q) : BWACUDA_EBASE);
            any = true;
            continue;
        }
        r->dev = false;  // settled: behaves like a copied request from here on
        r->ready = true;
        keep.push_back(r);
        any = true;
    }
    S->admitted.swap(keep);
    return any;
}

// A wave slot's buffer: at least twofold growth, since every regrowth frees the old buffer and
// cudaFree waits for the whole device (the other slots' waves and the admission copies).
cudaError_t srv_grow(DevBuf &b, size_t bytes)
{
    return bytes <= b.cap ? cudaSuccess : b.ensure(std::max(bytes, b.cap * 2));
}

// Launch one wave on a free slot from the admitted requests of one group.
bool launch_wave(ServerState *S)
{
    if (S->admitted.empty()) return false;
    WaveSlot *slot = nullptr;
    for (auto &w : S->slots)
        if (!w.busy) { slot = &w; break; }
    if (!slot) return false;
    Request *lead = nullptr;
    for (Request *r : S->admitted)
        if (r->ready) { lead = r; break; }
    if (!lead) return false;
    std::vector<Request *> group, rest;
    size_t n = 0;
    for (Request *r : S->admitted) (r->ready && same_group(lead, r) ? group : rest).push_back(r);
    for (Request *r : group) n += r->n;
    S->admitted.swap(rest);
    cudaStream_t s = slot->stream;
    cudaError_t e = cudaSuccess;
    auto fail = [&](cudaError_t err) {
        for (Request *r : group) finish(S, r, cuda_status(err));
        return true;
    };
    for (Request *r : group)
        if ((e = cudaStreamWaitEvent(s, r->h2d, 0)) != cudaSuccess) return fail(e);
    const size_t rsz = lead->kind == 0 ? sizeof(bwacuda_ext_result) : sizeof(bwacuda_rescue_result);
    if ((e = srv_grow(slot->desc, n * 32 + 64)) != cudaSuccess) return fail(e);
    if ((e = srv_grow(slot->out, n * rsz + 64)) != cudaSuccess) return fail(e);
    if (lead->kind == 1 && (e = srv_grow(slot->soff, n * 8 + 64)) != cudaSuccess) return fail(e);
    // gather descriptors (and tracker offsets) of the wave
    size_t at = 0;
    int qmax = 0;
    bool wide = false;
    for (Request *r : group) {
        if ((e = cudaMemcpyAsync((char *)slot->desc.p + at * 32, S->d_arena + r->off + r->desc_at, r->n * 32,
                                 cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return fail(e);
        if (r->kind == 1 && (e = cudaMemcpyAsync((char *)slot->soff.p + at * 8, S->d_arena + r->off + r->soff_at,
                                                 r->n * 8, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return fail(e);
        at += r->n;
        qmax = std::max(qmax, r->qmax);
        wide |= r->wide;
    }
    uint32_t *err = static_cast<uint32_t *>(slot->flags.p);
    unsigned long long *cells = reinterpret_cast<unsigned long long *>((char *)slot->flags.p + 8);
    if ((e = cudaMemsetAsync(slot->flags.p, 0, 16, s)) != cudaSuccess) return fail(e);
    if (lead->kind == 0) {
        e = batched_enqueue(S->c, slot->bb, S->d_arena, static_cast<const bwacuda_dev_ext_job *>(slot->desc.p), n,
                            lead->P, static_cast<bwacuda_ext_result *>(slot->out.p), s, err, cells);
        if (e != cudaSuccess) return fail(e);
    } else {
        RescueLaunch L;
        L.seq = S->d_arena;
        L.jobs = static_cast<const bwacuda_dev_rescue_job *>(slot->desc.p);
        L.order = nullptr;
        L.count_ptr = nullptr;
        L.n = n;
        L.sc = lead->sc;
        L.mode = 0;
        L.lanes = 0;
        L.minsc = lead->minsc;
        L.qcap = (qmax + 15) / 16 * 16 + 16;
        L.only_wide = 0;
        L.scratch = reinterpret_cast<uint2 *>(S->d_arena);
        L.scratch_off = static_cast<const uint64_t *>(slot->soff.p);
        L.out_aln = static_cast<bwacuda_rescue_result *>(slot->out.p);
        L.out_fwd = nullptr;
        L.err = err;
        L.stream = s;
        if ((e = rescue_narrow_launch(S->c, L)) != cudaSuccess) return fail(e);
        if (wide) {
            L.only_wide = 1;
            if ((e = rescue_tpj_launch(L, true)) != cudaSuccess) return fail(e);
        }
    }
    // scatter results back to each request's range (they stay on the GPU)
    at = 0;
    for (Request *r : group) {
        if ((e = cudaMemcpyAsync(S->d_arena + r->off + r->res_at, (char *)slot->out.p + at * rsz, r->n * rsz,
                                 cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return fail(e);
        at += r->n;
    }
    if ((e = cudaMemcpyAsync(slot->h_flags.p, slot->flags.p, 16, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return fail(e);
    if ((e = cudaEventRecord(slot->done, s)) != cudaSuccess) return fail(e);
    for (Request *r : group) r->state = LAUNCHED;
    slot->reqs = group;
    slot->busy = true;
    S->waves++;
    return true;
}

// Retire waves whose completion event has fired.
bool retire(ServerState *S)
{
    bool any = false;
    for (auto &w : S->slots) {
        if (!w.busy) continue;
        const cudaError_t q = cudaEventQuery(w.done);
        if (q == cudaErrorNotReady) continue;
        const uint32_t flags = *static_cast<uint32_t *>(w.h_flags.p);
        const uint64_t cells = *reinterpret_cast<uint64_t *>((char *)w.h_flags.p + 8);
        int rc = q == cudaSuccess ? BWACUDA_OK : cuda_status(q);
        if (rc == BWACUDA_OK && (flags & ERR_BASE)) rc = BWACUDA_EBASE;
        if (rc == BWACUDA_OK && (flags & (ERR_RANGE | ERR_SCRATCH))) rc = BWACUDA_EUNSUPPORTED;
        for (Request *r : w.reqs) {
            finish(S, r, rc);
            S->served_jobs += r->n;
            if (r->kind == 1)
                for (size_t k = 0; k < r->n; ++k)
                    S->served_rescue_cells += (uint64_t)r->rjobs[k].qlen * (uint64_t)r->rjobs[k].tlen;
        }
        S->served_ext_cells += cells;  // extension waves count their inner-loop cells on the device
        w.reqs.clear();
        w.busy = false;
        any = true;
    }
    return any;
}

void scheduler(ServerState *S)
{
    cudaSetDevice(S->c->device);
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        bool progress = retire(S);
        if (progress) S->cv_done.notify_all();
        admit(S);
        progress |= settle_admitted(S);
        while (launch_wave(S)) progress = true;
        // notify waiters of requests that failed at admission
        S->cv_done.notify_all();
        bool busy = false;
        for (auto &w : S->slots) busy |= w.busy;
        for (Request *r : S->admitted) busy |= !r->ready;  // gathers in flight are polled too
        if (S->stop && !busy) {
            for (Request *r : S->pending) finish(S, r, BWACUDA_EBUSY);
            for (Request *r : S->admitted) finish(S, r, BWACUDA_EBUSY);
            S->pending.clear();
            S->admitted.clear();
            S->cv_done.notify_all();
            return;
        }
        if (!progress) {
            // GPU progress is polled; new submissions wake the thread at once
            S->cv_work.wait_for(lk, std::chrono::microseconds(busy ? 50 : 2000));
        }
    }
}

void release_request(ServerState *S, Request *r)
{
    if (r->bytes) S->alloc->release(r->off, r->bytes);
    if (r->h2d) cudaEventDestroy(r->h2d);
    delete r;
}

}  // namespace

void server_shutdown(bwacuda_ctx *c)
{
    ServerState *S = c->server;
    if (!S) return;
    {
        std::lock_guard<std::mutex> g(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    if (S->thread.joinable()) S->thread.join();
    cudaSetDevice(c->device);
    for (auto &kv : S->reqs) {
        if (kv.second->h2d) cudaEventDestroy(kv.second->h2d);
        delete kv.second;
    }
    for (auto &w : S->slots) {
        if (w.stream) cudaStreamSynchronize(w.stream);
        w.desc.release();
        w.out.release();
        w.soff.release();
        w.flags.release();
        w.h_flags.release();
        if (w.bb) batchbufs_destroy(w.bb);
        if (w.done) cudaEventDestroy(w.done);
        if (w.stream) cudaStreamDestroy(w.stream);
    }
    if (S->copy_stream) cudaStreamDestroy(S->copy_stream);
    if (S->read_stream) cudaStreamDestroy(S->read_stream);
    if (S->d_arena) cudaFree(S->d_arena);
    if (S->h_arena) cudaFreeHost(S->h_arena);
    delete S->alloc;
    delete S->pool;
    delete S;
    c->server = nullptr;
}

}  // namespace bwacuda

using namespace bwacuda;

extern "C" int bwacuda_server_start(bwacuda_ctx *c, const bwacuda_server_config *cfg)
{
    if (!c) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    if (c->server) return BWACUDA_EBUSY;
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    int rc = batched_prepare(c);
    if (rc) return rc;
    ServerState *S = new (std::nothrow) ServerState();
    if (!S) return BWACUDA_ENOMEM;
    S->c = c;
    S->budget = cfg && cfg->hbm_budget_bytes ? (size_t)cfg->hbm_budget_bytes : ((size_t)4 << 30);
    const int nw = cfg && cfg->max_waves > 0 ? cfg->max_waves : 3;
    if (cfg && cfg->max_requests > 0) S->max_requests = (size_t)cfg->max_requests;
    // admission by device gather where the device reads pageable host memory (no
    // pinned mirror of the arena then), else host packing through a pinned mirror
    S->dev = c->pageable_access && c->host_gather != BWACUDA_GATHER_HOST;
    cudaError_t e = cudaMalloc(&S->d_arena, S->budget);
    if (e == cudaSuccess && !S->dev)
        e = cudaHostAlloc(reinterpret_cast<void **>(&S->h_arena), S->budget, cudaHostAllocDefault);
    int lo_prio = 0, hi_prio = 0;
    // admission gathers use no shared memory but should leave an empty SM configured for the
    // waves' bucket kernels (maximum shared memory)
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(srv_gather_kernel<0>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(srv_gather_kernel<1>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    // admission copies run beside the waves' persistent kernels: highest priority
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&S->copy_stream, cudaStreamNonBlocking, hi_prio);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->read_stream, cudaStreamNonBlocking);
    S->slots.resize(nw);
    for (auto &w : S->slots) {
        if (e != cudaSuccess) break;
        e = cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = w.flags.ensure(64);
        if (e == cudaSuccess) e = w.h_flags.ensure(64);
        if (e == cudaSuccess) w.bb = batchbufs_create();
        if (e == cudaSuccess && !w.bb) e = cudaErrorMemoryAllocation;
        // room for one admission-gather block per SM beside the wave's bucket kernels
        if (e == cudaSuccess) batched_set_reserve(w.bb, SRV_GATHER_THREADS * 64, SRV_GATHER_THREADS);
        // buffers sized ahead for waves of budget / 1024 jobs (at most 8M): growing them while
        // other waves run would wait for the whole device at every regrowth
        const size_t n0 = std::min<size_t>(S->budget / 1024, size_t(1) << 23);
        if (e == cudaSuccess) e = w.desc.ensure(n0 * 32 + 64);
        if (e == cudaSuccess) e = w.out.ensure(n0 * sizeof(bwacuda_rescue_result) + 64);
        if (e == cudaSuccess) e = w.soff.ensure(n0 * 8 + 64);
        if (e == cudaSuccess) e = batched_reserve(w.bb, n0);
    }
    if (e != cudaSuccess) {
        c->server = S;
        server_shutdown(c);
        return cuda_status(e);
    }
    S->alloc = new ArenaAlloc(S->budget);
    S->pool = new WorkerPool((int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), 16u));
    c->server = S;
    S->thread = std::thread(scheduler, S);
    return BWACUDA_OK;
}

extern "C" int bwacuda_server_stop(bwacuda_ctx *c)
{
    if (!c) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    if (!c->server) return BWACUDA_EINVAL;
    server_shutdown(c);
    return BWACUDA_OK;
}

// Queues the requests together (all or none; r[1] may be null).  *mixed_id, when given,
// receives one id naming both.
static int submit_all(bwacuda_ctx *c, Request *r0, Request *r1, uint64_t *mixed_id)
{
    ServerState *S = c->server;
    Request *rs[2] = {r0, r1};
    auto drop = [&]() { delete r0; delete r1; };
    if (!S) { drop(); return BWACUDA_EINVAL; }
    size_t bytes = 0;
    for (Request *r : rs) {
        if (!r) continue;
        r->dev = S->dev;
        int rc = plan_request(r, r->kind == 0 ? r->P.sc.m : r->sc.m);
        if (rc != BWACUDA_OK) { drop(); return rc; }
        bytes += r->bytes;
    }
    if (bytes > S->budget) { drop(); return BWACUDA_ENOMEM; }  // could never be admitted
    std::lock_guard<std::mutex> g(S->mu);
    if (S->stop) { drop(); return BWACUDA_EBUSY; }
    if (S->reqs.size() + (r1 ? 2 : 1) > S->max_requests) { drop(); return BWACUDA_EBUSY; }
    const auto now = Clock::now();
    for (Request *r : rs) {
        if (!r) continue;
        r->id = S->next_id++;
        r->t_submit = now;
        S->reqs[r->id] = r;
        S->pending.push_back(r);
    }
    if (mixed_id) {
        *mixed_id = S->next_id++;
        S->mixed[*mixed_id] = {r0->id, r1->id};
    }
    S->cv_work.notify_one();
    return BWACUDA_OK;
}

static int submit(bwacuda_ctx *c, Request *r) { return submit_all(c, r, nullptr, nullptr); }

static Request *new_ext_request(bwacuda_ctx *c, const bwacuda_ext_job *jobs, size_t n, const bwacuda_scoring *sc,
                                int w, int end_bonus, int zdrop)
{
    Request *r = new (std::nothrow) Request();
    if (!r) return nullptr;
    r->kind = 0;
    r->ejobs = jobs;
    r->n = n;
    r->w = w;
    r->P.sc = make_scoring(sc->m, sc->mat, sc->o_del, sc->e_del, sc->o_ins, sc->e_ins);
    r->P.end_bonus = end_bonus;
    r->P.zdrop = zdrop;
    r->P.ug = ungapped_rule(c, sc->m, sc->mat, sc->o_del, sc->e_del, sc->o_ins, sc->e_ins);
    return r;
}

static Request *new_rescue_request(const bwacuda_rescue_job *jobs, size_t n, const bwacuda_scoring *sc, int minsc,
                                   int max_sc)
{
    Request *r = new (std::nothrow) Request();
    if (!r) return nullptr;
    r->kind = 1;
    r->rjobs = jobs;
    r->n = n;
    r->minsc = minsc;
    r->max_sc = max_sc;
    r->sc = make_scoring(sc->m, sc->mat, sc->o_del, sc->e_del, sc->o_ins, sc->e_ins);
    r->sc.max_sc = max_sc;
    return r;
}

extern "C" int bwacuda_server_submit_extend(bwacuda_ctx *c, const bwacuda_ext_job *jobs, size_t n,
                                            const bwacuda_scoring *sc, int w, int end_bonus, int zdrop,
                                            uint64_t *req_id)
{
    if (!c || !sc || !req_id || (n && !jobs) || n == 0 || w < 0) return BWACUDA_EINVAL;
    int rc = validate_scoring(sc->m, sc->mat, sc->o_del, sc->e_del, sc->o_ins, sc->e_ins);
    if (rc) return rc;
    Request *r = new_ext_request(c, jobs, n, sc, w, end_bonus, zdrop);
    if (!r) return BWACUDA_ENOMEM;
    rc = submit(c, r);
    if (rc == BWACUDA_OK) *req_id = r->id;
    return rc;
}

extern "C" int bwacuda_server_submit_rescue(bwacuda_ctx *c, const bwacuda_rescue_job *jobs, size_t n,
                                            const bwacuda_scoring *sc, int minsc, int max_sc, uint64_t *req_id)
{
    if (!c || !sc || !req_id || (n && !jobs) || n == 0 || max_sc < 1) return BWACUDA_EINVAL;
    int rc = validate_scoring(sc->m, sc->mat, sc->o_del, sc->e_del, sc->o_ins, sc->e_ins);
    if (rc) return rc;
    Request *r = new_rescue_request(jobs, n, sc, minsc, max_sc);
    if (!r) return BWACUDA_ENOMEM;
    rc = submit(c, r);
    if (rc == BWACUDA_OK) *req_id = r->id;
    return rc;
}

extern "C" int bwacuda_server_submit_mixed(bwacuda_ctx *c, const bwacuda_ext_job *ext_jobs, size_t n_ext,
                                           const bwacuda_rescue_job *rescue_jobs, size_t n_rescue,
                                           const bwacuda_scoring *sc, int w, int end_bonus, int zdrop, int minsc,
                                           int max_sc, uint64_t *req_id)
{
    if (!c || !sc || !req_id || (n_ext && !ext_jobs) || (n_rescue && !rescue_jobs) || n_ext + n_rescue == 0 ||
        w < 0 || max_sc < 1)
        return BWACUDA_EINVAL;
    int rc = validate_scoring(sc->m, sc->mat, sc->o_del, sc->e_del, sc->o_ins, sc->e_ins);
    if (rc) return rc;
    if (n_rescue == 0) return bwacuda_server_submit_extend(c, ext_jobs, n_ext, sc, w, end_bonus, zdrop, req_id);
    if (n_ext == 0) return bwacuda_server_submit_rescue(c, rescue_jobs, n_rescue, sc, minsc, max_sc, req_id);
    Request *re = new_ext_request(c, ext_jobs, n_ext, sc, w, end_bonus, zdrop);
    Request *rr = new_rescue_request(rescue_jobs, n_rescue, sc, minsc, max_sc);
    if (!re || !rr) {
        delete re;
        delete rr;
        return BWACUDA_ENOMEM;
    }
    return submit_all(c, re, rr, req_id);
}

extern "C" int bwacuda_server_wait(bwacuda_ctx *c, uint64_t req_id, void *out, int64_t timeout_us,
                                   int64_t *latency_ns)
{
    if (!c || !c->server || !out) return BWACUDA_EINVAL;
    ServerState *S = c->server;
    std::unique_lock<std::mutex> lk(S->mu);
    // a mixed request is its extension part then its rescue part, results in that order
    Request *parts[2] = {nullptr, nullptr};
    const auto mit = S->mixed.find(req_id);
    if (mit != S->mixed.end()) {
        auto a = S->reqs.find(mit->second.first), b = S->reqs.find(mit->second.second);
        if (a == S->reqs.end() || b == S->reqs.end()) return BWACUDA_EINVAL;
        parts[0] = a->second;
        parts[1] = b->second;
    } else {
        auto it = S->reqs.find(req_id);
        if (it == S->reqs.end()) return BWACUDA_EINVAL;
        parts[0] = it->second;
    }
    auto all_done = [&]() { return parts[0]->state == DONE && (!parts[1] || parts[1]->state == DONE); };
    if (!all_done()) {
        if (timeout_us == 0) return BWACUDA_EAGAIN;
        const auto deadline = Clock::now() + std::chrono::microseconds(timeout_us < 0 ? (int64_t)1 << 40 : timeout_us);
        while (!all_done()) {
            if (S->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !all_done())
                return BWACUDA_ETIMEOUT;
        }
    }
    // take the requests out of the table, copy their results without holding the
    // lock, then release their arena ranges
    int rc = BWACUDA_OK;
    for (Request *r : parts)
        if (r) {
            S->reqs.erase(r->id);
            if (rc == BWACUDA_OK) rc = r->rc;
        }
    if (parts[1]) S->mixed.erase(req_id);
    lk.unlock();
    if (rc == BWACUDA_OK) {
        cudaError_t e = cudaSetDevice(c->device);
        cudaStream_t rs = nullptr;
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&rs, cudaStreamNonBlocking);
        size_t at = 0;
        for (Request *r : parts) {
            if (!r || e != cudaSuccess) continue;
            const size_t rsz = r->kind == 0 ? sizeof(bwacuda_ext_result) : sizeof(bwacuda_rescue_result);
            e = cudaMemcpyAsync(static_cast<char *>(out) + at, S->d_arena + r->off + r->res_at, r->n * rsz,
                                cudaMemcpyDeviceToHost, rs);
            at += r->n * rsz;
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(rs);
        if (rs) cudaStreamDestroy(rs);
        if (e != cudaSuccess) rc = cuda_status(e);
    }
    if (latency_ns) {
        int64_t ns = 0;
        for (Request *r : parts)
            if (r) ns = std::max<int64_t>(ns, std::chrono::duration_cast<std::chrono::nanoseconds>(r->t_done - r->t_submit).count());
        *latency_ns = ns;
    }
    lk.lock();
    for (Request *r : parts)
        if (r) release_request(S, r);
    S->cv_work.notify_one();  // memory freed: admission may proceed
    return rc;
}

extern "C" int bwacuda_server_cells(bwacuda_ctx *c, uint64_t *ext_cells, uint64_t *rescue_cells)
{
    if (!c || !c->server) return BWACUDA_EINVAL;
    ServerState *S = c->server;
    std::lock_guard<std::mutex> g(S->mu);
    if (ext_cells) *ext_cells = S->served_ext_cells;
    if (rescue_cells) *rescue_cells = S->served_rescue_cells;
    return BWACUDA_OK;
}

extern "C" int bwacuda_server_stats(bwacuda_ctx *c, uint64_t *served_jobs, uint64_t *waves, uint64_t *queued)
{
    if (!c || !c->server) return BWACUDA_EINVAL;
    ServerState *S = c->server;
    std::lock_guard<std::mutex> g(S->mu);
    if (served_jobs) *served_jobs = S->served_jobs;
    if (waves) *waves = S->waves;
    if (queued) *queued = S->pending.size() + S->admitted.size();
    return BWACUDA_OK;
}
