// retry.cu -- the band-doubling retry of bwa-mem's extension loop on the device
// (run_side, crates/bwa-mem/src/across.rs:1357-1500; bwamem.cpp's MAX_BAND_TRY).
//
// Round 0 runs every job on the batched path at its own band w.  An acceptance
// kernel then applies the reference's test to each job of the round,
//     accept = score == prev || max_off < (w >> 1) + (w >> 2) || last round,
// scatters the round's results to the caller's output (original job order),
// records the band each job ran with, and compacts the rejected jobs into the
// next round's descriptor list with the band doubled and prev = this score.  One
// 4-byte readback sizes the next round.  The jobs never leave the GPU between
// rounds; a job's result depends only on (query, target, h0, w), so the order in
// which the compaction places them does not matter.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>

#include "kernels.h"
#include "runtime.h"

namespace bwacuda {

namespace {

// Round r's acceptance over m jobs.  map == nullptr means the round's job s is job s
// (round 0, whose results already sit in out).  next_* receive the rejected jobs.
__global__ void retry_accept_kernel(const bwacuda_dev_ext_job *__restrict__ desc, const uint32_t *__restrict__ map,
                                    const bwacuda_ext_result *__restrict__ res, uint32_t m, bool last,
                                    int32_t *__restrict__ prev, bwacuda_ext_result *__restrict__ out,
                                    int32_t *__restrict__ w_used, bwacuda_dev_ext_job *__restrict__ next_desc,
                                    uint32_t *__restrict__ next_map, uint32_t *__restrict__ next_cnt)
{
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < m; s += gridDim.x * blockDim.x) {
        const uint32_t k = map ? map[s] : s;
        const bwacuda_ext_result r = res[s];
        bwacuda_dev_ext_job D = desc[s];
        const int w = D.w;
        const bool accept = r.score == prev[k] || r.max_off < (w >> 1) + (w >> 2) || last;
        if (map) out[k] = r;
        if (w_used) w_used[k] = w;
        if (!accept) {
            prev[k] = r.score;
            const uint32_t slot = atomicAdd(next_cnt, 1u);
            D.w = w >= (1 << 30) ? 0x7fffffff : w << 1;
            next_desc[slot] = D;
            next_map[slot] = k;
        }
    }
}

__global__ void retry_prev_init_kernel(const int32_t *__restrict__ src, uint32_t n, int32_t *__restrict__ prev)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        prev[k] = src ? src[k] : -1;
}

}  // namespace

struct RetryState {
    DevBuf desc[2], map[2], prev, res, cnt;
    HostBuf h_cnt;
    // host-buffer entry
    DevBuf seq, jobs, out, wused, gtmp, dprev;
    HostBuf hstage, htmp;
};

void retry_release(bwacuda_ctx *c)
{
    if (!c->retry) return;
    RetryState &R = *c->retry;
    for (int i = 0; i < 2; ++i) { R.desc[i].release(); R.map[i].release(); }
    R.prev.release(); R.res.release(); R.cnt.release(); R.h_cnt.release();
    R.seq.release(); R.jobs.release(); R.out.release(); R.wused.release(); R.gtmp.release(); R.dprev.release();
    R.hstage.release(); R.htmp.release();
    delete c->retry;
    c->retry = nullptr;
}

namespace {

// The rounds over n device-resident jobs (context lock held, batched path prepared).
int retry_rounds(bwacuda_ctx *c, const uint8_t *d_seq, const bwacuda_dev_ext_job *d_jobs, size_t n,
                 const ExtParams &P, int max_tries, const int32_t *d_prev_in, bwacuda_ext_result *d_out,
                 int32_t *d_wused, cudaStream_t s)
{
    RetryState &R = *c->retry;
    cudaError_t e;
    if ((e = R.prev.ensure(n * 4 + 16)) != cudaSuccess) return cuda_status(e);
    if ((e = R.cnt.ensure(64)) != cudaSuccess) return cuda_status(e);
    if ((e = R.h_cnt.ensure(64)) != cudaSuccess) return cuda_status(e);
    const int nsm = batched_nsm(c);
    const uint32_t grid = (uint32_t)std::min<size_t>((n + 255) / 256, (size_t)nsm * 8);
    int32_t *prev = static_cast<int32_t *>(R.prev.p);
    retry_prev_init_kernel<<<grid, 256, 0, s>>>(d_prev_in, (uint32_t)n, prev);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
    // round 0: every job, results straight into d_out
    e = batched_enqueue(c, batched_slot_bufs(c, 0), d_seq, d_jobs, n, P, d_out, s, nullptr, nullptr);
    if (e != cudaSuccess) return cuda_status(e);
    c->stats.kernel_launches += 4 + (uint64_t)batched_bucket_count(c);
    const bwacuda_dev_ext_job *desc = d_jobs;
    const uint32_t *map = nullptr;
    const bwacuda_ext_result *res = d_out;
    size_t m = n;
    uint32_t *cnt = static_cast<uint32_t *>(R.cnt.p);
    for (int round = 0; round < max_tries && m > 0; ++round) {
        const bool last = round + 1 == max_tries;
        const int nx = round & 1;
        if ((e = R.desc[nx].ensure(m * sizeof(bwacuda_dev_ext_job) + 16)) != cudaSuccess) return cuda_status(e);
        if ((e = R.map[nx].ensure(m * 4 + 16)) != cudaSuccess) return cuda_status(e);
        if ((e = cudaMemsetAsync(cnt, 0, 4, s)) != cudaSuccess) return cuda_status(e);
        const uint32_t g = (uint32_t)std::min<size_t>((m + 255) / 256, (size_t)nsm * 8);
        retry_accept_kernel<<<g, 256, 0, s>>>(desc, map, res, (uint32_t)m, last, prev, d_out, d_wused,
                                              static_cast<bwacuda_dev_ext_job *>(R.desc[nx].p),
                                              static_cast<uint32_t *>(R.map[nx].p), cnt);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
        c->stats.kernel_launches += 1;
        if (last) break;
        if ((e = cudaMemcpyAsync(R.h_cnt.p, cnt, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_status(e);
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e);
        m = *static_cast<const uint32_t *>(R.h_cnt.p);
        if (m == 0) break;
        // the next round over the rejected jobs, results compact in R.res
        if ((e = R.res.ensure(m * sizeof(bwacuda_ext_result) + 16)) != cudaSuccess) return cuda_status(e);
        desc = static_cast<const bwacuda_dev_ext_job *>(R.desc[nx].p);
        map = static_cast<const uint32_t *>(R.map[nx].p);
        res = static_cast<const bwacuda_ext_result *>(R.res.p);
        e = batched_enqueue(c, batched_slot_bufs(c, 1), d_seq, desc, m, P,
                            static_cast<bwacuda_ext_result *>(R.res.p), s, nullptr, nullptr);
        if (e != cudaSuccess) return cuda_status(e);
        c->stats.kernel_launches += 4 + (uint64_t)batched_bucket_count(c);
        c->stats.ext_retry_jobs += m;
    }
    return BWACUDA_OK;
}

int retry_prepare(bwacuda_ctx *c)
{
    int rc = batched_prepare(c);
    if (rc) return rc;
    if (!c->retry) {
        c->retry = new (std::nothrow) RetryState();
        if (!c->retry) return BWACUDA_ENOMEM;
    }
    return BWACUDA_OK;
}

}  // namespace

}  // namespace bwacuda

using namespace bwacuda;

extern "C" int bwacuda_extend_retry_device(bwacuda_ctx *c, const uint8_t *d_seq, const bwacuda_dev_ext_job *d_jobs,
                                           size_t n, const bwacuda_scoring *scp, int end_bonus, int zdrop,
                                           int max_tries, const int32_t *d_prev, bwacuda_ext_result *d_out,
                                           int32_t *d_w_used, void *stream)
{
    if (!c || !scp) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    int rc = validate_scoring(scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
    if (rc) return rc;
    if (max_tries < 1 || max_tries > 8) return BWACUDA_EINVAL;
    if (n == 0) return BWACUDA_OK;
    if (!d_seq || !d_jobs || !d_out) return BWACUDA_EINVAL;
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    if ((rc = retry_prepare(c)) != BWACUDA_OK) return rc;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    ExtParams P;
    P.sc = make_scoring(scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
    P.end_bonus = end_bonus;
    P.zdrop = zdrop;
    P.ug = ungapped_rule(c, scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
    // consecutive pieces on the stream (every job's rounds are its own)
    for (size_t off = 0; off < n && rc == BWACUDA_OK; off += c->dev_piece) {
        const size_t m = std::min(c->dev_piece, n - off);
        rc = retry_rounds(c, d_seq, d_jobs + off, m, P, max_tries, d_prev ? d_prev + off : nullptr, d_out + off,
                          d_w_used ? d_w_used + off : nullptr, s);
    }
    c->stats.ext_jobs += n;
    c->dev_pending_stream = s;
    return rc;
}

extern "C" int bwacuda_extend_batch_retry(bwacuda_ctx *c, const bwacuda_ext_job *jobs, size_t n, int m,
                                          const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins, int w,
                                          int end_bonus, int zdrop, int max_tries, const int32_t *prev,
                                          bwacuda_ext_result *out, int32_t *w_used)
{
    if (!c) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    int rc = validate_scoring(m, mat, o_del, e_del, o_ins, e_ins);
    if (rc) return rc;
    if (w < 0 || max_tries < 1 || max_tries > 8 || (n && (!jobs || !out))) return BWACUDA_EINVAL;
    if (n == 0) return BWACUDA_OK;
    if (n > ((size_t)1 << 28)) return BWACUDA_EUNSUPPORTED;  // one gather of 16 chunks at most
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    if ((rc = retry_prepare(c)) != BWACUDA_OK) return rc;
    RetryState &R = *c->retry;
    cudaStream_t s = c->stream;
    cudaError_t e;
    const bool device_gather = c->host_gather == BWACUDA_GATHER_DEVICE ||
                               (c->host_gather == BWACUDA_GATHER_AUTO && c->pageable_access);
    if (device_gather) {
        if ((rc = ats_gather_ext(c, jobs, n, w, R.seq, R.jobs, R.gtmp, R.htmp, s)) != BWACUDA_OK) return rc;
    } else {
        // host packing: validate, lay out, copy through pinned staging
        uint64_t bytes = 0;
        for (size_t k = 0; k < n; ++k) {
            const bwacuda_ext_job &J = jobs[k];
            if (J.qlen < 0 || J.tlen < 0 || J.h0 <= 0 || (J.qlen && !J.query) || (J.tlen && !J.target))
                return BWACUDA_EINVAL;
            bytes += (uint64_t)J.qlen + (uint64_t)J.tlen;
        }
        const size_t jb = n * sizeof(bwacuda_dev_ext_job);
        if ((e = R.hstage.ensure(bytes + jb + 16)) != cudaSuccess) return cuda_status(e);
        if ((e = R.seq.ensure(bytes + 16)) != cudaSuccess) return cuda_status(e);
        if ((e = R.jobs.ensure(jb)) != cudaSuccess) return cuda_status(e);
        uint8_t *hs = static_cast<uint8_t *>(R.hstage.p);
        bwacuda_dev_ext_job *hj = reinterpret_cast<bwacuda_dev_ext_job *>(hs + ((bytes + 15) & ~(uint64_t)15));
        uint64_t off = 0;
        for (size_t k = 0; k < n; ++k) {
            const bwacuda_ext_job &J = jobs[k];
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
        if (bytes && (e = cudaMemcpyAsync(R.seq.p, hs, bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess) return cuda_status(e);
        if ((e = cudaMemcpyAsync(R.jobs.p, hj, jb, cudaMemcpyHostToDevice, s)) != cudaSuccess) return cuda_status(e);
        c->stats.h2d_bytes += bytes + jb;
    }
    if ((e = R.out.ensure(n * sizeof(bwacuda_ext_result))) != cudaSuccess) return cuda_status(e);
    if ((e = R.wused.ensure(n * 4 + 16)) != cudaSuccess) return cuda_status(e);
    const int32_t *dprev = nullptr;
    if (prev) {
        if ((e = R.dprev.ensure(n * 4 + 16)) != cudaSuccess) return cuda_status(e);
        if ((e = cudaMemcpyAsync(R.dprev.p, prev, n * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess) return cuda_status(e);
        dprev = static_cast<const int32_t *>(R.dprev.p);
    }
    ExtParams P;
    P.sc = make_scoring(m, mat, o_del, e_del, o_ins, e_ins);
    P.end_bonus = end_bonus;
    P.zdrop = zdrop;
    P.ug = ungapped_rule(c, m, mat, o_del, e_del, o_ins, e_ins);
    rc = retry_rounds(c, static_cast<const uint8_t *>(R.seq.p), static_cast<const bwacuda_dev_ext_job *>(R.jobs.p), n,
                      P, max_tries, dprev, static_cast<bwacuda_ext_result *>(R.out.p),
                      static_cast<int32_t *>(R.wused.p), s);
    if (rc) {
        uint64_t dummy;
        collect_device_status(c, s, &dummy);
        return rc;
    }
    if ((e = cudaMemcpyAsync(out, R.out.p, n * sizeof(bwacuda_ext_result), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_status(e);
    if (w_used && (e = cudaMemcpyAsync(w_used, R.wused.p, n * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_status(e);
    c->stats.d2h_bytes += n * (sizeof(bwacuda_ext_result) + (w_used ? 4 : 0));
    uint64_t cells = 0;
    rc = collect_device_status(c, s, &cells);  // synchronises the stream
    c->stats.ext_jobs += n;
    c->stats.ext_cells += cells;
    return rc;
}
