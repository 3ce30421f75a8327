// tune.cu -- the autotuner: picks the launch shape of the batched extension
// path (threads per block, 32-job rounds per work grab, length-bucket width)
// and of the rescue kernels (wavefront lanes per job, or thread-per-job) by
// timing every candidate with CUDA events on a strided sample of the caller's
// device-resident batch.  The DP results do not depend on any of these knobs.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>

#include "kernels.h"
#include "runtime.h"

namespace bwacuda {
namespace {

// dst[k] = src[k * stride]: a sample spread over the whole batch (both job
// descriptor types are 32 bytes and address the caller's base buffer).
__global__ void tune_sample_kernel(const uint4 *__restrict__ src, uint64_t stride, uint32_t count,
                                   uint4 *__restrict__ dst)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        dst[2 * k] = src[2 * (uint64_t)k * stride];
        dst[2 * k + 1] = src[2 * (uint64_t)k * stride + 1];
    }
}

// Forward-pass rescue cells (qlen x tlen) of the sample.
__global__ void tune_rescue_cells_kernel(const bwacuda_dev_rescue_job *__restrict__ jobs, uint32_t n,
                                         unsigned long long *__restrict__ cells)
{
    unsigned long long s = 0;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        s += (unsigned long long)max(jobs[k].qlen, 0) * (unsigned long long)max(jobs[k].tlen, 0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(cells, s);
}

struct Timer {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~Timer()
    {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    }
    cudaError_t init()
    {
        cudaError_t e = cudaEventCreate(&e0);
        return e == cudaSuccess ? cudaEventCreate(&e1) : e;
    }
};

// Time `reps` runs of fn after one warm-up run; returns ms per run (or a negative BWACUDA code).
template <class Fn>
double time_runs(Timer &T, cudaStream_t s, int reps, const Fn &fn)
{
    int rc = fn();
    if (rc) return rc;
    cudaError_t e = cudaEventRecord(T.e0, s);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) {
        rc = fn();
        if (rc) return rc;
    }
    if (e == cudaSuccess) e = cudaEventRecord(T.e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(T.e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, T.e0, T.e1);
    if (e != cudaSuccess) return cuda_status(e);
    return (double)ms / reps;
}

// The sample's descriptors: the batch itself, or every stride-th job copied to tmp.
cudaError_t take_sample(const void *d_jobs, size_t n, size_t count, DevBuf &tmp, const void **jp, cudaStream_t s)
{
    if (count == n) {
        *jp = d_jobs;
        return cudaSuccess;
    }
    cudaError_t e = tmp.ensure(count * 32);
    if (e != cudaSuccess) return e;
    const uint32_t grid = (uint32_t)std::min<size_t>((count + 255) / 256, 4096);
    tune_sample_kernel<<<grid, 256, 0, s>>>(static_cast<const uint4 *>(d_jobs), (uint64_t)(n / count), (uint32_t)count,
                                            static_cast<uint4 *>(tmp.p));
    *jp = tmp.p;
    return cudaGetLastError();
}

}  // namespace
}  // namespace bwacuda

using namespace bwacuda;

extern "C" int bwacuda_get_tuning(bwacuda_ctx *c, bwacuda_tuning *out)
{
    if (!c || !out) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    int tb, grab, step;
    batched_get_tuning(c, &tb, &grab, &step);
    out->persist_block = tb;
    out->grab = grab;
    out->bucket_step = step;
    out->rescue_lanes = c->rescue_lanes;
    out->rescue_kernel = c->rescue_kernel;
    out->candidates = c->tune_candidates;
    out->ext_gcups = c->tuned_ext_gcups;
    out->rescue_gcups = c->tuned_rescue_gcups;
    const int lq = batched_get_long(c);
    out->long_qlen = lq == INT_MAX ? 0 : lq;
    out->long_lanes = c->long_lanes;
    out->rescue_pair = c->rescue_pair;
    out->reserved = 0;
    return BWACUDA_OK;
}

extern "C" int bwacuda_autotune_extend(bwacuda_ctx *c, const uint8_t *d_seq, const bwacuda_dev_ext_job *d_jobs,
                                       size_t n, const bwacuda_scoring *scp, int end_bonus, int zdrop, size_t sample,
                                       bwacuda_tuning *out)
{
    if (!c || !scp || !d_seq || !d_jobs || n == 0) return BWACUDA_EINVAL;
    {
        std::lock_guard<std::mutex> g(c->mu);
        int rc = validate_scoring(scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
        if (rc) return rc;
        if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
        if ((rc = batched_prepare(c)) != BWACUDA_OK) return rc;
        const size_t count = std::min(n, sample ? sample : (size_t)1 << 22);
        cudaStream_t s = c->stream;
        DevBuf tmp, dout;
        const void *jp = nullptr;
        cudaError_t e = take_sample(d_jobs, n, count, tmp, &jp, s);
        if (e == cudaSuccess) e = dout.ensure(count * sizeof(bwacuda_ext_result));
        Timer T;
        if (e == cudaSuccess) e = T.init();
        if (e != cudaSuccess) { tmp.release(); dout.release(); return cuda_status(e); }
        ExtParams P;
        P.sc = make_scoring(scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
        P.end_bonus = end_bonus;
        P.zdrop = zdrop;
        P.ug = ungapped_rule(c, scp->m, scp->mat, scp->o_del, scp->e_del, scp->o_ins, scp->e_ins);
        const bwacuda_stats saved = c->stats;
        // candidates run as the calls they tune do: replayed graphs when the context uses them
        // (each shape is captured on its untimed first run), plain stream launches otherwise
        const bool graphs = c->use_graphs;
        auto run = [&]() {
            return extend_device_batched(c, d_seq, static_cast<const bwacuda_dev_ext_job *>(jp), count, P,
                                         static_cast<bwacuda_ext_result *>(dout.p), s);
        };
        // one checked run: bad inputs fail here, and its cell count prices every candidate
        uint64_t cells = 0;
        rc = run();
        if (!rc) rc = collect_device_status(c, s, &cells);
        // Every shape is timed; among those within 1.5% of the fastest the one closest to the
        // default (1 round per grab, 32-column buckets, 128 threads) wins.  Device-resident the
        // near-ties are noise, but a host-buffer call runs every chunk's buckets separately,
        // where more buckets (narrower steps) and larger grabs add launches and bucket tails
        // (measured on 8.4M read-pair jobs: 31.8 ms end to end at the default shape, 37.2 ms at
        // 64 threads / 2 rounds / 16 columns, the same 27.3 ms device-resident).
        struct Cand {
            int tb, gr, st;
            double ms;
        };
        Cand cands[36];
        int ncand = 0;
        static const int kSteps[] = {16, 32, 64}, kBlocks[] = {32, 64, 128, 256}, kGrabs[] = {1, 2, 4};
        for (int st : kSteps) {
            if (rc) break;
            if ((rc = batched_set_bucket_step(c, st)) != BWACUDA_OK) break;
            for (int tb : kBlocks) {
                if (rc) break;
                batched_set_block(c, tb);
                for (int gr : kGrabs) {
                    batched_set_grab(c, gr);
                    const double ms = time_runs(T, s, 2, run);
                    if (ms < 0) { rc = (int)ms; break; }
                    cands[ncand++] = Cand{tb, gr, st, ms};
                }
            }
        }
        double best_ms = 0;
        for (int i = 0; i < ncand; ++i)
            if (best_ms == 0 || cands[i].ms < best_ms) best_ms = cands[i].ms;
        int best[3] = {128, 1, 32};
        int best_pen = 1 << 30;
        double chosen_ms = 0;
        for (int i = 0; i < ncand; ++i) {
            const Cand &cd = cands[i];
            if (cd.ms > best_ms * 1.015) continue;
            const int pen = (cd.gr != 1) * 4 + (cd.st != 32) * 2 + (cd.tb != 128);
            if (pen < best_pen || (pen == best_pen && cd.ms < chosen_ms)) {
                best_pen = pen;
                chosen_ms = cd.ms;
                best[0] = cd.tb; best[1] = cd.gr; best[2] = cd.st;
            }
        }
        best_ms = chosen_ms;
        if (!rc) rc = batched_set_bucket_step(c, best[2]);
        if (!rc) rc = batched_set_block(c, best[0]);
        if (!rc) rc = batched_set_grab(c, best[1]);
        // Then the group-per-job kernel against thread-per-job on the longer buckets: the query
        // length from which buckets switch kernels (225, 193 or 129) by lanes per job (8, 16 or
        // 32), kept only when more than 1.5% faster than thread-per-job at the chosen shape.
        const int long0 = batched_get_long(c), lanes0 = c->long_lanes;
        if (!rc) rc = batched_set_long(c, INT_MAX);
        double tpj_ms = rc ? 0 : time_runs(T, s, 2, run);
        if (tpj_ms < 0) rc = (int)tpj_ms;
        int long_best = INT_MAX, lanes_best = lanes0;
        double long_ms = 0;
        static const int kLongQ[] = {225, 193, 129}, kLanes[] = {8, 16, 32};
        for (int lq : kLongQ) {
            if (rc) break;
            if ((rc = batched_set_long(c, lq)) != BWACUDA_OK) break;
            for (int ln : kLanes) {
                batched_set_long_lanes(c, ln);
                const double ms = time_runs(T, s, 2, run);
                if (ms < 0) { rc = (int)ms; break; }
                ++ncand;
                if (long_ms == 0 || ms < long_ms) { long_ms = ms; long_best = lq; lanes_best = ln; }
            }
        }
        if (!rc && long_ms > 0 && long_ms * 1.015 < tpj_ms) {
            best_ms = long_ms;
        } else {
            long_best = INT_MAX;
            lanes_best = lanes0;
            if (tpj_ms > 0) best_ms = std::min(best_ms, tpj_ms);
        }
        if (!rc) rc = batched_set_long(c, long_best);
        if (!rc) rc = batched_set_long_lanes(c, lanes_best);
        if (rc) {
            batched_set_long(c, long0);
            batched_set_long_lanes(c, lanes0);
        }
        uint64_t dummy = 0;
        const int st = collect_device_status(c, s, &dummy);
        if (!rc) rc = st;
        c->use_graphs = graphs;
        c->stats = saved;
        tmp.release();
        dout.release();
        if (rc) return rc;
        c->tune_candidates = ncand;
        c->tuned_ext_gcups = best_ms > 0 ? (double)cells / (best_ms * 1e-3) / 1e9 : 0.0;
    }
    return out ? bwacuda_get_tuning(c, out) : BWACUDA_OK;
}

extern "C" int bwacuda_autotune_rescue(bwacuda_ctx *c, const uint8_t *d_seq, const bwacuda_dev_rescue_job *d_jobs,
                                       size_t n, const bwacuda_scoring *scp, int minsc, int max_sc, size_t sample,
                                       bwacuda_tuning *out)
{
    if (!c || !scp || !d_seq || !d_jobs || n == 0) return BWACUDA_EINVAL;
    {
        std::lock_guard<std::mutex> g(c->mu);
        if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
        const size_t count = std::min(n, sample ? sample : (size_t)262144);
        cudaStream_t s = c->stream;
        DevBuf tmp, dout, dcells;
        const void *jp = nullptr;
        cudaError_t e = take_sample(d_jobs, n, count, tmp, &jp, s);
        if (e == cudaSuccess) e = dout.ensure(count * sizeof(bwacuda_rescue_result));
        if (e == cudaSuccess) e = dcells.ensure(16);
        if (e == cudaSuccess) e = cudaMemsetAsync(dcells.p, 0, 8, s);
        if (e == cudaSuccess) {
            const uint32_t grid = (uint32_t)std::min<size_t>((count + 255) / 256, 1024);
            tune_rescue_cells_kernel<<<grid, 256, 0, s>>>(static_cast<const bwacuda_dev_rescue_job *>(jp),
                                                         (uint32_t)count, static_cast<unsigned long long *>(dcells.p));
            e = cudaGetLastError();
        }
        unsigned long long cells = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&cells, dcells.p, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        Timer T;
        if (e == cudaSuccess) e = T.init();
        if (e != cudaSuccess) { tmp.release(); dout.release(); dcells.release(); return cuda_status(e); }
        const bwacuda_stats saved = c->stats;
        const int kern0 = c->rescue_kernel, lanes0 = c->rescue_lanes;
        const int pair0 = c->rescue_pair;
        auto run = [&]() {
            return ksw_align2_device_locked(c, d_seq, static_cast<const bwacuda_dev_rescue_job *>(jp), count, scp,
                                            minsc, max_sc, 0, 0, static_cast<bwacuda_rescue_result *>(dout.p), s);
        };
        // one checked run (errors surface here)
        uint64_t dummy = 0;
        int rc = run();
        if (!rc) rc = collect_device_status(c, s, &dummy);
        // the paired candidates keep the 32-bit wavefront at 8 lanes for the jobs they leave
        struct Cand { int kernel, lanes, pair; } cands[] = {
            {BWACUDA_RESCUE_AUTO, 8, 0}, {BWACUDA_RESCUE_AUTO, 16, 0}, {BWACUDA_RESCUE_AUTO, 32, 0},
            {BWACUDA_RESCUE_TPJ, 16, 0}, {BWACUDA_RESCUE_AUTO, 8, 4}, {BWACUDA_RESCUE_AUTO, 8, 8},
            {BWACUDA_RESCUE_AUTO, 8, 16}};
        double best_ms = 0;
        Cand best = {kern0, lanes0, pair0};
        int ncand = 0;
        for (const Cand &cd : cands) {
            if (rc) break;
            c->rescue_kernel = cd.kernel;
            c->rescue_lanes = cd.lanes;
            c->rescue_pair = cd.pair;
            const double ms = time_runs(T, s, 2, run);
            if (ms < 0) { rc = (int)ms; break; }
            ++ncand;
            if (best_ms == 0 || ms < best_ms) { best_ms = ms; best = cd; }
        }
        const int st = collect_device_status(c, s, &dummy);
        if (!rc) rc = st;
        c->rescue_kernel = rc ? kern0 : best.kernel;
        c->rescue_lanes = rc ? lanes0 : best.lanes;
        c->rescue_pair = rc ? pair0 : best.pair;
        c->stats = saved;
        tmp.release();
        dout.release();
        dcells.release();
        if (rc) return rc;
        c->tune_candidates = ncand;
        c->tuned_rescue_gcups = best_ms > 0 ? (double)cells / (best_ms * 1e-3) / 1e9 : 0.0;
    }
    return out ? bwacuda_get_tuning(c, out) : BWACUDA_OK;
}
