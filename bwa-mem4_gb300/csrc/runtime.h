// runtime.h -- host runtime of the bwa-cuda engine: buffers, worker pool, context.
#pragma once
#include <cuda_runtime.h>

#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/bwacuda.h"
#include "common.cuh"

namespace bwacuda {

// Grow-only device buffer.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes);
    void release();
};

// Grow-only pinned host buffer.
struct HostBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes);
    void release();
};

// Fixed pool of host threads; run(fn) calls fn(id) once on every worker
// (id 0 on the caller's thread) and returns when all are done.
class WorkerPool {
public:
    explicit WorkerPool(int n);
    ~WorkerPool();
    void run(const std::function<void(int)> &fn);
    int size() const { return nthreads_; }

private:
    void loop(int id);
    std::vector<std::thread> threads_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::function<void(int)> *fn_ = nullptr;
    uint64_t gen_ = 0;
    int pending_ = 0;
    int nthreads_ = 1;
    bool stop_ = false;
};

// One staging slot of the host-buffer pipeline.
struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    HostBuf h_seq, h_jobs, h_out, h_aux;
    DevBuf d_seq, d_jobs, d_out, d_aux, d_scratch;
    DevBuf d_xl;  // group-per-job extension: work words and the deferred-job list
};

struct BatchedState;  // batched path (batched.cu)
struct ServerState;   // serving loop (server.cu)
struct AtsState;      // device-side gather of host buffers (ats.cu)
struct GlobalState;   // ksw_global2 buffers (global.cu)
struct RetryState;    // band-doubling retry buffers (retry.cu)
struct RefState;      // reference in HBM for rescue windows (window.cu)

int cuda_status(cudaError_t e);
Scoring make_scoring(int m, const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins);
int validate_scoring(int m, const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins);
int ext_bin_label(int qlen, int tlen, int h0, int m, const int8_t *mat);
UngappedRule ungapped_rule(const bwacuda_ctx *c, int m, const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins);

}  // namespace bwacuda

struct bwacuda_ctx {
    explicit bwacuda_ctx(int dev);
    int device;
    std::mutex mu;
    cudaStream_t stream = nullptr;  // default stream of device-resident calls
    cudaStream_t dev_pending_stream = nullptr;
    bwacuda::Slot slot[2];
    bwacuda::DevBuf d_misc;   // error flags, counters
    bwacuda::HostBuf h_misc;
    bwacuda::DevBuf d_dev_aux, d_dev_scratch;
    bwacuda::DevBuf d_dev_xl;  // group-per-job extension of device-resident plain calls
    bwacuda::WorkerPool pool;
    bwacuda_stats stats{};
    int ext_path = BWACUDA_PATH_BATCHED;
    bool use_graphs = true;
    int rescue_kernel = BWACUDA_RESCUE_AUTO;
    int rescue_lanes = 16;  // lanes per job of the register wavefront (8, 16, 32)
    int rescue_pair = 0;  // lanes of a group holding two byte-range jobs (rescue_wf2.cuh): 4, 8, 16; 0 off
    bool ungapped = false;  // ungapped-diagonal fast path on the batched extension path
    int long_lanes = 16;    // lanes per job of the group-per-job extension kernel (8, 16, 32)
    int long_slide = 1;     // thread-per-job window kernel on the open-ended buckets: 0 off, 1 auto, 2 always
    int tune_candidates = 0;        // last autotune call
    double tuned_ext_gcups = 0.0;   // best candidates' rates on their samples
    double tuned_rescue_gcups = 0.0;
    size_t chunk_jobs = 1048576;
    size_t dev_piece = size_t(1) << 30;  // jobs per launch sequence of a device-resident call
    int host_gather = BWACUDA_GATHER_AUTO;
    bool pageable_access = false;  // the device reads pageable host memory (host page tables)
    bwacuda::BatchedState *batched = nullptr;
    bwacuda::AtsState *ats = nullptr;
    bwacuda::GlobalState *global = nullptr;
    bwacuda::RetryState *retry = nullptr;
    bwacuda::RefState *ref = nullptr;
    bwacuda::ServerState *server = nullptr;
};

namespace bwacuda {

int collect_device_status(bwacuda_ctx *c, cudaStream_t s, uint64_t *cells);
struct RescueLaunch;
cudaError_t rescue_narrow_launch(bwacuda_ctx *c, const RescueLaunch &L);

// One packed chunk of extension jobs, resident on the device.
struct ExtChunkInfo {
    const uint8_t *d_seq;
    const bwacuda_dev_ext_job *d_jobs;
    const uint32_t *d_wide;  // indices of jobs needing int32 cells (plain path)
    size_t n;
    uint32_t nwide;
    int qmax;
    int w;  // the call's band
    ExtParams P;
    bwacuda_ext_result *d_out;
};
using ExtRunner = std::function<int(int slot, const ExtChunkInfo &info, cudaStream_t s)>;
int extend_host_pipeline(bwacuda_ctx *c, const bwacuda_ext_job *jobs, size_t n, int m, const int8_t *mat,
                         const ExtParams &P, int w, bwacuda_ext_result *out, const ExtRunner &run);
int extend_batch_host(bwacuda_ctx *c, const bwacuda_ext_job *jobs, size_t n, int m, const int8_t *mat,
                      int o_del, int e_del, int o_ins, int e_ins, int w, int end_bonus, int zdrop,
                      bwacuda_ext_result *out);

// batched.cu
int extend_batch_host_batched(bwacuda_ctx *c, const bwacuda_ext_job *jobs, size_t n, int m, const int8_t *mat,
                              const ExtParams &P, int w, bwacuda_ext_result *out);
int extend_device_batched(bwacuda_ctx *c, const uint8_t *d_seq, const bwacuda_dev_ext_job *d_jobs, size_t n,
                          const ExtParams &P, bwacuda_ext_result *d_out, cudaStream_t s);
void batched_release(bwacuda_ctx *c);
int batched_set_block(bwacuda_ctx *c, int tb);
int batched_set_grab(bwacuda_ctx *c, int grab);
int batched_set_bucket_step(bwacuda_ctx *c, int step);
void batched_get_tuning(bwacuda_ctx *c, int *tb, int *grab, int *step);
int batched_set_long(bwacuda_ctx *c, int long_qlo);
int batched_get_long(bwacuda_ctx *c);
int batched_set_long_lanes(bwacuda_ctx *c, int lanes);
int batched_set_long_slide(bwacuda_ctx *c, int mode);

struct BatchBufs;
int batched_prepare(bwacuda_ctx *c);
BatchBufs *batchbufs_create();
void batchbufs_destroy(BatchBufs *bb);
cudaError_t batched_enqueue(bwacuda_ctx *c, BatchBufs *bb, const uint8_t *d_seq, const bwacuda_dev_ext_job *d_jobs,
                            size_t n, const ExtParams &P, bwacuda_ext_result *d_out, cudaStream_t s, uint32_t *err,
                            unsigned long long *cells);
BatchBufs *batched_slot_bufs(bwacuda_ctx *c, int slot);  // work buffers of host-pipeline slot 0 or 1
cudaError_t batched_reserve(BatchBufs *bb, size_t n);
// registers / threads per SM that bb's bucket kernels leave free (0, 0: none)
void batched_set_reserve(BatchBufs *bb, int regs, int threads);
int batched_nsm(bwacuda_ctx *c);
int batched_bucket_count(bwacuda_ctx *c);

// ats.cu
int extend_batch_ats(bwacuda_ctx *c, const bwacuda_ext_job *jobs, size_t n, int m, const int8_t *mat,
                     const ExtParams &P, int w, bwacuda_ext_result *out);
void ats_release(bwacuda_ctx *c);
int ats_gather_ext(bwacuda_ctx *c, const bwacuda_ext_job *hj, size_t n, int w, DevBuf &seq, DevBuf &djobs,
                   DevBuf &tmp, HostBuf &htmp, cudaStream_t s);

// retry.cu
void retry_release(bwacuda_ctx *c);

// window.cu
void ref_release(bwacuda_ctx *c);

// global.cu
void global_release(bwacuda_ctx *c);

// server.cu
void server_shutdown(bwacuda_ctx *c);

// abi.cu: group-per-job launches over the jobs of one call that the thread-per-job kernels
// leave (qlen >= min16 in 16-bit cells, qlen >= min32 in 32-bit cells; INT_MAX: none)
int launch_long_unbucketed(bwacuda_ctx *c, DevBuf &xl, const uint8_t *seq, const bwacuda_dev_ext_job *jobs, size_t n,
                           const ExtParams &P, bwacuda_ext_result *out, int min16, int min32, int ring, cudaStream_t s);

// abi.cu (device-resident rescue with the context lock held)
int ksw_align2_device_locked(bwacuda_ctx *c, const uint8_t *d_seq, const bwacuda_dev_rescue_job *d_jobs, size_t n,
                             const bwacuda_scoring *scp, int minsc, int max_sc, int mode, int lanes,
                             bwacuda_rescue_result *d_out, void *stream);

}  // namespace bwacuda
