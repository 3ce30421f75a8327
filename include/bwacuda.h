/*
 * bwacuda.h -- C ABI of the GB300 (sm_103a) Smith-Waterman engine for the
 * bwa-mem4 seed-extension and mate-rescue hot path.
 *
 * The entry points replace, one for one, the reference's Rust interfaces
 * (paths relative to the reference project root):
 *
 *   bwacuda_backend_name        SwBackend::name            crates/bwa-extend/src/lib.rs:85
 *   bwacuda_extend              SwBackend::extend          crates/bwa-extend/src/lib.rs:115-129
 *   bwacuda_extend_batch        SwBackend::extend_batch    crates/bwa-extend/src/lib.rs:154-175
 *   bwacuda_ksw_align2_batch    bwa_neon::batched_ksw_align2  crates/bwa-neon/src/matesw.rs:299-309
 *   bwacuda_ksw_align2_scalar_batch  bwa_extend::ksw_align2 (per job)  crates/bwa-extend/src/sw.rs:1108-1185
 *   bwacuda_ksw_local_fwd_batch bwa_extend::ksw_local_fwd (per job)  crates/bwa-extend/src/sw.rs:921-1075
 *   bwacuda_ksw_global2_batch   bwa_extend::ksw_global2 (per job)    crates/bwa-extend/src/sw.rs:561-740
 *
 * Conventions (all entry points):
 *  - Plain pointers and sizes only.  The caller owns every input and output
 *    buffer; host-buffer calls bring the inputs to device memory (pinned
 *    staging and copies, or device loads from host memory, see
 *    BWACUDA_OPT_HOST_GATHER) and store every result before returning.
 *  - Bases are one byte per base, codes 0..m-1 (bwa: 0=A 1=C 2=G 3=T 4=N).
 *  - Return 0 on success or a negative BWACUDA_E* code; nothing throws across
 *    the ABI.  On error the output buffer contents are unspecified.
 *  - There is no CPU fallback: every job runs on the GPU or the call fails.
 *  - A context may be shared between threads: calls on one context are
 *    serialised by an internal lock.  Use one context per thread for overlap.
 *  - Results are bit-identical to the reference's integer semantics for every
 *    field.
 */
#ifndef BWACUDA_H
#define BWACUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BWACUDA_OK 0
#define BWACUDA_EINVAL (-1)       /* bad argument: m, gap extends <= 0, w < 0, h0 <= 0, max_sc <= 0, negative length */
#define BWACUDA_EBASE (-2)        /* a base code >= m in some query or target */
#define BWACUDA_ENOMEM (-3)       /* device or pinned host allocation failed */
#define BWACUDA_ECUDA (-4)        /* a CUDA runtime call failed */
#define BWACUDA_ETIMEOUT (-5)     /* a bounded device wait gave up */
#define BWACUDA_EUNSUPPORTED (-6) /* input beyond the kernels' limits (e.g. score range) */
#define BWACUDA_EBUSY (-7)        /* serving queue full / request not admitted */
#define BWACUDA_EAGAIN (-8)       /* serving request not finished yet */
#define BWACUDA_ESHORT (-9)       /* output buffer too small; the sizes it needs were written */

/* Largest alphabet the kernels' score profile holds. */
#define BWACUDA_MAX_M 7

/* crates/bwa-extend/src/lib.rs:181-195 ExtendJob */
typedef struct {
    const uint8_t *query;
    const uint8_t *target;
    int32_t qlen;
    int32_t tlen;
    int32_t h0;
} bwacuda_ext_job;

/* crates/bwa-extend/src/sw.rs:139-162 ExtendResult */
typedef struct {
    int32_t score, qle, tle, gtle, gscore, max_off;
} bwacuda_ext_result;

/* crates/bwa-neon/src/matesw.rs:104-116 KswJob */
typedef struct {
    const uint8_t *query;
    const uint8_t *target;
    int32_t qlen;
    int32_t tlen;
} bwacuda_rescue_job;

/* crates/bwa-extend/src/sw.rs:750-774 KswAlignResult */
typedef struct {
    int32_t score, qb, qe, tb, te, score2, te2;
} bwacuda_rescue_result;

/* crates/bwa-neon/src/matesw.rs:131-142 FwdJob (per-job minsc / endsc) */
typedef struct {
    const uint8_t *query;
    const uint8_t *target;
    int32_t qlen;
    int32_t tlen;
    int32_t minsc;
    int32_t endsc;
} bwacuda_fwd_job;

/* Return tuple of ksw_local_fwd, crates/bwa-extend/src/sw.rs:921-934 */
typedef struct {
    int32_t score, te, qe, score2, te2;
} bwacuda_fwd_result;

typedef struct bwacuda_ctx bwacuda_ctx;

/* Kernel family used for extension batches (bwacuda_set_option).  Both give the same
 * results; BATCHED (default) is several times faster on every workload measured. */
#define BWACUDA_OPT_EXT_PATH 1
#define BWACUDA_PATH_PLAIN 0   /* one launch per chunk, jobs in caller order */
#define BWACUDA_PATH_BATCHED 1 /* length-bucketed, persistent, graph-replayed (default) */
/* Jobs per device chunk (pipelining granularity of the host-buffer calls; default 1048576:
 * smaller chunks cost each length bucket's tail once more per chunk, which dominates when most
 * jobs are settled before the DP -- 23.1 against 16.1 ms per 8.4M read-pair jobs at 262144 with
 * BWACUDA_OPT_UNGAPPED).  Device-gather extension calls ramp up to it from 65536 jobs, doubling
 * chunk by chunk; bwacuda_ksw_global2_batch takes 4 x this many jobs per chunk, at most
 * 1,048,576. */
#define BWACUDA_OPT_CHUNK_JOBS 2
/* Batched device calls: replay a captured CUDA graph (1, default) or enqueue every call (0). */
#define BWACUDA_OPT_GRAPHS 3
/* Threads per block of the persistent extension kernels (32, 64, 128 or 256). */
#define BWACUDA_OPT_PERSIST_BLOCK 4
/* Mate-rescue kernel: register wavefront where it fits (AUTO) or thread-per-job (TPJ). */
#define BWACUDA_OPT_RESCUE_KERNEL 5
#define BWACUDA_RESCUE_AUTO 0
#define BWACUDA_RESCUE_TPJ 1
/* How host-buffer extension batches on the batched path reach the device.
 * DEVICE: GPU kernels read the caller's job array and sequence slices through
 * the host page tables (devices reporting cudaDevAttrPageableMemoryAccess, e.g.
 * Grace-Blackwell over NVLink-C2C) and write results straight into out[].
 * HOST: worker threads pack into pinned staging, then H2D/D2H copies.
 * AUTO (default): DEVICE where the device supports it, else HOST.  Asking for
 * DEVICE on a device without pageable access makes the calls fail with
 * BWACUDA_EUNSUPPORTED. */
#define BWACUDA_OPT_HOST_GATHER 6
#define BWACUDA_GATHER_AUTO 0
#define BWACUDA_GATHER_HOST 1
#define BWACUDA_GATHER_DEVICE 2
/* Batched extension: 32-job rounds a warp takes per work-counter grab (1, 2 or 4). */
#define BWACUDA_OPT_GRAB 7
/* Batched extension: query-length bucket width below 257 columns (16, 32 or 64). */
#define BWACUDA_OPT_BUCKET_STEP 8
/* Rescue register wavefront: lanes per job (8, 16 or 32). */
#define BWACUDA_OPT_RESCUE_LANES 9
/* Batched extension: settle jobs whose seed diagonal carries at most
 * (o_min + e_min - 1) / (a + b) mismatches in closed form before the DP (the
 * reference's ungapped_hit fast path, crates/bwa-neon/src/batched.rs:602-697;
 * uniform 5x5 matrices only).  Results are identical with it on or off; 0 = off
 * (default), 1 = on. */
#define BWACUDA_OPT_UNGAPPED 10
/* Device-resident calls (bwacuda_extend_device, bwacuda_ksw_align2_device,
 * bwacuda_extend_retry_device): jobs per
 * launch sequence, 1 .. 1,073,741,824 (default, the maximum: the sorts, scans and kernels
 * index a sequence's jobs in 32 bits).  A larger batch runs as consecutive sequences on
 * the call's stream, with the same results. */
#define BWACUDA_OPT_DEVICE_PIECE 11
/* Batched extension: query length from which the length buckets run the group-per-job
 * kernel (a group of 8, 16 or 32 lanes per job, the DP row processed in parallel across
 * the group) instead of thread-per-job; 0 (default) = only the open-ended buckets, which
 * hold the queries too long for a thread's shared-memory row.  Results never depend on it. */
#define BWACUDA_OPT_LONG_QLEN 12
/* Lanes per job of the group-per-job extension kernel: 8, 16 (default) or 32. */
#define BWACUDA_OPT_LONG_LANES 13
/* Mate rescue, register wavefront: 4, 8 or 16 = jobs whose every value fits a byte
 * (min(qlen, tlen) * max_sc <= 255, padded query <= 256 columns, bwa-shaped matrix) run two
 * per group of that many lanes, one in each 16-bit lane of the DPX instructions (4 lanes: the
 * most columns per lane); the others stay in the 32-bit wavefront.  1 = 4.  0 (default before
 * tuning) = one job per group.  Results never depend on it. */
#define BWACUDA_OPT_RESCUE_PAIR 14
/* Batched extension, the open-ended query-length buckets (queries too long for a thread's
 * shared-memory row): 1 (default) = a thread-per-job kernel holding each job's row in a window
 * of the band that slides along the query runs the jobs of bands up to 101 columns when the
 * bucket holds at least 32 jobs per SM, the group-per-job kernel the rest; 2 = the window
 * kernel whatever the bucket's size; 0 = the group-per-job kernel only.  Results never depend
 * on it. */
#define BWACUDA_OPT_LONG_SLIDE 15

int bwacuda_ctx_create(int device, bwacuda_ctx **out);
void bwacuda_ctx_destroy(bwacuda_ctx *ctx);
int bwacuda_set_option(bwacuda_ctx *ctx, int option, int64_t value);
const char *bwacuda_strerror(int code);
/* SwBackend::name, crates/bwa-extend/src/lib.rs:85 */
const char *bwacuda_backend_name(void);

/* SwBackend::extend: one banded seed extension (ksw_extend2). */
int bwacuda_extend(bwacuda_ctx *ctx, const uint8_t *query, int32_t qlen, const uint8_t *target,
                   int32_t tlen, int m, const int8_t *mat, int o_del, int e_del, int o_ins,
                   int e_ins, int w, int end_bonus, int zdrop, int h0, bwacuda_ext_result *out);

/* SwBackend::extend_batch: n extensions sharing scoring / band; out[k] is the
 * ksw_extend2 result of jobs[k].  A job with qlen == 0 yields the production
 * batched path's answer (crates/bwa-neon/src/batched.rs:1025-1039). */
int bwacuda_extend_batch(bwacuda_ctx *ctx, const bwacuda_ext_job *jobs, size_t n, int m,
                         const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins, int w,
                         int end_bonus, int zdrop, bwacuda_ext_result *out);

/* The extension loop of bwa-mem's run_side (crates/bwa-mem/src/across.rs:1357-1500)
 * with its band-doubling retry on the device: round r runs the still-active jobs
 * at band w << r; a job is accepted when score == prev, or max_off < (w >> 1) +
 * (w >> 2), or r + 1 == max_tries (bwa's MAX_BAND_TRY is 2); a rejected job's prev
 * becomes this round's score.  prev[k] is the job's value before round 0 (bwa-mem:
 * -1 for a left extension, h0 for a right one; NULL means -1 for every job).
 * out[k] is the accepted round's result, w_used[k] (may be NULL) its band.  The
 * jobs stay on the GPU across rounds (one count readback per round).  No
 * single-call counterpart in the reference, which loops on the host around
 * SwBackend::extend_batch.  At most 268,435,456 jobs per call (BWACUDA_EUNSUPPORTED
 * above). */
int bwacuda_extend_batch_retry(bwacuda_ctx *ctx, const bwacuda_ext_job *jobs, size_t n, int m,
                               const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins, int w,
                               int end_bonus, int zdrop, int max_tries, const int32_t *prev,
                               bwacuda_ext_result *out, int32_t *w_used);

/* batched_ksw_align2: forward pass with bwa's padding rule, then the reverse
 * start-recovery pass over the truncated reversed prefixes. */
int bwacuda_ksw_align2_batch(bwacuda_ctx *ctx, const bwacuda_rescue_job *jobs, size_t n, int m,
                             const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins,
                             int minsc, int max_sc, bwacuda_rescue_result *out);

/* ksw_align2 per job: the reverse pass scans the whole target with only
 * target[..=te] reversed.  lanes = 16 or 8 (query padding width), or 0 for
 * bwa's rule per job (qlen * max_sc < 250 ? 16 : 8). */
int bwacuda_ksw_align2_scalar_batch(bwacuda_ctx *ctx, const bwacuda_rescue_job *jobs, size_t n,
                                    int m, const int8_t *mat, int o_del, int e_del, int o_ins,
                                    int e_ins, int minsc, int max_sc, int lanes,
                                    bwacuda_rescue_result *out);

/* ksw_global2 (crates/bwa-extend/src/sw.rs:561-740), the banded global
 * alignment with traceback that bwa-mem's CIGAR step calls per alignment
 * (crates/bwa-mem/src/cigar.rs:446).  w is per job (the caller sizes it per
 * region).  Outputs: score[k]; job k's CIGAR runs (len << 4 | op, op 0=M 1=I
 * 2=D, left to right) are cigar[cigar_off[k] .. cigar_off[k+1]) with
 * cigar_off[0] = 0 (n + 1 entries).  When cigar_cap words are too few (or
 * cigar is NULL) the call still writes score and cigar_off and returns
 * BWACUDA_ESHORT; cigar_cap >= sum(qlen + tlen) always suffices.  A traceback
 * that the reference could not complete (its index leaves the matrix; its
 * caller's band sizing rules that out) makes the call return
 * BWACUDA_EUNSUPPORTED. */
typedef struct {
    const uint8_t *query;
    const uint8_t *target;
    int32_t qlen;
    int32_t tlen;
    int32_t w;
} bwacuda_global_job;

int bwacuda_ksw_global2_batch(bwacuda_ctx *ctx, const bwacuda_global_job *jobs, size_t n, int m,
                              const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins,
                              int32_t *score, uint64_t *cigar_off, uint32_t *cigar, size_t cigar_cap);

/* ------------------------------------------------------------------------
 * Mate rescue with the windows fetched on the device (matesw_collect +
 * bns_fetch_seq, crates/bwa-mem/src/pe.rs:232-270 and :596-679).  The reference
 * stays in HBM as bwa's 2-bit forward-strand .pac (4 bases per byte, first base
 * in the top two bits; position p >= l_pac reads the complement of forward base
 * 2*l_pac - 1 - p) with its contig table (offsets ascending from 0).  For each
 * request the device computes the orientation's window from the anchor, clamps it
 * to [0, 2*l_pac) and to the contig holding its midpoint, accepts it when that
 * contig is the anchor's and the window holds >= min_seed_len bases, unpacks it,
 * reverse-complements the mate where the orientation asks, and runs
 * batched_ksw_align2 on every accepted window.  Which orientations to request
 * (the pes / existing-region skip test) stays with the caller. */
int bwacuda_ref_set(bwacuda_ctx *ctx, const uint8_t *pac, int64_t l_pac, const int64_t *contig_offset,
                    const int32_t *contig_len, int32_t n_contigs);

typedef struct {
    const uint8_t *mate;  /* the mate read, codes 0..4, sequencing orientation */
    int32_t l_ms;         /* its length */
    int32_t orient;       /* pes index r: 0 FF, 1 FR, 2 RF, 3 RR */
    int64_t anchor_rb;    /* the anchor region's rb (2*l_pac space) */
    int32_t anchor_rid;   /* the anchor region's contig */
    int32_t low, high;    /* pes[r].low, pes[r].high */
} bwacuda_window_req;

typedef struct {
    int64_t rb, re;       /* the clamped window (2*l_pac space) */
    int32_t rid;          /* contig of the window's midpoint, -1 if none */
    int32_t valid;        /* 1: rid == anchor_rid and re - rb >= min_seed_len, aln holds the result */
    bwacuda_rescue_result aln;
} bwacuda_window_result;

int bwacuda_mate_rescue_windows(bwacuda_ctx *ctx, const bwacuda_window_req *reqs, size_t n, int m,
                                const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins, int minsc,
                                int max_sc, int min_seed_len, bwacuda_window_result *out);

/* ksw_local_fwd per job with its own minsc / endsc (lanes as above). */
int bwacuda_ksw_local_fwd_batch(bwacuda_ctx *ctx, const bwacuda_fwd_job *jobs, size_t n, int m,
                                const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins,
                                int max_sc, int lanes, bwacuda_fwd_result *out);

/* ------------------------------------------------------------------------
 * Device-resident form.  Inputs already in device memory: `d_seq` holds all
 * bases, each job addresses its query and target by byte offset.  Results are
 * written to device memory; the call is asynchronous on `stream` (a
 * cudaStream_t, NULL = the context's own stream) and returns after enqueueing.
 * bwacuda_ctx_sync() waits and reports device-side errors (bad base codes).
 * These calls carry no counterpart in the reference (which has no device);
 * they expose the same computation for callers that keep data in HBM.
 * ------------------------------------------------------------------------ */
typedef struct {
    uint64_t q_off, t_off;
    int32_t qlen, tlen;
    int32_t h0; /* extension: seed score */
    int32_t w;  /* extension: band half-width for this job */
} bwacuda_dev_ext_job;

typedef struct {
    uint64_t q_off, t_off;
    int32_t qlen, tlen;
    int32_t minsc, endsc; /* used by the forward-pass-only entry */
} bwacuda_dev_rescue_job;

typedef struct {
    int32_t m;
    int8_t mat[64]; /* m*m row-major, mat[t*m + q] */
    int32_t o_del, e_del, o_ins, e_ins;
} bwacuda_scoring;

int bwacuda_extend_device(bwacuda_ctx *ctx, const uint8_t *d_seq, const bwacuda_dev_ext_job *d_jobs,
                          size_t n, const bwacuda_scoring *sc, int end_bonus, int zdrop,
                          int path, bwacuda_ext_result *d_out, void *stream);
/* bwacuda_extend_batch_retry on device-resident jobs: round 0 uses each job's own
 * w (doubled per round); d_prev as prev above (NULL: -1); returns after the last
 * round is enqueued on stream (bwacuda_ctx_sync waits and reports errors).  Runs in
 * pieces of BWACUDA_OPT_DEVICE_PIECE jobs, as bwacuda_extend_device. */
int bwacuda_extend_retry_device(bwacuda_ctx *ctx, const uint8_t *d_seq, const bwacuda_dev_ext_job *d_jobs,
                                size_t n, const bwacuda_scoring *sc, int end_bonus, int zdrop, int max_tries,
                                const int32_t *d_prev, bwacuda_ext_result *d_out, int32_t *d_w_used,
                                void *stream);

/* mode 0 = batched_ksw_align2 semantics, 1 = scalar ksw_align2 (lanes as above). */
int bwacuda_ksw_align2_device(bwacuda_ctx *ctx, const uint8_t *d_seq,
                              const bwacuda_dev_rescue_job *d_jobs, size_t n,
                              const bwacuda_scoring *sc, int minsc, int max_sc, int mode,
                              int lanes, bwacuda_rescue_result *d_out, void *stream);

int bwacuda_ctx_sync(bwacuda_ctx *ctx);

/* bwacuda_ksw_align2_device for callers that cannot allocate device memory (a
 * pool allocator owns the whole device budget, or cudaMalloc/cudaFree would
 * synchronise a latency-critical stream).  No counterpart in the reference.
 * Same inputs, outputs and results as bwacuda_ksw_align2_device; the tracker
 * scratch lives in a static device array of this library (128 MiB of entries,
 * 4 MiB of offsets, held by every GPU that loads the library until exit).
 * A call may hold at most 524288 jobs and n * (max tlen / 2 + 2) <= 16 Mi
 * tracker entries, else it returns BWACUDA_EUNSUPPORTED without launching.
 * Synchronous: every call synchronises its stream before returning (errors
 * included).  Calls share the static array: calls that overlap on the GPU race.
 * The first call on a device resolves the array's address (cudaGetSymbolAddress)
 * and must come before any stream capture. */
int bwacuda_ksw_align2_device_noalloc(bwacuda_ctx *ctx, const uint8_t *d_seq,
                                      const bwacuda_dev_rescue_job *d_jobs, size_t n,
                                      const bwacuda_scoring *sc, int minsc, int max_sc, int mode,
                                      int lanes, bwacuda_rescue_result *d_out, void *stream);

/* ------------------------------------------------------------------------
 * Serving loop.  Requests (a batch of extension or rescue jobs each) are
 * submitted at any time and admitted to the GPU as space in a fixed HBM budget
 * frees up; admitted requests that share a scoring run together in the next
 * "wave" (continuous batching) and several waves overlap on the device.
 * Results stay in device memory until bwacuda_server_wait copies them out.
 * The job arrays and base buffers passed to a submit call must stay valid
 * until its wait returns.  No counterpart in the reference, which has no
 * device; each result equals what the batch calls return for the same jobs.
 * ------------------------------------------------------------------------ */
typedef struct {
    uint64_t hbm_budget_bytes; /* device arena for admitted requests (0 = 4 GiB); a pinned host arena of the same size mirrors it
                                  where the device cannot read pageable host memory.  Each wave slot also holds work buffers
                                  sized at start for waves of min(budget / 1024, 8M) jobs (about 80 bytes a job), grown
                                  twofold past that */
    int32_t max_waves;         /* waves in flight (0 = 3), one work-buffer slot each */
    int32_t max_requests;      /* requests held (queued, running or unread; 0 = 4096) */
} bwacuda_server_config;

int bwacuda_server_start(bwacuda_ctx *ctx, const bwacuda_server_config *cfg);
/* Finishes waves in flight; requests not yet launched end with BWACUDA_EBUSY. */
int bwacuda_server_stop(bwacuda_ctx *ctx);
/* BWACUDA_EBUSY when max_requests are held; BWACUDA_ENOMEM when the request
 * alone exceeds the HBM budget. */
int bwacuda_server_submit_extend(bwacuda_ctx *ctx, const bwacuda_ext_job *jobs, size_t n,
                                 const bwacuda_scoring *sc, int w, int end_bonus, int zdrop,
                                 uint64_t *req_id);
int bwacuda_server_submit_rescue(bwacuda_ctx *ctx, const bwacuda_rescue_job *jobs, size_t n,
                                 const bwacuda_scoring *sc, int minsc, int max_sc, uint64_t *req_id);
/* One request of both kinds (a chunk's extension and rescue jobs together): its wait
 * writes the n_ext extension results, then the n_rescue rescue results, into out, and
 * reports the later part's latency.  The parts are admitted together and join the
 * waves of their kind.  Either count may be 0 (then it is a one-kind request). */
int bwacuda_server_submit_mixed(bwacuda_ctx *ctx, const bwacuda_ext_job *ext_jobs, size_t n_ext,
                                const bwacuda_rescue_job *rescue_jobs, size_t n_rescue, const bwacuda_scoring *sc,
                                int w, int end_bonus, int zdrop, int minsc, int max_sc, uint64_t *req_id);
/* Waits up to timeout_us (0 = poll: BWACUDA_EAGAIN if not done; < 0 = no
 * limit, BWACUDA_ETIMEOUT when the limit passes), copies the n results into
 * out (bwacuda_ext_result or bwacuda_rescue_result) and releases the request.
 * latency_ns (may be NULL) receives submit-to-completion time. */
int bwacuda_server_wait(bwacuda_ctx *ctx, uint64_t req_id, void *out, int64_t timeout_us,
                        int64_t *latency_ns);
int bwacuda_server_stats(bwacuda_ctx *ctx, uint64_t *served_jobs, uint64_t *waves, uint64_t *queued);
/* Cells served since the loop started: extension cells as the kernels count them (one
 * inner-loop iteration of ksw_extend2 each), rescue cells as qlen x tlen per job. */
int bwacuda_server_cells(bwacuda_ctx *ctx, uint64_t *ext_cells, uint64_t *rescue_cells);

/* Counters accumulated since the context was created (or last reset). */
typedef struct {
    uint64_t ext_jobs, ext_cells;       /* cells = sum over rows of (end - beg) */
    uint64_t ext_bin_u8, ext_bin_i16, ext_bin_i32; /* reference 8/16-bit bin labels */
    uint64_t rescue_jobs, rescue_cells; /* cells = qlen * tlen of the forward pass */
    uint64_t rescue_width_u8, rescue_width_i16, rescue_width_i32; /* per call */
    uint64_t kernel_launches;
    uint64_t h2d_bytes, d2h_bytes;
    uint64_t global_jobs, global_cells; /* ksw_global2: cells = sum over rows of the band width */
    uint64_t ext_retry_jobs;            /* band-doubling retry: jobs run again at a wider band */
} bwacuda_stats;

int bwacuda_get_stats(bwacuda_ctx *ctx, bwacuda_stats *out);
int bwacuda_reset_stats(bwacuda_ctx *ctx);

/* Measured integer ALU-pipe throughput of the context's device, in 1e9 fused
 * add-max operations per second (one ALU-pipe instruction per lane each): the
 * roofline denominator of the DP kernels.  Runs a few short kernels (~5 ms
 * each) on the context's stream; synchronous.  A measurement helper with no
 * counterpart in the reference. */
int bwacuda_measure_alu_peak(bwacuda_ctx *ctx, double *gops);

/* Measured throughput of one integer operation the DP kernels are built from, in 1e9
 * lane-operations per second: every thread of a few short launches runs 8 independent chains
 * of it, so an operation that is one ALU-pipe instruction runs at bwacuda_measure_alu_peak's
 * rate and one that takes two instructions at half of it.  Synchronous.  A measurement helper
 * with no counterpart in the reference. */
#define BWACUDA_OPR_VIADDMAX_S32 0        /* __viaddmax_s32 */
#define BWACUDA_OPR_VIADDMAX_S32_RELU 1   /* __viaddmax_s32_relu */
#define BWACUDA_OPR_VIADDMAX_S16X2 2      /* __viaddmax_s16x2 */
#define BWACUDA_OPR_VIADDMAX_S16X2_RELU 3 /* __viaddmax_s16x2_relu */
#define BWACUDA_OPR_VIADDMIN_S16X2 4      /* __viaddmin_s16x2 */
#define BWACUDA_OPR_VIMAX3_S16X2 5        /* __vimax3_s16x2 */
#define BWACUDA_OPR_VIMAX3_U16X2 6        /* __vimax3_u16x2 */
#define BWACUDA_OPR_VIMAX_S16X2_RELU 7    /* __vimax_s16x2_relu */
#define BWACUDA_OPR_VIMAX3_S32 8          /* __vimax3_s32 */
#define BWACUDA_OPR_PRMT 9                /* prmt.b32 byte permute */
#define BWACUDA_OPR_C_ADD_MAX 10          /* max(a + b, c) written in C */
#define BWACUDA_OPR_IMAD 11               /* a * b + c */
#define BWACUDA_OPR_LOP3 12               /* (a & b) | c */
#define BWACUDA_OPR_COUNT 13
int bwacuda_measure_op_rate(bwacuda_ctx *ctx, int op, double *gops);

/* Host-link bandwidth in GB/s (1e9 bytes/s) over `bytes` (1 MiB .. 16 GiB) of pinned host memory:
 * the device reading it with 16-byte loads (the device-gather route's access), the copy engine's
 * host-to-device copy, and the device writing it (the host-buffer calls' result stores).  The
 * bytes a host-buffer call moves over these rates bound its end-to-end time.  Allocates and frees
 * its buffers. */
int bwacuda_measure_host_link(bwacuda_ctx *ctx, size_t bytes, double *read_gbs, double *copy_gbs,
                              double *write_gbs);

/* ------------------------------------------------------------------------
 * Autotuner.  No counterpart in the reference (its NEON kernels have fixed
 * lane counts).  The launch shape of the batched extension path (threads per
 * block, jobs per warp grab, length-bucket width) and of the rescue kernels
 * (register wavefront with 8, 16 or 32 lanes per job, or thread-per-job) is
 * picked by timing every candidate on a strided sample of a device-resident
 * batch; the best is kept in the context and used by every later call.
 * Results never depend on the tuning; only speed does.  Synchronous. */
typedef struct {
    int32_t persist_block;  /* 32, 64, 128, 256 */
    int32_t grab;           /* 1, 2, 4 */
    int32_t bucket_step;    /* 16, 32, 64 */
    int32_t rescue_lanes;   /* 8, 16, 32 */
    int32_t rescue_kernel;  /* BWACUDA_RESCUE_AUTO (wavefront where it fits) or BWACUDA_RESCUE_TPJ */
    int32_t candidates;     /* candidates timed by the last autotune call */
    double ext_gcups;       /* best extension candidate on its sample (0 if not tuned) */
    double rescue_gcups;    /* best rescue candidate on its sample (0 if not tuned) */
    int32_t long_qlen;      /* batched extension: buckets from this query length up use the group-per-job
                               kernel (0: only the open-ended buckets, queries beyond the thread-per-job rows) */
    int32_t long_lanes;     /* lanes per job of the group-per-job kernel: 8, 16 or 32 */
    int32_t rescue_pair;    /* lanes of a group holding two byte-range rescue jobs, 4, 8 or 16 (0: off;
                               BWACUDA_OPT_RESCUE_PAIR) */
    int32_t reserved;
} bwacuda_tuning;

int bwacuda_get_tuning(bwacuda_ctx *ctx, bwacuda_tuning *out);
/* sample = jobs timed per candidate (0: up to 4,194,304 for extension, 262,144 for rescue). */
int bwacuda_autotune_extend(bwacuda_ctx *ctx, const uint8_t *d_seq, const bwacuda_dev_ext_job *d_jobs,
                            size_t n, const bwacuda_scoring *sc, int end_bonus, int zdrop, size_t sample,
                            bwacuda_tuning *out);
int bwacuda_autotune_rescue(bwacuda_ctx *ctx, const uint8_t *d_seq, const bwacuda_dev_rescue_job *d_jobs,
                            size_t n, const bwacuda_scoring *sc, int minsc, int max_sc, size_t sample,
                            bwacuda_tuning *out);

#ifdef __cplusplus
}
#endif
#endif /* BWACUDA_H */
