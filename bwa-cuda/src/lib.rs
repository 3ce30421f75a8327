//! bwa-cuda: bwa-mem4's seed extension (`SwBackend`) and mate rescue (`batched_ksw_align2`) on a
//! GB300 GPU, through the C ABI of `libbwacuda.so` (`include/bwacuda.h` of the bwa-cuda tree).
//!
//! Drop-in points (two edits in bwa-mem4):
//! * `crates/bwa-cli/src/cmd_mem.rs:2214` passes `&NeonBackend` to `align_reads_batched`; pass
//!   `&bwa_cuda::CudaBackend` (the call is generic over `B: SwBackend`).
//! * `crates/bwa-mem/src/pe.rs:1090` calls `bwa_neon::batched_ksw_align2`; call
//!   [`batched_ksw_align2`] with the same arguments.
//!
//! Results are integer-identical to the reference's for every field, so the acceptance gates
//! `assert_backend_matches_scalar` / `assert_backend_batch_matches_scalar`
//! (`crates/bwa-extend/src/lib.rs:283-525`) and `matesw_equals_scalar`
//! (`crates/bwa-neon/src/matesw.rs:5045-5139`) apply unchanged.  The library has no CPU
//! fallback: a call the GPU cannot run returns an error code, which these wrappers turn into a
//! panic, as the reference backends panic on bugs (they are infallible by signature).
//!
//! Concurrency: the reference calls the backend from one rayon worker per chunk, concurrently.
//! A `bwacuda_ctx` serialises the calls made on it, so each worker thread gets its own context
//! (created on the thread's first call, destroyed when the thread exits) and the threads'
//! batches overlap on the device.
//!
//! NOT COMPILED: the machines this crate was written on carry no Rust toolchain.  The `ffi`
//! declarations below are checked against the library's exported symbols and against the C
//! header's prototypes (names and argument counts) by the bwa-cuda test suite.

use std::ffi::CStr;
use std::os::raw::c_int;

use bwa_extend::{ExtendJob, ExtendResult, KswAlignResult, SwBackend};
use bwa_neon::KswJob;

/// The C ABI, one declaration per entry point of `include/bwacuda.h`.
#[allow(non_camel_case_types, dead_code)]
pub mod ffi {
    use std::os::raw::{c_char, c_int, c_void};

    /// Opaque `bwacuda_ctx`.
    #[repr(C)]
    pub struct bwacuda_ctx {
        _private: [u8; 0],
    }

    pub const BWACUDA_OK: c_int = 0;
    pub const BWACUDA_EAGAIN: c_int = -8;
    pub const BWACUDA_ESHORT: c_int = -9;
    pub const BWACUDA_OPT_EXT_PATH: c_int = 1;
    pub const BWACUDA_OPT_HOST_GATHER: c_int = 6;
    pub const BWACUDA_OPT_UNGAPPED: c_int = 10;

    #[repr(C)]
    pub struct bwacuda_ext_job {
        pub query: *const u8,
        pub target: *const u8,
        pub qlen: i32,
        pub tlen: i32,
        pub h0: i32,
    }

    #[repr(C)]
    #[derive(Clone, Copy, Default)]
    pub struct bwacuda_ext_result {
        pub score: i32,
        pub qle: i32,
        pub tle: i32,
        pub gtle: i32,
        pub gscore: i32,
        pub max_off: i32,
    }

    #[repr(C)]
    pub struct bwacuda_rescue_job {
        pub query: *const u8,
        pub target: *const u8,
        pub qlen: i32,
        pub tlen: i32,
    }

    #[repr(C)]
    #[derive(Clone, Copy, Default)]
    pub struct bwacuda_rescue_result {
        pub score: i32,
        pub qb: i32,
        pub qe: i32,
        pub tb: i32,
        pub te: i32,
        pub score2: i32,
        pub te2: i32,
    }

    #[repr(C)]
    pub struct bwacuda_fwd_job {
        pub query: *const u8,
        pub target: *const u8,
        pub qlen: i32,
        pub tlen: i32,
        pub minsc: i32,
        pub endsc: i32,
    }

    #[repr(C)]
    #[derive(Clone, Copy, Default)]
    pub struct bwacuda_fwd_result {
        pub score: i32,
        pub te: i32,
        pub qe: i32,
        pub score2: i32,
        pub te2: i32,
    }

    #[repr(C)]
    pub struct bwacuda_global_job {
        pub query: *const u8,
        pub target: *const u8,
        pub qlen: i32,
        pub tlen: i32,
        pub w: i32,
    }

    #[repr(C)]
    pub struct bwacuda_window_req {
        pub mate: *const u8,
        pub l_ms: i32,
        pub orient: i32,
        pub anchor_rb: i64,
        pub anchor_rid: i32,
        pub low: i32,
        pub high: i32,
    }

    #[repr(C)]
    #[derive(Clone, Copy, Default)]
    pub struct bwacuda_window_result {
        pub rb: i64,
        pub re: i64,
        pub rid: i32,
        pub valid: i32,
        pub aln: bwacuda_rescue_result,
    }

    #[repr(C)]
    pub struct bwacuda_dev_ext_job {
        pub q_off: u64,
        pub t_off: u64,
        pub qlen: i32,
        pub tlen: i32,
        pub h0: i32,
        pub w: i32,
    }

    #[repr(C)]
    pub struct bwacuda_dev_rescue_job {
        pub q_off: u64,
        pub t_off: u64,
        pub qlen: i32,
        pub tlen: i32,
        pub minsc: i32,
        pub endsc: i32,
    }

    #[repr(C)]
    pub struct bwacuda_scoring {
        pub m: i32,
        pub mat: [i8; 64],
        pub o_del: i32,
        pub e_del: i32,
        pub o_ins: i32,
        pub e_ins: i32,
    }

    #[repr(C)]
    pub struct bwacuda_server_config {
        pub hbm_budget_bytes: u64,
        pub max_waves: i32,
        pub max_requests: i32,
    }

    #[repr(C)]
    #[derive(Clone, Copy, Default)]
    pub struct bwacuda_stats {
        pub ext_jobs: u64,
        pub ext_cells: u64,
        pub ext_bin_u8: u64,
        pub ext_bin_i16: u64,
        pub ext_bin_i32: u64,
        pub rescue_jobs: u64,
        pub rescue_cells: u64,
        pub rescue_width_u8: u64,
        pub rescue_width_i16: u64,
        pub rescue_width_i32: u64,
        pub kernel_launches: u64,
        pub h2d_bytes: u64,
        pub d2h_bytes: u64,
        pub global_jobs: u64,
        pub global_cells: u64,
        pub ext_retry_jobs: u64,
    }

    #[repr(C)]
    #[derive(Clone, Copy, Default)]
    pub struct bwacuda_tuning {
        pub persist_block: i32,
        pub grab: i32,
        pub bucket_step: i32,
        pub rescue_lanes: i32,
        pub rescue_kernel: i32,
        pub candidates: i32,
        pub ext_gcups: f64,
        pub rescue_gcups: f64,
        pub long_qlen: i32,
        pub long_lanes: i32,
        pub rescue_pair: i32,
        pub reserved: i32,
    }

    extern "C" {
        pub fn bwacuda_ctx_create(device: c_int, out: *mut *mut bwacuda_ctx) -> c_int;
        pub fn bwacuda_ctx_destroy(ctx: *mut bwacuda_ctx);
        pub fn bwacuda_set_option(ctx: *mut bwacuda_ctx, option: c_int, value: i64) -> c_int;
        pub fn bwacuda_strerror(code: c_int) -> *const c_char;
        pub fn bwacuda_backend_name() -> *const c_char;
        pub fn bwacuda_extend(ctx: *mut bwacuda_ctx, query: *const u8, qlen: i32, target: *const u8, tlen: i32,
                              m: c_int, mat: *const i8, o_del: c_int, e_del: c_int, o_ins: c_int, e_ins: c_int,
                              w: c_int, end_bonus: c_int, zdrop: c_int, h0: c_int,
                              out: *mut bwacuda_ext_result) -> c_int;
        pub fn bwacuda_extend_batch(ctx: *mut bwacuda_ctx, jobs: *const bwacuda_ext_job, n: usize, m: c_int,
                                    mat: *const i8, o_del: c_int, e_del: c_int, o_ins: c_int, e_ins: c_int,
                                    w: c_int, end_bonus: c_int, zdrop: c_int,
                                    out: *mut bwacuda_ext_result) -> c_int;
        pub fn bwacuda_extend_batch_retry(ctx: *mut bwacuda_ctx, jobs: *const bwacuda_ext_job, n: usize, m: c_int,
                                          mat: *const i8, o_del: c_int, e_del: c_int, o_ins: c_int, e_ins: c_int,
                                          w: c_int, end_bonus: c_int, zdrop: c_int, max_tries: c_int,
                                          prev: *const i32, out: *mut bwacuda_ext_result,
                                          w_used: *mut i32) -> c_int;
        pub fn bwacuda_ksw_align2_batch(ctx: *mut bwacuda_ctx, jobs: *const bwacuda_rescue_job, n: usize,
                                        m: c_int, mat: *const i8, o_del: c_int, e_del: c_int, o_ins: c_int,
                                        e_ins: c_int, minsc: c_int, max_sc: c_int,
                                        out: *mut bwacuda_rescue_result) -> c_int;
        pub fn bwacuda_ksw_align2_scalar_batch(ctx: *mut bwacuda_ctx, jobs: *const bwacuda_rescue_job, n: usize,
                                               m: c_int, mat: *const i8, o_del: c_int, e_del: c_int,
                                               o_ins: c_int, e_ins: c_int, minsc: c_int, max_sc: c_int,
                                               lanes: c_int, out: *mut bwacuda_rescue_result) -> c_int;
        pub fn bwacuda_ksw_global2_batch(ctx: *mut bwacuda_ctx, jobs: *const bwacuda_global_job, n: usize,
                                         m: c_int, mat: *const i8, o_del: c_int, e_del: c_int, o_ins: c_int,
                                         e_ins: c_int, score: *mut i32, cigar_off: *mut u64, cigar: *mut u32,
                                         cigar_cap: usize) -> c_int;
        pub fn bwacuda_ref_set(ctx: *mut bwacuda_ctx, pac: *const u8, l_pac: i64, contig_offset: *const i64,
                               contig_len: *const i32, n_contigs: i32) -> c_int;
        pub fn bwacuda_mate_rescue_windows(ctx: *mut bwacuda_ctx, reqs: *const bwacuda_window_req, n: usize,
                                           m: c_int, mat: *const i8, o_del: c_int, e_del: c_int, o_ins: c_int,
                                           e_ins: c_int, minsc: c_int, max_sc: c_int, min_seed_len: c_int,
                                           out: *mut bwacuda_window_result) -> c_int;
        pub fn bwacuda_ksw_local_fwd_batch(ctx: *mut bwacuda_ctx, jobs: *const bwacuda_fwd_job, n: usize,
                                           m: c_int, mat: *const i8, o_del: c_int, e_del: c_int, o_ins: c_int,
                                           e_ins: c_int, max_sc: c_int, lanes: c_int,
                                           out: *mut bwacuda_fwd_result) -> c_int;
        pub fn bwacuda_extend_device(ctx: *mut bwacuda_ctx, d_seq: *const u8, d_jobs: *const bwacuda_dev_ext_job,
                                     n: usize, sc: *const bwacuda_scoring, end_bonus: c_int, zdrop: c_int,
                                     path: c_int, d_out: *mut bwacuda_ext_result, stream: *mut c_void) -> c_int;
        pub fn bwacuda_extend_retry_device(ctx: *mut bwacuda_ctx, d_seq: *const u8,
                                           d_jobs: *const bwacuda_dev_ext_job, n: usize,
                                           sc: *const bwacuda_scoring, end_bonus: c_int, zdrop: c_int,
                                           max_tries: c_int, d_prev: *const i32, d_out: *mut bwacuda_ext_result,
                                           d_w_used: *mut i32, stream: *mut c_void) -> c_int;
        pub fn bwacuda_ksw_align2_device(ctx: *mut bwacuda_ctx, d_seq: *const u8,
                                         d_jobs: *const bwacuda_dev_rescue_job, n: usize,
                                         sc: *const bwacuda_scoring, minsc: c_int, max_sc: c_int, mode: c_int,
                                         lanes: c_int, d_out: *mut bwacuda_rescue_result,
                                         stream: *mut c_void) -> c_int;
        pub fn bwacuda_ctx_sync(ctx: *mut bwacuda_ctx) -> c_int;
        pub fn bwacuda_ksw_align2_device_noalloc(ctx: *mut bwacuda_ctx, d_seq: *const u8,
                                                 d_jobs: *const bwacuda_dev_rescue_job, n: usize,
                                                 sc: *const bwacuda_scoring, minsc: c_int, max_sc: c_int,
                                                 mode: c_int, lanes: c_int, d_out: *mut bwacuda_rescue_result,
                                                 stream: *mut c_void) -> c_int;
        pub fn bwacuda_server_start(ctx: *mut bwacuda_ctx, cfg: *const bwacuda_server_config) -> c_int;
        pub fn bwacuda_server_stop(ctx: *mut bwacuda_ctx) -> c_int;
        pub fn bwacuda_server_submit_extend(ctx: *mut bwacuda_ctx, jobs: *const bwacuda_ext_job, n: usize,
                                            sc: *const bwacuda_scoring, w: c_int, end_bonus: c_int, zdrop: c_int,
                                            req_id: *mut u64) -> c_int;
        pub fn bwacuda_server_submit_rescue(ctx: *mut bwacuda_ctx, jobs: *const bwacuda_rescue_job, n: usize,
                                            sc: *const bwacuda_scoring, minsc: c_int, max_sc: c_int,
                                            req_id: *mut u64) -> c_int;
        pub fn bwacuda_server_submit_mixed(ctx: *mut bwacuda_ctx, ext_jobs: *const bwacuda_ext_job, n_ext: usize,
                                           rescue_jobs: *const bwacuda_rescue_job, n_rescue: usize,
                                           sc: *const bwacuda_scoring, w: c_int, end_bonus: c_int, zdrop: c_int,
                                           minsc: c_int, max_sc: c_int, req_id: *mut u64) -> c_int;
        pub fn bwacuda_server_cells(ctx: *mut bwacuda_ctx, ext_cells: *mut u64, rescue_cells: *mut u64) -> c_int;
        pub fn bwacuda_server_wait(ctx: *mut bwacuda_ctx, req_id: u64, out: *mut c_void, timeout_us: i64,
                                   latency_ns: *mut i64) -> c_int;
        pub fn bwacuda_server_stats(ctx: *mut bwacuda_ctx, served_jobs: *mut u64, waves: *mut u64,
                                    queued: *mut u64) -> c_int;
        pub fn bwacuda_get_stats(ctx: *mut bwacuda_ctx, out: *mut bwacuda_stats) -> c_int;
        pub fn bwacuda_reset_stats(ctx: *mut bwacuda_ctx) -> c_int;
        pub fn bwacuda_measure_alu_peak(ctx: *mut bwacuda_ctx, gops: *mut f64) -> c_int;
        pub fn bwacuda_measure_op_rate(ctx: *mut bwacuda_ctx, op: c_int, gops: *mut f64) -> c_int;
        pub fn bwacuda_measure_host_link(ctx: *mut bwacuda_ctx, bytes: usize, read_gbs: *mut f64,
                                         copy_gbs: *mut f64, write_gbs: *mut f64) -> c_int;
        pub fn bwacuda_get_tuning(ctx: *mut bwacuda_ctx, out: *mut bwacuda_tuning) -> c_int;
        pub fn bwacuda_autotune_extend(ctx: *mut bwacuda_ctx, d_seq: *const u8, d_jobs: *const bwacuda_dev_ext_job,
                                       n: usize, sc: *const bwacuda_scoring, end_bonus: c_int, zdrop: c_int,
                                       sample: usize, out: *mut bwacuda_tuning) -> c_int;
        pub fn bwacuda_autotune_rescue(ctx: *mut bwacuda_ctx, d_seq: *const u8,
                                       d_jobs: *const bwacuda_dev_rescue_job, n: usize,
                                       sc: *const bwacuda_scoring, minsc: c_int, max_sc: c_int, sample: usize,
                                       out: *mut bwacuda_tuning) -> c_int;
    }
}

/// Panics with the library's message on a non-zero return code: the reference's backends are
/// infallible by signature and panic on bugs, and a drop-in must not return a wrong answer
/// silently.
fn check(rc: c_int, what: &str) {
    if rc != ffi::BWACUDA_OK {
        // SAFETY: bwacuda_strerror returns a static NUL-terminated string for every code.
        let msg = unsafe { CStr::from_ptr(ffi::bwacuda_strerror(rc)) };
        panic!("{what}: {} ({rc})", msg.to_string_lossy());
    }
}

/// One device context, owned by one thread.
struct Ctx(*mut ffi::bwacuda_ctx);

impl Ctx {
    fn new() -> Ctx {
        let device: c_int = std::env::var("BWACUDA_DEVICE").ok().and_then(|v| v.parse().ok()).unwrap_or(0);
        let mut p = std::ptr::null_mut();
        // SAFETY: out-pointer to a local; the library writes a context or leaves it null.
        check(unsafe { ffi::bwacuda_ctx_create(device, &mut p) }, "bwacuda_ctx_create");
        Ctx(p)
    }
}

impl Drop for Ctx {
    fn drop(&mut self) {
        // SAFETY: created by bwacuda_ctx_create, destroyed once.
        unsafe { ffi::bwacuda_ctx_destroy(self.0) }
    }
}

thread_local! {
    static CTX: Ctx = Ctx::new();
}

fn with_ctx<R>(f: impl FnOnce(*mut ffi::bwacuda_ctx) -> R) -> R {
    CTX.with(|c| f(c.0))
}

fn to_extend_result(r: &ffi::bwacuda_ext_result) -> ExtendResult {
    ExtendResult { score: r.score, qle: r.qle, tle: r.tle, gtle: r.gtle, gscore: r.gscore, max_off: r.max_off }
}

fn to_align_result(r: &ffi::bwacuda_rescue_result) -> KswAlignResult {
    KswAlignResult { score: r.score, qb: r.qb, qe: r.qe, tb: r.tb, te: r.te, score2: r.score2, te2: r.te2 }
}

fn len_i32(s: &[u8]) -> i32 {
    i32::try_from(s.len()).expect("sequence longer than i32::MAX bases")
}

/// The GPU backend: `extend` and `extend_batch` return exactly what `ksw_extend2` returns
/// (`crates/bwa-extend/src/lib.rs:83-176`).
#[derive(Debug, Default, Clone, Copy)]
pub struct CudaBackend;

impl SwBackend for CudaBackend {
    fn name(&self) -> &'static str {
        "cuda"
    }

    #[allow(clippy::too_many_arguments)]
    fn extend(
        &self,
        query: &[u8],
        target: &[u8],
        m: usize,
        mat: &[i8],
        o_del: i32,
        e_del: i32,
        o_ins: i32,
        e_ins: i32,
        w: i32,
        end_bonus: i32,
        zdrop: i32,
        h0: i32,
    ) -> ExtendResult {
        let job = ExtendJob { query, target, h0 };
        self.extend_batch(&[job], m, mat, o_del, e_del, o_ins, e_ins, w, end_bonus, zdrop)[0]
    }

    #[allow(clippy::too_many_arguments)]
    fn extend_batch(
        &self,
        jobs: &[ExtendJob],
        m: usize,
        mat: &[i8],
        o_del: i32,
        e_del: i32,
        o_ins: i32,
        e_ins: i32,
        w: i32,
        end_bonus: i32,
        zdrop: i32,
    ) -> Vec<ExtendResult> {
        assert!(mat.len() >= m * m, "mat holds fewer than m * m entries");
        let cj: Vec<ffi::bwacuda_ext_job> = jobs
            .iter()
            .map(|j| ffi::bwacuda_ext_job {
                query: j.query.as_ptr(),
                target: j.target.as_ptr(),
                qlen: len_i32(j.query),
                tlen: len_i32(j.target),
                h0: j.h0,
            })
            .collect();
        let mut out = vec![ffi::bwacuda_ext_result::default(); jobs.len()];
        with_ctx(|ctx| {
            // SAFETY: every slice outlives the synchronous call; out has one entry per job.
            let rc = unsafe {
                ffi::bwacuda_extend_batch(ctx, cj.as_ptr(), cj.len(), m as c_int, mat.as_ptr(), o_del, e_del,
                                          o_ins, e_ins, w, end_bonus, zdrop, out.as_mut_ptr())
            };
            check(rc, "bwacuda_extend_batch");
        });
        out.iter().map(to_extend_result).collect()
    }
}

/// `bwa_neon::batched_ksw_align2` (`crates/bwa-neon/src/matesw.rs:299-309`): same arguments,
/// same results, in job order.
#[allow(clippy::too_many_arguments)]
pub fn batched_ksw_align2(
    jobs: &[KswJob],
    m: usize,
    mat: &[i8],
    o_del: i32,
    e_del: i32,
    o_ins: i32,
    e_ins: i32,
    minsc: i32,
    max_sc: i32,
) -> Vec<KswAlignResult> {
    assert!(mat.len() >= m * m, "mat holds fewer than m * m entries");
    let cj: Vec<ffi::bwacuda_rescue_job> = jobs
        .iter()
        .map(|j| ffi::bwacuda_rescue_job {
            query: j.query.as_ptr(),
            target: j.target.as_ptr(),
            qlen: len_i32(j.query),
            tlen: len_i32(j.target),
        })
        .collect();
    let mut out = vec![ffi::bwacuda_rescue_result::default(); jobs.len()];
    with_ctx(|ctx| {
        // SAFETY: as in extend_batch.
        let rc = unsafe {
            ffi::bwacuda_ksw_align2_batch(ctx, cj.as_ptr(), cj.len(), m as c_int, mat.as_ptr(), o_del, e_del,
                                          o_ins, e_ins, minsc, max_sc, out.as_mut_ptr())
        };
        check(rc, "bwacuda_ksw_align2_batch");
    });
    out.iter().map(to_align_result).collect()
}

/// `bwa_extend::ksw_align2` (`crates/bwa-extend/src/sw.rs:1108-1185`) for one pair: the scalar
/// form, whose reverse pass scans the whole target with only `target[..=te]` reversed.
#[allow(clippy::too_many_arguments)]
pub fn ksw_align2(
    query: &[u8],
    target: &[u8],
    m: usize,
    mat: &[i8],
    o_del: i32,
    e_del: i32,
    o_ins: i32,
    e_ins: i32,
    minsc: i32,
    max_sc: i32,
    lanes: usize,
) -> KswAlignResult {
    assert!(mat.len() >= m * m, "mat holds fewer than m * m entries");
    let job = ffi::bwacuda_rescue_job {
        query: query.as_ptr(),
        target: target.as_ptr(),
        qlen: len_i32(query),
        tlen: len_i32(target),
    };
    let mut out = ffi::bwacuda_rescue_result::default();
    with_ctx(|ctx| {
        // SAFETY: one job, one result, both outlive the synchronous call.
        let rc = unsafe {
            ffi::bwacuda_ksw_align2_scalar_batch(ctx, &job, 1, m as c_int, mat.as_ptr(), o_del, e_del, o_ins,
                                                 e_ins, minsc, max_sc, lanes as c_int, &mut out)
        };
        check(rc, "bwacuda_ksw_align2_scalar_batch");
    });
    to_align_result(&out)
}

/// `bwa_extend::ksw_global2` (`crates/bwa-extend/src/sw.rs:561-740`) over a batch: job `k` is
/// `(query, target, w)`, result `k` the `(score, cigar)` the reference returns for it.  The
/// reference's CIGAR step (`crates/bwa-mem/src/cigar.rs:446`) calls it once per alignment; batch a
/// chunk's alignments here instead.
#[allow(clippy::too_many_arguments)]
pub fn ksw_global2_batch(
    jobs: &[(&[u8], &[u8], i32)],
    m: usize,
    mat: &[i8],
    o_del: i32,
    e_del: i32,
    o_ins: i32,
    e_ins: i32,
) -> Vec<(i32, Vec<u32>)> {
    assert!(mat.len() >= m * m, "mat holds fewer than m * m entries");
    let cj: Vec<ffi::bwacuda_global_job> = jobs
        .iter()
        .map(|(q, t, w)| ffi::bwacuda_global_job {
            query: q.as_ptr(),
            target: t.as_ptr(),
            qlen: len_i32(q),
            tlen: len_i32(t),
            w: *w,
        })
        .collect();
    // sum(qlen + tlen) CIGAR words always suffice
    let cap: usize = jobs.iter().map(|(q, t, _)| q.len() + t.len()).sum::<usize>().max(1);
    let mut score = vec![0i32; cj.len()];
    let mut off = vec![0u64; cj.len() + 1];
    let mut cig = vec![0u32; cap];
    with_ctx(|ctx| {
        // SAFETY: output arrays sized as the header requires (n scores, n + 1 offsets, cap words).
        let rc = unsafe {
            ffi::bwacuda_ksw_global2_batch(ctx, cj.as_ptr(), cj.len(), m as c_int, mat.as_ptr(), o_del, e_del,
                                           o_ins, e_ins, score.as_mut_ptr(), off.as_mut_ptr(), cig.as_mut_ptr(),
                                           cap)
        };
        check(rc, "bwacuda_ksw_global2_batch");
    });
    (0..cj.len()).map(|k| (score[k], cig[off[k] as usize..off[k + 1] as usize].to_vec())).collect()
}

/// `run_side`'s band-doubling loop (`crates/bwa-mem/src/across.rs:1357-1500`) in one call: each
/// job is extended at `w << r` until the reference's acceptance test passes or `max_tries` rounds
/// ran.  `prev[k]` is the job's value before round 0 (`-1` for a left extension, `h0` for a right
/// one).  Returns each job's accepted result and the band it was accepted at.
#[allow(clippy::too_many_arguments)]
pub fn extend_batch_retry(
    jobs: &[ExtendJob],
    prev: &[i32],
    m: usize,
    mat: &[i8],
    o_del: i32,
    e_del: i32,
    o_ins: i32,
    e_ins: i32,
    w: i32,
    end_bonus: i32,
    zdrop: i32,
    max_tries: i32,
) -> Vec<(ExtendResult, i32)> {
    assert_eq!(jobs.len(), prev.len(), "one prev value per job");
    assert!(mat.len() >= m * m, "mat holds fewer than m * m entries");
    let cj: Vec<ffi::bwacuda_ext_job> = jobs
        .iter()
        .map(|j| ffi::bwacuda_ext_job {
            query: j.query.as_ptr(),
            target: j.target.as_ptr(),
            qlen: len_i32(j.query),
            tlen: len_i32(j.target),
            h0: j.h0,
        })
        .collect();
    let mut out = vec![ffi::bwacuda_ext_result::default(); jobs.len()];
    let mut w_used = vec![0i32; jobs.len()];
    with_ctx(|ctx| {
        // SAFETY: every array holds one entry per job and outlives the synchronous call.
        let rc = unsafe {
            ffi::bwacuda_extend_batch_retry(ctx, cj.as_ptr(), cj.len(), m as c_int, mat.as_ptr(), o_del, e_del,
                                            o_ins, e_ins, w, end_bonus, zdrop, max_tries, prev.as_ptr(),
                                            out.as_mut_ptr(), w_used.as_mut_ptr())
        };
        check(rc, "bwacuda_extend_batch_retry");
    });
    out.iter().zip(w_used).map(|(r, wu)| (to_extend_result(r), wu)).collect()
}

/// The library's backend name (`"cuda"`), as `SwBackend::name` reports it.
pub fn library_name() -> &'static str {
    // SAFETY: a static NUL-terminated string.
    let s: &'static CStr = unsafe { CStr::from_ptr(ffi::bwacuda_backend_name()) };
    s.to_str().unwrap_or("cuda")
}

/// Counters of the calling thread's context since it was created.
pub fn stats() -> ffi::bwacuda_stats {
    let mut s = ffi::bwacuda_stats::default();
    with_ctx(|ctx| {
        // SAFETY: out-pointer to a local.
        check(unsafe { ffi::bwacuda_get_stats(ctx, &mut s) }, "bwacuda_get_stats");
    });
    s
}
