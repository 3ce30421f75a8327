/*
 * ksw_oracle.h -- CPU restatement of bwa-mem4's seed-extension / mate-rescue
 * Smith-Waterman semantics.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker the CUDA kernels are
 * compared against.  Only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference legs of bench.py may load it.  The product path (libbwacuda.so)
 * neither links nor calls anything here.
 *
 * Parity pinning: the reference is Rust and cannot be compiled on this machine,
 * so the restatement is pinned by the known-answer tests in the reference's own
 * test modules and by the cross-form equalities those tests assert (scalar vs
 * lockstep extension, ungapped fast path vs DP, scalar ksw_align2 vs the
 * batched truncated form) replayed on the reference's own LCG input streams.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the reference project root).
 */
#ifndef KSW_ORACLE_H
#define KSW_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* crates/bwa-extend/src/sw.rs:139-162 ExtendResult */
typedef struct { int32_t score, qle, tle, gtle, gscore, max_off; } ko_ext_result;
/* crates/bwa-extend/src/sw.rs:750-774 KswAlignResult */
typedef struct { int32_t score, qb, qe, tb, te, score2, te2; } ko_aln_result;
/* crates/bwa-extend/src/sw.rs:921-934 return tuple of ksw_local_fwd */
typedef struct { int32_t score, te, qe, score2, te2; } ko_fwd_result;

/* Banded extension, crates/bwa-extend/src/sw.rs:203-493.  qlen == 0 follows the
 * production lockstep path (crates/bwa-neon/src/batched.rs:1025-1039) because
 * the scalar form indexes past its buffer there.  *cells (may be NULL) receives
 * the number of inner-loop iterations, sum over processed rows of (end-beg). */
ko_ext_result ko_extend2(const uint8_t *q, int qlen, const uint8_t *t, int tlen,
                         int m, const int8_t *mat, int o_del, int e_del,
                         int o_ins, int e_ins, int w, int end_bonus, int zdrop,
                         int h0, uint64_t *cells);

/* Lockstep restatement of batched_extend_scalar, crates/bwa-neon/src/batched.rs:947-1251:
 * `lanes` jobs share one row counter.  Used to pin ko_extend2 (the reference
 * asserts both forms agree) and the qlen == 0 convention. */
void ko_extend_lockstep(int n, const uint8_t *const *qs, const int *qlens,
                        const uint8_t *const *ts, const int *tlens, const int *h0s,
                        int m, const int8_t *mat, int o_del, int e_del, int o_ins,
                        int e_ins, int w, int end_bonus, int zdrop, int lanes,
                        ko_ext_result *out);

/* Band clamp, crates/bwa-neon/src/batched.rs:1305-1329 / sw.rs:296-308. */
int ko_clamp_band(int w, int qlen, int max_sc, int end_bonus, int o_ins, int e_ins,
                  int o_del, int e_del);

/* Unbanded extension used by the reference's own unit test, sw.rs:1255-1310. */
int ko_ref_extend(const uint8_t *q, int qlen, const uint8_t *t, int tlen, int m,
                  const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins, int h0);

/* Ungapped diagonal fast path, crates/bwa-neon/src/batched.rs:602-697, with the
 * mismatch budget of :756-764.  Returns 1 and fills *out on a hit, 0 on decline. */
int ko_ungapped_hit(const uint8_t *q, int qlen, const uint8_t *t, int tlen, int h0,
                    int a, int b, int x_threshold, int zdrop, ko_ext_result *out);
int ko_x_threshold(int a, int b, int o_del, int e_del, int o_ins, int e_ins);

/* 8/16/32-bit bin label of one extension job, crates/bwa-neon/src/batched.rs:817-865.
 * 0 = u8, 1 = i16, 2 = scalar (i32). */
int ko_ext_bin(int qlen, int tlen, int h0, int m, const int8_t *mat);

/* Query padding width rule, crates/bwa-neon/src/matesw.rs:676-686. */
int ko_padded_qlen(int qlen, int max_sc);
/* Batch-wide rescue width label, crates/bwa-neon/src/matesw.rs:780-795.
 * 0 = u8, 1 = i16, 2 = scalar. */
int ko_rescue_width(int n, const int *qlens, const int *tlens, int m, const int8_t *mat,
                    int max_sc);

/* Forward local SW pass, crates/bwa-extend/src/sw.rs:921-1075 (with the
 * SuboptimalTracker of :789-852).  lanes = 16 or 8 (query padding width). */
ko_fwd_result ko_local_fwd(const uint8_t *q, int qlen, const uint8_t *t, int tlen,
                           int m, const int8_t *mat, int o_del, int e_del, int o_ins,
                           int e_ins, int minsc, int endsc, int max_sc, int lanes);

/* Scalar ksw_align2, crates/bwa-extend/src/sw.rs:1108-1185: reverse pass over
 * the whole target with only target[..=te] reversed (untruncated). */
ko_aln_result ko_align2_scalar(const uint8_t *q, int qlen, const uint8_t *t, int tlen,
                               int m, const int8_t *mat, int o_del, int e_del,
                               int o_ins, int e_ins, int minsc, int max_sc, int lanes);

/* One job of the production batched_ksw_align2, crates/bwa-neon/src/matesw.rs:299-497:
 * forward padding from qlen, reverse pass over the truncated prefixes
 * target[..=te], query[..=qe] with padding recomputed from qe + 1. */
ko_aln_result ko_align2_batched(const uint8_t *q, int qlen, const uint8_t *t, int tlen,
                                int m, const int8_t *mat, int o_del, int e_del,
                                int o_ins, int e_ins, int minsc, int max_sc);

/* ---- flat batch drivers (multi-threaded, for tests and the CPU baseline) ----
 * seq: all bases; q_off/t_off: byte offsets into seq; results in job order.
 * nthreads <= 0 means "all host threads".  cells_out (may be NULL) receives the
 * summed work units. */
void ko_extend_batch(const uint8_t *seq, int64_t n, const int64_t *q_off,
                     const int64_t *t_off, const int32_t *qlen, const int32_t *tlen,
                     const int32_t *h0, const int32_t *w, int m, const int8_t *mat,
                     int o_del, int e_del, int o_ins, int e_ins, int end_bonus,
                     int zdrop, int nthreads, ko_ext_result *out, uint64_t *cells_out);

/* mode 0: batched_ksw_align2 semantics; mode 1: scalar ksw_align2 with the
 * padding rule per job (lanes == 0) or a fixed lanes value. */
void ko_align2_batch(const uint8_t *seq, int64_t n, const int64_t *q_off,
                     const int64_t *t_off, const int32_t *qlen, const int32_t *tlen,
                     int m, const int8_t *mat, int o_del, int e_del, int o_ins,
                     int e_ins, int minsc, int max_sc, int mode, int lanes,
                     int nthreads, ko_aln_result *out, uint64_t *cells_out);

/* Forward pass only, per-job minsc/endsc (the FwdJob unit of matesw.rs:131-142). */
void ko_local_fwd_batch(const uint8_t *seq, int64_t n, const int64_t *q_off,
                        const int64_t *t_off, const int32_t *qlen, const int32_t *tlen,
                        const int32_t *minsc, const int32_t *endsc, int m,
                        const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins,
                        int max_sc, int lanes, int nthreads, ko_fwd_result *out);

/* ksw_global2, crates/bwa-extend/src/sw.rs:561-740: banded global alignment with traceback.
 * cigar (room for qlen + tlen + 1 words) receives the runs (len << 4 | op, op 0=M 1=I 2=D).
 * Returns 0, or -1 where the reference's traceback index would go out of range. */
int ko_global2(const uint8_t *q, int qlen, const uint8_t *t, int tlen, int m, const int8_t *mat,
               int o_del, int e_del, int o_ins, int e_ins, int w, int32_t *score, uint32_t *cigar,
               int *n_cigar);
int ko_global2_batch(const uint8_t *seq, int64_t n, const int64_t *q_off, const int64_t *t_off,
                     const int32_t *qlen, const int32_t *tlen, const int32_t *w, int m,
                     const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins, int nthreads,
                     int32_t *score, const int64_t *cig_off, uint32_t *cigar, int32_t *n_cigar);

/* Mate-rescue windows: the 2-bit reference base at 2L-space position pos, and one
 * orientation's window (matesw_collect + bns_fetch_seq); returns 1 when accepted. */
uint8_t ko_ref_base(const uint8_t *pac, int64_t l_pac, int64_t pos);
int ko_rescue_window(const uint8_t *pac, int64_t l_pac, const int64_t *off, const int32_t *len, int32_t n,
                     int64_t anchor_rb, int32_t anchor_rid, int orient, int low, int high, int l_ms,
                     int min_seed_len, int64_t *rb_out, int64_t *re_out, int32_t *rid_out);

/* bwa_fill_scmat, crates/bwa-core/src/opt.rs:419-460 (match a, mismatch -b, N -1). */
void ko_fill_scmat(int a, int b, int8_t mat[25]);

/* The reference's production dispatch for an extension batch (crates/bwa-neon/src/batched.rs:716-775):
 * the ungapped closed form first (uniform DNA matrices), the scalar DP for the jobs it declines;
 * OpenMP over jobs.  *settled_out = jobs the closed form settled, *cells_out = DP cells evaluated. */
void ko_extend_batch_dispatch(const uint8_t *seq, int64_t n, const int64_t *q_off,
                              const int64_t *t_off, const int32_t *qlen, const int32_t *tlen,
                              const int32_t *h0, const int32_t *w, int m, const int8_t *mat,
                              int o_del, int e_del, int o_ins, int e_ins, int end_bonus,
                              int zdrop, int nthreads, ko_ext_result *out, uint64_t *settled_out,
                              uint64_t *cells_out);

#ifdef __cplusplus
}
#endif
#endif
