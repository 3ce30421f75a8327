// bwacuda.hpp -- C++ mirror of the reference's Rust interfaces for this path,
// header-only over the C ABI in bwacuda.h.
//
//   bwa_cuda::SwBackend / CudaBackend   <->  trait SwBackend (crates/bwa-extend/src/lib.rs:83-176)
//   bwa_cuda::ExtendJob                 <->  ExtendJob (crates/bwa-extend/src/lib.rs:181-195)
//   bwa_cuda::ExtendResult              <->  ExtendResult (crates/bwa-extend/src/sw.rs:139-162)
//   bwa_cuda::KswJob                    <->  KswJob (crates/bwa-neon/src/matesw.rs:104-116)
//   bwa_cuda::KswAlignResult            <->  KswAlignResult (crates/bwa-extend/src/sw.rs:750-774)
//   bwa_cuda::batched_ksw_align2        <->  bwa_neon::batched_ksw_align2 (crates/bwa-neon/src/matesw.rs:299-309)
//   bwa_cuda::ksw_align2                <->  bwa_extend::ksw_align2 (crates/bwa-extend/src/sw.rs:1108-1185)
//   bwa_cuda::ksw_global2               <->  bwa_extend::ksw_global2 (crates/bwa-extend/src/sw.rs:561-740)
//   bwa_cuda::ksw_global2_batch            (the same over many alignments, per-job band)
//   bwa_cuda::run_side_extend           <->  the band-doubling loop of run_side (crates/bwa-mem/src/across.rs:1357-1500)
//
// Same argument names, meanings and result order.  The reference's calls are
// infallible (they panic on bugs); these throw bwa_cuda::Error with the C ABI's
// code instead, and never fall back to a CPU implementation.
#pragma once
#include <cstddef>
#include <cstdint>
#include <memory>
#include <utility>
#include <stdexcept>
#include <string>
#include <vector>

#include "bwacuda.h"

namespace bwa_cuda {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &what) : std::runtime_error(what + ": " + bwacuda_strerror(c)), code(c) {}
};

inline void check(int rc, const char *what)
{
    if (rc != BWACUDA_OK) throw Error(rc, what);
}

// A borrowed slice, like Rust's &[u8].
struct Bytes {
    const uint8_t *ptr = nullptr;
    size_t len = 0;
    Bytes() = default;
    Bytes(const uint8_t *p, size_t n) : ptr(p), len(n) {}
    Bytes(const std::vector<uint8_t> &v) : ptr(v.data()), len(v.size()) {}
};

struct ExtendJob {
    Bytes query, target;
    int32_t h0;
};

using ExtendResult = bwacuda_ext_result;

struct KswJob {
    Bytes query, target;
};

using KswAlignResult = bwacuda_rescue_result;

// One GPU context (device, pinned staging, streams).  Thread-safe; calls on
// one context are serialised, so use one per worker thread for overlap.
class Context {
public:
    explicit Context(int device = 0)
    {
        bwacuda_ctx *c = nullptr;
        check(bwacuda_ctx_create(device, &c), "bwacuda_ctx_create");
        ctx_.reset(c);
    }
    bwacuda_ctx *get() const { return ctx_.get(); }
    void set_option(int opt, int64_t v) { check(bwacuda_set_option(ctx_.get(), opt, v), "bwacuda_set_option"); }
    bwacuda_stats stats() const
    {
        bwacuda_stats s;
        check(bwacuda_get_stats(ctx_.get(), &s), "bwacuda_get_stats");
        return s;
    }

private:
    struct Del {
        void operator()(bwacuda_ctx *c) const { bwacuda_ctx_destroy(c); }
    };
    std::unique_ptr<bwacuda_ctx, Del> ctx_;
};

// The SwBackend trait: one extension and a batch sharing scoring and band.
class SwBackend {
public:
    virtual ~SwBackend() = default;
    virtual const char *name() const = 0;
    virtual ExtendResult extend(Bytes query, Bytes target, size_t m, const int8_t *mat, int o_del, int e_del,
                                int o_ins, int e_ins, int w, int end_bonus, int zdrop, int h0) const = 0;
    virtual std::vector<ExtendResult> extend_batch(const std::vector<ExtendJob> &jobs, size_t m, const int8_t *mat,
                                                   int o_del, int e_del, int o_ins, int e_ins, int w, int end_bonus,
                                                   int zdrop) const = 0;
};

class CudaBackend final : public SwBackend {
public:
    explicit CudaBackend(Context &ctx) : ctx_(&ctx) {}
    const char *name() const override { return bwacuda_backend_name(); }

    ExtendResult extend(Bytes query, Bytes target, size_t m, const int8_t *mat, int o_del, int e_del, int o_ins,
                        int e_ins, int w, int end_bonus, int zdrop, int h0) const override
    {
        ExtendResult r;
        check(bwacuda_extend(ctx_->get(), query.ptr, (int32_t)query.len, target.ptr, (int32_t)target.len, (int)m,
                             mat, o_del, e_del, o_ins, e_ins, w, end_bonus, zdrop, h0, &r),
              "bwacuda_extend");
        return r;
    }

    std::vector<ExtendResult> extend_batch(const std::vector<ExtendJob> &jobs, size_t m, const int8_t *mat,
                                           int o_del, int e_del, int o_ins, int e_ins, int w, int end_bonus,
                                           int zdrop) const override
    {
        std::vector<bwacuda_ext_job> cj(jobs.size());
        for (size_t k = 0; k < jobs.size(); ++k)
            cj[k] = bwacuda_ext_job{jobs[k].query.ptr, jobs[k].target.ptr, (int32_t)jobs[k].query.len,
                                    (int32_t)jobs[k].target.len, jobs[k].h0};
        std::vector<ExtendResult> out(jobs.size());
        check(bwacuda_extend_batch(ctx_->get(), cj.data(), cj.size(), (int)m, mat, o_del, e_del, o_ins, e_ins, w,
                                   end_bonus, zdrop, out.data()),
              "bwacuda_extend_batch");
        return out;
    }

private:
    Context *ctx_;
};

inline std::vector<bwacuda_rescue_job> to_c(const std::vector<KswJob> &jobs)
{
    std::vector<bwacuda_rescue_job> cj(jobs.size());
    for (size_t k = 0; k < jobs.size(); ++k)
        cj[k] = bwacuda_rescue_job{jobs[k].query.ptr, jobs[k].target.ptr, (int32_t)jobs[k].query.len,
                                   (int32_t)jobs[k].target.len};
    return cj;
}

// bwa_neon::batched_ksw_align2
inline std::vector<KswAlignResult> batched_ksw_align2(Context &ctx, const std::vector<KswJob> &jobs, size_t m,
                                                      const int8_t *mat, int o_del, int e_del, int o_ins,
                                                      int e_ins, int minsc, int max_sc)
{
    auto cj = to_c(jobs);
    std::vector<KswAlignResult> out(jobs.size());
    check(bwacuda_ksw_align2_batch(ctx.get(), cj.data(), cj.size(), (int)m, mat, o_del, e_del, o_ins, e_ins, minsc,
                                   max_sc, out.data()),
          "bwacuda_ksw_align2_batch");
    return out;
}

// bwa_extend::ksw_align2 (one job; lanes = 16 or 8)
inline KswAlignResult ksw_align2(Context &ctx, Bytes query, Bytes target, size_t m, const int8_t *mat, int o_del,
                                 int e_del, int o_ins, int e_ins, int minsc, int max_sc, int lanes)
{
    bwacuda_rescue_job j{query.ptr, target.ptr, (int32_t)query.len, (int32_t)target.len};
    KswAlignResult r;
    check(bwacuda_ksw_align2_scalar_batch(ctx.get(), &j, 1, (int)m, mat, o_del, e_del, o_ins, e_ins, minsc, max_sc,
                                          lanes, &r),
          "bwacuda_ksw_align2_scalar_batch");
    return r;
}

// bwa_extend::ksw_global2 over many alignments: (score, CIGAR runs) per job,
// the CIGAR as the reference's packed words (len << 4 | op, op 0=M 1=I 2=D).
struct GlobalJob {
    Bytes query, target;
    int32_t w;
};

inline std::vector<std::pair<int32_t, std::vector<uint32_t>>> ksw_global2_batch(
    Context &ctx, const std::vector<GlobalJob> &jobs, size_t m, const int8_t *mat, int o_del, int e_del, int o_ins,
    int e_ins)
{
    std::vector<bwacuda_global_job> cj(jobs.size());
    size_t cap = 0;
    for (size_t k = 0; k < jobs.size(); ++k) {
        cj[k] = bwacuda_global_job{jobs[k].query.ptr, jobs[k].target.ptr, (int32_t)jobs[k].query.len,
                                   (int32_t)jobs[k].target.len, jobs[k].w};
        cap += jobs[k].query.len + jobs[k].target.len;  // always enough words
    }
    std::vector<int32_t> score(jobs.size());
    std::vector<uint64_t> off(jobs.size() + 1);
    std::vector<uint32_t> words(cap + 1);
    check(bwacuda_ksw_global2_batch(ctx.get(), cj.data(), cj.size(), (int)m, mat, o_del, e_del, o_ins, e_ins,
                                    score.data(), off.data(), words.data(), words.size()),
          "bwacuda_ksw_global2_batch");
    std::vector<std::pair<int32_t, std::vector<uint32_t>>> out(jobs.size());
    for (size_t k = 0; k < jobs.size(); ++k)
        out[k] = {score[k], std::vector<uint32_t>(words.begin() + (ptrdiff_t)off[k], words.begin() + (ptrdiff_t)off[k + 1])};
    return out;
}

// bwa_extend::ksw_global2: one alignment.
inline std::pair<int32_t, std::vector<uint32_t>> ksw_global2(Context &ctx, Bytes query, Bytes target, size_t m,
                                                            const int8_t *mat, int o_del, int e_del, int o_ins,
                                                            int e_ins, int w)
{
    return ksw_global2_batch(ctx, {GlobalJob{query, target, w}}, m, mat, o_del, e_del, o_ins, e_ins)[0];
}

// run_side's band-doubling loop over one side's jobs: results and the band each
// job was accepted at; prev as run_side starts it (-1 left, h0 right).
inline std::pair<std::vector<ExtendResult>, std::vector<int32_t>> run_side_extend(
    Context &ctx, const std::vector<ExtendJob> &jobs, const std::vector<int32_t> &prev, size_t m, const int8_t *mat,
    int o_del, int e_del, int o_ins, int e_ins, int w, int pen_clip, int zdrop, int max_band_try)
{
    std::vector<bwacuda_ext_job> cj(jobs.size());
    for (size_t k = 0; k < jobs.size(); ++k)
        cj[k] = bwacuda_ext_job{jobs[k].query.ptr, jobs[k].target.ptr, (int32_t)jobs[k].query.len,
                                (int32_t)jobs[k].target.len, jobs[k].h0};
    std::vector<ExtendResult> out(jobs.size());
    std::vector<int32_t> w_used(jobs.size());
    check(bwacuda_extend_batch_retry(ctx.get(), cj.data(), cj.size(), (int)m, mat, o_del, e_del, o_ins, e_ins, w,
                                     pen_clip, zdrop, max_band_try, prev.empty() ? nullptr : prev.data(), out.data(),
                                     w_used.data()),
          "bwacuda_extend_batch_retry");
    return {out, w_used};
}

}  // namespace bwa_cuda
