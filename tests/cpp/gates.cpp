// The reference's SwBackend acceptance gates, restated in C++ and run against
// bwa_cuda::CudaBackend through the C++ mirror (include/bwacuda.hpp):
//   assert_backend_matches_scalar        crates/bwa-extend/src/lib.rs:283-354
//   assert_backend_batch_matches_scalar  crates/bwa-extend/src/lib.rs:426-525
//   matesw_equals_scalar (first 500 jobs) crates/bwa-neon/src/matesw.rs:5045-5139
// The expected values come from the CPU oracle (oracle/ksw_oracle.c), the checker.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "bwacuda.hpp"
#include "ksw_oracle.h"

namespace {

struct Lcg {
    uint64_t s;
    explicit Lcg(uint64_t seed) : s(seed) {}
    uint64_t operator()() { s = s * 6364136223846793005ull + 1442695040888963407ull; return s >> 33; }
};

bool same(const bwa_cuda::ExtendResult &a, const ko_ext_result &b)
{
    return a.score == b.score && a.qle == b.qle && a.tle == b.tle && a.gtle == b.gtle && a.gscore == b.gscore &&
           a.max_off == b.max_off;
}

int gate_single(bwa_cuda::CudaBackend &be)
{
    Lcg nx(0x9E3779B97F4A7C15ull);
    for (int c = 0; c < 2000; ++c) {
        int ql = 1 + nx() % 60, tl = 1 + nx() % 60;
        std::vector<uint8_t> q(ql), t(tl);
        for (auto &x : q) x = nx() % 4;
        for (auto &x : t) x = nx() % 4;
        int w = 1 + nx() % 30, zdrop = nx() % 120, eb = nx() % 10, h0 = 1 + nx() % 20;
        int a = 1, b = 4, od = 6, ed = 1, oi = 6, ei = 1;
        if (c) { a = 1 + nx() % 4; b = 1 + nx() % 6; od = 1 + nx() % 8; ed = 1 + nx() % 3; oi = 1 + nx() % 8; ei = 1 + nx() % 3; }
        int8_t mat[25];
        ko_fill_scmat(a, b, mat);
        auto got = be.extend(q, t, 5, mat, od, ed, oi, ei, w, eb, zdrop, h0);
        auto want = ko_extend2(q.data(), ql, t.data(), tl, 5, mat, od, ed, oi, ei, w, eb, zdrop, h0, nullptr);
        if (!same(got, want)) { std::printf("single case %d diverged\n", c); return 1; }
    }
    return 0;
}

int gate_batch(bwa_cuda::CudaBackend &be)
{
    Lcg nx(0x123456789ABCDEF0ull);
    const int sizes[] = {1, 2, 3, 4, 7, 8, 9, 15, 16, 17, 20, 31};
    int8_t mat[25];
    ko_fill_scmat(1, 4, mat);
    for (int r = 0; r < 200; ++r) {
        int bs = sizes[nx() % 12];
        int w = 1 + nx() % 30, zdrop = nx() % 120, eb = nx() % 10;
        int od = 4 + nx() % 4, ed = 1 + nx() % 2, oi = 4 + nx() % 4, ei = 1 + nx() % 2;
        std::vector<std::vector<uint8_t>> qs(bs), ts(bs);
        for (auto &q : qs) { q.resize(1 + nx() % 80); for (auto &x : q) x = nx() % 4; }
        for (auto &t : ts) { t.resize(1 + nx() % 80); for (auto &x : t) x = nx() % 4; }
        std::vector<bwa_cuda::ExtendJob> jobs(bs);
        for (int k = 0; k < bs; ++k) jobs[k] = {qs[k], ts[k], (int32_t)(1 + nx() % 20)};
        auto got = be.extend_batch(jobs, 5, mat, od, ed, oi, ei, w, eb, zdrop);
        for (int k = 0; k < bs; ++k) {
            auto want = ko_extend2(qs[k].data(), (int)qs[k].size(), ts[k].data(), (int)ts[k].size(), 5, mat, od, ed,
                                   oi, ei, w, eb, zdrop, jobs[k].h0, nullptr);
            if (!same(got[k], want)) { std::printf("batch round %d job %d diverged\n", r, k); return 1; }
        }
    }
    return 0;
}

int gate_rescue(bwa_cuda::Context &ctx)
{
    Lcg nx(0x123456789ABCDEF1ull);
    std::vector<std::vector<uint8_t>> qs, ts;
    for (int k = 0; k < 500; ++k) {
        int ql = 5 + nx() % 146, tl = ql + nx() % 500;
        std::vector<uint8_t> t(tl), q(ql);
        for (auto &x : t) x = nx() % 5;
        for (auto &x : q) x = nx() % 5;
        int copies = 1 + nx() % 2;
        if (nx() % 5 != 0) {
            for (int c = 0; c < copies; ++c)
                if (tl > ql) { int at = nx() % (tl - ql + 1); std::memcpy(&t[at], q.data(), ql); }
            int nm = nx() % 4;
            for (int c = 0; c < nm; ++c) { int p = nx() % ql; q[p] = nx() % 4; }
        }
        if (nx() % 4 == 0) q[nx() % ql] = 4;
        if (nx() % 4 == 0) t[nx() % tl] = 4;
        qs.push_back(q);
        ts.push_back(t);
    }
    int8_t mat[25];
    ko_fill_scmat(1, 4, mat);
    std::vector<bwa_cuda::KswJob> jobs;
    for (size_t k = 0; k < qs.size(); ++k) jobs.push_back({qs[k], ts[k]});
    auto got = bwa_cuda::batched_ksw_align2(ctx, jobs, 5, mat, 6, 1, 6, 1, 19, 1);
    for (size_t k = 0; k < qs.size(); ++k) {
        auto w = ko_align2_batched(qs[k].data(), (int)qs[k].size(), ts[k].data(), (int)ts[k].size(), 5, mat, 6, 1,
                                   6, 1, 19, 1);
        auto &g = got[k];
        if (g.score != w.score || g.qb != w.qb || g.qe != w.qe || g.tb != w.tb || g.te != w.te ||
            g.score2 != w.score2 || g.te2 != w.te2) {
            std::printf("rescue job %zu diverged\n", k);
            return 1;
        }
    }
    return 0;
}

// crates/bwa-extend/src/sw.rs:1358-1380 through the C++ mirror, and a batch of
// random alignments against the oracle's restatement.
int gate_global(bwa_cuda::Context &ctx)
{
    int8_t mat[25];
    ko_fill_scmat(1, 4, mat);
    const std::vector<uint8_t> s = {0, 1, 2, 3, 0, 1, 2, 3, 0, 1};
    auto r = bwa_cuda::ksw_global2(ctx, s, s, 5, mat, 6, 1, 6, 1, 100);
    if (r.first != (int)s.size() || r.second != std::vector<uint32_t>{(uint32_t)s.size() << 4}) {
        std::printf("global exact match diverged\n");
        return 1;
    }
    std::vector<uint8_t> q = {0, 1, 2, 3, 0, 1, 2, 3}, t = q;
    t.insert(t.begin() + 4, 2);
    r = bwa_cuda::ksw_global2(ctx, q, t, 5, mat, 6, 1, 6, 1, 100);
    uint32_t dsum = 0, msum = 0;
    for (uint32_t c : r.second) {
        if ((c & 0xf) == 2) dsum += c >> 4;
        if ((c & 0xf) == 0) msum += c >> 4;
    }
    if (dsum != 1 || msum != q.size()) {
        std::printf("global single deletion diverged\n");
        return 1;
    }
    uint64_t x = 88172645463325252ull;
    auto rnd = [&x]() { x ^= x << 13; x ^= x >> 7; x ^= x << 17; return x; };
    std::vector<std::vector<uint8_t>> qs(400), ts(400);
    std::vector<bwa_cuda::GlobalJob> jobs;
    for (int k = 0; k < 400; ++k) {
        const int len = 20 + (int)(rnd() % 200);
        for (int i = 0; i < len; ++i) ts[k].push_back((uint8_t)(rnd() % 4));
        qs[k] = ts[k];
        for (int e = 0; e < 3; ++e) qs[k][rnd() % qs[k].size()] = (uint8_t)(rnd() % 4);
        if (rnd() % 3 == 0) qs[k].erase(qs[k].begin() + (ptrdiff_t)(rnd() % qs[k].size()));
        const int diff = std::abs((int)qs[k].size() - (int)ts[k].size());
        jobs.push_back(bwa_cuda::GlobalJob{qs[k], ts[k], diff + 3 + (int)(rnd() % 40)});
    }
    auto got = bwa_cuda::ksw_global2_batch(ctx, jobs, 5, mat, 6, 1, 6, 1);
    std::vector<uint32_t> cig(1024);
    for (size_t k = 0; k < jobs.size(); ++k) {
        int32_t sc = 0;
        int nc = 0;
        if (ko_global2(qs[k].data(), (int)qs[k].size(), ts[k].data(), (int)ts[k].size(), 5, mat, 6, 1, 6, 1,
                       jobs[k].w, &sc, cig.data(), &nc) != 0)
            continue;
        if (got[k].first != sc || got[k].second != std::vector<uint32_t>(cig.begin(), cig.begin() + nc)) {
            std::printf("global job %zu diverged\n", k);
            return 1;
        }
    }
    return 0;
}

}  // namespace

int main()
{
    try {
        bwa_cuda::Context ctx(0);
        bwa_cuda::CudaBackend be(ctx);
        if (std::strcmp(be.name(), "cuda") != 0) return 2;
        int rc = gate_single(be) | gate_batch(be);
        ctx.set_option(BWACUDA_OPT_EXT_PATH, BWACUDA_PATH_BATCHED);
        rc |= gate_batch(be) | gate_rescue(ctx) | gate_global(ctx);
        std::printf(rc ? "FAIL\n" : "gates ok\n");
        return rc;
    } catch (const bwa_cuda::Error &e) {
        std::printf("error: %s\n", e.what());
        return 3;
    }
}
