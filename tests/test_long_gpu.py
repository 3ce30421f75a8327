"""Extension of queries of any length (the group-per-job kernel, csrc/ext_long.cuh) against the
oracle, bit-exact on every field.

The reference's ksw_extend2 (crates/bwa-extend/src/sw.rs:203-493) takes any query length, and its
batched dispatch sends long jobs to the 16-bit bins up to 32767 and to the scalar path beyond
(crates/bwa-neon/src/batched.rs:850-866).  Covered here: queries of 1,000-10,000 bases with
substitutions, indels, N and z-drop tails, 16-bit and 32-bit cells (h0 near 32768, a 40,000-base
query), long queries against short targets (8-bit values), bands too wide for the first launch's
ring (the deferred launch), every host-buffer route, the device-resident calls, the band-doubling
retry and the serving loop, and the knobs that route shorter buckets to the same kernel (every
lane count), including the reference's swept-scoring gate stream run through it entirely."""
import numpy as np
import pytest

import bwacuda as B
import oracle
import refstreams as R

pytestmark = pytest.mark.gpu


def _mutate(rng, t, ql, sub=0.01, indel=0.001, tail_from=None, tail_rate=0.3):
    """A query of about ql bases copied from target t: substitutions, 1-3 bp indels, and an
    error-dense tail from tail_from on (to trigger z-drop)."""
    q = t[:ql].copy()
    mask = rng.random(ql) < sub
    q[mask] = (q[mask] + rng.integers(1, 4, int(mask.sum()))) % 4
    if tail_from is not None and tail_from < ql:
        m2 = rng.random(ql - tail_from) < tail_rate
        seg = q[tail_from:]
        seg[m2] = (seg[m2] + rng.integers(1, 4, int(m2.sum()))) % 4
    out = []
    i = 0
    while i < len(q):
        if rng.random() < indel:
            ln = int(rng.integers(1, 4))
            if rng.random() < 0.5:
                i += ln  # deletion from the query
                continue
            out.extend(rng.integers(0, 4, ln).tolist())  # insertion
        out.append(int(q[i]))
        i += 1
    return np.array(out, dtype=np.uint8)


def long_jobs(n, qmin, qmax, w, seed, h0=(20, 60), short_targets=False):
    rng = np.random.default_rng(seed)
    qs, ts, h0s = [], [], []
    for k in range(n):
        ql = int(rng.integers(qmin, qmax + 1))
        tl = ql + w + 8
        t = rng.integers(0, 4, tl).astype(np.uint8)
        t[rng.random(tl) < 0.001] = 4
        tail = int(rng.integers(ql // 4, ql)) if k % 5 == 0 else None
        q = _mutate(rng, t, ql, tail_from=tail)
        if short_targets:
            t = t[:int(rng.integers(20, 120))]
        qs.append(q)
        ts.append(t)
        h0s.append(int(rng.integers(h0[0], h0[1] + 1)))
    return B.JobSet.from_lists(qs, ts, h0s, w)


def _mix(long_js, short_n, seed, w):
    """The long jobs interleaved with read-pair jobs (one call holds both kinds)."""
    sh = B.synth_ext(2, short_n, seed=seed)
    qs = [long_js.query(k) for k in range(len(long_js))] + [sh.query(k) for k in range(len(sh))]
    ts = [long_js.target(k) for k in range(len(long_js))] + [sh.target(k) for k in range(len(sh))]
    h0 = np.concatenate([long_js.h0, sh.h0])
    perm = np.random.default_rng(seed).permutation(len(qs))
    return B.JobSet.from_lists([qs[i] for i in perm], [ts[i] for i in perm], h0[perm], w)


# (path, gather route, window-kernel mode): mode 2 runs the thread-per-job window kernel
# (csrc/ext_slide.cu) on every open-ended bucket however few jobs it holds; mode 1 (the default)
# leaves buckets under 32 jobs per SM, every bucket of these small cases, to the group kernel
ROUTES = [pytest.param((B.PATH_PLAIN, B.GATHER_AUTO, 1), id="plain"),
          pytest.param((B.PATH_BATCHED, B.GATHER_HOST, 1), id="batched-hostpack"),
          pytest.param((B.PATH_BATCHED, B.GATHER_DEVICE, 1), id="batched-devgather"),
          pytest.param((B.PATH_BATCHED, B.GATHER_HOST, 2), id="batched-hostpack-window"),
          pytest.param((B.PATH_BATCHED, B.GATHER_DEVICE, 2), id="batched-devgather-window")]


@pytest.fixture(params=ROUTES)
def rctx(ctx, request):
    path, gather, slide = request.param
    ctx.set_option(B.OPT_EXT_PATH, path)
    ctx.set_option(B.OPT_HOST_GATHER, gather)
    ctx.set_option(B.OPT_LONG_SLIDE, slide)
    yield ctx
    ctx.set_option(B.OPT_EXT_PATH, B.PATH_BATCHED)
    ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)
    ctx.set_option(B.OPT_LONG_SLIDE, 1)


@pytest.fixture
def wctx(ctx):
    """Batched path with the window kernel on every open-ended bucket."""
    ctx.set_option(B.OPT_EXT_PATH, B.PATH_BATCHED)
    ctx.set_option(B.OPT_LONG_SLIDE, 2)
    yield ctx
    ctx.set_option(B.OPT_LONG_SLIDE, 1)


def _check(ctx, js, w, mat=None, **kw):
    got = ctx.extend_batch(js, mat, w=w, **kw)
    want, _ = oracle.extend_batch(js, mat, **kw)
    bad = np.nonzero(got != want)[0]
    assert len(bad) == 0, (f"{len(bad)} of {len(js)} differ; first job {bad[0]} qlen={js.qlen[bad[0]]} "
                           f"tlen={js.tlen[bad[0]]} h0={js.h0[bad[0]]}: {got[bad[0]]} vs {want[bad[0]]}")
    return got


def test_long_queries_16bit(rctx):
    js = long_jobs(48, 1000, 10000, 100, seed=1)
    assert js.qlen.max() > 5000
    got = _check(rctx, js, 100)
    assert (got["qle"] > 1438).sum() > 10  # past the thread-per-job rows


def test_long_queries_mixed_with_read_pairs(rctx):
    js = _mix(long_jobs(24, 1200, 6000, 100, seed=2), 3000, seed=3, w=100)
    _check(rctx, js, 100)


def test_long_queries_32bit_cells(rctx):
    # h0 close to 32768: every long job needs 32-bit cells; one 40,000-base query beyond 32767
    js = long_jobs(12, 1500, 4000, 100, seed=4, h0=(31000, 32000))
    big = long_jobs(1, 40000, 40000, 100, seed=5)
    js = B.JobSet.from_lists([js.query(k) for k in range(len(js))] + [big.query(0)],
                             [js.target(k) for k in range(len(js))] + [big.target(0)],
                             np.concatenate([js.h0, big.h0]), 100)
    _check(rctx, js, 100)


def test_long_queries_short_targets(rctx):
    # long queries against short targets keep 8-bit values (the 8-bit class's open-ended bucket)
    js = long_jobs(40, 1500, 5000, 100, seed=6, short_targets=True)
    _check(rctx, js, 100)


@pytest.mark.parametrize("w", [300, 700, 3000])
def test_wide_bands_deferred_launch(rctx, w):
    # bands whose ring exceeds the first launch's (2w + 3 > 512 columns on the batched path)
    js = long_jobs(10, 1200, 4000, w, seed=7 + w)
    _check(rctx, js, w)


def test_other_scorings(rctx):
    mat = oracle.scmat(2, 3)
    js = long_jobs(16, 1000, 3000, 100, seed=9)
    _check(rctx, js, 100, mat, o_del=5, e_del=2, o_ins=4, e_ins=3, end_bonus=0, zdrop=40)
    _check(rctx, js, 100, mat, o_del=5, e_del=2, o_ins=4, e_ins=3, end_bonus=7, zdrop=0)


@pytest.mark.parametrize("w", [99, 100, 101, 102, 140])
def test_window_kernel_band_limit(wctx, w):
    # bands up to 101 columns run in the window kernel's 272-column window (2w + 5 + 64 <= 272),
    # wider ones in the group kernel beside it
    js = long_jobs(40, 1030, 6000, w, seed=40 + w)
    _check(wctx, js, w)


def test_window_kernel_row_minus1_beyond_window(wctx):
    # h0 ~ 20000: row -1 stays positive for thousands of columns, so every column that enters
    # the window on the right carries a nonzero row -1 value
    js = long_jobs(24, 2000, 6000, 100, seed=50, h0=(19000, 23000))
    _check(wctx, js, 100)
    _check(wctx, js, 100, zdrop=0)


def test_window_kernel_target_lengths(wctx):
    # targets much longer than the query (rows past the query's end empty the band) and much
    # shorter (the 8-bit class's open-ended bucket), with the query-code check past the band
    rng = np.random.default_rng(51)
    qs, ts, h0s = [], [], []
    for k in range(30):
        ql = int(rng.integers(1100, 3000))
        tl = ql * 3 if k % 2 == 0 else int(rng.integers(30, 400))
        t = rng.integers(0, 4, max(tl, ql)).astype(np.uint8)
        q = _mutate(rng, t, ql)
        qs.append(q)
        ts.append(t[:tl])
        h0s.append(int(rng.integers(5, 90)))
    js = B.JobSet.from_lists(qs, ts, h0s, 100)
    _check(wctx, js, 100)
    _check(wctx, js, 100, end_bonus=0, zdrop=30)


def test_window_kernel_cells_and_asymmetric_gaps(wctx):
    js = long_jobs(30, 1030, 5000, 100, seed=52)
    wctx.reset_stats()
    got = wctx.extend_batch(js, w=100)
    want, cells = oracle.extend_batch(js)
    assert np.array_equal(got, want)
    assert wctx.stats()["ext_cells"] == cells
    mat = oracle.scmat(1, 4)
    _check(wctx, js, 100, mat, o_del=6, e_del=1, o_ins=4, e_ins=2, zdrop=60)


def test_window_kernel_option_values(ctx):
    for bad in (-1, 3):
        with pytest.raises(B.BwaCudaError) as e:
            ctx.set_option(B.OPT_LONG_SLIDE, bad)
        assert e.value.code == B.EINVAL
    for ok in (0, 2, 1):
        ctx.set_option(B.OPT_LONG_SLIDE, ok)


def test_window_kernel_auto_threshold(ctx):
    # default mode: a bucket of at least 32 jobs per SM runs in the window kernel, a smaller one
    # in the group kernel; results are the same either way
    ctx.set_option(B.OPT_EXT_PATH, B.PATH_BATCHED)
    rng = np.random.default_rng(53)
    n = 5200
    ql = rng.integers(1030, 1300, n)
    tl = ql + rng.integers(0, 200, n)
    ts = [rng.integers(0, 4, int(x)).astype(np.uint8) for x in tl]
    qs = []
    for k in range(n):  # substitutions at 1%, an error-dense tail on every fourth job
        q = ts[k][:ql[k]].copy()
        rate = np.where(np.arange(ql[k]) > ql[k] // 2, 0.3 if k % 4 == 0 else 0.01, 0.01)
        mask = rng.random(ql[k]) < rate
        q[mask] = (q[mask] + rng.integers(1, 4, int(mask.sum()))) % 4
        qs.append(q)
    js = B.JobSet.from_lists(qs, ts, rng.integers(20, 60, n), 100)
    want, _ = oracle.extend_batch(js)
    got = ctx.extend_batch(js, w=100)
    assert np.array_equal(got, want)
    head = js.take(np.arange(300))
    assert np.array_equal(ctx.extend_batch(head, w=100), want[:300])


@pytest.mark.parametrize("path", [B.PATH_PLAIN, B.PATH_BATCHED])
def test_device_resident_per_job_bands(ctx, path):
    import torch

    js = _mix(long_jobs(20, 1000, 5000, 100, seed=10), 2000, seed=11, w=100)
    js.w = np.where(np.arange(len(js)) % 3 == 0, 700, 100).astype(np.int32)  # some need the deferred ring
    want, _ = oracle.extend_batch(js)
    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_ext_jobs().view(np.uint8)).cuda()
    d_out = torch.zeros(len(js) * 24, dtype=torch.uint8, device="cuda")
    for _ in range(2):  # the batched path replays its captured graph on the second call
        d_out.zero_()
        ctx.extend_device(d_seq.data_ptr(), d_jobs.data_ptr(), len(js), d_out.data_ptr(), path=path)
        ctx.sync()
        got = d_out.cpu().numpy().view(oracle.EXT_DTYPE)
        assert np.array_equal(got, want)


@pytest.mark.parametrize("lanes", [8, 16, 32])
@pytest.mark.parametrize("qlo", [1, 129])
def test_knobs_route_shorter_buckets(ctx, lanes, qlo):
    ctx.set_option(B.OPT_EXT_PATH, B.PATH_BATCHED)
    ctx.set_option(B.OPT_LONG_QLEN, qlo)
    ctx.set_option(B.OPT_LONG_LANES, lanes)
    try:
        js = B.synth_ext(3, 20000, seed=12)
        want, _ = oracle.extend_batch(js)
        for wv in np.unique(js.w):
            idx = np.nonzero(js.w == wv)[0]
            got = ctx.extend_batch(js.take(idx), w=int(wv))
            assert np.array_equal(got, want[idx])
        js = long_jobs(12, 1000, 3000, 100, seed=13)
        _check(ctx, js, 100)
    finally:
        ctx.set_option(B.OPT_LONG_QLEN, 0)
        ctx.set_option(B.OPT_LONG_LANES, 16)


@pytest.mark.parametrize("lanes", [8, 32])
def test_gate_stream_through_group_kernel(ctx, lanes):
    # crates/bwa-extend/src/lib.rs:283-354 (2000 cases, scoring swept), every job in the group kernel
    ctx.set_option(B.OPT_EXT_PATH, B.PATH_BATCHED)
    ctx.set_option(B.OPT_LONG_QLEN, 1)
    ctx.set_option(B.OPT_LONG_LANES, lanes)
    try:
        groups = {}
        for c in R.backend_matches_scalar():
            key = (c["a"], c["b"], c["o_del"], c["e_del"], c["o_ins"], c["e_ins"], c["w"], c["end_bonus"],
                   c["zdrop"])
            groups.setdefault(key, []).append(c)
        for key, cs in groups.items():
            a, b, od, ed, oi, ei, w, eb, zd = key
            mat = oracle.scmat(a, b)
            js = B.JobSet.from_lists([c["q"] for c in cs], [c["t"] for c in cs], [c["h0"] for c in cs], w)
            got = ctx.extend_batch(js, mat, od, ed, oi, ei, w, eb, zd)
            want = [oracle.extend2(c["q"], c["t"], c["h0"], mat, od, ed, oi, ei, w, eb, zd) for c in cs]
            for k, (g, x) in enumerate(zip(got, want)):
                assert tuple(int(v) for v in g) == x, f"{key} job {k}"
    finally:
        ctx.set_option(B.OPT_LONG_QLEN, 0)
        ctx.set_option(B.OPT_LONG_LANES, 16)


def test_retry_with_long_queries(ctx):
    from test_retry_gpu import _oracle_retry

    js = long_jobs(20, 1000, 4000, 100, seed=14)
    prev = np.where(np.arange(len(js)) % 2 == 0, -1, js.h0).astype(np.int32)
    want, want_w = _oracle_retry(js, prev, 2, np.full(len(js), 100))
    got, got_w = ctx.extend_batch_retry(js, prev, 2, w=100)
    assert np.array_equal(got, want)
    assert np.array_equal(got_w, want_w)


def test_serving_long_queries(ctx):
    js = _mix(long_jobs(10, 1000, 4000, 100, seed=15), 1500, seed=16, w=100)
    want, _ = oracle.extend_batch(js)
    ctx.server_start(hbm_budget_bytes=256 << 20, max_waves=2)
    try:
        out, _ = ctx.wait(ctx.submit_extend(js))
    finally:
        ctx.server_stop()
    assert np.array_equal(out, want)
