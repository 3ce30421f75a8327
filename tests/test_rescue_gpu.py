"""Mate-rescue parity: ksw_align2 / batched_ksw_align2 / ksw_local_fwd on the GPU
against the oracle, bit-exact on (score, qb, qe, tb, te, score2, te2)."""
import numpy as np
import pytest

import bwacuda as B
import oracle
import refstreams as R

pytestmark = pytest.mark.gpu

# (kernel family, lanes per job of the register wavefront)
KERNELS = [pytest.param((B.RESCUE_AUTO, 16, 0), id="wavefront16"), pytest.param((B.RESCUE_AUTO, 8, 0), id="wavefront8"),
           pytest.param((B.RESCUE_AUTO, 32, 0), id="wavefront32"), pytest.param((B.RESCUE_TPJ, 16, 0), id="tpj"),
           pytest.param((B.RESCUE_AUTO, 8, 4), id="paired4"), pytest.param((B.RESCUE_AUTO, 8, 8), id="paired8"),
           pytest.param((B.RESCUE_AUTO, 16, 16), id="paired16")]


@pytest.fixture(params=KERNELS)
def rctx(ctx, request):
    """The context with the rescue kernel family under test selected."""
    kernel, lanes, pair = request.param
    ctx.set_option(B.OPT_RESCUE_KERNEL, kernel)
    ctx.set_option(B.OPT_RESCUE_LANES, lanes)
    ctx.set_option(B.OPT_RESCUE_PAIR, pair)
    yield ctx
    ctx.set_option(B.OPT_RESCUE_KERNEL, B.RESCUE_AUTO)
    ctx.set_option(B.OPT_RESCUE_LANES, 16)
    ctx.set_option(B.OPT_RESCUE_PAIR, 0)


def _js(pairs):
    return B.JobSet.from_lists([p[0] for p in pairs], [p[1] for p in pairs])


def test_known_answers(rctx):
    js = _js([([0, 1, 2, 3, 0, 1, 2, 3], [0, 1, 2, 3, 0, 1, 2, 3])])
    r = rctx.ksw_align2_scalar_batch(js, oracle.scmat(1, 4), 6, 1, 6, 1, 4, 1, 16)[0]
    assert tuple(int(x) for x in r)[:5] == (8, 0, 7, 0, 7)
    js = _js([([3, 3, 0, 0, 1, 1, 3, 3], [2, 0, 0, 1, 1, 2])])
    r = rctx.ksw_align2_scalar_batch(js, oracle.scmat(1, 4), 6, 1, 6, 1, 1, 1, 16)[0]
    assert tuple(int(x) for x in r)[:5] == (4, 2, 5, 1, 4)


@pytest.mark.parametrize("a,b,minsc", [(1, 4, 19), (10, 40, 190)])
def test_matesw_stream_batched_and_scalar(rctx, a, b, minsc):
    # crates/bwa-neon/src/matesw.rs:5045-5139
    pairs = R.matesw_jobs()
    js = _js(pairs)
    mat = oracle.scmat(a, b)
    want_b, _ = oracle.align2_batch(js, mat, 6, 1, 6, 1, minsc, a, mode=0)
    got_b = rctx.ksw_align2_batch(js, mat, 6, 1, 6, 1, minsc, a)
    assert np.array_equal(got_b, want_b)
    want_s, _ = oracle.align2_batch(js, mat, 6, 1, 6, 1, minsc, a, mode=1)
    got_s = rctx.ksw_align2_scalar_batch(js, mat, 6, 1, 6, 1, minsc, a, 0)
    assert np.array_equal(got_s, want_s)


def test_pad_columns_stream(rctx):
    js = _js(R.matesw_pad_columns())
    want = oracle.local_fwd_batch(js, 19, oracle.INT_MAX)
    got = rctx.ksw_local_fwd_batch(js, 19, B.INT_MAX)
    assert np.array_equal(got, want)
    assert int((got["score2"] >= 0).sum()) >= 8


def test_ragged_tlen_endsc_stream(rctx):
    js = _js(R.matesw_ragged())
    want = oracle.local_fwd_batch(js, 19, 60)
    got = rctx.ksw_local_fwd_batch(js, 19, 60)
    assert np.array_equal(got, want)


def test_bench_jobs_stream(rctx):
    js = _js(R.rescue_bench_jobs(2048))
    want, _ = oracle.align2_batch(js, minsc=19)
    assert np.array_equal(rctx.ksw_align2_batch(js, minsc=19), want)


@pytest.mark.parametrize("lanes", [8, 16])
def test_fixed_lanes(rctx, lanes):
    js = _js(R.matesw_jobs()[:500])
    want, _ = oracle.align2_batch(js, minsc=19, mode=1, lanes=lanes)
    assert np.array_equal(rctx.ksw_align2_scalar_batch(js, minsc=19, lanes=lanes), want)


def test_workload_windows(rctx):
    js = B.synth_rescue(20000, seed=4)
    want, _ = oracle.align2_batch(js, minsc=20)
    got = rctx.ksw_align2_batch(js, minsc=20)
    assert np.array_equal(got, want)


def test_device_entry(rctx):
    import torch

    js = B.synth_rescue(5000, seed=6)
    want, _ = oracle.align2_batch(js, minsc=20)
    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_res_jobs().view(np.uint8)).cuda()
    d_out = torch.zeros(len(js) * 28, dtype=torch.uint8, device="cuda")
    rctx.ksw_align2_device(d_seq.data_ptr(), d_jobs.data_ptr(), len(js), d_out.data_ptr(), minsc=20)
    rctx.sync()
    assert np.array_equal(d_out.cpu().numpy().view(B.ALN_RES), want)


def test_device_entry_in_pieces(rctx):
    import torch

    js = B.synth_rescue(5000, seed=16)
    want, _ = oracle.align2_batch(js, minsc=20)
    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_res_jobs().view(np.uint8)).cuda()
    d_out = torch.zeros(len(js) * 28, dtype=torch.uint8, device="cuda")
    rctx.set_option(B.OPT_DEVICE_PIECE, 1201)  # four whole pieces and a ragged one
    try:
        rctx.ksw_align2_device(d_seq.data_ptr(), d_jobs.data_ptr(), len(js), d_out.data_ptr(), minsc=20)
        rctx.sync()
    finally:
        rctx.set_option(B.OPT_DEVICE_PIECE, 1 << 30)
    assert np.array_equal(d_out.cpu().numpy().view(B.ALN_RES), want)


def test_edge_cases(rctx):
    pairs = [([], [0, 1, 2]), ([0, 1], []), ([], []), ([4, 4, 4], [4, 4, 4]), ([0] * 300, [0] * 400),
             ([1, 2, 3, 0] * 70, [1, 2, 3, 0] * 100), ([2], [2])]
    js = _js(pairs)
    for minsc in (0, 1, 19):
        want, _ = oracle.align2_batch(js, minsc=minsc)
        assert np.array_equal(rctx.ksw_align2_batch(js, minsc=minsc), want)
        want, _ = oracle.align2_batch(js, minsc=minsc, mode=1)
        assert np.array_equal(rctx.ksw_align2_scalar_batch(js, minsc=minsc), want)


def test_wide_scores(rctx):
    # min(q,t) * max_sc >= 32768 needs int32 cells
    rng = np.random.default_rng(3)
    q = rng.integers(0, 4, 400).tolist()
    t = rng.integers(0, 4, 100).tolist() + q + rng.integers(0, 4, 100).tolist()
    mat = oracle.scmat(100, 120)
    js = _js([(q, t), (q[:50], t)])
    want, _ = oracle.align2_batch(js, mat, 6, 1, 6, 1, 500, 100)
    assert np.array_equal(rctx.ksw_align2_batch(js, mat, 6, 1, 6, 1, 500, 100), want)


def test_invalid_inputs(ctx):
    js = _js([([0, 1, 7], [0, 1, 2])])
    with pytest.raises(B.BwaCudaError) as e:
        ctx.ksw_align2_batch(js)
    assert e.value.code == B.EBASE
    with pytest.raises(B.BwaCudaError) as e:
        ctx.ksw_align2_batch(_js([([0], [0])]), max_sc=0)
    assert e.value.code == B.EINVAL


def test_autotune_rescue_keeps_results(ctx):
    import torch

    js = B.synth_rescue(20000, seed=41)
    want, _ = oracle.align2_batch(js, minsc=20, mode=0)
    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_res_jobs().view(np.uint8)).cuda()
    d_out = torch.zeros(len(js) * 28, dtype=torch.uint8, device="cuda")
    try:
        t = ctx.autotune_rescue(d_seq.data_ptr(), d_jobs.data_ptr(), len(js), minsc=20, max_sc=1, sample=8192)
        # the 32-bit wavefront at 8/16/32 lanes, thread-per-job, the paired wavefront in groups of
        # 4/8/16 lanes
        assert t["candidates"] == 7 and t["rescue_gcups"] > 0
        assert (t["rescue_kernel"], t["rescue_lanes"], t["rescue_pair"]) in {
            (B.RESCUE_AUTO, 8, 0), (B.RESCUE_AUTO, 16, 0), (B.RESCUE_AUTO, 32, 0), (B.RESCUE_TPJ, 16, 0),
            (B.RESCUE_AUTO, 8, 4), (B.RESCUE_AUTO, 8, 8), (B.RESCUE_AUTO, 8, 16)}
        ctx.ksw_align2_device(d_seq.data_ptr(), d_jobs.data_ptr(), len(js), d_out.data_ptr(), minsc=20, max_sc=1)
        ctx.sync()
        assert np.array_equal(d_out.cpu().numpy().view(B.ALN_RES), want)
    finally:
        ctx.set_option(B.OPT_RESCUE_KERNEL, B.RESCUE_AUTO)
        ctx.set_option(B.OPT_RESCUE_LANES, 16)


def _pair_mix(seed, n):
    """Jobs on both sides of the paired wavefront's limits in one batch: byte-range windows,
    queries whose score can pass 255 (qlen 260-300 at a = 1), short and empty targets, ragged
    target lengths inside a pair, N in queries and targets."""
    rng = np.random.default_rng(seed)
    pairs = []
    for k in range(n):
        kind = k % 5
        ql = int(rng.integers(100, 160)) if kind < 3 else int(rng.integers(256, 300))
        tl = int(rng.integers(0, 40)) if kind == 4 else int(rng.integers(200, 900))
        t = rng.integers(0, 4, tl)
        q = rng.integers(0, 4, ql)
        if tl > ql and kind != 2:
            at = int(rng.integers(0, tl - ql + 1))
            t[at:at + ql] = q
            flip = rng.random(ql) < 0.02
            q[flip] = (q[flip] + 1) % 4
        q[rng.random(ql) < 0.01] = 4
        if tl:
            t[rng.random(tl) < 0.01] = 4
        pairs.append((q.tolist(), t.tolist()))
    return pairs


@pytest.mark.parametrize("lanes", [4, 8, 16])
@pytest.mark.parametrize("scoring", [(1, 4, 6, 1), (2, 3, 5, 2)])
def test_paired_wavefront_limits(ctx, lanes, scoring):
    a, b, o, e = scoring
    mat = oracle.scmat(a, b)
    js = _js(_pair_mix(100 + lanes + a, 3001))  # odd: the last pair has one job
    ctx.set_option(B.OPT_RESCUE_PAIR, lanes)
    ctx.set_option(B.OPT_RESCUE_LANES, 16 if lanes == 16 else 8)
    try:
        for mode in (0, 1):
            want, _ = oracle.align2_batch(js, mat, o, e, o, e, 19 * a, a, mode=mode)
            got = (ctx.ksw_align2_batch(js, mat, o, e, o, e, 19 * a, a) if mode == 0 else
                   ctx.ksw_align2_scalar_batch(js, mat, o, e, o, e, 19 * a, a, 0))
            assert np.array_equal(got, want), mode
        want = oracle.local_fwd_batch(js, 19 * a, 40 * a, mat, o, e, o, e, a)
        assert np.array_equal(ctx.ksw_local_fwd_batch(js, 19 * a, 40 * a, mat, o, e, o, e, a), want)
    finally:
        ctx.set_option(B.OPT_RESCUE_PAIR, 0)
        ctx.set_option(B.OPT_RESCUE_LANES, 16)


def test_paired_wavefront_other_matrices(ctx):
    # an N column or N row of several values, or o_del + e_del above 128, keeps every job in the
    # 32-bit wavefront; an asymmetric 4x4 block with a constant N row and column runs paired, and
    # so do gap costs whose two opens differ (F then opens from M0, not from the shared H - o - e)
    js = _js(_pair_mix(7, 800))
    odd = oracle.scmat(1, 4).copy()
    odd[4] = -2  # mat[0][4]: the N column is no longer one value
    odd_row = oracle.scmat(1, 4).copy()
    odd_row[20 + 1] = -2  # mat[4][1]: the N row is no longer one value
    asym = oracle.scmat(1, 4).copy()
    asym[1], asym[5 + 2], asym[10 + 3] = -3, -2, -1  # mat[0][1], mat[1][2], mat[2][3]
    ctx.set_option(B.OPT_RESCUE_PAIR, 1)  # 1: groups of 4 lanes
    ctx.set_option(B.OPT_RESCUE_LANES, 8)
    try:
        for mat in (odd, odd_row, asym):
            want, _ = oracle.align2_batch(js, mat, 6, 1, 6, 1, 19, 1)
            assert np.array_equal(ctx.ksw_align2_batch(js, mat, 6, 1, 6, 1, 19, 1), want)
        mat = oracle.scmat(1, 4)
        for gaps in ((5, 2, 4, 3), (6, 1, 4, 1), (4, 1, 6, 1), (0, 1, 0, 1), (127, 1, 6, 1), (128, 1, 6, 1)):
            want, _ = oracle.align2_batch(js, mat, *gaps, 19, 1)
            assert np.array_equal(ctx.ksw_align2_batch(js, mat, *gaps, 19, 1), want), gaps
    finally:
        ctx.set_option(B.OPT_RESCUE_PAIR, 0)
        ctx.set_option(B.OPT_RESCUE_LANES, 16)
