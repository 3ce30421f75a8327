"""The GPU rescue kernels against the independent Gotoh local SW (tests/gotoh.py) on the
reference's third-party cross-check stream (crates/bwa-extend/tests/third_party_oracle.rs:
246-361), with the reference's assertions: the score on every pair, (score, qb, qe, tb, te)
wherever the start recovery ran, (score, te, score2, te2) on lane-aligned queries.  Every
rescue kernel family is run: the register wavefront with 8, 16 and 32 lanes per job and the
thread-per-job kernel, through the scalar ksw_align2 (lanes 16) and batched_ksw_align2 entries."""
import numpy as np
import pytest

import bwacuda as B
import gotoh
import oracle
import refstreams as R

pytestmark = pytest.mark.gpu

KERNELS = [pytest.param((B.RESCUE_AUTO, 16, 0), id="wavefront16"), pytest.param((B.RESCUE_AUTO, 8, 0), id="wavefront8"),
           pytest.param((B.RESCUE_AUTO, 32, 0), id="wavefront32"), pytest.param((B.RESCUE_TPJ, 16, 0), id="tpj"),
           pytest.param((B.RESCUE_AUTO, 8, 4), id="paired4"), pytest.param((B.RESCUE_AUTO, 8, 8), id="paired8"),
           pytest.param((B.RESCUE_AUTO, 16, 16), id="paired16")]
SCORINGS = [(1, 4, 6, 1), (2, 3, 5, 2)]


@pytest.fixture(scope="module")
def stream():
    pairs = R.third_party_oracle_pairs()
    js = B.JobSet.from_lists([p[0] for p in pairs], [p[1] for p in pairs])
    want = {}
    for a, b, o, e in SCORINGS:
        mat = oracle.scmat(a, b)
        want[(a, b, o, e)] = [gotoh.align(q, t, mat, o, e, 19 * a, a) for q, t in pairs]
    return pairs, js, want


@pytest.fixture(params=KERNELS)
def rctx(ctx, request):
    kernel, lanes, pair = request.param
    ctx.set_option(B.OPT_RESCUE_KERNEL, kernel)
    ctx.set_option(B.OPT_RESCUE_LANES, lanes)
    ctx.set_option(B.OPT_RESCUE_PAIR, pair)
    yield ctx
    ctx.set_option(B.OPT_RESCUE_KERNEL, B.RESCUE_AUTO)
    ctx.set_option(B.OPT_RESCUE_LANES, 16)
    ctx.set_option(B.OPT_RESCUE_PAIR, 0)


def _check(pairs, got, want, score_only=False):
    spans = quads = 0
    for (q, _), r, g in zip(pairs, got, want):
        r = tuple(int(x) for x in r)
        assert r[0] == g[0]
        if score_only:
            continue
        if r[1] >= 0:
            assert r[:5] == g[:5]
            spans += 1
        if len(q) % 16 == 0:
            assert (r[4], r[5], r[6]) == (g[4], g[5], g[6])
            quads += 1
    return spans, quads


@pytest.mark.parametrize("a,b,o,e", SCORINGS)
def test_scalar_entry_matches_gotoh(rctx, stream, a, b, o, e):
    pairs, js, want = stream
    mat = oracle.scmat(a, b)
    got = rctx.ksw_align2_scalar_batch(js, mat, o, e, o, e, B.INT_MAX, a, 16)
    _check(pairs, got, want[(a, b, o, e)], score_only=True)
    got = rctx.ksw_align2_scalar_batch(js, mat, o, e, o, e, 19 * a, a, 16)
    spans, quads = _check(pairs, got, want[(a, b, o, e)])
    assert spans > 200 and quads > 0


@pytest.mark.parametrize("a,b,o,e", SCORINGS)
def test_batched_entry_matches_gotoh(rctx, stream, a, b, o, e):
    pairs, js, want = stream
    mat = oracle.scmat(a, b)
    got = rctx.ksw_align2_batch(js, mat, o, e, o, e, 19 * a, a)
    spans, quads = _check(pairs, got, want[(a, b, o, e)])
    assert spans > 200 and quads > 0
    assert np.array_equal(got, oracle.align2_batch(js, mat, o, e, o, e, 19 * a, a, mode=0)[0])
