"""The reference's 8-bit / 16-bit / scalar bin rule of batched_extend
(crates/bwa-neon/src/batched.rs:817-866: 8-bit iff q < 256, t < 256 and
h0 + min(q, t) * max_sc + max(b, |npen|, 0) + max_sc < 256; else 16-bit iff every
term is < 32768; else scalar; non-uniform matrices always scalar), as the
library labels each job in bwacuda_stats (ext_bin_u8 / _i16 / _i32), against
oracle.ext_bin: per job on a stream built around every threshold (one call per
job, so the counter that moves is the job's label), and as counts on the
mixed-length workload and the reference's u8 / i16 kernel sweep, through both
host-buffer routes (device gather and host packing)."""
import numpy as np
import pytest

import bwacuda as B
import oracle
import refstreams as R

pytestmark = pytest.mark.gpu

ROUTES = [pytest.param(B.GATHER_DEVICE, id="device-gather"), pytest.param(B.GATHER_HOST, id="host-packing")]


@pytest.fixture(params=ROUTES)
def gctx(ctx, request):
    ctx.set_option(B.OPT_HOST_GATHER, request.param)
    ctx.set_option(B.OPT_EXT_PATH, B.PATH_BATCHED)
    yield ctx
    ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)


def _bins(st):
    return (st["ext_bin_u8"], st["ext_bin_i16"], st["ext_bin_i32"])


def _boundary_jobs():
    """(qlen, tlen, h0) on both sides of each threshold at default scoring (head room 4 + 1)."""
    cases = []
    for h0 in (148, 149, 150, 151):            # q = t = 100: bound 100 + h0 + 5 vs 256
        cases.append((100, 100, h0))
    for ql, tl in ((255, 255), (255, 256), (256, 255), (256, 256), (120, 400), (400, 120)):
        cases.append((ql, tl, 1))
    for h0 in (32562, 32563, 32564):           # q = t = 200: bound 200 + h0 + 5 vs 32768
        cases.append((200, 200, h0))
    cases.append((5, 40000, 10))               # tlen >= 32768: scalar bin
    return cases


def test_per_job_labels_at_thresholds(ctx):
    rng = np.random.default_rng(3)
    mat = oracle.scmat(1, 4)
    for ql, tl, h0 in _boundary_jobs():
        t = rng.integers(0, 4, tl).astype(np.uint8)
        q = rng.integers(0, 4, ql).astype(np.uint8)
        k = min(ql, tl)
        q[:k] = t[:k]
        js = B.JobSet.from_lists([q], [t], h0=[h0])
        before = np.array(_bins(ctx.stats()))
        got = ctx.extend_batch(js, mat)
        after = np.array(_bins(ctx.stats()))
        label = int(np.nonzero(after - before)[0][0])
        assert (after - before).sum() == 1
        assert len(q) == ql and len(t) == tl
        assert label == oracle.ext_bin(ql, tl, h0, mat), (ql, tl, h0)
        assert np.array_equal(got, oracle.extend_batch(js, mat)[0])


def test_non_uniform_matrix_is_scalar_bin(ctx):
    mat = oracle.scmat(1, 4).copy()
    mat[6] = 2  # C:C scores 2, A:A 1
    js = B.synth_ext(1, 500, seed=4)
    ctx.reset_stats()
    ctx.extend_batch(js, mat)
    assert _bins(ctx.stats()) == (0, 0, len(js))
    assert all(oracle.ext_bin(int(js.qlen[k]), int(js.tlen[k]), int(js.h0[k]), mat) == 2 for k in range(len(js)))


def _oracle_counts(js, mat):
    lab = [oracle.ext_bin(int(js.qlen[k]), int(js.tlen[k]), int(js.h0[k]), mat) for k in range(len(js))]
    return tuple(int(x) for x in np.bincount(lab, minlength=3))


def test_counts_mixed_lengths(gctx):
    js = B.synth_ext(3, 60000, seed=11)
    mat = oracle.scmat(1, 4)
    gctx.reset_stats()
    gctx.extend_batch(js, mat)
    want = _oracle_counts(js, mat)
    assert _bins(gctx.stats()) == want
    assert want[0] > 0 and want[1] > 0


def test_counts_reference_kernel_sweep(gctx):
    mat = oracle.scmat(1, 4)
    tot_got = np.zeros(3, np.int64)
    tot_want = np.zeros(3, np.int64)
    for k, c in enumerate(R.simd_verify()):
        if k >= 60:
            break
        js = B.JobSet.from_lists(c["qs"], c["ts"], h0=c["h0s"])
        gctx.reset_stats()
        gctx.extend_batch(js, mat, c["o_del"], c["e_del"], c["o_ins"], c["e_ins"], c["w"], c["end_bonus"],
                          c["zdrop"])
        tot_got += np.array(_bins(gctx.stats()))
        tot_want += np.array(_oracle_counts(js, mat))
    assert np.array_equal(tot_got, tot_want)
    assert tot_want[0] > 0 and tot_want[1] > 0
