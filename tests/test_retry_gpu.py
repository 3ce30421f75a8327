"""The band-doubling retry of bwa-mem's run_side (crates/bwa-mem/src/across.rs:1357-1500) on the
GPU, against the same loop written over the oracle: results and accepted bands bit-exact."""
import numpy as np
import pytest

import bwacuda as B
import oracle

pytestmark = pytest.mark.gpu


def _oracle_retry(js, prev, max_tries, w_of_job, **kw):
    """run_side's loop: round r runs the active jobs at w << r; accept on score == prev, on
    max_off < (w >> 1) + (w >> 2), or in the last round."""
    n = len(js)
    out = np.zeros(n, dtype=oracle.EXT_DTYPE)
    w_used = np.zeros(n, dtype=np.int32)
    prev = np.array(prev if prev is not None else [-1] * n, dtype=np.int64)
    active = np.arange(n)
    for r in range(max_tries):
        if len(active) == 0:
            break
        sub = js.take(active)
        sub.w = np.ascontiguousarray(np.asarray(w_of_job)[active].astype(np.int64) << r).astype(np.int32)
        res, _ = oracle.extend_batch(sub, **kw)
        keep = []
        for i, k in enumerate(active):
            w = int(sub.w[i])
            accept = (int(res[i]["score"]) == prev[k] or int(res[i]["max_off"]) < (w >> 1) + (w >> 2)
                      or r + 1 == max_tries)
            out[k] = res[i]
            w_used[k] = w
            if not accept:
                prev[k] = int(res[i]["score"])
                keep.append(k)
        active = np.array(keep, dtype=np.int64)
    return out, w_used


def _prev_left_right(js):
    # bwa-mem: -1 before a left extension's first round, h0 before a right one's
    return np.where(np.arange(len(js)) % 2 == 0, -1, js.h0).astype(np.int32)


@pytest.mark.parametrize("route", [B.GATHER_HOST, B.GATHER_AUTO])
@pytest.mark.parametrize("w0,max_tries", [(100, 2), (8, 2), (3, 4), (0, 2)])
def test_host_retry_matches_run_side(ctx, route, w0, max_tries):
    js = B.synth_ext(1, 20000, seed=50 + w0)  # 1% substitutions, 0.1% 1-3 bp indels
    prev = _prev_left_right(js)
    want, want_w = _oracle_retry(js, prev, max_tries, np.full(len(js), w0))
    ctx.set_option(B.OPT_HOST_GATHER, route)
    ctx.reset_stats()
    try:
        got, got_w = ctx.extend_batch_retry(js, prev, max_tries, w=w0)
    finally:
        ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)
    assert np.array_equal(got, want)
    assert np.array_equal(got_w, want_w)
    if w0 <= 3:
        assert ctx.stats()["ext_retry_jobs"] > 0  # narrow bands do send jobs round again


@pytest.mark.parametrize("piece", [1 << 30, 7001])
def test_device_retry_per_job_bands(ctx, piece):
    import torch

    js = B.synth_ext(3, 30000, seed=61)
    js.w = (js.w // 10).astype(np.int32)  # narrow per-job bands (5, 10, 20): many retries
    prev = _prev_left_right(js)
    want, want_w = _oracle_retry(js, prev, 3, js.w)
    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_ext_jobs().view(np.uint8)).cuda()
    d_out = torch.zeros(len(js) * 24, dtype=torch.uint8, device="cuda")
    d_w = torch.zeros(len(js), dtype=torch.int32, device="cuda")
    d_prev = torch.from_numpy(prev).cuda()
    ctx.set_option(B.OPT_DEVICE_PIECE, piece)  # 7001: four whole pieces and a ragged one
    try:
        ctx.extend_retry_device(d_seq.data_ptr(), d_jobs.data_ptr(), len(js), d_out.data_ptr(), d_w.data_ptr(),
                                d_prev.data_ptr(), max_tries=3)
        ctx.sync()
    finally:
        ctx.set_option(B.OPT_DEVICE_PIECE, 1 << 30)
    assert np.array_equal(d_out.cpu().numpy().view(B.EXT_RES), want)
    assert np.array_equal(d_w.cpu().numpy(), want_w)


def test_retry_edge_cases(ctx):
    # empty batch, invalid max_tries, a single job, qlen = 0 jobs
    empty = B.JobSet.from_lists([], [])
    assert len(ctx.extend_batch_retry(empty)[0]) == 0
    js = B.JobSet.from_lists([[0, 1, 2, 3] * 5, [], [1, 2]], [[0, 1, 2, 3] * 8, [1, 2, 3], []], [10, 5, 7])
    with pytest.raises(B.BwaCudaError) as e:
        ctx.extend_batch_retry(js, max_tries=0)
    assert e.value.code == B.EINVAL
    want, want_w = _oracle_retry(js, None, 2, np.full(len(js), 2))
    got, got_w = ctx.extend_batch_retry(js, None, 2, w=2)
    assert np.array_equal(got, want) and np.array_equal(got_w, want_w)
