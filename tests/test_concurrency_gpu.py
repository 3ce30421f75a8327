"""Concurrent callers, as the reference's rayon workers call one shared backend: several host
threads on one context (the context serialises them) and on separate contexts (their
streams overlap on the device), every result bit-exact against the oracle."""
import threading

import numpy as np
import pytest

import bwacuda as B
import oracle

pytestmark = pytest.mark.gpu


def _work(k):
    js = B.synth_ext(2 if k % 2 else 3, 30000, seed=700 + k)
    rs = B.synth_rescue(2000, seed=800 + k)
    return js, rs


def _run(ctx, js, rs, results, k):
    try:
        ext = ctx.extend_batch(js)  # one band for the whole call (w = 100), as extend_batch takes it
        res = ctx.ksw_align2_batch(rs, minsc=20)
        results[k] = (ext, res)
    except Exception as e:  # reported by the main thread
        results[k] = e


def _check(works, results):
    for k, (js, rs) in enumerate(works):
        got = results[k]
        assert not isinstance(got, Exception), got
        want_e, _ = oracle.extend_batch(js)
        want_r, _ = oracle.align2_batch(rs, minsc=20)
        assert np.array_equal(got[0], want_e), f"thread {k}: extension differs"
        assert np.array_equal(got[1], want_r), f"thread {k}: rescue differs"


@pytest.mark.parametrize("path", [B.PATH_BATCHED, B.PATH_PLAIN])
def test_threads_share_one_context(ctx, path):
    ctx.set_option(B.OPT_EXT_PATH, path)
    works = [_work(k) for k in range(4)]
    for js, _ in works:
        js.w[:] = 100
    results = [None] * len(works)
    threads = [threading.Thread(target=_run, args=(ctx, js, rs, results, k)) for k, (js, rs) in enumerate(works)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    ctx.set_option(B.OPT_EXT_PATH, B.PATH_BATCHED)
    _check(works, results)


def test_threads_with_their_own_contexts(ctx):
    works = [_work(10 + k) for k in range(3)]
    for js, _ in works:
        js.w[:] = 100
    ctxs = [B.Context(0) for _ in works]
    results = [None] * len(works)
    try:
        threads = [threading.Thread(target=_run, args=(c, js, rs, results, k))
                   for k, (c, (js, rs)) in enumerate(zip(ctxs, works))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    finally:
        for c in ctxs:
            c.close()
    _check(works, results)
