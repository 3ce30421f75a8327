"""The serving loop: requests admitted against an HBM budget, run in waves
(continuous batching), results identical alone and in the mix."""
import threading
import time

import numpy as np
import pytest

import bwacuda as B
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[pytest.param(B.GATHER_AUTO, id="admit-auto"),
                        pytest.param(B.GATHER_HOST, id="admit-hostpack")])
def server(ctx, request):
    """A serving loop admitting by device gather (where the device reads host memory) or by host
    packing through a pinned mirror of the arena."""
    ctx.set_option(B.OPT_HOST_GATHER, request.param)
    ctx.server_start(hbm_budget_bytes=256 << 20, max_waves=3)
    yield ctx
    ctx.server_stop()
    ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)


def _mixed_requests(seed, count, lo=200, hi=6000):
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(count):
        n = int(rng.integers(lo, hi))
        kind = "rescue" if rng.random() < 0.25 else "extend"
        if kind == "extend":
            js = B.synth_ext(int(rng.choice([2, 3])), n, seed=seed * 1000 + k)
            js.w[:] = 100  # one band per request (the host form shares w per call)
        else:
            js = B.synth_rescue(n, seed=seed * 1000 + k)
        reqs.append((kind, js))
    return reqs


def _submit(ctx, kind, js):
    return ctx.submit_extend(js) if kind == "extend" else ctx.submit_rescue(js, minsc=20)


def test_results_equal_alone_and_in_the_mix(server):
    reqs = _mixed_requests(1, 24)
    # each request alone
    alone = []
    for kind, js in reqs:
        out, _ = server.wait(_submit(server, kind, js))
        alone.append(out)
    # all together: they are admitted and batched while earlier waves run
    ids = [_submit(server, kind, js) for kind, js in reqs]
    mixed = [server.wait(i)[0] for i in ids]
    for a, b in zip(alone, mixed):
        assert np.array_equal(a, b)
    # and equal to the oracle
    for (kind, js), a in zip(reqs[:6], alone[:6]):
        want = oracle.extend_batch(js)[0] if kind == "extend" else oracle.align2_batch(js, minsc=20)[0]
        assert np.array_equal(a, want)
    st = server.server_stats()
    assert st["waves"] < 2 * len(reqs)  # the mixed pass batched requests together


def test_admission_by_hbm_budget(ctx):
    # a budget that holds only a few requests at a time: the rest wait and still complete
    ctx.server_start(hbm_budget_bytes=64 << 20, max_waves=2)
    try:
        reqs = _mixed_requests(2, 16, 2000, 6000)
        ids = [_submit(ctx, kind, js) for kind, js in reqs]
        outs = [ctx.wait(i)[0] for i in ids]
        for (kind, js), o in zip(reqs, outs):
            want = oracle.extend_batch(js)[0] if kind == "extend" else oracle.align2_batch(js, minsc=20)[0]
            assert np.array_equal(o, want)
        # a request larger than the whole budget can never be admitted
        big = B.synth_ext(2, 400000, seed=9)
        with pytest.raises(B.BwaCudaError) as e:
            ctx.submit_extend(big)
        assert e.value.code == B.ENOMEM
    finally:
        ctx.server_stop()


def test_concurrent_clients_and_bad_request(server):
    # several host threads submit at once; one request carries an invalid base and
    # fails alone, without disturbing the others
    reqs = _mixed_requests(3, 12)
    bad = B.JobSet.from_lists([[0, 1, 9]], [[0, 1, 2]], [5])
    results, errors = {}, {}

    def client(k):
        kind, js = reqs[k]
        results[k] = server.wait(_submit(server, kind, js))[0]

    th = [threading.Thread(target=client, args=(k,)) for k in range(len(reqs))]
    for t in th:
        t.start()
    rid = server.submit_extend(bad)
    with pytest.raises(B.BwaCudaError) as e:
        server.wait(rid)
    assert e.value.code == B.EBASE
    for t in th:
        t.join()
    for k, (kind, js) in enumerate(reqs):
        want = oracle.extend_batch(js)[0] if kind == "extend" else oracle.align2_batch(js, minsc=20)[0]
        assert np.array_equal(results[k], want)


def test_poll_and_bounded_wait(server):
    js = B.synth_ext(2, 50000, seed=4)
    rid = server.submit_extend(js)
    deadline = time.time() + 60
    while True:
        try:
            out, lat = server.wait(rid, timeout_us=0)  # poll
            break
        except B.BwaCudaError as e:
            assert e.code == B.EAGAIN
            assert time.time() < deadline
            time.sleep(0.001)
    assert lat > 0
    assert np.array_equal(out, oracle.extend_batch(js)[0])


def _mixed_kind_requests(seed, count, lo=500, hi=8000):
    """Requests that each carry extension and rescue jobs (a chunk's extensions and its rescue
    windows together), with a rescue share between 0 and 1."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(rng.integers(lo, hi))
        nr = int(n * rng.random())
        ejs = B.synth_ext(int(rng.choice([2, 3])), max(n - nr, 1), seed=seed * 1000 + k)
        ejs.w[:] = 100
        rjs = B.synth_rescue(max(nr, 1), seed=seed * 1000 + 500 + k)
        out.append((ejs, rjs))
    return out


def test_mixed_kind_requests_alone_and_in_the_mix(server):
    reqs = _mixed_kind_requests(7, 16)
    alone = [server.wait(server.submit_mixed(e, r, minsc=20))[0] for e, r in reqs]
    ids = [server.submit_mixed(e, r, minsc=20) for e, r in reqs]
    mixed = [server.wait(i)[0] for i in ids]
    for (ae, ar), (me, mr) in zip(alone, mixed):
        assert np.array_equal(ae, me) and np.array_equal(ar, mr)
    for (e, r), (oe, orr) in zip(reqs[:6], alone[:6]):
        assert np.array_equal(oe, oracle.extend_batch(e)[0])
        assert np.array_equal(orr, oracle.align2_batch(r, minsc=20)[0])
    ext_cells, res_cells = server.server_cells()
    assert ext_cells > 0 and res_cells == 2 * sum(int((r.qlen.astype(np.int64) * r.tlen).sum()) for _, r in reqs)


def test_mixed_kind_requests_beside_one_kind_requests(server):
    # mixed-kind, extension-only and rescue-only requests in flight together
    mk = _mixed_kind_requests(8, 6)
    one = _mixed_requests(9, 6)
    ids = [("m", server.submit_mixed(e, r, minsc=20), (e, r)) for e, r in mk]
    ids += [("1", _submit(server, kind, js), (kind, js)) for kind, js in one]
    for tag, rid, what in ids:
        out = server.wait(rid)[0]
        if tag == "m":
            assert np.array_equal(out[0], oracle.extend_batch(what[0])[0])
            assert np.array_equal(out[1], oracle.align2_batch(what[1], minsc=20)[0])
        else:
            kind, js = what
            want = oracle.extend_batch(js)[0] if kind == "extend" else oracle.align2_batch(js, minsc=20)[0]
            assert np.array_equal(out, want)
