"""ksw_global2 parity: the CUDA kernel through the C ABI against the oracle, bit-exact on the
score and on every CIGAR run, plus the reference's own known answers."""
import numpy as np
import pytest

import bwacuda as B
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[pytest.param(B.GATHER_DEVICE, id="devgather"), pytest.param(B.GATHER_HOST, id="hostpack")])
def gctx(ctx, request):
    """The context with the host-buffer route under test (device gather needs pageable access)."""
    ctx.set_option(B.OPT_HOST_GATHER, request.param)
    if request.param == B.GATHER_DEVICE:
        try:
            ctx.ksw_global2_batch(B.JobSet.from_lists([[0, 1]], [[0, 1]], w=[3]))
        except B.BwaCudaError as e:
            ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)
            assert e.code == B.EUNSUPPORTED
            pytest.skip("device cannot read pageable host memory")
    yield ctx
    ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)


def _cigars(offs, words):
    return [[int(x) for x in words[offs[k]:offs[k + 1]]] for k in range(len(offs) - 1)]


def _check(ctx, js, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1):
    mat = oracle.scmat() if mat is None else mat
    sc, offs, words = ctx.ksw_global2_batch(js, mat, o_del, e_del, o_ins, e_ins)
    wsc, woffs, wwords = oracle.global2_batch(js, mat, o_del, e_del, o_ins, e_ins)
    bad = np.nonzero(sc != wsc)[0]
    assert len(bad) == 0, f"{len(bad)} score mismatches, first job {bad[0]}: {sc[bad[0]]} vs {wsc[bad[0]]}"
    assert np.array_equal(offs, woffs)
    assert np.array_equal(words, wwords)
    return sc, offs, words


def test_known_answers(gctx):
    # crates/bwa-extend/src/sw.rs:1358-1380
    s = [0, 1, 2, 3, 0, 1, 2, 3, 0, 1]
    q = [0, 1, 2, 3, 0, 1, 2, 3]
    t = q[:4] + [2] + q[4:]
    js = B.JobSet.from_lists([s, q], [s, t], w=[100, 100])
    sc, offs, words = gctx.ksw_global2_batch(js)
    cig = _cigars(offs, words)
    assert sc[0] == len(s) and cig[0] == [len(s) << 4]
    assert sum(c >> 4 for c in cig[1] if c & 0xf == 2) == 1
    assert sum(c >> 4 for c in cig[1] if c & 0xf == 0) == len(q)


def test_cigar_stage_workload(gctx):
    js = B.synth_global(200000, seed=3)
    _check(gctx, js)


def test_random_lengths_bands_and_scoring(gctx):
    rng = np.random.default_rng(11)
    qs, ts, ws = [], [], []
    for k in range(3000):
        t = rng.integers(0, 5 if k % 5 == 0 else 4, int(rng.integers(0, 300))).tolist()
        q = list(t)
        for _ in range(int(rng.integers(0, 6))):
            if not q:
                break
            p = int(rng.integers(0, len(q)))
            r = rng.random()
            if r < 0.4:
                q[p] = int(rng.integers(0, 4))
            elif r < 0.7:
                del q[p:p + int(rng.integers(1, 4))]
            else:
                q[p:p] = rng.integers(0, 4, int(rng.integers(1, 4))).tolist()
        diff = abs(len(q) - len(t))
        ws.append(int(rng.choice([diff + 3, diff + 10, 100, 2 * max(len(q), len(t)) + 1])))
        qs.append(q)
        ts.append(t)
    js = B.JobSet.from_lists(qs, ts, w=ws)
    _check(gctx, js)
    # other scoring: larger match / gap values and a non-uniform matrix
    _check(gctx, js, oracle.scmat(2, 5), 5, 2, 4, 3)
    mat = rng.integers(-6, 4, 25).astype(np.int8)
    mat[0] = 3
    _check(gctx, js, mat, 7, 1, 5, 2)


def _pairs_with_edits(rng, lengths, ends=20):
    qs, ts = [], []
    for L in lengths:
        t = rng.integers(0, 4, int(L)).tolist()
        q = list(t)
        for _ in range(int(rng.integers(0, 8))):
            p = int(rng.integers(0, max(1, len(q))))
            r = rng.random()
            if r < 0.5 and q:
                q[p] = int(rng.integers(0, 4))
            elif r < 0.75:
                del q[p:p + int(rng.integers(1, 4))]
            else:
                q[p:p] = rng.integers(0, 4, int(rng.integers(1, 4))).tolist()
        ts.append(t + rng.integers(0, 4, int(rng.integers(0, ends))).tolist())
        qs.append(q)
    return qs, ts


def test_narrow_and_wide_cells(gctx):
    # Jobs whose (qlen + tlen) x (largest per-step cost) stays small run in 16-bit cells, the
    # rest in 32-bit cells; a batch mixes both (long reads in their own buckets, and one
    # length bucket holding both kinds through long targets), and large gap costs make every
    # job wide.  Sentinel values enter every band edge (H left of the band, E entering it), so
    # the traceback bytes compare sentinel-derived values in both cell forms.
    rng = np.random.default_rng(23)
    lengths = np.concatenate([rng.integers(40, 250, 300), rng.integers(560, 760, 60), rng.integers(260, 320, 60)])
    qs, ts = _pairs_with_edits(rng, lengths)
    for k in range(360, 390):  # same query-length bucket as the next 30, targets long enough to be wide
        ts[k] = ts[k] + rng.integers(0, 4, 1200).tolist()
    ws = [int(rng.choice([3, 12, 40, 150])) for _ in qs]
    js = B.JobSet.from_lists(qs, ts, w=ws)
    keep = np.array([k for k in range(len(qs)) if oracle.global2(qs[k], ts[k], ws[k]) is not None])
    js = js.take(keep)
    _check(gctx, js)
    _check(gctx, js, oracle.scmat(2, 5), 5, 2, 4, 3)
    _check(gctx, js, oracle.scmat(1, 4), 3000, 1, 2000, 1)


def test_edge_conventions(gctx):
    # empty query, empty target, both empty, narrow bands that cannot reach the corner
    qs = [[], [1, 2, 3], [], [0, 1, 2, 3] * 10, [0] * 30, [1, 2]]
    ts = [[1, 2, 3], [], [], [0, 1, 2, 3] * 12, [0] * 5, [1, 2, 3, 0, 0, 0, 0, 0]]
    ws = [5, 2, 3, 0, 1, 0]
    js = B.JobSet.from_lists(qs, ts, w=ws)
    want = [oracle.global2(q, t, w) for q, t, w in zip(qs, ts, ws)]
    keep = [k for k, r in enumerate(want) if r is not None]
    sub = js.take(np.array(keep))
    sc, offs, words = gctx.ksw_global2_batch(sub)
    cig = _cigars(offs, words)
    for i, k in enumerate(keep):
        assert (int(sc[i]), cig[i]) == want[k], k
    # where the reference's traceback index leaves the matrix, the call fails loudly
    for k in [k for k, r in enumerate(want) if r is None]:
        with pytest.raises(B.BwaCudaError) as e:
            gctx.ksw_global2_batch(js.take(np.array([k])))
        assert e.value.code == B.EUNSUPPORTED


def test_many_chunks(gctx):
    # small chunks (4 x 777 jobs on the device route, 262,144 on the host route) exercise the
    # per-chunk output offsets and the narrow / wide choice per chunk and bucket
    js = B.synth_global(20000, seed=6)
    gctx.set_option(B.OPT_CHUNK_JOBS, 777)
    try:
        _check(gctx, js)
    finally:
        gctx.set_option(B.OPT_CHUNK_JOBS, 1 << 20)


def test_short_buffer_reports_sizes(gctx):
    js = B.synth_global(5000, seed=4)
    wsc, woffs, wwords = oracle.global2_batch(js)
    import ctypes as C

    base = js.seq.ctypes.data
    jobs = np.zeros(len(js), dtype=B.GLOBAL_JOB)
    jobs["query"] = base + js.q_off.astype(np.uint64)
    jobs["target"] = base + js.t_off.astype(np.uint64)
    jobs["qlen"], jobs["tlen"], jobs["w"] = js.qlen, js.tlen, js.w
    mat = oracle.scmat()
    score = np.zeros(len(js), np.int32)
    offs = np.zeros(len(js) + 1, np.uint64)
    small = np.zeros(10, np.uint32)
    rc = B.lib().bwacuda_ksw_global2_batch(gctx.h, C.c_void_p(jobs.ctypes.data), len(js), 5,
                                           C.c_void_p(mat.ctypes.data), 6, 1, 6, 1,
                                           C.c_void_p(score.ctypes.data), C.c_void_p(offs.ctypes.data),
                                           C.c_void_p(small.ctypes.data), len(small))
    assert rc == B.ESHORT
    assert np.array_equal(score, wsc) and np.array_equal(offs.astype(np.int64), woffs)
    # sizes only: a NULL buffer
    rc = B.lib().bwacuda_ksw_global2_batch(gctx.h, C.c_void_p(jobs.ctypes.data), len(js), 5,
                                           C.c_void_p(mat.ctypes.data), 6, 1, 6, 1,
                                           C.c_void_p(score.ctypes.data), C.c_void_p(offs.ctypes.data), None, 0)
    assert rc == B.ESHORT and int(offs[-1]) == len(wwords)


def test_invalid_inputs(gctx):
    js = B.JobSet.from_lists([[0, 1, 7]], [[0, 1, 2]], w=[5])
    with pytest.raises(B.BwaCudaError) as e:
        gctx.ksw_global2_batch(js)
    assert e.value.code == B.EBASE
    js = B.JobSet.from_lists([[0, 1]], [[0, 1, 2]], w=[5])
    js.qlen[0] = -1
    with pytest.raises(B.BwaCudaError) as e:
        gctx.ksw_global2_batch(js)
    assert e.value.code == B.EINVAL
    # the context stays usable
    js = B.synth_global(100, seed=5)
    _check(gctx, js)
