"""Seed-extension parity: the CUDA kernels through the C ABI against the oracle.

Bit-exact on every field of every job (score, qle, tle, gtle, gscore, max_off).
Inputs are the reference's own test streams (replayed bit for bit), the
benchmark workloads at sizes the oracle finishes in seconds, and edge cases.
"""
import numpy as np
import pytest

import bwacuda as B
import oracle
import refstreams as R

pytestmark = pytest.mark.gpu

FIELDS = ("score", "qle", "tle", "gtle", "gscore", "max_off")


def _tuples(res):
    return [tuple(int(r[f]) for f in FIELDS) for r in res]


_GATHER_OK = {}


def _device_gather_supported(ctx):
    """Whether this device reads pageable host memory (the device-gather route)."""
    if id(ctx) not in _GATHER_OK:
        ctx.set_option(B.OPT_EXT_PATH, B.PATH_BATCHED)
        ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_DEVICE)
        try:
            ctx.extend_batch(B.JobSet.from_lists([[0, 1, 2]], [[0, 1, 2]], [5]))
            _GATHER_OK[id(ctx)] = True
        except B.BwaCudaError as e:
            assert e.code == B.EUNSUPPORTED
            _GATHER_OK[id(ctx)] = False
        finally:
            ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)
    return _GATHER_OK[id(ctx)]


def _set_path(ctx, path):
    """path: PATH_PLAIN / PATH_BATCHED (host-buffer route AUTO) or a (path, gather) pair."""
    path, gather = path if isinstance(path, tuple) else (path, B.GATHER_AUTO)
    if gather == B.GATHER_DEVICE and not _device_gather_supported(ctx):
        pytest.skip("device cannot read pageable host memory")
    ctx.set_option(B.OPT_EXT_PATH, path)
    ctx.set_option(B.OPT_HOST_GATHER, gather)


def _check_batch(ctx, qs, ts, h0s, a=1, b=4, o_del=6, e_del=1, o_ins=6, e_ins=1, w=100, end_bonus=5,
                 zdrop=100, path=B.PATH_PLAIN, what=""):
    mat = oracle.scmat(a, b)
    js = B.JobSet.from_lists(qs, ts, h0s, w)
    _set_path(ctx, path)
    got = _tuples(ctx.extend_batch(js, mat, o_del, e_del, o_ins, e_ins, w, end_bonus, zdrop))
    want = [oracle.extend2(q, t, h, mat, o_del, e_del, o_ins, e_ins, w, end_bonus, zdrop)
            for q, t, h in zip(qs, ts, h0s)]
    for k, (g, x) in enumerate(zip(got, want)):
        assert g == x, f"{what} job {k}: qlen={len(qs[k])} tlen={len(ts[k])} h0={h0s[k]} got {g} want {x}"


def test_known_answers(ctx):
    s = [0, 1, 2, 3] * 4
    assert ctx.extend(s, s, 1, oracle.scmat(1, 4), 6, 1, 6, 1, 100, 0, 100) == (17, 16, 16, 16, 17, 0)
    q = [0] * 10 + [1] * 40
    t = [0] * 10 + [2] * 40
    r = ctx.extend(q, t, 1, oracle.scmat(1, 4), 6, 1, 6, 1, 100, 0, 100)
    assert r[0] == 11 and r[2] == 10


@pytest.mark.parametrize("path", [pytest.param(B.PATH_PLAIN, id="plain"),
                                  pytest.param((B.PATH_BATCHED, B.GATHER_HOST), id="batched")])
def test_gate_stream_scoring_swept(ctx, path):
    # crates/bwa-extend/src/lib.rs:283-354: 2000 cases, scoring swept; batched per scoring.
    groups = {}
    for c in R.backend_matches_scalar():
        key = (c["a"], c["b"], c["o_del"], c["e_del"], c["o_ins"], c["e_ins"], c["w"], c["end_bonus"], c["zdrop"])
        groups.setdefault(key, []).append(c)
    for key, cs in groups.items():
        a, b, od, ed, oi, ei, w, eb, zd = key
        _check_batch(ctx, [c["q"] for c in cs], [c["t"] for c in cs], [c["h0"] for c in cs], a, b, od, ed, oi,
                     ei, w, eb, zd, path=path, what=f"gate {key}")


@pytest.mark.parametrize("path", [pytest.param(B.PATH_PLAIN, id="plain"),
                                  pytest.param((B.PATH_BATCHED, B.GATHER_HOST), id="batched")])
@pytest.mark.parametrize("stream", ["batch", "read_sized", "ungapped", "simd_verify"])
def test_reference_batch_streams(ctx, stream, path):
    gen = {"batch": R.backend_batch_matches_scalar, "read_sized": R.read_sized, "ungapped": R.ungapped,
           "simd_verify": R.simd_verify}[stream]
    for k, c in enumerate(gen()):
        _check_batch(ctx, c["qs"], c["ts"], c["h0s"], c["a"], c["b"], c["o_del"], c["e_del"], c["o_ins"],
                     c["e_ins"], c["w"], c["end_bonus"], c["zdrop"], path=path, what=f"{stream} round {k}")


def _check_jobset(ctx, js, w=100, path=B.PATH_PLAIN, **kw):
    _set_path(ctx, path)
    # per-job band: group by w (the host ABI shares w per call, as the reference does)
    want, _ = oracle.extend_batch(js, **kw)
    for wv in np.unique(js.w):
        idx = np.nonzero(js.w == wv)[0]
        sub = js.take(idx) if len(idx) != len(js) else js
        got = ctx.extend_batch(sub, w=int(wv), **kw)
        bad = np.nonzero(got != want[idx])[0]
        assert len(bad) == 0, f"{len(bad)} mismatches, first job {idx[bad[0]]}: {got[bad[0]]} vs {want[idx[bad[0]]]}"


# host-buffer routes: plain kernels; batched kernels fed by host packing or by the device's own gather
PATHS = [pytest.param(B.PATH_PLAIN, id="plain"),
         pytest.param((B.PATH_BATCHED, B.GATHER_HOST), id="batched-hostpack"),
         pytest.param((B.PATH_BATCHED, B.GATHER_DEVICE), id="batched-devgather")]


@pytest.mark.parametrize("path", PATHS)
def test_workload_20k_jobs(ctx, path):
    js = B.synth_ext(1, 20000, seed=0)
    _check_jobset(ctx, js, path=path)


@pytest.mark.parametrize("path", PATHS)
def test_workload_read_pairs(ctx, path):
    js = B.synth_ext(2, 200000, seed=1)
    _check_jobset(ctx, js, path=path)


@pytest.mark.parametrize("path", PATHS)
def test_workload_mixed_lengths_and_bands(ctx, path):
    js = B.synth_ext(3, 60000, seed=2)
    _check_jobset(ctx, js, path=path)


@pytest.mark.parametrize("path", PATHS)
def test_batch_streams_through_both_paths(ctx, path):
    # the reference's lane-cross-talk stream, every batch through the chosen path
    for k, c in enumerate(R.backend_batch_matches_scalar()):
        if k >= 60:
            break
        _check_batch(ctx, c["qs"], c["ts"], c["h0s"], c["a"], c["b"], c["o_del"], c["e_del"], c["o_ins"],
                     c["e_ins"], c["w"], c["end_bonus"], c["zdrop"], path=path, what=f"batch round {k}")


def test_chunked_pipeline_boundaries(ctx):
    # chunks smaller than the batch exercise both staging slots and the tail chunk
    js = B.synth_ext(3, 5000, seed=12)
    want, _ = oracle.extend_batch(js)
    routes = [B.PATH_PLAIN, (B.PATH_BATCHED, B.GATHER_HOST)]
    if _device_gather_supported(ctx):
        routes.append((B.PATH_BATCHED, B.GATHER_DEVICE))
    try:
        for path in routes:
            _set_path(ctx, path)
            ctx.set_option(B.OPT_CHUNK_JOBS, 777)
            for wv in np.unique(js.w):
                idx = np.nonzero(js.w == wv)[0]
                got = ctx.extend_batch(js.take(idx), w=int(wv))
                assert np.array_equal(got, want[idx])
    finally:
        ctx.set_option(B.OPT_CHUNK_JOBS, 1 << 20)
        ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)


def _device_run(ctx, js, path, reps=1):
    import torch

    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_ext_jobs().view(np.uint8)).cuda()
    d_out = torch.zeros(len(js) * 24, dtype=torch.uint8, device="cuda")
    outs = []
    for _ in range(reps):
        d_out.zero_()
        ctx.extend_device(d_seq.data_ptr(), d_jobs.data_ptr(), len(js), d_out.data_ptr(), path=path)
        ctx.sync()
        outs.append(d_out.cpu().numpy().view(B.EXT_RES).copy())
    return outs


DEVICE_PATHS = [pytest.param(B.PATH_PLAIN, id="plain"), pytest.param(B.PATH_BATCHED, id="batched")]


@pytest.mark.parametrize("path", DEVICE_PATHS)
def test_device_entry_equals_oracle(ctx, path):
    js = B.synth_ext(3, 50000, seed=3)
    want, _ = oracle.extend_batch(js)
    for got in _device_run(ctx, js, path, reps=3):  # batched: capture, then two graph replays
        assert np.array_equal(got, want)


@pytest.mark.parametrize("path", DEVICE_PATHS)
def test_device_batch_in_pieces(ctx, path):
    # a device-resident batch larger than the piece size runs as consecutive launch sequences
    # (each piece sorted and bucketed on its own, a ragged last piece), with the same results
    js = B.synth_ext(3, 20000, seed=15)
    want, _ = oracle.extend_batch(js)
    ctx.set_option(B.OPT_DEVICE_PIECE, 6007)
    try:
        outs = _device_run(ctx, js, path, reps=2)
    finally:
        ctx.set_option(B.OPT_DEVICE_PIECE, 1 << 30)
    for got in outs:
        assert np.array_equal(got, want)
    for bad in (0, -1, (1 << 30) + 1):
        with pytest.raises(B.BwaCudaError):
            ctx.set_option(B.OPT_DEVICE_PIECE, bad)


@pytest.mark.parametrize("block", [32, 64, 128, 256])
def test_persistent_block_sizes(ctx, block):
    js = B.synth_ext(2, 20000, seed=13)
    want, _ = oracle.extend_batch(js)
    ctx.set_option(B.OPT_PERSIST_BLOCK, block)
    try:
        got = _device_run(ctx, js, B.PATH_BATCHED)[0]
    finally:
        ctx.set_option(B.OPT_PERSIST_BLOCK, 128)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("step,grab", [(16, 1), (16, 4), (32, 2), (64, 1), (64, 4)])
def test_bucket_width_and_grab(ctx, step, grab):
    # the launch-shape knobs the autotuner turns: results never change
    js = B.synth_ext(3, 30000, seed=14)
    want, _ = oracle.extend_batch(js)
    ctx.set_option(B.OPT_BUCKET_STEP, step)
    ctx.set_option(B.OPT_GRAB, grab)
    try:
        outs = _device_run(ctx, js, B.PATH_BATCHED, reps=2)  # capture and replay under the new shape
    finally:
        ctx.set_option(B.OPT_BUCKET_STEP, 32)
        ctx.set_option(B.OPT_GRAB, 1)
    for got in outs:
        assert np.array_equal(got, want)


def test_autotune_extend_keeps_results(ctx):
    import torch

    js = B.synth_ext(3, 60000, seed=15)
    want, _ = oracle.extend_batch(js)
    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_ext_jobs().view(np.uint8)).cuda()
    try:
        t = ctx.autotune_extend(d_seq.data_ptr(), d_jobs.data_ptr(), len(js), sample=20000)
        # 36 launch shapes, then 9 group-per-job settings (3 query lengths x 3 lane counts)
        assert t["candidates"] == 45 and t["ext_gcups"] > 0
        assert t["persist_block"] in (32, 64, 128, 256) and t["grab"] in (1, 2, 4)
        assert t["bucket_step"] in (16, 32, 64)
        assert t["long_qlen"] in (0, 129, 193, 225) and t["long_lanes"] in (8, 16, 32)
        assert ctx.tuning() == t
        got = _device_run(ctx, js, B.PATH_BATCHED)[0]
        assert np.array_equal(got, want)
        # host-buffer calls run under the tuned shape too
        _check_jobset(ctx, js.take(np.arange(5000)), path=(B.PATH_BATCHED, B.GATHER_AUTO))
    finally:
        ctx.set_option(B.OPT_PERSIST_BLOCK, 128)
        ctx.set_option(B.OPT_BUCKET_STEP, 32)
        ctx.set_option(B.OPT_GRAB, 1)
        ctx.set_option(B.OPT_LONG_QLEN, 0)
        ctx.set_option(B.OPT_LONG_LANES, 16)


@pytest.mark.parametrize("path", PATHS)
def test_edge_cases(ctx, path):
    mat = oracle.scmat(1, 4)
    qs = [[], [0, 1, 2], [], [1] * 5, [0, 4, 4, 1], [2] * 300, [3] * 7, [0, 1] * 600]
    ts = [[1, 2, 3], [], [], [1] * 5, [4, 0, 1, 1], [2] * 300, [3] * 7, [0, 1] * 700]
    h0s = [10, 5, 3, 1, 20, 40, 250, 30]
    for w in (0, 1, 2, 100):
        for zd in (0, 1, 100):
            _check_batch(ctx, qs, ts, h0s, w=w, zdrop=zd, path=path, what=f"edge w={w} zdrop={zd}")
    # a single job, and empty batches
    assert ctx.extend([], [1, 2, 3], 10) == (10, 0, 0, 1, 3, 0)
    empty = B.JobSet.from_lists([], [])
    assert len(ctx.extend_batch(empty)) == 0


def _mutated_pairs(rng, n, qmax, h0_choices):
    """Query/target pairs that share most bases (long, high-scoring alignments with
    indels), lengths 0..qmax, h0 drawn from h0_choices ranges."""
    qs, ts, h0s = [], [], []
    for _ in range(n):
        ql = int(rng.integers(0, qmax + 1)) if rng.random() < 0.5 else int(rng.integers(0, 150))
        q = rng.integers(0, 4, ql)
        t = q.copy()
        for _ in range(int(rng.integers(0, 6))):  # point edits, N bases, short indels
            if len(t) == 0:
                break
            p = int(rng.integers(0, len(t)))
            op = int(rng.integers(0, 4))
            if op == 0:
                t[p] = (t[p] + 1) % 4
            elif op == 1:
                t[p] = 4
            elif op == 2:
                t = np.delete(t, slice(p, p + int(rng.integers(1, 4))))
            else:
                t = np.insert(t, p, rng.integers(0, 4, int(rng.integers(1, 4))))
        tail = rng.integers(0, 4, int(rng.integers(0, 40)))
        t = np.concatenate([t, tail]) if rng.random() < 0.7 else t
        lo, hi = h0_choices[int(rng.integers(0, len(h0_choices)))]
        qs.append(q.tolist())
        ts.append(t.tolist())
        h0s.append(int(rng.integers(lo, hi)))
    return qs, ts, h0s


@pytest.mark.parametrize("scoring", [(1, 4, 6, 1, 6, 1, 5, 100), (2, 3, 5, 2, 4, 3, 0, 40), (1, 1, 0, 1, 0, 1, 9, 0),
                                     (3, 5, 11, 1, 7, 2, 1, 200), (1, 4, 6, 1, 6, 1, 5, 1),
                                     (1, 4, 16383, 1, 16000, 384, 5, 100), (2, 4, 30000, 3000, 17000, 5, 5, 100)])
def test_pair_cell_classes_swept(ctx, scoring):
    # jobs of the 8-bit and 16-bit classes (two columns per lane operation) with odd and
    # even band edges, swept scoring and bands, through the batched route; the last two
    # scorings sit at and beyond the largest gap costs the 16-bit lanes take
    a, b, od, ed, oi, ei, eb, zd = scoring
    rng = np.random.default_rng(sum(scoring))
    qs, ts, h0s = _mutated_pairs(rng, 1500, 700, [(1, 60), (100, 250), (300, 3000), (8000, 20000)])
    for w in (1, 4, 33, 100):
        _check_batch(ctx, qs, ts, h0s, a, b, od, ed, oi, ei, w, eb, zd, path=(B.PATH_BATCHED, B.GATHER_HOST),
                     what=f"classes {scoring} w={w}")


@pytest.mark.parametrize("scoring", [(1, 4, 6, 1, 6, 1, 5, 100), (2, 3, 5, 2, 4, 3, 0, 40)])
def test_long_queries_short_targets(ctx, scoring):
    # queries past 512 columns against short targets stay in the 8-bit class (the value bound
    # follows min(qlen, tlen)): the open-ended 8-bit bucket, whose rows keep 32-bit maxima;
    # longer targets put the same queries in the 16-bit class
    a, b, od, ed, oi, ei, eb, zd = scoring
    rng = np.random.default_rng(31 + a)
    qs, ts, h0s = [], [], []
    for k in range(600):
        ql = int(rng.integers(513, 1400))
        q = rng.integers(0, 4, ql)
        tl = int(rng.integers(1, 120)) if k % 3 else int(rng.integers(200, 400))
        start = int(rng.integers(0, 8))
        t = q[start:start + tl].copy()
        for _ in range(int(rng.integers(0, 4))):
            if len(t):
                t[int(rng.integers(0, len(t)))] = int(rng.integers(0, 5))
        qs.append(q.tolist())
        ts.append(t.tolist())
        h0s.append(int(rng.integers(1, 40)))
    for w in (5, 100):
        _check_batch(ctx, qs, ts, h0s, a, b, od, ed, oi, ei, w, eb, zd, path=(B.PATH_BATCHED, B.GATHER_HOST),
                     what=f"long queries {scoring} w={w}")


@pytest.mark.parametrize("path", PATHS)
def test_wide_cells_for_large_scores(ctx, path):
    # h0 + min(q,t)*a >= 32768 needs int32 cells (the reference's scalar bin)
    rng = np.random.default_rng(5)
    qs, ts, h0s = [], [], []
    for k in range(40):
        q = rng.integers(0, 4, 60 + k).tolist()
        t = list(q) + rng.integers(0, 4, 30).tolist()
        qs.append(q)
        ts.append(t)
        h0s.append(32760 + k if k % 2 else 100 + k)
    _check_batch(ctx, qs, ts, h0s, path=path, what="wide")


def test_non_uniform_matrix_is_exact(ctx):
    rng = np.random.default_rng(7)
    mat = rng.integers(-5, 4, 25).astype(np.int8)
    mat[0] = 3
    qs = [rng.integers(0, 5, rng.integers(1, 80)).tolist() for _ in range(300)]
    ts = [list(q[: len(q) // 2]) + rng.integers(0, 5, 40).tolist() for q in qs]
    h0s = rng.integers(1, 60, 300).tolist()
    js = B.JobSet.from_lists(qs, ts, h0s)
    got = _tuples(ctx.extend_batch(js, mat, 5, 2, 4, 1, 30, 3, 40))
    want = [oracle.extend2(q, t, h, mat, 5, 2, 4, 1, 30, 3, 40) for q, t, h in zip(qs, ts, h0s)]
    assert got == want


def _raw_extend(ctx, jobs, out, m=5, mat=None):
    mat = np.ascontiguousarray(oracle.scmat() if mat is None else mat, dtype=np.int8)
    return B.lib().bwacuda_extend_batch(ctx.h, jobs.ctypes.data, len(jobs), m, mat.ctypes.data, 6, 1, 6, 1, 100, 5,
                                        100, out.ctypes.data)


@pytest.mark.parametrize("path", PATHS)
def test_invalid_inputs_fail_loudly(ctx, path):
    _set_path(ctx, path)
    try:
        js = B.JobSet.from_lists([[0, 1, 5]], [[0, 1, 2]], [10])
        with pytest.raises(B.BwaCudaError) as e:
            ctx.extend_batch(js)
        assert e.value.code == B.EBASE
        js = B.JobSet.from_lists([[0, 1]], [[0, 1, 2]], [0])
        with pytest.raises(B.BwaCudaError) as e:
            ctx.extend_batch(js)
        assert e.value.code == B.EINVAL
        js = B.JobSet.from_lists([[0, 1]], [[0, 1, 2]], [3])
        with pytest.raises(B.BwaCudaError) as e:
            ctx.extend_batch(js, e_del=0)
        assert e.value.code == B.EINVAL
        # null sequence pointers with non-zero lengths, and negative lengths, among valid jobs:
        # rejected before anything reads them
        js = B.synth_ext(2, 3000, seed=21)
        out = np.zeros(len(js), dtype=B.EXT_RES)
        for field, val in (("query", 0), ("target", 0), ("qlen", -1), ("tlen", -5)):
            jobs = ctx._host_jobs(js, B.EXT_JOB)
            jobs[1234][field] = val
            assert _raw_extend(ctx, jobs, out) == B.EINVAL, field
        # null pointers are fine where the length is zero
        jobs = ctx._host_jobs(js, B.EXT_JOB)
        jobs[7]["qlen"], jobs[7]["query"] = 0, 0
        jobs[8]["tlen"], jobs[8]["target"] = 0, 0
        assert _raw_extend(ctx, jobs, out) == B.OK
        t7 = js.seq[js.t_off[7]:js.t_off[7] + js.tlen[7]]
        q8 = js.seq[js.q_off[8]:js.q_off[8] + js.qlen[8]]
        assert _tuples(out[7:9]) == [oracle.extend2([], t7, int(js.h0[7])), oracle.extend2(q8, [], int(js.h0[8]))]
        # the context stays usable after an error
        assert ctx.extend([0, 1, 2], [0, 1, 2], 5) == oracle.extend2([0, 1, 2], [0, 1, 2], 5)
        want, _ = oracle.extend_batch(js)
        assert np.array_equal(ctx.extend_batch(js), want)
    finally:
        ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)


@pytest.mark.parametrize("path", PATHS)
def test_invalid_job_in_a_later_chunk(ctx, path):
    # many small chunks (the device gather's ring wraps several times); an invalid job or a bad
    # base code late in the batch fails the call, and the context then runs the batch cleanly
    _set_path(ctx, path)
    js = B.synth_ext(2, 9000, seed=22)
    want, _ = oracle.extend_batch(js)
    out = np.zeros(len(js), dtype=B.EXT_RES)
    ctx.set_option(B.OPT_CHUNK_JOBS, 700)
    try:
        jobs = ctx._host_jobs(js, B.EXT_JOB)
        jobs[8000]["qlen"] = -3
        assert _raw_extend(ctx, jobs, out) == B.EINVAL
        import copy

        bad = copy.copy(js)  # same offsets, its own copy of the bases
        bad.seq = js.seq.copy()
        seq = bad.seq
        k = 7777
        if js.qlen[k] == 0:
            k += 1
        seq[js.q_off[k]] = 6  # a base code >= m
        with pytest.raises(B.BwaCudaError) as e:
            ctx.extend_batch(bad)
        assert e.value.code == B.EBASE
        got = ctx.extend_batch(js)
        assert np.array_equal(got, want)
    finally:
        ctx.set_option(B.OPT_CHUNK_JOBS, 1 << 20)
        ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)


def test_device_gather_equals_host_packing(ctx):
    # the two feeds of the batched kernels agree on results, cell counts and bin statistics,
    # and the device gather writes every result word of the caller's array
    if not _device_gather_supported(ctx):
        pytest.skip("device cannot read pageable host memory")
    js = B.synth_ext(3, 40000, seed=22)
    runs = {}
    try:
        for gather in (B.GATHER_HOST, B.GATHER_DEVICE):
            _set_path(ctx, (B.PATH_BATCHED, gather))
            for chunk in (262144, 4099):
                ctx.set_option(B.OPT_CHUNK_JOBS, chunk)
                sub = js.take(np.nonzero(js.w == 100)[0])
                jobs = ctx._host_jobs(sub, B.EXT_JOB)
                out = np.full(len(sub), -7, dtype=B.EXT_RES)
                ctx.reset_stats()
                assert _raw_extend(ctx, jobs, out) == B.OK
                st = ctx.stats()
                runs[(gather, chunk)] = (out, {k: st[k] for k in ("ext_jobs", "ext_cells", "ext_bin_u8",
                                                                  "ext_bin_i16", "ext_bin_i32")})
    finally:
        ctx.set_option(B.OPT_CHUNK_JOBS, 1 << 20)
        ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)
    want, _ = oracle.extend_batch(sub)
    for key, (out, st) in runs.items():
        assert np.array_equal(out, want), key
        assert st == runs[(B.GATHER_HOST, 262144)][1], key
    assert runs[(B.GATHER_HOST, 262144)][1]["ext_bin_u8"] > 0


def test_cell_counter_matches_oracle(ctx):
    js = B.synth_ext(2, 30000, seed=9)
    ctx.reset_stats()
    ctx.extend_batch(js)
    _, cells = oracle.extend_batch(js)
    st = ctx.stats()
    assert st["ext_cells"] == cells
    assert st["ext_jobs"] == len(js)
    assert st["ext_bin_u8"] + st["ext_bin_i16"] + st["ext_bin_i32"] == len(js)


@pytest.fixture
def ugctx(ctx):
    """The context with the ungapped-diagonal fast path on (batched path)."""
    ctx.set_option(B.OPT_UNGAPPED, 1)
    yield ctx
    ctx.set_option(B.OPT_UNGAPPED, 0)


def test_ungapped_prefilter_on_reference_streams(ugctx):
    # the reference's own ungapped stream (random z-drop, N bases, 1..3 mismatches) and the
    # swept-scoring gate stream: the closed form must agree with the DP wherever it fires
    for k, c in enumerate(R.ungapped()):
        _check_batch(ugctx, c["qs"], c["ts"], c["h0s"], c["a"], c["b"], c["o_del"], c["e_del"], c["o_ins"],
                     c["e_ins"], c["w"], c["end_bonus"], c["zdrop"], path=(B.PATH_BATCHED, B.GATHER_AUTO),
                     what=f"ungapped round {k}")
    groups = {}
    for c in R.backend_matches_scalar():
        key = (c["a"], c["b"], c["o_del"], c["e_del"], c["o_ins"], c["e_ins"], c["w"], c["end_bonus"], c["zdrop"])
        groups.setdefault(key, []).append(c)
    for key, cs in groups.items():
        a, b, od, ed, oi, ei, w, eb, zd = key
        _check_batch(ugctx, [c["q"] for c in cs], [c["t"] for c in cs], [c["h0"] for c in cs], a, b, od, ed, oi,
                     ei, w, eb, zd, path=(B.PATH_BATCHED, B.GATHER_AUTO), what=f"gate {key}")


def test_ungapped_prefilter_edges(ugctx):
    # the fast path at its edges: queries of 1-300 bases, exact diagonals past 128 columns
    # (settled), mismatches before and after column 127 (only the former can settle), N in
    # either sequence, targets shorter than the query, h0 of 1 or 2 (runs that die on the first
    # mismatch), and batch sizes that end inside a warp
    rng = np.random.default_rng(77)
    qs, ts, h0s = [], [], []
    for k in range(2500):
        ql = int(rng.integers(1, 301))
        t = rng.integers(0, 4, ql + int(rng.integers(0, 40))).astype(np.uint8)
        q = t[:ql].copy()
        kind = k % 7
        if kind in (1, 2):  # 1-3 mismatches anywhere
            for c in rng.integers(0, ql, int(rng.integers(1, 4))):
                q[c] = (q[c] + 1) % 4
        elif kind == 3 and ql > 130:  # one mismatch past column 127
            c = int(rng.integers(128, ql))
            q[c] = (q[c] + 1) % 4
        elif kind == 4:  # an N in the query or the target's diagonal
            c = int(rng.integers(0, ql))
            if rng.random() < 0.5:
                q[c] = 4
            else:
                t[c] = 4
        elif kind == 5:  # target shorter than the query
            t = t[:max(0, ql - int(rng.integers(1, 5)))]
        qs.append(q)
        ts.append(t)
        h0s.append(int(rng.integers(1, 3)) if kind == 6 else int(rng.integers(1, 60)))
    for n in (2500, 2497, 33, 1):
        _check_batch(ugctx, qs[:n], ts[:n], h0s[:n], path=(B.PATH_BATCHED, B.GATHER_AUTO), what=f"ungapped edges {n}")


@pytest.mark.parametrize("cfg,n", [(1, 20000), (2, 200000), (3, 60000)])
def test_ungapped_prefilter_on_workloads(ugctx, cfg, n):
    js = B.synth_ext(cfg, n, seed=30 + cfg)
    want, cells = oracle.extend_batch(js)
    got = _device_run(ugctx, js, B.PATH_BATCHED, reps=2)
    for g in got:
        assert np.array_equal(g, want)
    _check_jobset(ugctx, js, path=(B.PATH_BATCHED, B.GATHER_AUTO))
    if cfg == 2:
        # the fast path settled most clean read-pair jobs: far fewer DP cells were run
        ugctx.reset_stats()
        ugctx.extend_batch(js, w=100) if len(np.unique(js.w)) == 1 else None
        assert ugctx.stats()["ext_cells"] < cells // 4


@pytest.mark.parametrize("gather", [B.GATHER_DEVICE, B.GATHER_HOST])
@pytest.mark.parametrize("offset", [0, 4, 8, 12])
def test_output_array_alignment(ctx, gather, offset):
    # the caller's result array at every 4-byte alignment, an odd job count, both host-buffer
    # routes: nothing written outside the array
    import ctypes as C

    js = B.synth_ext(2, 70001, seed=81)
    want, _ = oracle.extend_batch(js)
    jobs = B.Context._host_jobs(js, B.EXT_JOB)
    raw = np.zeros(len(js) * B.EXT_RES.itemsize + 64, np.uint8)
    base = (-raw.ctypes.data) % 16 + offset
    out = np.frombuffer(raw.data, dtype=B.EXT_RES, count=len(js), offset=base)
    mat = oracle.scmat()
    ctx.set_option(B.OPT_HOST_GATHER, gather)
    try:
        rc = B.lib().bwacuda_extend_batch(ctx.h, C.c_void_p(jobs.ctypes.data), len(js), 5, C.c_void_p(mat.ctypes.data),
                                          6, 1, 6, 1, 100, 5, 100, C.c_void_p(out.ctypes.data))
    finally:
        ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)
    assert rc == B.OK
    assert np.array_equal(out, want)
    assert not raw[:base].any() and not raw[base + len(js) * B.EXT_RES.itemsize:].any()
