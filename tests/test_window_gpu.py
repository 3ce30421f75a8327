"""Mate rescue with windows fetched on the device from a reference in HBM (matesw_collect +
bns_fetch_seq + batched_ksw_align2) against the oracle's restatement of the same steps."""
import numpy as np
import pytest

import bwacuda as B
import oracle

pytestmark = pytest.mark.gpu

ALN = ("score", "qb", "qe", "tb", "te", "score2", "te2")


def _expected(rw, reqs, min_seed_len=19, minsc=20):
    ref = oracle.Reference(rw.bases, rw.contig_lens)
    two = np.concatenate([rw.bases, 3 - rw.bases[::-1]])
    # the 2L text used below is the oracle's unpack rule
    for p in (0, 1, rw.l_pac - 1, rw.l_pac, 2 * rw.l_pac - 1):
        assert two[p] == oracle.lib().ko_ref_base(ref.pac.ctypes.data_as(oracle.C.POINTER(oracle.C.c_uint8)),
                                                  ref.l_pac, p)
    win = []
    qs, ts = [], []
    for k in range(len(reqs)):
        l_ms = int(reqs[k]["l_ms"])
        mate = rw.mates[k][:l_ms] if l_ms else np.zeros(0, np.uint8)
        v, rb, re, rid = oracle.rescue_window(ref, int(reqs[k]["anchor_rb"]), int(reqs[k]["anchor_rid"]),
                                              int(reqs[k]["orient"]), int(reqs[k]["low"]), int(reqs[k]["high"]),
                                              l_ms, min_seed_len)
        win.append((rb, re, rid, int(v)))
        if v:
            qs.append(oracle.mate_for_orientation(mate, int(reqs[k]["orient"])))
            ts.append(two[rb:re])
    js = B.JobSet.from_lists(qs, ts)
    aln, _ = oracle.align2_batch(js, minsc=minsc, mode=0)
    return win, aln


def _check(got, win, aln):
    w = np.array([(g["rb"], g["re"], g["rid"], g["valid"]) for g in got])
    assert np.array_equal(w, np.array(win)), "window mismatch"
    valid = got[got["valid"] == 1]
    for f in ALN:
        assert np.array_equal(valid[f], aln[f]), f


@pytest.mark.parametrize("route", [pytest.param(B.GATHER_AUTO, id="in-place"),
                                   pytest.param(B.GATHER_HOST, id="staged")])
def test_windows_and_alignments(ctx, route):
    rw = B.RescueWindows(20000, seed=3, contig_lens=(300_000, 100_000, 50_000, 200_000))
    ctx.ref_set(rw)
    reqs = rw.requests()
    ctx.set_option(B.OPT_HOST_GATHER, route)
    try:
        got = ctx.mate_rescue_windows(reqs, minsc=20)
    finally:
        ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)
    win, aln = _expected(rw, reqs)
    _check(got, win, aln)
    assert got["valid"].mean() > 0.9 and (got["score"][got["valid"] == 1] >= 20).mean() > 0.5


def test_window_edges(ctx):
    # anchors at contig starts/ends on both strands, tiny windows, empty mates
    rw = B.RescueWindows(64, seed=5, contig_lens=(1000, 300, 2000, 77))
    L2 = 2 * rw.l_pac
    edge = [0, 1, 999, 1000, 1299, 1300, 3299, 3300, rw.l_pac - 1, rw.l_pac, L2 - 1, L2 - 1000]
    reqs = rw.requests()
    for i, a in enumerate(edge):
        for r in range(4):
            k = (i * 4 + r) % len(reqs)
            reqs[k]["anchor_rb"] = a
            reqs[k]["orient"] = r
    reqs[3]["low"], reqs[3]["high"] = 5, 8          # shorter than min_seed_len after clamps
    reqs[7]["l_ms"] = 0                              # an empty mate
    ctx.ref_set(rw)
    got = ctx.mate_rescue_windows(reqs, minsc=20)
    win, aln = _expected(rw, reqs)
    _check(got, win, aln)


def test_window_invalid_inputs():
    c = B.Context(0)
    try:
        rw = B.RescueWindows(10, seed=6, contig_lens=(5000,))
        reqs = rw.requests()
        with pytest.raises(B.BwaCudaError) as e:  # no reference set on this context
            c.mate_rescue_windows(reqs)
        assert e.value.code == B.EINVAL
        c.ref_set(rw)
        bad = reqs.copy()
        bad[2]["orient"] = 4
        with pytest.raises(B.BwaCudaError) as e:
            c.mate_rescue_windows(bad)
        assert e.value.code == B.EINVAL
        assert c.mate_rescue_windows(reqs)["valid"].sum() > 0
    finally:
        c.close()
