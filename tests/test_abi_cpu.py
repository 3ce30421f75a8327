"""CPU-side checks of the C ABI library: it loads, exports every symbol the public
header declares, and its host-only helpers behave; no GPU compute is called."""
import ctypes
import os
import re

import numpy as np
import pytest

import bwacuda as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.usefixtures("built")


def _declared_symbols():
    src = open(os.path.join(ROOT, "include", "bwacuda.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(bwacuda_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(B.LIB_PATH)
    declared = _declared_symbols()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(lib, name), f"{name} declared in include/bwacuda.h but not exported"
    assert set(declared) == set(B.EXPORTS)


def test_static_strings_need_no_gpu():
    L = B.lib()
    assert L.bwacuda_backend_name() == b"cuda"
    assert L.bwacuda_strerror(B.EBASE).startswith(b"base code")
    assert L.bwacuda_strerror(12345) == b"unknown error"


def test_null_context_is_rejected():
    L = B.lib()
    assert L.bwacuda_set_option(None, B.OPT_EXT_PATH, 0) == B.EINVAL
    assert L.bwacuda_extend_batch(None, None, 0, 5, None, 6, 1, 6, 1, 100, 5, 100, None) == B.EINVAL
    assert L.bwacuda_ksw_align2_batch(None, None, 0, 5, None, 6, 1, 6, 1, 19, 1, None) == B.EINVAL


def test_struct_layouts_match_header():
    assert B.EXT_RES.itemsize == 24 and B.ALN_RES.itemsize == 28 and B.FWD_RES.itemsize == 20
    assert ctypes.sizeof(B.Scoring) == 84
    assert ctypes.sizeof(B.Tuning) == 56


def test_synthetic_workloads_are_deterministic():
    # integer-only generators: the same jobs on every host (a fixed digest)
    import hashlib

    js = B.synth_ext(2, 2000, seed=11)
    js2 = B.synth_ext(2, 2000, seed=11)
    assert np.array_equal(js.seq, js2.seq)
    assert js.qlen.max() <= 131 and js.qlen.min() >= 0
    assert np.all(js.tlen == js.qlen + 100)
    js3 = B.synth_ext(3, 3000, seed=11)
    assert js3.qlen.max() <= 231 and set(np.unique(js3.w)) <= {50, 100, 200} and js3.h0.max() <= 250
    r = B.synth_rescue(100, seed=11)
    assert np.all(r.qlen == 150) and np.all(r.tlen == 750)
    digest = hashlib.sha256(js.seq.tobytes() + js.h0.tobytes()).hexdigest()[:16]
    from golden_digests import SYNTH_EXT2_2000_SEED11
    assert digest == SYNTH_EXT2_2000_SEED11


def test_header_constants_match_binding():
    src = open(os.path.join(ROOT, "include", "bwacuda.h")).read()
    defs = dict((k, int(v)) for k, v in re.findall(r"#define BWACUDA_([A-Z0-9_]+) (-?\d+)", src))
    for name, val in defs.items():
        if hasattr(B, name):
            assert getattr(B, name) == val, name
    for name in ("OPT_EXT_PATH", "OPT_CHUNK_JOBS", "OPT_GRAPHS", "OPT_PERSIST_BLOCK", "OPT_RESCUE_KERNEL",
                 "OPT_HOST_GATHER", "OPT_GRAB", "OPT_BUCKET_STEP", "OPT_RESCUE_LANES", "OPT_UNGAPPED", "OPT_DEVICE_PIECE", "OPT_LONG_QLEN", "OPT_LONG_LANES", "OPT_RESCUE_PAIR", "OPT_LONG_SLIDE", "GATHER_AUTO", "GATHER_HOST", "GATHER_DEVICE", "PATH_PLAIN", "PATH_BATCHED"):
        assert getattr(B, name) == defs[name], name
