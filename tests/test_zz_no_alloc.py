"""The allocation-free mate-rescue entry point, bwacuda_ksw_align2_device_noalloc.

It serves callers that cannot allocate device memory (a pool allocator owns the
whole device budget, or cudaMalloc/cudaFree would synchronise a latency-critical
stream): its tracker scratch is a static device array of the library.  Its results
must equal those of bwacuda_ksw_align2_device, exactly, on consecutive calls (the
static array keeps the previous call's contents).  This file is collected last.
"""
import numpy as np
import pytest

import bwacuda as B

pytestmark = pytest.mark.gpu


def _device_jobs(js):
    import torch

    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_res_jobs().view(np.uint8)).cuda()
    return d_seq, d_jobs


def test_noalloc_matches_allocating_entry_on_consecutive_calls(ctx):
    import torch

    # two different batches in a row, both modes: stale scratch must not leak
    for call, (seed, n, mode) in enumerate([(21, 3000, 0), (22, 2500, 1)]):
        js = B.synth_rescue(n, seed=seed)
        d_seq, d_jobs = _device_jobs(js)
        want = torch.zeros(n * 28, dtype=torch.uint8, device="cuda")
        got = torch.full((n * 28,), 0xAB, dtype=torch.uint8, device="cuda")
        ctx.ksw_align2_device(d_seq.data_ptr(), d_jobs.data_ptr(), n, want.data_ptr(), minsc=20, mode=mode)
        ctx.sync()
        ctx.ksw_align2_device_noalloc(d_seq.data_ptr(), d_jobs.data_ptr(), n, got.data_ptr(), minsc=20, mode=mode)
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"call {call}: no-alloc results differ"


def test_noalloc_rejects_oversized_calls(ctx):
    import torch

    # 60,000 jobs of 750-base windows need 60000 * 377 entries > 16 Mi: rejected before launch
    js = B.synth_rescue(60000, seed=23)
    d_seq, d_jobs = _device_jobs(js)
    out = torch.zeros(len(js) * 28, dtype=torch.uint8, device="cuda")
    with pytest.raises(B.BwaCudaError) as e:
        ctx.ksw_align2_device_noalloc(d_seq.data_ptr(), d_jobs.data_ptr(), len(js), out.data_ptr(), minsc=20)
    assert e.value.code == B.EUNSUPPORTED


def test_noalloc_error_call_then_clean_call(ctx):
    import torch

    # a bad base code in the last job's target makes the call fail with BWACUDA_EBASE; the next
    # call on clean input must not see that call's error flag or its scratch
    n = 2000
    js = B.synth_rescue(n, seed=24)
    bad = js.seq.copy()
    bad[int(js.t_off[-1]) + int(js.tlen[-1]) - 1] = 9
    d_bad = torch.from_numpy(bad).cuda()
    d_seq, d_jobs = _device_jobs(js)
    out = torch.zeros(n * 28, dtype=torch.uint8, device="cuda")
    with pytest.raises(B.BwaCudaError) as e:
        ctx.ksw_align2_device_noalloc(d_bad.data_ptr(), d_jobs.data_ptr(), n, out.data_ptr(), minsc=20)
    assert e.value.code == B.EBASE
    want = torch.zeros(n * 28, dtype=torch.uint8, device="cuda")
    got = torch.full((n * 28,), 0xCD, dtype=torch.uint8, device="cuda")
    ctx.ksw_align2_device(d_seq.data_ptr(), d_jobs.data_ptr(), n, want.data_ptr(), minsc=20)
    ctx.sync()
    ctx.ksw_align2_device_noalloc(d_seq.data_ptr(), d_jobs.data_ptr(), n, got.data_ptr(), minsc=20)
    torch.cuda.synchronize()
    assert torch.equal(got, want)


def test_noalloc_rejects_more_than_max_jobs(ctx):
    import torch

    # 524,289 jobs is one past the offsets array: rejected before anything is read or launched
    n = (512 << 10) + 1
    d_seq = torch.zeros(16, dtype=torch.uint8, device="cuda")
    d_jobs = torch.zeros(n * 32, dtype=torch.uint8, device="cuda")
    out = torch.zeros(n * 28, dtype=torch.uint8, device="cuda")
    with pytest.raises(B.BwaCudaError) as e:
        ctx.ksw_align2_device_noalloc(d_seq.data_ptr(), d_jobs.data_ptr(), n, out.data_ptr(), minsc=20)
    assert e.value.code == B.EUNSUPPORTED
