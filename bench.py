"""Benchmark: bit-exact banded seed-extension GCUPS on one GB300.

Workload (one "step"): 8,388,608 seed-extension jobs drawn as left/right
extension pairs of 2x150 bp reads (seed 19-60 bp, qlen 0..131, tlen = qlen +
100, w = 100, 0.1% SNV / 0.01% indel divergence, 2% of jobs with a 5%-error
tail), bwa default scoring.  Inputs are larger than L2 (about 2.1 GB of bases
and descriptors), so no flush is needed between steps.

value    : GCUPS of the batched path (length-sorted buckets, persistent
           kernels, graph replay) with the inputs resident in HBM.
e2e      : the same metric through bwacuda_extend_batch with HOST buffers, every
           transfer inside the timed region.  Two routes are timed: "device-gather"
           (GPU kernels load the caller's job array and sequence slices from host
           memory over NVLink-C2C and store the results into the caller's array)
           and "host-pack" (worker threads pack pinned staging, copy-engine
           transfers); the headline is device-gather where the device supports it.
plain    : the plain path (one launch per 256k-job chunk, caller order).
configs  : the mixed-length extension workload (32M jobs, per-job bands) and
           mate rescue (2M jobs), device-resident; the CIGAR stage
           (ksw_global2 with traceback, 1M jobs) through host buffers.
served   : the serving loop replaying Poisson arrivals of mixed extension and
           rescue requests, p50/p99 latency and jobs/s against a FIFO of
           synchronous plain-path calls on the same arrivals.
GCUPS    = extension cells (one inner-loop iteration of ksw_extend2, counted by
           the kernels themselves and equal to the oracle's count) / time.

--impl reference times the CPU restatement of the reference algorithm (the
reference is Rust and no Rust toolchain exists on these hosts) on every host
core, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "bwa-mem4_gb300")
sys.path.insert(0, PKG)
sys.path.insert(0, ROOT)

METRIC = "bit-exact SW extension GCUPS: batched/served vs plain on 1 GB300; p50/p99 latency"
N_JOBS = 8 * 1024 * 1024
OPS_PER_CELL = 9  # minimal fused integer op count of one extension cell
RESCUE_OPS_PER_CELL = 10  # minimal fused integer ops per rescue cell (max(0,Hd+s), max3, E, F, max/argmax)
# minimal fused integer ops per ksw_global2 cell with traceback: M = H + s (1), max(M, E) and max(., F)
# with their direction bits (2), E and F each open, extend and a direction-keeping max (3 + 3), the
# traceback byte (1)
GLOBAL_OPS_PER_CELL = 10
# DRAM bytes per read-pair job of the batched step, from an ncu capture of every persistent bucket
# kernel of a 2,000,000-job call (dram__bytes_read.sum + dram__bytes_write.sum = 862.4 MB + 68.9 MB)
DRAM_BYTES_PER_JOB = 931294208 / 2000000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--jobs", type=int, default=N_JOBS)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-chunk", type=int, default=1 << 20, help="jobs per pipelined chunk of the host-buffer call")
    ap.add_argument("--no-graphs", action="store_true", help="enqueue the batched path every step (profiling)")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--no-configs", action="store_true", help="skip the mixed-length and rescue workloads")
    ap.add_argument("--mixed-jobs", type=int, default=32 * 1024 * 1024)
    ap.add_argument("--rescue-jobs", type=int, default=2 * 1024 * 1024)
    ap.add_argument("--global-jobs", type=int, default=1024 * 1024)
    ap.add_argument("--window-jobs", type=int, default=1024 * 1024)
    ap.add_argument("--serve-rates", default="50,500,2000", help="Poisson arrival rates (requests/s)")
    ap.add_argument("--serve-requests", type=int, default=600, help="requests per arrival rate")
    ap.add_argument("--case", choices=["ext-batched", "ext-plain", "ext-mixed", "ext-gather", "ext-long", "rescue",
                                       "global", "windows", "retry", "serve", "op-rates"],
                    help="profiling case: run the small workload twice through one path, no timing")
    ap.add_argument("--lanes", type=int, default=8, help="rescue case: wavefront lanes per job")
    ap.add_argument("--pair", type=int, default=0, choices=[0, 1, 4, 8, 16],
                    help="rescue case: lanes of a group holding two byte-range jobs (0: one job per group)")
    ap.add_argument("--rescue-kernel", choices=["auto", "tpj"], default="auto",
                    help="rescue case: the wavefronts where the jobs fit (auto) or thread-per-job for all")
    ap.add_argument("--gaps", default="6,1,6,1", help="extension cases: o_del,e_del,o_ins,e_ins")
    ap.add_argument("--ungapped", type=int, default=0, help="extension cases: the ungapped pre-pass on (1)")
    ap.add_argument("--persist-block", type=int, default=0,
                    help="extension cases: threads per block of the persistent kernels (0: the library's default)")
    ap.add_argument("--h0-add", type=int, default=0,
                    help="extension cases: add this to every h0 (300 moves read pairs into the 16-bit cell class)")
    return ap.parse_args()


# ---------------------------------------------------------------- serving (continuous batching)

SERVE_MAX, SERVE_MIN = 262144, 1000
RES_POOL = 1 << 18


class ServePools:
    """Job pools the requests are windows of, with their caller-side job arrays built once."""

    def __init__(self, B, seed):
        self.B = B
        self.ext = {2: B.synth_ext(2, 1 << 21, seed=seed + 1), 3: B.synth_ext(3, 1 << 21, seed=seed + 2)}
        self.res = B.synth_rescue(RES_POOL, seed=seed + 3)
        self.ext_jobs = {k: B.Context._host_jobs(js, B.EXT_JOB) for k, js in self.ext.items()}
        self.res_jobs = B.Context._host_jobs(self.res, B.RES_JOB, minsc=20, endsc=0)
        self.res_cells = np.concatenate([[0], np.cumsum(self.res.qlen.astype(np.int64) * self.res.tlen)])


def serve_trace(rate, count, seed):
    """Poisson arrivals of mixed requests: each carries n jobs, n log-uniform in [1k, 256k], of
    which a share s are rescue jobs (150 bp vs 750 bp windows) and the rest extension jobs from
    the read-pair or mixed-length pool (one band per request); s is 1 for 10% of the requests
    (rescue-only, up to 256k jobs), 0 for 10% (extension-only), else uniform in [0.05, 0.4].
    Entries: (arrival, pool, ext start, n_ext, w, rescue start, n_rescue)."""
    rng = np.random.default_rng(seed)
    t, trace = 0.0, []
    for _ in range(count):
        t += rng.exponential(1.0 / rate)
        n = int(np.exp(rng.uniform(np.log(SERVE_MIN), np.log(SERVE_MAX))))
        u = rng.random()
        share = 1.0 if u < 0.1 else (0.0 if u < 0.2 else rng.uniform(0.05, 0.4))
        nr = int(round(n * share))
        ne = n - nr
        cfg = int(rng.choice([2, 3]))
        w = 100 if cfg == 2 else int(rng.choice([50, 100, 200]))
        es = int(rng.integers(0, (1 << 21) - ne + 1))
        rs = int(rng.integers(0, RES_POOL - nr + 1))
        trace.append((t, cfg, es, ne, w, rs, nr))
    return trace


def _out_layout(B, trace):
    offs, tot = [], 0
    for _, _, _, ne, _, _, nr in trace:
        offs.append(tot)
        tot += ne * B.EXT_RES.itemsize + nr * B.ALN_RES.itemsize
    return offs, tot


def apply_tuning(B, ctx, t):
    if t:
        ctx.set_option(B.OPT_PERSIST_BLOCK, t["persist_block"])
        ctx.set_option(B.OPT_GRAB, t["grab"])
        ctx.set_option(B.OPT_BUCKET_STEP, t["bucket_step"])
        ctx.set_option(B.OPT_RESCUE_KERNEL, t["rescue_kernel"])
        ctx.set_option(B.OPT_RESCUE_LANES, t["rescue_lanes"])
        ctx.set_option(B.OPT_RESCUE_PAIR, t.get("rescue_pair", 0))
        ctx.set_option(B.OPT_LONG_QLEN, t.get("long_qlen", 0))
        ctx.set_option(B.OPT_LONG_LANES, t.get("long_lanes", 16))


def run_served(B, pools, trace, budget, tuning=None):
    """Real-time replay through the serving loop: a submitter thread submits each request at its
    arrival time (one bwacuda_server_submit_mixed call); the caller's thread waits on them in
    order.  Latency = completion - arrival.  Returns latencies, the last completion time, the
    results and the cells served (extension + rescue)."""
    import ctypes as C

    L = B.lib()
    ctx = B.Context(0)
    apply_tuning(B, ctx, tuning)
    ctx.server_start(hbm_budget_bytes=budget, max_waves=3, max_requests=8192)
    sc = ctx.scoring()
    offs, tot = _out_layout(B, trace)
    out = np.zeros(max(tot, 1), np.uint8)
    rids, submit_t = [None] * len(trace), [0.0] * len(trace)
    ready = threading.Semaphore(0)
    err = []

    def submitter(t0):
        for i, (ta, cfg, es, ne, w, rs, nr) in enumerate(trace):
            d = t0 + ta - time.perf_counter()
            if d > 0:
                time.sleep(d)
            rid = C.c_uint64()
            submit_t[i] = time.perf_counter() - t0
            ejp = pools.ext_jobs[cfg].ctypes.data + es * B.EXT_JOB.itemsize
            rjp = pools.res_jobs.ctypes.data + rs * B.RES_JOB.itemsize
            rc = L.bwacuda_server_submit_mixed(ctx.h, C.c_void_p(ejp), ne, C.c_void_p(rjp), nr, C.byref(sc), w, 5,
                                               100, 20, 1, C.byref(rid))
            if rc != B.OK:
                err.append(rc)
            rids[i] = rid.value
            ready.release()

    lat = np.zeros(len(trace))
    t0 = time.perf_counter() + 0.05
    th = threading.Thread(target=submitter, args=(t0,), daemon=True)
    th.start()
    last = 0.0
    for i in range(len(trace)):
        ready.acquire()
        if err:
            break
        ns = C.c_int64()
        rc = L.bwacuda_server_wait(ctx.h, rids[i], C.c_void_p(out.ctypes.data + offs[i]), -1, C.byref(ns))
        if rc != B.OK:
            err.append(rc)
            break
        done = submit_t[i] + ns.value * 1e-9
        lat[i] = done - trace[i][0]
        last = max(last, done)
    th.join()
    ext_cells, res_cells = ctx.server_cells()
    ctx.server_stop()
    ctx.close()
    if err:
        raise B.BwaCudaError(err[0], "serving replay")
    return lat, last, out, ext_cells + res_cells


def run_plain_fifo(B, pools, trace):
    """The same arrivals served one request at a time in arrival order by synchronous plain-path
    calls (host packing, one launch per 256k-job chunk): the request's extension jobs, then its
    rescue jobs.  Latency = completion - arrival."""
    import ctypes as C

    L = B.lib()
    ctx = B.Context(0)
    ctx.set_option(B.OPT_EXT_PATH, B.PATH_PLAIN)
    ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_HOST)
    mat = B.scmat()
    offs, tot = _out_layout(B, trace)
    out = np.zeros(max(tot, 1), np.uint8)
    lat = np.zeros(len(trace))
    ctx.reset_stats()
    t0 = time.perf_counter()
    now = 0.0
    for i, (ta, cfg, es, ne, w, rs, nr) in enumerate(trace):
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        if ne:
            jp = C.c_void_p(pools.ext_jobs[cfg].ctypes.data + es * B.EXT_JOB.itemsize)
            op = C.c_void_p(out.ctypes.data + offs[i])
            rc = L.bwacuda_extend_batch(ctx.h, jp, ne, 5, C.c_void_p(mat.ctypes.data), 6, 1, 6, 1, w, 5, 100, op)
            if rc != B.OK:
                raise B.BwaCudaError(rc, "plain replay")
        if nr:
            jp = C.c_void_p(pools.res_jobs.ctypes.data + rs * B.RES_JOB.itemsize)
            op = C.c_void_p(out.ctypes.data + offs[i] + ne * B.EXT_RES.itemsize)
            rc = L.bwacuda_ksw_align2_batch(ctx.h, jp, nr, 5, C.c_void_p(mat.ctypes.data), 6, 1, 6, 1, 20, 1, op)
            if rc != B.OK:
                raise B.BwaCudaError(rc, "plain replay")
        now = time.perf_counter() - t0
        lat[i] = now - ta
    st = ctx.stats()
    ctx.close()
    return lat, now, out, st["ext_cells"] + st["rescue_cells"]


def serve_bench(B, rates, count, seed=5, budget=8 << 30, tuning=None):
    pools = ServePools(B, seed)
    # warm both sides (allocations, module loading) on short traces: the served side's covers the
    # request mix (read-pair and mixed-length extension, rescue) so that every kernel variant its
    # waves use is loaded (CUDA loads a kernel's module at its first launch in the process)
    run_served(B, pools, serve_trace(2000.0, 64, seed + 99), budget, tuning)
    run_plain_fifo(B, pools, serve_trace(1000.0, 8, seed + 99))
    rows = []
    for rate in rates:
        # at most ~4 s of arrivals per rate (and at least 100 requests)
        trace = serve_trace(rate, min(count, max(100, int(rate * 4))), seed + int(rate))
        ext_jobs = sum(r[3] for r in trace)
        res_jobs = sum(r[6] for r in trace)
        jobs = ext_jobs + res_jobs
        ls, end_s, out_s, cells_s = run_served(B, pools, trace, budget, tuning)
        lp, end_p, out_p, cells_p = run_plain_fifo(B, pools, trace)
        pct = lambda a, q: round(float(np.percentile(a, q)) * 1e3, 3)
        g_s, g_p = cells_s / end_s / 1e9, cells_p / end_p / 1e9
        rows.append({"rate_req_s": rate, "requests": len(trace), "jobs": jobs, "extension_jobs": ext_jobs,
                     "rescue_jobs": res_jobs, "max_rescue_jobs_per_request": max(r[6] for r in trace),
                     "cells": cells_s,
                     "served": {"p50_ms": pct(ls, 50), "p99_ms": pct(ls, 99), "jobs_per_s": round(jobs / end_s, 1),
                                "gcups": round(g_s, 2)},
                     "plain": {"p50_ms": pct(lp, 50), "p99_ms": pct(lp, 99), "jobs_per_s": round(jobs / end_p, 1),
                               "gcups": round(g_p, 2)},
                     "gcups_vs_plain": round(g_s / g_p, 3) if g_p > 0 else None,
                     "cells_equal": bool(cells_s == cells_p),
                     "identical": bool(np.array_equal(out_s, out_p))})
    return {"workload": "Poisson arrivals of mixed requests: each 1k-256k jobs (log-uniform), a share of them "
                        "rescue jobs (150 bp vs 750 bp windows, minsc 20) and the rest extension jobs from the "
                        "read-pair or mixed-length/band pool; share 1 for 10% of requests (rescue-only, up to 256k "
                        "jobs), 0 for 10%, else uniform in [0.05, 0.4]; one submit per request; latency = "
                        "completion - arrival; GCUPS = extension cells + rescue qlen x tlen cells over the replay",
            "hbm_budget_bytes": budget, "plain": "FIFO, synchronous plain-path calls per request (extension, then rescue)",
            "rates": rows}


def other_configs(args, B, ctx, st, barrier, max_over_ranks, world, rank):
    """The mixed-length extension workload (one batched call over all jobs, per-job bands) and
    the mate-rescue workload, both device-resident, each timed with CUDA events over 3 steps."""
    import torch

    res = {}
    stream = st.cuda_stream

    def timed(fn, steps=3, warmup=1):
        for _ in range(warmup):
            fn()
        ctx.sync()
        ctx.reset_stats()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(steps):
            fn()
        e1.record(st)
        ctx.sync()
        barrier()
        return max_over_ranks(e0.elapsed_time(e1)) / steps, ctx.stats()

    # mixed read lengths 100/150/250 bp, w in {50, 100, 200} per job, h0 up to 250
    n = args.mixed_jobs
    js = B.synth_ext(3, n, seed=2000 + rank)
    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_ext_jobs().view(np.uint8)).cuda()
    d_out = torch.zeros(n * 24, dtype=torch.uint8, device="cuda")
    # the reference's 8/16-bit kernel choice for these jobs (crates/bwa-neon/src/batched.rs:846-866:
    # both lengths < 256 and h0 + min(qlen, tlen) * a + max(b, N penalty) + a < 256); this
    # library picks its cell width from the value bound alone, with the same results
    mn = np.minimum(js.qlen, js.tlen).astype(np.int64)
    u8 = (js.qlen < 256) & (js.tlen < 256) & (js.h0.astype(np.int64) + mn * 1 + 5 < 256)
    ref_bins = {"8-bit": round(float(u8.mean()), 4), "16-bit": round(float(1 - u8.mean()), 4)}
    tuning_mixed = ctx.autotune_extend(d_seq.data_ptr(), d_jobs.data_ptr(), n)
    ms, stt = timed(lambda: ctx.extend_device(d_seq.data_ptr(), d_jobs.data_ptr(), n, d_out.data_ptr(),
                                              path=B.PATH_BATCHED, stream=stream))
    batched = d_out.cpu().numpy().copy()
    cells = stt["ext_cells"] / 3
    # the plain path on the same jobs (one pass, 256k-job launches) must give the same results
    ctx.reset_stats()
    t0 = time.perf_counter()
    for c0 in range(0, n, 262144):
        cn = min(262144, n - c0)
        ctx.extend_device(d_seq.data_ptr(), d_jobs.data_ptr() + c0 * 32, cn, d_out.data_ptr() + c0 * 24,
                          path=B.PATH_PLAIN, stream=stream)
    ctx.sync()
    tp = time.perf_counter() - t0
    res["mixed_lengths"] = {
        "workload": f"ksw_extend2, {n} jobs per GPU: reads 30% 100 / 50% 150 / 20% 250 bp, per-job w in "
                    "{50, 100, 200}, h0 <= 250; one batched call",
        "value": round(cells * world / (ms / 1e3) / 1e9, 2), "unit": "GCUPS", "ms_per_step": round(ms, 2),
        "plain": {"value": round(ctx.stats()["ext_cells"] * world / tp / 1e9, 2), "unit": "GCUPS"},
        "plain_equals_batched": bool(np.array_equal(batched, d_out.cpu().numpy())), "tuning": tuning_mixed,
        "reference_bins": ref_bins}
    del d_seq, d_jobs, d_out, js
    torch.cuda.empty_cache()

    # the 16-bit cell class: read-pair jobs with 300 added to every h0 (256 <= h0 + min(qlen, tlen)
    # < 32768), batched, device-resident; the plain path checks the results
    n = args.mixed_jobs // 8
    js = B.synth_ext(2, n, seed=6000 + rank)
    js.h0 = js.h0 + 300
    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_ext_jobs().view(np.uint8)).cuda()
    d_out = torch.zeros(n * 24, dtype=torch.uint8, device="cuda")
    ms, stt = timed(lambda: ctx.extend_device(d_seq.data_ptr(), d_jobs.data_ptr(), n, d_out.data_ptr(),
                                              path=B.PATH_BATCHED, stream=stream))
    batched = d_out.cpu().numpy().copy()
    for c0 in range(0, n, 262144):
        cn = min(262144, n - c0)
        ctx.extend_device(d_seq.data_ptr(), d_jobs.data_ptr() + c0 * 32, cn, d_out.data_ptr() + c0 * 24,
                          path=B.PATH_PLAIN, stream=stream)
    ctx.sync()
    res["sixteen_bit_cells"] = {
        "workload": f"ksw_extend2, {n} read-pair jobs per GPU with h0 + 300 (every job in the 16-bit cell "
                    "class); one batched call",
        "value": round(stt["ext_cells"] / 3 * world / (ms / 1e3) / 1e9, 2), "unit": "GCUPS",
        "ms_per_step": round(ms, 2),
        "plain_equals_batched": bool(np.array_equal(batched, d_out.cpu().numpy()))}
    del d_seq, d_jobs, d_out, js
    torch.cuda.empty_cache()

    # mate rescue: 150 bp query vs 750 bp window, minsc 20
    n = args.rescue_jobs
    js = B.synth_rescue(n, seed=3000 + rank)
    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_res_jobs().view(np.uint8)).cuda()
    d_out = torch.zeros(n * 28, dtype=torch.uint8, device="cuda")
    rcells = int((js.qlen.astype(np.int64) * js.tlen.astype(np.int64)).sum())
    tuning_res = ctx.autotune_rescue(d_seq.data_ptr(), d_jobs.data_ptr(), n, minsc=20, max_sc=1)
    ms, stt = timed(lambda: ctx.ksw_align2_device(d_seq.data_ptr(), d_jobs.data_ptr(), n, d_out.data_ptr(),
                                                  minsc=20, max_sc=1, mode=0, stream=stream))
    res["rescue"] = {
        "workload": f"batched_ksw_align2, {n} jobs per GPU: 150 bp query (0.5% error) vs 750 bp window, "
                    "10% without the true mate, minsc 20",
        "value": round(rcells * world / (ms / 1e3) / 1e9, 2), "unit": "GCUPS",
        "cells": "qlen x tlen of the forward pass per job (padding and reverse pass not counted)",
        "ms_per_step": round(ms, 2), "jobs_per_s": round(n * world / (ms / 1e3), 1),
        "tuning": {k: tuning_res[k] for k in ("rescue_kernel", "rescue_lanes", "rescue_pair", "rescue_gcups",
                                            "candidates")}}
    if rank == 0:
        # CPU baseline: the oracle's batched_ksw_align2 (forward pass, truncated reverse pass) on every
        # host core over the first 20,000 jobs of the same workload
        import oracle

        sample = js.head(min(n, 20000))
        oracle.align2_batch(sample.head(min(n, 2000)), minsc=20)  # warm the thread pool
        t0 = time.perf_counter()
        _, ccells = oracle.align2_batch(sample, minsc=20)
        cdt = time.perf_counter() - t0
        res["rescue"]["cpu_baseline"] = {
            "value": round(ccells / cdt / 1e9, 3), "unit": "GCUPS", "cores": os.cpu_count(), "kind": "port",
            "isa": host_isa(), "sample": f"first {len(sample)} jobs of the workload ({ccells} cells)",
            "form": "batched_ksw_align2 restated (crates/bwa-neon/src/matesw.rs:299-497), scalar per job"}
        res["rescue"]["over_cpu"] = round(res["rescue"]["value"] / res["rescue"]["cpu_baseline"]["value"], 2)
    del d_seq, d_jobs, d_out
    torch.cuda.empty_cache()

    # queries of 2,000-10,000 bases (the group-per-job kernel, one group of lanes per job, the DP
    # row in a shared-memory ring), device-resident, every lane count timed
    res["long_queries"] = long_query_config(B, ctx, st, stream, timed, world)

    # mate rescue with the windows fetched on the device from the reference in HBM
    n = args.window_jobs
    rw = B.RescueWindows(n, seed=5000 + rank)
    ctx.ref_set(rw)
    reqs = rw.requests()
    ctx.mate_rescue_windows(reqs[: min(n, 65536)], minsc=20)  # warm-up
    # timed through the C call with the caller's request and record arrays held across calls
    import ctypes as C

    wres = np.zeros(n, dtype=B.WINDOW_RES)
    wmat = B.scmat()

    def window_call():
        rc = B.lib().bwacuda_mate_rescue_windows(ctx.h, C.c_void_p(reqs.ctypes.data), n, 5,
                                                 C.c_void_p(wmat.ctypes.data), 6, 1, 6, 1, 20, 1, 19,
                                                 C.c_void_p(wres.ctypes.data))
        if rc != B.OK:
            raise B.BwaCudaError(rc, "bwacuda_mate_rescue_windows")

    window_call()
    ctx.reset_stats()
    t0 = time.perf_counter()
    for _ in range(3):
        window_call()
    dt = max_over_ranks((time.perf_counter() - t0) / 3)
    stw = ctx.stats()
    res["rescue_windows"] = {
        "workload": f"mate rescue from {n} requests per GPU: anchors on both strands of a 6.5 Mbp 4-contig genome "
                    "held in HBM as a 2-bit .pac, all four orientations, insert window [100, 700] (750 bp windows), "
                    "150 bp mates; windows planned, clamped and unpacked on the device, then batched_ksw_align2; "
                    "host buffers in and out",
        "value": round(stw["rescue_cells"] / 3 * world / dt / 1e9, 2), "unit": "GCUPS",
        "ms_per_step": round(dt * 1e3, 2), "requests_per_s": round(n * world / dt, 1),
        "accepted_windows": float(round(wres["valid"].mean(), 4))}
    del rw, reqs, wres

    # CIGAR stage: banded global alignment with traceback, through the host-buffer C call (the
    # caller's job array and output arrays built once, as a C or Rust caller holds them)
    n = args.global_jobs
    js = B.synth_global(n, seed=4000 + rank)
    ctx.ksw_global2_batch(js.head(min(n, 65536)))  # warm-up (buffers)
    gjobs = np.zeros(n, dtype=B.GLOBAL_JOB)
    gjobs["query"] = js.seq.ctypes.data + js.q_off.astype(np.uint64)
    gjobs["target"] = js.seq.ctypes.data + js.t_off.astype(np.uint64)
    gjobs["qlen"], gjobs["tlen"], gjobs["w"] = js.qlen, js.tlen, js.w
    gmat = B.scmat()
    gscore = np.zeros(n, np.int32)
    offs = np.zeros(n + 1, np.uint64)
    words = np.zeros(8 * n, np.uint32)  # 1.15 runs per job on this workload

    def cigar_call():
        rc = B.lib().bwacuda_ksw_global2_batch(ctx.h, C.c_void_p(gjobs.ctypes.data), n, 5,
                                               C.c_void_p(gmat.ctypes.data), 6, 1, 6, 1,
                                               C.c_void_p(gscore.ctypes.data), C.c_void_p(offs.ctypes.data),
                                               C.c_void_p(words.ctypes.data), len(words))
        if rc != B.OK:
            raise B.BwaCudaError(rc, "bwacuda_ksw_global2_batch")

    cigar_call()
    ctx.reset_stats()
    t0 = time.perf_counter()
    for _ in range(3):
        cigar_call()
    dt = max_over_ranks((time.perf_counter() - t0) / 3)
    stg = ctx.stats()
    res["cigar_stage"] = {
        "workload": f"ksw_global2 with traceback, {n} jobs per GPU: reads of 100/150/250 bp against their aligned "
                    "reference interval (1% substitutions, 1-3 bp indels), per-job band from bwa-mem's sizing rule; "
                    "host buffers in and out (CIGAR runs compacted on the device)",
        "value": round(stg["global_cells"] / 3 * world / dt / 1e9, 2), "unit": "GCUPS",
        "cells": "sum over target rows of the band width",
        "ms_per_step": round(dt * 1e3, 2), "jobs_per_s": round(n * world / dt, 1),
        "cigar_runs_per_job": round(float(offs[-1]) / n, 3)}
    return res


def long_query_jobs(B, m, seed):
    """m extension jobs with queries of 2,000-10,000 bases (1% substitutions), tlen = qlen + 100,
    w = 100, h0 20-60."""
    rng = np.random.default_rng(seed)
    ql = rng.integers(2000, 10001, m).astype(np.int32)
    tl = (ql + 100).astype(np.int32)
    qo, to, total = B._layout(ql, tl)
    seq = np.zeros(total, np.uint8)
    for k in range(m):
        t_ = rng.integers(0, 4, int(tl[k])).astype(np.uint8)
        q_ = t_[:ql[k]].copy()
        mk = rng.random(int(ql[k])) < 0.01
        q_[mk] = (q_[mk] + 1) % 4
        seq[qo[k]:qo[k] + ql[k]] = q_
        seq[to[k]:to[k] + tl[k]] = t_
    return B.JobSet(seq, qo, to, ql, tl, rng.integers(20, 61, m).astype(np.int32), np.full(m, 100, np.int32))


def long_query_config(B, ctx, st, stream, timed, world, m=20000, seed=7000):
    """ksw_extend2 on m queries of 2,000-10,000 bases (1% substitutions), tlen = qlen + 100,
    w = 100, device-resident: the group-per-job kernel at 8, 16 and 32 lanes per job on the plain
    path (the long queries go straight to it) and on the batched path with the window kernel off,
    then the batched path's default (the thread-per-job window kernel takes these jobs)."""
    import torch

    js = long_query_jobs(B, m, seed)
    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_ext_jobs().view(np.uint8)).cuda()
    d_out = torch.zeros(m * 24, dtype=torch.uint8, device="cuda")
    rows, ref = {}, None

    def run(name, path):
        nonlocal ref
        ms, stt = timed(lambda: ctx.extend_device(d_seq.data_ptr(), d_jobs.data_ptr(), m, d_out.data_ptr(),
                                                  path=path, stream=stream), steps=2)
        out = d_out.cpu().numpy().copy()
        ref = out if ref is None else ref
        rows[name] = {"value": round(stt["ext_cells"] / 2 * world / (ms / 1e3) / 1e9, 2),
                      "ms_per_step": round(ms, 2), "identical": bool(np.array_equal(out, ref))}

    ctx.set_option(B.OPT_LONG_SLIDE, 0)
    for lanes in (8, 16, 32):
        ctx.set_option(B.OPT_LONG_LANES, lanes)
        for path, name in ((B.PATH_PLAIN, "plain"), (B.PATH_BATCHED, "batched")):
            run(f"{name}_lanes{lanes}", path)
    ctx.set_option(B.OPT_LONG_LANES, 16)
    ctx.set_option(B.OPT_LONG_SLIDE, 1)
    run("batched_window", B.PATH_BATCHED)
    best = max(rows, key=lambda k: rows[k]["value"])
    window = best == "batched_window"
    del d_seq, d_jobs, d_out
    torch.cuda.empty_cache()
    return {"workload": f"ksw_extend2, {m} jobs per GPU: qlen 2000-10000 (1% substitutions), tlen = qlen + 100, "
                        "w = 100, h0 20-60; queries too long for the full-row thread-per-job kernels",
            "value": rows[best]["value"], "unit": "GCUPS", "best": best, "runs": rows,
            "lanes_per_op": 2 if window else 1,
            "kernel": ("ext_slide_kernel: one thread per job, 16-bit pair cells, the row in a window of the band "
                       "sliding along the query" if window else
                       "ext_long_kernel: one group of lanes per job, 32-bit lane arithmetic")}


def alu_roofline(gcups, ops_per_cell, peak_g, lanes_per_op):
    """The integer-ALU roofline of a DP path: achieved = GCUPS x the minimal fused operation count
    of a cell; peak = the measured ALU instruction rate x the operations one instruction does at
    the width the cells need (2 for 16-bit lanes: one DPX instruction updates two cells)."""
    achieved = gcups * ops_per_cell
    peak = peak_g * lanes_per_op
    return {"bound": "alu", "ops_per_cell": ops_per_cell, "lanes_per_op": lanes_per_op,
            "achieved": round(achieved, 1), "peak": round(peak, 1), "unit": "Gop/s",
            "frac": round(achieved / peak, 4), "frac_32bit_lanes": round(achieved / peak_g, 4)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx or None, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


def int_peak_gops(nsm, mhz):
    # integer ALU pipe (min/max/compare/select/permute): half a warp-instruction per cycle per
    # scheduler, i.e. 64 lanes per SM per clock (ncu: the rescue kernel's ALU pipe at 84.6% of
    # peak while issuing 0.80 warp-instructions per cycle per scheduler)
    return nsm * 64 * mhz * 1e6 / 1e9


def cpu_baseline(js_sample, nthreads=0):
    """The oracle's scalar DP on every job: (cells, seconds)."""
    import oracle

    t0 = time.perf_counter()
    _, cells = oracle.extend_batch(js_sample, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return cells, dt


def cpu_dispatch(js_sample, nthreads=0):
    """The reference's production flow restated on the CPU: the ungapped closed form first
    (crates/bwa-neon/src/batched.rs:773), the scalar DP for the jobs it declines.
    Returns (jobs settled by the closed form, DP cells evaluated, seconds)."""
    import oracle

    t0 = time.perf_counter()
    _, settled, cells = oracle.extend_batch_dispatch(js_sample, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return settled, cells, dt


def host_isa():
    """Host architecture and CPU model as /proc/cpuinfo names them."""
    import platform

    model = ""
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                k = ln.split(":")[0].strip().lower()
                if k in ("model name", "cpu part") and not model:
                    model = ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return f"{platform.machine()} {model}".strip() + " (scalar C, gcc -O2, OpenMP over jobs)"


def cpu_extension_baseline(js_sample):
    """Both CPU forms on one sample: the production dispatch (headline, equivalent GCUPS over
    the sample's full-DP cells) and the plain scalar DP on every job."""
    for _ in range(2):  # warm the thread pool and the pages
        cpu_baseline(js_sample.head(min(len(js_sample), 20000)))
    cells, dt_plain = cpu_baseline(js_sample)
    settled, dp_cells, dt_disp = cpu_dispatch(js_sample)
    return {"value": round(cells / dt_disp / 1e9, 3), "unit": "GCUPS", "cores": os.cpu_count(), "kind": "port",
            "isa": host_isa(),
            "sample": f"first {len(js_sample)} jobs of the step ({cells} full-DP cells)",
            "form": "production dispatch: ungapped closed form first, scalar ksw_extend2 for the jobs it declines "
                    "(crates/bwa-neon/src/batched.rs:716-775); value = the sample's full-DP cells / time",
            "settled_by_closed_form": round(settled / len(js_sample), 4),
            "dp_cells_evaluated": int(dp_cells),
            "plain_scalar": {"value": round(cells / dt_plain / 1e9, 3), "unit": "GCUPS",
                             "form": "scalar ksw_extend2 on every job"}}


def run_reference(args, rank, world):
    if rank != 0:
        return
    import bwacuda as B

    cores = os.cpu_count() or 1
    n = min(args.jobs, 1_000_000)
    js = B.synth_ext(2, n, seed=0)
    # the full-DP cell count of the sample (the workload's cells, the unit of the metric)
    cells, dt_plain = cpu_baseline(js)
    for _ in range(max(args.warmup, 0)):
        cpu_dispatch(js.head(min(n, 100000)))
    tot_t, settled = 0.0, 0
    for _ in range(args.steps):
        settled, _, dt = cpu_dispatch(js)
        tot_t += dt
    g = cells * args.steps / tot_t / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(g, 3), "unit": "GCUPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(tot_t / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": f"ksw_extend2 read-pair extensions, {n} of the {args.jobs}-job step per sample",
                   "jobs_per_step": n, "parallelism": "host threads"},
        "cpu_baseline": {"value": round(g, 3), "unit": "GCUPS", "cores": cores, "kind": "port", "isa": host_isa(),
                         "sample": f"{n} jobs per step ({cells} full-DP cells), all host threads; the reference's "
                                   "production flow restated (ungapped closed form, then scalar ksw_extend2; the "
                                   "reference is Rust and no Rust toolchain exists on the host)",
                         "settled_by_closed_form": round(settled / n, 4),
                         "plain_scalar": {"value": round(cells / dt_plain / 1e9, 3), "unit": "GCUPS"}},
        "e2e": {"value": round(g, 3), "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_case(args):
    """Small fixed case for ncu captures: two calls of one path, nothing timed."""
    import ctypes as C

    import numpy as np
    import torch

    import bwacuda as B

    ctx = B.Context(0)
    ctx.set_option(B.OPT_GRAPHS, 0)  # plain stream launches (no graph nodes) under the profiler
    if args.case == "op-rates":
        # the instruction-rate microbenchmark: one line per operation (1e9 lane-ops/s); under ncu
        # each launch's smsp__inst_executed / sm__inst_executed_pipe_alu counts per operation
        for name, g in ctx.measure_op_rates().items():
            print(f"{name} {g:.1f}")
        print("alu_peak", round(ctx.measure_alu_peak(), 1))
        ctx.close()
        return
    if args.case in ("ext-batched", "ext-plain", "ext-mixed", "ext-long"):
        if args.case == "ext-long":
            js = long_query_jobs(B, args.jobs, seed=0)
        else:
            js = B.synth_ext(3 if args.case == "ext-mixed" else 2, args.jobs, seed=0)
        js.h0 = js.h0 + args.h0_add
        od, ed, oi, ei = (int(x) for x in args.gaps.split(","))
        sc = ctx.scoring(o_del=od, e_del=ed, o_ins=oi, e_ins=ei)
        ctx.set_option(B.OPT_UNGAPPED, args.ungapped)
        if args.persist_block:
            ctx.set_option(B.OPT_PERSIST_BLOCK, args.persist_block)
        d_seq = torch.from_numpy(js.seq).cuda()
        d_jobs = torch.from_numpy(js.dev_ext_jobs().view(np.uint8)).cuda()
        d_out = torch.zeros(len(js) * 24, dtype=torch.uint8, device="cuda")
        path = B.PATH_PLAIN if args.case == "ext-plain" else B.PATH_BATCHED
        for _ in range(2):
            ctx.extend_device(d_seq.data_ptr(), d_jobs.data_ptr(), len(js), d_out.data_ptr(), sc=sc, path=path)
            ctx.sync()
    elif args.case == "ext-gather":
        # host buffers, batched path fed by the device gather (one chunk per call)
        js = B.synth_ext(2, args.jobs, seed=0)
        ctx.set_option(B.OPT_EXT_PATH, B.PATH_BATCHED)
        ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_DEVICE)
        ctx.set_option(B.OPT_CHUNK_JOBS, args.jobs)
        for _ in range(2):
            ctx.extend_batch(js)
    elif args.case == "global":
        # through the C ABI with the host arrays held across calls, as the timed CIGAR stage
        # (the first call touches the output pages; the second is the one to read)
        js = B.synth_global(args.jobs, seed=0)
        n = len(js)
        gjobs = np.zeros(n, dtype=B.GLOBAL_JOB)
        gjobs["query"] = js.seq.ctypes.data + js.q_off.astype(np.uint64)
        gjobs["target"] = js.seq.ctypes.data + js.t_off.astype(np.uint64)
        gjobs["qlen"], gjobs["tlen"], gjobs["w"] = js.qlen, js.tlen, js.w
        gmat = B.scmat()
        gscore = np.zeros(n, np.int32)
        offs = np.zeros(n + 1, np.uint64)
        words = np.zeros(8 * n, np.uint32)
        for _ in range(2):
            rc = B.lib().bwacuda_ksw_global2_batch(ctx.h, C.c_void_p(gjobs.ctypes.data), n, 5,
                                                   C.c_void_p(gmat.ctypes.data), 6, 1, 6, 1,
                                                   C.c_void_p(gscore.ctypes.data), C.c_void_p(offs.ctypes.data),
                                                   C.c_void_p(words.ctypes.data), len(words))
            if rc != B.OK:
                raise B.BwaCudaError(rc, "bwacuda_ksw_global2_batch")
    elif args.case == "windows":
        # mate rescue with the windows planned, clamped and unpacked on the device
        rw = B.RescueWindows(args.jobs, seed=0)
        ctx.ref_set(rw)
        reqs = rw.requests()
        for _ in range(2):
            ctx.mate_rescue_windows(reqs, minsc=20)
    elif args.case == "retry":
        # run_side's band-doubling loop on the device, starting at w = 20 so a share of the jobs
        # is rejected and re-run at 40
        js = B.synth_ext(2, args.jobs, seed=0)
        js.w = np.full(len(js), 20, dtype=np.int32)
        d_seq = torch.from_numpy(js.seq).cuda()
        d_jobs = torch.from_numpy(js.dev_ext_jobs().view(np.uint8)).cuda()
        d_out = torch.zeros(len(js) * 24, dtype=torch.uint8, device="cuda")
        for _ in range(2):
            ctx.extend_retry_device(d_seq.data_ptr(), d_jobs.data_ptr(), len(js), d_out.data_ptr())
            ctx.sync()
    elif args.case == "serve":
        # the serving loop: mixed requests (extension and rescue jobs) from host buffers, the
        # gather kernel packing each request's slices on the device; the requests are windows
        # of the job pools, as in the timed replay, and the trace runs twice (the second pass
        # reads host memory the first one already mapped)
        pools = ServePools(B, seed=0)
        ctx.server_start(hbm_budget_bytes=1 << 30, max_waves=4)
        sc = ctx.scoring()
        L = B.lib()
        out = np.zeros(64 << 20, np.uint8)
        try:
            for _ in range(2):
                for t in serve_trace(1000.0, 8, seed=0):
                    _, cfg, es, ne, w, rs, nr = t
                    ne, nr = min(ne, args.jobs), min(nr, args.jobs)
                    rid = C.c_uint64()
                    ejp = pools.ext_jobs[cfg].ctypes.data + es * B.EXT_JOB.itemsize
                    rjp = pools.res_jobs.ctypes.data + rs * B.RES_JOB.itemsize
                    rc = L.bwacuda_server_submit_mixed(ctx.h, C.c_void_p(ejp), ne, C.c_void_p(rjp), nr, C.byref(sc),
                                                       w, 5, 100, 20, 1, C.byref(rid))
                    if rc != B.OK:
                        raise B.BwaCudaError(rc, "bwacuda_server_submit_mixed")
                    ns = C.c_int64()
                    rc = L.bwacuda_server_wait(ctx.h, rid.value, C.c_void_p(out.ctypes.data), -1, C.byref(ns))
                    if rc != B.OK:
                        raise B.BwaCudaError(rc, "bwacuda_server_wait")
        finally:
            ctx.server_stop()
    else:
        js = B.synth_rescue(args.jobs, seed=0)
        ctx.set_option(B.OPT_RESCUE_LANES, args.lanes)
        ctx.set_option(B.OPT_RESCUE_PAIR, args.pair)
        ctx.set_option(B.OPT_RESCUE_KERNEL, B.RESCUE_TPJ if args.rescue_kernel == "tpj" else B.RESCUE_AUTO)
        d_seq = torch.from_numpy(js.seq).cuda()
        d_jobs = torch.from_numpy(js.dev_res_jobs().view(np.uint8)).cuda()
        d_out = torch.zeros(len(js) * 28, dtype=torch.uint8, device="cuda")
        for _ in range(2):
            ctx.ksw_align2_device(d_seq.data_ptr(), d_jobs.data_ptr(), len(js), d_out.data_ptr(), minsc=20)
            ctx.sync()
    ctx.close()
    print("ok")


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.case:
        return run_case(args)
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import numpy as np
    import torch

    import bwacuda as B

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    ctx = B.Context(local)
    if args.no_graphs:
        ctx.set_option(B.OPT_GRAPHS, 0)
    n = args.jobs
    # each rank extends its own shard of reads (weak scaling: per-GPU work fixed)
    js = B.synth_ext(2, n, seed=1000 + rank)
    d_seq = torch.from_numpy(js.seq).cuda()
    d_jobs = torch.from_numpy(js.dev_ext_jobs().view(np.uint8)).cuda()
    d_out = torch.zeros(n * 24, dtype=torch.uint8, device="cuda")
    # a dedicated (non-default) stream: the library's kernels and the timing
    # events must be ordered on the same stream
    st = torch.cuda.Stream()
    torch.cuda.set_stream(st)
    stream = st.cuda_stream

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    from bwacuda import shard

    def max_over_ranks(x):
        return shard.max_over_ranks(x, device="cuda")

    def timed_device(path, steps, warmup):
        for _ in range(warmup):
            ctx.extend_device(d_seq.data_ptr(), d_jobs.data_ptr(), n, d_out.data_ptr(), path=path, stream=stream)
        ctx.sync()
        ctx.reset_stats()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(steps):
            ctx.extend_device(d_seq.data_ptr(), d_jobs.data_ptr(), n, d_out.data_ptr(), path=path, stream=stream)
        e1.record(st)
        ctx.sync()
        barrier()
        ms = e0.elapsed_time(e1)
        stt = ctx.stats()
        return ms, stt

    # plain path: one launch per 256k-job chunk, caller order
    plain_res = None
    CH = 262144

    def timed_plain(steps, warmup):
        def one_step():
            for c0 in range(0, n, CH):
                cn = min(CH, n - c0)
                ctx.extend_device(d_seq.data_ptr(), d_jobs.data_ptr() + c0 * 32, cn, d_out.data_ptr() + c0 * 24,
                                  path=B.PATH_PLAIN, stream=stream)
        for _ in range(warmup):
            one_step()
        ctx.sync()
        ctx.reset_stats()
        barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            one_step()
        ctx.sync()
        barrier()
        return (time.perf_counter() - t0) * 1e3, ctx.stats()

    # launch shape of the batched path picked by the autotuner on a sample of this batch (untimed)
    tuning = ctx.autotune_extend(d_seq.data_ptr(), d_jobs.data_ptr(), n)
    with ClockSampler(local) as clk:
        ms_b, st_b = timed_device(B.PATH_BATCHED, args.steps, args.warmup)
    clocks = clk.summary()
    ms_b = max_over_ranks(ms_b)
    cells_step = st_b["ext_cells"] / args.steps
    gcups_b = cells_step * world / (ms_b / args.steps / 1e3) / 1e9
    launches = st_b["kernel_launches"]
    batched_out = d_out.cpu().numpy().view(B.EXT_RES).copy()

    psteps = max(1, min(args.steps, 3))
    ms_p, st_p = timed_plain(psteps, 1)
    ms_p = max_over_ranks(ms_p)
    gcups_p = (st_p["ext_cells"] / psteps) * world / (ms_p / psteps / 1e3) / 1e9
    same = bool(np.array_equal(batched_out, d_out.cpu().numpy().view(B.EXT_RES)))

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        import ctypes

        ctx.set_option(B.OPT_EXT_PATH, B.PATH_BATCHED)
        ctx.set_option(B.OPT_CHUNK_JOBS, args.e2e_chunk)
        # the caller's ExtendJob array (pointers into its own host buffers), built
        # once like a Rust or C caller's; the timed call is the C ABI itself
        host_jobs = ctx._host_jobs(js, B.EXT_JOB)
        host_out = np.zeros(n, dtype=B.EXT_RES)
        mat = B.scmat()
        L = B.lib()

        def call():
            rc = L.bwacuda_extend_batch(ctx.h, ctypes.c_void_p(host_jobs.ctypes.data), n, 5,
                                        ctypes.c_void_p(mat.ctypes.data), 6, 1, 6, 1, 100, 5, 100,
                                        ctypes.c_void_p(host_out.ctypes.data))
            if rc != B.OK:
                raise B.BwaCudaError(rc, "bwacuda_extend_batch")

        seq_bytes = int(js.qlen.astype(np.int64).sum() + js.tlen.astype(np.int64).sum())

        def timed_route(gather):
            ctx.set_option(B.OPT_HOST_GATHER, gather)
            host_out[:] = 0
            for _ in range(max(1, args.warmup)):  # warm-up (staging allocation, first touches)
                call()
            ctx.reset_stats()
            barrier()
            t0 = time.perf_counter()
            esteps = max(1, min(args.steps, 10))
            call_ms = []
            for _ in range(esteps):
                tc = time.perf_counter()
                call()
                call_ms.append(round((time.perf_counter() - tc) * 1e3, 2))
            barrier()
            et = max_over_ranks(time.perf_counter() - t0)
            ste = ctx.stats()
            r = {"value": round(ste["ext_cells"] / esteps * world / (et / esteps) / 1e9, 2), "unit": "GCUPS",
                 "ms_per_step": round(et / esteps * 1e3, 2), "call_ms": call_ms,
                 "bit_identical_to_device_path": bool(np.array_equal(host_out, batched_out))}
            if ste["h2d_bytes"]:
                r["h2d_bytes_per_step"] = int(ste["h2d_bytes"] / esteps)
                r["d2h_bytes_per_step"] = int(ste["d2h_bytes"] / esteps)
            else:
                # device gather: the GPU loads the job array and the sequence slices from host memory
                # and stores the results into the caller's array (no copy engine involved)
                r["h2d_bytes_per_step"] = n * B.EXT_JOB.itemsize + seq_bytes
                r["d2h_bytes_per_step"] = n * B.EXT_RES.itemsize
            return r

        routes = {}
        try:
            routes["device-gather"] = timed_route(B.GATHER_DEVICE)
        except B.BwaCudaError as err:
            if err.code != B.EUNSUPPORTED:
                raise
        routes["host-pack"] = timed_route(B.GATHER_HOST)
        # the same call with the reference's ungapped closed form on (its production flow)
        ctx.set_option(B.OPT_UNGAPPED, 1)
        ug_route = timed_route(B.GATHER_DEVICE if "device-gather" in routes else B.GATHER_HOST)
        ctx.set_option(B.OPT_UNGAPPED, 0)
        ctx.set_option(B.OPT_HOST_GATHER, B.GATHER_AUTO)
        best = "device-gather" if "device-gather" in routes else "host-pack"
        e2e = dict(routes[best])
        e2e["route"] = best
        e2e["routes"] = {k: {"value": v["value"], "ms_per_step": v["ms_per_step"], "call_ms": v["call_ms"]}
                         for k, v in routes.items()}
        e2e.pop("call_ms", None)
        ug_e2e_eq = round(cells_step * world / (ug_route["ms_per_step"] / 1e3) / 1e9, 2)

    # the reference's ungapped-diagonal fast path (opt-in): same results, most clean read-pair
    # jobs settled in closed form before the DP
    ug = None
    if not args.no_e2e:
        ctx.set_option(B.OPT_UNGAPPED, 1)
        ms_u, st_u = timed_device(B.PATH_BATCHED, max(1, min(args.steps, 5)), 2)
        ms_u = max_over_ranks(ms_u) / max(1, min(args.steps, 5))
        ug_same = bool(np.array_equal(batched_out, d_out.cpu().numpy().view(B.EXT_RES)))
        ctx.set_option(B.OPT_UNGAPPED, 0)
        ug = {"ms_per_step": round(ms_u, 3), "jobs_per_s": round(n * world / (ms_u / 1e3), 1),
              "equivalent_gcups": round(cells_step * world / (ms_u / 1e3) / 1e9, 2),
              "dp_cells_per_step": int(st_u["ext_cells"] / max(1, min(args.steps, 5))),
              "identical_to_full_dp": ug_same,
              "note": "BWACUDA_OPT_UNGAPPED: equivalent_gcups = the full DP's cells / this time (the "
                      "reference's production path applies the same fast path)"}

    # run_side's band-doubling loop on the device (bwa's MAX_BAND_TRY = 2), left/right prev
    retry = None
    if not args.no_e2e:
        prev = torch.from_numpy(np.where(np.arange(n) % 2 == 0, -1, js.h0).astype(np.int32)).cuda()
        d_w = torch.zeros(n, dtype=torch.int32, device="cuda")

        def retry_step():
            ctx.extend_retry_device(d_seq.data_ptr(), d_jobs.data_ptr(), n, d_out.data_ptr(), d_w.data_ptr(),
                                    prev.data_ptr(), max_tries=2, stream=stream)

        rsteps = max(1, min(args.steps, 3))
        retry_step()
        ctx.sync()
        ctx.reset_stats()
        barrier()
        t0 = time.perf_counter()
        for _ in range(rsteps):
            retry_step()
        ctx.sync()
        barrier()
        rt = max_over_ranks((time.perf_counter() - t0) / rsteps)
        str_ = ctx.stats()
        retry = {"ms_per_step": round(rt * 1e3, 2), "jobs_per_s": round(n * world / rt, 1),
                 "gcups": round(str_["ext_cells"] / rsteps * world / rt / 1e9, 2),
                 "retried_jobs_per_step": int(str_["ext_retry_jobs"] / rsteps),
                 "note": "bwacuda_extend_retry_device: round 0 at w = 100, rejected jobs again at 200, "
                         "acceptance as run_side (across.rs:1357-1500); host clock around the call "
                         "(one count readback per round)"}
        del prev, d_w

    # roofline: integer-ALU bound (no tensor cores, about 0.03 B of HBM per cell)
    pk, kind = peaks()
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = clocks["sm_mhz"] or pk.get("sm_max_mhz", 2070.0)
    peak_nominal = int_peak_gops(nsm, mhz)
    peak_g = ctx.measure_alu_peak()  # fused add-max instructions per second, measured on this GPU now
    line = {
        "metric": METRIC, "value": round(gcups_b, 2), "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_b / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": f"ksw_extend2 read-pair extensions (2x150 bp reads, w=100), {n} jobs per GPU per step",
                   "jobs_per_step": n * world, "cells_per_step": int(cells_step * world),
                   "parallelism": f"shard{world}", "l2": "inputs larger than L2 (about 2.1 GB per GPU)",
                   "path": "batched: length-sorted buckets, persistent kernels, CUDA graph replay",
                   "tuning": tuning},
        "jobs_per_s": round(n * world / (ms_b / args.steps / 1e3), 1),
        "plain": {"value": round(gcups_p, 2), "unit": "GCUPS", "ms_per_step": round(ms_p / psteps, 3),
                  "note": "one launch per 262144-job chunk, jobs in caller order"},
        "batched_over_plain": round(gcups_b / gcups_p, 3) if gcups_p else None,
        "plain_equals_batched": same,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": dict(alu_roofline(gcups_b / world, OPS_PER_CELL, peak_g, 2),
                         traffic=int(DRAM_BYTES_PER_JOB * n),
                         traffic_unit="bytes per step (ncu capture of all bucket kernels, scaled by jobs)",
                         peak_nominal=round(2 * peak_nominal, 1),
                         note=f"integer ops = GCUPS x {OPS_PER_CELL} ops/cell (minimal fused count) over the whole step "
                              "(the persistent extension kernels hold ~95% of its device time); the read-pair cells "
                              "fit 16-bit lanes, where one DPX instruction does two operations, so peak = 2 x "
                              "bwacuda_measure_alu_peak (a chain-free __viaddmax_s32 loop on every SM, measured in this "
                              "run; frac_32bit_lanes divides by the single-lane peak instead); peak_nominal = 2 x "
                              f"{nsm} SMs x 64 ALU lanes x median SM clock. The {kind} peaks file has HBM and bf16 "
                              "figures only; this path touches ~0.05 B of HBM per cell and no tensor core"),
    }
    if e2e:
        # the host link's roofline: the bytes a step moves over NVLink-C2C at the measured rates
        # (device loads from host memory for the inputs, device stores for the results; the two
        # directions overlap), for the full-DP call and for the production flow (ungapped on)
        link = ctx.measure_host_link(1 << 30)
        hb, db = e2e["h2d_bytes_per_step"], e2e["d2h_bytes_per_step"]
        floor_ms = max(hb / (link["device_read_gbs"] * 1e6), db / (link["device_write_gbs"] * 1e6))
        e2e["link_roofline"] = {
            "bound": "host link", "unit": "GB/s", "measured": {k: round(v, 1) for k, v in link.items()},
            "bytes_per_step": hb + db, "floor_ms": round(floor_ms, 2),
            "achieved": round((hb + db) / (e2e["ms_per_step"] * 1e6), 1),
            "frac_of_floor": round(floor_ms / e2e["ms_per_step"], 4),
            "ungapped_route": {"ms_per_step": ug_route["ms_per_step"] if ug_route else None,
                               "frac_of_floor": round(floor_ms / ug_route["ms_per_step"], 4) if ug_route else None},
            "note": "bwacuda_measure_host_link over 1 GiB of pinned host memory in this run; floor = max(inputs / "
                    "device read rate, results / device write rate)"}
        line["e2e"] = e2e
    if ug:
        line["ungapped_prefilter"] = ug
    if retry:
        line["band_retry"] = retry
    if not args.no_configs:
        line["configs"] = other_configs(args, B, ctx, st, barrier, max_over_ranks, world, rank)
        # the rescue kernel against the same measured ALU peak, at the reference's minimal fused
        # count for a rescue cell (10: max(0, Hd + s), max3, E and F updates, max / argmax)
        for key, opc, lanes, note in (
                ("rescue", RESCUE_OPS_PER_CELL, 2, "byte-range scores: the paired kernel's 16-bit lanes"),
                ("cigar_stage", GLOBAL_OPS_PER_CELL, 2, "the whole host-buffer stage (gather, DP, traceback, CIGAR "
                 "compaction) over its wall time; 16-bit lanes (every job of the workload fits them)"),
                ("long_queries", OPS_PER_CELL, 1, "the best run's kernel on the device (see kernel)")):
            cfg = line["configs"].get(key)
            if cfg:
                lanes = cfg.pop("lanes_per_op", lanes)
                cfg["roofline"] = dict(alu_roofline(cfg["value"] / world, opc, peak_g, lanes), note=note)
    if not args.no_serve and world == 1:
        rates = [float(r) for r in args.serve_rates.split(",") if r]
        line["served"] = serve_bench(B, rates, args.serve_requests, tuning=ctx.tuning())
    if rank == 0:
        # CPU baseline: the oracle port on a bounded sample of the same workload
        sample = js.head(min(n, 400_000))
        cb = cpu_extension_baseline(sample)
        line["cpu_baseline"] = cb
        if ug and e2e:
            # like for like: the reference's production flow on both sides (ungapped closed form,
            # then the DP), the workload's full-DP cells over each side's time
            line["like_for_like"] = {
                "gpu_device_equivalent_gcups": ug["equivalent_gcups"], "gpu_e2e_equivalent_gcups": ug_e2e_eq,
                "cpu_equivalent_gcups": cb["value"],
                "gpu_device_over_cpu": round(ug["equivalent_gcups"] / cb["value"], 2),
                "gpu_e2e_over_cpu": round(ug_e2e_eq / cb["value"], 2),
                "dp_only": {"gpu_device_gcups": round(gcups_b, 2), "gpu_e2e_gcups": e2e["value"],
                            "cpu_plain_scalar_gcups": cb["plain_scalar"]["value"],
                            "gpu_e2e_over_cpu": round(e2e["value"] / cb["plain_scalar"]["value"], 2)},
                "note": "the reference arm (--impl reference) times the production flow; the headline value / e2e "
                        "evaluate every DP cell (no closed form), so the ratio against that arm is conservative"}
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
