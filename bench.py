#!/usr/bin/env python
"""Benchmark: DOCI sigma throughput on the L=32, N=16 Hamiltonian (D = 601,080,390).

One step = one sigma = H x over all D determinants, FP32 storage and
accumulation (the sigma of the mixed-precision Davidson), on a seeded
synthetic FCIDUMP of the benchmark's integral model.  x and sigma are 2.4 GB
each, far larger than the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value          sigma determinants per second (whole job, Gdet/s), device-timed
               with CUDA events on the launching stream, inputs resident in HBM.
e2e            the same metric through the C ABI call on host buffers
               (doci_sigma_host: H2D of x, sigma, D2H of sigma inside the call),
               pinned host memory, wall-clock timed.
roofline       algorithmic bytes per launch (x read 4 B + FP32 diagonal read
               4 B + sigma write 4 B per determinant) / mean launch time,
               against the measured HBM copy bandwidth.
cpu_baseline   the oracle's port of the reference's race-free gather matvec
               (FP64, all host cores) on a bounded sample of determinants.
--impl reference  times that CPU path alone, one bounded sample per step.

With torchrun (N > 1) every rank runs its own replica (the sigma has no
cross-GPU exchange at this size); value sums the ranks' work over the slowest
rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sigma Gdet/s; time to |ΔE|<1e-8 Ha mixed vs FP64 at L=32,N=16; p50/p99"
UNIT = "Gdet/s"


def parse():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--L", type=int, default=32)
    ap.add_argument("--N", type=int, default=16)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--kernel", choices=["auto", "gather", "row1", "rowx", "pair", "tc", "rowff"], default="auto")
    ap.add_argument("--block", type=int, default=1,
                    help="sigma: vectors per step through doci_sigma_block (1 = doci_sigma)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the FP64-accurate sigma (device-resident and end to end) of an FP32 run")
    ap.add_argument("--no-converge", action="store_true", help="skip the time-to-converge measurement")
    ap.add_argument("--converge-repeats", type=int, default=20,
                    help="mixed solves of the L=28 N=14 Hamiltonian for time-to-converge p50/p99 (0 = none)")
    ap.add_argument("--workload", choices=["sigma", "batch", "serve", "solve", "l28-solvers"], default="sigma",
                    help="sigma: the headline sigma benchmark; batch: many Hamiltonians, several roots; "
                         "serve: Poisson request stream through the request server")
    ap.add_argument("--problems", type=int, default=256, help="batch: number of Hamiltonians")
    ap.add_argument("--sequential-sample", type=int, default=64, help="batch: one-at-a-time baseline sample")
    ap.add_argument("--roots", type=int, default=4)
    ap.add_argument("--workers", type=int, default=16)
    ap.add_argument("--requests", type=int, default=2000, help="serve: number of requests")
    ap.add_argument("--rate", type=float, default=20.0, help="serve: Poisson arrival rate, requests/s")
    ap.add_argument("--lmin", type=int, default=None)
    ap.add_argument("--lmax", type=int, default=None)
    ap.add_argument("--max-vec", type=int, default=16, help="DAVIDSON_MAX_VEC of the convergence runs")
    ap.add_argument("--mode", choices=["mixed", "fp64"], default="mixed", help="solve: precision mode")
    ap.add_argument("--max-its", type=int, default=200, help="solve: iteration limit")
    ap.add_argument("--tol", type=float, default=1e-7, help="solve: residual tolerance")
    ap.add_argument("--mixed-tol", type=float, default=1e-4,
                    help="residual that ends the FP32 phase of the time-to-converge run")
    ap.add_argument("--batch-mixed-tol", type=float, default=1e-5,
                    help="batch / serve: residual that ends the FP32 phase of each solve")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload_path(L: int, N: int, seed: int, rank: int, ws: int) -> str:
    from doci_gb300.fcidump import write_synthetic_fcidump
    d = os.environ.get("DOCI_BENCH_CACHE", os.path.join(tempfile.gettempdir(), "doci_bench"))
    os.makedirs(d, exist_ok=True)
    p = os.path.join(d, f"synthetic_L{L}_N{N}_s{seed}.FCIDUMP")
    if rank == 0 and not os.path.exists(p):
        tmp = p + f".tmp{os.getpid()}"
        write_synthetic_fcidump(tmp, L, N, seed)
        os.replace(tmp, p)
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    return p


def max_over_ranks(x: float, ws: int) -> float:
    """The slowest rank's time (replicas: no collective in the data path;
    this is the only cross-rank operation)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_gdets(dets_per_rank: int, steps: int, ws: int, seconds: float) -> float:
    """Whole-job determinants per second: every rank processed its own
    replica's dets_per_rank x steps in at most `seconds`."""
    return dets_per_rank * steps * ws / seconds / 1e9


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid: str | None):
        self.uuid = uuid
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
            if self.uuid:
                cmd += ["-i", self.uuid]
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(cmd, stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                c = [x.strip() for x in line.split(",")]
                if len(c) < 9:
                    continue
                try:
                    sms.append(float(c[1]))
                    mx = float(c[2])
                except ValueError:
                    continue
                for n, v in zip(names, c[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.remove(self.path)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sms)}


def fp64_like_for_like(h, D, dg, torch, steps: int):
    """The FP64-accurate sigma on the same Hamiltonian (the reference computes
    in FP64): device-resident (CUDA events on its stream, after a warm-up) and
    end to end through doci_sigma_host on pinned FP64 host buffers (copies
    inside each call; wall clock over the calls after a warm-up call)."""
    import ctypes as C
    kind, _ = h.sigma_plan(dg.FP64)
    x = torch.randn(D, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(77))
    y = torch.empty_like(x)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    h.sigma_device(x.data_ptr(), y.data_ptr(), dg.FP64, sp)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        h.sigma_device(x.data_ptr(), y.data_ptr(), dg.FP64, sp)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    del x, y
    torch.cuda.empty_cache()
    hx = torch.randn(D, dtype=torch.float64, generator=torch.Generator().manual_seed(6)).pin_memory()
    hy = torch.empty(D, dtype=torch.float64).pin_memory()
    lib = dg.lib()
    assert lib.doci_sigma_host(h.handle, C.c_void_p(hx.data_ptr()), C.c_void_p(hy.data_ptr()), dg.FP64) == 0
    calls = []
    t0 = time.perf_counter()
    for _ in range(steps):
        tc = time.perf_counter()
        assert lib.doci_sigma_host(h.handle, C.c_void_p(hx.data_ptr()), C.c_void_p(hy.data_ptr()), dg.FP64) == 0
        calls.append(time.perf_counter() - tc)
    te = (time.perf_counter() - t0) / steps
    return {"value": round(D / ms / 1e6, 4), "unit": UNIT, "sigma_ms": round(ms, 3),
            "sigma_kernel": KERNEL_NAMES.get(kind, kind), "dtype": "f64 (float-float pair form)" if kind == 9 else "f64",
            "e2e": {"value": round(D / te / 1e9, 4), "unit": UNIT, "ms_per_call": round(te * 1e3, 3),
                    "h2d_bytes_per_step": D * 8, "d2h_bytes_per_step": D * 8,
                    "call": "doci_sigma_host FP64 (C ABI, pinned host buffers)", "steps": steps,
                    "per_call_ms": [round(c * 1e3, 2) for c in calls]}}


def converge_report(h, max_vec: int, mixed_tol: float, threshold: float = 1e-8):
    """Time to |E - E_FP64| < threshold Ha from a handle-ready Hamiltonian:
    the plain FP64 Davidson (whose tightly converged energy is E_FP64) and
    the mixed FP32/FP64 Davidson.  Only FP64-phase iterations of the mixed
    solve count (their energy is an FP64 Rayleigh quotient)."""
    import numpy as np
    common = dict(solver="D", davidson_max_vec=max_vec, davidson_keep=2)
    # E_FP64: the plain FP64 Davidson converged to a residual of 1e-10
    r64, _, t64 = h.solve_trace(tol=1e-10, mode="fp64", max_its=400, **common)
    e_ref = r64["energy"]
    rmx, _, tmx = h.solve_trace(tol=1e-7, mode="mixed", mixed_tol=mixed_tol, max_its=200, **common)

    def first_time(tr, phase_ok):
        for ph, res, e, t in tr:
            if phase_ok(ph) and abs(e - e_ref) < threshold:
                return float(t), float(res)
        return None, None

    tf, _ = first_time(t64, lambda ph: ph == 1)
    tm, _ = first_time(tmx, lambda ph: ph == 1)
    return {"threshold_Ha": threshold, "E_fp64": e_ref, "fp64_s": tf, "mixed_s": tm,
            "fp64_solve_s": float(t64[-1, 3]) if len(t64) else None,
            "mixed_solve_s": float(tmx[-1, 3]) if len(tmx) else None,
            "speedup": (tf / tm) if tf and tm else None,
            "dE_mixed_final": abs(rmx["energy"] - e_ref),
            "fp64_iterations_total": r64["iterations"], "mixed_iterations_fp32": rmx["iterations_fp32"],
            "mixed_iterations_fp64": rmx["iterations"] - rmx["iterations_fp32"],
            "fp64_residual_final": r64["residual"], "fp64_tol": 1e-10, "max_vec": max_vec, "mixed_tol": mixed_tol,
            "note": "wall time from a built Hamiltonian (integrals, tables, diagonal on the device)"}


def converge_repeats(L: int, N: int, seed: int, repeats: int, max_vec: int, mixed_tol: float,
                     threshold: float = 1e-8):
    """p50/p99 of the time to |E - E_FP64| < threshold over `repeats` mixed
    solves of one Hamiltonian (the FP32 pair-form sigma adds with atomics, so
    repeats differ in their last bits and timings), E_FP64 from one FP64
    solve of the same Hamiltonian."""
    import numpy as np
    import doci_gb300 as dg
    common = dict(solver="D", davidson_max_vec=max_vec, davidson_keep=2, max_its=400)
    with dg.Hamiltonian.from_fcidump(workload_path(L, N, seed, 0, 1)) as h:
        r64, _, t64 = h.solve_trace(tol=1e-10, mode="fp64", **common)
        e_ref = r64["energy"]
        hit64 = next((float(t) for ph, _, e, t in t64 if abs(e - e_ref) < threshold), None)
        times, dEs = [], []
        for _ in range(repeats):
            rmx, _, tmx = h.solve_trace(tol=1e-7, mode="mixed", mixed_tol=mixed_tol, **common)
            hit = next((float(t) for ph, _, e, t in tmx if ph == 1 and abs(e - e_ref) < threshold), None)
            if hit is not None:
                times.append(hit)
            dEs.append(abs(rmx["energy"] - e_ref))
    return {"workload": f"L={L} N={N} seed={seed}", "repeats": repeats, "reached": len(times),
            "fp64_s": hit64, "mixed_p50_s": pct(times, 50), "mixed_p99_s": pct(times, 99),
            "mixed_max_s": max(times) if times else None, "dE_final_max": max(dEs) if dEs else None,
            "max_vec": max_vec, "mixed_tol": mixed_tol}


def cpu_sample(path: str, seconds: float, seed: int = 0):
    """Time the oracle's FP64 gather matvec (port of the reference's race-free
    doci_full_matvec, doci.c:314-376, with O(1) prefix-sum neighbour ranks in
    place of the live doci_matvec's prev_bitstring walk, doci.c:164-238 and
    :851-978) on evenly spread determinant chunks, all host cores.

    The sample's rows and their diagonal are prepared once per sample size
    (the diagonal on all host threads) and reused by every later call: only
    the matvec itself is timed and repeated."""
    import numpy as np

    import oracle
    h = oracle.Ham(path, keep_diag=False)
    D = h.D
    x = np.empty(D, dtype=np.float64)
    step = 1 << 24
    pattern = 1.0 / (1.0 + (np.arange(step) % 7))
    for a in range(0, D, step):
        n = min(step, D - a)
        x[a:a + n] = pattern[:n]
    threads = os.cpu_count() or 1
    nchunks = 64
    prepared = {}

    def prepare(total: int):
        # nch evenly spread chunks of `per` determinants (fewer for small spaces)
        total = max(1, min(total, D))
        nch = min(nchunks, total)
        per = max(1, total // nch)
        if (nch, per) not in prepared:
            first = np.array([(c * (D - per)) // max(1, nch - 1) for c in range(nch)], dtype=np.uint64)
            length = np.full(nch, per, dtype=np.uint64)
            diag = np.concatenate([h.diagonal_range(int(f), per) for f in first])
            prepared.clear()  # keep one sample size
            prepared[(nch, per)] = (first, length, diag)
            prepare.count += 1
        return prepared[(nch, per)]

    prepare.count = 0

    def run(total: int):
        first, length, diag = prepare(total)
        t0 = time.perf_counter()
        h.gather_rows(x, first, length, diag, threads)
        dt = time.perf_counter() - t0
        return int(length.sum()), dt

    n0, t0 = run(min(64 * 2048, D))
    rate = n0 / max(t0, 1e-6)
    total = int(min(rate * seconds, D))
    n, dt = run(max(total, min(64 * 2048, D)))
    return {"dets": n, "seconds": dt, "rate": n / dt, "threads": threads, "D": D, "run": run,
            "prepared": lambda: prepare.count}


def pct(v, q):
    import numpy as np
    return float(np.percentile(np.asarray(v), q)) if len(v) else None


def batch_workload(a):
    """Many seeded Hamiltonians (L uniform in [lmin, lmax], N = L // 2), the
    `roots` lowest eigenpairs each, mixed precision; the whole batch in the
    batch engine (lockstep, graph-captured iterations) against one at a time
    through the same engine (a sample spread over the batch)."""
    import numpy as np
    import doci_gb300 as dg
    from doci_gb300.fcidump import raw_integrals
    lmin, lmax = a.lmin or 12, a.lmax or 24
    rng = np.random.default_rng(4)
    Ls = rng.integers(lmin, lmax + 1, size=a.problems)
    t0 = time.perf_counter()
    hams = []
    for i, L in enumerate(Ls):
        one, two = raw_integrals(int(L), 1000 + i)
        hams.append(dg.Hamiltonian.from_integrals(int(L), int(L) // 2, 0.0, one, two))
    t_build = time.perf_counter() - t0
    # the batch engine's sigma tile shape, tuned once per (L, N) shape
    # (process-wide choices), before both the sequential and the batched runs
    t0 = time.perf_counter()
    tuned = {}
    for i, L in enumerate(Ls):
        if int(L) not in tuned:
            tuned[int(L)] = hams[i].engine_autotune(min(8, a.roots))
    t_tune = time.perf_counter() - t0
    opts = dict(nroots=a.roots, tol=1e-5, mode="mixed", mixed_tol=a.batch_mixed_tol,
                max_vec=min(32, max(16, 8 * a.roots)))
    k = min(a.sequential_sample, a.problems)
    idx = np.linspace(0, a.problems - 1, k).astype(int)
    t0 = time.perf_counter()
    seq = [dg.solve_roots(hams[i], **opts) for i in idx]
    t_seq = time.perf_counter() - t0
    t0 = time.perf_counter()
    st, res = dg.batch_solve(hams, **opts)
    t_bat = time.perf_counter() - t0
    same = all(res[i]["energies"] == seq[j]["energies"] for j, i in enumerate(idx))
    dE_alone = max(max(abs(u - v) for u, v in zip(res[i]["energies"], seq[j]["energies"])) for j, i in enumerate(idx))
    lat = [r["end_s"] - r["queued_s"] for r in res]
    for h in hams:
        h.close()
    line = {"metric": "batched solves/s (4 lowest roots, mixed precision)", "value": round(a.problems / t_bat, 3),
            "unit": "solves/s", "n_gpus": 1, "higher_is_better": True, "impl": "ours", "dtype": "f32+f64",
            "data": "synthetic", "status": st, "one_at_a_time": round(k / t_seq, 3),
            "speedup_vs_one_at_a_time": round((a.problems / t_bat) / (k / t_seq), 3),
            "p50_latency_s": pct(lat, 50), "p99_latency_s": pct(lat, 99), "same_alone_and_in_batch": same,
            "max_dE_alone_vs_batch_Ha": dE_alone,
            "converged": int(sum(r["converged"] for r in res)), "build_s": round(t_build, 2),
            "iterations_fp32_mean": float(np.mean([r["iterations_fp32"] for r in res])),
            "iterations_fp64_mean": float(np.mean([r["iterations"] - r["iterations_fp32"] for r in res])),
            "iterations_max": int(max(r["iterations"] for r in res)),
            "autotune_s": round(t_tune, 2), "tile_dets_per_thread": {str(k): v for k, v in sorted(tuned.items())},
            "config": {"workload": f"{a.problems} Hamiltonians, L uniform in {lmin}..{lmax}, N=L//2, "
                                   f"{a.roots} roots", "opts": opts,
                       "sequential_sample": k}}
    print(json.dumps(line), flush=True)


def serve_workload(a):
    """Poisson request stream into the request server (continuous batching):
    per-request seeded integrals, L uniform in [lmin, lmax], N = L // 2 + d,
    d uniform in -2..2, mixed precision to a residual of 1e-6.  Reported:
    solves/s over the stream, p50/p99 latency (queued to done), the server's
    concurrency, and, on a sample of the same requests spread over the
    stream: one-at-a-time solves/s (one worker, each request waited for) and
    |E - E_FP64| against an independent plain FP64 Davidson solve of the
    request (residual 1e-8)."""
    import numpy as np
    import doci_gb300 as dg
    from doci_gb300.fcidump import raw_integrals
    lmin, lmax = a.lmin or 16, a.lmax or 30
    rng = np.random.default_rng(7)
    gaps = rng.exponential(1.0 / a.rate, size=a.requests)
    shapes = []
    for i in range(a.requests):
        L = int(rng.integers(lmin, lmax + 1))
        N = max(1, min(L - 1, L // 2 + int(rng.integers(-2, 3))))
        shapes.append((L, N))
    opts = dict(nroots=1, tol=1e-6, mode="mixed", mixed_tol=a.batch_mixed_tol, max_its=400)
    ints = [raw_integrals(L, 2000 + i) for i, (L, N) in enumerate(shapes)]  # made before the stream starts
    tickets, conc = [], []
    with dg.Server(workers=a.workers, **opts) as srv:
        t0 = time.perf_counter()
        at = 0.0
        for i, ((L, N), g) in enumerate(zip(shapes, gaps)):
            at += g
            one, two = ints[i]
            wait = at - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            tickets.append(srv.submit(L, N, one, two))
            conc.append(srv.stats()["running"])
        res = [srv.wait(t) for t in tickets]
        span = time.perf_counter() - t0
    lat = [r["end_s"] - r["queued_s"] for r in res]
    del tickets
    # sample of the stream for the one-at-a-time and FP64 comparisons
    k = min(a.sequential_sample, a.requests)
    idx = np.linspace(0, a.requests - 1, k).astype(int)
    t_seq = 0.0
    with dg.Server(workers=1, **opts) as one_srv:
        for i in idx:
            L, N = shapes[i]
            one, two = ints[i]
            t1 = time.perf_counter()
            one_srv.wait(one_srv.submit(L, N, one, two))
            t_seq += time.perf_counter() - t1
    dE, dE_by_L = [], {}
    for i in idx:
        L, N = shapes[i]
        one, two = ints[i]
        with dg.Hamiltonian.from_integrals(L, N, 0.0, one, two) as h:
            r64, _ = h.solve(solver="D", tol=1e-8, max_its=1000, davidson_max_vec=30, davidson_keep=2, mode="fp64")
        d = abs(res[i]["energies"][0] - r64["energy"])
        dE.append(d)
        dE_by_L[L] = max(dE_by_L.get(L, 0.0), d)
    line = {"metric": "serving p50/p99 latency and solves/s (Poisson arrivals)", "value": round(a.requests / span, 3),
            "unit": "solves/s", "n_gpus": 1, "higher_is_better": True, "impl": "ours", "dtype": "f32+f64",
            "data": "synthetic", "p50_latency_s": pct(lat, 50), "p99_latency_s": pct(lat, 99),
            "max_latency_s": max(lat), "span_s": round(span, 2), "offered_rate": a.rate, "requests": a.requests,
            "ok": int(sum(r["status"] == 0 for r in res)), "converged": int(sum(r["converged"] for r in res)),
            "residual_max": max(r["residuals"][0] for r in res),
            "running_at_submit": {"p50": pct(conc, 50), "max": max(conc)},
            "one_at_a_time": {"solves_per_s": round(k / t_seq, 3), "sample": k},
            "speedup_vs_one_at_a_time": round((a.requests / span) / (k / t_seq), 3),
            "dE_vs_fp64": {"max_Ha": max(dE), "median_Ha": pct(dE, 50), "sample": k,
                           "max_by_L": {str(L): v for L, v in sorted(dE_by_L.items())},
                           "reference": "independent plain FP64 Davidson of the same request, residual 1e-8"},
            "config": {"workload": f"{a.requests} requests, L uniform in {lmin}..{lmax}, N=L//2+-2, "
                                   f"Poisson {a.rate}/s, workers={a.workers}", "opts": opts}}
    print(json.dumps(line), flush=True)


KERNEL_NAMES = {1: "gather", 3: "row1", 4: "rowx", 6: "pair", 8: "tc", 9: "rowff"}


def solve_workload(a):
    """One Davidson solve of the sigma workload's Hamiltonian through the
    public solve_trace: iterations, energy and wall time (a profiling target
    for the solver's vector passes)."""
    import doci_gb300 as dg
    path = workload_path(a.L, a.N, a.seed, 0, 1)
    with dg.Hamiltonian.from_fcidump(path) as h:
        r, _, tr = h.solve_trace(solver="D", davidson_max_vec=a.max_vec, davidson_keep=2, max_its=a.max_its,
                                 tol=a.tol, mode=a.mode, mixed_tol=a.mixed_tol)
    line = {"metric": "Davidson solve wall time", "value": float(tr[-1, 3]) if len(tr) else None, "unit": "s",
            "higher_is_better": False, "impl": "ours", "energy": r["energy"], "residual": r["residual"],
            "iterations": r["iterations"], "iterations_fp32": r["iterations_fp32"],
            "config": {"workload": f"Davidson L={a.L} N={a.N} seed={a.seed} mode={a.mode} max_vec={a.max_vec} "
                                   f"tol={a.tol} mixed_tol={a.mixed_tol} max_its={a.max_its}"}}
    print(json.dumps(line), flush=True)


def l28_solvers_workload(a):
    """The plain FP64 GPU Davidson (DAVIDSON_MAX_VEC 30, DAVIDSON_KEEP 2, TOL
    1e-8, HF start) and CGP (MAX_ITS 40) on the L=28, N=14 Hamiltonian (seed
    2), wall time from a built Hamiltonian, beside the reference executable's
    wall times for the same runs recorded in tests/golden/golden.json (its
    host and thread count stated there)."""
    import doci_gb300 as dg
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        gold = json.load(f)["cases"]["synthetic_L28_N14_s2"]
    path = workload_path(28, 14, 2, 0, 1)
    t0 = time.perf_counter()
    with dg.Hamiltonian.from_fcidump(path) as h:
        t_build = time.perf_counter() - t0
        t0 = time.perf_counter()
        rd, _ = h.solve(solver="D", tol=1e-8, max_its=1000, davidson_max_vec=30, davidson_keep=2, mode="fp64")
        t_d = time.perf_counter() - t0
        t0 = time.perf_counter()
        rc, _ = h.solve(solver="CGP", tol=1e-8, max_its=40)
        t_c = time.perf_counter() - t0
    ref_d, ref_c = gold["D_exe"], gold["CGP_exe"]
    line = {"metric": "FP64 Davidson / CGP solve wall time, L=28 N=14", "unit": "s", "higher_is_better": False,
            "impl": "ours", "n_gpus": 1, "dtype": "f64", "data": "synthetic",
            "davidson": {"gpu_s": round(t_d, 3), "iterations": rd["iterations"], "energy": rd["energy"],
                         "sigma_s": round(rd.get("sigma_seconds", 0.0), 3),
                         "reference_s": ref_d["wall_s"], "reference_iterations": len(ref_d["trace"]),
                         "reference_energy": ref_d["energy_printed"],
                         "speedup": round(ref_d["wall_s"] / t_d, 1)},
            "cgp": {"gpu_s": round(t_c, 3), "iterations": rc["iterations"], "energy": rc["energy"],
                    "reference_s": ref_c["wall_s"], "reference_iterations": len(ref_c["trace"]) - 1,
                    "reference_energy": ref_c["energy_printed"], "speedup": round(ref_c["wall_s"] / t_c, 1)},
            "reference_host": gold["host"], "build_s": round(t_build, 2),
            "config": {"workload": "DOCI L=28 N=14 D=40116600 seed=2, Davidson MAX_VEC 30 KEEP 2 TOL 1e-8; "
                                   "CGP MAX_ITS 40"}}
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    ws, rank, local = dist_env()
    if a.impl == "reference":
        return reference_arm(a, ws, rank)
    if a.workload == "batch":
        return batch_workload(a)
    if a.workload == "serve":
        return serve_workload(a)
    if a.workload == "solve":
        return solve_workload(a)
    if a.workload == "l28-solvers":
        return l28_solvers_workload(a)
    import numpy as np
    import torch
    import doci_gb300 as dg
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    path = workload_path(a.L, a.N, a.seed, rank, ws)
    prec = dg.FP32 if a.precision == "fp32" else dg.FP64
    tdt = torch.float32 if prec == dg.FP32 else torch.float64
    esize = 4 if prec == dg.FP32 else 8
    h = dg.Hamiltonian.from_fcidump(path)
    h.set_sigma_kernel(a.kernel)
    D = h.D
    g = torch.Generator(device="cuda").manual_seed(1234 + rank)
    nv = max(1, a.block)
    x = torch.randn(D * nv, dtype=tdt, device="cuda", generator=g)
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    if nv > 1:  # a block of vectors per step: the device-timed figure only
        a.no_e2e = a.no_converge = True

    plan_kind, plan_launches = h.sigma_plan(prec)
    # kernel launches of one step: doci_sigma's plan, or the block sigma's groups of up to 4 vectors
    launches_per_step = plan_launches if nv == 1 else (nv + 3) // 4

    def step():
        if nv == 1:
            h.sigma_device(x.data_ptr(), y.data_ptr(), prec, sptr)
        else:
            h.sigma_block_device(x.data_ptr(), D, y.data_ptr(), D, nv, prec, sptr)
    # a dedicated stream: the sigma launches and the CUDA events share it
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    assert sptr != 0
    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(torch.cuda.current_device()).uuid)
    except Exception:
        pass
    clocks = ClockSampler(uuid)
    clocks.start()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps + 1)]
    ev[0].record(stream)
    for k in range(a.steps):
        step()
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clk = clocks.stop()
    per_launch = [ev[k].elapsed_time(ev[k + 1]) * 1e-3 for k in range(a.steps)]
    total = max_over_ranks(ev[0].elapsed_time(ev[a.steps]) * 1e-3, ws)
    value = replica_gdets(D * nv, a.steps, ws, total)
    mean_launch = statistics.mean(per_launch)
    bytes_alg = D * (2 * nv + 1) * esize  # x and sigma per vector, the diagonal once
    peaks, peak_kind = measured_peaks()
    achieved = bytes_alg / mean_launch / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", f"sigma_{a.precision}_L{a.L}_N{a.N}.json")
    limiter = None
    if os.path.exists(prof):
        with open(prof) as f:
            pj = json.load(f)
        traffic = pj.get("dram_bytes_per_launch")
        limiter = {"what": pj.get("limiter"), **pj.get("same_kernel_L28_ncu_full", {})} if pj.get("limiter") else None
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": traffic,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
                "limiter": limiter, "bytes_per_det": (2 * nv + 1) * esize, "mean_launch_ms": round(mean_launch * 1e3, 4)}
    e2e = None
    if not a.no_e2e:
        hx = torch.randn(D, dtype=tdt, generator=torch.Generator().manual_seed(5)).pin_memory()
        hy = torch.empty(D, dtype=tdt).pin_memory()
        import ctypes as C
        lib = dg.lib()
        st = lib.doci_sigma_host(h.handle, C.c_void_p(hx.data_ptr()), C.c_void_p(hy.data_ptr()), prec)
        assert st == 0, st
        if ws > 1:
            dist.barrier()
        calls = []
        t0 = time.perf_counter()
        for _ in range(a.e2e_steps):
            tc = time.perf_counter()
            st = lib.doci_sigma_host(h.handle, C.c_void_p(hx.data_ptr()), C.c_void_p(hy.data_ptr()), prec)
            calls.append(time.perf_counter() - tc)
            assert st == 0, st
        te = max_over_ranks(time.perf_counter() - t0, ws)
        e2e = {"value": round(replica_gdets(D, a.e2e_steps, ws, te), 4), "unit": UNIT,
               "h2d_bytes_per_step": D * esize, "d2h_bytes_per_step": D * esize,
               "call": "doci_sigma_host (C ABI, pinned host buffers)", "steps": a.e2e_steps,
               "per_call_ms": [round(c * 1e3, 2) for c in calls]}
    fp64 = None
    if prec == dg.FP32 and nv == 1 and not a.no_fp64 and rank == 0:
        fp64 = fp64_like_for_like(h, D, dg, torch, a.e2e_steps)
    conv = None
    if not a.no_converge and rank == 0:
        del x, y
        torch.cuda.empty_cache()
        conv = converge_report(h, a.max_vec, a.mixed_tol)
        if a.converge_repeats > 0:
            conv["repeats_L28"] = converge_repeats(28, 14, 2, a.converge_repeats, a.max_vec, a.mixed_tol)
    cpu = None
    if rank == 0 and ws == 1 and not a.no_cpu_baseline:
        s = cpu_sample(path, a.cpu_seconds)
        cpu = {"value": round(s["rate"] / 1e9, 6), "unit": UNIT, "cores": s["threads"], "kind": "port",
               "sample": f"{s['dets']} of {s['D']} determinants in 64 evenly spread chunks, FP64 gather form "
                         f"of the reference's doci_full_matvec (oracle/doci_oracle.c), {s['seconds']:.1f} s"}
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": round(total / a.steps * 1e3, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec == dg.FP32 else "f64",
                "data": "synthetic (seeded FCIDUMP of the benchmark integral model)",
                "config": {"workload": f"DOCI sigma L={a.L} N={a.N} D={D} seed={a.seed}"
                                       + (f" block of {nv} vectors" if nv > 1 else ""),
                           "block": nv,
                           "L": a.L, "N": a.N, "D": D, "seed": a.seed, "precision": a.precision,
                           "l2": "inputs larger than L2 (x and sigma are D*4 B = %.2f GB each)" % (D * esize / 1e9),
                           "parallelism": f"replicas x{ws}"},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": a.steps * launches_per_step,
                "sigma_kernel": KERNEL_NAMES.get(plan_kind, plan_kind),
                "clocks": clk, "time_to_converge": conv, "fp64": fp64, "impl": "ours"}
        print(json.dumps(line), flush=True)
    h.close()
    if ws > 1:
        dist.destroy_process_group()


def reference_arm(a, ws, rank):
    """The reference's CPU path on this host's cores: the oracle port of its
    gather matvec (the reference is C with no installable package, and its
    compiled build cannot be made where the reference checkout is absent).
    Each step is one bounded sample of the workload, sized so that all
    warm-up and timed steps take about 150 s; the sample is prepared once."""
    if rank != 0:
        return
    t_start = time.perf_counter()
    path = workload_path(a.L, a.N, a.seed, 0, 1)
    budget = max(0.05, min(a.cpu_seconds, 150.0 / max(1, a.steps + a.warmup)))
    s = cpu_sample(path, budget)
    run = s["run"]
    for _ in range(a.warmup):
        run(s["dets"])
    times = []
    for _ in range(a.steps):
        n, dt = run(s["dets"])
        times.append(dt)
    total = sum(times)
    value = s["dets"] * a.steps / total / 1e9
    line = {"metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": 0, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": round(total / a.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"DOCI sigma L={a.L} N={a.N} D={s['D']} seed={a.seed}",
                       "L": a.L, "N": a.N, "D": s["D"], "seed": a.seed, "precision": "fp64",
                       "sample": "bounded CPU sample per step (cpu_baseline.sample)"},
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": s["threads"], "kind": "port",
                             "sample": f"{s['dets']} determinants per step in 64 evenly spread chunks, FP64 "
                                       "gather form of the reference's doci_full_matvec (doci.c:314-376) with "
                                       "O(1) neighbour ranks (oracle/doci_oracle.c), not the live doci_matvec "
                                       "+ prev_bitstring walk (doci.c:164-238, :851-978)"},
            "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "sample_preparations": s["prepared"](), "wall_s": round(time.perf_counter() - t_start, 1)}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
