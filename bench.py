#!/usr/bin/env python
"""Benchmark of the Pauli-sum product H psi on GB300 (one JSON line).

Workload (default): the 26-qubit Jordan-Wigner-style operator -- 8,000 pair
terms (X/Y at i and j, Z strictly between) + 2,000 pure-Z terms on 1-4
qubits, coefficients ~ N(0, 0.1), seed 20262 -- applied to one unit-norm
2^26-amplitude state.  A step is one H psi over the whole state.
Metric: term*amp/s = (input terms) * 2^n * states / seconds.

Arms:
  (default)          our sm_103a kernels through libqrusty_gpu's C ABI.
                     `value` = compensated-complex64 kernel, device-resident
                     inputs; `e2e` = the C-ABI host entry (qr_apply_host) with
                     pinned host buffers, copies included; the plain complex128
                     kernel is reported beside it.
  --impl reference   the reference's CPU method (rowwise CSR build + chunked
                     CSR*vector, restated in C in oracle/) on all host cores, on
                     a bounded row sample of the same workload.

Multi-GPU (torchrun, N > 1): replicas -- every rank applies the operator to
its own state (weak scaling, no data-path collective); max time over ranks.

The default line also carries, under "secondary", compact measurements of
the other configurations (each on its own CUDA-event clock, each checked
against the FP64 oracle): chain, grad, batch, csr and spmv below
(--no-secondary leaves them out).

Secondary workloads (--workload, one JSON line each, 1 GPU):
  chain   the 22-qubit TFIM+XXZ chain (85 terms), same metric.
  batch   256 uneven operators (n 10-20, 50-5,000 terms) x 8 complex64 states
          in ONE graph-replayed persistent launch, against one complex128
          launch per operator.  term*amp/s summed over operators and states.
  grad    y = H(c) psi, L = Re<y, w>, backward to c (2,000 terms) and psi
          (n = 20, complex64): one training step per step.
  vec     the eigensolver-loop helpers (axpby, axpy, ax, precond2) over 2^26
          complex128 / complex64 elements: GB/s against the HBM peak.
  csr     device CSR build (indptr, indices, data) of the chain at n = 22:
          bytes written per second, and the oracle's CPU build beside it.
  spmv    CSR * vector (qr_csr_spmv) on that matrix: 24 B per stored entry
          plus the gathered vector reads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Pauli-sum H·ψ term·amp/s & %HBM peak; c64-compensated vs c128 at stated rel err"
UNIT = "term*amp/s"
L2_BYTES = 129 * 1024 * 1024


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------------------- helpers
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, device=None) -> float:
    """Largest x over the ranks of the default process group (x itself when
    there is none): a step's time is the slowest rank's."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world_size: int, units_per_rank: float, seconds: float) -> float:
    """Aggregate throughput of replicas: every rank processes units_per_rank
    in the same (max-over-ranks) time."""
    return world_size * units_per_rank / seconds


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


_FP64 = {}


def fp64_peak():
    """Measured FP64 FMA rate of this GPU (TFLOP/s, 2 flops per DFMA) from
    libqrusty_probe.so's chain kernel, or None when the probe is unavailable."""
    if "v" not in _FP64:
        _FP64["v"] = None
        try:
            import ctypes as C
            from qrusty_gb300 import build as B
            L = C.CDLL(B.PROBE)
            L.qr_probe_fp64_peak.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_float)]
            L.qr_probe_fp64_peak.restype = C.c_int
            best = 0.0
            for _ in range(3):
                tf, ms = C.c_double(), C.c_float()
                if L.qr_probe_fp64_peak(20000, C.byref(tf), C.byref(ms)) == 0:
                    best = max(best, tf.value)
            _FP64["v"] = best or None
        except Exception as e:  # reported as absent, never guessed
            log("fp64 probe unavailable: %s" % e)
    return _FP64["v"]


# Sources whose change invalidates a recorded DRAM-traffic figure: the apply
# kernels, their shared types and the plan builder.
TRAFFIC_SOURCES = ("qrusty_gb300/csrc/qr_apply.cu", "qrusty_gb300/csrc/qr_common.cuh",
                   "qrusty_gb300/csrc/qr_host.cu")


def source_hash() -> str:
    import hashlib
    h = hashlib.sha256()
    for rel in TRAFFIC_SOURCES:
        with open(os.path.join(ROOT, rel), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def ncu_traffic():
    """DRAM bytes per launch of the c64c apply kernel from the committed ncu
    summary (profiles/ncu_traffic.json).  Used only when it was captured from
    the same kernel sources as this run (source hash), else None."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
    except Exception:
        return None
    return d if d.get("source_sha256_16") == source_hash() else None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev_index: int):
        self.dev = dev_index
        self.proc = None
        self.path = None

    def start(self):
        import tempfile
        fd, self.path = tempfile.mkstemp(prefix="qr_clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        load = sorted(sm)
        return {"sm_mhz": statistics.median(load) if load else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ----------------------------------------------------------------------------- workloads
def make_terms(args):
    from qrusty_gb300 import workloads as W
    if args.workload == "jw":
        t = W.cfg2(n=args.n, npair=args.pairs, nz=args.zterms)
        desc = ("jordan-wigner n=%d: %d pair terms + %d pure-Z terms (seed %d)"
                % (args.n, args.pairs, args.zterms, W.SEED0 + 2))
    elif args.workload == "chain":
        t, _ = W.cfg1(with_state=False, n=args.n)
        desc = "tfim+xxz open chain n=%d, %d terms (seed %d)" % (args.n, t.T, W.SEED0 + 1)
    else:
        raise SystemExit("unknown workload %s" % args.workload)
    return t, desc


# ----------------------------------------------------------------------------- CPU arm
def cpu_reference(t, rows, reps, nthreads):
    """Reference method on host cores: rowwise CSR build of a row sample,
    then chunked CSR*vector (1024-row chunks) over it."""
    from oracle import oracle as O
    O.build()
    N = 1 << t.n
    rng = np.random.default_rng(5)
    psi = np.empty(N, dtype=np.complex128)
    psi.real = rng.standard_normal(N)
    psi.imag = rng.standard_normal(N)
    cp = O.make_params(t.phase, t.coeff)
    t0 = time.perf_counter()
    ip, ij, d = O.csr_build(t.n, t.x, t.z, cp, step=1024, nthreads=nthreads, rows=(0, rows))
    t_build = time.perf_counter() - t0
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        O.spmv(ip, ij, d, psi, step=1024, nthreads=nthreads)
        times.append(time.perf_counter() - t0)
    return t_build, times


def cpu_sample_text(rows, n, t_build, ms_spmv, nthreads):
    """What the CPU figure is: qrusty's method on a row sample, CSR*vector
    timed with the CSR already built; the build is excluded although one
    H psi from scratch costs build + CSR*vector."""
    full = t_build * (1 << n) / rows
    return ("rows [0, %d) of 2^%d on %d thread(s): CSR*vector %.2f ms per step, CSR prebuilt "
            "(the most favourable reading for the CPU); the sample's CSR build (make_row, "
            "1024-row chunks) took %.2f s and is excluded -- %.0f s extrapolated to all rows"
            % (rows, n, nthreads, ms_spmv, t_build, full))


def cpu_one_thread(t, rows):
    """The same method on one host thread (a smaller row sample)."""
    t_build, times = cpu_reference(t, rows, 3, 1)
    ms = 1e3 * statistics.median(times)
    return {"value": t.T * rows / (ms / 1e3), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": cpu_sample_text(rows, t.n, t_build, ms, 1)}


def run_reference_arm(args, t, desc):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    rows = args.cpu_rows
    t_build, times = cpu_reference(t, rows, args.warmup + args.steps, nthreads)
    timed = times[args.warmup:]
    ms = 1e3 * statistics.mean(timed)
    units = t.T * rows
    value = units / (ms / 1e3)
    sample = cpu_sample_text(rows, t.n, t_build, ms, nthreads)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": desc, "n": t.n, "terms": t.T, "states": 1},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "csr_build_s": t_build,
        "cpu_baseline_1thread": cpu_one_thread(t, max(1024, rows // 8)),
    }
    print(json.dumps(out), flush=True)


# ----------------------------------------------------------------------------- GPU arm
def run_gpu_arm(args, t, desc):
    import torch
    from qrusty_gb300 import PauliOperator, _lib
    from qrusty_gb300 import workloads as W

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    n, N, T = t.n, 1 << t.n, t.T
    op = PauliOperator(n, t.x, t.z, t.phase, t.coeff)
    info = op.info()
    P = W.alg_blocks(t, 13)
    g = torch.Generator(device=dev).manual_seed(1000 + rank)
    psi128 = torch.complex(torch.randn(N, device=dev, dtype=torch.float64, generator=g),
                           torch.randn(N, device=dev, dtype=torch.float64, generator=g))
    psi128 /= torch.linalg.vector_norm(psi128)
    psi64 = psi128.to(torch.complex64)
    y64 = torch.empty_like(psi64)
    y128 = torch.empty_like(psi128)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        barrier()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        l0 = _lib.launch_count()
        e_all0 = torch.cuda.Event(enable_timing=True)
        e_all1 = torch.cuda.Event(enable_timing=True)
        e_all0.record(stream)
        for a, b in evs:
            a.record(stream)
            fn()
            b.record(stream)
        e_all1.record(stream)
        barrier()
        launches = _lib.launch_count() - l0
        per = [a.elapsed_time(b) for a, b in evs]
        total = max_over_ranks(e_all0.elapsed_time(e_all1), dev)
        return total, per, launches

    clocks = ClockSampler(dev.index if dev.index is not None else 0)

    # --- compensated complex64 (headline)
    f64c = lambda: op.apply(psi64, out=y64)
    clocks.start() if rank == 0 and not args.quick else None
    tot64, per64, launches = timed(f64c, args.steps, args.warmup)
    clk = clocks.stop() if rank == 0 and not args.quick else None
    op.sync_check()
    ms64 = tot64 / args.steps

    # --- plain complex128
    s128 = max(1, args.steps // 10) if not args.quick else 1
    f128 = lambda: op.apply(psi128, out=y128)
    tot128, per128, _ = timed(f128, s128, max(1, min(args.warmup, 3)))
    op.sync_check()
    ms128 = tot128 / s128

    # --- accuracy at full size (outside the timed region): c64c against c128
    # over the whole state, and both against the FP64 oracle on a block of
    # 65,536 rows (16 output tiles, unaligned start)
    rel64 = float(torch.linalg.vector_norm(y64.to(torch.complex128) - y128)
                  / torch.linalg.vector_norm(y128))
    rel_rows = None
    if rank == 0 and not args.quick and not args.no_cpu:
        rel_rows = oracle_rows_errors(t, psi128, psi64, y128, y64)

    # --- end to end through the C-ABI host entry (pinned host buffers)
    e2e = None
    if not args.quick:
        h_in = torch.empty(N, dtype=torch.complex64, pin_memory=True)
        h_out = torch.empty(N, dtype=torch.complex64, pin_memory=True)
        h_in.copy_(psi64.cpu())
        a_in, a_out = h_in.numpy(), h_out.numpy()
        for _ in range(max(3, min(args.warmup, 5))):
            op.apply(a_in, out=a_out)
        e_steps = max(3, args.steps // 5)
        barrier()
        t0 = time.perf_counter()
        for _ in range(e_steps):
            op.apply(a_in, out=a_out)
        barrier()
        e_ms = max_over_ranks(1e3 * (time.perf_counter() - t0) / e_steps, dev)
        e2e = {"value": whole_job_rate(ws, T * N, e_ms / 1e3), "unit": UNIT, "ms_per_step": e_ms,
               "h2d_bytes_per_step": N * 8, "d2h_bytes_per_step": N * 8,
               "path": "qr_apply_host (C ABI), pinned host buffers",
               "ratio_to_kernel": e_ms / ms64}
        del h_in, h_out, a_in, a_out
        if ws == 1:
            # four states per call: the copy of state s + 1 overlaps the
            # kernel on state s, so only one copy is exposed
            ns4 = 4
            h4i = torch.empty(ns4 * N, dtype=torch.complex64, pin_memory=True)
            h4o = torch.empty(ns4 * N, dtype=torch.complex64, pin_memory=True)
            for k in range(ns4):
                h4i[k * N:(k + 1) * N].copy_(psi64.cpu())
            b_in, b_out = h4i.numpy(), h4o.numpy()
            for _ in range(2):
                op.apply(b_in, out=b_out)
            t0 = time.perf_counter()
            for _ in range(3):
                op.apply(b_in, out=b_out)
            e4 = 1e3 * (time.perf_counter() - t0) / 3
            e2e["four_states"] = {"ms_per_call": e4, "value": T * N * ns4 / (e4 / 1e3),
                                  "ratio_to_kernel": e4 / (ns4 * ms64),
                                  "h2d_bytes_per_call": ns4 * N * 8,
                                  "d2h_bytes_per_call": ns4 * N * 8}
            del h4i, h4o, b_in, b_out

    if rank != 0:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    hbm, peak_kind = peaks()
    alg64 = (P + 1) * N * 8
    alg128 = (P + 1) * N * 16
    mean_launch64 = statistics.mean(per64) / 1e3
    mean_launch128 = statistics.mean(per128) / 1e3
    ach64 = alg64 / mean_launch64 / 1e9
    ach128 = alg128 / mean_launch128 / 1e9
    tr = ncu_traffic()
    traffic = None
    if tr and tr.get("workload") == desc:
        traffic = tr.get("bytes_per_launch")
    rel_err = {"c64c_vs_c128_full": rel64}
    if rel_rows:
        rel_err.update(rel_rows)
    out = {
        "metric": METRIC, "value": whole_job_rate(ws, T * N, ms64 / 1e3), "unit": UNIT,
        "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms64,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64c (fp32 + two-sum)", "data": "synthetic",
        "config": {"workload": desc, "n": n, "terms": T, "states_per_gpu": 1,
                   "groups": int(info["ngroups"]), "merged_strings": int(info["nmerged"]),
                   "partner_tiles_P": P, "tile_bits": int(info["tile_bits"]),
                   "l2": "inputs 2^%d amplitudes (%d MiB c64) > L2 129 MB; no flush"
                         % (n, (N * 8) >> 20),
                   "parallelism": "replicas x%d" % ws},
        "roofline": {"bound": "hbm", "achieved": ach64, "peak": hbm, "unit": "GB/s",
                     "frac": ach64 / hbm, "traffic": traffic,
                     "alg_bytes_per_launch": alg64,
                     "alg_bytes_rule": "(P+1)*2^n*8, P=%d distinct x>>13" % P,
                     "b_group_bytes": (int(info["ngroups"]) + 1) * N * 8,
                     "b_group_rule": "(G+1)*2^n*8: one gather pass per distinct x mask",
                     "peak_source": peak_kind},
        "c128": c128_line(ws, T, N, int(info["ngroups"]), ms128, s128, ach128, hbm, alg128),
        "speedup_c64c_vs_c128": ms128 / ms64,
        "rel_err": rel_err,
        "e2e": e2e,
        "clocks": clk,
        "gpu_launches": int(launches),
        "device": torch.cuda.get_device_name(dev),
    }
    if not args.no_cpu and not args.quick and ws == 1:
        nthreads = os.cpu_count() or 1
        t_build, times = cpu_reference(t, args.cpu_rows, 4, nthreads)
        ms_cpu = 1e3 * statistics.median(times[1:])
        cpu_val = T * args.cpu_rows / (ms_cpu / 1e3)
        out["cpu_baseline"] = {
            "value": cpu_val, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": cpu_sample_text(args.cpu_rows, n, t_build, ms_cpu, nthreads)}
        out["cpu_baseline_1thread"] = cpu_one_thread(t, max(1024, args.cpu_rows // 8))
    del y64, y128, psi64, psi128
    if not args.quick and not args.no_secondary and ws == 1:
        out["secondary"] = run_secondary(args)
    print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def c128_line(ws, T, N, G, ms128, steps, ach128, hbm, alg128):
    """The plain complex128 kernel: 4 DFMA (8 flops) per amplitude and x
    group, so GB300's FP64 rate bounds it long before HBM does; the fraction
    is against the FP64 rate measured on this GPU by the probe kernel."""
    flops = 8.0 * N * G
    tf = flops / (ms128 / 1e3) / 1e12
    peak = fp64_peak()
    d = {"value": whole_job_rate(ws, T * N, ms128 / 1e3), "ms_per_step": ms128, "steps": steps,
         "fp64_tflops": tf, "fp64_peak_measured_tflops": peak,
         "fp64_frac_of_measured": (tf / peak) if peak else None,
         "fp64_floor_ms": (flops / (peak * 1e12) * 1e3) if peak else None,
         "hbm_floor_ms": alg128 / (hbm * 1e9) * 1e3,
         "hbm_achieved_gbs": ach128, "hbm_frac": ach128 / hbm,
         "note": "FP64-bound: >= 70% of HBM is out of reach for native FP64 on GB300"}
    return d


def oracle_rows_errors(t, psi128, psi64, y128, y64, rows=65536):
    """Relative errors of both kernels against the FP64 oracle on one block of
    rows: c128 and c64c on their own inputs, and c64c against the oracle on
    the FP64 state before its rounding to complex64."""
    from oracle import oracle as O
    O.build()
    N = 1 << t.n
    lo = ((0x2A5B << 12) + 777) % max(1, N - rows) if N > rows else 0
    hi = min(N, lo + rows)
    cp = O.make_params(t.phase, t.coeff)
    p128 = psi128.cpu().numpy()
    p64 = psi64.cpu().numpy().astype(np.complex128)
    r128 = O.apply_rows(t.x, t.z, cp, p128, lo, hi)
    r64 = O.apply_rows(t.x, t.z, cp, p64, lo, hi)
    a = y128[lo:hi].cpu().numpy()
    b = y64[lo:hi].cpu().numpy().astype(np.complex128)
    e = lambda u, v: float(np.linalg.norm(u - v) / np.linalg.norm(v))
    return {"c128_vs_oracle_rows": e(a, r128), "c64c_vs_oracle_rows": e(b, r64),
            "c64c_vs_oracle_rows_fp64_input": e(b, r128),
            "oracle_rows": "[%d, %d) of 2^%d" % (lo, hi, t.n)}


# ----------------------------------------------------------------------------- secondary
def _events_time(fn, steps, warmup, stream):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def _base_line(args, metric, value, unit, ms, dtype, config, **kw):
    out = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
           "config": config}
    out.update(kw)
    return out


def _roof(alg_bytes, ms, hbm, peak_kind, rule, note=None):
    ach = alg_bytes / (ms / 1e3) / 1e9
    d = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
         "traffic": None, "alg_bytes_per_launch": alg_bytes, "alg_bytes_rule": rule,
         "peak_source": peak_kind}
    if note:
        d["note"] = note
    return d


def _randn_state(n_amp, dev, seed, dtype):
    import torch
    g = torch.Generator(device=dev).manual_seed(seed)
    p = torch.complex(torch.randn(n_amp, device=dev, dtype=torch.float64, generator=g),
                      torch.randn(n_amp, device=dev, dtype=torch.float64, generator=g))
    return (p / torch.linalg.vector_norm(p)).to(dtype)


def measure_chain(steps=3, warmup=3, matvecs=100, n=22):
    """The TFIM+XXZ open chain, n = 22 (85 terms, G = 44): a step is 100
    repeated matvecs y = H psi (the reference's driver shape: CSR built once,
    then repeated CSR*vector), complex64-compensated and complex128.  The
    state (32 / 64 MiB) sits in L2, so the HBM fraction is nominal."""
    import torch
    from oracle import oracle as O
    from qrusty_gb300 import PauliOperator, _lib
    from qrusty_gb300 import workloads as W
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    t, _ = W.cfg1(with_state=False, n=n)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    N = 1 << n
    P = W.alg_blocks(t, 13)
    hbm, peak_kind = peaks()
    psi = _randn_state(N, dev, 21, torch.complex128)
    O.build()
    ref = O.apply(n, t.x, t.z, O.make_params(t.phase, t.coeff), psi.cpu().numpy())
    out = {"workload": "tfim+xxz open chain n=%d, %d terms, %d matvecs per step (seed %d)"
                       % (n, t.T, matvecs, W.SEED0 + 1)}
    for name, dt, esz in (("c64c", torch.complex64, 8), ("c128", torch.complex128, 16)):
        x = psi.to(dt)
        y = torch.empty_like(x)

        def step():
            for _ in range(matvecs):
                op.apply(x, out=y)
        l0 = _lib.launch_count()
        ms = _events_time(step, steps, warmup, stream)
        launches = (_lib.launch_count() - l0) / (steps + warmup)
        op.sync_check()
        yh = y.cpu().numpy().astype(np.complex128)
        mv = ms / matvecs
        out[name] = {
            "ms_per_step": ms, "ms_per_matvec": mv, "value": t.T * N * matvecs / (ms / 1e3),
            "unit": UNIT, "gpu_launches_per_step": launches,
            "roofline": _roof((P + 1) * N * esz, mv, hbm, peak_kind,
                              "(P+1)*2^n*%d per matvec, P=%d" % (esz, P),
                              "state L2-resident: nominal"),
            "rel_err_vs_oracle": float(np.linalg.norm(yh - ref) / np.linalg.norm(ref))}
    return out


def measure_batch(steps=3, warmup=3, per_op=True):
    """256 uneven operators (n ~ U{10..20}, T ~ U{50..5000}) x 8 complex64
    states behind one graph launch per step; a dozen operators (every qubit
    count) against the FP64 oracle on row blocks of every state."""
    import torch
    from oracle import oracle as O
    from qrusty_gb300 import Batch, PauliOperator, _lib
    from qrusty_gb300 import workloads as W
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    terms = W.cfg3()
    ns = 8
    t0 = time.perf_counter()
    ops = [PauliOperator(t.n, t.x, t.z, t.phase, t.coeff) for t in terms]
    t_create = time.perf_counter() - t0
    g = torch.Generator(device=dev).manual_seed(7)
    psis, ys = [], []
    for t in terms:
        p = torch.complex(torch.randn(ns << t.n, device=dev, generator=g),
                          torch.randn(ns << t.n, device=dev, generator=g))
        psis.append(p)
        ys.append(torch.empty_like(p))
    units = sum(t.T * (ns << t.n) for t in terms)
    alg = sum((W.alg_blocks(t, 13) + 1) * (ns << t.n) * 8 for t in terms)
    t0 = time.perf_counter()
    b = Batch(ops, [ns] * len(ops))
    b.apply(psis, ys)  # autotune + graph capture
    torch.cuda.synchronize()
    t_tune = time.perf_counter() - t0
    l0 = _lib.launch_count()
    ms_b = _events_time(lambda: b.apply(psis, ys), steps, warmup, stream)
    launches = (_lib.launch_count() - l0) / (steps + warmup)
    torch.cuda.synchronize()
    # oracle on row blocks of every state of one operator per qubit count
    O.build()
    by_n = {}
    for i, t in enumerate(terms):
        by_n.setdefault(t.n, []).append(i)
    pick = [max(v, key=lambda i: terms[i].T) for _, v in sorted(by_n.items())]
    rng = np.random.default_rng(0)
    worst = 0.0
    for i in pick:
        t = terms[i]
        N = 1 << t.n
        cp = O.make_params(t.phase, t.coeff)
        Pm = psis[i].cpu().numpy().reshape(ns, N).astype(np.complex128)
        Ym = ys[i].cpu().numpy().reshape(ns, N).astype(np.complex128)
        for s_ in range(ns):
            lo = 0 if N <= 8192 else int(rng.integers(0, N - 4096))
            hi = N if N <= 8192 else lo + 4096
            r = O.apply_rows(t.x, t.z, cp, Pm[s_], lo, hi)
            worst = max(worst, float(np.linalg.norm(Ym[s_, lo:hi] - r) / np.linalg.norm(r)))
    hbm, peak_kind = peaks()
    out = {"workload": "256 operators, n ~ U{10..20}, T ~ U{50..5000} random letters (seed %d), "
                       "8 complex64 states each" % (W.SEED0 + 3),
           "ms_per_step": ms_b, "value": units / (ms_b / 1e3), "unit": UNIT,
           "mode": {0: "persistent work-list kernel", 1: "graph of per-operator kernels",
                    2: "persistent kernel for the small operators + per-operator kernels"}
                   .get(b.mode, str(b.mode)),
           "mode_code": b.mode,
           "tile_bits": b.tile_bits, "gpu_launches_per_step": launches,
           "roofline": _roof(alg, ms_b, hbm, peak_kind,
                             "sum over ops of (P+1)*states*2^n*8"),
           "rel_err_vs_oracle": {"worst": worst, "operators": len(pick),
                                 "rows": "4096-row block (all rows for 2^n <= 8192), every state"},
           "setup_s": {"create_ops": t_create, "autotune_and_capture": t_tune}}
    if per_op:
        def per_op_apply():
            for op, p, y in zip(ops, psis, ys):
                op.apply(p, out=y)
        ms_64 = _events_time(per_op_apply, 2, 1, stream)
        out["per_op_c64c_ms"] = ms_64
        out["speedup_vs_per_op_c64c"] = ms_64 / ms_b
        # every launch form on its own clock (the autotuner keeps the fastest)
        forms = {}
        for m, name in ((0, "persistent"), (1, "per_operator_graph"), (2, "hybrid")):
            bm = Batch(ops, [ns] * len(ops))
            bm.set_mode(m)
            forms[name] = _events_time(lambda: bm.apply(psis, ys), 2, 1, stream)
            del bm
        out["forms_ms"] = forms
    return out, (ops, psis, ys, terms, b)


def measure_grad(steps=10, warmup=3):
    """y = H(c) psi, L = Re<y, w> (n = 20, 2,000 terms, complex64 psi): one
    training step = forward, backward to c and psi, SGD update of c."""
    import torch
    from oracle import oracle as O
    from qrusty_gb300 import _lib
    from qrusty_gb300 import workloads as W
    from qrusty_gb300.autograd import PauliTerms, pauli_apply
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    t, psi, w = W.cfg4()
    terms = PauliTerms(t.n, t.x, t.z, t.phase)
    c = torch.tensor(t.coeff.real, dtype=torch.float64, device=dev, requires_grad=True)
    p = torch.from_numpy(psi.astype(np.complex64)).to(dev).requires_grad_(True)
    wd = torch.from_numpy(w.astype(np.complex64)).to(dev)

    def step():
        c.grad = None
        p.grad = None
        y = pauli_apply(c, p, terms)
        torch.vdot(y, wd).real.backward()
        with torch.no_grad():
            c.add_(c.grad, alpha=-1e-3)  # SGD: the next step sees new coefficients

    l0 = _lib.launch_count()
    ms = _events_time(step, steps, warmup, stream)
    launches = (_lib.launch_count() - l0) / (steps + warmup)
    # gradients at the current coefficients against the FP64 oracle
    c.grad = None
    p.grad = None
    y = pauli_apply(c, p, terms)
    torch.vdot(y, wd).real.backward()
    torch.cuda.synchronize()
    O.build()
    ch = c.detach().cpu().numpy().astype(np.complex128)
    ph = p.detach().cpu().numpy().astype(np.complex128)
    wh = wd.cpu().numpy().astype(np.complex128)
    tg = O.term_grad(t.n, t.x, t.z, t.phase, ph, wh).real
    gc = c.grad.cpu().numpy()
    cp = O.make_params(t.phase, ch)
    yref = O.apply(t.n, t.x, t.z, cp, ph)
    yh = y.detach().cpu().numpy().astype(np.complex128)
    N = 1 << t.n
    # where a step goes: the pieces on their own clocks
    op = terms.operator(c.detach())
    pd = p.detach()
    ms_fwd = _events_time(lambda: op.apply(pd), 10, 3, stream)
    ms_adj = _events_time(lambda: op.apply(wd, adjoint=True), 10, 3, stream)
    ms_tg = _events_time(lambda: op.term_grad(pd, wd), 10, 3, stream)
    ms_cu = _events_time(lambda: op.set_coeffs_device(c.detach()), 10, 3, stream)
    return {"workload": "n=%d, %d random-letter terms, real c, complex64 psi, L = Re<H(c)psi, w> "
                        "(seed %d)" % (t.n, t.T, W.SEED0 + 4),
            "step": "forward + backward (grad_c, grad_psi) + SGD update of c",
            "ms_per_step": ms, "value": t.T * N / (ms / 1e3), "unit": UNIT,
            "gpu_launches_per_step": launches,
            "breakdown_ms": {"forward_apply": ms_fwd, "adjoint_apply": ms_adj,
                             "term_grad": ms_tg, "device_coefficient_update": ms_cu},
            "rel_err_vs_oracle": {
                "forward_y": float(np.linalg.norm(yh - yref) / np.linalg.norm(yref)),
                "grad_c": float(np.linalg.norm(gc - tg) / np.linalg.norm(tg))}}


def measure_csr(steps=5, warmup=3, n=22):
    """Device CSR build (indptr, indices, data) of the chain at n = 22 and
    CSR*vector on it; 64 rows of the build against make_row bit for bit and
    the CSR*vector against the oracle's on a row sample."""
    import torch
    from oracle import oracle as O
    from qrusty_gb300 import PauliOperator, _lib
    from qrusty_gb300 import workloads as W
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    t, _ = W.cfg1(with_state=False, n=n)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    nr, nz = op.csr_size()
    G = nz // nr
    indptr = torch.empty(nr + 1, dtype=torch.int64, device=dev)
    indices = torch.empty(nz, dtype=torch.int64, device=dev)
    data = torch.empty(nz, dtype=torch.complex128, device=dev)
    L = _lib.load()
    st = stream.cuda_stream
    fn = lambda: _lib.check(L.qr_csr_build(op.handle, indptr.data_ptr(), indices.data_ptr(),
                                           data.data_ptr(), _lib.QR_MEM_DEVICE, st))
    l0 = _lib.launch_count()
    ms = _events_time(fn, steps, warmup, stream)
    launches = (_lib.launch_count() - l0) / (steps + warmup)
    op.sync_check()
    hbm, peak_kind = peaks()
    written = 8 * (nr + 1) + 24 * nz
    O.build()
    cp = O.make_params(t.phase, t.coeff)
    rng = np.random.default_rng(7)
    rows = np.unique(np.concatenate([[0, nr - 1], rng.integers(0, nr, 62)])).astype(np.int64)
    rd = torch.from_numpy(rows).to(dev)
    pos = (rd[:, None] * G + torch.arange(G, device=dev)[None, :]).reshape(-1)
    cols = indices[pos].cpu().numpy().view(np.uint64).reshape(len(rows), G)
    vals = data[pos].cpu().numpy().reshape(len(rows), G)
    exact = 0
    for k, r in enumerate(rows.tolist()):
        oc, ov = O.make_row(t.x, t.z, cp, r)
        exact += int(np.array_equal(cols[k], oc)
                     and np.array_equal(vals[k].view(np.uint64), ov.view(np.uint64)))
    csr = {"workload": "tfim+xxz open chain n=%d, %d terms, G=%d, %d stored entries (seed %d)"
                       % (n, t.T, G, nz, W.SEED0 + 1),
           "ms_per_step": ms, "value": nz / (ms / 1e3), "unit": "nnz/s",
           "gpu_launches_per_step": launches,
           "roofline": _roof(written, ms, hbm, peak_kind, "8(N+1) + 24 nnz written"),
           "rows_bit_exact_vs_make_row": "%d/%d" % (exact, len(rows))}
    # CSR * vector on the matrix just built
    v = _randn_state(nr, dev, 3, torch.complex128)
    y = torch.empty_like(v)
    fs = lambda: L.qr_csr_spmv(nr, nr, indptr.data_ptr(), indices.data_ptr(), data.data_ptr(),
                               v.data_ptr(), y.data_ptr(), st)
    l0 = _lib.launch_count()
    ms_s = _events_time(fs, steps, warmup, stream)
    launches_s = (_lib.launch_count() - l0) / (steps + warmup)
    torch.cuda.synchronize()
    srows = 1 << 16
    ipc, ijc, dc = O.csr_build(n, t.x, t.z, cp, rows=(0, srows))
    ys = O.spmv(ipc, ijc, dc, v.cpu().numpy())
    yg = y[:srows].cpu().numpy()
    alg = 24 * nz + 8 * (nr + 1) + 16 * nr
    spmv = {"workload": csr["workload"] + ", CSR built on the device",
            "ms_per_step": ms_s, "value": nz / (ms_s / 1e3), "unit": "nnz/s",
            "gpu_launches_per_step": launches_s,
            "roofline": _roof(alg, ms_s, hbm, peak_kind, "24 nnz + 8 (N+1) + 16 N",
                              "FP64-bound on GB300 (4 DFMA per stored entry)"),
            "fp64_tflops": 8.0 * nz / (ms_s / 1e3) / 1e12,
            "fp64_frac_of_measured": (8.0 * nz / (ms_s / 1e3) / 1e12 / fp64_peak())
                                     if fp64_peak() else None,
            "rel_err_vs_oracle_rows": float(np.linalg.norm(yg - ys) / np.linalg.norm(ys)),
            "oracle_rows": "[0, %d)" % srows}
    return csr, spmv


def run_secondary(args):
    """Compact lines of the other configurations, each on its own clock (CUDA
    events on the launching stream), for the default bench line."""
    out = {}
    for name, fn in (("chain", lambda: measure_chain()),
                     ("grad", lambda: measure_grad()),
                     ("batch", lambda: measure_batch(per_op=True)[0]),
                     ("csr_spmv", lambda: measure_csr())):
        t0 = time.perf_counter()
        try:
            r = fn()
        except Exception as e:  # reported, never silently dropped
            r = {"error": "%s: %s" % (type(e).__name__, e)}
        if name == "csr_spmv" and isinstance(r, tuple):
            out["csr"], out["spmv"] = r
        else:
            out[name] = r
        log("secondary %s: %.1f s" % (name, time.perf_counter() - t0))
        import torch
        torch.cuda.empty_cache()
    return out


def run_batch(args):
    r, (ops, psis, ys, terms, b) = measure_batch(args.steps, args.warmup, per_op=True)
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    # one complex128 launch per operator on the same states
    p128 = [p.to(torch.complex128) for p in psis]
    y128 = [torch.empty_like(p) for p in p128]

    def per_op():
        for op, p, y in zip(ops, p128, y128):
            op.apply(p, out=y)
    ms_128 = _events_time(per_op, 2, 1, stream)
    out = _base_line(args, "batched Pauli-sum H·ψ term·amp/s (sum over operators and states)",
                     r["value"], UNIT, r["ms_per_step"], "c64c (fp32 + two-sum)",
                     {"workload": r["workload"], "tile_bits_autotuned": r["tile_bits"],
                      "mode": r["mode"]},
                     roofline=r["roofline"], rel_err=r["rel_err_vs_oracle"],
                     per_op_c128={"ms_per_step": ms_128, "launches_per_step": len(ops)},
                     speedup_vs_per_op_c128=ms_128 / r["ms_per_step"],
                     per_op_c64c_ms=r.get("per_op_c64c_ms"), forms_ms=r.get("forms_ms"),
                     setup_s=r["setup_s"], gpu_launches=r["gpu_launches_per_step"])
    print(json.dumps(out), flush=True)


def run_grad(args):
    r = measure_grad(args.steps, args.warmup)
    out = _base_line(args, "differentiable H(c)·ψ training step term·amp/s "
                           "(forward terms x amplitudes / step)",
                     r["value"], UNIT, r["ms_per_step"], "c64c forward / adjoint, fp64 reductions",
                     {"workload": r["workload"], "step": r["step"],
                      "l2": "state 8 MiB: L2-resident"},
                     rel_err=r["rel_err_vs_oracle"], gpu_launches=r["gpu_launches_per_step"],
                     breakdown_ms=r["breakdown_ms"])
    print(json.dumps(out), flush=True)


def run_vec(args):
    import ctypes as C
    import torch
    from qrusty_gb300 import _lib
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    st = stream.cuda_stream
    L = _lib.load()
    N = 1 << args.n
    hbm, peak_kind = peaks()
    res = {}
    a = (C.c_double * 2)(0.5, -1.25)
    b = (C.c_double * 2)(-0.75, 0.5)
    for name, dt, tdt, esz in (("c128", _lib.QR_C128, torch.complex128, 16),
                               ("c64", _lib.QR_C64C, torch.complex64, 8)):
        x = torch.randn(N, dtype=tdt, device=dev)
        y = torch.randn(N, dtype=tdt, device=dev)
        z = torch.empty_like(x)
        fns = {
            "axpby": (lambda: L.qr_axpby(dt, N, a, x.data_ptr(), b, y.data_ptr(), z.data_ptr(), st),
                      3),
            "axpy": (lambda: L.qr_axpy(dt, N, a, x.data_ptr(), y.data_ptr(), z.data_ptr(), st), 3),
            "ax": (lambda: L.qr_ax(dt, N, a, x.data_ptr(), z.data_ptr(), st), 2),
            "precond2": (lambda: L.qr_precond2(dt, N, x.data_ptr(), y.data_ptr(), a, 1e-12,
                                               z.data_ptr(), st), 3),
        }
        for op, (fn, passes) in fns.items():
            ms = _events_time(fn, args.steps, args.warmup, stream)
            gbs = passes * N * esz / (ms / 1e3) / 1e9
            res["%s_%s" % (op, name)] = {"ms": ms, "GB/s": gbs, "frac": gbs / hbm}
        del x, y, z
    head = res["axpby_c128"]
    out = _base_line(
        args, "axpby z = a x + b y GB/s (HBM-bound vector helper)", head["GB/s"], "GB/s",
        head["ms"], "c128",
        {"workload": "axpby / axpy / ax / precond2 over 2^%d elements" % args.n,
         "l2": "inputs %d MiB > L2; no flush" % ((N * 16) >> 20)},
        roofline=_roof(48 * N, head["ms"], hbm, peak_kind, "read x, y + write z"),
        all=res)
    print(json.dumps(out), flush=True)


def run_csr(args):
    csr, _ = measure_csr(args.steps, args.warmup, n=args.n if args.n != 26 else 22)
    out = _base_line(args, "rowwise CSR build nnz/s (indptr, indices, data on the device)",
                     csr["value"], "nnz/s", csr["ms_per_step"], "u64 indices, c128 data",
                     {"workload": csr["workload"]}, roofline=csr["roofline"],
                     rows_bit_exact_vs_make_row=csr["rows_bit_exact_vs_make_row"],
                     gpu_launches=csr["gpu_launches_per_step"])
    print(json.dumps(out), flush=True)


def run_spmv(args):
    _, sp = measure_csr(args.steps, args.warmup, n=args.n if args.n != 26 else 22)
    out = _base_line(args, "CSR*vector nnz/s (qr_csr_spmv, complex128)", sp["value"], "nnz/s",
                     sp["ms_per_step"], "c128", {"workload": sp["workload"]},
                     roofline=sp["roofline"], fp64_tflops=sp["fp64_tflops"],
                     rel_err_vs_oracle_rows=sp["rel_err_vs_oracle_rows"],
                     gpu_launches=sp["gpu_launches_per_step"])
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__,
                                 formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["jw", "chain", "batch", "grad", "vec", "csr", "spmv"],
                    default="jw")
    ap.add_argument("--qubits", "--n", dest="n", type=int, default=26,
                    help="qubits of the workload (--n is accepted outside torchrun)")
    ap.add_argument("--pairs", type=int, default=8000)
    ap.add_argument("--zterms", type=int, default=2000)
    ap.add_argument("--cpu-rows", type=int, default=1 << 16,
                    help="row sample of the CPU reference arm / baseline")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--quick", action="store_true",
                    help="no clock sampling, e2e or CPU baseline (profiling runs)")
    ap.add_argument("--no-secondary", action="store_true",
                    help="headline only: skip the secondary workloads of the default line")
    args = ap.parse_args()
    if args.warmup < 3 and not args.quick:
        raise SystemExit("--warmup must be >= 3")
    if args.workload in ("batch", "grad", "vec", "csr", "spmv"):
        if args.impl == "reference":
            raise SystemExit("--impl reference measures the headline workloads (jw, chain)")
        {"batch": run_batch, "grad": run_grad, "vec": run_vec, "csr": run_csr,
         "spmv": run_spmv}[args.workload](args)
        return
    if args.workload == "chain" and args.n == 26:
        args.n = 22
    t, desc = make_terms(args)
    if args.impl == "reference":
        run_reference_arm(args, t, desc)
    else:
        run_gpu_arm(args, t, desc)


if __name__ == "__main__":
    main()
