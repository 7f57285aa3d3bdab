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


def ncu_traffic():
    """DRAM bytes per launch of the c64c apply kernel from the committed ncu
    summary (profiles/ncu_traffic.json), scaled to the bench workload."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


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
    sample = ("rows [0, %d) of 2^%d: CSR build %.2f s (make_row, chunks of 1024), then one "
              "CSR*vector per step; value = sample term*amp / SpMV time" % (rows, t.n, t_build))
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

    # --- accuracy at full size: c64c against c128 (checked against the FP64
    # oracle on sampled rows in the test suite)
    rel64 = float(torch.linalg.vector_norm(y64.to(torch.complex128) - y128)
                  / torch.linalg.vector_norm(y128))

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
               "path": "qr_apply_host (C ABI), pinned host buffers"}

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
        "c128": {"value": whole_job_rate(ws, T * N, ms128 / 1e3), "ms_per_step": ms128,
                 "steps": s128,
                 # 4 DFMA (8 flops) per amplitude and x group; GB300 FP64 is
                 # 1.25 TFLOP/s nominal (no measured FP64 peak is recorded)
                 "fp64_tflops": 8.0 * N * int(info["ngroups"]) / (ms128 / 1e3) / 1e12,
                 "fp64_frac_of_nominal": 8.0 * N * int(info["ngroups"]) / (ms128 / 1e3)
                                         / 1.25e12,
                 "hbm_achieved_gbs": ach128, "hbm_frac": ach128 / hbm},
        "speedup_c64c_vs_c128": ms128 / ms64,
        "rel_err": {"c64c_vs_c128_full": rel64},
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
            "sample": ("rows [0, %d) of 2^%d; CSR build %.2f s, CSR*vector %.1f ms (median of 3)"
                       % (args.cpu_rows, n, t_build, ms_cpu))}
    print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


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


def run_batch(args):
    import torch
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
    psis, ys, psis128, ys128 = [], [], [], []
    for t in terms:
        p = torch.complex(torch.randn(ns << t.n, device=dev, generator=g),
                          torch.randn(ns << t.n, device=dev, generator=g))
        psis.append(p)
        ys.append(torch.empty_like(p))
        psis128.append(p.to(torch.complex128))
        ys128.append(torch.empty_like(psis128[-1]))
    units = sum(t.T * (ns << t.n) for t in terms)
    alg = sum((W.alg_blocks(t, 13) + 1) * (ns << t.n) * 8 for t in terms)
    t0 = time.perf_counter()
    b = Batch(ops, [ns] * len(ops))
    b.apply(psis, ys)  # autotune + graph capture
    torch.cuda.synchronize()
    t_tune = time.perf_counter() - t0
    l0 = _lib.launch_count()
    ms_b = _events_time(lambda: b.apply(psis, ys), args.steps, args.warmup, stream)
    launches = (_lib.launch_count() - l0) / (args.steps + args.warmup)

    def per_op(ps, outs):
        for op, p, y in zip(ops, ps, outs):
            op.apply(p, out=y)
    s2 = max(3, args.steps // 5)
    ms_128 = _events_time(lambda: per_op(psis128, ys128), s2, 3, stream)
    ms_64 = _events_time(lambda: per_op(psis, ys), s2, 3, stream)
    # accuracy: batched c64c against per-operator c128 on the same states
    b.apply(psis, ys)
    per_op(psis128, ys128)
    torch.cuda.synchronize()
    worst = max(float(torch.linalg.vector_norm(y.to(torch.complex128) - r)
                      / torch.linalg.vector_norm(r)) for y, r in zip(ys, ys128))
    hbm, peak_kind = peaks()
    ach = alg / (ms_b / 1e3) / 1e9
    out = _base_line(
        args, "batched Pauli-sum H·ψ term·amp/s (sum over operators and states)",
        units / (ms_b / 1e3), UNIT, ms_b, "c64c (fp32 + two-sum)",
        {"workload": "256 operators, n ~ U{10..20}, T ~ U{50..5000} random letters (seed %d), "
                     "8 complex64 states each" % (W.SEED0 + 3),
         "operators": len(terms), "states_per_op": ns,
         "amplitudes_total": int(sum(ns << t.n for t in terms)),
         "tile_bits_autotuned": b.tile_bits,
         "l2": "total state %d MiB; no flush" % (sum((ns << t.n) * 8 for t in terms) >> 20)},
        roofline={"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                  "frac": ach / hbm, "traffic": None, "alg_bytes_per_launch": alg,
                  "alg_bytes_rule": "sum over ops of (P+1)*states*2^n*8", "peak_source": peak_kind},
        per_op_c128={"ms_per_step": ms_128, "launches_per_step": len(ops),
                     "value": units / (ms_128 / 1e3)},
        per_op_c64c={"ms_per_step": ms_64, "value": units / (ms_64 / 1e3)},
        speedup_vs_per_op_c128=ms_128 / ms_b,
        rel_err={"batched_c64c_vs_c128_worst_op": worst},
        setup_s={"create_ops": t_create, "autotune_and_capture": t_tune},
        gpu_launches=launches)
    print(json.dumps(out), flush=True)


def run_grad(args):
    import torch
    from qrusty_gb300 import workloads as W
    from qrusty_gb300.autograd import PauliTerms, pauli_apply
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    t, psi, w = W.cfg4()
    terms = PauliTerms(t.n, t.x, t.z, t.phase)
    c = torch.tensor(t.coeff.real, dtype=torch.float64, requires_grad=True)
    p = torch.from_numpy(psi.astype(np.complex64)).to(dev).requires_grad_(True)
    wd = torch.from_numpy(w.astype(np.complex64)).to(dev)

    def step():
        c.grad = None
        p.grad = None
        y = pauli_apply(c, p, terms)
        torch.vdot(y, wd).real.backward()
        with torch.no_grad():
            c.add_(c.grad, alpha=-1e-3)  # an SGD update: the next step sees new coefficients

    ms = _events_time(step, args.steps, args.warmup, stream)
    N = 1 << t.n
    # where a step goes: coefficient update (plans rebuilt), forward, adjoint,
    # per-term inner products
    cc = t.coeff.real.astype(np.complex128)
    reps = 5
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(reps):
        cc[0] += 1e-6
        op = terms.operator(cc)
        op.apply(p.detach(), out=torch.empty_like(p))  # plans are rebuilt lazily on first use
        torch.cuda.synchronize()
    ms_update_fwd = 1e3 * (time.perf_counter() - t0) / reps
    pd, gd = p.detach(), wd
    ms_fwd = _events_time(lambda: op.apply(pd), 10, 3, stream)
    ms_adj = _events_time(lambda: op.apply(gd, adjoint=True), 10, 3, stream)
    ms_tg = _events_time(lambda: op.term_grad(pd, gd), 10, 3, stream)
    out = _base_line(
        args, "differentiable H(c)·ψ training step term·amp/s (forward terms x amplitudes / step)",
        t.T * N / (ms / 1e3), UNIT, ms, "c64c forward / adjoint, fp64 reductions",
        {"workload": "n=%d, %d random-letter terms, real c, complex64 psi, L = Re<H(c)psi, w> "
                     "(seed %d)" % (t.n, t.T, W.SEED0 + 4),
         "step": "forward + backward (grad_c, grad_psi) + SGD update of c",
         "l2": "state 8 MiB: L2-resident"},
        breakdown_ms={"coeff_update_and_forward_incl_plan_rebuild": ms_update_fwd,
                      "forward_apply": ms_fwd, "adjoint_apply": ms_adj, "term_grad": ms_tg})
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
        roofline={"bound": "hbm", "achieved": head["GB/s"], "peak": hbm, "unit": "GB/s",
                  "frac": head["GB/s"] / hbm, "traffic": None,
                  "alg_bytes_per_launch": 48 * N, "alg_bytes_rule": "read x, y + write z",
                  "peak_source": peak_kind},
        all=res)
    print(json.dumps(out), flush=True)


def run_csr(args):
    import torch
    from qrusty_gb300 import PauliOperator
    from qrusty_gb300 import workloads as W
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    n = args.n if args.n != 26 else 22
    t, _ = W.cfg1(with_state=False, n=n)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    nr, nz = op.csr_size()
    indptr = torch.empty(nr + 1, dtype=torch.int64, device=dev)
    indices = torch.empty(nz, dtype=torch.int64, device=dev)
    data = torch.empty(nz, dtype=torch.complex128, device=dev)
    from qrusty_gb300 import _lib
    L = _lib.load()
    st = stream.cuda_stream
    fn = lambda: _lib.check(L.qr_csr_build(op.handle, indptr.data_ptr(), indices.data_ptr(),
                                           data.data_ptr(), _lib.QR_MEM_DEVICE, st))
    ms = _events_time(fn, args.steps, args.warmup, stream)
    op.sync_check()
    written = 8 * (nr + 1) + 24 * nz
    hbm, peak_kind = peaks()
    gbs = written / (ms / 1e3) / 1e9
    out = _base_line(
        args, "rowwise CSR build nnz/s (indptr, indices, data on the device)",
        nz / (ms / 1e3), "nnz/s", ms, "u64 indices, c128 data",
        {"workload": "tfim+xxz open chain n=%d, %d terms, G=%d (seed %d)"
                     % (n, t.T, nz // nr, W.SEED0 + 1),
         "nnz": int(nz), "bytes_written": int(written)},
        roofline={"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                  "frac": gbs / hbm, "traffic": None, "alg_bytes_per_launch": written,
                  "alg_bytes_rule": "8(N+1) + 24 nnz written", "peak_source": peak_kind})
    if not args.no_cpu:
        from oracle import oracle as O
        O.build()
        rows = min(nr, args.cpu_rows * 4)
        cp = O.make_params(t.phase, t.coeff)
        nth = os.cpu_count() or 1
        t0 = time.perf_counter()
        O.csr_build(t.n, t.x, t.z, cp, step=1024, nthreads=nth, rows=(0, rows))
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": rows * (nz // nr) / dt, "unit": "nnz/s", "cores": nth,
                               "kind": "port",
                               "sample": "rows [0, %d) of 2^%d, make_row chunks of 1024" % (rows, n)}
    print(json.dumps(out), flush=True)


def run_spmv(args):
    import torch
    from qrusty_gb300 import PauliOperator, _lib
    from qrusty_gb300 import workloads as W
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    n = args.n if args.n != 26 else 22
    t, _ = W.cfg1(with_state=False, n=n)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    ip, ij, d = op.csr_device()
    N = 1 << n
    g = torch.Generator(device=dev).manual_seed(3)
    v = torch.randn(N, dtype=torch.complex128, device=dev, generator=g)
    y = torch.empty_like(v)
    L = _lib.load()
    st = stream.cuda_stream
    fn = lambda: L.qr_csr_spmv(N, N, ip.data_ptr(), ij.data_ptr(), d.data_ptr(), v.data_ptr(),
                               y.data_ptr(), st)
    ms = _events_time(fn, args.steps, args.warmup, stream)
    nnz = d.numel()
    alg = 24 * nnz + 8 * (N + 1) + 16 * N  # entries + indptr + y; v gathers hit L2 (64 MiB)
    ref = op.apply(v)
    err = float(torch.linalg.vector_norm(y - ref) / torch.linalg.vector_norm(ref))
    hbm, peak_kind = peaks()
    gbs = alg / (ms / 1e3) / 1e9
    out = _base_line(
        args, "CSR*vector nnz/s (qr_csr_spmv, complex128)", nnz / (ms / 1e3), "nnz/s", ms,
        "c128",
        {"workload": "tfim+xxz open chain n=%d, %d terms, CSR built on the device (seed %d)"
                     % (n, t.T, W.SEED0 + 1), "nnz": int(nnz),
         "l2": "CSR %d MiB > L2; vector 64 MiB" % ((24 * nnz) >> 20)},
        roofline={"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                  "frac": gbs / hbm, "traffic": None, "alg_bytes_per_launch": alg,
                  "alg_bytes_rule": "24 nnz + 8 (N+1) + 16 N", "peak_source": peak_kind},
        rel_err={"vs_matrix_free_c128": err},
        # complex128 multiply-add = 4 FP64 FMAs (8 flops) per entry; GB300's
        # nominal FP64 rate (1.25 TFLOP/s) bounds this kernel before HBM does
        fp64={"tflops": 8.0 * nnz / (ms / 1e3) / 1e12,
              "frac_of_nominal": 8.0 * nnz / (ms / 1e3) / 1.25e12,
              "hbm_floor_ms": alg / (hbm * 1e9) * 1e3,
              "fp64_floor_ms": 8.0 * nnz / 1.25e12 * 1e3})
    if not args.no_cpu:
        from oracle import oracle as O
        O.build()
        rows = min(N, args.cpu_rows * 4)
        ipc, ijc, dc = O.csr_build(n, t.x, t.z, O.make_params(t.phase, t.coeff), rows=(0, rows))
        vh = v.cpu().numpy()
        nth = os.cpu_count() or 1
        O.spmv(ipc, ijc, dc, vh, nthreads=nth)
        t0 = time.perf_counter()
        for _ in range(3):
            O.spmv(ipc, ijc, dc, vh, nthreads=nth)
        dt = (time.perf_counter() - t0) / 3
        out["cpu_baseline"] = {"value": len(dc) / dt, "unit": "nnz/s", "cores": nth, "kind": "port",
                               "sample": "rows [0, %d) of 2^%d, chunks of 1024 rows" % (rows, n)}
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
