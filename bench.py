#!/usr/bin/env python3
"""Benchmark of the engine's hot path: QSimulator::simulate on the full
quantum Fourier transform.

Workload (default): 30-qubit complex64 register holding i.i.d. standard-normal
complex amplitudes (normalised, seed 3); circuit = aqs::fourier_transform(30)
(H + controlled-phase ladder, src/quantum_algo.cpp:103-114) plus the final
Swap(i, 29-i) for i < 15: 30 H + 435 CPhase + 15 Swap = 480 gate
applications, one gate per kernel pass over HBM.  A "step" is one pass of the
whole circuit over the resident register.  The register (8 GiB) is larger
than L2, so no L2 flush is needed between steps.

Printed: one JSON line (rank 0).  `value` is gate applications per second
with the register resident in HBM; `e2e` is the same metric through the
public C-ABI with the register uploaded from pinned host memory and the result
downloaded every step; `roofline` is the dominant kernel (controlled-phase
pass) against the measured HBM copy bandwidth; `cpu_baseline` is the
per-gate CPU restatement (oracle port, all host threads) on a bounded sample
of the same workload.

`--impl reference` times the CPU implementation instead (rank 0 only).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

GiB = 1 << 30


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=30, help="qubits")
    ap.add_argument("--dtype", choices=["c64", "c128"], default="c64")
    ap.add_argument("--mode", choices=["per_gate", "tiled"], default="per_gate")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--only", choices=["fused_brickwork", "fused_tc", "fused_cc", "tiled_brickwork", "plain12", "tile_shape", "vqe_batch", "vqe_ansatz", "serving",
                                       "qft_grid", "noise"],
                    help="run one secondary workload alone (at --n qubits where it takes a size) "
                         "and print its JSON; for profiling")
    ap.add_argument("--depth", type=int, default=20,
                    help="brick-work depth for --only fused_brickwork, layers for --only vqe_ansatz")
    ap.add_argument("--count", type=int, default=0, help="circuits for --only vqe_batch / serving")
    return ap.parse_args()


# ---- workload ---------------------------------------------------------------------

def qft_ops(n):
    import afquantumsim_gb300 as aq
    return aq.fourier_transform(n, swaps=True)


def algorithmic_bytes(n, amp_bytes):
    """Bytes a gate can change (read + write) summed over the QFT:
    H: N amplitudes, CPhase: N/4 (control = target = 1), Swap: N/2."""
    N = 1 << n
    nh, ncp, nsw = n, n * (n - 1) // 2, n // 2
    per = {"H": 2 * amp_bytes * N, "CPhase": 2 * amp_bytes * N // 4, "Swap": 2 * amp_bytes * N // 2}
    total = nh * per["H"] + ncp * per["CPhase"] + nsw * per["Swap"]
    return total, per, (nh, ncp, nsw)


def gate_alg_bytes(op, n, amp_bytes):
    """Algorithmic bytes of one gate applied on its own: the amplitudes it can
    change, read and written.  General 1-qubit gates and RotZ: N; Z/Phase:
    N/2; single-control gates: N/2; CZ/CPhase: N/4; Swap: N/2; CSwap, CCNot:
    N/4; Or: 3N/4; k-qubit unitaries: N; each extra control halves it."""
    import afquantumsim_gb300 as aq
    k = aq.kinds
    N = 1 << n
    frac = {k.Z: 0.5, k.PHASE: 0.5, k.CX: 0.5, k.CY: 0.5, k.CH: 0.5, k.CRX: 0.5, k.CRY: 0.5, k.CRZ: 0.5,
            k.CZ: 0.25, k.CPHASE: 0.25, k.SWAP: 0.5, k.CSWAP: 0.25, k.CCX: 0.25, k.OR: 0.75,
            k.BARRIER: 0.0}.get(op.kind, 1.0)
    return 2 * amp_bytes * N * frac / (1 << op.num_controls)


def qft_cpu_sample(n):
    """Gates of the QFT with swaps in the proportions of the whole circuit:
    every 15th H, CPhase and Swap (2 H, 29 CPhase, 1 Swap at 30 qubits)."""
    import afquantumsim_gb300 as aq
    ops = qft_ops(n)
    out = []
    for kind in (aq.kinds.H, aq.kinds.CPHASE, aq.kinds.SWAP):
        same = [o for o in ops if o.kind == kind]
        out += same[7::15] or same[:1]
    return out


def metric_name(n, dtype):
    return f"QFT gate-apps/s at {n}q ({dtype}, one gate per pass) + HBM GB/s"


def workload_config(n, dtype, world):
    """The workload both arms run (the same dict in both JSON lines)."""
    _, _, counts = algorithmic_bytes(n, 8)
    amp_b = 8 if dtype == "c64" else 16
    return {"workload": f"qft{n}+swaps", "qubits": n, "gates": sum(counts),
            "gate_mix": {"H": counts[0], "CPhase": counts[1], "Swap": counts[2]},
            "input": "seeded i.i.d. standard-normal complex amplitudes, normalised",
            "parallelism": f"replicas{world}",
            "l2": ("register (2^%d x %d B) larger than L2; no flush" % (n, amp_b)
                   if (amp_b << n) > 129e6 else "register fits in L2 (2^%d x %d B)" % (n, amp_b))}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_bf16_tflops():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["bf16_tflops"]), "measured (burst)"
    return 1900.0, "fallback (burst)"


# ---- clocks -------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid: str | None):
        self.uuid = uuid
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            if self.uuid and self.uuid not in f[0]:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- CPU baseline -----------------------------------------------------------------

def cpu_baseline(n, host_sv, ops, dtype, what):
    """Per-gate CPU restatement of the reference's simulate (oracle port) on
    `ops` (a sample of the workload's gates, described by `what`), all host
    threads."""
    from oracle import oracle
    threads = len(os.sched_getaffinity(0))
    oracle.set_threads(threads)
    t0 = time.perf_counter()
    if dtype == "c64":
        oracle.apply_f32(host_sv, ops)
    else:
        oracle.apply_f64(host_sv, ops)
    dt = time.perf_counter() - t0
    kinds = {}
    for o in ops:
        kinds[o.kind] = kinds.get(o.kind, 0) + 1
    return {"value": len(ops) / dt, "unit": "gate-apps/s", "cores": threads, "kind": "port",
            "sample": f"{what}: {kinds.get(4, 0)} H, {kinds.get(14, 0)} CPhase, {kinds.get(6, 0)} Swap "
                      f"on the full 2^{n} register, {dtype}, {dt:.1f} s", "seconds": dt}


def reference_algorithm_small(n=12):
    """The reference ALGORITHM (dense Kronecker / CSR operators, faithful FP32
    restatement) on the n-qubit QFT: context for how the reference scales."""
    from oracle import oracle
    ops = qft_ops(n)
    v = np.zeros(1 << n, dtype=np.complex64)
    v[0] = 1
    t0 = time.perf_counter()
    oracle.ref32_apply(v, n, ops)
    dt = time.perf_counter() - t0
    return {"n": n, "gate_apps_per_s": len(ops) / dt, "seconds": dt}


# ---- secondary workloads (reported under "extras") -----------------------------------

def _time_ms(stream, fn, reps):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def bench_fused_brickwork(ctx, st, stream, n, depth):
    """Depth-`depth` brick-work circuit (Haar SU(2) as RotZ.RotY.RotZ + CZ
    layers, seed 4) on |0...0>: one gate per pass, plain tile passes, and the
    compiled program (<= 5-qubit fused unitaries) on tensor cores and on CUDA
    cores; error and 1 - fidelity of the tensor-core result against the same
    circuit run one gate per pass in complex128."""
    import afquantumsim_gb300 as aq
    from afquantumsim_gb300 import circuits
    ops = aq.op_array(circuits.brickwork(n, depth, seed=4))
    N = 1 << n
    prog = aq.Program(n, list(ops), aq.C64, max_qubits=5)
    fused, src = prog.info()
    res = {"workload": f"brickwork{n}x{depth}", "gates": src, "fused_ops": fused}

    def reset():
        st.set_basis(0)

    def launches_of(fn):
        l0 = ctx.launch_count()
        fn()
        return ctx.launch_count() - l0

    reset()
    st.apply(ops, aq.EXEC_PER_GATE)
    res["per_gate_ms"] = round(_time_ms(stream, lambda: st.apply(ops, aq.EXEC_PER_GATE), 1), 2)
    tiled_passes = launches_of(lambda: st.apply(ops, aq.EXEC_TILED))
    res["tiled_ms"] = round(_time_ms(stream, lambda: st.apply(ops, aq.EXEC_TILED), 2), 2)
    ctx.set_tensor_cores(False)
    fused_passes = launches_of(lambda: prog.run(st, aq.EXEC_TILED))
    res["fused_cuda_core_ms"] = round(_time_ms(stream, lambda: prog.run(st, aq.EXEC_TILED), 2), 2)
    ctx.set_tensor_cores(True)
    tc_launches = launches_of(lambda: prog.run(st, aq.EXEC_TILED))
    res["fused_tensor_core_ms"] = round(_time_ms(stream, lambda: prog.run(st, aq.EXEC_TILED), 3), 2)
    # HBM roofline of each mode.  One gate per pass: the algorithmic bytes of
    # each gate (the amplitudes it can change); tile passes: one read and one
    # write of the register per pass (2 x 8 B x 2^n), so no mode can exceed
    # 1.0; the tensor-core run also rescales the register once for its FP64
    # norm (its first and last passes carry the norm sums) -- the program's
    # plan (aqsg_program_plan) gives the passes and bytes of both fused runs
    peak, peak_src = measured_peaks()
    reg = 8 * N
    per_gate_bytes = sum(gate_alg_bytes(o, n, 8) for o in ops)
    plan_tc, plan_cc = prog.plan(tensor_cores=True), prog.plan(tensor_cores=False)
    res["fused_plan"] = {"tensor_cores": plan_tc, "cuda_cores": plan_cc, "tc_run_launches": tc_launches,
                         "cuda_core_run_launches": fused_passes}
    modes = {"per_gate": (per_gate_bytes, res["per_gate_ms"], len(ops)),
             "tiled": (2 * reg * tiled_passes, res["tiled_ms"], tiled_passes),
             "fused_cuda_core": (plan_cc["hbm_bytes"], res["fused_cuda_core_ms"], plan_cc["passes"]),
             "fused_tensor_core": (plan_tc["hbm_bytes"], res["fused_tensor_core_ms"], plan_tc["passes"])}
    res["hbm"] = {m: {"passes": p, "bytes": b, "achieved_gbs": round(b / (ms / 1e3) / 1e9, 1), "peak_gbs": peak,
                      "frac": round(b / (ms / 1e3) / 1e9 / peak, 4), "peak_source": peak_src}
                  for m, (b, ms, p) in modes.items()}
    res["speedup_fused_vs_tiled"] = round(res["tiled_ms"] / res["fused_tensor_core_ms"], 2)
    # tensor-pipe work of the fused run: a k-qubit unitary on the tensor
    # cores is three bf16 products of (2^n / 2^k) x 2^(k+1) x 2^(k+1) per
    # register = 24 x 2^n x 2^k flops (k >= 3, not a permutation)
    flops = 0.0
    for o in prog.export():
        k = o.num_qubits
        if o.kind == aq.kinds.UNITARY and k >= 3:
            m = np.ctypeslib.as_array(o.matrix, shape=(2 * (1 << k) * (1 << k),))
            mat = m[0::2] + 1j * m[1::2]
            if not np.all((mat == 0) | (mat == 1)):
                flops += 24.0 * N * (1 << k)
    bf16_peak = measured_bf16_tflops()
    tflops = flops / (res["fused_tensor_core_ms"] / 1e3) / 1e12
    res["tensor"] = {"flops_per_run": flops, "tflops": round(tflops, 1), "peak_tflops": bf16_peak[0],
                     "peak_source": bf16_peak[1], "frac": round(tflops / bf16_peak[0], 4),
                     "note": "3-term split-bf16 products of the fused unitaries of >= 3 qubits"}
    # what the autotuner picks for this circuit (all choices timed once)
    best, every = aq.autotune(ctx, n, ops, aq.C64, reps=1)
    res["autotune_best"] = {k: best[k] for k in ("exec_mode", "fuse_qubits", "tensor_cores", "ms")}
    res["autotune_all_ms"] = {f"{'per_gate' if e['exec_mode'] == aq.EXEC_PER_GATE else 'tiled'}"
                              f"_fuse{e['fuse_qubits']}{'_tc' if e['tensor_cores'] else ''}": round(e["ms"], 2)
                              for e in every}
    res["speedup_fused_vs_per_gate"] = round(res["per_gate_ms"] / res["fused_tensor_core_ms"], 2)
    # accuracy: fused (tensor cores, c64) vs one gate per pass in c128
    reset()
    prog.run(st, aq.EXEC_TILED)
    with aq.State(ctx, n, aq.C128) as ref:
        ref.set_basis(0)
        ref.apply(ops, aq.EXEC_PER_GATE)
        mx, ov, na, nb = st.compare(ref)
    res["max_abs_err_vs_fp64"] = mx
    res["one_minus_fidelity"] = max(0.0, 1.0 - abs(ov) ** 2 / (na * nb))
    res["max_rel_err_scaled"] = mx * np.sqrt(N)  # error relative to a typical |a| = 2^(-n/2)
    res["l2_bytes_note"] = "fused/tiled passes move 2 x 8 B x 2^n each"
    return res


def bench_fused_tc(ctx, stream, n, depth):
    """Only the compiled brick-work program on the tensor cores (two untimed
    runs, then three timed): the launches a profiler of the tensor-core
    tile pass captures, without the other modes of fused_brickwork."""
    import afquantumsim_gb300 as aq
    from afquantumsim_gb300 import circuits
    prog = aq.Program(n, circuits.brickwork(n, depth, seed=4), aq.C64, max_qubits=5)
    ctx.set_tensor_cores(True)
    with aq.State(ctx, n, aq.C64) as st:
        st.set_basis(0)
        prog.run(st, aq.EXEC_TILED)
        prog.run(st, aq.EXEC_TILED)
        ms = _time_ms(stream, lambda: prog.run(st, aq.EXEC_TILED), 3)
    fused, src = prog.info()
    prog.free()
    return {"workload": f"brickwork{n}x{depth}", "gates": src, "fused_ops": fused, "fused_tensor_core_ms": round(ms, 2)}


def bench_fused_cc(ctx, stream, n, depth, width=3):
    """Only the brick-work program fused to `width` qubits on the CUDA cores
    (tensor cores off; two untimed runs, then three timed): the launches a
    profiler of the dense k-qubit tile path captures."""
    import afquantumsim_gb300 as aq
    from afquantumsim_gb300 import circuits
    prog = aq.Program(n, circuits.brickwork(n, depth, seed=4), aq.C64, max_qubits=width)
    ctx.set_tensor_cores(False)
    with aq.State(ctx, n, aq.C64) as st:
        st.set_basis(0)
        prog.run(st, aq.EXEC_TILED)
        prog.run(st, aq.EXEC_TILED)
        ms = _time_ms(stream, lambda: prog.run(st, aq.EXEC_TILED), 3)
    ctx.set_tensor_cores(True)
    fused, src = prog.info()
    plan = prog.plan(tensor_cores=False)
    prog.free()
    return {"workload": f"brickwork{n}x{depth}", "fuse_qubits": width, "gates": src, "fused_ops": fused,
            "passes": plan["passes"], "fused_cuda_core_ms": round(ms, 2)}


def bench_tiled_brickwork(ctx, stream, n, depth):
    """Only the brick-work circuit in plain tile passes (no fusion, CUDA
    cores; two untimed runs, then three timed): the launches a profiler of
    the CUDA-core tile pass captures."""
    import afquantumsim_gb300 as aq
    from afquantumsim_gb300 import circuits
    ops = aq.op_array(circuits.brickwork(n, depth, seed=4))
    with aq.State(ctx, n, aq.C64) as st:
        st.set_basis(0)
        l0 = ctx.launch_count()
        st.apply(ops, aq.EXEC_TILED)
        passes = ctx.launch_count() - l0
        st.apply(ops, aq.EXEC_TILED)
        ms = _time_ms(stream, lambda: st.apply(ops, aq.EXEC_TILED), 3)
    return {"workload": f"brickwork{n}x{depth}", "gates": len(ops), "passes": passes, "tiled_ms": round(ms, 2)}


def bench_noise(ctx, n=12, layers=8, trajectories=4096, seed=7):
    """Noise by trajectories: a hardware-efficient ansatz (RotY + RotZ per
    qubit, CX ring; seeded angles) under depolarizing noise (p = 1e-3 after
    one-qubit gates, 1e-2 per qubit after CX), <Z_q> and <Z_q Z_q+1> averaged
    over `trajectories` seeded trajectories run as one batch; wall time of
    aqsg_noise_expect_z (sampling, batch planning, the run and the averages)."""
    import time as _t

    import afquantumsim_gb300 as aq
    from afquantumsim_gb300 import circuits
    params = np.random.default_rng(seed).uniform(-np.pi, np.pi, size=(layers, n, 2)).astype(np.float32)
    ops = circuits.vqe_ansatz(n, layers, params)
    noise = aq.Noise.depolarizing(1e-3, 1e-2)
    aq.noisy_expect_z(ctx, n, ops, noise, seed, 64)  # warm-up (tuning caches, kernels)
    t0 = _t.perf_counter()
    z, zz, ze, zze = aq.noisy_expect_z(ctx, n, ops, noise, seed, trajectories)
    dt = _t.perf_counter() - t0
    return {"workload": f"ansatz{n}x{layers}_depolarizing", "gates": len(ops), "trajectories": trajectories,
            "seconds": round(dt, 3), "trajectories_per_s": round(trajectories / dt, 1),
            "max_std_err_z": float(np.max(ze)), "mean_z": float(np.mean(z))}


def bench_tile_shape(ctx, sizes=(13, 14), depth=20, seed=4):
    """Tile shape as the autotuner times it: a brick-work circuit on a
    register that fits one whole-register tile (one CTA, one launch) run in
    that shape and in streaming 4096-amplitude tiles (several CTAs, one
    launch per pass), every execution choice in each; c64."""
    import afquantumsim_gb300 as aq
    from afquantumsim_gb300 import circuits
    out = {}
    for n in sizes:
        ops = aq.op_array(circuits.brickwork(n, depth, seed=seed))
        best, every = aq.autotune(ctx, n, ops, aq.C64, reps=3)
        per_shape = {}
        for e in every:
            if e["exec_mode"] != aq.EXEC_TILED:
                continue
            key = "whole" if e["tile_bits"] == n else f"stream{e['tile_bits']}"
            name = f"fuse{e['fuse_qubits']}{'_tc' if e['tensor_cores'] else ''}"
            per_shape.setdefault(key, {})[name] = round(e["ms"] * 1e3, 1)
        out[f"brickwork{n}x{depth}"] = {
            "best": {k: best[k] for k in ("exec_mode", "fuse_qubits", "tensor_cores", "tile_bits")},
            "best_us": round(best["ms"] * 1e3, 1), "tiled_us": per_shape}
    return out


def bench_qft_grid(ctx, stream, sizes=((24, "c64"), (28, "c64"), (24, "c128"), (28, "c128"), (30, "c128"))):
    """The other sizes and dtypes of the QFT workload (with swaps, one gate per
    pass, register resident in HBM, starting from |0...0>): gate-apps/s and
    algorithmic HBM GB/s for each (n, dtype), 1 warm-up and 2 timed steps."""
    import afquantumsim_gb300 as aq
    out = {}
    for n, dt in sizes:
        amp_b = 8 if dt == "c64" else 16
        total_bytes, _, _ = algorithmic_bytes(n, amp_b)
        ops = aq.op_array(qft_ops(n))
        with aq.State(ctx, n, aq.C64 if dt == "c64" else aq.C128) as st:
            st.set_basis(0)  # the kernels do not branch on amplitude values
            st.apply(ops, aq.EXEC_PER_GATE)  # warm-up
            ms = _time_ms(stream, lambda: st.apply(ops, aq.EXEC_PER_GATE), 2)
        out[f"qft{n}_{dt}"] = {"ms_per_step": round(ms, 2), "gate_apps_per_s": round(len(ops) / (ms / 1e3), 1),
                               "hbm_gbs": round(total_bytes / (ms / 1e3) / 1e9, 1)}
    return out


def bench_vqe_ansatz(ctx, stream, n=26, layers=8, reps=3):
    """One large VQE ansatz register (RotY + RotZ on every qubit and a CX ring
    per layer; angles seeded) in tile passes at every fusion width, on the
    CUDA cores (register phases) and, for widths >= 3, with the fused
    unitaries on the tensor cores: ms per run and passes (launches) per run,
    from |0...0>."""
    import afquantumsim_gb300 as aq
    from afquantumsim_gb300 import circuits
    params = np.random.default_rng(1).uniform(-np.pi, np.pi, size=(layers, n, 2)).astype(np.float32)
    ops = aq.op_array(circuits.vqe_ansatz(n, layers, params))
    res = {"workload": f"vqe_ansatz{n}x{layers}", "gates": len(ops), "runs": {}}
    with aq.State(ctx, n, aq.C64) as st:
        st.set_basis(0)
        for fuse in range(0, 6):
            for tc in ((False, True) if fuse >= 3 else (False,)):
                ctx.set_tensor_cores(tc)
                prog = aq.Program(n, ops, max_qubits=fuse) if fuse else None
                run = (lambda: prog.run(st, aq.EXEC_TILED)) if prog else (lambda: st.apply(ops, aq.EXEC_TILED))
                run()
                l0 = ctx.launch_count()
                ms = _time_ms(stream, run, reps)
                key = f"fuse{fuse}{'_tc' if tc else ''}"
                res["runs"][key] = {"ms": round(ms, 3), "launches": (ctx.launch_count() - l0) // reps,
                                    "ops": prog.info()[0] if prog else len(ops)}
                if prog:
                    prog.free()
        ctx.set_tensor_cores(True)
    best = min(res["runs"], key=lambda k: res["runs"][k]["ms"])
    res["best"] = best
    return res


def bench_plain12(ctx, stream, n=12, layers=10):
    """The 12-qubit plain-method workload (H layer, then 10 layers of seeded
    random RotX/RotY/RotZ + CX chain) with a 1000-shot histogram: one launch
    in tiled mode (the register is one shared-memory tile) vs one gate per
    pass; end to end through the C ABI; and the reference ALGORITHM (faithful
    FP32 restatement: dense Kronecker / CSR operators) on the host."""
    import time as _t

    import afquantumsim_gb300 as aq
    from afquantumsim_gb300 import circuits
    from oracle import oracle
    ops = aq.op_array(circuits.plain_layers(n, layers, seed=1))
    res = {"workload": f"plain{n}x{layers}", "gates": len(ops)}
    with aq.State(ctx, n, aq.C64) as s:
        def run(mode):
            s.set_basis(0)
            s.apply(ops, mode)
        run(aq.EXEC_TILED)
        res["tiled_us"] = round(1e3 * _time_ms(stream, lambda: run(aq.EXEC_TILED), 200), 2)
        run(aq.EXEC_PER_GATE)
        res["per_gate_us"] = round(1e3 * _time_ms(stream, lambda: run(aq.EXEC_PER_GATE), 20), 2)
        u = np.random.default_rng(2).random(1000)
        t0 = _t.perf_counter()
        reps = 50
        for _ in range(reps):
            run(aq.EXEC_TILED)
            sv = s.download()
            counts = np.bincount(s.sample(u).astype(np.int64), minlength=1 << n)
        res["e2e_us_per_simulate_sv_and_1000_shots"] = round(1e6 * (_t.perf_counter() - t0) / reps, 1)
    v = np.zeros(1 << n, dtype=np.complex64)
    v[0] = 1
    t0 = _t.perf_counter()
    ref = oracle.ref32_apply(v, n, list(ops))
    res["reference_algorithm_s"] = round(_t.perf_counter() - t0, 3)
    res["reference_algorithm_threads"] = oracle.threads()
    res["max_abs_diff_vs_reference_algorithm"] = float(np.max(np.abs(ref - sv)))
    res["shots_total"] = int(counts.sum())
    return res


def bench_vqe_batch(ctx, count=4096, seed=5):
    """The batched VQE sweep: `count` hardware-efficient-ansatz circuits
    (qubits uniform in 8..20, layers uniform in 4..12, angles uniform in
    [-pi, pi], seed 5), each to <Z_q> and <Z_q Z_q+1> in FP64, as one
    CUDA-graph replay; then new angles for every circuit and another replay.
    CPU baseline: the FP64 per-gate oracle on every 64th circuit, all host
    threads, scaled to the sweep by amplitude-gate work."""
    import time as _t

    import afquantumsim_gb300 as aq
    from afquantumsim_gb300 import circuits
    from oracle import oracle
    items = circuits.vqe_sweep(count, seed=seed)
    gates = sum(len(ops) for _, ops in items)
    work = sum(len(ops) * (1 << n) for n, ops in items)
    t0 = _t.perf_counter()
    b = aq.Batch(ctx, items)
    create_s = _t.perf_counter() - t0
    info = b.info()
    b.run()
    b.run()
    reps = 5
    t0 = _t.perf_counter()
    for _ in range(reps):
        z, zz = b.run()
    sweep_s = (_t.perf_counter() - t0) / reps
    # one more replay inside an NVTX range "vqe_sweep", untimed: the range an
    # ncu launch list of one sweep filters on
    import torch
    torch.cuda.nvtx.range_push("vqe_sweep")
    b.run()
    torch.cuda.nvtx.range_pop()
    rng = np.random.default_rng(seed + 1)

    def new_angles():
        out = []
        for n, ops in items:  # same shapes (n >= 8: 3n ops per layer), new angles
            L = len(ops) // (3 * n)
            out.append((n, circuits.vqe_ops_array(n, L, rng.uniform(-np.pi, np.pi, size=(L, n, 2)))))
        return out

    # the first update after creation, then one in steady state (what an
    # optimiser loop pays per step), followed by its run
    first, new = new_angles(), new_angles()
    t0 = _t.perf_counter()
    b.update(first)
    first_update_s = _t.perf_counter() - t0
    t0 = _t.perf_counter()
    b.update(new)
    update_s = _t.perf_counter() - t0
    z, zz = b.run()
    update_run_s = _t.perf_counter() - t0
    # accuracy on a sample against the FP64 oracle
    err = 0.0
    sample = list(range(0, count, 64))
    threads = len(os.sched_getaffinity(0))
    oracle.set_threads(threads)
    cpu_s = 0.0
    cpu_work = 0
    for i in sample:
        n, ops = new[i]
        v = np.zeros(1 << n, dtype=np.complex128)
        v[0] = 1
        olist = list((aq.Op * len(ops)).from_buffer_copy(ops.tobytes()))
        t0 = _t.perf_counter()
        v = oracle.apply_f64(v, olist)
        cpu_s += _t.perf_counter() - t0
        cpu_work += len(ops) * (1 << n)
        p = np.abs(v) ** 2
        idx = np.arange(1 << n)
        wz = np.array([np.sum(p * (1 - 2 * ((idx >> (n - 1 - q)) & 1))) for q in range(n)])
        err = max(err, float(np.max(np.abs(wz - z[i]))))
    b.free()
    cpu_sweep_est = cpu_s * work / cpu_work
    from collections import Counter
    tuned = Counter(f"fuse{f}{'_tc' if t else ''}" for f, t in zip(info["fuse_qubits"], info["tensor_cores"]))
    peak, peak_src = measured_peaks()
    hbm = {"bytes_per_sweep": info["hbm_bytes"], "achieved_gbs": round(info["hbm_bytes"] / sweep_s / 1e9, 1),
           "peak_gbs": peak, "frac": round(info["hbm_bytes"] / sweep_s / 1e9 / peak, 4), "peak_source": peak_src,
           "note": "registers of > 14 qubits: clear, one read + one write per tile pass, expectation read; "
                   "registers of <= 14 qubits stay in shared memory"}
    return {"workload": f"vqe_sweep{count}", "gates": gates, "small_circuits": info["small"],
            "large_circuits": info["large"], "kernels_per_replay": info["kernels"], "hbm": hbm,
            "large_circuit_tuning": dict(tuned),
            "create_s": round(create_s, 3), "sweep_ms": round(1e3 * sweep_s, 3),
            "circuits_per_s": round(count / sweep_s, 1), "gate_apps_per_s": round(gates / sweep_s, 1),
            "first_update_ms": round(1e3 * first_update_s, 3), "update_ms": round(1e3 * update_s, 3),
            "update_and_run_ms": round(1e3 * update_run_s, 3),
            "max_abs_err_z_vs_fp64_sample": err,
            "cpu_baseline": {"kind": "port", "cores": threads, "sample": f"{len(sample)} circuits (every 64th)",
                             "sample_s": round(cpu_s, 3), "sweep_s_scaled": round(cpu_sweep_est, 2)}}


def serving_requests(count, seed=6):
    """The serving stream's requests: brick-work circuits (Haar SU(2) as
    RotZ.RotY.RotZ + CZ layers) with qubits uniform in 10..28 and depth
    uniform in 5..30, each with its own sampling seed."""
    import afquantumsim_gb300 as aq
    from afquantumsim_gb300 import circuits
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        n = int(rng.integers(10, 29))
        d = int(rng.integers(5, 31))
        reqs.append((n, aq.op_array(circuits.brickwork(n, d, seed=10_000 + i)), int(rng.integers(1 << 40))))
    return reqs


def bench_serving(ctx, count=160, seed=6, shots=1024, fuse=5, lanes=8, budget_gib=32, load=0.7):
    """The serving loop: `count` requests through aqsg_server (HBM slab of
    `budget_gib` GiB cut by register size 2^n x 8 B, `lanes` concurrent
    lanes, fusion width `fuse`, 1024 seeded shots each).  First every request
    arrives at t = 0 (capacity, circuits/s); then the same requests arrive as
    a Poisson stream (seed 6) at `load` x that capacity, and latency
    (arrival -> outcomes on the host) is reported as p50/p99.  Accuracy: the
    fused c64 state of the three smallest requests against the same circuit
    one gate per pass in c128 (the server's outcomes are those of the direct
    path, which the tests check bit for bit)."""
    import time as _t

    import afquantumsim_gb300 as aq
    t0 = _t.perf_counter()
    reqs = serving_requests(count, seed)
    gen_s = _t.perf_counter() - t0
    gates = sum(len(o) for _, o, _ in reqs)

    def run(arrivals):
        srv = aq.Server(0, aq.C64, budget_gib << 30, lanes, 28, shots)
        t1 = _t.perf_counter()
        for (n, ops, sd), a in zip(reqs, arrivals):
            srv.submit(n, ops, shots, sd, float(a), fuse)
        submit_s = _t.perf_counter() - t1
        srv.start()
        srv.wait_idle(900)
        done = srv.poll(count + 8)
        stats = srv.stats()
        srv.close()
        assert len(done) == count and all(d["status"] == 0 for d in done)
        lat = np.array([d["done_s"] - d["arrival_s"] for d in done])
        span = max(d["done_s"] for d in done) - min(d["arrival_s"] for d in done)
        peak, peak_src = measured_peaks()
        hbm = {"bytes": stats["hbm_bytes"], "achieved_gbs": round(stats["hbm_bytes"] / span / 1e9, 1),
               "peak_gbs": peak, "frac": round(stats["hbm_bytes"] / span / 1e9 / peak, 4), "peak_source": peak_src}
        return {"hbm": hbm, "circuits_per_s": round(count / span, 2), "gate_apps_per_s": round(gates / span, 1),
                "makespan_s": round(span, 3), "p50_latency_ms": round(1e3 * float(np.percentile(lat, 50)), 2),
                "p99_latency_ms": round(1e3 * float(np.percentile(lat, 99)), 2),
                "peak_running": stats["peak_running"], "peak_slab_gib": round(stats["peak_bytes"] / 2**30, 2),
                "host_submit_s": round(submit_s, 2), "kernel_launches": stats["launches"]}

    sat = run(np.zeros(count))
    rate = load * sat["circuits_per_s"]
    arrivals = np.cumsum(np.random.default_rng(seed).exponential(1.0 / rate, size=count))
    poisson = run(arrivals)
    poisson["arrival_rate_per_s"] = round(rate, 2)
    err = 0.0
    for n, ops, _ in sorted(reqs, key=lambda r: r[0])[:3]:
        prog = aq.Program(n, list(ops), aq.C64, max_qubits=fuse)
        with aq.State(ctx, n, aq.C64) as a, aq.State(ctx, n, aq.C128) as b:
            a.set_basis(0)
            prog.run(a, aq.EXEC_TILED)
            b.set_basis(0)
            b.apply(ops, aq.EXEC_PER_GATE)
            err = max(err, a.compare(b)[0])
        prog.free()
    return {"workload": f"serving{count}_brickwork_n10-28_d5-30", "shots": shots, "fuse_qubits": fuse,
            "lanes": lanes, "hbm_budget_gib": budget_gib, "gates": gates, "requests_gen_s": round(gen_s, 2),
            "saturated": sat, "poisson": poisson, "max_abs_err_vs_fp64_3_smallest": err}


# ---- our arm ------------------------------------------------------------------------

def run_ours(args, rank, world, local_rank):
    import torch
    import afquantumsim_gb300 as aq
    from afquantumsim_gb300 import replicas

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    n = args.n
    N = 1 << n
    dt_np = np.complex64 if args.dtype == "c64" else np.complex128
    dt_t = torch.complex64 if args.dtype == "c64" else torch.complex128
    amp_b = 8 if args.dtype == "c64" else 16
    mode = aq.EXEC_PER_GATE if args.mode == "per_gate" else aq.EXEC_TILED

    ctx = aq.Context(local_rank)
    st = aq.State(ctx, n, aq.C64 if args.dtype == "c64" else aq.C128)

    # seeded input, normalised, staged in pinned host memory (not timed)
    g = torch.Generator(device=dev)
    g.manual_seed(replicas.rank_seed(3, rank))
    x = torch.randn(N, dtype=dt_t, device=dev, generator=g)
    x /= torch.linalg.vector_norm(x)
    host_in = torch.empty(N, dtype=dt_t, pin_memory=True)
    host_in.copy_(x)
    del x
    torch.cuda.synchronize()
    host_out = torch.empty(N, dtype=dt_t, pin_memory=True)

    ops = aq.op_array(qft_ops(n))
    total_bytes, per_kind, counts = algorithmic_bytes(n, amp_b)
    gates = len(ops)

    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=dev)

    st.upload_ptr(host_in.data_ptr())
    for _ in range(args.warmup):
        st.apply(ops, mode)
    ctx.synchronize()

    uuid = None
    try:
        uuid = str(torch.cuda.get_device_properties(local_rank).uuid)
    except Exception:
        pass

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(uuid) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            st.apply(ops, mode)
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize()
    launches = ctx.launch_count() - launches0
    ms = ev0.elapsed_time(ev1)
    ms, total_gates = replicas.reduce_timing(ms, gates * args.steps, dev if world > 1 else None)
    if world > 1:
        torch.distributed.barrier()
    ms_per_step = ms / args.steps
    value = total_gates / (ms / 1e3)
    hbm_gbs = total_gates / gates * total_bytes / (ms / 1e3) / 1e9

    # dominant kernel in isolation: the controlled-phase pass (N/4 amplitudes)
    cp_ops = aq.op_array([o for o in qft_ops(n) if o.kind == aq.kinds.CPHASE])
    h_ops = aq.op_array([o for o in qft_ops(n) if o.kind == aq.kinds.H])
    sw_ops = aq.op_array([o for o in qft_ops(n) if o.kind == aq.kinds.SWAP])

    def per_launch_ms(arr, reps=1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        st.apply(arr, aq.EXEC_PER_GATE)
        e0.record(stream)
        for _ in range(reps):
            st.apply(arr, aq.EXEC_PER_GATE)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / (reps * len(arr))

    cp_ms = per_launch_ms(cp_ops)
    h_ms = per_launch_ms(h_ops, 2)
    sw_ms = per_launch_ms(sw_ops, 2)
    peak, peak_kind = measured_peaks()
    cp_achieved = per_kind["CPhase"] / (cp_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": "k_diag1 (CPhase pass)",
                "achieved": round(cp_achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(cp_achieved / peak, 4), "peak_source": peak_kind,
                "traffic": traffic_per_launch(n, args.dtype),
                "traffic_note": "ncu mean over the 378 CPhase launches of a 28-qubit QFT, scaled by 2^(n-28)",
                "algorithmic_bytes_per_launch": per_kind["CPhase"],
                "ms_per_launch": round(cp_ms, 4)}
    kernels = {
        "H_pass": {"ms": round(h_ms, 4), "GBps": round(per_kind["H"] / (h_ms / 1e3) / 1e9, 1)},
        "CPhase_pass": {"ms": round(cp_ms, 4), "GBps": round(cp_achieved, 1)},
        "Swap_pass": {"ms": round(sw_ms, 4), "GBps": round(per_kind["Swap"] / (sw_ms / 1e3) / 1e9, 1)},
    }

    # end to end through the C ABI with host buffers.  Per step: upload the
    # step's input from pinned host memory, run the circuit, copy its result
    # to pinned host memory.  Two registers on two contexts (streams) take the
    # steps in turn: a step's upload and the previous step's result copy
    # overlap the gates of the other register, and aqsg_ctx_after keeps the
    # two registers' gates one after the other (HBM-bound passes of two
    # registers interleaved run slower than back to back).
    e2e_steps = max(8, args.steps)  # the first upload and the last read-back are not hidden
    ctx2 = aq.Context(local_rank)
    st2 = aq.State(ctx2, n, aq.C64 if args.dtype == "c64" else aq.C128)
    host_out2 = torch.empty(N, dtype=dt_t, pin_memory=True)
    lanes = [(ctx, st, host_out), (ctx2, st2, host_out2)]
    for c, r, ho in lanes:  # warm-up
        r.upload_ptr(host_in.data_ptr())
        r.apply(ops, mode)
        r.download_async_ptr(ho.data_ptr())
        c.synchronize()
    # the host link's copy rate on this run (the pipeline hides the copies
    # only while each takes less than a step's gates)
    t_c = time.perf_counter()
    st.upload_ptr(host_in.data_ptr())
    ctx.synchronize()
    h2d_s = time.perf_counter() - t_c
    t_c = time.perf_counter()
    st.download_async_ptr(host_out.data_ptr())
    ctx.synchronize()
    d2h_s = time.perf_counter() - t_c
    # events on each register's stream around its gate batches, the first
    # upload and the last result copy: where the end-to-end time goes
    lane_streams = [stream, torch.cuda.ExternalStream(ctx2.stream_handle(), device=dev)]

    def mark(li):
        e = torch.cuda.Event(enable_timing=True)
        e.record(lane_streams[li])
        return e

    gate_ev = []
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for step in range(e2e_steps):
        li = step % 2
        c, r, ho = lanes[li]
        c.synchronize()  # this register's previous step (its result copy) is done
        if step == 0:
            up0 = mark(li)
        r.upload_ptr(host_in.data_ptr())
        if step > 0:
            pc, pr, pho = lanes[(step - 1) % 2]
            c.after(pc)  # after the previous step's gates (its queue holds nothing else)
            g0 = mark(li)
            r.apply(ops, mode)
            gate_ev.append((g0, mark(li)))
            pr.download_async_ptr(pho.data_ptr())  # previous result, under this step's gates
        else:
            g0 = mark(li)
            r.apply(ops, mode)
            gate_ev.append((g0, mark(li)))
    li = (e2e_steps - 1) % 2
    c, r, ho = lanes[li]
    r.download_async_ptr(ho.data_ptr())
    down_end = mark(li)
    ctx.synchronize()
    ctx2.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_gates_ms = sum(a.elapsed_time(b) for a, b in gate_ev)
    e2e_span_ms = up0.elapsed_time(down_end)
    e2e_first_upload_ms = up0.elapsed_time(gate_ev[0][0])
    e2e_last_copy_ms = gate_ev[-1][1].elapsed_time(down_end)
    st2.free()
    ctx2.close()
    if world > 1:
        t = torch.tensor([e2e_s], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": round(world * gates * e2e_steps / e2e_s, 3), "unit": "gate-apps/s",
           "h2d_bytes_per_step": N * amp_b, "d2h_bytes_per_step": N * amp_b,
           "ms_per_step": round(e2e_s / e2e_steps * 1e3, 3), "steps": e2e_steps,
           "h2d_gbs": round(N * amp_b / h2d_s / 1e9, 1), "d2h_gbs": round(N * amp_b / d2h_s / 1e9, 1),
           # device time of the loop (first upload to last result copy), of
           # its gate batches, and the copies that no gates hide
           "device_span_ms": round(e2e_span_ms, 1), "gates_ms_per_step": round(e2e_gates_ms / e2e_steps, 2),
           "first_upload_ms": round(e2e_first_upload_ms, 1), "last_copy_ms": round(e2e_last_copy_ms, 1),
           "pipeline": "two registers on two streams, gates of consecutive steps ordered (aqsg_ctx_after); "
                       "each step uploads its input and reads its result under the other register's gates"}

    # accuracy of one step against FP64: the circuit applied once to the
    # seeded input, against the same gates applied to it in complex128 with
    # PyTorch's own operations (tests/fp64_torch.py, which the tests pin to
    # the C oracle); both compared on the device
    from tests import fp64_torch
    st.upload_ptr(host_in.data_ptr())
    st.apply(ops, mode)
    st.download_ptr(host_out.data_ptr())
    want = fp64_torch.apply_ops(host_in.to(dev).to(torch.complex128), n, qft_ops(n))
    accuracy = fp64_torch.errors(host_out.to(dev), want)
    del want
    torch.cuda.empty_cache()

    extras = {}
    if not args.no_extras and rank == 0:
        # the same circuit in shared-memory tiled mode, for comparison
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        st.apply(ops, aq.EXEC_TILED)
        e0.record(stream)
        for _ in range(2):
            st.apply(ops, aq.EXEC_TILED)
        e1.record(stream)
        e1.synchronize()
        extras["tiled_ms_per_step"] = round(e0.elapsed_time(e1) / 2, 3)
        if args.dtype == "c64":
            extras["fused_brickwork"] = bench_fused_brickwork(ctx, st, stream, n, depth=20)
        extras["qft_grid"] = bench_qft_grid(ctx, stream)
        extras["plain12"] = bench_plain12(ctx, stream)
        extras["tile_shape"] = bench_tile_shape(ctx)
        extras["vqe_batch"] = bench_vqe_batch(ctx)
        extras["noise"] = bench_noise(ctx)
        if args.dtype == "c64":
            extras["serving"] = bench_serving(ctx)

    cpu = None
    if rank == 0:
        host_np = host_out.numpy()  # scratch register for the CPU sample
        cpu = cpu_baseline(n, host_np, qft_cpu_sample(n), args.dtype,
                           "every 15th gate of each kind of the same circuit (its gate mix)")
        if not args.no_extras:
            extras["reference_algorithm_qft12"] = reference_algorithm_small(12)

    st.free()
    ctx.close()
    if rank != 0:
        return None
    return {
        "metric": metric_name(n, args.dtype),
        "value": round(value, 3),
        "unit": "gate-apps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": args.dtype,
        "data": "synthetic (seeded standard-normal complex amplitudes)",
        "config": workload_config(n, args.dtype, world),
        "exec_mode": args.mode,
        "max_abs_err_vs_fp64": accuracy["max_abs_err"],
        "l2_err_vs_fp64": accuracy["l2_err"],
        "one_minus_fidelity": accuracy["one_minus_fidelity"],
        "accuracy_reference": "one step on the seeded input against the same gates in complex128 "
                              "(PyTorch operations, pinned to the C oracle by the tests)",
        "hbm_gbs": round(hbm_gbs, 1),
        "hbm_frac": round(hbm_gbs / world / measured_peaks()[0], 4),
        "algorithmic_bytes_per_step": total_bytes,
        "e2e": e2e,
        "roofline": roofline,
        "kernels": kernels,
        "cpu_baseline": {k: v for k, v in cpu.items() if k != "seconds"},
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
        "extras": extras,
    }


# Mean DRAM bytes (read + write) per controlled-phase launch over the 378
# CPhase launches of one 28-qubit complex64 QFT, from an ncu capture of
# dram__bytes_read.sum + dram__bytes_write.sum.  Traffic grows with the
# register (2^n), so other sizes scale it.
CPHASE_TRAFFIC_C64_28Q = 1256.4e6


def traffic_per_launch(n, dtype):
    if dtype != "c64":
        return None
    return round(CPHASE_TRAFFIC_C64_28Q * 2.0 ** (n - 28))


def run_reference(args):
    """CPU implementation of the path (the per-gate oracle port, all host
    threads) on the same workload: the same seeded 2^n register, and step s
    times the s-th contiguous slice of the circuit's gates, so that the K
    steps together run the whole circuit once, in order (each step holds
    ceil(gates / K) gates; steps past the end of the circuit start it
    again).  A warm-up step runs one gate."""
    import afquantumsim_gb300 as aq
    n = args.n
    N = 1 << n
    dt_np = np.complex64 if args.dtype == "c64" else np.complex128
    rng = np.random.default_rng(3)
    sv = np.empty(N, dtype=dt_np)
    chunk = 1 << 24
    for i in range(0, N, chunk):
        m = min(chunk, N - i)
        sv[i:i + m] = (rng.standard_normal(m) + 1j * rng.standard_normal(m)).astype(dt_np)
    sv /= np.sqrt(np.vdot(sv, sv).real)
    ops = qft_ops(n)
    gates = len(ops)
    for _ in range(args.warmup):
        cpu_baseline(n, sv, ops[:1], args.dtype, "warm-up")
    per = -(-gates // max(args.steps, 1))
    res, timed = [], 0
    for s_ in range(args.steps):
        lo = (s_ * per) % gates
        sl = ops[lo:lo + per]
        res.append(cpu_baseline(n, sv, sl, args.dtype, f"gates {lo}..{lo + len(sl) - 1}"))
        timed += len(sl)
    tot_s = sum(r["seconds"] for r in res)
    value = timed / tot_s
    kinds = {}
    for o in ops[:timed] if timed <= gates else ops:
        kinds[o.kind] = kinds.get(o.kind, 0) + 1
    sample = (f"the whole {gates}-gate circuit once in order, {per} gates per step over {args.steps} steps "
              f"({timed} gates: {kinds.get(aq.kinds.H, 0)} H, {kinds.get(aq.kinds.CPHASE, 0)} CPhase, "
              f"{kinds.get(aq.kinds.SWAP, 0)} Swap), {args.dtype}, {tot_s:.1f} s")
    cb = {"value": value, "unit": "gate-apps/s", "cores": res[0]["cores"], "kind": "port", "sample": sample}
    return {
        "impl": "reference",
        "metric": metric_name(n, args.dtype),
        "value": round(value, 4),
        "unit": "gate-apps/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(tot_s / args.steps * 1e3, 1),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": args.dtype,
        "data": "synthetic (seeded standard-normal complex amplitudes)",
        "config": workload_config(n, args.dtype, args.gpus),
        "exec_mode": "cpu per-gate (oracle port)",
        "sample": sample,
        "cpu_baseline": cb,
        "e2e": {"value": round(value, 4), "unit": "gate-apps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def run_only(args):
    import torch
    import afquantumsim_gb300 as aq
    ctx = aq.Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=torch.device("cuda", 0))
    if args.only == "fused_brickwork":
        with aq.State(ctx, args.n, aq.C64) as st:
            res = bench_fused_brickwork(ctx, st, stream, args.n, args.depth)
    elif args.only == "fused_tc":
        res = bench_fused_tc(ctx, stream, args.n, args.depth)
    elif args.only == "fused_cc":
        res = bench_fused_cc(ctx, stream, args.n, args.depth)
    elif args.only == "tiled_brickwork":
        res = bench_tiled_brickwork(ctx, stream, args.n, args.depth)
    elif args.only == "plain12":
        res = bench_plain12(ctx, stream)
    elif args.only == "noise":
        res = bench_noise(ctx)
    elif args.only == "qft_grid":
        res = bench_qft_grid(ctx, stream)
    elif args.only == "tile_shape":
        res = bench_tile_shape(ctx)
    elif args.only == "vqe_batch":
        res = bench_vqe_batch(ctx, count=args.count or 4096)
    elif args.only == "vqe_ansatz":
        res = bench_vqe_ansatz(ctx, stream, n=args.n, layers=args.depth)
    else:
        res = bench_serving(ctx, count=args.count or 160)
    ctx.close()
    return res


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.only:
        print(json.dumps(run_only(args)), flush=True)
        return 0
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args)), flush=True)
        return 0
    if world > 1:
        import torch
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    out = run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
