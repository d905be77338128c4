"""Benchmark: 30-qubit complex128 forward (gate applies/s) on one GB300.

Workload (the forward that the headline metric is quoted on): 30 qubits,
complex128 (17.2 GB statevector), Hadamard on every qubit then 20 layers of
[RX, RY, RZ on every qubit; CNOT i->i+1], angles uniform [0, 2pi) from seed
1: 2410 gates, fusion windows on. A step is one reset to |0...0> plus the
forward of all 2410 gates with the state resident in HBM; `value` = gates /
step time (CUDA events on the library's stream, max over ranks). The state
(17.2 GB) is larger than L2 (129 MB), so no flush is needed between steps.

`e2e` runs the same forward through the Circuit API with host buffers: per
step the parameters are set from a pinned host array (the gate list is
uploaded), the forward runs, and the whole statevector comes back to pinned
host memory as split real/imaginary arrays (the reference's
retrieve_amplitudes_on_host layout, which its forward() performs every call).

`adjoint` reports the adjoint-gradient part of the metric on the 24-qubit,
1152-parameter ring ansatz (loss sum_q w_q <Z_q>, params seed 2, weights
seed 3): adjoint grads/s, and parameter shift timed on a sample of the
parameters through the same GPU kernels.

`--impl reference` times the CPU oracle (a C/OpenMP restatement of the
reference's multithreading path) on the host cores on a bounded sample of the
same workload. Under torchrun every rank runs an independent replica
(the path does not shard on one node here); rank 0 prints the JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "30-qubit gate applies/s + HBM GB/s; adjoint vs param-shift grads/s at 1e-10"
UNIT = "gate-applies/s"
DTYPES = {"fp64": "f64 (complex128 storage, IEEE FP64 arithmetic; fused passes as real rotations, one "
                  "multiply-add per output with their factors multiplied back once, and per-amplitude phase "
                  "tables)",
          "fp64-direct": "f64 (complex128 storage, IEEE FP64 arithmetic; every fused 2x2 as a full complex "
                         "multiply-add)",
          "fp32x2": "f32x2 (complex128 storage, FP32-pair arithmetic, ~48-bit)",
          "int64": "int64 (complex128 storage, block fixed point: 54-bit fraction per tile, exact products)",
          "tc": "int64 (complex128 storage, block fixed point: 56-bit fraction per tile; fused gates as dense "
                "5-qubit blocks, exact products of FP16 digits on the tcgen05 tensor cores)"}
# Integer multiply-add (IMAD) throughput of a GB300 measured with an independent-chain kernel.
INT_MAD_PEAK_T = 18.85
# FP64 multiply-add throughput of a GB300 measured with an independent-FMA-chain kernel
# (0.504 T FMA/s = 1.0 TFLOP/s); complex128 arithmetic is bounded by it.
FP64_FMA_PEAK_T = 0.504
FP32_FMA_PEAK_T = 35.9
# dram__bytes_read.sum + dram__bytes_write.sum per launch divided by the amplitudes of
# the captured case: one ncu capture per kernel on a smaller state of the same ladder
# workload (dram__bytes.sum.per_second x gpu__time_duration.sum: k_window_tma<PolF64>
# 479.1 MB at 2^24 amplitudes; k_window_phases<PolF32> 1012.4 MB at 2^26; k_window_tc
# 476.1 MB at 2^24; k_apply_window<PolDF> 492.7 MB and k_apply_window<PolFX> 493.1 MB at
# 2^24). Traffic is the state read plus written once per pass, so it scales with the
# number of amplitudes.
NCU_TRAFFIC_PER_AMPLITUDE = {("window", "c128"): 479.1e6 / (1 << 24),
                             ("window", "c64"): 1012.4e6 / (1 << 26),
                             ("window", "c128", "tc"): 476.1e6 / (1 << 24),
                             ("window", "c128", "fp32x2"): 492.7e6 / (1 << 24),
                             ("window", "c128", "int64"): 493.1e6 / (1 << 24)}
# The kernel that runs a fused window pass, by arithmetic and precision.
WINDOW_KERNEL = {("fp64", "c128"): "k_window_tma<PolF64>", ("fp64-direct", "c128"): "k_window_tma<PolF64>",
                 ("fp32x2", "c128"): "k_apply_window<PolDF>",
                 ("int64", "c128"): "k_apply_window<PolFX>", ("tc", "c128"): "k_window_tc",
                 ("fp32", "c64"): "k_window_phases<PolF32>"}


def load_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_tensor_peak():
    """Dense bf16 tensor throughput (TFLOP/s) sustained over a seconds-long loop: the window
    passes run back to back inside a multi-second forward."""
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["bf16_tflops_sustained"]), "measured (cuBLAS bf16, sustained)"
    except Exception:
        return 1700.0, "fallback (sustained)"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ reference
def workloads_standalone():
    """damavand_gb300/workloads.py loaded by file path, outside the package: importing the
    package maps libdamavand_gpu.so, which the CPU reference arm must not load."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("dmv_workloads_standalone",
                                                  os.path.join(REPO, "damavand_gb300", "workloads.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def run_reference(args, world, rank):
    """CPU oracle (port of the reference's multithreading path) on the host cores."""
    if rank != 0:
        return None
    wl = workloads_standalone()
    count, ladder_circuit = wl.count, wl.ladder_circuit
    from oracle import oracle
    oracle.build()
    n = args.qubits
    gates = [g for g in ladder_circuit(n, args.layers, seed=1) if not g[3]]
    state = oracle.zero_state(n)
    per_step = args.ref_gates
    pos = 0

    def step():
        nonlocal pos, state
        sel = [gates[(pos + i) % len(gates)] for i in range(per_step)]
        pos += per_step
        t0 = time.perf_counter()
        oracle.forward(n, sel, state)
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        step()
    times = [step() for _ in range(args.steps)]
    total = sum(times)
    value = per_step * args.steps / total
    threads = oracle.num_threads()
    sample = (f"{per_step} consecutive gates of the {count(gates)}-gate {n}-qubit forward per step "
              f"(clone + per-amplitude update per gate, as the reference does)")
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 (complex128)", "data": "synthetic",
        "impl": "reference",
        "config": workload_config(args, count(gates)),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def workload_config(args, gates):
    return {"workload": f"{args.qubits}-qubit complex128 forward: H on all qubits + {args.layers} x "
                        f"[RX,RY,RZ per qubit; CNOT i->i+1], angles U[0,2pi) seed 1",
            "qubits": args.qubits, "gates": gates, "layers": args.layers, "precision": "complex128",
            "arithmetic": args.arith,
            "fusion": "qubit windows" if not args.no_fusion else "none",
            "l2": "inputs larger than L2 (statevector 2^n x 16 B), no flush", "parallelism": "replicas"}


# ------------------------------------------------------------------------ ours
def cpu_baseline(args):
    """Times the oracle on a bounded sample at the bench's size on the host cores."""
    from damavand_gb300.workloads import ladder_circuit
    from oracle import oracle
    oracle.build()
    n = args.qubits
    gates = [g for g in ladder_circuit(n, args.layers, seed=1) if not g[3]]
    state = oracle.zero_state(n)
    done, t0 = 0, time.perf_counter()
    while done < len(gates) and (time.perf_counter() - t0) < args.cpu_seconds:
        oracle.forward(n, [gates[done]], state)
        done += 1
    el = time.perf_counter() - t0
    cores = oracle.num_threads()
    # the same port on one host core: the next gate of the forward
    single = None
    if done < len(gates):
        oracle.set_num_threads(1)
        try:
            t1 = time.perf_counter()
            oracle.forward(n, [gates[done]], state)
            el1 = time.perf_counter() - t1
        finally:
            oracle.set_num_threads(cores)
        single = {"value": 1.0 / el1, "unit": UNIT, "cores": 1,
                  "sample": f"gate {done + 1} of the same forward on one thread ({el1:.1f} s)"}
    del state
    return {"value": done / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"first {done} gates of the {len(gates)}-gate {n}-qubit forward ({el:.1f} s)",
            "single_core": single}


def adjoint_section(args):
    from damavand_gb300 import Circuit
    from damavand_gb300._lib import KERNEL_ADJOINT
    from damavand_gb300.workloads import add_to_circuit, loss_weights, parameters, ring_ansatz
    n, layers = 24, 16
    gates = ring_ansatz(n, layers, seed=2)
    w = loss_weights(n, 3)
    p = parameters(gates)
    c = Circuit(n)
    add_to_circuit(c, gates)
    c.adjoint_gradient(w)  # warm-up
    t0 = time.perf_counter()
    reps = 2
    for _ in range(reps):
        loss, g = c.adjoint_gradient(w)
    t_adj = (time.perf_counter() - t0) / reps
    # parameter shift on the same GPU kernels, on a sample of parameters
    k = min(args.ps_params, p.size)
    idx = np.linspace(0, p.size - 1, k).astype(int)
    ps = np.empty(k)
    t0 = time.perf_counter()
    for j, i in enumerate(idx):
        up, dn = p.copy(), p.copy()
        up[i] += math.pi / 2
        dn[i] -= math.pi / 2
        c.set_parameters(up)
        lu = c.loss(w)
        c.set_parameters(dn)
        ld = c.loss(w)
        ps[j] = 0.5 * (lu - ld)
    t_ps_per_param = (time.perf_counter() - t0) / k
    c.set_parameters(p)
    t_ps = t_ps_per_param * p.size
    out = {"qubits": n, "params": int(p.size), "gates": len(gates), "adjoint_s": t_adj,
           "adjoint_grads_per_s": p.size / t_adj, "param_shift_s_extrapolated": t_ps,
           "param_shift_grads_per_s": p.size / t_ps, "param_shift_sampled_params": int(k),
           "speedup_vs_param_shift": t_ps / t_adj, "max_abs_diff_vs_param_shift": float(np.max(np.abs(g[idx] - ps))),
           "loss": loss}
    # The same sweep in the other complex128 arithmetics (psi and lambda updates in that
    # arithmetic; FP32 pairs also form the gradient terms), checked against the FP64 gradient.
    alts = {}
    for arith in ("fp32x2", "int64"):
        ca = Circuit(n, arithmetic=arith)
        add_to_circuit(ca, gates)
        ca.adjoint_gradient(w)  # warm-up
        t0 = time.perf_counter()
        for _ in range(reps):
            la, ga = ca.adjoint_gradient(w)
        ta = (time.perf_counter() - t0) / reps
        alts[arith] = {"adjoint_s": ta, "adjoint_grads_per_s": p.size / ta, "speedup_vs_fp64_adjoint": t_adj / ta,
                       "max_abs_diff_vs_fp64_grads": float(np.max(np.abs(ga - g))), "loss_diff": abs(la - loss)}
        del ca
    out["alt_arithmetic"] = alts
    if not args.no_cpu:
        # The reference has no gradient; its route is parameter shift (circuit.rs:529-546):
        # two CPU forwards (clone per gate) per parameter. One loss evaluation timed here.
        from oracle import oracle
        oracle.build()
        og = [(kk, t, cc, int(o), th) for kk, t, cc, o, th in gates]
        t0 = time.perf_counter()
        oracle.loss(n, og, p, w, clone=True)
        t_loss = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / (2.0 * t_loss), "unit": "grads/s", "cores": oracle.num_threads(),
                               "kind": "port", "extrapolated": True,
                               "sample": f"one oracle loss evaluation ({n} qubits, {len(gates)} gates, clone per gate: "
                                         f"{t_loss:.1f} s); parameter shift needs two per parameter, "
                                         f"{2 * t_loss * p.size:.0f} s for all {p.size}"}
    return out


def normwise_err(got, ref, chunk: int = 1 << 26) -> float:
    """max|got - ref| / max|ref| over two device tensors, in slices (no full-size temporaries)."""
    import torch
    num, den = 0.0, 0.0
    for i in range(0, ref.numel(), chunk):
        x = got[i:i + chunk].to(torch.complex128)
        y = ref[i:i + chunk]
        num = max(num, float((x - y).abs().max().item()))
        den = max(den, float(y.abs().max().item()))
    return num / den if den else num


def batch_section(args):
    """The batched configuration: 512 circuits, 10..22 qubits, depth 5..40, seed 4, one persistent
    launch in a CUDA graph; complex128 and complex64 (FP64 reductions); c64 <Z> error vs c128."""
    from damavand_gb300.batch import Batch
    from damavand_gb300.workloads import count, uneven_batch
    circuits = uneven_batch(512, seed=4)
    gates_total = sum(count(g) for _, g in circuits)
    amps = sum(1 << n for n, _ in circuits)
    out, ez = {}, {}
    runs = [("complex128", "fp64", 16), ("complex128", "fp32x2", 16), ("complex128", "int64", 16),
            ("complex64", "fp32", 8)]
    for prec, arith, size in runs:
        b = Batch(circuits, prec, "fp64" if prec == "complex64" else arith)
        tune = b.autotune()
        b.run()
        times = [b.run() for _ in range(max(3, min(args.steps, 5)))]
        ms = float(np.median(times))
        st = b.stats()
        key = prec if arith in ("fp64", "fp32") else f"{prec}_{arith}"
        out[key] = {"arithmetic": arith, "ms_per_run": ms, "circuits_per_s": len(circuits) / (ms / 1e3),
                    "gate_applies_per_s": gates_total / (ms / 1e3), "autotuned": tune, "items": st["items"],
                    "passes": st["passes"], "grid": st["grid"], "cuda_graph": st["cuda_graph"],
                    "arena_gb": amps * size / 1e9}
        ez[key] = b.expect_z()
        del b
    for key in ez:
        if key == "complex128":
            continue
        err = [float(np.max(np.abs(a - b))) for a, b in zip(ez[key], ez["complex128"])]
        out[key]["expect_z_err_vs_complex128_fp64"] = {"max": max(err), "median": float(np.median(err))}
    out["complex64_expect_z_err_vs_complex128"] = out["complex64"]["expect_z_err_vs_complex128_fp64"]
    out["circuits"] = len(circuits)
    out["gates"] = gates_total
    if not args.no_cpu:
        # The reference runs one circuit per process: the oracle (clone per gate) over the
        # circuits in order, for about cpu_seconds, scaled to the batch.
        from oracle import oracle
        oracle.build()
        done, g_done, t0 = 0, 0, time.perf_counter()
        while done < len(circuits) and time.perf_counter() - t0 < args.cpu_seconds:
            nq, gates = circuits[done]
            oracle.forward(nq, [(kk, t, cc, int(o), th) for kk, t, cc, o, th in gates], clone=True)
            g_done += count(gates)
            done += 1
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": done / el, "unit": "circuits/s", "cores": oracle.num_threads(),
                               "kind": "port", "gate_applies_per_s": g_done / el,
                               "sample": f"the first {done} of the {len(circuits)} circuits ({g_done} gates, {el:.1f} s)"}
    return out


def config1_section(args):
    """The 20-qubit configuration end to end through the Circuit API: H on every qubit + 10 x
    [RX, RY, RZ per qubit; CNOT i->i+1] (seed 0, 810 gates), forward, measure (2^20
    probabilities to the host), 1000 samples and the per-qubit <Z> (readout observables),
    against the same pipeline in the oracle (clone per gate, the sampler rebuilding its
    cumulative sum for every sample as sample_from_discrete_distribution does)."""
    import torch

    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, count, ladder_circuit
    n = 20
    gates = ladder_circuit(n, 10, seed=0)
    u = np.random.default_rng([0, 1]).random(1000)
    c = Circuit(n)
    add_to_circuit(c, gates)

    def run():
        c.reset_amplitudes()
        c.forward()
        probs = c.probabilities()
        samples = c.sample_array(1000, uniforms=u)
        ev = np.asarray(c.extract_expectation_values(samples)).mean(axis=0)
        return probs, samples, ev

    for _ in range(3):
        run()
    reps = 10
    t0 = time.perf_counter()
    for _ in range(reps):
        probs, samples, ev = run()
    t_gpu = (time.perf_counter() - t0) / reps
    out = {"qubits": n, "gates": count(gates), "samples": 1000, "seconds_per_run": t_gpu,
           "runs_per_s": 1.0 / t_gpu, "gate_applies_per_s": count(gates) / t_gpu,
           "pipeline": "forward + measure (probabilities to host) + 1000 samples + extract_expectation_values"}
    if not args.no_cpu:
        from oracle import oracle
        oracle.build()
        og = [(kk, t, cc, int(o), th) for kk, t, cc, o, th in gates]
        t0 = time.perf_counter()
        st = oracle.forward(n, og, clone=True)
        t_fwd = time.perf_counter() - t0
        p = oracle.measure(st)
        t1 = time.perf_counter()
        s_ref = oracle.sample(p, u, rebuild_per_sample=True)
        t_smp = time.perf_counter() - t1
        oracle.extract_expectation_values(s_ref, list(range(n)))
        t_cpu = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / t_cpu, "unit": "runs/s", "cores": oracle.num_threads(), "kind": "port",
                               "sample": f"the whole pipeline once: forward {t_fwd:.2f} s, 1000 samples with the "
                                         f"per-sample cumulative sum {t_smp:.2f} s, total {t_cpu:.2f} s"}
        out["speedup_vs_cpu_baseline"] = t_cpu / t_gpu
        out["samples_equal_oracle"] = int(np.sum(np.asarray(samples, dtype=np.uint64) == s_ref))
        out["probabilities_normwise_err_vs_oracle"] = float(np.max(np.abs(probs - p)) / np.max(p))
    del c
    torch.cuda.empty_cache()
    return out


def large_section(args):
    """The large-state configuration. 31 qubits complex128 (three 34.4 GB statevectors for the
    adjoint): forward + adjoint of the 12-layer ring ansatz (1116 parameters, seed 5, loss =
    mean <Z_i>), two sampled gradients checked against parameter shift through the same GPU
    kernels. 32 qubits complex64 (34.4 GB) forward with FP64 reductions; its error is reported
    against complex128 (FP64 arithmetic) on the 30-qubit prefix of the same circuit (its gates
    on qubits 0..29, same angles), run in both precisions."""
    import torch

    from damavand_gb300 import Circuit
    from damavand_gb300.workloads import add_to_circuit, parameters, ring_ansatz
    res = {}
    n = 31
    gates = ring_ansatz(n, 12, seed=5)
    c = Circuit(n)
    add_to_circuit(c, gates)
    c.forward()  # warm-up (plans, tensor maps, first-touch of the 34.4 GB state)
    c.reset_amplitudes()
    c.synchronize()
    t0 = time.perf_counter()
    c.forward()
    c.synchronize()
    res["forward31_s"] = time.perf_counter() - t0
    res["forward31_gate_applies_per_s"] = len(gates) / res["forward31_s"]
    w = np.full(n, 1.0 / n)
    t0 = time.perf_counter()
    loss, grads = c.adjoint_gradient(w)
    res["adjoint31_s"] = time.perf_counter() - t0
    res["adjoint31_params"] = int(grads.size)
    res["adjoint31_grads_per_s"] = grads.size / res["adjoint31_s"]
    res["adjoint31_loss"] = loss
    p = parameters(gates)
    which = [0, p.size - 1]
    diffs = []
    for j in which:
        up, dn = p.copy(), p.copy()
        up[j] += math.pi / 2
        dn[j] -= math.pi / 2
        c.set_parameters(up)
        lu = c.loss(w)
        c.set_parameters(dn)
        ld = c.loss(w)
        diffs.append(abs(0.5 * (lu - ld) - grads[j]))
    c.set_parameters(p)
    res["adjoint31_check"] = {"against": "parameter shift through the same GPU kernels", "params": which,
                              "max_abs_diff": float(max(diffs)), "tolerance": 1e-10, "ok": bool(max(diffs) <= 1e-10)}
    del c
    torch.cuda.empty_cache()
    if not args.no_cpu:
        # The reference's CPU path at 31 qubits: one gate of this forward (clone + sweep of the
        # 34.4 GB state) timed, scaled to the forward and to parameter shift (two forwards per
        # parameter; the reference has no adjoint).
        from oracle import oracle
        oracle.build()
        st31 = oracle.zero_state(n)
        t0 = time.perf_counter()
        oracle.forward(n, [(kk, t, cc, int(o), th) for kk, t, cc, o, th in gates[:1]], st31, clone=True)
        t_gate = time.perf_counter() - t0
        del st31
        res["cpu_baseline"] = {"value": 1.0 / t_gate, "unit": "gate-applies/s", "cores": oracle.num_threads(),
                               "kind": "port", "extrapolated": True,
                               "forward31_s_extrapolated": t_gate * len(gates),
                               "param_shift31_grads_per_s_extrapolated": 1.0 / (2.0 * t_gate * len(gates)),
                               "sample": f"gate 1 of the {len(gates)}-gate 31-qubit forward on the host "
                                         f"({t_gate:.1f} s), scaled"}

    m = 32
    g32 = ring_ansatz(m, 12, seed=5)
    c64 = Circuit(m, precision="complex64")
    add_to_circuit(c64, g32)
    c64.forward()
    c64.reset_amplitudes()
    c64.synchronize()
    t0 = time.perf_counter()
    c64.forward()
    c64.synchronize()
    res["forward32_c64_s"] = time.perf_counter() - t0
    res["forward32_c64_gate_applies_per_s"] = len(g32) / res["forward32_c64_s"]
    ez = c64.expectation_z()
    res["forward32_c64_norm"] = float(c64.norm())
    res["forward32_c64_mean_abs_expect_z"] = float(np.mean(np.abs(ez)))
    del c64
    torch.cuda.empty_cache()
    prefix = [g for g in g32 if g[1] < 30 and g[2] < 30]
    a = Circuit(30, precision="complex64")
    b = Circuit(30)  # complex128, FP64 arithmetic
    for cc in (a, b):
        add_to_circuit(cc, prefix)
        cc.forward()
    res["c64_vs_c128_prefix30"] = {
        "gates": len(prefix),
        "expect_z_max_abs_err": float(np.max(np.abs(a.expectation_z() - b.expectation_z()))),
        "amplitude_normwise_err": normwise_err(a.state().torch(), b.state().torch()),
        "against": "complex128 (FP64 arithmetic) forward of the 32-qubit circuit's gates on qubits 0..29"}
    del a, b
    torch.cuda.empty_cache()
    return res


def read_families(lib, check):
    import ctypes

    from damavand_gb300._lib import KERNEL_ADJOINT, KERNEL_REDUCE, KERNEL_SINGLE, KERNEL_WINDOW
    fam = {}
    for name, f in (("window", KERNEL_WINDOW), ("single", KERNEL_SINGLE), ("reduce", KERNEL_REDUCE),
                    ("adjoint", KERNEL_ADJOINT)):
        l, t, b, fm = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(lib.dmv_profile_read(f, ctypes.byref(l), ctypes.byref(t), ctypes.byref(b), ctypes.byref(fm)))
        fam[name] = {"launches": l.value, "ms": t.value, "bytes": b.value, "arith_ops": fm.value}
    return fam


def timed_forward(c, args, world, local, steps=None, warmup=None):
    """W warm-up steps, then K steps between CUDA events on the library's stream (profiled).
    The headline uses the command line's K and W; the secondary lines pass fewer."""
    import ctypes

    from damavand_gb300._lib import check, lib
    st = c.state()
    steps = args.steps if steps is None else steps
    warmup = args.warmup if warmup is None else warmup

    def step():
        c.reset_amplitudes()
        c.forward()

    for _ in range(warmup):
        step()
    st.synchronize()
    barrier(world)
    st.synchronize()
    lib.dmv_profile_reset()
    lib.dmv_profile_enable(1)
    launches0 = lib.dmv_kernel_launch_count()
    with ClockSampler(local) as clocks:
        check(lib.dmv_state_event_begin(st.handle))
        for _ in range(steps):
            step()
        ms = ctypes.c_double()
        check(lib.dmv_state_event_end(st.handle, ctypes.byref(ms)))
    launches = lib.dmv_kernel_launch_count() - launches0
    lib.dmv_profile_enable(0)
    barrier(world)
    step_ms = max_over_ranks(world, ms.value / steps)
    return step_ms, read_families(lib, check), launches, clocks.summary(), step


def tc_stats(c):
    """Window passes of the last forward that ran on the tensor cores, their dense blocks and exchanges."""
    import ctypes

    from damavand_gb300._lib import check, lib
    p, b, x = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    check(lib.dmv_last_tc_stats(c.state().handle, ctypes.byref(p), ctypes.byref(b), ctypes.byref(x)))
    return {"passes": p.value, "dense_blocks": b.value, "exchanges": x.value}


def rooflines(fam, n, arith, prec="c128"):
    dom = max(fam, key=lambda k: fam[k]["ms"])
    d = fam[dom]
    peak, peak_kind = load_peaks()
    per_launch_bytes = d["bytes"] / max(d["launches"], 1)
    avg_launch_s = d["ms"] / max(d["launches"], 1) / 1e3
    achieved = per_launch_bytes / avg_launch_s / 1e9 if avg_launch_s > 0 else 0.0
    # DRAM bytes per launch from one ncu capture of the same kernel, scaled by state size.
    traffic = None
    key = (dom, prec, arith) if (dom, prec, arith) in NCU_TRAFFIC_PER_AMPLITUDE else (dom, prec)
    if key in NCU_TRAFFIC_PER_AMPLITUDE:
        traffic = NCU_TRAFFIC_PER_AMPLITUDE[key] * (1 << n)
    kernel = WINDOW_KERNEL.get((arith, prec), "window") if dom == "window" else f"k_apply_{dom}"
    roofline = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": per_launch_bytes, "avg_launch_ms": avg_launch_s * 1e3}
    # The same kernel against the arithmetic ceiling it meets on GB300: FP64
    # multiply-adds for IEEE FP64 arithmetic, FP32 operations for FP32-pair arithmetic.
    rate = d["arith_ops"] / (d["ms"] / 1e3) / 1e12 if d["ms"] else 0.0
    if arith in ("fp64", "fp64-direct"):
        ra = {"bound": "fp64", "achieved": rate, "peak": FP64_FMA_PEAK_T, "unit": "T FMA/s",
              "frac": rate / FP64_FMA_PEAK_T, "peak_source": "measured (FP64 FMA chain kernel on this pool's GB300)"}
    elif arith == "tc":
        tpeak, tkind = load_tensor_peak()
        ra = {"bound": "tensor", "achieved": rate, "peak": tpeak, "unit": "TFLOP/s",
              "frac": rate / tpeak, "peak_source": tkind,
              "counts": "FP16 digit-product FLOPs: 34 products of a 128x64x64 real product per 4096-amplitude tile "
                        "and dense block"}
    elif arith == "int64":
        ra = {"bound": "int-mad", "achieved": rate, "peak": INT_MAD_PEAK_T, "unit": "T IMAD/s",
              "frac": rate / INT_MAD_PEAK_T,
              "peak_source": "measured (32-bit IMAD chain kernel on this pool's GB300); counts IMAD.WIDE limb products"}
    else:
        ra = {"bound": "fp32", "achieved": rate, "peak": FP32_FMA_PEAK_T, "unit": "T op/s",
              "frac": rate / FP32_FMA_PEAK_T, "peak_source": "measured (FP32 FMA chain kernel on this pool's GB300)"}
    total_bytes = sum(v["bytes"] for v in fam.values())
    total_ms = sum(v["ms"] for v in fam.values())
    return roofline, ra, (total_bytes / (total_ms / 1e3) / 1e9 if total_ms else None)


def run_ours(args, world, rank, local):
    import ctypes

    from damavand_gb300 import Circuit
    from damavand_gb300._lib import check, dptr, lib
    from damavand_gb300.workloads import add_to_circuit, count, ladder_circuit, parameters

    check(lib.dmv_set_device(local))
    n = args.qubits
    gates = ladder_circuit(n, args.layers, seed=1)
    G = count(gates)
    S = (1 << n) * 16
    c = Circuit(n, "gpu", fusion=not args.no_fusion, arithmetic=args.arith)
    add_to_circuit(c, gates)
    st = c.state()
    step_ms, fam, launches, clocks, step = timed_forward(c, args, world, local)
    value = world * G / (step_ms / 1e3)
    passes, fused_ops, bytes_moved = c.plan_stats()
    roofline, roofline_arith, pass_gbs = rooflines(fam, n, args.arith)

    # ---- e2e through the Circuit API with pinned host buffers
    params = parameters(gates)
    pin_params = np.ascontiguousarray(params)
    re = np.empty(1 << n)
    im = np.empty(1 << n)
    registered = []
    for a in (pin_params, re, im):
        if lib.dmv_host_register(a.ctypes.data, a.nbytes) == 0:
            registered.append(a)
    up_total, up_tab = ctypes.c_int64(), ctypes.c_int64()
    check(lib.dmv_last_upload_bytes(st.handle, ctypes.byref(up_total), ctypes.byref(up_tab)))
    h2d = pin_params.nbytes + up_total.value  # parameters + the plan's op list and phase tables
    d2h = re.nbytes + im.nbytes
    c.set_parameters(pin_params)
    step()
    check(lib.dmv_state_copy_to_host(st.handle, dptr(re), dptr(im)))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        c.set_parameters(pin_params)
        step()
        check(lib.dmv_state_copy_to_host(st.handle, dptr(re), dptr(im)))
    e2e_s = max_over_ranks(world, (time.perf_counter() - t0) / args.steps)
    for a in registered:
        lib.dmv_host_unregister(a.ctypes.data)
    del re, im

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPES[args.arith], "data": "synthetic (seeded angles, seed 1)",
        "config": workload_config(args, G),
        "hbm_gbs_pass_bytes": pass_gbs,
        "per_gate_equiv_gbs": G * 2 * S / (step_ms / 1e3) / 1e9,
        "plan": {"passes": passes, "fused_ops": fused_ops, "bytes_per_forward": bytes_moved},
        "kernels": fam,
        "roofline": roofline,
        "roofline_arith": roofline_arith,
        "e2e": {"value": world * G / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
                "h2d_phase_table_bytes": int(up_tab.value)},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }

    # ---- readout of the final 30-qubit state: <Z_q>, 1000 samples, probabilities on the device
    import torch
    u = np.random.default_rng([1, 1]).random(1000)
    c.expectation_z()
    t0 = time.perf_counter()
    ez = c.expectation_z()
    t_ez = time.perf_counter() - t0
    t0 = time.perf_counter()
    samples = c.sample_array(1000, uniforms=u)
    t_s = time.perf_counter() - t0
    probs = torch.empty(1 << n, dtype=torch.float64, device="cuda")
    check(lib.dmv_measure_device(st.handle, ctypes.cast(probs.data_ptr(), ctypes.POINTER(ctypes.c_double))))
    st.synchronize()
    t0 = time.perf_counter()
    check(lib.dmv_measure_device(st.handle, ctypes.cast(probs.data_ptr(), ctypes.POINTER(ctypes.c_double))))
    st.synchronize()
    t_p = time.perf_counter() - t0
    del probs
    torch.cuda.empty_cache()
    # sampled <Z_q> for every qubit from 2^20 samples drawn and counted on the device (seeded stream)
    k_se = 1 << 20
    qs = np.arange(n, dtype=np.int32)
    se_means = np.empty(n)
    qptr = qs.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    check(lib.dmv_sample_expect_z(st.handle, None, 5, 4096, qptr, n, dptr(se_means), None))
    t0 = time.perf_counter()
    check(lib.dmv_sample_expect_z(st.handle, None, 5, k_se, qptr, n, dptr(se_means), None))
    t_se = time.perf_counter() - t0
    se_sigma = np.sqrt(np.maximum(1.0 - ez ** 2, 1e-12) / k_se)
    out["readout"] = {"expect_z_ms": t_ez * 1e3, "expect_z_gbs": S / t_ez / 1e9, "sample_1000_ms": t_s * 1e3,
                      "probabilities_on_device_ms": t_p * 1e3, "probabilities_gbs": (S + S // 2) / t_p / 1e9,
                      "sample_expect_z": {"samples": k_se, "ms": t_se * 1e3, "samples_per_s": k_se / t_se,
                                          "max_dev_over_sigma_vs_exact": float(np.max(np.abs(se_means - ez) / se_sigma))},
                      "norm": float(c.norm()), "first_samples": [int(x) for x in samples[:4]],
                      "mean_abs_expect_z": float(np.mean(np.abs(ez)))}

    # ---- the other complex128 arithmetics, same workload and protocol, each checked against FP64
    if not args.no_alt:
        import torch
        # secondary lines: fewer steps than the headline (each is reported with its own count)
        sec_steps, sec_warmup = max(1, min(args.steps, 5)), min(args.warmup, 3)
        alts = [a for a in ("fp64", "fp64-direct", "fp32x2", "int64", "tc") if a != args.arith]
        out["alt_arithmetic"] = []
        for alt in alts:
            c2 = Circuit(n, "gpu", fusion=not args.no_fusion, arithmetic=alt)
            add_to_circuit(c2, gates)
            ms2, fam2, launches2, clocks2, _ = timed_forward(c2, args, world, local, steps=sec_steps,
                                                             warmup=sec_warmup)
            rl2, ra2, gbs2 = rooflines(fam2, n, alt)
            ta, tb = c2.state().torch(), c.state().torch()  # both hold one forward from |0...0>
            if args.arith == "fp64":
                ref, other = tb, ta
            elif alt == "fp64":
                ref, other = ta, tb
            else:
                ref, other = None, None
            err = normwise_err(other, ref) if ref is not None else None
            del ta, tb, ref, other
            entry = {
                "arithmetic": alt, "dtype": DTYPES[alt], "value": world * G / (ms2 / 1e3), "unit": UNIT,
                "ms_per_step": ms2, "steps": sec_steps, "warmup": sec_warmup, "roofline": rl2, "roofline_arith": ra2, "hbm_gbs_pass_bytes": gbs2,
                "gpu_launches": int(launches2), "clocks": clocks2}
            if alt == "tc":
                entry["tensor_core_passes"] = tc_stats(c2)
            if err is not None:
                entry["parity"] = {"against": "the FP64-arithmetic forward of this run", "normwise_max_err": err,
                                   "tolerance": 1e-12, "ok": bool(err <= 1e-12)}
            out["alt_arithmetic"].append(entry)
            del c2
            torch.cuda.empty_cache()
        # complex64 storage and FP32 arithmetic, same workload and protocol (the
        # TMA window kernel's register-phase variant); error against this run's
        # complex128 state.
        c3 = Circuit(n, "gpu", fusion=not args.no_fusion, precision="complex64")
        add_to_circuit(c3, gates)
        ms3, fam3, launches3, clocks3, _ = timed_forward(c3, args, world, local, steps=sec_steps,
                                                         warmup=sec_warmup)
        rl3, ra3, gbs3 = rooflines(fam3, n, "fp32", prec="c64")
        err = normwise_err(c3.state().torch(), c.state().torch())
        out["complex64"] = {
            "dtype": "c64 (complex64 storage, FP32 arithmetic)", "value": world * G / (ms3 / 1e3), "unit": UNIT,
            "ms_per_step": ms3, "steps": sec_steps, "warmup": sec_warmup, "roofline": rl3, "roofline_arith": ra3, "hbm_gbs_pass_bytes": gbs3,
            "gpu_launches": int(launches3), "clocks": clocks3,
            "error": {"against": f"the {args.arith} complex128 forward of this run", "normwise_max_err": err}}
        del c3
        torch.cuda.empty_cache()
    if rank == 0 and not args.no_adjoint:
        out["adjoint"] = adjoint_section(args)
    if rank == 0 and not args.no_batch:
        out["batch"] = batch_section(args)
    if rank == 0 and not args.no_config1:
        out["config1"] = config1_section(args)
    if rank == 0 and not args.no_large:
        out["large"] = large_section(args)
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args)
        if "complex64" in out:
            # the reference has complex128 only: the same CPU forward is the baseline of the c64 line
            out["complex64"]["cpu_baseline"] = dict(out["cpu_baseline"], note="the reference's complex128 CPU "
                                                    "forward of the same workload (it has no complex64 path)")
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--layers", type=int, default=20)
    ap.add_argument("--no-fusion", action="store_true")
    ap.add_argument("--no-alt", action="store_true",
                    help="skip the other complex128 arithmetics (timed and checked against FP64)")
    ap.add_argument("--arith", choices=["fp64", "fp64-direct", "fp32x2", "int64", "tc"], default="fp64",
                    help="complex128 arithmetic: IEEE FP64 (rotations and phase tables, or every 2x2 "
                         "as a full complex multiply-add), FP32 pairs (error-free transformations), "
                         "int64 block fixed point, or the same with dense blocks on the tensor cores")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the 31-qubit forward + adjoint and the 32-qubit complex64 forward")
    ap.add_argument("--no-config1", action="store_true",
                    help="skip the 20-qubit forward + measure + 1000 samples pipeline")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-gates", type=int, default=3, help="gates per reference step")
    ap.add_argument("--ps-params", type=int, default=8, help="parameters sampled for parameter shift")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        out = run_reference(args, world, rank)
    else:
        out = run_ours(args, world, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out, default=lambda o: o.item() if hasattr(o, "item") else str(o)))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
