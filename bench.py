#!/usr/bin/env python
"""Benchmark of the qandle hot path on GB300.

Headline workload (one JSON line on rank 0): the fused forward of the
strongly-entangling re-uploading circuit, 20 qubits x batch 256 (complex64
state 2 GiB, larger than L2): AngleEmbedding(rx), 10 layers of RZ RY RZ per
qubit with a CNOT ring of range (layer mod 19) + 1, named RX re-uploading of
the inputs before layers 0 and 5, <Z> per qubit.  Metric: amplitude-updates/s
= gates x batch x 2^n per forward / time (860 gates, the embedding counted as
20 rotations).

Also on the line:
* roofline of the pass kernel from CUDA events around every pass launch:
  HBM (algorithmic bytes) and FP32 (counted FMAs against the FP32 peak that
  the library's own probe kernel measures), and per-pass figures;
* the end-to-end time through the public API (Circuit.__call__, which
  replays a captured CUDA graph) with pinned host inputs and results;
* the forward replayed from one CUDA graph, the plain per-gate form;
* config 1 (8 qubits x 64, plain method) on the GPU, and the reference's own
  torch path on the host cores at that size and at 10 qubits;
* the adjoint (16 qubits x 1024, MSE(<Z>, targets)) against the per-gate
  adjoint, with its backward passes' roofline;
* the deep 28-qubit circuit against the per-gate form;
* the fusion-width sweep k = 1..6, and the autotuner's choice of tile shape,
  k and qubit-remap schedule;
* the serving loop against one per-gate run per request, live, at two
  Poisson rates;
* the error against the complex128 oracle for every config;
* SM clocks sampled during the timed region; the oracle timed on the host.

`--impl reference` times the CPU implementation of the same path (the
complex128 oracle, all host threads) on a bounded sample per step, and the
reference's own torch path at the sizes it can run.
Under torchrun every rank runs its own batch (weak scaling, no collective on
the data path); rank 0 prints.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


EXTRAS = ("graph", "plain", "config1", "adjoint", "deep28", "sweep", "autotune", "serving")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", action="store_true", help="headline only")
    ap.add_argument("--extras", default=",".join(EXTRAS),
                    help="comma-separated records after the headline (default: all of " + ",".join(EXTRAS) + ")")
    ap.add_argument("--adjoint-batch", type=int, default=1024)
    ap.add_argument("--cpu-samples", type=int, default=16, help="samples in the CPU baseline")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baselines (profiling runs)")
    ap.add_argument("--tile-bits", type=int, default=13)
    ap.add_argument("--low-bits", type=int, default=6)
    ap.add_argument("--k", type=int, default=0, help="max strided qubits per pass (0 = tile limit)")
    ap.add_argument("--reg-bits", type=int, default=5, help="amplitudes per thread = 2^reg_bits")
    ap.add_argument("--reg-search", type=int, default=0, help="qubit-remap schedule: 0 greedy, 1 searched")
    ap.add_argument("--serving-requests", type=int, default=500, help="requests at the high rate")
    ap.add_argument("--serving-rate", type=float, default=2000.0)
    ap.add_argument("--serving-low-requests", type=int, default=60, help="requests at the low rate")
    ap.add_argument("--serving-low-rate", type=float, default=2.0)
    ap.add_argument("--serving-repeated-requests", type=int, default=300,
                    help="requests drawn from a few fixed structures, at the high rate")
    ap.add_argument("--autotune", action="store_true",
                    help="run the headline with the autotuner's options")
    ap.add_argument("--interpreted", action="store_true",
                    help="run the prebuilt op interpreter instead of the per-program compiled passes")
    ap.add_argument("--n", type=int, default=20)
    ap.add_argument("--batch", type=int, default=256)
    args = ap.parse_args()
    args.extras = set() if args.no_extras else {e for e in args.extras.split(",") if e}
    unknown = args.extras - set(EXTRAS)
    if unknown:
        ap.error(f"unknown extras {sorted(unknown)}")
    return args


def peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for name, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------- CPU baselines --

def cpu_baseline(desc, samples: int):
    """The oracle (complex128 port, all host threads) on the first `samples`
    samples of the workload.  Returns (record, measured output of those
    samples) -- the output is the oracle value the GPU result is checked
    against."""
    from oracle import oracle
    from qandle_gb300 import workloads

    threads = len(os.sched_getaffinity(0))
    lo = oracle.Lowered(desc, samples)
    t0 = time.perf_counter()
    st = oracle.run(desc, batch=samples, nthreads=threads, lowered=lo)
    dt = time.perf_counter() - t0
    amp = workloads.gate_count(desc) * samples * (1 << desc["n"])
    rec = {"value": amp / dt, "unit": "amp-updates/s", "cores": threads, "kind": "port",
           "sample": f"{samples} of {desc['batch']} samples of the {desc['n']}-qubit workload, {dt:.2f} s"}
    return rec, oracle.measure(desc, st)


def reference_torch_baseline(gpu_ms: dict | None = None):
    """The reference's own torch path (qandle 0.1.8 from baseline/_ref) on
    the host cores, all threads, at config 1 (8 qubits x 64, the plain
    circuit, joint probabilities) and at 10 qubits x 64 (the largest its
    dense 2^n x 2^n matrices reach in seconds).  Median of timed forwards
    after one untimed forward.  `gpu_ms` maps the same keys to our GPU
    times, for the ratio."""
    from oracle import oracle
    from oracle import reference_torch as rt
    from qandle_gb300 import workloads

    why = rt.unavailable_reason()
    if why:
        return {"unavailable": why}
    import torch

    threads = len(os.sched_getaffinity(0))
    torch.set_num_threads(threads)
    qandle = rt.import_reference()
    out = {"kind": "reference", "cores": threads,
           "what": "qandle 0.1.8 Circuit.forward (dense matmul per layer) on the host CPU, torch "
                   f"{torch.__version__}, {threads} threads, remapping=None, qw_map stand-in"}
    for key, n, reps in (("config1_n8_b64", 8, 3), ("n10_b64", 10, 1)):
        desc = workloads.plain_small(n=n, batch=64, layers=4)
        t_build = time.perf_counter()
        circ = rt.build_circuit(qandle, desc)
        build_s = time.perf_counter() - t_build
        kw = rt.inputs(desc)
        with torch.no_grad():
            t0 = time.perf_counter()
            res = circ(**kw)
            first = time.perf_counter() - t0
            times = []
            for _ in range(reps):
                t0 = time.perf_counter()
                res = circ(**kw)
                times.append(time.perf_counter() - t0)
        ms = 1e3 * float(np.median(times))
        amp = workloads.gate_count(desc) * 64 * (1 << n)
        rec = {"ms_per_forward": ms, "value": amp / (ms * 1e-3), "unit": "amp-updates/s",
               "first_forward_ms": 1e3 * first, "build_s": build_s, "timed_forwards": reps,
               "max_abs_err_vs_oracle": float(np.abs(res.numpy() - oracle.forward(desc)).max())}
        if gpu_ms and key in gpu_ms:
            rec["gpu"] = gpu_ms[key]
            rec["gpu_speedup_plain"] = ms / gpu_ms[key]["plain_ms"]
            rec["gpu_speedup_fused"] = ms / gpu_ms[key]["fused_ms"]
        out[key] = rec
        if first > 60.0:
            break
    return out


def run_reference(args):
    """CPU arm: the oracle port on the host cores, each step a bounded sample
    of the headline workload; the reference's own torch path beside it at the
    sizes it can run."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from qandle_gb300 import workloads

    desc = workloads.sel_reupload(n=args.n, batch=args.batch)
    samples = args.cpu_samples
    for _ in range(args.warmup):
        cpu_baseline(desc, samples)
    times = []
    for _ in range(args.steps):
        r, _ = cpu_baseline(desc, samples)
        times.append(r)
    value = float(np.mean([r["value"] for r in times]))
    amp_step = workloads.gate_count(desc) * samples * (1 << desc["n"])
    line = {"impl": "reference", "metric": "amplitude-updates/s", "value": value, "unit": "amp-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * amp_step / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded)",
            "config": {"workload": f"sel_reupload n={args.n} batch={args.batch} (860 gates), fused-path "
                                   f"circuit on the CPU oracle, {samples} samples per step",
                       "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": value, "unit": "amp-updates/s", "cores": times[0]["cores"],
                             "kind": "port", "sample": times[0]["sample"]},
            "e2e": {"value": value, "unit": "amp-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_cpu:
        line["reference_torch"] = reference_torch_baseline()
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- roofline bits --

def fp32_peak(dev) -> dict:
    """FP32 FMA throughput of the library's probe kernel (packed FMAs, all
    SMs), median of three launches of a few milliseconds."""
    import torch

    from qandle_gb300 import _lib

    lib = _lib.load()
    blocks = lib.qg_fp32_probe_blocks()
    out = torch.empty(blocks, dtype=torch.float32, device=dev)
    cnt = ctypes.c_int64()
    iters = 1 << 16

    def launch():
        _lib.check(lib.qg_fp32_probe(out.data_ptr(), blocks, iters, ctypes.byref(cnt), _lib.stream()))

    launch()
    torch.cuda.synchronize(dev)
    ms = []
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        launch()
        e1.record()
        torch.cuda.synchronize(dev)
        ms.append(e0.elapsed_time(e1))
    t = float(np.median(ms))
    return {"tflops": 2.0 * cnt.value / (t * 1e-3) / 1e12, "fma_per_launch": cnt.value, "ms": t,
            "kernel": "k_fp32_probe (fma.rn.f32x2, 8 chains per thread, 4 x 256 threads per SM)"}


def pass_fmas(prog, backward: bool, amps: int) -> np.ndarray:
    """Counted FMAs of every pass: a 2x2 on a register qubit is 8 FMAs per
    amplitude, a diagonal 4; the backward applies each gate to psi and lambda
    and a gradient partial adds 2 per amplitude."""
    out = []
    for pd in prog.passes(backward):
        ops = pd["ops"]
        mats = int(np.sum(ops[:, 0] == 2)) if len(ops) else 0
        diags = int(np.sum(ops[:, 0] == 3)) if len(ops) else 0
        if backward:
            grads = int(np.sum((ops[:, 0] == 2) & ((ops[:, 3] & 2) != 0))) if len(ops) else 0
            f = 16 * mats + 8 * diags + 2 * grads
        else:
            f = 8 * mats + 4 * diags
        out.append(f * amps)
    return np.array(out, dtype=np.float64)


def pass_bytes_fwd(prog, amps: int) -> np.ndarray:
    """Algorithmic bytes of every forward pass: 8 B per amplitude read, 8 B
    per amplitude written (state or checkpoint), 4 B per probability."""
    out = []
    for pd in prog.passes(False):
        b = 0
        if pd["init"] == 0:
            b += 8 * amps
        if pd["epi"] & 1:
            b += 8 * amps
        if pd["epi"] & 2:
            b += 4 * amps
        if pd["ckpt"] >= 0:
            b += 8 * amps
        out.append(b)
    return np.array(out, dtype=np.float64)


def pass_bytes_bwd(prog, amps: int) -> np.ndarray:
    """Algorithmic bytes of every backward pass: psi and lambda read (16 B
    per amplitude), and written back (16 B) by the passes that store (the
    last pass of the backward stores nothing unless the input-state gradient
    is wanted, which this workload does not)."""
    out = []
    for pd in prog.passes(True):
        b = 16 * amps
        if pd["epi"] & 1:
            b += 16 * amps
        out.append(b)
    return np.array(out, dtype=np.float64)


def combined_roof(ms: np.ndarray, bytes_: np.ndarray, fmas: np.ndarray, hbm_gbs: float, fp32_tflops: float):
    """Per pass the time the better of the two roofs allows:
    max(bytes / HBM, 2 FMAs / FP32), and its sum against the measured sum."""
    t_mem = bytes_ / (hbm_gbs * 1e9) * 1e3
    t_fp = 2.0 * fmas / (fp32_tflops * 1e12) * 1e3
    t_roof = np.maximum(t_mem, t_fp)
    return float(t_roof.sum() / ms.sum()), t_mem, t_fp


# ------------------------------------------------------------------- main --

def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    import torch.distributed as dist

    from qandle_gb300 import engine, workloads

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl")

    def sync_all():
        torch.cuda.synchronize(dev)
        if world > 1:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        if world == 1:
            return x
        t = torch.tensor([x], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    hbm_peak, peak_kind = peaks()
    K, W = args.steps, args.warmup
    desc = workloads.sel_reupload(n=args.n, batch=args.batch)
    n, B = desc["n"], desc["batch"]
    amp_step = workloads.gate_count(desc) * B * (1 << n)

    # ---------------- fused forward, inputs resident in HBM ----------------
    opts = dict(tile_bits=args.tile_bits, low_bits=args.low_bits, max_high=args.k, reg_bits=args.reg_bits,
                reg_search=args.reg_search, compiled=not args.interpreted)
    tuned = None
    if args.autotune:
        from qandle_gb300 import tune

        tuned = tune.autotune(workloads.build_circuit(desc, engine="fused"), B, dev,
                              compiled=not args.interpreted)
        opts.update(tuned["options"])
    circ = workloads.build_circuit(desc, engine="fused", **opts).to(dev)
    kw = workloads.circuit_inputs(desc, dev)
    with torch.no_grad():
        circ(**kw)
    ex = circ._executor
    bound = engine.BoundForward(ex, B, dev)
    bound.set_inputs(**kw)
    prog = bound.prog
    P = prog.info.forward_passes
    for _ in range(W):
        bound.launch()
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(2 * P)] for _ in range(K)]
    for row in events:
        for e in row:
            e.record()
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    sync_all()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for s in range(K):
        bound.launch(events[s])
    t1.record()
    sync_all()
    clock_info = clocks.stop()
    ms = max_over_ranks(t0.elapsed_time(t1)) / K
    value = world * amp_step / (ms * 1e-3)
    headline_out = bound.result().clone()
    pass_ms = np.array([[events[s][2 * p].elapsed_time(events[s][2 * p + 1]) for p in range(P)]
                        for s in range(K)])
    amps = B * (1 << n)
    pbytes = pass_bytes_fwd(prog, amps)
    pfmas = pass_fmas(prog, False, amps)
    avg_bytes = float(pbytes.mean())
    avg_pass_ms = float(pass_ms.mean())
    achieved = avg_bytes / (avg_pass_ms * 1e-3) / 1e9
    # per-pass bandwidth of the middle passes (load + store, 16 B / amplitude)
    mid = [p for p in range(P) if pbytes[p] == 16 * amps]
    mid_gbs = float(16 * amps / (pass_ms[:, mid].mean() * 1e-3) / 1e9) if mid else None
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "fwd_pass_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get("dram_bytes_per_launch")
    gpu_launches = K * (P + 3)  # matrix build, embedding factors, P passes, <Z> reduction
    fp32 = fp32_peak(dev)
    mean_ms = pass_ms.mean(0)
    comb, t_mem, t_fp = combined_roof(mean_ms, pbytes, pfmas, hbm_peak, fp32["tflops"])
    fp_frac = 2.0 * pfmas / (mean_ms * 1e-3) / (fp32["tflops"] * 1e12)
    heavy = [p for p in range(P) if t_fp[p] > t_mem[p]]

    line = {
        "metric": "amplitude-updates/s", "value": value, "unit": "amp-updates/s", "n_gpus": world,
        "steps": K, "warmup": W, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 (fp32 math; fp64 final sums)", "data": "synthetic (seeded)",
        "config": {"workload": f"sel_reupload: fused forward, {n} qubits x batch {B} per GPU, 10 SEL layers + "
                               "2 re-uploads, <Z> out (860 gates)",
                   "global_batch": B * world, "qubits": n, "parallelism": f"batch shards x{world}",
                   "l2": "inputs larger than L2 (2 GiB state per GPU)",
                   "plan": prog.summary(), "tile": opts},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "peak_kind": peak_kind, "traffic": traffic,
                     "kernel": ("k_fwd_pass (op interpreter)" if args.interpreted else
                                "qg_fwd_pass (compiled per pass)") + f", 2^{args.tile_bits}-amplitude tiles",
                     "launches_per_step": P,
                     "avg_launch_ms": avg_pass_ms, "algorithmic_bytes_per_launch": avg_bytes,
                     "middle_pass_GBps": mid_gbs,
                     "fp32": {"peak_tflops": fp32["tflops"], "peak_kind": "measured (library probe kernel)",
                              "achieved_tflops": float(2.0 * pfmas.sum() / (mean_ms.sum() * 1e-3) / 1e12),
                              "frac": float(2.0 * pfmas.sum() / (mean_ms.sum() * 1e-3) / (fp32["tflops"] * 1e12)),
                              "fma_per_amp_per_pass": [round(float(f) / amps, 1) for f in pfmas],
                              "heavy_passes": len(heavy),
                              "heavy_pass_frac": (float(2.0 * pfmas[heavy].sum() / (mean_ms[heavy].sum() * 1e-3)
                                                        / (fp32["tflops"] * 1e12)) if heavy else None),
                              "probe": fp32},
                     "combined_frac": comb,
                     "per_pass": [{"ms": round(float(mean_ms[p]), 4), "GBps": round(float(
                         pbytes[p] / (mean_ms[p] * 1e-3) / 1e9), 1), "hbm_frac": round(float(
                             pbytes[p] / (mean_ms[p] * 1e-3) / 1e9 / hbm_peak), 3),
                         "fp32_frac": round(float(fp_frac[p]), 3),
                         "roof_frac": round(float(max(t_mem[p], t_fp[p]) / mean_ms[p]), 3)} for p in range(P)]},
        "clocks": clock_info,
        "gpu_launches": gpu_launches,
    }
    if tuned is not None:
        line["autotune_headline"] = {"options": tuned["options"], "cached": tuned["cached"],
                                     "timings_ms": [[o, round(t, 3)] for o, t in tuned["timings"]]}

    # ---------------- end to end through the public API ----------------
    x_host = torch.tensor(desc["inputs"]["x"]).pin_memory()
    names = [f"up{q}" for q in range(n)]

    def e2e_step():
        x = x_host.to(dev, non_blocking=True)
        kw2 = {"x": x}
        for q, nm in enumerate(names):
            kw2[nm] = x[:, q]
        with torch.no_grad():
            out = circ(**kw2)
        return out.cpu()

    for _ in range(W):
        e2e_step()
    sync_all()
    t_e2e = time.perf_counter()
    for _ in range(K):
        res = e2e_step()
    sync_all()
    e2e_ms = max_over_ranks((time.perf_counter() - t_e2e) * 1e3 / K)
    line["e2e"] = {"value": world * amp_step / (e2e_ms * 1e-3), "unit": "amp-updates/s",
                   "h2d_bytes_per_step": int(x_host.numel() * 4), "d2h_bytes_per_step": int(res.numel() * 4),
                   "ms_per_step": e2e_ms,
                   "path": "Circuit.__call__ (inference: replays the captured forward graph)",
                   "captured": any(b.graph is not None for b in circ._executor._bounds.values())}
    oracle_err = {}

    ext = args.extras
    gpu_ms_small = None
    if "graph" in ext:
        # ---------------- one CUDA graph per forward ----------------
        bound.capture()
        for _ in range(W):
            bound.replay()
        sync_all()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record()
        for _ in range(K):
            bound.replay()
        g1.record()
        sync_all()
        gms = g0.elapsed_time(g1) / K
        line["graph"] = {"value": amp_step / (gms * 1e-3), "ms_per_step": gms,
                         "max_abs_diff_vs_launch": float((bound.result() - headline_out).abs().max())}
    del bound

    if "plain" in ext:
        # ---------------- plain per-gate form, same workload ----------------
        circ_p = workloads.build_circuit(desc, engine="plain").to(dev)
        with torch.no_grad():
            circ_p(**kw)
            sync_all()
            p0 = torch.cuda.Event(enable_timing=True)
            p1 = torch.cuda.Event(enable_timing=True)
            steps_p = 2
            p0.record()
            for _ in range(steps_p):
                ref_out = circ_p(**kw)
            p1.record()
            sync_all()
        pms = p0.elapsed_time(p1) / steps_p
        line["plain"] = {"value": amp_step / (pms * 1e-3), "ms_per_step": pms,
                         "fused_speedup": pms / ms,
                         "max_abs_diff_vs_fused": float((headline_out - ref_out).abs().max())}
        del circ_p, ref_out
        torch.cuda.empty_cache()

    if "config1" in ext:
        # ---------------- config 1: 8 qubits x 64, plain method ----------------
        line["config1"], gpu_ms_small = bench_config1(dev, sync_all, oracle_err)

    if "adjoint" in ext:
        # ---------------- adjoint: 16 qubits x batch 1024, MSE(<Z>, t) ----------------
        line["adjoint"] = bench_adjoint(dev, sync_all, W, hbm_peak, fp32["tflops"], oracle_err, args.adjoint_batch)
        torch.cuda.empty_cache()

    if "deep28" in ext:
        # ---------------- deep single state: 28 qubits x batch 1 ----------------
        line["deep28"] = bench_deep(dev, sync_all, W, oracle_err)
        torch.cuda.empty_cache()

    # ---------------- fusion width sweep, autotuner ----------------
    if "sweep" in ext:
        line["k_sweep"] = bench_k_sweep(desc, kw, dev, sync_all, amp_step, ms)
        torch.cuda.empty_cache()
    if "autotune" in ext:
        line["autotune"] = bench_autotune(desc, dev, amp_step, ms)
        torch.cuda.empty_cache()

    if "serving" in ext:
        # ---------------- serving: Poisson arrivals of mixed-width requests ----------------
        line["serving"] = {
            "high_rate": bench_serving(dev, args.serving_requests, args.serving_rate, seed=7,
                                       oracle_err=oracle_err, policies=("srpt", "all", "srpt_interpreted")),
            "low_rate": bench_serving(dev, args.serving_low_requests, args.serving_low_rate, seed=8,
                                      oracle_err=oracle_err),
            "repeated_structures": bench_serving_repeated(dev, args.serving_repeated_requests, args.serving_rate,
                                                          seed=9, structures=6, oracle_err=oracle_err)}
        torch.cuda.empty_cache()

    if rank == 0:
        if args.no_cpu:
            line["cpu_baseline"] = None
        else:
            rec, ref = cpu_baseline(desc, args.cpu_samples)
            line["cpu_baseline"] = rec
            got = headline_out[:args.cpu_samples].cpu().numpy()
            oracle_err["config2_z_first_%d_samples" % args.cpu_samples] = float(np.abs(got - ref).max())
            line["reference_torch"] = reference_torch_baseline(gpu_ms_small)
        line["oracle_error"] = dict(oracle_err, tolerance=1e-5,
                                    note="max-abs against the complex128 oracle on the same seeded inputs; the "
                                         "bar is 1e-5 on probabilities and P0 (<Z> = 2 P0 - 1 doubles the P0 "
                                         "error), 1e-4 on gradients")
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def bench_config1(dev, sync_all, oracle_err):
    """Config 1 on the GPU: 8 qubits x 64, AngleEmbedding(rx), 4 layers of
    RY + CNOT ring, joint probabilities; plain per-gate form and fused
    engine, each a median over 20 forwards, both checked against the oracle.
    Also 10 qubits x 64 (the reference's largest size) for the CPU ratio."""
    import torch

    from oracle import oracle
    from qandle_gb300 import workloads

    out, gpu_ms = {}, {}
    for key, n in (("config1_n8_b64", 8), ("n10_b64", 10)):
        desc = workloads.plain_small(n=n, batch=64, layers=4)
        kw = workloads.circuit_inputs(desc, dev)
        ref = oracle.forward(desc)
        rec = {}
        for eng in ("plain", "fused"):
            circ = workloads.build_circuit(desc, engine=eng).to(dev)
            with torch.no_grad():
                for _ in range(3):
                    res = circ(**kw)
                sync_all()
                times = []
                for _ in range(20):
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record()
                    res = circ(**kw)
                    e1.record()
                    sync_all()
                    times.append(e0.elapsed_time(e1))
            rec[f"{eng}_ms"] = float(np.median(times))
            err = float(np.abs(res.cpu().numpy() - ref).max())
            rec[f"{eng}_max_abs_err_vs_oracle"] = err
            oracle_err[f"{key}_{eng}_probs"] = err
        amp = workloads.gate_count(desc) * 64 * (1 << n)
        rec["plain_value"] = amp / (rec["plain_ms"] * 1e-3)
        rec["fused_value"] = amp / (rec["fused_ms"] * 1e-3)
        out[key] = rec
        gpu_ms[key] = {"plain_ms": rec["plain_ms"], "fused_ms": rec["fused_ms"]}
    return out, gpu_ms


def bench_deep(dev, sync_all, W, oracle_err):
    """28 qubits, batch 1 (2 GiB), 50 layers of U per qubit with CNOT+SWAP
    brickwork, |psi|^2 out: fused forward against the per-gate form; the
    20-qubit prefix circuit against the oracle."""
    import torch

    from oracle import oracle
    from qandle_gb300 import engine, workloads

    desc = workloads.deep_u()
    n = desc["n"]
    amp = workloads.gate_count(desc) * (1 << n)
    circ = workloads.build_circuit(desc, engine="fused").to(dev)
    with torch.no_grad():
        circ()
    bound = engine.BoundForward(circ._executor, 1, dev)
    bound.set_inputs()  # the circuit's U matrices
    for _ in range(max(3, W)):
        bound.launch()
    sync_all()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    steps = 3
    e0.record()
    for _ in range(steps):
        bound.launch()
    e1.record()
    sync_all()
    fms = e0.elapsed_time(e1) / steps
    fused_probs = bound.result().reshape(-1)
    norm = float(fused_probs.double().sum())
    del bound
    circ_p = workloads.build_circuit(desc, engine="plain").to(dev)
    with torch.no_grad():
        plain_probs = circ_p().reshape(-1)  # warm-up
        sync_all()
        times = []
        for _ in range(3):
            p0 = torch.cuda.Event(enable_timing=True)
            p1 = torch.cuda.Event(enable_timing=True)
            p0.record()
            plain_probs = circ_p().reshape(-1)
            p1.record()
            sync_all()
            times.append(p0.elapsed_time(p1))
    pms = float(np.median(times))
    diff = float((plain_probs - fused_probs).abs().max())
    del circ_p, plain_probs, fused_probs
    torch.cuda.empty_cache()
    pre = workloads.restrict(desc, 20)
    cpre = workloads.build_circuit(pre, engine="fused").to(dev)
    with torch.no_grad():
        got = cpre().reshape(-1).cpu().numpy()
    perr = float(np.abs(got - oracle.forward(pre).reshape(-1)).max())
    oracle_err["config4_prefix20_probs"] = perr
    return {"workload": f"deep_u: {n} qubits x batch 1, 50 layers of U + CNOT/SWAP brickwork, |psi|^2 out "
                        f"({workloads.gate_count(desc)} gates)",
            "plan": circ._executor.program(False).summary(),
            "ms_per_step_fused": fms, "ms_per_step_per_gate": pms, "fused_speedup": pms / fms,
            "per_gate_timing": "median of 3 after one untimed forward",
            "amp_updates_per_s_fused": amp / (fms * 1e-3), "amp_updates_per_s_per_gate": amp / (pms * 1e-3),
            "norm_fused": norm, "max_abs_prob_diff_fused_vs_per_gate": diff,
            "prefix20_max_abs_err_vs_oracle": perr}


def bench_k_sweep(desc, kw, dev, sync_all, amp_step, headline_ms):
    """Fused forward with at most k strided qubits per pass, k = 1..6 (the
    default plan takes up to the tile's limit, 7 at 2^13 tiles and 64-
    amplitude runs)."""
    import torch

    from qandle_gb300 import engine, workloads

    sweep = {}
    for k in range(1, 7):
        c = workloads.build_circuit(desc, engine="fused", max_high=k, graphs=False).to(dev)
        with torch.no_grad():
            c(**kw)  # plans and compiles the k-limited program
        bk = engine.BoundForward(c._executor, desc["batch"], dev)
        bk.set_inputs(**kw)
        bk.launch()
        sync_all()
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record()
        for _ in range(3):
            bk.launch()
        a1.record()
        sync_all()
        kms = a0.elapsed_time(a1) / 3
        sweep[str(k)] = {"passes": bk.prog.info.forward_passes, "exchanges_ops": bk.prog.summary(),
                         "ms_per_step": kms, "value": amp_step / (kms * 1e-3)}
        del bk, c
    sweep["default (k = 7)"] = {"ms_per_step": headline_ms, "value": amp_step / (headline_ms * 1e-3)}
    return sweep


def bench_autotune(desc, dev, amp_step, default_ms):
    """The autotuner's staged search (tile shapes, then k, then the
    qubit-remap schedule) on the headline circuit at its batch; its pick
    against the default plan."""
    from qandle_gb300 import tune, workloads

    path = os.path.join(tempfile.mkdtemp(prefix="qgtune"), "tune.json")
    t0 = time.perf_counter()
    res = tune.autotune(workloads.build_circuit(desc, engine="fused"), desc["batch"], dev, cache_path=path)
    return {"options": res["options"], "ms": res["ms"], "value": amp_step / (res["ms"] * 1e-3),
            "default_ms": default_ms, "speedup_vs_default": default_ms / res["ms"],
            "search_s": time.perf_counter() - t0,
            "timings_ms": [[o, round(t, 3)] for o, t in res["timings"]]}


def _serve_live(dev, reqs, offs, amp, policy, compile_min_tiles=1024, warm=()):
    """One live run of the continuous-batching server on the given arrival
    offsets; returns (stats, outputs).  The server starts cold (its
    structures are planned, and large ones compiled, inside the run) unless
    `warm` lists descriptions to prepare before the first arrival."""
    import torch

    from qandle_gb300 import serve

    count = len(reqs)
    srv = serve.Server(dev, hbm_budget=160 << 30, policy=policy, compile_min_tiles=compile_min_tiles)
    t_warm = time.perf_counter()
    for d in warm:
        srv.prepare(d)
    t_warm = time.perf_counter() - t_warm
    try:
        t0 = time.perf_counter()
        handles = []
        for d, o in zip(reqs, offs):
            wait = t0 + o - time.perf_counter()
            if wait > 0:
                time.sleep(wait)
            handles.append(srv.submit(d, arrival=t0 + o))
        outs = [h.future.result(timeout=1800) for h in handles]
        t_end = max(h.completed for h in handles)
        steps, launches, claunches = srv.steps, srv.launches, srv.compiled_launches
        compiled = sum(1 for h in handles if h.prog is not None and srv.compile_min_tiles is not None
                       and serve._tiles_per_pass(h.lowered[0].n, h.desc["batch"] or 1, srv.tile_bits)
                       >= srv.compile_min_tiles)
    finally:
        srv.close()
    lat = np.array([h.latency for h in handles]) * 1e3
    span = t_end - t0
    stats = {"policy": policy, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
             "circuits_per_s": count / span, "amp_updates_per_s": amp / span, "wall_s": span,
             "steps": steps, "launches": launches, "compiled_launches": claunches,
             "compile_min_tiles": srv.compile_min_tiles, "requests_at_or_above_compile_min_tiles": compiled,
             "structures_compiled": srv.compiled_programs, "compile_errors": srv.compile_errors[:3]}
    if warm:
        stats["prepared_before_arrivals_s"] = t_warm
    del handles
    torch.cuda.empty_cache()
    return stats, outs


def bench_serving(dev, count: int, rate: float, seed: int, oracle_err: dict, policies=("srpt",)):
    """Open-loop Poisson arrivals (`rate` per second) of `count` mixed
    strongly-entangling requests: n ~ U{4..24}, depth ~ U{2..30}, batch
    log-uniform in [1, 512], <Z> out.  Live runs on the same arrival times:
    the continuous-batching server (with each scheduling policy asked for;
    the first is the record's headline), and a worker that serves the
    requests one after another in arrival order with the plain per-gate form
    (one launch per gate per request), starting each when it has arrived and
    the previous one is done.  Both include their per-request preparation in
    the latency (the server's lowering and planning, the per-gate form's
    module construction)."""
    import torch

    from oracle import oracle
    from qandle_gb300 import serve, workloads

    rng = np.random.default_rng(seed)
    reqs = [workloads.random_sel_request(rng) for _ in range(count)]
    offs = np.concatenate([[0.0], np.cumsum(rng.exponential(1.0 / rate, size=count - 1))])
    amp = float(sum(workloads.gate_count(d) * d["batch"] * (1 << d["n"]) for d in reqs))

    def live(variant):
        # "<policy>" compiles large structures in the background;
        # "<policy>_interpreted" runs everything on the interpreted kernel
        pol, _, interp = variant.partition("_")
        return _serve_live(dev, reqs, offs, amp, pol, compile_min_tiles=None if interp else 1024)

    fused, outs = live(policies[0])
    others = {}
    for pol in policies[1:]:
        st, o2 = live(pol)
        st["max_abs_diff_vs_" + policies[0]] = max(float((a - b).abs().max()) for a, b in zip(outs, o2))
        others[pol] = st

    # live per-gate FIFO on the same arrival times
    done_at = [None] * count
    diff = [0.0]
    stream = torch.cuda.Stream(device=dev)

    def worker(t_start):
        with torch.cuda.device(dev), torch.cuda.stream(stream):
            for i, (d, o) in enumerate(zip(reqs, offs)):
                wait = t_start + o - time.perf_counter()
                if wait > 0:
                    time.sleep(wait)
                out = serve.run_plain(d, dev).cpu()  # .cpu() waits for the request's kernels
                done_at[i] = time.perf_counter()
                diff[0] = max(diff[0], float((out - outs[i]).abs().max()))

    t0p = time.perf_counter()
    th = threading.Thread(target=worker, args=(t0p,))
    th.start()
    th.join()
    lat_p = np.array([(done_at[i] - (t0p + offs[i])) * 1e3 for i in range(count)])
    span_p = max(done_at) - t0p
    plain = {"p50_ms": float(np.percentile(lat_p, 50)), "p99_ms": float(np.percentile(lat_p, 99)),
             "circuits_per_s": count / span_p, "amp_updates_per_s": amp / span_p, "wall_s": span_p}
    # the oracle on the requests it finishes quickly (up to 14 qubits)
    err = 0.0
    checked = 0
    for d, o in zip(reqs, outs):
        if d["n"] <= 14:
            err = max(err, float(np.abs(o.numpy() - oracle.forward(d)).max()))
            checked += 1
    oracle_err[f"serving_{rate:g}_per_s_z_{checked}_requests_n_le_14"] = err
    return {"workload": f"{count} requests, Poisson {rate:g}/s, n ~ U{{4..24}}, depth ~ U{{2..30}}, "
                        f"batch log-uniform [1, 512], <Z> out (seed {seed})",
            "offered_s": float(offs[-1]), "amp_updates": amp, "continuous_batching": fused,
            "continuous_batching_other_policies": others,
            "per_gate_fifo_live": plain,
            "throughput_ratio": fused["circuits_per_s"] / plain["circuits_per_s"],
            "p99_ratio_per_gate_over_batched": plain["p99_ms"] / fused["p99_ms"],
            "max_abs_diff_vs_per_gate": diff[0], "max_abs_err_vs_oracle_n_le_14": err}


def bench_serving_repeated(dev, count: int, rate: float, seed: int, structures: int, oracle_err: dict):
    """Open-loop Poisson arrivals of `count` requests drawn from a few fixed
    circuit structures, as a deployment serving a handful of models sees
    them: strongly-entangling circuits, each structure with its own n ~
    U{12..24} (distinct) and depth ~ U{2..30}; each request with its own
    batch (log-uniform [1, 512]), angles and inputs, <Z> out.  Live runs on
    the same arrivals, shortest remaining work first: a cold server that
    plans and compiles inside the run, a warm server (every structure
    prepared before the first arrival), and the interpreted kernel only."""
    from oracle import oracle
    from qandle_gb300 import workloads

    rng = np.random.default_rng(seed)
    ns = rng.choice(np.arange(12, 25), size=structures, replace=False)
    pool = [(int(n), int(rng.integers(2, 31))) for n in ns]
    reqs = []
    for _ in range(count):
        n, depth = pool[int(rng.integers(len(pool)))]
        reqs.append(workloads.random_sel_request(rng, n_range=(n, n), depth_range=(depth, depth)))
    offs = np.concatenate([[0.0], np.cumsum(rng.exponential(1.0 / rate, size=count - 1))])
    amp = float(sum(workloads.gate_count(d) * d["batch"] * (1 << d["n"]) for d in reqs))
    warm = [workloads.random_sel_request(np.random.default_rng(0), n_range=(n, n), depth_range=(dp, dp), batch_max=1)
            for n, dp in pool]
    cold, outs = _serve_live(dev, reqs, offs, amp, "srpt")
    warm_st, outs_w = _serve_live(dev, reqs, offs, amp, "srpt", warm=warm)
    interp, outs_i = _serve_live(dev, reqs, offs, amp, "srpt", compile_min_tiles=None)
    for st, o in ((cold, outs), (warm_st, outs_w)):
        st["max_abs_diff_vs_interpreted"] = max(float((a - b).abs().max()) for a, b in zip(o, outs_i))
    err, checked = 0.0, 0
    for d, o in zip(reqs, outs_w):
        if d["n"] <= 14:
            err = max(err, float(np.abs(o.numpy() - oracle.forward(d)).max()))
            checked += 1
    oracle_err[f"serving_repeated_z_{checked}_requests_n_le_14"] = err
    return {"workload": f"{count} requests, Poisson {rate:g}/s, {structures} structures (n, depth) = {pool}, "
                        f"batch log-uniform [1, 512], <Z> out (seed {seed})",
            "offered_s": float(offs[-1]), "amp_updates": amp, "compiled_cold": cold, "compiled_warm": warm_st,
            "interpreted": interp,
            "throughput_ratio_warm_over_interpreted": warm_st["circuits_per_s"] / interp["circuits_per_s"],
            "max_abs_err_vs_oracle_n_le_14": err}


def bench_adjoint(dev, sync_all, W, hbm_peak, fp32_tflops, oracle_err, batch: int = 1024):
    import torch

    import qandle_gb300 as q
    from oracle import oracle
    from qandle_gb300 import plain, workloads

    desc = workloads.adjoint_brick(batch=batch)
    desc["measure"] = "p0"
    n, B = desc["n"], desc["batch"]
    targets = torch.tensor(desc["targets"], device=dev)
    st = torch.zeros(B, 1 << n, dtype=torch.complex64, device=dev)
    st[:, 0] = 1
    circ = workloads.build_circuit(desc, engine="fused", checkpoint_segments=4).to(dev)
    params = [m.theta for m in circ.circuit.layers if isinstance(m, q.BuiltParametrizedOperator)]

    def step():
        for p in params:
            p.grad = None
        p0 = circ(st)
        loss = ((2.0 * p0 - 1.0 - targets) ** 2).mean()
        loss.backward()
        return loss

    for _ in range(max(1, W)):
        step()
    sync_all()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    steps = 5
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    sync_all()
    fms = e0.elapsed_time(e1) / steps
    g_fused = torch.stack([p.grad.reshape(()) for p in params])

    # backward passes timed one by one (CUDA events on the launching stream)
    ex = circ._executor
    prog = ex.program(True)
    NB = prog.info.backward_passes
    amps = B * (1 << n)
    bms = []
    for _ in range(3):
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(2 * NB)]
        ex.backward_events = evs
        step()
        sync_all()
        bms.append([evs[2 * p].elapsed_time(evs[2 * p + 1]) for p in range(NB)])
    bms = np.array(bms).mean(0)
    bbytes = pass_bytes_bwd(prog, amps)
    bfmas = pass_fmas(prog, True, amps)
    comb, t_mem, t_fp = combined_roof(bms, bbytes, bfmas, hbm_peak, fp32_tflops)
    achieved = float(bbytes.mean() / (bms.mean() * 1e-3) / 1e9)

    # per-gate adjoint on the same circuit (one kernel pass per gate and state)
    circ_p = workloads.build_circuit(desc, engine="plain").to(dev)
    with torch.no_grad():
        p0 = circ_p(st)
    zexp = 2.0 * p0 - 1.0
    gp0 = (2.0 * (zexp - targets) / zexp.numel() * 2.0).contiguous()
    plain.adjoint_per_gate(list(circ_p.circuit.layers), n, gp0, state=st)
    sync_all()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    e2.record()
    g_plain = plain.adjoint_per_gate(list(circ_p.circuit.layers), n, gp0, state=st)
    e3.record()
    sync_all()
    pms = e2.elapsed_time(e3)
    g_plain = torch.stack([g.reshape(()) for g in g_plain])
    del circ_p
    torch.cuda.empty_cache()

    # the same workload at its full depth on 8 samples against the oracle
    small = workloads.adjoint_brick(batch=8)
    small["measure"] = "p0"
    cs = workloads.build_circuit(small, engine="fused", checkpoint_segments=4).to(dev)
    sts = torch.zeros(8, 1 << n, dtype=torch.complex64, device=dev)
    sts[:, 0] = 1
    pz = cs(sts)
    loss = ((2.0 * pz - 1.0 - torch.tensor(small["targets"], device=dev)) ** 2).mean()
    loss.backward()
    dth = np.array([m.theta.grad.item() for m in cs.circuit.layers if isinstance(m, q.BuiltParametrizedOperator)])
    p0_ref = oracle.forward(small)
    _, gref = oracle.mse_z_grad(2.0 * p0_ref - 1.0, small["targets"].astype(np.float64))
    rdp, _, _ = oracle.adjoint(small, gref, "p0")
    p_err = float(np.abs(pz.detach().cpu().numpy() - p0_ref).max())
    z_err = float(np.abs((2.0 * pz.detach().cpu().numpy() - 1.0) - (2.0 * p0_ref - 1.0)).max())
    g_err = float(np.abs(dth - rdp).max())
    oracle_err["config3_p0_8_samples"] = p_err
    oracle_err["config3_z_8_samples"] = z_err
    oracle_err["config3_grad_8_samples"] = g_err

    gates = len(desc["gates"])
    amp = gates * B * (1 << n)
    return {"workload": f"adjoint_brick: {n} qubits x batch {B}, 20 layers, {len(params)} angles, "
                        "MSE(<Z>, targets), 4 checkpoint segments",
            "ms_per_step_fused": fms, "ms_per_step_per_gate": pms,
            "fused_speedup": pms / fms,
            "amp_updates_per_s_fused": 3 * amp / (fms * 1e-3),
            "amp_updates_per_s_per_gate": 3 * amp / (pms * 1e-3),
            "gradients_per_s_fused": len(params) * B / (fms * 1e-3),
            "max_abs_grad_diff_fused_vs_per_gate": float((g_fused - g_plain).abs().max()),
            "plan": prog.summary(),
            "roofline": {"bound": "hbm", "kernel": "qg_bwd_pass (compiled per pass), 2^12-amplitude tiles",
                         "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                         "launches_per_step": NB, "avg_launch_ms": float(bms.mean()),
                         "algorithmic_bytes_per_launch": float(bbytes.mean()),
                         "bytes_per_amp": "32 (psi and lambda read and written), 16 on passes that only read",
                         "backward_ms_per_step": float(bms.sum()),
                         "fp32_frac": float(2.0 * bfmas.sum() / (bms.sum() * 1e-3) / (fp32_tflops * 1e12)),
                         "combined_frac": comb,
                         "passes_fp32_bound": int(np.sum(t_fp > t_mem)),
                         "per_pass": [{"ms": round(float(bms[p]), 4),
                                       "fma_per_amp": round(float(bfmas[p]) / amps, 1),
                                       "hbm_frac": round(float(bbytes[p] / (bms[p] * 1e-3) / 1e9 / hbm_peak), 3),
                                       "fp32_frac": round(float(2.0 * bfmas[p] / (bms[p] * 1e-3)
                                                                / (fp32_tflops * 1e12)), 3)}
                                      for p in range(NB)]},
            "max_abs_err_vs_oracle_8_samples": {"p0": p_err, "z": z_err, "grad": g_err},
            "note": "step = forward + backward; amp-updates count each gate once forward and twice "
                    "backward (state and cotangent)"}


if __name__ == "__main__":
    main()
