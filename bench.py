#!/usr/bin/env python
"""Benchmark of the qandle hot path on GB300.

Headline workload (one JSON line on rank 0): the fused forward of the
strongly-entangling re-uploading circuit, 20 qubits x batch 256 (complex64
state 2 GiB, larger than L2): AngleEmbedding(rx), 10 layers of RZ RY RZ per
qubit with a CNOT ring of range (layer mod 19) + 1, named RX re-uploading of
the inputs before layers 0 and 5, <Z> per qubit.  Metric: amplitude-updates/s
= gates x batch x 2^n per forward / time (860 gates, the embedding counted as
20 rotations).

Also on the line: the plain per-gate form on the same workload, the forward
replayed from one CUDA graph, the adjoint backward (16 qubits x batch 1024,
MSE(<Z>, targets)) against the per-gate adjoint, the fusion-width sweep
(--sweep), the HBM roofline of the pass kernel from CUDA events around every
pass launch, the end-to-end time through the public API with host buffers,
SM clocks sampled during the timed region, and the CPU oracle timed on the
host cores.

`--impl reference` times the CPU implementation of the same path (the
complex128 oracle, all host threads) on a bounded sample per step.
Under torchrun every rank runs its own batch (weak scaling, no collective on
the data path); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sweep", action="store_true", help="fusion-width sweep k = 1..7")
    ap.add_argument("--no-extras", action="store_true", help="headline only")
    ap.add_argument("--cpu-samples", type=int, default=16, help="samples in the CPU baseline")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--tile-bits", type=int, default=13)
    ap.add_argument("--low-bits", type=int, default=6)
    ap.add_argument("--k", type=int, default=0, help="max strided qubits per pass (0 = tile limit)")
    ap.add_argument("--reg-bits", type=int, default=5, help="amplitudes per thread = 2^reg_bits")
    ap.add_argument("--serving-requests", type=int, default=48, help="requests in the serving run")
    ap.add_argument("--autotune", action="store_true",
                    help="time the candidate plans first and run the headline with the fastest")
    ap.add_argument("--interpreted", action="store_true",
                    help="run the prebuilt op interpreter instead of the per-program compiled passes")
    ap.add_argument("--n", type=int, default=20)
    ap.add_argument("--batch", type=int, default=256)
    return ap.parse_args()


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


def cpu_baseline(desc, samples: int):
    """The oracle (complex128 port, all host threads) on `samples` samples of
    the workload; returns amplitude-updates/s and what was timed."""
    from oracle import oracle
    from qandle_gb300 import workloads

    threads = len(os.sched_getaffinity(0))
    lo = oracle.Lowered(desc, samples)
    t0 = time.perf_counter()
    oracle.run(desc, batch=samples, nthreads=threads, lowered=lo)
    dt = time.perf_counter() - t0
    amp = workloads.gate_count(desc) * samples * (1 << desc["n"])
    return {"value": amp / dt, "unit": "amp-updates/s", "cores": threads, "kind": "port",
            "sample": f"{samples} of {desc['batch']} samples of the {desc['n']}-qubit workload, "
                      f"{dt:.2f} s"}


def run_reference(args):
    """CPU arm: the oracle port on the host cores, each step a bounded sample."""
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
        r = cpu_baseline(desc, samples)
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
    print(json.dumps(line), flush=True)


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
                compiled=not args.interpreted)
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
    pass_ms = np.array([[events[s][2 * p].elapsed_time(events[s][2 * p + 1]) for p in range(P)]
                        for s in range(K)])
    # algorithmic bytes of each pass launch: 8 B per amplitude read, 8 B per
    # amplitude written (state), 4 B per probability written
    amps = B * (1 << n)
    pass_bytes = []
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
        pass_bytes.append(b)
    pass_bytes = np.array(pass_bytes, dtype=np.float64)
    avg_bytes = float(pass_bytes.mean())
    avg_pass_ms = float(pass_ms.mean())
    achieved = avg_bytes / (avg_pass_ms * 1e-3) / 1e9
    # per-pass bandwidth of the middle passes (load + store, 16 B / amplitude)
    mid = [p for p in range(P) if pass_bytes[p] == 16 * amps]
    mid_gbs = float(16 * amps / (pass_ms[:, mid].mean() * 1e-3) / 1e9) if mid else None
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "fwd_pass_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get("dram_bytes_per_launch")
    gpu_launches = K * (P + 3)  # matrix build, embedding factors, P passes, <Z> reduction

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
                     "middle_pass_GBps": mid_gbs},
        "clocks": clock_info,
        "gpu_launches": gpu_launches,
    }
    if tuned is not None:
        line["autotune"] = {"options": tuned["options"], "cached": tuned["cached"],
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
                   "ms_per_step": e2e_ms}

    if not args.no_extras:
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
        line["graph"] = {"value": amp_step / (gms * 1e-3), "ms_per_step": gms}
        del bound

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
        with torch.no_grad():
            fused_out = circ(**kw)
        line["plain"] = {"value": amp_step / (pms * 1e-3), "ms_per_step": pms,
                         "fused_speedup": pms / ms,
                         "max_abs_diff_vs_fused": float((fused_out - ref_out).abs().max())}
        del circ_p
        torch.cuda.empty_cache()

        # ---------------- adjoint: 16 qubits x batch 1024, MSE(<Z>, t) ----------------
        line["adjoint"] = bench_adjoint(dev, sync_all, W)
        torch.cuda.empty_cache()

        # ---------------- deep single state: 28 qubits x batch 1 ----------------
        line["deep28"] = bench_deep(dev, sync_all, W)
        torch.cuda.empty_cache()

        # ---------------- serving: Poisson arrivals of mixed-width requests ----------------
        line["serving"] = bench_serving(dev, args.serving_requests)
        torch.cuda.empty_cache()

        # ---------------- fusion width sweep ----------------
        if args.sweep:
            sweep = {}
            for k in range(1, 8):
                c = workloads.build_circuit(desc, engine="fused", max_high=k).to(dev)
                ex_k = None
                with torch.no_grad():
                    c(**kw)
                ex_k = c._executor
                bk = engine.BoundForward(ex_k, B, dev)
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
                sweep[str(k)] = {"passes": bk.prog.info.forward_passes, "ms_per_step": kms,
                                 "value": amp_step / (kms * 1e-3)}
                del bk, c
            line["k_sweep"] = sweep

    if rank == 0:
        line["cpu_baseline"] = None if args.no_cpu else cpu_baseline(desc, args.cpu_samples)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def bench_deep(dev, sync_all, W):
    """28 qubits, batch 1 (2 GiB), 50 layers of U per qubit with CNOT+SWAP
    brickwork, |psi|^2 out: fused forward against the per-gate form."""
    import torch

    from qandle_gb300 import engine, workloads

    desc = workloads.deep_u()
    n = desc["n"]
    amp = workloads.gate_count(desc) * (1 << n)
    circ = workloads.build_circuit(desc, engine="fused").to(dev)
    with torch.no_grad():
        circ()
    bound = engine.BoundForward(circ._executor, 1, dev)
    bound.set_inputs()  # the circuit's U matrices
    for _ in range(max(1, W)):
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
        sync_all()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record()
        plain_probs = circ_p().reshape(-1)
        p1.record()
        sync_all()
    pms = p0.elapsed_time(p1)
    diff = float((plain_probs - fused_probs).abs().max())
    return {"workload": f"deep_u: {n} qubits x batch 1, 50 layers of U + CNOT/SWAP brickwork, |psi|^2 out "
                        f"({workloads.gate_count(desc)} gates)",
            "plan": circ._executor.program(False).summary(),
            "ms_per_step_fused": fms, "ms_per_step_per_gate": pms, "fused_speedup": pms / fms,
            "amp_updates_per_s_fused": amp / (fms * 1e-3), "amp_updates_per_s_per_gate": amp / (pms * 1e-3),
            "norm_fused": norm, "max_abs_prob_diff_fused_vs_per_gate": diff}


def bench_serving(dev, count: int, rate: float = 2000.0, seed: int = 7):
    """Open-loop Poisson arrivals (rate per second) of mixed strongly-
    entangling requests: n ~ U{4..24}, depth ~ U{2..30}, batch log-uniform in
    [1, 512], <Z> out.  The continuous-batching server against the same
    requests served one after another in arrival order by the per-gate form
    (one launch per gate per request)."""
    import numpy as np
    import torch

    from qandle_gb300 import serve, workloads

    rng = np.random.default_rng(seed)
    reqs = [workloads.random_sel_request(rng) for _ in range(count)]
    offs = np.concatenate([[0.0], np.cumsum(rng.exponential(1.0 / rate, size=count - 1))])
    amp = float(sum(workloads.gate_count(d) * d["batch"] * (1 << d["n"]) for d in reqs))

    srv = serve.Server(dev, hbm_budget=160 << 30)
    try:
        t0 = time.perf_counter()
        handles = []
        for d, o in zip(reqs, offs):
            wait = t0 + o - time.perf_counter()
            if wait > 0:
                time.sleep(wait)
            handles.append(srv.submit(d, arrival=t0 + o))
        outs = [h.future.result(timeout=900) for h in handles]
        t_end = max(h.completed for h in handles)
        steps, launches = srv.steps, srv.launches
    finally:
        srv.close()
    lat = np.array([h.latency for h in handles]) * 1e3
    span = t_end - t0
    fused = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
             "circuits_per_s": count / span, "amp_updates_per_s": amp / span, "wall_s": span,
             "steps": steps, "launches": launches}
    del handles
    torch.cuda.empty_cache()

    service, diff = [], 0.0
    for i, d in enumerate(reqs):
        torch.cuda.synchronize(dev)
        s = time.perf_counter()
        out = serve.run_plain(d, dev).cpu()
        service.append(time.perf_counter() - s)
        diff = max(diff, float((out - outs[i]).abs().max()))
        del out
    done, lat_p = 0.0, []
    for o, sv in zip(offs, service):
        done = max(done, o) + sv
        lat_p.append((done - o) * 1e3)
    lat_p = np.array(lat_p)
    plain = {"p50_ms": float(np.percentile(lat_p, 50)), "p99_ms": float(np.percentile(lat_p, 99)),
             "circuits_per_s": count / done, "amp_updates_per_s": amp / done, "wall_s": done}
    return {"workload": f"{count} requests, Poisson {rate:g}/s, n ~ U{{4..24}}, depth ~ U{{2..30}}, "
                        "batch log-uniform [1, 512], <Z> out (seed 7)",
            "amp_updates": amp, "continuous_batching": fused, "per_gate_fifo": plain,
            "throughput_ratio": fused["circuits_per_s"] / plain["circuits_per_s"],
            "max_abs_diff_vs_per_gate": diff,
            "note": "per-gate latencies replay the measured service times in arrival order (FIFO)"}


def bench_adjoint(dev, sync_all, W):
    import torch

    import qandle_gb300 as q
    from qandle_gb300 import plain, workloads

    desc = workloads.adjoint_brick()
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
            "note": "step = forward + backward; amp-updates count each gate once forward and twice "
                    "backward (state and cotangent)"}


if __name__ == "__main__":
    main()
