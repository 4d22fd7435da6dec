#!/usr/bin/env python3
"""Throughput benchmark of the G-MCTDH propagation core on one GB300.

Workload: the 3-state quadratic vibronic-coupling model over 12 DOFs combined
pairwise into 6 logical modes of 20x20 harmonic DVR grids, 8 SPFs per mode and
state (262,144 complex coefficients per state), propagated with the CMF2
integrator and short-iterative Lanczos (seeded synthetic parameters,
``macaw_gb300.generate.qvc12``).  A step is one accepted CMF2 step of the
resident wavefunction; the metric is simulated femtoseconds per second of
device time (EOM evaluations per second reported beside it).

``--impl reference`` times the CPU oracle (the NumPy restatement of the
reference's Fortran path) on the host cores instead.  Under torchrun every rank
propagates an independent replica (the path has no data-parallel exchange).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from macaw_gb300.model import AU2FS, INT_CMF2, INT_RK45, initial_wavefunction  # noqa: E402
from macaw_gb300.generate import qvc12  # noqa: E402

METRIC = "simulated fs/s & EOM evals/s vs plain FP64 GPU path at |dC(t)|<=1e-6"
WORKLOAD = "qvc12: 3-state QVC, 12 DOFs -> 6 modes of 20x20 HO DVR, 8 SPFs/mode/state, CMF2+Lanczos"
EPS_CMF = 1e-5
PRE_FS = 1.0
MFX_EPOCHS = 12
TRAFFIC_PER_ALG_BYTE = 0.51   # ncu DRAM bytes per algorithmic byte, mode products of this model
ACC_FS = 0.5   # interval over which the split path is compared with the FP64 path
REF_STEP_FS = 0.1   # CMF2 step length the reference arm times (steady-state steps are of this order)


def make_model():
    return qvc12(eps_int=EPS_CMF, eps_lanczos=1e-8, eps_spf=1e-7)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.lines = []
        self.idx = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.idx), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
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
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        tdist.init_process_group("nccl")
        return ws, rank, tdist
    return 1, 0, None


def barrier(tdist):
    if tdist is not None:
        tdist.barrier()


def max_over_ranks(vals, tdist, device="cuda"):
    """Each value's maximum over the ranks (the slowest rank's time); the values
    themselves without a process group."""
    if tdist is None:
        return [float(v) for v in vals]
    import torch
    t = torch.tensor([float(v) for v in vals], device=device, dtype=torch.float64)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def flush_l2(buf):
    buf.add_(1.0)


def cpu_baseline(model, A, psi, h, budget_s=40.0):
    """The oracle on a bounded sample: fixed-length CMF2 attempts of length h."""
    from oracle.mctdh import Oracle
    o = Oracle(model)
    t0 = time.perf_counter()
    n = 0
    A_, p_ = A.copy(), psi.copy()
    while True:
        A_, p_, _ = o.cmf2_fixed(A_, p_, 0.0, h)
        n += 1
        el = time.perf_counter() - t0
        if el > budget_s or n >= 3:
            break
    return dict(value=n * h * AU2FS / el, unit="fs/s", cores=os.cpu_count(), kind="port",
                sample=f"{n} CMF2 step(s) of {h * AU2FS:.4f} fs on the full qvc12 model, NumPy oracle "
                       f"(BLAS threads = host cores), {el:.1f} s")


def run_reference(args):
    ws, rank, tdist = dist_setup()
    if rank != 0:
        return 0
    model = make_model()
    A, psi = initial_wavefunction(model)
    h = REF_STEP_FS / AU2FS
    from oracle.mctdh import Oracle
    o = Oracle(model)
    # each step: one fixed-length CMF2 step of the oracle; bounded to a few minutes
    t_total, fs_total, n = 0.0, 0.0, 0
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        A, psi, _ = o.cmf2_fixed(A, psi, 0.0, h)
        el = time.perf_counter() - t0
        if i >= min(args.warmup, 1):
            t_total += el
            fs_total += h * AU2FS
            n += 1
        if t_total > 150.0 and n >= 1:
            break
    v = fs_total / t_total
    line = {"metric": METRIC, "value": v, "unit": "fs/s", "n_gpus": ws, "steps": n, "warmup": min(args.warmup, 1),
            "ms_per_step": 1e3 * t_total / n, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128", "data": "synthetic (seeded qvc12 model)", "impl": "reference",
            "config": {"workload": WORKLOAD, "integrator": "cmf2", "step_fs": h * AU2FS},
            "cpu_baseline": {"value": v, "unit": "fs/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"{n} fixed CMF2 steps of {h * AU2FS} fs, NumPy oracle on host cores"},
            "e2e": {"value": v, "unit": "fs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def timed_steps(core, t, h, steps, l2, torch):
    """K accepted CMF2 steps on the resident state, each bracketed by CUDA events on
    the library's stream after an L2 flush; returns (t, h, device ms, simulated fs, hdids)."""
    ms_total, fs_total, hdids = 0.0, 0.0, []
    for _ in range(steps):
        flush_l2(l2)
        torch.cuda.synchronize()
        core.event_record(0)
        hdid, hnext, _ = core.step(INT_CMF2, t, h)
        core.event_record(1)
        ms_total += core.event_elapsed(0, 1)
        t += hdid
        h = hnext
        fs_total += hdid * AU2FS
        hdids.append(hdid * AU2FS)
    return t, h, ms_total, fs_total, hdids


def run_arm(model, precision, state, t0, h0, args, l2, torch, tdist, profile, mfx_net=None):
    from macaw_gb300.capi import GpuCore
    A0, psi0, A1, psi1 = state
    core = GpuCore(model, precision=precision)
    core.set_state(A0, psi0, as_start=True)
    core.set_state(A1, psi1, as_start=False)
    warm = args.warmup
    if mfx_net is not None:
        # the extrapolator needs five accepted step starts of history
        core.mfx_attach(*mfx_net, tol=model.eps_int)
        warm = max(warm, 6)
    t, h = t0, h0
    for _ in range(warm):
        hdid, h, _ = core.step(INT_CMF2, t, h)
        t += hdid
    c0 = core.counters()
    barrier(tdist)
    torch.cuda.synchronize()
    t, h, ms, fs, hdids = timed_steps(core, t, h, args.steps, l2, torch)
    torch.cuda.synchronize()
    barrier(tdist)
    c1 = core.counters()
    prof, prof_ms = None, None
    if profile:
        # per-kernel-class CUDA events on the same number of further steps (a
        # separate pass: the events and the launches without graphs it needs
        # stay out of the timed region above)
        core.profile(2)
        torch.cuda.synchronize()
        core.event_record(0)
        tp, hp = t, h
        for _ in range(args.steps):
            hdid, hp, _ = core.step(INT_CMF2, tp, hp)
            tp += hdid
        core.event_record(1)
        torch.cuda.synchronize()
        prof_ms = core.event_elapsed(0, 1)
        prof = core.profile_read()
        core.profile(0)
    return core, dict(t=t, h=h, ms=ms, fs=fs, hdids=hdids, prof=prof, prof_ms=prof_ms,
                      eom=c1["eom"] - c0["eom"], hb=c1["hb"] - c0["hb"], launches=c1["launches"] - c0["launches"])


def run_size_scan(args):
    """qvc12n: the benchmark model with `--nspf` SPFs per mode and state (12: 2.99 M
    configurations per state, 143 MB of coefficients, beyond the 129 MB L2), split
    path against the FP64 path from the same state at 1 fs, as the benchmark line
    does (no learned extrapolator, no CPU baseline)."""
    import torch
    from macaw_gb300.capi import GpuCore
    _, _, tdist = dist_setup()
    torch.cuda.init()
    model = qvc12(nspf=args.nspf, eps_int=EPS_CMF, eps_lanczos=1e-8, eps_spf=1e-7)
    A0, psi0 = initial_wavefunction(model)
    l2 = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    pre = GpuCore(model, precision=0)
    pre.set_state(A0, psi0, as_start=True)
    t1, h1, _, _, _ = pre.propagate_interval(INT_CMF2, PRE_FS / AU2FS, 0.0, model.tout * model.eps_int)
    A1, psi1 = pre.get_state()
    pre.close()
    state = (A0, psi0, A1, psi1)
    with ClockSampler(torch.cuda.current_device()) as clk:
        ref_core, ref = run_arm(model, 0, state, t1, h1, args, l2, torch, tdist, profile=False)
        mix_core, mix = run_arm(model, args.precision, state, t1, h1, args, l2, torch, tdist, profile=False)
    cmp = {}
    for name, core in (("fp64", ref_core), ("mixed", mix_core)):
        core.set_state(A1, psi1, as_start=False)
        tt, _, _, _, _ = core.propagate_interval(INT_CMF2, t1 + ACC_FS / AU2FS, t1, h1)
        cmp[name] = core.observables(tt)
    value = mix["fs"] / (mix["ms"] * 1e-3)
    fp64_value = ref["fs"] / (ref["ms"] * 1e-3)
    ntot = int(model.naconftot)
    line = {"metric": f"simulated fs/s (qvc12, {args.nspf} SPFs, CMF2)", "value": value, "unit": "fs/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": mix["ms"] / args.steps,
            "higher_is_better": True, "precision": args.precision,
            "fp64_path": {"value": fp64_value, "ms_per_step": ref["ms"] / args.steps},
            "speedup_vs_fp64_path": value / fp64_value,
            "accuracy_vs_fp64_path": {"dC": abs(cmp["mixed"]["auto"] - cmp["fp64"]["auto"]),
                                      "dpop": float(np.abs(cmp["mixed"]["pop"] - cmp["fp64"]["pop"]).max()),
                                      "over_fs": ACC_FS, "from_fs": PRE_FS},
            "eom_per_s": mix["eom"] / (mix["ms"] * 1e-3), "hb_per_s": mix["hb"] / (mix["ms"] * 1e-3),
            "fp64_eom_per_s": ref["eom"] / (ref["ms"] * 1e-3),
            "clocks": clk.summary(),
            "device_bytes": {"fp64": ref_core.device_bytes(), "split": mix_core.device_bytes()},
            "config": {"workload": "qvc12n", "nspf": args.nspf, "coefficients": ntot,
                       "coefficient_bytes": 16 * ntot, "dimpsi": int(model.dimpsi),
                       "l2": "flushed (256 MB write) before every timed step"}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import torch
    from macaw_gb300.capi import GpuCore, fp64_peak_tflops
    ws, rank, tdist = dist_setup()
    torch.cuda.init()
    model = make_model()
    A0, psi0 = initial_wavefunction(model)
    l2 = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2
    # leave the start-up transient of the step control (the reference starts at
    # tout * eps_int, propagator.f90:103, and grows by at most 1.5x per CMF2 step):
    # propagate 1 fs untimed with the FP64 path; both arms start from that state
    pre = GpuCore(model, precision=0)
    pre.set_state(A0, psi0, as_start=True)
    pre.mfx_record(2)   # the untimed FP64 steps are the extrapolator's training data
    t1, h1, _, _, _ = pre.propagate_interval(INT_CMF2, PRE_FS / AU2FS, 0.0, model.tout * model.eps_int)
    A1, psi1 = pre.get_state()
    from macaw_gb300 import mfx
    tr0 = time.perf_counter()
    X, R, ks = mfx.build_dataset(*pre.mfx_fetch())
    net, fscale, tscale, tr_loss = mfx.train(X, R, steps=ks, epochs=MFX_EPOCHS)
    train_s = time.perf_counter() - tr0
    pre.close()
    state = (A0, psi0, A1, psi1)
    with ClockSampler(torch.cuda.current_device()) as clk:
        ref_core, ref = run_arm(model, 0, state, t1, h1, args, l2, torch, tdist, profile=False)
        mix_core, mix = run_arm(model, args.precision, state, t1, h1, args, l2, torch, tdist, profile=True)
        mfx_core, mfxr = run_arm(model, args.precision, state, t1, h1, args, l2, torch, tdist, profile=False,
                                 mfx_net=(net, fscale, tscale))
    # accuracy against the plain FP64 path: every arm propagates the same state over
    # the same output interval; C(t) and populations are compared there
    cmp = {}
    for name, core in (("fp64", ref_core), ("mixed", mix_core), ("mfx", mfx_core)):
        core.set_state(A1, psi1, as_start=False)
        tt, _, _, _, _ = core.propagate_interval(INT_CMF2, t1 + ACC_FS / AU2FS, t1, h1)
        cmp[name] = core.observables(tt)
    dC = abs(cmp["mixed"]["auto"] - cmp["fp64"]["auto"])
    dpop = float(np.abs(cmp["mixed"]["pop"] - cmp["fp64"]["pop"]).max())
    mfx_stats = mfx_core.mfx_stats()
    ms_total, fs_total = mix["ms"], mix["fs"]
    ms_total, ref["ms"], mfxr["ms"] = max_over_ranks([ms_total, ref["ms"], mfxr["ms"]], tdist)
    value = ws * fs_total / (ms_total * 1e-3)
    fp64_value = ws * ref["fs"] / (ref["ms"] * 1e-3)
    mfx_value = ws * mfxr["fs"] / (mfxr["ms"] * 1e-3)

    # e2e: the reference-facing host-buffer call (mctdh_cmf2) with pinned buffers,
    # host<->device copies of A and psi inside every step
    Ah, ph = mix_core.get_state()
    pA = torch.from_numpy(Ah.copy()).pin_memory()
    pP = torch.from_numpy(ph.copy()).pin_memory()
    import ctypes as C
    DPp = C.POINTER(C.c_double)
    hd, hn = C.c_double(), C.c_double()
    e2e_fs, e2e_s = 0.0, 0.0
    te, he = mix["t"], mix["h"]
    for _ in range(max(1, args.steps // 2)):
        flush_l2(l2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = mix_core.lib.mctdh_cmf2(mix_core.h, C.cast(pA.data_ptr(), DPp), C.cast(pP.data_ptr(), DPp), te, he,
                                     C.byref(hd), C.byref(hn))
        e2e_s += time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError(mix_core.lib.mctdh_last_error(mix_core.h).decode())
        te += hd.value
        he = hn.value
        e2e_fs += hd.value * AU2FS
    nbytes = 16 * (model.naconftot + model.dimpsi)

    prof = mix["prof"]
    peaks, peak_src = load_peaks()
    fp64_peak = fp64_peak_tflops()
    dom = max(prof.items(), key=lambda kv: kv[1]["ms"])
    dname, d = dom
    avg_ms = d["ms"] / max(d["launches"], 1)
    fl_launch = d["flops"] / max(d["launches"], 1)
    by_launch = d["bytes"] / max(d["launches"], 1)
    achieved_gbs = by_launch / (avg_ms * 1e-3) / 1e9 if avg_ms > 0 else 0.0
    achieved_tf = fl_launch / (avg_ms * 1e-3) / 1e12 if avg_ms > 0 else 0.0
    clocks = clk.summary()
    tot_ms = max(sum(x["ms"] for x in prof.values()), 1e-9)
    line = {
        "metric": METRIC, "value": value, "unit": "fs/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded qvc12 model)",
        "config": {"workload": WORKLOAD, "integrator": "cmf2",
                   "precision": {0: "fp64", 1: "split-fp32", 2: "split-fp32-compensated"}[args.precision],
                   "eps_cmf": EPS_CMF, "l2": "flushed (256 MB write) before every timed step",
                   "step_fs_mean": statistics.mean(mix["hdids"]), "parallelism": f"replicas x{ws}"},
        "fp64_path": {"value": fp64_value, "unit": "fs/s", "ms_per_step": ref["ms"] / args.steps,
                      "step_fs_mean": statistics.mean(ref["hdids"])},
        "speedup_vs_fp64_path": value / fp64_value,
        "accuracy_vs_fp64_path": {"dC": dC, "dpop": dpop, "over_fs": ACC_FS, "from_fs": t1 * AU2FS},
        "mfx_path": {"value": mfx_value, "unit": "fs/s", "ms_per_step": mfxr["ms"] / args.steps,
                     "step_fs_mean": statistics.mean(mfxr["hdids"]),
                     "speedup_vs_fp64_path": mfx_value / fp64_value,
                     "accuracy_vs_fp64_path": {
                         "dC": abs(cmp["mfx"]["auto"] - cmp["fp64"]["auto"]),
                         "dpop": float(np.abs(cmp["mfx"]["pop"] - cmp["fp64"]["pop"]).max())},
                     "eom_per_s": mfxr["eom"] / (mfxr["ms"] * 1e-3),
                     "extrapolated_steps": mfx_stats["mlp_steps"], "fallbacks": mfx_stats["fallbacks"],
                     "rejected": mfx_stats["rejected"], "last_step_end_mismatch": mfx_stats["last_rel"],
                     "training": {"rows": int(len(X)), "epochs": MFX_EPOCHS, "loss": tr_loss,
                                  "seconds": train_s,
                                  "data": f"the untimed FP64 CMF2 steps from 0 to {PRE_FS} fs"}},
        "eom_per_s": mix["eom"] / (ms_total * 1e-3), "hb_per_s": mix["hb"] / (ms_total * 1e-3),
        "e2e": {"value": e2e_fs / e2e_s, "unit": "fs/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes},
        "gpu_launches": mix["launches"],
        "roofline": {"bound": "hbm", "kernel": dname, "achieved": achieved_gbs, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved_gbs / peaks["hbm_gbs"],
                     "traffic": by_launch * TRAFFIC_PER_ALG_BYTE if dname == "mode_product" else None,
                     "traffic_source": "ncu DRAM bytes / algorithmic bytes of the mean-field chain product launches of "
                                       "this model (profiles/qvc12_cmf2_split32_ncu.md), times the "
                                       "algorithmic bytes per launch",
                     "peak_source": peak_src},
        "compute": ({"kernel": dname, "achieved": achieved_tf, "unit": "TFLOP/s (complex MAC = 8 flop)",
                     "fp64_peak": fp64_peak, "frac_of_fp64_peak": achieved_tf / fp64_peak if fp64_peak > 0 else None,
                     "peak_source": "measured FP64 FMA chain on this GPU"} if args.precision == 0 else
                    {"kernel": dname, "achieved": achieved_tf, "unit": "TFLOP/s (complex MAC = 8 flop)",
                     "note": "FP32 mode products: issue-bound in ncu (issue 52-68 %, FMA pipe 27-32 %)"}),
        "kernel_profile": {k: {"ms": round(v["ms"], 3), "launches": v["launches"],
                               "share": round(v["ms"] / tot_ms, 4)}
                           for k, v in prof.items() if v["launches"]},
        "gpu_busy_frac_profiled_pass": tot_ms / mix["prof_ms"] if mix["prof_ms"] else None,
        "clocks": clocks,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(model, A0, psi0, statistics.mean(mix["hdids"]) / AU2FS)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ref_core.close()
    mix_core.close()
    mfx_core.close()
    if tdist is not None:
        tdist.destroy_process_group()
    return 0


def run_accuracy(args):
    """Accuracy of the split-precision arms against the plain FP64 path over the
    full propagation of the benchmark model (qvc12, CMF2 at tolerance 1e-5, 200 fs
    from the initial state): every arm propagates from t = 0 with its own step
    control, and C(t) and the state populations are compared at every output
    time (0.5 fs).  Reported: the largest |dC| and |dpop| over the run, their
    values at the end, device seconds and simulated fs/s of each arm."""
    import torch
    from macaw_gb300.capi import GpuCore
    torch.cuda.init()
    model = make_model()
    A0, psi0 = initial_wavefunction(model)
    t_end = args.acc_fs / AU2FS
    arms = [0] + [int(p) for p in args.acc_precisions.split(",") if p.strip()]
    series, info = {}, {}
    for prec in arms:
        core = GpuCore(model, precision=prec)
        core.set_state(A0, psi0, as_start=True)
        t, h = 0.0, model.tout * model.eps_int
        rows = [core.observables(t)]
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        nsteps = 0
        while t < t_end - 1e-9:
            t, h, ns, _, _ = core.propagate_interval(INT_CMF2, min(t + model.tout, t_end), t, h)
            nsteps += ns
            rows.append(core.observables(t))
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
        series[prec] = rows
        info[prec] = {"wall_s": wall, "fs_per_s": args.acc_fs / wall, "steps": nsteps,
                      "device_bytes": core.device_bytes()}
        core.close()
    ref = series[0]
    out = {"workload": "accuracy: qvc12 CMF2 (tolerance 1e-5) from t = 0, outputs every "
                       f"{model.tout * AU2FS:g} fs", "over_fs": args.acc_fs, "fp64": info[0], "arms": {}}
    for prec in arms[1:]:
        rows = series[prec]
        n = min(len(rows), len(ref))
        dC = [abs(rows[i]["auto"] - ref[i]["auto"]) for i in range(n)]
        dpop = [float(np.abs(rows[i]["pop"] - ref[i]["pop"]).max()) for i in range(n)]
        dE = [abs(rows[i]["energy"] - ref[i]["energy"]) for i in range(n)]
        dN = [abs(rows[i]["norm"] - ref[i]["norm"]) for i in range(n)]
        imax = int(np.argmax(dC))
        out["arms"][str(prec)] = dict(info[prec], max_dC=max(dC), t_max_dC_fs=rows[imax]["t"] * AU2FS,
                                      max_dpop=max(dpop), end_dC=dC[n - 1], end_dpop=dpop[n - 1],
                                      max_denergy=max(dE), max_dnorm=max(dN), outputs=n,
                                      speedup_vs_fp64_wall=info[0]["wall_s"] / info[prec]["wall_s"])
    print(json.dumps(out), flush=True)
    return 0


def run_profile_case(args):
    """A short, fixed piece of the workload for profiler captures: three CMF2 steps
    of 1e-3 fs from the initial state of the qvc12 model (about 1,700 launches), or
    with `--workload gmctdh16` three EOM evaluations of the Gaussian model."""
    from macaw_gb300.capi import GpuCore
    if args.workload == "gmctdh16":
        # three EOM evaluations of the Gaussian model on its initial state
        from macaw_gb300.generate import gmctdh16
        model = gmctdh16()
        A0, psi0 = initial_wavefunction(model)
        core = GpuCore(model, precision=args.precision)
        for _ in range(3):
            core.calc_derivs(A0, psi0, 0.0)
        print(json.dumps({"profile_case": "gmctdh16", "precision": args.precision,
                          "launches": core.launch_count()}), flush=True)
        core.close()
        return 0
    # `--workload qvc12n`: the same with `--nspf` SPFs
    model = (qvc12(nspf=args.nspf, eps_int=EPS_CMF, eps_lanczos=1e-8, eps_spf=1e-7)
             if args.workload == "qvc12n" else make_model())
    A0, psi0 = initial_wavefunction(model)
    core = GpuCore(model, precision=args.precision)
    core.set_state(A0, psi0, as_start=True)
    t, h = 0.0, 1e-3 / AU2FS
    if args.profile_from_fs > 0.0:
        # untimed propagation into the regime of the benchmark line; only the three
        # steps after it run between cudaProfilerStart/Stop (ncu --profile-from-start off)
        import torch
        torch.cuda.init()
        t, h, _, _, _ = core.propagate_interval(INT_CMF2, args.profile_from_fs / AU2FS, t, model.tout * model.eps_int)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
    l0 = core.launch_count()
    for _ in range(3):
        hdid, h, _ = core.step(INT_CMF2, t, h)
        t += hdid
    if args.profile_from_fs > 0.0:
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    print(json.dumps({"profile_case": args.workload, "precision": args.precision, "t_fs": t * AU2FS,
                      "launches": core.launch_count() - l0}), flush=True)
    core.close()
    return 0


def run_ensemble(args):
    """Batched-ensemble workload: ragged LVC members (2-4 states, 4-10 modes,
    4-10 SPFs, 16-48 points per mode, configurations per state capped) advanced
    together with lockstep RK45, against the same members propagated one context
    at a time.  Unit: member-fs/s (simulated fs summed over members per second)."""
    import torch
    from macaw_gb300.capi import Ensemble, GpuCore
    from macaw_gb300.generate import ensemble
    torch.cuda.init()
    models = ensemble(count=args.members, max_conf=args.max_conf)
    starts = [initial_wavefunction(m) for m in models]
    ens = Ensemble(models)
    for i, (A, psi) in enumerate(starts):
        ens.set_state(i, A, psi, as_start=True)
    t = np.zeros(len(models))
    step = np.array([m.tout * m.eps_int for m in models])
    # untimed start-up transient (steps grow from tout * eps_int)
    ens.propagate(INT_RK45, 0.1 / AU2FS, t, step)
    t0 = t.copy()
    es = torch.cuda.ExternalStream(ens.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0 = ens.counters()
    torch.cuda.synchronize()
    ev0.record(es)
    rounds, neom = ens.propagate(INT_RK45, (0.1 + args.ens_fs) / AU2FS, t, step)
    ev1.record(es)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    c1 = ens.counters()
    fs_total = float(np.sum(t - t0)) * AU2FS
    # the same members one context at a time (sequential), same interval
    seq_ms = 0.0
    nseq = min(len(models), args.seq_members)
    seq_fs = 0.0
    for i in range(nseq):
        core = GpuCore(models[i])
        A, psi = starts[i]
        core.set_state(A, psi, as_start=True)
        tt, ss, _, _, _ = core.propagate_interval(INT_RK45, 0.1 / AU2FS, 0.0, models[i].tout * models[i].eps_int)
        torch.cuda.synchronize()
        w = time.perf_counter()
        tt2, _, _, _, _ = core.propagate_interval(INT_RK45, (0.1 + args.ens_fs) / AU2FS, tt, ss)
        torch.cuda.synchronize()
        seq_ms += 1e3 * (time.perf_counter() - w)
        seq_fs += (tt2 - tt) * AU2FS
        core.close()
    sizes = [m.naconftot + m.dimpsi for m in models]
    line = {"metric": "member-fs/s of a batched ensemble (lockstep RK45)", "value": fs_total / (ms * 1e-3),
            "unit": "member-fs/s", "n_gpus": 1, "members": len(models), "ms": ms, "rounds": rounds,
            "eom_member_evals_per_s": (c1["eom"] - c0["eom"]) * len(models) / (ms * 1e-3),
            "launches": c1["launches"] - c0["launches"],
            "sequential": {"members": nseq, "member_fs_per_s": seq_fs / (seq_ms * 1e-3) if seq_ms else None,
                           "timing": "host wall clock around each member's propagate call"},
            "config": {"workload": "ragged LVC ensemble", "interval_fs": args.ens_fs, "max_conf": args.max_conf,
                       "coefficients_total": int(sum(sizes)), "largest_member": int(max(sizes)),
                       "smallest_member": int(min(sizes))}}
    if line["sequential"]["member_fs_per_s"]:
        line["batched_over_sequential"] = line["value"] / line["sequential"]["member_fs_per_s"]
    print(json.dumps(line), flush=True)
    ens.close()
    return 0


def run_rk_workload(args):
    """RK configurations: lvc5 (2-state LVC over 5 HO modes, Cash-Karp, eps 1e-8)
    and gmctdh16 (2-state LVC, 4 HO modes + one 12-DOF Gaussian mode with 32
    Gaussians per state) and lvc5mix (lvc5 as a 4-packet mixture under Lindblad
    dephasing of mode 1: type-1 and type-2 dissipation).  After 0.2 fs untimed, `--rk-fs` fs timed with CUDA
    events on the library's stream; C(t) against the FP64 path when the
    precision is split."""
    import torch
    from macaw_gb300.capi import GpuCore
    from macaw_gb300.generate import lvc5, gmctdh16, lvc5_mixture
    torch.cuda.init()
    model = {"lvc5": lvc5, "gmctdh16": gmctdh16, "lvc5mix": lvc5_mixture}[args.workload]()
    A0, psi0 = initial_wavefunction(model)
    out = {}
    for prec in sorted({0, args.precision}):
        core = GpuCore(model, precision=prec)
        core.set_state(A0, psi0, as_start=True)
        t, h, _, _, _ = core.propagate_interval(INT_RK45, 0.2 / AU2FS, 0.0, model.tout * model.eps_int)
        torch.cuda.synchronize()
        e0 = core.counters()["eom"]
        core.event_record(0)
        t1, h1, nsteps, natt, _ = core.propagate_interval(INT_RK45, t + args.rk_fs / AU2FS, t, h)
        core.event_record(1)
        torch.cuda.synchronize()
        ms = core.event_elapsed(0, 1)
        ob = core.observables(t1)
        out[prec] = dict(fs_per_s=(t1 - t) * AU2FS / (ms * 1e-3), ms=ms, steps=nsteps, attempts=natt,
                         eom_per_s=(core.counters()["eom"] - e0) / (ms * 1e-3), auto=ob["auto"], pop=ob["pop"])
        core.close()
    line = {"metric": f"simulated fs/s ({args.workload}, RK45)", "value": out[args.precision]["fs_per_s"],
            "unit": "fs/s", "n_gpus": 1, "precision": args.precision,
            "fp64_fs_per_s": out[0]["fs_per_s"], "eom_per_s": out[args.precision]["eom_per_s"],
            "steps": out[args.precision]["steps"], "attempts": out[args.precision]["attempts"],
            "ms": out[args.precision]["ms"],
            "config": {"workload": args.workload, "interval_fs": args.rk_fs, "from_fs": 0.2,
                       "coefficients": int(model.naconftot * model.npackets), "dimpsi": int(model.dimpsi),
                       "npackets": int(model.npackets), "dissipative_operators": len(model.dissipation),
                       "eps_int": model.eps_int}}
    if args.precision != 0:
        line["accuracy_vs_fp64_path"] = {
            "dC": abs(out[args.precision]["auto"] - out[0]["auto"]),
            "dpop": float(np.abs(out[args.precision]["pop"] - out[0]["pop"]).max())}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--acc-fs", type=float, default=200.0, help="accuracy: propagated interval in fs")
    ap.add_argument("--acc-precisions", default="1,3", help="accuracy: split arms compared with FP64")
    ap.add_argument("--precision", type=int, default=1, choices=[0, 1, 2, 3],
                    help="arm timed against the FP64 path: 1 split FP32, 2 compensated split FP32")
    ap.add_argument("--workload", default="qvc12",
                    choices=["qvc12", "qvc12n", "ensemble", "lvc5", "gmctdh16", "lvc5mix", "accuracy"],
                    help="qvc12: the CMF2 benchmark line; ensemble: the batched ragged-ensemble measurement; "
                         "lvc5 / gmctdh16: RK configurations")
    ap.add_argument("--rk-fs", type=float, default=0.5)
    ap.add_argument("--nspf", type=int, default=12, help="qvc12n: SPFs per mode and state")
    ap.add_argument("--members", type=int, default=128)
    ap.add_argument("--max-conf", type=int, default=1 << 14)
    ap.add_argument("--ens-fs", type=float, default=0.5)
    ap.add_argument("--seq-members", type=int, default=16)
    ap.add_argument("--profile-from-fs", type=float, default=0.0,
                    help="profile case: propagate this far first, profile only the three steps after it")
    ap.add_argument("--profile-case", action="store_true",
                    help="run a short fixed piece of the workload (for profiler captures) instead of the benchmark")
    args = ap.parse_args()
    if args.profile_case:
        return run_profile_case(args)
    if args.workload == "ensemble":
        return run_ensemble(args)
    if args.workload == "accuracy":
        return run_accuracy(args)
    if args.workload == "qvc12n":
        return run_size_scan(args)
    if args.workload in ("lvc5", "gmctdh16", "lvc5mix"):
        return run_rk_workload(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
