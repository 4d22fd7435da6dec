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
# extrapolate a step start only after a step whose first attempt used less than
# half of the CMF2 error tolerance: at the step control's operating point (error
# ~1) the extrapolation's error shifts the CMF2 error estimate enough to cost
# rejected attempts
MFX_GATE = 0.5
# ncu DRAM bytes per algorithmic byte of a kernel class in the benchmark regime
# (one capture of the profile case), and what bounds each class there
# DRAM bytes per algorithmic byte of the mode products: 177.5 MB of DRAM traffic
# over 461 MB of operand bytes in the eight mode-product launches of one ncu
# capture of the profile case at precision 5 (`--profile-case --precision 5
# --profile-from-fs 1`: five compensated mean-field chain launches, three FP32
# H_B*B launches)
TRAFFIC_PER_ALG_BYTE = {"mode_product": 0.385}
ROOF_BOUND = {"mode_product": "hbm", "hole_contract": "hbm", "spf_derivative": "hbm"}
ROOF_NOTE = {"mode_product": "not HBM: the compensated mean-field products are FMA-issue bound (55 % of the FMA "
                             "pipe), the FP32 H_B products load-latency bound; operands mostly L2-resident "
                             "(12.6 MB state)",
             "hole_contract": "compensated FP32 sums: FP32 issue",
             "spf_derivative": "small per-mode problems: latency and occupancy"}
ACC_FS = 0.5   # short comparison interval of the size scan
REF_BUDGET_S = 150.0   # timed seconds after which the reference arm stops early


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


PRECISION_LABEL = {0: "fp64", 1: "fp32 products, compensated fp32 contractions",
                   2: "compensated fp32 products and contractions", 3: "fp32 products and contractions",
                   4: "fp32 mean-field products, compensated H_B products and contractions",
                   5: "compensated mean-field products and contractions, fp32 H_B products",
                   6: "fp32 products and mean-field contractions, compensated densities"}


def precision_label(prec):
    return PRECISION_LABEL[prec]


def static_config(ws):
    """The workload definition both arms report (nothing measured in it)."""
    return {"workload": WORKLOAD, "integrator": "cmf2", "eps_cmf": EPS_CMF, "start_fs": PRE_FS,
            "step": "one accepted adaptive CMF2 step (reference step control)",
            "l2": "flushed (256 MB write) before every timed step", "parallelism": f"replicas x{ws}"}


_ONE_THREAD = r"""
import sys, time, numpy as np
sys.path.insert(0, sys.argv[1])
from bench import make_model
from oracle.mctdh import Oracle
d = np.load(sys.argv[2])
o = Oracle(make_model())
t0 = time.perf_counter()
o.cmf2_fixed(d["A"], d["psi"], float(d["t"]), float(d["h"]))
print(time.perf_counter() - t0)
"""


def cpu_baseline(model, A1, psi1, t1, h, gpu64, steps=2):
    """The oracle on a bounded sample of the workload: `steps` CMF2 steps of the
    GPU arm's mean step length from the state the GPU arm starts from, with all
    host cores (NumPy's BLAS threads), and one step single-threaded in a child
    process.  The same steps through the FP64 device path (mctdh_cmf2_attempt)
    give the parity check carried in the line."""
    import tempfile
    from oracle.mctdh import Oracle
    o = Oracle(model)
    rA, rp = A1.copy(), psi1.copy()
    gA, gp = A1.copy(), psi1.copy()
    el = 0.0
    for k in range(steps):
        w0 = time.perf_counter()
        rA, rp, _ = o.cmf2_fixed(rA, rp, t1 + k * h, h)
        el += time.perf_counter() - w0
        gA, gp, _ = gpu64.cmf2_attempt(gA, gp, t1 + k * h, h)
    tend = t1 + steps * h
    gpu64.set_state(gA, gp, as_start=False)
    go = gpu64.observables(tend)
    ro = o.observables(rA, rp, *initial_wavefunction(model), tend)
    parity = {"max_abs_dA": float(np.abs(gA - rA).max()), "max_abs_dpsi": float(np.abs(gp - rp).max()),
              "d_auto": abs(go["auto"] - ro["auto"]), "d_pop": float(np.abs(go["pop"] - ro["pop"]).max()),
              "d_energy": abs(go["energy"] - ro["energy"]), "d_norm": abs(go["norm"] - ro["norm"]),
              "steps": steps, "step_fs": h * AU2FS, "from_fs": t1 * AU2FS,
              "what": "FP64 device path vs the CPU oracle on the same CMF2 steps: observables and A within "
                      "1e-10, SPF values within 1e-9"}
    out = dict(value=steps * h * AU2FS / el, unit="fs/s", cores=os.cpu_count(), kind="port",
               sample=f"{steps} CMF2 steps of {h * AU2FS:.4f} fs from the {t1 * AU2FS:.2f} fs state of the qvc12 "
                      f"model, NumPy oracle, BLAS threads = host cores, {el:.1f} s")
    try:
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "state.npz")
            np.savez(path, A=A1, psi=psi1, t=t1, h=h)
            env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1", MKL_NUM_THREADS="1")
            r = subprocess.run([sys.executable, "-c", _ONE_THREAD, ROOT, path], env=env, capture_output=True,
                               text=True, timeout=600)
            sec = float(r.stdout.strip().splitlines()[-1])
        out["single_thread"] = {"value": h * AU2FS / sec, "unit": "fs/s", "cores": 1, "kind": "port",
                                "sample": f"1 CMF2 step of {h * AU2FS:.4f} fs, NumPy oracle, one BLAS thread, "
                                          f"{sec:.1f} s"}
    except Exception as exc:   # the single-thread row is informative only
        out["single_thread"] = {"unavailable": f"{type(exc).__name__}: {exc}"[:200]}
    return out, parity


def run_reference(args):
    """The CPU oracle on the GPU arm's workload and schedule: it brings the qvc12
    model from t = 0 to 1 fs untimed with five fixed CMF2 steps of 0.2 fs (the
    start state of the timed part; an adaptive run from tout * eps_int would take
    ~40 steps of ~6 s), then `warmup` untimed and up to `steps` timed accepted
    CMF2 steps under the reference's step control from the GPU arm's step length
    at 1 fs (0.034 fs), with all host cores (NumPy's BLAS threads); the timed
    part stops early after REF_BUDGET_S and the line says how many steps it
    took."""
    ws, rank, tdist = dist_setup()
    if rank != 0:
        return 0
    from oracle.mctdh import Oracle
    model = make_model()
    A, psi = initial_wavefunction(model)
    o = Oracle(model)
    t = 0.0
    w0 = time.perf_counter()
    for _ in range(5):
        A, psi, _ = o.cmf2_fixed(A, psi, t, 0.2 * PRE_FS / AU2FS)
        t += 0.2 * PRE_FS / AU2FS
    h = 0.034 / AU2FS
    pre_s = time.perf_counter() - w0
    for _ in range(args.warmup):
        A, psi, hdid, h, _ = o.cmf2(A, psi, t, h)
        t += hdid
    t_total, fs_total, n, hd = 0.0, 0.0, 0, []
    for i in range(args.steps):
        w0 = time.perf_counter()
        A, psi, hdid, h, _ = o.cmf2(A, psi, t, h)
        t_total += time.perf_counter() - w0
        t += hdid
        fs_total += hdid * AU2FS
        hd.append(hdid * AU2FS)
        n += 1
        if t_total > REF_BUDGET_S:
            break
    v = fs_total / t_total
    line = {"metric": METRIC, "value": v, "unit": "fs/s", "n_gpus": ws, "steps": n, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_total / n, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128", "data": "synthetic (seeded qvc12 model)", "impl": "reference",
            "config": static_config(ws), "precision": "fp64", "step_fs_mean": statistics.mean(hd),
            "cpu_baseline": {"value": v, "unit": "fs/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"{n} adaptive CMF2 steps from {PRE_FS} fs (mean {statistics.mean(hd):.4f} "
                                       f"fs), NumPy oracle on the host cores; untimed 0 -> {PRE_FS} fs (five fixed "
                                       f"steps) took {pre_s:.0f} s"},
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
        core.mfx_gate(MFX_GATE)
        warm = max(warm, 6)
    t, h = t0, h0
    for _ in range(warm):
        hdid, h, _ = core.step(INT_CMF2, t, h)
        t += hdid
    # the state the timed steps start from (the e2e leg repeats the same steps)
    start = (*core.get_state(), t, h)
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
    return core, dict(t=t, h=h, ms=ms, fs=fs, hdids=hdids, prof=prof, prof_ms=prof_ms, start=start,
                      eom=c1["eom"] - c0["eom"], hb=c1["hb"] - c0["hb"], launches=c1["launches"] - c0["launches"])


def run_size_scan(args):
    """qvc12n: the benchmark model with `--nspf` SPFs per mode and state (12: 2.99 M
    configurations per state, 143 MB of coefficients, beyond the 129 MB L2); qvc24:
    4 states, 24 DOFs in 8 three-DOF modes of 12^3 grids, 8 SPFs (16.8 M
    configurations per state, 1.07 GB).  Split path against the FP64 path from the
    same state (1 fs of FP64 CMF2 for qvc12n, `--pre-fs` for qvc24), as the
    benchmark line does (no learned extrapolator, no CPU baseline)."""
    import torch
    from macaw_gb300.capi import GpuCore
    from macaw_gb300.generate import qvc24
    _, _, tdist = dist_setup()
    torch.cuda.init()
    if args.workload == "qvc24":
        model = qvc24(eps_int=EPS_CMF, eps_lanczos=1e-8, eps_spf=1e-7)
        pre_fs = args.pre_fs
    else:
        model = qvc12(nspf=args.nspf, eps_int=EPS_CMF, eps_lanczos=1e-8, eps_spf=1e-7)
        pre_fs = PRE_FS
    A0, psi0 = initial_wavefunction(model)
    l2 = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    pre = GpuCore(model, precision=0)
    pre.set_state(A0, psi0, as_start=True)
    w0 = time.perf_counter()
    t1, h1, _, _, _ = pre.propagate_interval(INT_CMF2, pre_fs / AU2FS, 0.0, model.tout * model.eps_int)
    pre_s = time.perf_counter() - w0
    A1, psi1 = pre.get_state()
    pre.close()
    state = (A0, psi0, A1, psi1)
    # one context at a time (the FP64 arm is closed before the split arm is set up),
    # so the device holds a single plan: each arm's timed steps, then its
    # continuation over the accuracy interval
    acc_fs = ACC_FS if args.workload != "qvc24" else 0.1
    cmp, dev_bytes = {}, {}
    with ClockSampler(torch.cuda.current_device()) as clk:
        arms = {}
        for name, prec in (("fp64", 0), ("mixed", args.precision)):
            core, arms[name] = run_arm(model, prec, state, t1, h1, args, l2, torch, tdist, profile=False)
            dev_bytes[name] = core.device_bytes()
            core.set_state(A1, psi1, as_start=False)
            tt, _, _, _, _ = core.propagate_interval(INT_CMF2, t1 + acc_fs / AU2FS, t1, h1)
            cmp[name] = core.observables(tt)
            core.close()
    ref, mix = arms["fp64"], arms["mixed"]
    value = mix["fs"] / (mix["ms"] * 1e-3)
    fp64_value = ref["fs"] / (ref["ms"] * 1e-3)
    ntot = int(model.naconftot)
    wl = f"qvc12, {args.nspf} SPFs" if args.workload != "qvc24" else "qvc24, 8 modes x 8 SPFs, 4 states"
    line = {"metric": f"simulated fs/s ({wl}, CMF2)", "value": value, "unit": "fs/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": mix["ms"] / args.steps,
            "higher_is_better": True, "precision": precision_label(args.precision),
            "fp64_path": {"value": fp64_value, "ms_per_step": ref["ms"] / args.steps},
            "speedup_vs_fp64_path": value / fp64_value,
            "accuracy_vs_fp64_path": {"dC": abs(cmp["mixed"]["auto"] - cmp["fp64"]["auto"]),
                                      "dpop": float(np.abs(cmp["mixed"]["pop"] - cmp["fp64"]["pop"]).max()),
                                      "over_fs": acc_fs, "from_fs": t1 * AU2FS},
            "untimed_pre_propagation_s": pre_s,
            "eom_per_s": mix["eom"] / (mix["ms"] * 1e-3), "hb_per_s": mix["hb"] / (mix["ms"] * 1e-3),
            "fp64_eom_per_s": ref["eom"] / (ref["ms"] * 1e-3),
            "clocks": clk.summary(),
            "device_bytes": {"fp64": dev_bytes["fp64"], "split": dev_bytes["mixed"]},
            "config": {"workload": args.workload, "nspf": args.nspf if args.workload != "qvc24" else 8,
                       "coefficients": ntot,
                       "coefficient_bytes": 16 * ntot, "dimpsi": int(model.dimpsi),
                       "l2": "flushed (256 MB write) before every timed step"}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import torch
    from macaw_gb300.capi import GpuCore, fp64_peak_tflops, tensor_core_status
    ws, rank, tdist = dist_setup()
    torch.cuda.init()
    model = make_model()
    A0, psi0 = initial_wavefunction(model)
    l2 = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2
    # leave the start-up transient of the step control (the reference starts at
    # tout * eps_int, propagator.f90:103, and grows by at most 1.5x per CMF2 step):
    # propagate 1 fs untimed with the FP64 path; every arm starts from that state
    pre = GpuCore(model, precision=0)
    pre.set_state(A0, psi0, as_start=True)
    pre.mfx_record(2)   # the untimed FP64 steps are the extrapolator's training data
    t1, h1, _, _, _ = pre.propagate_interval(INT_CMF2, PRE_FS / AU2FS, 0.0, model.tout * model.eps_int)
    A1, psi1 = pre.get_state()
    from macaw_gb300 import mfx
    tr0 = time.perf_counter()
    # training data: the start state's own 0 -> 1 fs and that of seeded variants of
    # it (displaced initial Gaussians); the last variant is held back for the gating
    records = [pre.mfx_fetch()]
    for Av, pv in mfx.variant_states(model, 1 + args.mfx_variants, seed=11)[1:]:
        pre.set_state(Av, pv, as_start=True)
        pre.mfx_record(2)
        pre.propagate_interval(INT_CMF2, PRE_FS / AU2FS, 0.0, model.tout * model.eps_int)
        records.append(pre.mfx_fetch())
    X, R, ks = mfx.build_datasets(records)
    net, fscale, tscale, tr_loss = mfx.train(X, R, steps=ks, epochs=MFX_EPOCHS,
                                             val_frac=1.0 / len(records) if len(records) > 1 else 0.2)
    train_s = time.perf_counter() - tr0
    pre.close()
    mfx_net = (net, fscale, tscale)
    state = (A0, psi0, A1, psi1)
    head_is_mfx = args.headline == "mfx"
    with ClockSampler(torch.cuda.current_device()) as clk:
        ref_core, ref = run_arm(model, 0, state, t1, h1, args, l2, torch, tdist, profile=False)
        mix_core, mix = run_arm(model, args.precision, state, t1, h1, args, l2, torch, tdist,
                                profile=not head_is_mfx)
        mfx_core, mfxr = run_arm(model, args.precision, state, t1, h1, args, l2, torch, tdist,
                                 profile=head_is_mfx, mfx_net=mfx_net)
    mfx_stats = mfx_core.mfx_stats()
    ref["ms"], mix["ms"], mfxr["ms"] = max_over_ranks([ref["ms"], mix["ms"], mfxr["ms"]], tdist)
    fp64_value = ws * ref["fs"] / (ref["ms"] * 1e-3)
    split_value = ws * mix["fs"] / (mix["ms"] * 1e-3)
    mfx_value = ws * mfxr["fs"] / (mfxr["ms"] * 1e-3)
    head, head_core = (mfxr, mfx_core) if head_is_mfx else (mix, mix_core)
    value = mfx_value if head_is_mfx else split_value

    # e2e: the reference-facing host-buffer call (mctdh_cmf2) of the headline arm
    # with pinned buffers, host<->device copies of A and psi inside every step,
    # over the same steps as the device-timed ones (from the same state, the same
    # step sequence)
    Ah, ph, te, he = head["start"]
    pA = torch.from_numpy(Ah.copy()).pin_memory()
    pP = torch.from_numpy(ph.copy()).pin_memory()
    import ctypes as C
    DPp = C.POINTER(C.c_double)
    hd, hn = C.c_double(), C.c_double()
    e2e_fs, e2e_s = 0.0, 0.0
    for _ in range(max(1, args.steps)):
        flush_l2(l2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = head_core.lib.mctdh_cmf2(head_core.h, C.cast(pA.data_ptr(), DPp), C.cast(pP.data_ptr(), DPp), te, he,
                                      C.byref(hd), C.byref(hn))
        e2e_s += time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError(head_core.lib.mctdh_last_error(head_core.h).decode())
        te += hd.value
        he = hn.value
        e2e_fs += hd.value * AU2FS
    nbytes = 16 * (model.naconftot + model.dimpsi)

    tc = tensor_core_status()
    # accuracy of the split arms against the FP64 path over the whole propagation
    # (outside the timed region; rank 0 of a single-GPU run)
    acc_split, acc_mfx = None, None
    if rank == 0 and ws == 1 and args.acc_fs > 0:
        acc = accuracy_arms(model, [args.precision], args.acc_fs, mfx_net=mfx_net, mfx_precision=args.precision)

        def summary(a):
            return {"max_dC": a["max_dC"], "max_dpop": a["max_dpop"], "end_dC": a["end_dC"],
                    "end_dpop": a["end_dpop"], "max_denergy": a["max_denergy"], "over_fs": args.acc_fs,
                    "from_fs": 0.0, "compared_every_fs": model.tout * AU2FS, "bars": {"dC": 1e-6, "dpop": 1e-5},
                    "within_bars": bool(a["max_dC"] <= 1e-6 and a["max_dpop"] <= 1e-5),
                    "free_running_fs_per_s": a["fs_per_s"],
                    "free_running_fp64_fs_per_s": acc["fp64"]["fs_per_s"],
                    "eom_per_fs": a["eom"] / args.acc_fs, "fp64_eom_per_fs": acc["fp64"]["eom"] / args.acc_fs}
        acc_split = summary(acc["arms"][str(args.precision)])
        acc_mfx = summary(acc["arms"]["mfx"])
        acc_mfx["extrapolator"] = acc["arms"]["mfx"].get("extrapolator")

    prof = head["prof"]
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
    prec_label = precision_label(args.precision)
    line = {
        "metric": METRIC, "value": value, "unit": "fs/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128 state; " + prec_label,
        "data": "synthetic (seeded qvc12 model)",
        "config": static_config(ws),
        "arm": ("split precision with the learned mean-field extrapolator" if head_is_mfx else
                "split precision"),
        "precision": prec_label,
        "tensor_cores": {"enabled": bool(tc["enabled"]), "mma_wait_timeouts": tc["timeouts"],
                         "served": "not by default in single contexts: the FP32 CUDA-core mode product is "
                                   "faster on this model (mctdh_tensor_core_config switches it on)"},
        "step_fs_mean": statistics.mean(head["hdids"]),
        "fp64_path": {"value": fp64_value, "unit": "fs/s", "ms_per_step": ref["ms"] / args.steps,
                      "step_fs_mean": statistics.mean(ref["hdids"]),
                      "eom_per_s": ref["eom"] / (ref["ms"] * 1e-3)},
        "speedup_vs_fp64_path": value / fp64_value,
        "accuracy_vs_fp64_path": acc_mfx if head_is_mfx else acc_split,
        "split_path": {"value": split_value, "unit": "fs/s", "ms_per_step": mix["ms"] / args.steps,
                       "step_fs_mean": statistics.mean(mix["hdids"]),
                       "speedup_vs_fp64_path": split_value / fp64_value,
                       "eom_per_s": mix["eom"] / (mix["ms"] * 1e-3),
                       "accuracy_vs_fp64_path": acc_split},
        "mfx_path": {"value": mfx_value, "unit": "fs/s", "ms_per_step": mfxr["ms"] / args.steps,
                     "step_fs_mean": statistics.mean(mfxr["hdids"]),
                     "speedup_vs_fp64_path": mfx_value / fp64_value,
                     "eom_per_s": mfxr["eom"] / (mfxr["ms"] * 1e-3),
                     "extrapolated_steps": mfx_stats["mlp_steps"], "fallbacks": mfx_stats["fallbacks"],
                     "rejected": mfx_stats["rejected"], "last_mismatch": mfx_stats["last_rel"],
                     "training": {"rows": int(len(X)), "epochs": MFX_EPOCHS, "loss": tr_loss,
                                  "seconds": train_s,
                                  "data": f"untimed FP64 CMF2 steps from 0 to {PRE_FS} fs of the start state "
                                          f"and of {args.mfx_variants} seeded variants (initial Gaussians "
                                          f"displaced by up to 0.3 in position and momentum)"},
                     "accuracy_vs_fp64_path": acc_mfx},
        "eom_per_s": head["eom"] / (head["ms"] * 1e-3), "hb_per_s": head["hb"] / (head["ms"] * 1e-3),
        "e2e": {"value": e2e_fs / e2e_s, "unit": "fs/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes},
        "gpu_launches": head["launches"],
        "roofline": {"bound": ROOF_BOUND.get(dname, "hbm"), "kernel": dname, "achieved": achieved_gbs,
                     "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved_gbs / peaks["hbm_gbs"],
                     "traffic": (by_launch * TRAFFIC_PER_ALG_BYTE[dname]) if dname in TRAFFIC_PER_ALG_BYTE else None,
                     "traffic_source": "scaled: DRAM bytes per algorithmic byte of this kernel class from one ncu "
                                       "capture of the profile case (bench.py --profile-case --precision 5 --profile-from-fs 1), "
                                       "times this run's algorithmic bytes per launch",
                     "what_bounds_it": ROOF_NOTE.get(dname, ""),
                     "peak_source": peak_src},
        "compute": ({"kernel": dname, "achieved": achieved_tf, "unit": "TFLOP/s (complex MAC = 8 flop)",
                     "fp64_peak": fp64_peak, "frac_of_fp64_peak": achieved_tf / fp64_peak if fp64_peak > 0 else None,
                     "peak_source": "measured FP64 FMA chain on this GPU"} if args.precision == 0 else
                    {"kernel": dname, "achieved": achieved_tf, "unit": "TFLOP/s (complex MAC = 8 flop)"}),
        "kernel_profile": {k: {"ms": round(v["ms"], 3), "launches": v["launches"],
                               "share": round(v["ms"] / tot_ms, 4)}
                           for k, v in prof.items() if v["launches"]},
        "gpu_busy_frac_profiled_pass": tot_ms / head["prof_ms"] if head["prof_ms"] else None,
        "clocks": clocks,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"], line["parity_vs_oracle"] = cpu_baseline(
            model, A1, psi1, t1, statistics.mean(head["hdids"]) / AU2FS, ref_core)
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
    torch.cuda.init()
    out = accuracy_arms(make_model(), [int(p) for p in args.acc_precisions.split(",") if p.strip()], args.acc_fs)
    print(json.dumps(out), flush=True)
    return 0


def accuracy_arms(model, precisions, acc_fs, mfx_net=None, mfx_precision=1):
    """The FP64 path and each split arm propagated from t = 0 to acc_fs (free
    running, CMF2 step control of each arm), compared at every output time.  With
    `mfx_net` (network, fscale, tscale) one more arm, "mfx": precision
    `mfx_precision` with the learned extrapolator attached."""
    import torch
    from macaw_gb300.capi import GpuCore
    A0, psi0 = initial_wavefunction(model)
    t_end = acc_fs / AU2FS
    arms = [0] + list(precisions) + (["mfx"] if mfx_net is not None else [])
    series, info = {}, {}
    for prec in arms:
        core = GpuCore(model, precision=mfx_precision if prec == "mfx" else prec)
        if prec == "mfx":
            core.mfx_attach(*mfx_net, tol=model.eps_int)
            core.mfx_gate(MFX_GATE)
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
        info[prec] = {"wall_s": wall, "fs_per_s": acc_fs / wall, "steps": nsteps,
                      "eom": core.counters()["eom"], "device_bytes": core.device_bytes()}
        if prec == "mfx":
            info[prec]["extrapolator"] = core.mfx_stats()
        core.close()
    ref = series[0]
    out = {"workload": "accuracy: qvc12 CMF2 (tolerance 1e-5) from t = 0, outputs every "
                       f"{model.tout * AU2FS:g} fs", "over_fs": acc_fs, "fp64": info[0], "arms": {}}
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
    return out


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
    together with lockstep RK45 (each attempt round one CUDA graph, launch shapes
    chosen by the ensemble autotuner), against the same members propagated one
    context at a time.  Unit: member-fs/s (simulated fs summed over members per
    second).  e2e: the same interval through the public calls with host buffers
    (every member's state uploaded before and downloaded after)."""
    import torch
    from macaw_gb300.capi import Ensemble, GpuCore
    from macaw_gb300.generate import ensemble
    torch.cuda.init()
    models = ensemble(count=args.members, max_conf=args.max_conf)
    starts = [initial_wavefunction(m) for m in models]
    w0 = time.perf_counter()
    ens = Ensemble(models, precision=args.precision)
    create_s = time.perf_counter() - w0
    for i, (A, psi) in enumerate(starts):
        ens.set_state(i, A, psi, as_start=True)
    t = np.zeros(len(models))
    step = np.array([m.tout * m.eps_int for m in models])
    # untimed start-up transient (steps grow from tout * eps_int); the first call
    # runs the autotuner and captures the attempt-round graphs
    ens.propagate(INT_RK45, 0.1 / AU2FS, t, step)
    tuning = ens.tuning()
    cost = ens.eom_cost()
    hbm_peak = load_peaks()[0]["hbm_gbs"]
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
    # e2e: host states in, the next interval, host states out
    states = [ens.get_state(i) for i in range(len(models))]
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for i, (A, psi) in enumerate(states):
        ens.set_state(i, A, psi, as_start=False)
    t2 = t.copy()
    ens.propagate(INT_RK45, (0.1 + 2 * args.ens_fs) / AU2FS, t2, step)
    back = [ens.get_state(i) for i in range(len(models))]
    e2e_s = time.perf_counter() - w0
    e2e_fs = float(np.sum(t2 - t)) * AU2FS
    nbytes = int(sum(16 * (m.naconftot + m.dimpsi) for m in models))
    # a sample of the members (every len/nseq-th, so small and large ones alike)
    # one context at a time (sequential), same interval
    seq_ms = 0.0
    nseq = min(len(models), args.seq_members)
    seq_fs = 0.0
    for i in np.linspace(0, len(models) - 1, nseq).round().astype(int):
        core = GpuCore(models[i], precision=args.precision)
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
            "precision": precision_label(args.precision),
            "eom_member_evals_per_s": (c1["eom"] - c0["eom"]) * len(models) / (ms * 1e-3),
            "launches": c1["launches"] - c0["launches"],
            "graphs": "one CUDA graph per attempt round and per step-start derivative",
            "autotune": tuning, "create_s": create_s,
            "roofline": {"bound": "hbm", "achieved": cost["bytes"] / (tuning["eom_ms"] * 1e-3) / 1e9,
                         "peak": hbm_peak, "unit": "GB/s",
                         "frac": cost["bytes"] / (tuning["eom_ms"] * 1e-3) / 1e9 / hbm_peak,
                         "traffic": None,
                         "kernel": "one merged EOM evaluation of all members (CUDA events, autotuner's "
                                   "timing); algorithmic bytes of its mode products and contractions",
                         "alg_bytes_per_eom": cost["bytes"], "alg_flops_per_eom": cost["flops"]}
            if tuning["eom_ms"] > 0 else None,
            "e2e": {"value": e2e_fs / e2e_s, "unit": "member-fs/s", "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": nbytes,
                    "what": "every member's state uploaded, the next interval, every state downloaded"},
            "sequential": {"members": nseq, "member_fs_per_s": seq_fs / (seq_ms * 1e-3) if seq_ms else None,
                           "sample": "evenly spaced member indices",
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
    ap.add_argument("--acc-precisions", default="1,5", help="accuracy: split arms compared with FP64")
    ap.add_argument("--headline", default="split", choices=["mfx", "split"],
                    help="qvc12: the arm the line's value is: split precision without (split, the default: the "
                         "arm that holds the 200 fs accuracy bars) or with the extrapolator (mfx)")
    ap.add_argument("--mfx-variants", type=int, default=3,
                    help="extrapolator: seeded initial-state variants recorded besides the start state")
    ap.add_argument("--pre-fs", type=float, default=0.3, help="qvc24: untimed FP64 propagation before the steps")
    ap.add_argument("--precision", type=int, default=5, choices=[0, 1, 2, 3, 4, 5, 6],
                    help="arm timed against the FP64 path (mode of mctdh_setup_t.precision; 5: compensated "
                         "mean-field products and contractions, FP32 Lanczos H_B products)")
    ap.add_argument("--workload", default="qvc12",
                    choices=["qvc12", "qvc12n", "qvc24", "ensemble", "lvc5", "gmctdh16", "lvc5mix", "accuracy"],
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
    if args.workload in ("qvc12n", "qvc24"):
        return run_size_scan(args)
    if args.workload in ("lvc5", "gmctdh16", "lvc5mix"):
        return run_rk_workload(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
