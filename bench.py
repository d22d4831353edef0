#!/usr/bin/env python
"""Benchmark of the shallow-water RK4 hot path on GB300.

Default workload: 6 panels x 385^2 nodes (N=384), SBP 4/2 operators, RK4
with dt = 120 s, seeded balanced zonal flow plus a degree<=64
spherical-harmonic height perturbation (synthetic; the reference's own test
cases are analytic and produce no checked-in data).  One "step" is one RK4
step of the whole state.  The headline value is the FP32 fused form
(compensated stage sums, FP64 metric precompute); the FP64 plain path is
measured beside it, and the FP32 state is compared with the FP64 state after
10 simulated days.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]
                  [--workload n384_d42|n1024_d63]

n1024_d63 is the large single instance: 6 x 1025^2 nodes, SBP 6/3, dt = 45 s,
balanced flow plus a barotropically unstable jet.  The default run also
measures it beside the headline (key "large_instance").

Every GPU result is stated with its error against the FP64 oracle (the C++
restatement of the reference) on the same initial state, and the oracle is
timed on the host cores as the CPU baseline (--impl reference; the default
run's cpu_baseline leg runs that same measurement in a fresh process).

Multi-GPU runs (torchrun) are independent replicas, one per GPU: the path
does not shard across GPUs here (all six panels live on one GPU).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("RK4 steps/s at 6×384² (FP32 form vs FP64 plain), "
          "adjoint/forward time ratio")
L2_FLUSH_BYTES = 256 << 20          # > 129 MB L2
# Algorithmic HBM words per node per RK4 step (4 stage launches; 3 state
# words, 5 metric words J, Qi1, Qi2, Qi3, f):
#   FP64 plain 68 = 14 + 20 + 20 + 14;
#   FP32 compensated 77 = 14 + 20 + 20 + 23 (stage 4 also reads the low part
#   of the state pair).  The derived 1/(J hx a) field the kernels read is not
#   counted.
BYTES_PER_NODE_STEP = {"fp32": 77 * 4, "fp64": 68 * 8}
KERNELS_PER_STEP = 8                # 4 x (stage kernel + cube-edge kernel)

# acc_dt: time step of the FP32-vs-FP64 accuracy run.  The workloads' own
# time steps (Courant number c*dt/(a*hx) = 1.11 with c = sqrt(g*5960 m)) lie
# beyond the RK4 stability limit of the undiffused SBP scheme: the FP64 state
# turns non-finite within 6 simulated hours.  Courant 0.84 (N=384, 90 s) and
# 0.74 (N=1024 d63, 30 s) stay stable over the full simulated period.  The
# per-step work, and so steps/s, does not depend on dt.
# oracle_hours: simulated hours of the run against the FP64 oracle (its CPU
# cost bounds it); acc_days_extra: the FP32-vs-FP64 GPU run when the workload
# is measured beside the headline.
WORKLOADS = {
    "n384_d42": dict(N=384, order=42, dt=120.0, cfg=2, days=10.0, acc_dt=90.0, oracle_hours=24.0,
                     acc_days_extra=10.0,
                     desc="6 panels x 385^2 nodes (N=384), SBP 4/2 (d42), RK4 dt=120 s"),
    "n1024_d63": dict(N=1024, order=63, dt=45.0, cfg=5, days=5.0, acc_dt=30.0, oracle_hours=0.5,
                      acc_days_extra=1.0,
                      desc="6 panels x 1025^2 nodes (N=1024), SBP 6/3 (d63), RK4 dt=45 s"),
}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _profile_traffic(workload):
    """Per-launch DRAM traffic of the stage kernel from the committed ncu
    summary (profiles/), or None."""
    path = os.path.join(ROOT, "profiles", f"stage_kernel_fp32_{workload}.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid: str | None):
        self.uuid = uuid
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                      text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                self.out, _ = self.p.communicate()

    def summary(self):
        if not getattr(self, "out", ""):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            if self.uuid and self.uuid not in f[0]:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _state(w):
    from cubedsphere_sbp_swm_gb300 import initial
    return initial.config_state(w["cfg"])


def _data_desc(w, info):
    if w["cfg"] == 5:
        return ("synthetic: seeded balanced zonal flow + Gaussian jet (peak 80 m/s) + 120 m "
                "height bump")
    return ("synthetic: seeded balanced zonal flow u0=%.2f m/s + Y_lm (l<=64) height "
            "perturbation, 10 m RMS" % info["u0"])


def accuracy_vs_oracle(w, h, u, v, local, hours):
    """The FP32 fused form and the FP64 plain path against the FP64 oracle
    (the C++ restatement of the reference) after `hours` simulated hours from
    the same initial state at the stable time step acc_dt: J-weighted
    relative L2 (vec_math_mod.f90:50-90 weighting) and relative Linf of h, u,
    v, and the SBP-quadrature mass of each run against the oracle's."""
    import numpy as np

    import cubedsphere_sbp_swm_gb300 as swm
    from cubedsphere_sbp_swm_gb300 import initial
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the checker

    dt = w["acc_dt"]
    nsteps = int(round(hours * 3600.0 / dt))
    J = initial.ecs_geometry(w["N"])["J"]
    oracle.set_threads(os.cpu_count() or 1)
    od = oracle.OracleDomain(w["N"], w["order"])
    t0 = time.perf_counter()
    ref = [a.copy() for a in (h, u, v)]
    od.rk4_inplace(*ref, dt, nsteps)
    oracle_s = time.perf_counter() - t0
    m_ref, m0 = od.mass(ref[0]), od.mass(h)
    out = {"reference": "FP64 oracle (C++ restatement of the reference), same initial state",
           "hours": hours, "dt_s": dt, "steps": nsteps, "oracle_run_s": round(oracle_s, 2),
           "oracle_mass_drift": (m_ref - m0) / m0}
    for prec in ("fp32", "fp64"):
        op = swm.OperatorSWM(swm.ModelConfig(N=w["N"], sbp_order=w["order"], precision=prec, device=local))
        s = op.create_stvec()
        s.upload(h, u, v)
        swm.RK4().step(s, op, dt, nsteps)
        got = s.download()
        del s, op
        r = {}
        for name, a, b in zip("huv", got, ref):
            r[f"{name}_rel_l2"] = float(np.sqrt(np.sum(J * (a - b) ** 2) / np.sum(J * b * b)))
            r[f"{name}_rel_linf"] = float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
        r["mass_rel_diff_vs_oracle"] = (od.mass(got[0]) - m_ref) / m_ref
        out[prec] = r
    return out


def accuracy_vs_fp64(w, h, u, v, local, days):
    """FP32 fused form against the FP64 plain path (which matches the FP64
    oracle to 1e-12 per step; accuracy_vs_oracle checks it over a shorter run)
    after `days` simulated days from the same initial state at the stable time
    step acc_dt: J-weighted relative L2 and relative Linf of h, u, v and the
    SBP-quadrature mass drift of both runs."""
    import numpy as np

    import cubedsphere_sbp_swm_gb300 as swm
    from cubedsphere_sbp_swm_gb300 import initial

    dt = w["acc_dt"]
    nsteps = int(round(days * 86400.0 / dt))
    J = initial.ecs_geometry(w["N"])["J"]
    res, drift = {}, {}
    for prec in ("fp64", "fp32"):
        op = swm.OperatorSWM(swm.ModelConfig(N=w["N"], sbp_order=w["order"], precision=prec, device=local))
        s = op.create_stvec()
        s.upload(h, u, v)
        m0 = op.get_diagnostics(s)["mass"]
        swm.RK4().step(s, op, dt, nsteps)
        res[prec] = s.download()
        drift[prec] = (op.get_diagnostics(s)["mass"] - m0) / m0
        del s, op
    out = {"days": days, "dt_s": dt, "steps": nsteps,
           "reference": "FP64 plain GPU path (matches the FP64 oracle to 1e-12 relative L2 per step)",
           "note": "the workload dt (Courant 1.11) is beyond the RK4 stability limit of the "
                   "undiffused scheme (FP64 state non-finite within 6 simulated hours); this run "
                   "uses the stable dt_s"}
    for name, a, b in zip("huv", res["fp32"], res["fp64"]):
        out[f"{name}_rel_l2"] = float(np.sqrt(np.sum(J * (a - b) ** 2) / np.sum(J * b * b)))
        out[f"{name}_rel_linf"] = float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    out["mass_drift_fp32"] = drift["fp32"]
    out["mass_drift_fp64"] = drift["fp64"]
    return out


# Ensemble: 32 members each at N = 48, 96, 192 (FP32 fused form), own seeds
# 1000+m; time step 600*48/N s (Courant 0.70 at every resolution).
ENSEMBLE_GROUPS = ((48, 32), (96, 32), (192, 32))


def ensemble_leg(local, steps, warmup, peak):
    """member-steps/s of the batched ensemble (autotuned tile shape, one
    graph per ensemble step) against looping the single-instance path over
    the same members; inputs (0.8 GB of state, work and metric) exceed L2."""
    import numpy as np
    import torch

    import cubedsphere_sbp_swm_gb300 as swm
    from cubedsphere_sbp_swm_gb300 import initial

    Ns = [N for N, k in ENSEMBLE_GROUPS for _ in range(k)]
    dts = [600.0 * 48 / N for N in Ns]
    ens = swm.Ensemble(swm.ModelConfig(N=Ns[0], precision="fp32", device=local), Ns, dts)
    for m, N in enumerate(Ns):
        ens.upload(m, *initial.balanced_zonal(N, 1000 + m, 16)[:3])
    tuned = ens.tune(steps=5)
    dev = torch.device("cuda", local)
    stream = torch.cuda.ExternalStream(ens.stream, device=dev)
    ens.step(warmup)
    ens.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    ens.step(steps)
    b.record(stream)
    ens.synchronize()
    ms = a.elapsed_time(b) / steps
    finite = bool(all(np.isfinite(x).all() for m in (0, len(Ns) // 2, len(Ns) - 1)
                      for x in ens.download(m)))
    # the same members, one single-instance RK4 step each (own graph and stream)
    L = ens._L
    handles = [ens.member(m) for m in range(len(Ns))]
    for (c, s), dt in zip(handles, dts):
        swm._abi.check(L.swm_rk4_step(c, s, dt, 1), c)
    for c, _ in handles:
        swm._abi.check(L.swm_ctx_synchronize(c), c)
    t0 = time.perf_counter()
    for _ in range(steps):
        for (c, s), dt in zip(handles, dts):
            L.swm_rk4_step(c, s, dt, 1)
    for c, _ in handles:
        swm._abi.check(L.swm_ctx_synchronize(c), c)
    loop_s = (time.perf_counter() - t0) / steps
    npts = sum(6 * (N + 1) ** 2 for N in Ns)
    achieved = BYTES_PER_NODE_STEP["fp32"] * npts / (ms / 1e3) / 1e9
    ens.close()
    return {
        "members": len(Ns), "resolutions": {str(N): k for N, k in ENSEMBLE_GROUPS},
        "dt_s": "600*48/N", "nodes_per_field": npts, "precision": "fp32 fused",
        "member_steps_per_s": round(len(Ns) / (ms / 1e3), 1),
        "ms_per_ensemble_step": round(ms, 4),
        "loop_single_instance_member_steps_per_s": round(len(Ns) / loop_s, 1),
        "speedup_vs_loop": round(loop_s * 1e3 / ms, 3),
        "tile_shape": tuned, "launches_per_step": KERNELS_PER_STEP,
        "roofline": {"achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "of": "whole ensemble step, algorithmic bytes"},
        "state_finite": finite,
    }


# Adjoint workload: N=192, 240 RK4 steps, 16 snapshots, FP64.  The workload's
# dt = 300 s (Courant 1.39) is past the RK4 stability limit of the undiffused
# scheme; 150 s (Courant 0.70) is used.
ADJOINT = dict(N=192, steps=240, dt=150.0, nsnap=16, seed_x0=3, seed_obs=4, ndir=20, eps=1e-6)


def adjoint_leg(local):
    """Cost of the discrete adjoint against the forward model and its
    checks: J = 1/2 sum w (h_T - h_obs)^2 with SBP quadrature weights w."""
    import numpy as np
    import torch

    import cubedsphere_sbp_swm_gb300 as swm
    from cubedsphere_sbp_swm_gb300 import adjoint as ad
    from cubedsphere_sbp_swm_gb300 import initial

    c = ADJOINT
    N, T, dt = c["N"], c["steps"], c["dt"]
    op = swm.OperatorSWM(swm.ModelConfig(N=N, precision="fp64", device=local))
    dev = torch.device("cuda", local)
    stream = torch.cuda.ExternalStream(op.stream, device=dev)
    rk4 = swm.RK4()

    def st(arrs):
        s = op.create_stvec()
        s.upload(*arrs)
        return s

    def timed(fn):
        op.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        op.synchronize()
        b.synchronize()
        return a.elapsed_time(b)

    x0 = initial.balanced_zonal(N, c["seed_x0"], 16)[:3]
    s = st(initial.balanced_zonal(N, c["seed_obs"], 16)[:3])
    rk4.step(s, op, dt, T)
    hobs = s.download()[0]
    w = ad.quadrature_weights(op)
    zeros = np.zeros(op.shape)

    # forward run and a single adjoint step
    s = st(x0)
    rk4.step(s, op, dt, 3)
    s.upload(*x0)
    fwd_ms = timed(lambda: rk4.step(s, op, dt, T))
    x = st(x0)
    lam = st((w, zeros, zeros))
    ad.rk4_ad(op, x, lam, dt)
    reps = 20
    adj_step_ms = timed(lambda: [ad.rk4_ad(op, x, lam, dt) for _ in range(reps)]) / reps

    # checkpointed gradient (forward with snapshots + reverse sweep)
    run = ad.CheckpointedRK4(op, dt, T, c["nsnap"])
    sx0, xT = st(x0), op.create_stvec()

    def gradient():
        f_ms = timed(lambda: run.forward(sx0, xT))
        hT = xT.download()[0]
        g = st((w * (hT - hobs), zeros, zeros))
        b_ms = timed(lambda: run.backward(g))
        return f_ms + b_ms, g, hT

    gradient()                                   # warm-up: graph captures
    grad_ms, g, hT = gradient()
    counts = run.counts()
    grad = g.download()
    J0 = 0.5 * float(np.sum(w * (hT - hobs) ** 2))

    # dot-product test over the whole trajectory
    rng = np.random.default_rng(2024)
    dx0 = tuple(rng.standard_normal(op.shape) for _ in range(3))
    lamT = tuple(rng.standard_normal(op.shape) for _ in range(3))
    xb, d = st(x0), st(dx0)
    for _ in range(T):
        ad.rk4_tl(op, xb, d, dt)
        rk4.step(xb, op, dt, 1)
    lt = st(lamT)
    run.forward(sx0, xT)
    run.backward(lt)
    dot_a = float(sum(np.sum(p * q) for p, q in zip(d.download(), lamT)))
    dot_b = float(sum(np.sum(p * q) for p, q in zip(dx0, lt.download())))
    dot_gap = abs(dot_a - dot_b) / max(abs(dot_a), abs(dot_b))

    # central finite differences of J along seeded directions
    def cost(arrs):
        s.upload(*arrs)
        rk4.step(s, op, dt, T)
        return 0.5 * float(np.sum(w * (s.download()[0] - hobs) ** 2))

    eps, gaps = c["eps"], []
    for k in range(c["ndir"]):
        r = np.random.default_rng(5 + k)
        dd = tuple(r.standard_normal(op.shape) for _ in range(3))
        jp = cost([a + eps * b for a, b in zip(x0, dd)])
        jm = cost([a - eps * b for a, b in zip(x0, dd)])
        an = float(sum(np.sum(p * q) for p, q in zip(grad, dd)))
        gaps.append(abs((jp - jm) / (2 * eps) - an) / abs(an))

    # the same gradient in the FP32 form: cost against the FP32 forward step,
    # and its gradient against the FP64 one
    op32 = swm.OperatorSWM(swm.ModelConfig(N=N, precision="fp32", device=local))
    st32 = torch.cuda.ExternalStream(op32.stream, device=dev)

    def timed32(fn):
        op32.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st32)
        fn()
        b.record(st32)
        op32.synchronize()
        b.synchronize()
        return a.elapsed_time(b)

    def st_32(arrs):
        v = op32.create_stvec()
        v.upload(*arrs)
        return v

    s32 = st_32(x0)
    rk4.step(s32, op32, dt, 3)
    s32.upload(*x0)
    fwd32_ms = timed32(lambda: rk4.step(s32, op32, dt, T))
    x32, lam32 = st_32(x0), st_32((w, zeros, zeros))
    ad.rk4_ad(op32, x32, lam32, dt)
    adj32_ms = timed32(lambda: [ad.rk4_ad(op32, x32, lam32, dt) for _ in range(reps)]) / reps
    run32 = ad.CheckpointedRK4(op32, dt, T, c["nsnap"])
    sx32, xT32 = st_32(x0), op32.create_stvec()
    for _ in range(2):                               # warm-up, then timed
        f32_ms = timed32(lambda: run32.forward(sx32, xT32))
        hT32 = xT32.download()[0]
        g32 = st_32((w * (hT32 - hobs), zeros, zeros))
        b32_ms = timed32(lambda: run32.backward(g32))
    grad32 = g32.download()
    gerr32 = float(np.sqrt(sum(np.sum((p - q) ** 2) for p, q in zip(grad32, grad)) /
                           sum(np.sum(q * q) for q in grad)))
    return {
        "N": N, "steps": T, "dt_s": dt, "snapshots": c["nsnap"], "precision": "fp64",
        "cost": "J = 1/2 sum_nodes w (h_T - h_obs)^2, w = SBP quadrature weights",
        "J": J0,
        "forward_step_ms": round(fwd_ms / T, 5), "adjoint_step_ms": round(adj_step_ms, 5),
        "adjoint_over_forward_step": round(adj_step_ms / (fwd_ms / T), 3),
        "forward_run_ms": round(fwd_ms, 3), "gradient_ms": round(grad_ms, 3),
        "gradient_over_forward_run": round(grad_ms / fwd_ms, 3),
        "forward_steps_in_gradient": counts["forward_steps"],
        "adjoint_steps_in_gradient": counts["adjoint_steps"],
        "dot_product_rel_gap": dot_gap,
        "fd_directions": c["ndir"], "fd_eps": eps, "fd_max_rel_gap": max(gaps),
        "fp32": {"forward_step_ms": round(fwd32_ms / T, 5), "adjoint_step_ms": round(adj32_ms, 5),
                 "adjoint_over_forward_step": round(adj32_ms / (fwd32_ms / T), 3),
                 "forward_run_ms": round(fwd32_ms, 3), "gradient_ms": round(f32_ms + b32_ms, 3),
                 "gradient_over_forward_run": round((f32_ms + b32_ms) / fwd32_ms, 3),
                 "gradient_rel_l2_vs_fp64": gerr32},
        "note": "the workload's dt = 300 s (Courant 1.39) is past the RK4 stability limit; "
                "dt = 150 s (Courant 0.70)",
    }


def single_instance_leg(w, local, steps, warmup, stage_shape=None, state=None, quick=False):
    """The RK4 step of one workload, FP32 fused form and FP64 plain path:
    device-timed steps (each from the initial state, L2 flushed before it),
    CUDA-event timing of the stage kernel, and end-to-end steps through the
    C-ABI with page-locked host buffers (upload, step, download inside the
    timed region).  Returns (result dict, FP32 per-step ms list, clocks, info)."""
    import numpy as np
    import torch

    import cubedsphere_sbp_swm_gb300 as swm
    from cubedsphere_sbp_swm_gb300 import replicas

    N, ORDER, DT = w["N"], w["order"], w["dt"]
    dev = torch.device("cuda", local)
    h, u, v, info = state if state is not None else _state(w)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    tuned = {"width": 128, "seg_rows": 0, "grid": 0, "box": "auto"}

    def time_steps(prec, nsteps, nwarm, kernel_timing=False):
        """Every timed step starts from the initial state (restored outside
        the timed region): at the workload's dt the scheme is past its RK4
        stability limit, and a state left to run for the whole timed region
        would turn non-finite."""
        op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=ORDER, precision=prec, device=local))
        s0 = op.create_stvec()
        s0.upload(h, u, v)
        if prec == "fp32":   # set-up: pick the stage kernel's fastest launch shape
            if stage_shape:
                parts = stage_shape.split(",")
                wdt, seg, grd = (int(x) for x in parts[:3])
                op.set_stage_shape(wdt, seg, grd, parts[3] if len(parts) > 3 else "auto")
                tuned.update(op.stage_shape)
            else:
                tuned.update(op.tune_stage(s0, DT, 10))
        s = op.create_stvec()
        s.assign_s1v1(1.0, s0)
        ts = swm.RK4()
        stream = torch.cuda.ExternalStream(op.stream, device=dev)
        for _ in range(nwarm):
            ts.step(s, op, DT, 1)
        op.synchronize()
        if kernel_timing:
            op.timing_enable(True)
            op.timing_read()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(nsteps)]
        torch.cuda.synchronize(dev)
        for a, b in evs:
            s.assign_s1v1(1.0, s0)                    # on the op stream, before the flush
            with torch.cuda.stream(stream):
                flush.zero_()                         # evict L2 between timed steps
            a.record(stream)
            ts.step(s, op, DT, 1)
            b.record(stream)
        torch.cuda.synchronize(dev)
        ms = [a.elapsed_time(b) for a, b in evs]
        kt = op.timing_read() if kernel_timing else None
        if kernel_timing:
            op.timing_enable(False)
        return op, s, ms, kt

    def e2e(op, s, nsteps):
        """Steps/s through the C-ABI with host buffers: every step moves the
        state in from page-locked FP64 host arrays, steps it, and moves it
        back out to page-locked FP64 host arrays.  Returns (pipelined,
        serial):
          pipelined: two states take turns; swm_state_upload_async and
            swm_state_download_async move the arrays with the copy engines
            (one stream per direction), so one step's download and the next
            step's upload run under the steps; the clock stops after the
            last download has landed (swm_ctx_synchronize);
          serial: swm_state_upload, swm_rk4_step, swm_state_download, one
            step at a time, each call synchronous."""
        pin = [torch.empty((6, N + 1, N + 1), dtype=torch.float64, pin_memory=True) for _ in range(9)]
        for t_, a_ in zip(pin[:3], (h, u, v)):
            t_.numpy()[...] = a_
        hin = [t_.numpy() for t_ in pin[:3]]
        outs = [tuple(t_.numpy() for t_ in pin[3:6]), tuple(t_.numpy() for t_ in pin[6:9])]
        ts = swm.RK4()
        states = [s, op.create_stvec()]

        def pipelined(n):
            for k in range(n):
                st = states[k % 2]
                st.upload_async(*hin)
                ts.step(st, op, DT, 1)
                st.download_async(outs[k % 2])
            op.synchronize()

        def serial(n):
            for _ in range(n):
                s.upload(*hin)
                ts.step(s, op, DT, 1)
                s.download(out=outs[0])

        pipelined(4)
        t0 = time.perf_counter()
        pipelined(nsteps)
        val, _ = replicas.job_rate(nsteps, time.perf_counter() - t0, dev)
        serial(2)
        t0 = time.perf_counter()
        serial(nsteps)
        val_serial, _ = replicas.job_rate(nsteps, time.perf_counter() - t0, dev)
        return val, val_serial

    uuid = None
    try:
        uuid = str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass
    torch.cuda.synchronize(dev)
    with ClockSampler(uuid) as clk:
        op32, s32, ms32, _ = time_steps("fp32", steps, warmup)
    clocks = clk.summary()
    if quick:
        return {}, ms32, clocks, info
    finite = bool(all(np.isfinite(a).all() for a in s32.download()))
    nsteps_e2e = max(10, steps // 2)
    e2e32, e2e32_serial = e2e(op32, s32, nsteps_e2e)
    del s32, op32

    # dominant kernel timing (stage kernel), events around every launch
    _, _, _, kt = time_steps("fp32", max(8, min(steps, 40)), 2, kernel_timing=True)
    stage_ms, stage_n, edge_ms, edge_n = kt
    npts = 6 * (N + 1) ** 2
    bytes_per_launch = BYTES_PER_NODE_STEP["fp32"] * npts / 4.0
    achieved = bytes_per_launch / (stage_ms / stage_n / 1e3) / 1e9
    peak, peak_kind = _measured_peak()

    op64, s64, ms64, _ = time_steps("fp64", max(10, steps // 2), warmup)
    fp64_ms = sum(ms64) / len(ms64)
    e2e64, e2e64_serial = e2e(op64, s64, nsteps_e2e)
    del op64, s64
    _, _, _, kt64 = time_steps("fp64", 10, 2, kernel_timing=True)
    fp32_ms = sum(ms32) / len(ms32)
    res = {
        "workload": w["desc"], "N": N, "sbp": "d%d" % ORDER, "dt_s": DT, "nodes_per_field": npts,
        "fp32": {"steps_per_s": round(1e3 / fp32_ms, 3), "ms_per_step": round(fp32_ms, 5),
                 "stage_shape": {k: tuned[k] for k in ("width", "seg_rows", "grid", "box")}},
        "fp64_plain": {"steps_per_s": round(1e3 / fp64_ms, 3), "ms_per_step": round(fp64_ms, 5),
                       "stage_kernel_avg_us": round(kt64[0] / kt64[1] * 1e3, 3),
                       "e2e_steps_per_s": round(e2e64, 3),
                       "e2e_serial_steps_per_s": round(e2e64_serial, 3)},
        "fp32_over_fp64": round(fp64_ms / fp32_ms, 3),
        "e2e": {"value": round(e2e32, 3), "unit": "steps/s",
                "h2d_bytes_per_step": 3 * npts * 8, "d2h_bytes_per_step": 3 * npts * 8,
                "path": "every step: swm_state_upload_async (pinned FP64 host arrays, copy engine, "
                        "upload stream) + swm_rk4_step + swm_state_download_async (copy engine, "
                        "download stream) on two states taking turns, so transfers run under the "
                        "steps; clock stopped after the last download landed (swm_ctx_synchronize)",
                "serial_value": round(e2e32_serial, 3),
                "serial_path": "swm_state_upload (pinned arrays read in place over the host link) "
                               "+ swm_rk4_step + swm_state_download, one synchronous step at a time"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4),
                     "traffic": _profile_traffic("n%d_d%d" % (N, ORDER)),
                     "kernel": "stage_tma_kernel<float,%d,mode,%d>" % (ORDER, tuned["width"]),
                     "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": bytes_per_launch,
                     "avg_launch_us": round(stage_ms / stage_n * 1e3, 3)},
        "launches_per_step": KERNELS_PER_STEP,
        "state_finite_after_timed_steps": finite,
    }
    if edge_n:
        res["roofline"]["edge_kernel_avg_us"] = round(edge_ms / edge_n * 1e3, 3)
    return res, ms32, clocks, info


def run_gpu_arm(args):
    import torch

    from cubedsphere_sbp_swm_gb300 import replicas

    w = WORKLOADS[args.workload]
    N, ORDER, DT = w["N"], w["order"], w["dt"]
    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    state = _state(w)
    h, u, v, info = state

    # CPU baseline first, in a fresh process (the same measurement as
    # --impl reference), before this process starts its GPU work
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu and not args.quick:
        cpu = cpu_baseline_subprocess(args)

    if ws > 1:
        torch.distributed.barrier()
    head, ms32, clocks, _ = single_instance_leg(w, local, args.steps, args.warmup, args.stage_shape, state,
                                                quick=args.quick)
    value, total_s = replicas.job_rate(args.steps, sum(ms32) / 1e3, dev)
    ms_per_step = total_s * 1e3 / args.steps
    if args.quick:  # profiling case: only the timed FP32 steps
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": round(value, 3), "unit": "steps/s",
                              "ms_per_step": round(ms_per_step, 5), "quick": True,
                              "workload": args.workload}), flush=True)
        return

    acc = acc_or = None
    if rank == 0 and not args.no_accuracy:
        acc = accuracy_vs_fp64(w, h, u, v, local, w["days"] if args.days is None else args.days)
        acc_or = accuracy_vs_oracle(w, h, u, v, local, w["oracle_hours"])
    large = None
    if rank == 0 and not args.no_large and args.workload != "n1024_d63":
        wl = WORKLOADS["n1024_d63"]
        st_l = _state(wl)
        large, _, clk_l, _ = single_instance_leg(wl, local, max(10, args.steps // 2), args.warmup, None, st_l)
        large["clocks"] = clk_l
        if not args.no_accuracy:
            large["accuracy_fp32_vs_fp64"] = accuracy_vs_fp64(wl, *st_l[:3], local, wl["acc_days_extra"])
            large["accuracy_vs_oracle"] = accuracy_vs_oracle(wl, *st_l[:3], local, wl["oracle_hours"])
        if cpu and "n1024_d63" in cpu.get("rates", {}):
            large["cpu_oracle"] = cpu["rates"]["n1024_d63"]
        del st_l
    ens = None
    if rank == 0 and not args.no_ensemble:
        ens = ensemble_leg(local, max(10, args.steps // 2), args.warmup, _measured_peak()[0])
    adj = None
    if rank == 0 and not args.no_adjoint:
        adj = adjoint_leg(local)
    dif = None
    if rank == 0 and not args.no_diffusion:
        dif = diffusion_leg(w, h, u, v, local, max(10, args.steps // 2), args.warmup)
    cg = None
    if rank == 0 and not args.no_cgrid:
        cg = cgrid_leg(local, max(10, args.steps // 2), args.warmup, cpu=not args.no_cpu)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 5),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": _data_desc(w, info),
            "config": {"workload": w["desc"] + ", FP32 fused form (compensated stage sums, FP64 "
                                               "metric precompute)",
                       "N": N, "sbp": "d%d" % ORDER, "dt_s": DT, "nodes_per_field": head["nodes_per_field"],
                       "l2": "256 MB buffer written between timed steps",
                       "stage_shape": head["fp32"]["stage_shape"],
                       "parallelism": "replicas" if ws > 1 else "1 GPU"},
            "e2e": head["e2e"],
            "roofline": head["roofline"],
            "fp64_plain": {"value": head["fp64_plain"]["steps_per_s"], "unit": "steps/s",
                           "ms_per_step": head["fp64_plain"]["ms_per_step"],
                           "stage_kernel_avg_us": head["fp64_plain"]["stage_kernel_avg_us"],
                           "e2e": {"value": head["fp64_plain"]["e2e_steps_per_s"], "unit": "steps/s",
                                   "h2d_bytes_per_step": head["e2e"]["h2d_bytes_per_step"],
                                   "d2h_bytes_per_step": head["e2e"]["d2h_bytes_per_step"],
                                   "serial_value": head["fp64_plain"]["e2e_serial_steps_per_s"]}},
            "fp32_over_fp64": head["fp32_over_fp64"],
            "clocks": clocks,
            "gpu_launches": KERNELS_PER_STEP * args.steps,
            "state_finite_after_timed_steps": head["state_finite_after_timed_steps"],
        }
        if acc_or:
            line["accuracy_vs_oracle"] = acc_or
        if acc:
            line["accuracy_fp32_vs_fp64"] = acc
        if large:
            line["large_instance"] = large
        if ens:
            line["ensemble"] = ens
        if adj:
            line["adjoint"] = adj
        if dif:
            line["model_step_with_diffusion"] = dif
        if cg:
            line["c_grid"] = cg
        if cpu:
            line["cpu_baseline"] = cpu["cpu_baseline"]
            line["cpu_rates"] = cpu["rates"]
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def diffusion_leg(w, h, u, v, local, steps, warmup):
    """The drivers' full time step (ts2_mod.f90:143-146): RK4, then one
    explicit Euler step of the hyperdiffusion operator, with the TS2 scripts'
    operators and coefficients (narrow-Laplacian order of the workload's SBP
    order, uv_diff_coeff 0.03, h_diff_coeff 0.01).  Each timed step starts
    from the initial state, with an L2 flush before it."""
    import numpy as np
    import torch
    import cubedsphere_sbp_swm_gb300 as swm
    dev = torch.device("cuda", local)
    narrow = 63 if w["order"] == 63 else 42
    names = ("hordiff_vec_xyz_Ah_sbp_%d_narrow" % narrow, "hordiff_scalar_Ah_sbp_%d_narrow" % narrow)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)
    out = {"operators": list(names), "uv_diff_coeff": 0.03, "h_diff_coeff": 0.01, "dt_s": w["dt"]}
    for prec in ("fp32", "fp64"):
        op = swm.OperatorSWM(swm.ModelConfig(N=w["N"], sbp_order=w["order"], precision=prec, device=local))
        dop = swm.OperatorSWMDiff(op, names[0], 0.03, names[1], 0.01)
        s0, s = op.create_stvec(), op.create_stvec()
        s0.upload(h, u, v)
        if prec == "fp32":   # set-up: the stage kernel's fastest launch shape
            op.tune_stage(s0, w["dt"], 10)
        s.assign_s1v1(1.0, s0)
        stream = torch.cuda.ExternalStream(op.stream, device=dev)
        eul, rk4 = swm.ExplicitEul1(), swm.RK4()
        legs = {"model_step": lambda: op.model_step(s, w["dt"], 1),
                "diffusion_step": lambda: eul.step(s, dop, w["dt"], 1),
                "rk4_step": lambda: rk4.step(s, op, w["dt"], 1)}
        r = {}
        for name, fn in legs.items():
            for _ in range(warmup):
                fn()
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(steps)]
            torch.cuda.synchronize(dev)
            for a, b in evs:
                s.assign_s1v1(1.0, s0)
                with torch.cuda.stream(stream):
                    flush.zero_()
                a.record(stream)
                fn()
                b.record(stream)
            torch.cuda.synchronize(dev)
            ms = sum(a.elapsed_time(b) for a, b in evs) / steps
            r[name + "_ms"] = round(ms, 5)
        r["model_steps_per_s"] = round(1e3 / r["model_step_ms"], 3)
        r["state_finite"] = bool(all(np.isfinite(a).all() for a in s.download()))
        out[prec] = r
        del op, dop
    return out


# The C-grid SBP family (&shallow_water_model_c) at N=384, SBP 4/2, FP64:
# six passes per RK4 stage (centre_a, faces_a, curl, w2uv with the curl's
# corner sync, centre_b, faces_b).  Algorithmic HBM words per point and stage of
# those passes (inputs and outputs of each pass, metric included):
#   centre_a 6 + faces_a 17 + curl 4 + w2uv 3 + centre_b 13 + faces_b 3,
#   plus the stage epilogues of the three state components (2, 4, 2 and 3
#   words in stages 1..4): 4 x 46 + 3 x 11 = 217 words per point and step.
CGRID_WORDS_PER_POINT_STEP = 217
CGRID_LAUNCHES_PER_STEP = 24          # 4 x 6 passes (the curl's corner sync rides in w2uv's reads)
# The namelist's C-grid model step adds one explicit Euler step of the
# hyperdiffusion (hordiff_c_biharm_curl_div, hordiff_scalar_C; 2/1
# operators).  Words per point of its passes, inputs + outputs + metric:
# co2contra / contra2co 15 (centre_a 5 + faces_a 10), div 6, grad 3, curl 4,
# grad_perp 5; curl part 2 x (4 + 5 + 15), div part 2 x (15 + 6 + 3), h part
# 2 x (3 + 15 + 6), the combine pass 11 (5 results, state read and written):
# 48 + 48 + 48 + 11 = 155 words per point.
CGRID_DIFF_WORDS_PER_POINT_STEP = 155
CGRID_DIFF_LAUNCHES_PER_STEP = 29     # 24 passes, 2 corner syncs of 2 kernels, combine


def cgrid_leg(local, steps, warmup, cpu=True):
    """The C-grid operator family's RK4 step (FP64) on a seeded balanced
    zonal flow at N=384, dt = 37.5 s (Courant number 0.4: the 4/2 C-grid
    scheme's RK4 limit is near 0.6): device-timed steps with an L2 flush
    before each, end-to-end steps through the C-ABI with page-locked host
    arrays, parity against the FP64 oracle after two steps, and the oracle's
    own rate on the host cores."""
    import numpy as np
    import torch

    import cubedsphere_sbp_swm_gb300 as swm
    from cubedsphere_sbp_swm_gb300 import initial

    N, ORDER, DT = 384, 42, 37.5
    dev = torch.device("cuda", local)
    h, u, v, _ = initial.balanced_zonal_c(N, 11, 24)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    ts = swm.RK4()

    def timed(prec, model=False):
        """Device-timed steps: RK4 (model False) or the drivers' model step
        with the namelist's hyperdiffusion (model True)."""
        op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=ORDER, names=swm.c_grid_names(ORDER),
                                             precision=prec, device=local))
        if model:
            swm.OperatorSWMDiff(op)  # hordiff_c_biharm_curl_div 0.03, hordiff_scalar_C 0.03

        def step(st, n):
            if model:
                op.model_step(st, DT, n)
            else:
                ts.step(st, op, DT, n)

        s0, s = op.create_stvec(), op.create_stvec()
        s0.upload(h, u, v)
        s.assign_s1v1(1.0, s0)
        stream = torch.cuda.ExternalStream(op.stream, device=dev)
        for _ in range(warmup):
            step(s, 1)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        torch.cuda.synchronize(dev)
        for a, b in evs:
            s.assign_s1v1(1.0, s0)
            with torch.cuda.stream(stream):
                flush.zero_()
            a.record(stream)
            step(s, 1)
            b.record(stream)
        torch.cuda.synchronize(dev)
        return op, s, sum(a.elapsed_time(b) for a, b in evs) / steps

    # end to end through the C-ABI with page-locked host arrays: pipelined
    # (two states take turns; swm_state_upload_async / _download_async on the
    # copy engines) and serial (synchronous upload, step, download)
    pins = [torch.empty(a.shape, dtype=torch.float64, pin_memory=True) for a in (h, u, v) for _ in range(3)]
    hin = [pins[3 * k].numpy() for k in range(3)]
    houts = [tuple(pins[3 * k + 1 + q].numpy() for k in range(3)) for q in range(2)]
    for t_, a_ in zip(hin, (h, u, v)):
        t_[...] = a_
    n_e2e = max(10, steps // 2)

    def e2e_rates(op, s):
        states = [s, op.create_stvec()]

        def pipelined(n):
            for k in range(n):
                st = states[k % 2]
                st.upload_async(*hin)
                ts.step(st, op, DT, 1)
                st.download_async(houts[k % 2])
            op.synchronize()

        def serial(n):
            for _ in range(n):
                s.upload(*hin)
                ts.step(s, op, DT, 1)
                s.download(out=houts[0])

        pipelined(3)
        t0 = time.perf_counter()
        pipelined(n_e2e)
        pv = n_e2e / (time.perf_counter() - t0)
        serial(2)
        t0 = time.perf_counter()
        serial(n_e2e)
        return pv, n_e2e / (time.perf_counter() - t0)

    # the namelist's model step (RK4 + explicit Euler hyperdiffusion), both
    # forms, and one step of each for parity
    model = {}
    for prec in ("fp32", "fp64"):
        opm, sm, msm = timed(prec, model=True)
        sm.upload(h, u, v)
        opm.model_step(sm, DT, 1)
        model[prec] = (msm, sm.download())
        del opm, sm
    op32, s32, ms32 = timed("fp32")
    e2e32, e2e32_serial = e2e_rates(op32, s32)
    s32.upload(h, u, v)
    ts.step(s32, op32, DT, 2)
    got32 = s32.download()
    del op32, s32
    op, s, ms = timed("fp64")
    e2e, e2e_serial = e2e_rates(op, s)
    nbytes = sum(a.size for a in (h, u, v)) * 8
    # parity after two steps against the oracle (and its rate)
    s.upload(h, u, v)
    ts.step(s, op, DT, 2)
    got = s.download()
    res = {"workload": "C-grid SBP 4/2 vector-invariant family (&shallow_water_model_c operators), "
                       "N=384 (6 x 384^2 centres, 6 x 385 x 384 faces per velocity component), FP64",
           "operators": swm.c_grid_names(ORDER), "dt_s": DT,
           "value": round(1e3 / ms, 3), "unit": "steps/s", "ms_per_step": round(ms, 5),
           "fp32_form": {"value": round(1e3 / ms32, 3), "unit": "steps/s", "ms_per_step": round(ms32, 5),
                         "e2e": {"value": round(e2e32, 3), "serial_value": round(e2e32_serial, 3),
                                 "unit": "steps/s"},
                         "note": "FP32 passes, FP32 (hi, lo) state pair, two-sum RK accumulation"},
           "launches_per_step": CGRID_LAUNCHES_PER_STEP,
           "e2e": {"value": round(e2e, 3), "unit": "steps/s", "h2d_bytes_per_step": nbytes,
                   "d2h_bytes_per_step": nbytes,
                   "path": "swm_state_upload_async + swm_rk4_step + swm_state_download_async on two states "
                           "taking turns (page-locked arrays, copy engines); clock stopped after the last "
                           "download landed",
                   "serial_value": round(e2e_serial, 3),
                   "serial_path": "swm_state_upload + swm_rk4_step + swm_state_download, one synchronous "
                                  "step at a time"}}
    npts = 6 * N * N
    peak, peak_kind = _measured_peak()
    achieved = CGRID_WORDS_PER_POINT_STEP * 8 * npts / (ms / 1e3) / 1e9
    res["roofline"] = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                       "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                       "algorithmic_bytes_per_step": CGRID_WORDS_PER_POINT_STEP * 8 * npts,
                       "scope": "whole RK4 step (%d launches)" % CGRID_LAUNCHES_PER_STEP}
    a32 = CGRID_WORDS_PER_POINT_STEP * 4 * npts / (ms32 / 1e3) / 1e9
    res["fp32_form"]["roofline"] = {"bound": "hbm", "achieved": round(a32, 1), "peak": peak, "unit": "GB/s",
                                    "frac": round(a32 / peak, 4), "peak_source": peak_kind,
                                    "algorithmic_bytes_per_step": CGRID_WORDS_PER_POINT_STEP * 4 * npts}
    mwords = CGRID_WORDS_PER_POINT_STEP + CGRID_DIFF_WORDS_PER_POINT_STEP
    mres = {"config": "the namelist's C-grid step (namelist_swm:80-102): RK4, then one explicit Euler step of "
                      "hordiff_c_biharm_curl_div (0.03) and hordiff_scalar_C (0.03)",
            "launches_per_step": CGRID_LAUNCHES_PER_STEP + CGRID_DIFF_LAUNCHES_PER_STEP}
    for prec, elt, key in (("fp64", 8, None), ("fp32", 4, "fp32_form")):
        msm = model[prec][0]
        am = mwords * elt * npts / (msm / 1e3) / 1e9
        r = {"value": round(1e3 / msm, 3), "unit": "steps/s", "ms_per_step": round(msm, 5),
             "diffusion_ms_per_step": round(msm - (ms if prec == "fp64" else ms32), 5),
             "roofline": {"bound": "hbm", "achieved": round(am, 1), "peak": peak, "unit": "GB/s",
                          "frac": round(am / peak, 4), "peak_source": peak_kind,
                          "algorithmic_bytes_per_step": mwords * elt * npts}}
        if key:
            mres[key] = r
        else:
            mres.update(r)
    res["model_step"] = mres
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle  # the checker and the timed CPU baseline
        od = oracle.OracleCDomain(N, ORDER)
        threads = os.cpu_count() or 1
        oracle.set_threads(threads)
        t0 = time.perf_counter()
        mwant = od.model_step(h, u, v, DT, 1)
        mel = time.perf_counter() - t0
        for prec, key in (("fp64", "parity_vs_oracle_1_step_max_rel_l2"),
                          ("fp32", "fp32_error_vs_oracle_1_step_max_rel_l2")):
            mres[key] = max(float(np.linalg.norm(a - b) / np.linalg.norm(b))
                            for a, b in zip(model[prec][1], mwant))
        mres["cpu_oracle"] = {"value": round(1 / mel, 4), "unit": "steps/s", "cores": threads, "kind": "port",
                              "sample": "1 model step of the same state at N=384 (C-grid oracle)"}
        t0 = time.perf_counter()
        want = od.rk4(h, u, v, DT, 2)
        el = time.perf_counter() - t0
        rel = max(float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(got, want))
        res["parity_vs_oracle_2_steps_max_rel_l2"] = rel
        res["fp32_form"]["error_vs_oracle_2_steps_max_rel_l2"] = max(
            float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(got32, want))
        res["cpu_oracle"] = {"value": round(2 / el, 4), "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": "2 RK4 steps of the same state at N=384 (C-grid oracle)"}
    return res


def _oracle_rate(od, state, dt, threads, window_s, warm_s, min_steps=1):
    """Oracle RK4 steps/s with `threads` OpenMP threads: whole steps on the
    caller's arrays in place, after warm_s seconds of untimed steps, timed
    over at least window_s seconds."""
    import oracle
    oracle.set_threads(threads)
    h, u, v = (a.copy() for a in state)
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < warm_s:
        od.rk4_inplace(h, u, v, dt, 1)
    steps, t0 = 0, time.perf_counter()
    while steps < min_steps or time.perf_counter() - t0 < window_s:
        od.rk4_inplace(h, u, v, dt, 1)
        steps += 1
    el = time.perf_counter() - t0
    return steps / el, steps, el


def _cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part", "hardware")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def run_reference_arm(args):
    """The reference's CPU path on the host cores: the FP64 oracle (C++
    restatement of the Fortran reference; the reference itself needs a
    Fortran compiler and MPI, which neither machine has).  Exactly K timed
    steps follow W warm-up steps and 2 s of untimed steps; the K-step
    measurement repeats until the timed window is at least 5 s.  OpenMP
    threads are pinned to cores (OMP_PROC_BIND=close, OMP_PLACES=cores, set
    before the runtime loads).  Also reported: the single-thread rate and the
    N=48 SBP 4/2 configuration's rates, and with --cpu-also the listed
    workloads' all-thread rates."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")
    w = WORKLOADS[args.workload]
    h, u, v, info = _state(w)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    od = oracle.OracleDomain(w["N"], w["order"])
    hh, uu, vv = h.copy(), u.copy(), v.copy()
    for _ in range(args.warmup):
        od.rk4_inplace(hh, uu, vv, w["dt"], 1)
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < 2.0:
        od.rk4_inplace(hh, uu, vv, w["dt"], 1)
    # the state turns non-finite after a few hours at the workload dt; every
    # K-step block restarts from the initial state (outside the timed region)
    el, blocks = 0.0, 0
    while blocks < 1 or el < 5.0:
        hh[...], uu[...], vv[...] = h, u, v
        t0 = time.perf_counter()
        for _ in range(args.steps):
            od.rk4_inplace(hh, uu, vv, w["dt"], 1)
        el += time.perf_counter() - t0
        blocks += 1
    timed = blocks * args.steps
    val = timed / el
    rates = {args.workload: {"threads": cores, "steps_per_s": round(val, 4), "timed_steps": timed,
                             "window_s": round(el, 3)}}
    r1, n1, e1 = _oracle_rate(od, (h, u, v), w["dt"], 1, 5.0, 1.0)
    rates[args.workload].update(single_thread_steps_per_s=round(r1, 4), single_thread_steps=n1,
                                single_thread_window_s=round(e1, 3),
                                thread_speedup=round(val / r1, 3))
    # configuration 1: N=48, SBP 4/2, dt = 900 s (the reference's CPU-runnable case)
    from cubedsphere_sbp_swm_gb300 import initial
    c1 = initial.CONFIGS[1]
    st1 = initial.config_state(1)[:3]
    od1 = oracle.OracleDomain(c1["N"], c1["sbp_order"])
    ra, na, ea = _oracle_rate(od1, st1, c1["dt"], cores, 5.0, 1.0)
    rb, nb, eb = _oracle_rate(od1, st1, c1["dt"], 1, 5.0, 1.0)
    rates["n48_d42"] = {"threads": cores, "steps_per_s": round(ra, 3), "timed_steps": na,
                        "single_thread_steps_per_s": round(rb, 3), "single_thread_steps": nb,
                        "dt_s": c1["dt"], "one_day_s": round(c1["steps"] / ra, 3)}
    for extra in (args.cpu_also or "").split(","):
        if extra and extra in WORKLOADS and extra not in rates:
            we = WORKLOADS[extra]
            ste = _state(we)[:3]
            ode = oracle.OracleDomain(we["N"], we["order"])
            re_, ne, ee = _oracle_rate(ode, ste, we["dt"], cores, 5.0, 1.0, min_steps=3)
            rates[extra] = {"threads": cores, "steps_per_s": round(re_, 4), "timed_steps": ne,
                            "window_s": round(ee, 3)}
            del ode, ste
    sample = (f"{timed} RK4 steps ({blocks} blocks of K={args.steps}, each from the initial state) "
              f"of the N={w['N']} d{w['order']} FP64 oracle, the C++ restatement of the reference "
              f"(the Fortran/MPI reference has no compiler on this image); {cores} OpenMP threads "
              f"pinned to cores, {el:.1f} s window")
    line = {
        "metric": METRIC, "value": round(val, 4), "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(el / timed * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": _data_desc(w, info),
        "config": {"workload": w["desc"] + ", FP64", "N": w["N"], "sbp": "d%d" % w["order"],
                   "dt_s": w["dt"]},
        "cpu_baseline": {"value": round(val, 4), "unit": "steps/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(val, 4), "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cpu_rates": rates,
        "host": {"cpu": _cpu_model(), "nproc": cores,
                 "omp": {k: os.environ.get(k) for k in ("OMP_PROC_BIND", "OMP_PLACES")}},
        "reference_fortran": "not measurable: no Fortran compiler or MPI on the build image or the GPU box",
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_subprocess(args):
    """The reference arm's measurement (run_reference_arm) in a fresh
    process, so that the default run's cpu_baseline and the reference arm
    are one procedure: same code, same thread pinning, no GPU process state.
    Adds the large instance's oracle rate."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--steps", str(args.steps), "--warmup", str(args.warmup), "--workload", args.workload,
           "--cpu-also", "n1024_d63" if not args.no_large else ""]
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    try:
        out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env)
    except (OSError, subprocess.TimeoutExpired) as e:
        return {"cpu_baseline": {"unavailable": str(e)}, "rates": {}}
    for line in out.stdout.splitlines()[::-1]:
        if line.startswith("{"):
            d = json.loads(line)
            cb = dict(d["cpu_baseline"])
            cb["same_procedure_as"] = "bench.py --impl reference"
            return {"cpu_baseline": cb, "rates": d.get("cpu_rates", {}), "host": d.get("host")}
    return {"cpu_baseline": {"unavailable": out.stderr[-300:]}, "rates": {}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--workload", default="n384_d42", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the FP32-vs-FP64 run over the workload's simulated days")
    ap.add_argument("--no-ensemble", action="store_true",
                    help="skip the 96-member ensemble leg")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the adjoint leg (N=192, 240 steps)")
    ap.add_argument("--stage-shape", default=None,
                    help="WIDTH,SEG_ROWS,GRID[,BOX] of the FP32 stage kernel instead of tuning it, "
                         "BOX one of auto, strip, widest (reproducible profiling runs)")
    ap.add_argument("--no-diffusion", action="store_true",
                    help="skip the RK4 + hyperdiffusion model-step leg")
    ap.add_argument("--days", type=float, default=None,
                    help="simulated days of the accuracy run (default: the workload's)")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the large single instance (N=1024, SBP 6/3) beside the headline")
    ap.add_argument("--cpu-also", default="",
                    help="reference arm: also time these workloads' oracle (comma-separated)")
    ap.add_argument("--quick", action="store_true",
                    help="profiling case: time only the FP32 steps, print a short line")
    ap.add_argument("--no-cgrid", action="store_true",
                    help="skip the C-grid operator family's RK4 leg")
    ap.add_argument("--only", choices=("ensemble", "adjoint", "diffusion", "cgrid"), default=None,
                    help="run one leg alone and print its JSON object")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.only:
        import torch
        _, _, local = _dist()
        torch.cuda.set_device(local)
        if args.only == "ensemble":
            res = ensemble_leg(local, max(10, args.steps // 2), args.warmup, _measured_peak()[0])
        elif args.only == "adjoint":
            res = adjoint_leg(local)
        elif args.only == "cgrid":
            res = cgrid_leg(local, max(10, args.steps // 2), args.warmup, cpu=not args.no_cpu)
        else:
            w = WORKLOADS[args.workload]
            h, u, v, _ = _state(w)
            res = diffusion_leg(w, h, u, v, local, max(10, args.steps // 2), args.warmup)
        print(json.dumps({args.only: res}), flush=True)
        return
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
