#!/usr/bin/env python3
"""Benchmark of the NormalModes eigensolve on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision mixed|fp64] [--block 32|0] [--workload NAME]

Workload (default "ball36-p2-lateral"): the seeded 3-layer ball (solid inner
core, fluid outer core, solid mantle; 36^3 * 6 = 279,936 P2 tetrahedra,
1,198,455 displacement + 67,590 pressure DOFs, ~83 non-zeros per row of Ad)
with a +-2 % degree-8 lateral perturbation of vp / vs / rho; all eigenpairs
in 0.1-2.0 mHz.  "ball36-p2" is the same ball without the perturbation,
"ball12-p1" the small P1 ball (10,368 tetrahedra, 0.2-1.0 mHz) that the CPU
runs whole.

One bench run is ONE complete solve of the workload through the public
C-ABI, timed as K contiguous steps (the driver's --steps K): the solve's
block-Lanczos steps (one 32-vector filter application + Gram-Schmidt each)
are cut into K equal groups; step 1 also holds nm_create from pinned host
CSR arrays (host-to-device copies) and the bounds, step K the Ritz vectors,
the FP64 refinement, the residual check and the eigenvectors' copy back to
the host.  The K steps together are the whole job, timed between a
barrier + synchronize on both sides, so
  value : eigenpairs that pass the residual gate (err_ref <= 1e-10, the
          reference's norm, src/mod_pevsl.f90:158) / time of nm_solve,
          timed with CUDA events on the context's stream (operators resident
          in HBM when it starts: the reference's timed region
          src/mainnm.f90:43-44 to src/mod_pevsl.f90:203-204);
  e2e   : the same eigenpairs / wall time of all K steps (create, solve,
          vectors to the host, destroy).
W warm-up steps are W block steps of a truncated solve on a context created
once (bounds, filter graph, Gram-Schmidt, Rayleigh-Ritz, refinement and
residual kernels all run).  Every operator and block vector is larger than
L2 (Ad alone is 1.2 GB), so no L2 flush is needed between steps.

`--impl reference` times the CPU path of the same workload (the FP64
C/OpenMP restatement under oracle/ on all host cores, since the
Fortran/MPI/pEVSL reference cannot be built) on a bounded sample and projects
eigenpairs/s; it never touches the GPU.
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

METRIC = "eigenpairs/s at resid<=1e-10: mixed+batched vs plain FP64 on GB300; SpMV HBM GB/s"
WORKLOADS = {
    "ball36-p2-lateral": dict(
        desc="layered ball, 279,936 P2 tets, 1.2M DOF, +-2% degree-8 lateral perturbation, 0.1-2.0 mHz",
        model=dict(n_cells=36, porder=2, lateral_pert=0.02, lateral_lmax=8), porder=2, interval=(0.1, 2.0)),
    "ball36-p2": dict(
        desc="layered ball, 279,936 P2 tets, 1.2M DOF, 0.1-2.0 mHz",
        model=dict(n_cells=36, porder=2), porder=2, interval=(0.1, 2.0)),
    "ball12-p1": dict(
        desc="layered ball, 10,368 P1 tets, 0.2-1.0 mHz",
        model=dict(n_cells=12, porder=1), porder=1, interval=(0.2, 1.0)),
    "ball36-p2-lateral-grav": dict(
        desc="layered ball, 279,936 P2 tets, 1.2M DOF, +-2% degree-8 lateral perturbation, reference gravity "
             "(JOB = 2), 0.1-2.0 mHz",
        model=dict(n_cells=36, porder=2, lateral_pert=0.02, lateral_lmax=8, gravity=True), porder=2,
        interval=(0.1, 2.0)),
}
# Step counts of the reference algorithm (single-vector ChebLanNr, FP64) on
# the 1.2M-DOF ball, used only to project the CPU samples: the filter degree
# (125) and eigenpair count (1232) are those of the GPU solves of this
# workload, FP64 and mixed alike; the Lanczos steps are the 4992 block
# vectors that both the FP64 and the mixed block paths take on this ball,
# times the single-vector / block ratio measured on the 24^3 ball at
# 0.1-1.0 mHz (801 single-vector steps against 1152 block vectors for the
# same 203 eigenpairs, both on one GB300): 4992 * 801 / 1152 = 3471.
REF_COUNTS = {"ball36-p2-lateral": dict(nev=1232, lanczos_steps=3471, degree=125),
              "ball36-p2": dict(nev=1232, lanczos_steps=3471, degree=125), "ball12-p1": None}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--block", type=int, default=32)
    ap.add_argument("--workload", default="ball36-p2-lateral", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    return ap.parse_args()


# ----------------------------------------------------------------------------- distributed
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce(x: float, ws: int, op: str) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def aggregate(t_solve: float, t_e2e: float, nev: int, ws: int):
    """Replicas: every rank solves its own copy of the workload, so the job's
    time is the slowest rank's and its eigenpairs are the sum over ranks.
    Returns (value, e2e value, solve seconds, e2e seconds)."""
    t = allreduce(t_solve, ws, "max")
    te = allreduce(t_e2e, ws, "max")
    n_all = allreduce(float(nev), ws, "sum")
    return n_all / t, n_all / te, t, te


# ----------------------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile(prefix="clk", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
        self.f.close()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.f.name):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        finally:
            try:
                os.unlink(self.f.name)
            except OSError:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_launch(key: str):
    """DRAM bytes (read + write) per launch of `key` from the committed ncu
    summary (profiles/traffic.json), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        d = json.load(open(path))
        v = d.get(key, {})
        if isinstance(v, dict) and v.get("bytes_per_launch") is not None:
            return float(v["bytes_per_launch"])
    return None


# ----------------------------------------------------------------------------- CPU sample
def gershgorin_bounds(mats: dict) -> dict:
    """Intervals for the Chebyshev set-ups of the CPU sample from the
    Gershgorin discs of the diagonally scaled B (and -Ap): the time of a
    filter degree step depends on the degrees (fixed by the reference's
    rules) and not on the coefficients, so the sample skips the 1000- and
    2000-step Lanczos runs of the full set-up."""
    import numpy as np

    def disc(m, sign):
        A = m.to_scipy().tocsr() * sign
        d = A.diagonal()
        s = 1.0 / np.sqrt(d)
        R = abs(A).multiply(s[:, None]).multiply(s[None, :]).tocsr()
        r = np.asarray(R.sum(axis=1)).ravel() - 1.0
        hi = float((1.0 + r).max())
        return (max(float((1.0 - r).min()), 1e-3 * hi), hi)

    out = {"B": disc(mats["B"], 1.0)}
    if "Ap" in mats:
        out["Ap"] = disc(mats["Ap"], -1.0)
    return out


def cpu_setup(name: str, mats, porder: int, bounds=None):
    """The FP64 CPU restatement of the operators (scaling, Chebyshev set-ups
    with the reference's degrees)."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    if bounds is None and REF_COUNTS.get(name) is not None:
        bounds = gershgorin_bounds(mats)
    op = O.setup_operator(mats, porder, bounds=bounds)
    return op, time.perf_counter() - t0


def cpu_sample(name: str, op, seconds: float, t_setup: float = 0.0):
    """Time filter degree steps of the FP64 CPU restatement (all host threads)
    and project the reference algorithm's eigenpairs/s for the workload; the
    small workload runs its whole solve."""
    from oracle import oracle as O
    import numpy as np
    wl = WORKLOADS[name]
    refc = REF_COUNTS.get(name)
    if refc is None:
        t1 = time.perf_counter()
        r = O.apply_pevsl(op, *wl["interval"])
        t_solve = time.perf_counter() - t1
        return {"value": len(r.lam) / t_solve, "unit": "eigenpairs/s", "cores": os.cpu_count(), "kind": "port",
                "sample": f"complete FP64 C/OpenMP solve: {len(r.lam)} eigenpairs in {t_solve:.1f} s",
                "t_setup_s": t_setup}
    # one degree step of the filter = one B~^-1 apply + one A-op + recurrence
    pol = O.Pol(deg=1, mu=np.array([0.0, 1.0]), cc=0.0, dd=1.0, gam=0.0, bar=0.0, kind="interior")
    v = O.start_vector(op.n)
    op.chebav(pol, v)  # warm
    steps, t = 0, 0.0
    while steps == 0 or (t < seconds and steps < 64):
        t1 = time.perf_counter()
        op.chebav(pol, v)
        t += time.perf_counter() - t1
        steps += 1
    t_deg = t / steps
    t_solve = refc["lanczos_steps"] * refc["degree"] * t_deg
    value = refc["nev"] / t_solve
    sample = (f"{steps} filter degree steps (B~^-1 Chebyshev solve of degree {op.b_cheb[2]} + A-op with "
              f"Ap Chebyshev of degree {op.ap_cheb[2] if op.ap_cheb else 0}) of the FP64 C/OpenMP restatement "
              f"on the full workload, {t_deg:.3f} s each; eigenpairs/s = {refc['nev']} / "
              f"({refc['lanczos_steps']} Lanczos steps x degree {refc['degree']} x step time)")
    return {"value": value, "unit": "eigenpairs/s", "cores": os.cpu_count(), "kind": "port",
            "sample": sample, "t_degree_step_s": t_deg, "t_setup_s": t_setup}


def step_cuts(t0: float, t_end: float, block_times: list, k: int) -> list:
    """K + 1 boundaries of the K steps of one solve: t0, the end of every
    (len / K)-th block-Lanczos step, t_end.  Step 1 thus also holds the set-up
    before the first block step and step K everything after the last cut.
    With fewer block steps than K the span is cut evenly."""
    nb = len(block_times)
    if nb < k:
        return [t0 + (t_end - t0) * i / k for i in range(k + 1)]
    return [t0] + [block_times[(i + 1) * nb // k - 1] for i in range(k - 1)] + [t_end]


# ----------------------------------------------------------------------------- main
def main():
    a = parse()
    ws, rank, local = dist_init()
    wl = WORKLOADS[a.workload]
    lo, hi = wl["interval"]
    from normalmodes_gb300.model import Model
    mdl = Model.ball(**wl["model"])
    mats = mdl.operators()
    info = mdl.info()

    if a.impl == "reference":
        if rank != 0:
            return
        op, t_setup = cpu_setup(a.workload, mats, wl["porder"])
        if REF_COUNTS.get(a.workload) is not None:
            for _ in range(a.warmup):  # warm-up: one short sample each
                cpu_sample(a.workload, op, 0.0)
        vals, b = [], None
        for _ in range(max(1, a.steps)):
            b = cpu_sample(a.workload, op, a.cpu_seconds, t_setup)
            vals.append(b["value"])
        op.close()
        v = statistics.mean(vals)
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "eigenpairs/s", "n_gpus": a.gpus,
                "steps": a.steps, "warmup": a.warmup, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": wl["desc"], "n_dof": info.n, "n_pressure": info.np},
                "cpu_baseline": {**b, "value": v},
                "e2e": {"value": v, "unit": "eigenpairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import numpy as np
    import torch
    from normalmodes_gb300.nmgpu import NM_PHASE_LANCZOS, NM_PREC_FP64, NM_PREC_MIXED, Solver
    prec = NM_PREC_MIXED if a.precision == "mixed" else NM_PREC_FP64
    dev = local
    torch.cuda.set_device(dev)
    K = max(1, a.steps)

    # pinned host copies of the operators: the inputs of the timed solve
    pinned = {}
    for k, m in mats.items():
        pinned[k] = type(m)(torch.from_numpy(m.rowptr).pin_memory().numpy(),
                            torch.from_numpy(m.col).pin_memory().numpy(),
                            torch.from_numpy(m.val).pin_memory().numpy(), m.shape)

    # warm-up: W block steps of a truncated solve on one context (kept for
    # the kernel timings below)
    warm = Solver(pinned, wl["porder"], device=dev, precision=prec)
    W = max(a.warmup, 1)
    warm.solve(lo, hi, block=a.block, maxit=W * max(a.block, 1), want_vectors=True, unscale=True,
               allow_noconv=True)
    torch.cuda.synchronize()

    # the timed job: one complete solve, cut into K steps at block boundaries
    marks = []  # (phase, done, host time) at the solve's synchronised boundaries

    def on_progress(phase, done, total):
        marks.append((phase, done, time.perf_counter()))

    barrier(ws)
    torch.cuda.synchronize()
    with Clocks(dev) as clk:
        t0 = time.perf_counter()
        sv = Solver(pinned, wl["porder"], device=dev, precision=prec)
        h2d = sv.info().h2d_bytes
        stream = torch.cuda.ExternalStream(sv.stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        res = sv.solve(lo, hi, block=a.block, want_vectors=True, unscale=True, progress=on_progress)
        e1.record(stream)
        e1.synchronize()
        t_solve = e0.elapsed_time(e1) / 1e3
        sv.close()
        torch.cuda.synchronize()
        t_end = time.perf_counter()
    barrier(ws)
    t_e2e = t_end - t0
    clocks = clk.summary()
    gate = 1e-10
    ok = res.err_ref <= gate
    nev_ok = int(ok.sum())
    value, value_e2e, t, te = aggregate(t_solve, t_e2e, nev_ok, ws)
    d2h = 8 * (res.vec.size if res.vec is not None else 0) + 8 * 3 * len(res.lam)

    cuts = step_cuts(t0, t_end, [tm for ph, _, tm in marks if ph == NM_PHASE_LANCZOS], K)
    steps_ms = [round(1e3 * (cuts[k + 1] - cuts[k]), 1) for k in range(K)]

    # roofline of the dominant kernel: the block mass Chebyshev step
    # (k_mass_cheb, one launch per inner Chebyshev degree), timed live with
    # CUDA events on the context's stream
    which = 4 if a.block > 1 else 2
    ms, by, la = warm.time_op(which, 10)
    per_launch_ms = ms / la
    achieved = (by / la) / (per_launch_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    kname = ("k_mass_cheb (block 32, " + ("fp32" if prec == NM_PREC_MIXED else "fp64") + ")" if a.block > 1
             else "k_cheb (fp64 SELL)")
    tkey = ("k_mass_cheb_block32_fp32" if prec == NM_PREC_MIXED else "k_mass_cheb_block32_fp64") if a.block > 1 \
        else "k_cheb_fp64"
    roof = {"kernel": kname, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
            "algorithmic_bytes_per_launch": by / la, "launch_ms": per_launch_ms,
            "traffic": traffic_per_launch(tkey)}
    spmv = {}
    ms_b, by_b, _ = warm.time_op(1, 20)
    spmv["fp64_sell_B_spmv_GBs"] = round(by_b / ms_b / 1e6, 1)
    ms_f, by_f, la_f = warm.time_op(6 if a.block > 1 else 3, 3)
    spmv["filter_degree_step_ms"] = round(ms_f, 3)
    spmv["filter_degree_step_GBs"] = round(by_f / ms_f / 1e6, 1)
    winfo = warm.info()
    tuned = {"mass": {"vector_gathers": winfo.mass_vec, "threads": winfo.mass_threads, "sweep": winfo.mass_sweep},
             "ap": {"vector_gathers": winfo.ap_vec, "threads": winfo.ap_threads, "sweep": winfo.ap_sweep},
             "a_op": {"threads": winfo.aop_threads, "sweep": winfo.aop_sweep}}

    cpu = None
    if rank == 0 and not a.no_cpu:
        op, t_setup = cpu_setup(a.workload, mats, wl["porder"],
                                {"B": tuple(winfo.b_bounds), "Ap": tuple(winfo.ap_bounds)} if winfo.fs else
                                {"B": tuple(winfo.b_bounds)})
        cpu = cpu_sample(a.workload, op, a.cpu_seconds, t_setup)
        op.close()
    warm.close()
    if rank != 0:
        return
    nev = len(res.lam)
    line = {
        "metric": METRIC, "value": value, "unit": "eigenpairs/s", "n_gpus": ws, "steps": K,
        "warmup": a.warmup, "ms_per_step": t * 1e3 / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 filter SpMM / f64 Lanczos, Rayleigh-Ritz, refinement residuals" if prec == NM_PREC_MIXED
        else "f64",
        "data": "synthetic",
        "config": {"workload": wl["desc"], "n_dof": info.n, "n_pressure": info.np, "nnz": list(info.nnz),
                   "interval_mhz": [lo, hi], "precision": a.precision, "block": a.block,
                   "step": f"1/{K} of one complete solve (block-Lanczos steps cut into {K} equal groups; "
                           "create + bounds in the first, Ritz + refinement + residual check + copy-out in the last)",
                   "l2": "operators and block vectors exceed L2 (Ad 1.2 GB); no flush",
                   "warmup_steps": f"{W} block steps of a truncated solve",
                   "residual_gate": f"err_ref <= {gate:g} (src/mod_pevsl.f90:158 RMS norm); value counts only those",
                   "eigenpairs_found": nev, "eigenpairs_gated": nev_ok,
                   "lanczos_vectors": res.lanczos_steps, "filter_degree": res.pol_deg,
                   "max_err_ref": float(res.err_ref.max()) if nev else None,
                   "median_err_ref": float(np.median(res.err_ref)) if nev else None,
                   "max_res2": float(res.res2.max()) if nev else None,
                   "median_res2": float(np.median(res.res2)) if nev else None,
                   "refinement": {k: res.counts[k] for k in ("refine_passes", "refine_blocks", "refine_maxdeg",
                                                             "refine_steps", "res2_before_refine",
                                                             "refine_guards")},
                   "parallelism": f"replicas x{ws}", "autotuned_gathers": tuned},
        "gpu_launches": res.counts["kernels"],
        "clocks": clocks,
        "roofline": roof,
        "spmv": spmv,
        "e2e": {"value": value_e2e, "unit": "eigenpairs/s", "h2d_bytes_per_step": h2d // K,
                "d2h_bytes_per_step": d2h // K, "seconds": te},
        "steps_ms": steps_ms,
        "cpu_baseline": cpu,
        "times_s": {**res.times, "solve_events": t_solve},
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
