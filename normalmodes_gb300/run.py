"""A NormalModes job on the GPU: the reference's driver (src/mainnm.f90)
with its configuration file and its result files, on this library.

    python -m normalmodes_gb300.run global_conf [--mixed] [--block 0|32] [--slices N] [--dry-run]

* ``global_conf`` is read as the reference reads it (para_init,
  src/mod_para.f90:79-137, with string_conf of src/mod_string.f90): on each
  line the text after ``#`` is dropped, ``=`` and tabs become blanks, and the
  first line whose first word is the key gives its second word.  Keys: JOB,
  basename, inputdir, outputdir, lowfreq, upfreq (REAL, mHz), pOrder.
* JOB 1 assembles without gravity; JOB 2 and 3 with the reference gravity of
  ``<inputdir><basename>_pod_<p>_potential_acceleration_true.dat``
  (src/mod_para.f90:133-138; JOB 3 adds no operator term, see the design
  notes).  Relative paths are taken from the directory the job runs in, as
  the reference takes them.
* The solve is nm_solve: by default the reference's algorithm (FP64,
  single-vector filtered Lanczos); ``--mixed`` selects the mixed-precision
  block path.  The eigenvalues are printed as pnm_apply_pevsl prints them
  (relative errors, then frequencies in mHz and periods in s,
  src/mod_pevsl.f90:164-186), and the eigenvectors, the node list and the
  node status are written in the reference's files (nmm_write_results,
  src/mod_pevsl.f90:188-247), with a JSON run record beside them
  (``<prefix>_run.json``: configuration, sizes, per slice the filter degree,
  Lanczos steps, timings and operator counts, per eigenpair both residuals).
* ``--slices N`` cuts the interval into N slices of equal estimated
  eigenvalue count (nm_slice_spectrum) and solves them on one context
  (nm_solve_batched); the eigenpairs are merged in ascending order.
* ``--dry-run`` stops before the GPU: configuration, model, assembly.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
from dataclasses import dataclass

import numpy as np

KEYS = ("JOB", "basename", "inputdir", "outputdir", "lowfreq", "upfreq", "pOrder")


class ConfError(ValueError):
    pass


def _words(line: str) -> list:
    i = line.find("#")
    if i >= 0:
        line = line[:i]
    return line.replace("=", " ").replace("\t", " ").split()


def conf_value(lines: list, key: str) -> str:
    """The second word of the first line whose first word is `key`."""
    for ln in lines:
        w = _words(ln)
        if w and w[0] == key:
            if len(w) < 2:
                raise ConfError(f"{key}: no value")
            return w[1]
    raise ConfError(f"there is no {key} on column 1")


@dataclass
class Job:
    job: int
    basename: str
    inputdir: str
    outputdir: str
    lowfreq: float
    upfreq: float
    porder: int

    @property
    def gravity(self) -> bool:
        return self.job in (2, 3)

    @property
    def base_path(self) -> str:
        return self.inputdir + self.basename


def read_global_conf(path: str) -> Job:
    if not os.path.exists(path):
        raise ConfError(f'File "{path}" does not exist.')
    with open(path) as f:
        lines = f.read().splitlines()
    v = {k: conf_value(lines, k) for k in KEYS}
    try:
        job = int(v["JOB"])
        porder = int(v["pOrder"])
        # REAL (single precision) in the reference
        lo, hi = float(np.float32(v["lowfreq"])), float(np.float32(v["upfreq"]))
    except ValueError as e:
        raise ConfError(f"bad number in {path}: {e}") from None
    if job not in (1, 2, 3):
        raise ConfError(f"JOB = {job} is not supported (1: no gravity, 2 and 3: reference gravity)")
    if porder not in (1, 2):
        raise ConfError(f"pOrder = {porder}: the element is built for pOrder 1 and 2")
    if lo >= hi:
        raise ConfError("Error: please check input frequencies")
    return Job(job, v["basename"], v["inputdir"], v["outputdir"], lo, hi, porder)


# the default-real PI literal of src/mod_pevsl.f90, widened to double
PI = float(np.float32(3.14159265359))


def report(lam, err, out=sys.stdout) -> None:
    """The tables pnm_apply_pevsl prints (src/mod_pevsl.f90:168-186)."""
    print(" Relative errors: from the smallest to largest eigens:", file=out)
    for j, e in enumerate(err, 1):
        print(f" Row {j:6d}  relative err. {e:.16e}", file=out)
    print(" " + "=" * 63, file=out)
    print(" Transform to frequencies (mHz), and periods (s)", file=out)
    for j, lm in enumerate(lam, 1):
        if lm > 1e-15:
            print(f" Row {j:6d} {math.sqrt(lm) / PI / 2.0 * 1e3:24.16f} {2.0 * PI / math.sqrt(lm):24.16f}", file=out)
        else:
            print(f" Row {j:6d} {lm:24.16e} ...too small...", file=out)
    print(" " + "=" * 64, file=out)


def make_solver(mats: dict, porder: int, mixed: bool):
    """The GPU context for the job's operators (fails without the CUDA
    library or a GPU; there is no CPU path)."""
    from .nmgpu import NM_PREC_FP64, NM_PREC_MIXED, Solver
    return Solver(mats, porder, precision=NM_PREC_MIXED if mixed else NM_PREC_FP64)


def _solve(sv, job: Job, block: int, slices: int, out):
    """One interval (nm_solve), or `slices` slices of equal estimated
    eigenvalue count (nm_slice_spectrum) solved on the same context
    (nm_solve_batched) and merged in ascending order."""
    if slices <= 1:
        cuts, counts = [(job.lowfreq, job.upfreq)], [None]
        rs = [sv.solve(job.lowfreq, job.upfreq, want_vectors=True, unscale=True, block=block)]
    else:
        cuts, counts = sv.slice_spectrum(job.lowfreq, job.upfreq, slices)
        print(" spectrum slices (mHz) and estimated eigenvalue counts:", file=out)
        for (a, b), c in zip(cuts, counts):
            print(f"   {a:.9f} {b:.9f} {c:10.1f}", file=out)
        rs = sv.solve_batched(cuts, want_vectors=True, unscale=True, block=block)
    lam = np.concatenate([r.lam for r in rs])
    err = np.concatenate([r.err_ref for r in rs])
    res2 = np.concatenate([r.res2 for r in rs])
    vec = np.concatenate([r.vec for r in rs], axis=1)
    order = np.argsort(lam, kind="stable")
    meta = [{"f_lo_mhz": float(a), "f_hi_mhz": float(b), "estimated_count": None if c is None else float(c),
             "nev": int(len(r.lam)), "xintv": [float(x) for x in r.xintv], "filter_degree": int(r.pol_deg),
             "lanczos_steps": int(r.lanczos_steps), "times_s": {k: float(v) for k, v in r.times.items()},
             "operator_counts": {k: int(v) for k, v in r.counts.items()}}
            for (a, b), c, r in zip(cuts, counts, rs)]
    return lam[order], err[order], res2[order], vec[:, order], meta


def run_record(job: Job, model, mixed: bool, block: int, lam, err, res2, meta) -> dict:
    """The JSON run record: configuration, model sizes, solver settings, per
    slice the interval, filter, steps, timings and operator counts, and per
    eigenpair its eigenvalue, frequency, period and both residual norms."""
    info = model.info()
    nnz = dict(zip(("A", "B", "Ad", "Ap", "E", "ET"), (int(x) for x in info.nnz)))
    pos = lam > 1e-15
    f = np.where(pos, np.sqrt(np.abs(lam)) / PI / 2.0 * 1e3, 0.0)
    T = np.where(pos, 2.0 * PI / np.sqrt(np.where(pos, lam, 1.0)), 0.0)
    return {
        "config": {"JOB": job.job, "basename": job.basename, "inputdir": job.inputdir, "outputdir": job.outputdir,
                   "lowfreq": job.lowfreq, "upfreq": job.upfreq, "pOrder": job.porder},
        "model": {"ntet": info.ntet, "n_fluid_tets": info.n_fluid_tets, "n": info.n, "np": info.np,
                  "nnz": {k: v for k, v in nnz.items() if v}, "gravity": job.gravity},
        "solver": {"precision": "mixed" if mixed else "fp64", "block": block, "slices": meta},
        "eigenpairs": {"lambda": lam.tolist(), "f_mhz": f.tolist(), "period_s": T.tolist(),
                       "err_ref": err.tolist(), "res2": res2.tolist()},
    }


def run(job: Job, mixed: bool = False, block: int | None = None, dry_run: bool = False, out=sys.stdout,
        slices: int = 0) -> dict:
    from .model import Model
    model = Model.load(job.base_path, job.porder, gravity=job.gravity)
    info = model.info()
    print(f" JOB = {job.job}{'  (reference gravity)' if job.gravity else ''}", file=out)
    print(f" mesh name: {job.basename}   polynomial order {job.porder}", file=out)
    print(f" input directory: {job.inputdir}   output directory: {job.outputdir}", file=out)
    print(f" lower / upper frequency in mHz {job.lowfreq} {job.upfreq}", file=out)
    print(f" {info.ntet} tetrahedra ({info.n_fluid_tets} fluid), {info.n} displacement and {info.np} pressure DOFs",
          file=out)
    summary = {"ntet": info.ntet, "n": info.n, "np": info.np, "gravity": job.gravity}
    if dry_run:
        return summary
    if block is None:
        block = 32 if mixed else 0
    with make_solver(model.operators(), job.porder, mixed) as sv:
        lam, err, res2, vec, meta = _solve(sv, job, block, slices, out)
    report(lam, err, out=out)
    os.makedirs(job.outputdir or ".", exist_ok=True)
    prefix = model.write_results(job.outputdir, job.basename, job.lowfreq, job.upfreq, vec, job=job.job, nproc=1)
    print(" save eigenvectors: " + prefix + "_<i>.dat", file=out)
    with open(prefix + "_run.json", "w") as f:
        json.dump(run_record(job, model, mixed, block, lam, err, res2, meta), f, indent=1)
    print(" run record: " + prefix + "_run.json", file=out)
    summary.update(nev=len(lam), prefix=prefix, lam=lam)
    return summary


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="NormalModes job on the GPU")
    ap.add_argument("conf", nargs="?", default="global_conf")
    ap.add_argument("--mixed", action="store_true", help="mixed-precision block path")
    ap.add_argument("--block", type=int, default=None, help="0: single-vector, 32: block (default by precision)")
    ap.add_argument("--dry-run", action="store_true", help="read, load and assemble only")
    ap.add_argument("--slices", type=int, default=0,
                    help="solve N slices of equal estimated eigenvalue count on one context")
    a = ap.parse_args(argv)
    try:
        job = read_global_conf(a.conf)
    except ConfError as e:
        print(e, file=sys.stderr)
        return 2
    run(job, mixed=a.mixed, block=a.block, dry_run=a.dry_run, slices=a.slices)
    return 0


if __name__ == "__main__":
    sys.exit(main())
