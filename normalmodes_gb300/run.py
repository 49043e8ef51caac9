"""A NormalModes job on the GPU: the reference's driver (src/mainnm.f90)
with its configuration file and its result files, on this library.

    python -m normalmodes_gb300.run global_conf [--mixed] [--block 0|32] [--slices N]
                                                [--checkpoint] [--resume] [--dry-run]
    python -m torch.distributed.run --nproc-per-node G -m normalmodes_gb300.run global_conf --slices N

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
* Under torchrun (one GPU per rank) every rank loads the operator and
  solves every size-th slice; only the slices, eigenvalues and file indices
  cross ranks (gloo), and the files are those of a one-GPU job.
* The first rank also writes the reference's run log,
  ``<outputdir><basename>_0.log`` (numbered phases and elapsed times,
  src/mod_utility.f90:39-148).
* ``--checkpoint`` saves every solved slice (and the slice list) as
  ``<prefix>_ckpt_slice<j>.npz``; ``--resume`` loads them instead of solving
  those slices again, so an interrupted multi-slice job redoes only what is
  missing.
* ``--dry-run`` stops before the GPU: configuration, model, assembly.
"""
from __future__ import annotations

import argparse
import io
import json
import math
import os
import sys
import time
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


class PhaseLog:
    """The reference's run log, <outputdir><basename>_0.log (openlogfile,
    writelog and report_time, src/mod_utility.f90:39-148): numbered phase
    messages and the wall time elapsed since the start.  The suffix is 0
    as in the reference, whose name takes the rank of process 0."""

    def __init__(self, job: "Job", enabled: bool):
        self.f = None
        self.n = 0
        self.t0 = time.perf_counter()
        if enabled:
            os.makedirs(job.outputdir or ".", exist_ok=True)
            self.f = open(f"{job.outputdir}{job.basename}_0.log", "w")
            self.f.write("  Start program at time elapsed = 0.0 second.\n")

    def phase(self, msg: str) -> None:
        if self.f:
            self.n += 1
            self.f.write(f"{self.n:4d}. {msg}\n")

    def stamp(self) -> None:
        if self.f:
            self.f.write(f"  Time elapsed = {time.perf_counter() - self.t0:24.15f}      seconds.\n")
            self.f.flush()

    def close(self) -> None:
        if self.f:
            self.f.close()
            self.f = None


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


def make_solver(mats: dict, porder: int, mixed: bool, device: int = 0):
    """The GPU context for the job's operators (fails without the CUDA
    library or a GPU; there is no CPU path)."""
    from .nmgpu import NM_PREC_FP64, NM_PREC_MIXED, Solver
    return Solver(mats, porder, device=device, precision=NM_PREC_MIXED if mixed else NM_PREC_FP64)


class Group:
    """The ranks of a job started by torchrun, one GPU each (RANK,
    WORLD_SIZE and LOCAL_RANK from the environment; MASTER_ADDR/PORT for the
    rendezvous).  Only small control messages cross ranks -- the slices,
    eigenvalues and file indices -- so they go over gloo.  Without torchrun
    it is a single rank and nothing is imported."""

    def __init__(self):
        self.size = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self._own = False
        if self.size > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
                dist.init_process_group("gloo", rank=self.rank, world_size=self.size)
                self._own = True

    def bcast(self, obj):
        if self.size == 1:
            return obj
        import torch.distributed as dist
        box = [obj]
        dist.broadcast_object_list(box, src=0)
        return box[0]

    def gather(self, obj) -> list:
        if self.size == 1:
            return [obj]
        import torch.distributed as dist
        out = [None] * self.size
        dist.all_gather_object(out, obj)
        return out

    def close(self) -> None:
        if self._own:
            import torch.distributed as dist
            dist.destroy_process_group()
            self._own = False


def _num(v):
    return float(v) if isinstance(v, float) else int(v)


def _save_slice(path: str, r, key: str) -> None:
    """Checkpoint of one solved slice (written to a temporary name first, so
    an interrupted write leaves no checkpoint).  `key` names the slice, the
    job and the solver settings it was solved with."""
    tmp = path + ".part.npz"
    vec = r.vec if r.vec is not None else np.zeros((0, 0))
    np.savez(tmp, lam=r.lam, err_ref=r.err_ref, res2=r.res2, vec=vec, xintv=np.asarray(r.xintv, dtype=np.float64),
             pol_deg=int(r.pol_deg), lanczos_steps=int(r.lanczos_steps),
             times=json.dumps({k: float(v) for k, v in r.times.items()}),
             counts=json.dumps({k: _num(v) for k, v in r.counts.items()}), key=key)
    os.replace(tmp, path)


def _load_slice(path: str, key: str):
    """The checkpoint at `path` if it was saved under the same `key` (slice,
    job, solver settings), else None."""
    from types import SimpleNamespace
    with np.load(path) as z:
        if "key" not in z.files or str(z["key"]) != key:
            return None
        return SimpleNamespace(lam=z["lam"], err_ref=z["err_ref"], res2=z["res2"], vec=z["vec"],
                               xintv=tuple(z["xintv"]), pol_deg=int(z["pol_deg"]),
                               lanczos_steps=int(z["lanczos_steps"]), times=json.loads(str(z["times"])),
                               counts=json.loads(str(z["counts"])))


def _write_json(path: str, obj) -> None:
    """JSON written to a temporary name and moved into place."""
    tmp = path + ".part"
    with open(tmp, "w") as f:
        json.dump(obj, f)
    os.replace(tmp, path)


def _solve(sv, job: Job, block: int, slices: int, out, grp: Group, ckpt: str | None = None, resume: bool = False,
           settings: str = ""):
    """One interval (nm_solve), or `slices` slices of equal estimated
    eigenvalue count (nm_slice_spectrum, on the first rank) solved on this
    rank's context (nm_solve_batched): slice j belongs to rank j mod size.
    With `ckpt` every solved slice (and the slice list) is saved under that
    prefix, keyed by `settings` (job and solver settings) and the slice's
    interval; with `resume` saved slices with the same key are loaded
    instead of solved, and any other is solved again.
    Returns this rank's eigenpairs in ascending order and per-slice records."""
    if slices <= 1:
        cuts, counts = [(job.lowfreq, job.upfreq)], [None]
    else:
        saved = ckpt + "_slices.json" if ckpt else None
        cc = None
        if grp.rank == 0 and resume and saved and os.path.exists(saved):
            with open(saved) as f:
                cs = json.load(f)
            if cs.get("settings") == settings and cs.get("slices") == slices:
                cc = ([tuple(c) for c in cs["cuts"]], cs["counts"])
            else:
                print(f" {saved} was saved for other settings: the slices are cut again", file=out)
        if grp.rank == 0 and cc is None:
            cc = sv.slice_spectrum(job.lowfreq, job.upfreq, slices)
            cc = ([tuple(map(float, c)) for c in cc[0]], [float(x) for x in cc[1]])
            if saved:
                _write_json(saved, {"settings": settings, "slices": slices, "cuts": cc[0], "counts": cc[1]})
        cuts, counts = grp.bcast(cc if grp.rank == 0 else None)
        print(" spectrum slices (mHz) and estimated eigenvalue counts:", file=out)
        for j, ((a, b), c) in enumerate(zip(cuts, counts)):
            print(f"   {a:.9f} {b:.9f} {c:10.1f}   rank {j % grp.size}", file=out)
    mine = [j for j in range(len(cuts)) if j % grp.size == grp.rank]
    rs = []
    for j in mine:
        path = f"{ckpt}_slice{j}.npz" if ckpt else None
        key = json.dumps({"settings": settings, "slice": [float(cuts[j][0]), float(cuts[j][1])]})
        if resume and path and os.path.exists(path):
            r = _load_slice(path, key)
            if r is not None:
                rs.append(r)
                print(f" slice {j}: resumed from {path}", file=out)
                continue
            print(f" slice {j}: {path} was saved for another slice or other settings: solved again", file=out)
        if len(cuts) == 1:
            r = sv.solve(job.lowfreq, job.upfreq, want_vectors=True, unscale=True, block=block)
        else:
            r = sv.solve_batched([cuts[j]], want_vectors=True, unscale=True, block=block)[0]
        if path:
            _save_slice(path, r, key)
        rs.append(r)
    if rs:
        lam = np.concatenate([r.lam for r in rs])
        err = np.concatenate([r.err_ref for r in rs])
        res2 = np.concatenate([r.res2 for r in rs])
        vs = [r.vec for r in rs if r.vec is not None and r.vec.size]
        vec = np.concatenate(vs, axis=1) if vs else np.zeros((0, 0))
    else:
        lam = err = res2 = np.zeros(0)
        vec = np.zeros((0, 0))
    order = np.argsort(lam, kind="stable")
    meta = [{"slice": j, "rank": grp.rank, "f_lo_mhz": float(cuts[j][0]), "f_hi_mhz": float(cuts[j][1]),
             "estimated_count": None if counts[j] is None else float(counts[j]), "nev": int(len(r.lam)),
             "xintv": [float(x) for x in r.xintv], "filter_degree": int(r.pol_deg),
             "lanczos_steps": int(r.lanczos_steps), "times_s": {k: float(v) for k, v in r.times.items()},
             "operator_counts": {k: _num(v) for k, v in r.counts.items()}}
            for j, r in zip(mine, rs)]
    return lam[order], err[order], res2[order], vec[:, order] if vec.size else vec, meta


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
        slices: int = 0, group: Group | None = None, checkpoint: bool = False, resume: bool = False) -> dict:
    """One job.  Under torchrun every rank holds the whole operator on its
    GPU and solves every size-th slice (at least one slice per rank); the
    first rank prints, writes the node lists and the run record, and every
    rank writes its own eigenvectors under their indices in the global
    ascending order."""
    grp = group or Group()
    lead = grp.rank == 0
    say = out if lead else io.StringIO()
    log = PhaseLog(job, lead and not dry_run)
    try:
        return _run(job, mixed, block, dry_run, out, say, slices, grp, lead, checkpoint, resume, log)
    finally:
        log.close()


def _run(job, mixed, block, dry_run, out, say, slices, grp, lead, checkpoint, resume, log) -> dict:
    from .model import Model, write_vector
    log.phase("Starting main program")
    log.phase("Loading the mesh and models")
    model = Model.load(job.base_path, job.porder, gravity=job.gravity, assemble=False)
    log.stamp()
    log.phase("Creating matrix")
    model.assemble()
    log.stamp()
    info = model.info()
    print(f" JOB = {job.job}{'  (reference gravity)' if job.gravity else ''}", file=say)
    print(f" mesh name: {job.basename}   polynomial order {job.porder}", file=say)
    print(f" input directory: {job.inputdir}   output directory: {job.outputdir}", file=say)
    print(f" lower / upper frequency in mHz {job.lowfreq} {job.upfreq}", file=say)
    print(f" {info.ntet} tetrahedra ({info.n_fluid_tets} fluid), {info.n} displacement and {info.np} pressure DOFs",
          file=say)
    summary = {"ntet": info.ntet, "n": info.n, "np": info.np, "gravity": job.gravity, "ranks": grp.size}
    if dry_run:
        return summary
    if block is None:
        block = 32 if mixed else 0
    if grp.size > 1:
        slices = max(slices, grp.size)
    # the result-file prefix (the first rank writes the node lists)
    prefix = None
    if lead:
        os.makedirs(job.outputdir or ".", exist_ok=True)
        prefix = model.write_results(job.outputdir, job.basename, job.lowfreq, job.upfreq, np.zeros((info.n, 0)),
                                     job=job.job, nproc=1)
    prefix = grp.bcast(prefix)
    ckpt = prefix + "_ckpt" if (checkpoint or resume) else None
    log.phase("Setting up the GPU operators")
    with make_solver(model.operators(), job.porder, mixed, device=grp.local) as sv:
        log.stamp()
        log.phase("solve the eigenvalue problem")
        settings = json.dumps({"base": job.base_path, "pOrder": job.porder, "JOB": job.job,
                               "lowfreq": job.lowfreq, "upfreq": job.upfreq, "precision": "mixed" if mixed else "fp64",
                               "block": block, "n": info.n, "np": info.np, "ntet": info.ntet})
        lam, err, res2, vec, meta = _solve(sv, job, block, slices, say, grp, ckpt, resume, settings)
        log.stamp()
    # global ascending order: the first rank ranks every eigenvalue, each
    # rank learns the file indices of its own
    parts = grp.gather((lam, err, res2, meta))
    index = None
    if lead:
        L = np.concatenate([p[0] for p in parts])
        order = np.argsort(L, kind="stable")
        pos = np.empty(len(L), dtype=np.int64)
        pos[order] = np.arange(len(L))
        bounds = np.cumsum([0] + [len(p[0]) for p in parts])
        index = [pos[bounds[r]:bounds[r + 1]].tolist() for r in range(grp.size)]
        glam = L[order]
        gerr = np.concatenate([p[1] for p in parts])[order]
        gres2 = np.concatenate([p[2] for p in parts])[order]
        gmeta = sorted((m for p in parts for m in p[3]), key=lambda m: m["slice"])
        report(glam, gerr, out=out)
    index = grp.bcast(index)
    log.phase("save eigenvectors")
    for k, i in enumerate(index[grp.rank]):
        write_vector(f"{prefix}_{i + 1}.dat", vec[:, k])
    grp.gather(None)  # every rank's files are written
    if not lead:
        return dict(summary, nev_local=len(lam), prefix=prefix)
    print(" save eigenvectors: " + prefix + "_<i>.dat", file=out)
    with open(prefix + "_run.json", "w") as f:
        json.dump(dict(run_record(job, model, mixed, block, glam, gerr, gres2, gmeta), ranks=grp.size), f, indent=1)
    print(" run record: " + prefix + "_run.json", file=out)
    log.stamp()
    log.phase("finalize everything")
    log.stamp()
    summary.update(nev=len(glam), prefix=prefix, lam=glam)
    return summary


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="NormalModes job on the GPU")
    ap.add_argument("conf", nargs="?", default="global_conf")
    ap.add_argument("--mixed", action="store_true", help="mixed-precision block path")
    ap.add_argument("--block", type=int, default=None, help="0: single-vector, 32: block (default by precision)")
    ap.add_argument("--dry-run", action="store_true", help="read, load and assemble only")
    ap.add_argument("--slices", type=int, default=0,
                    help="solve N slices of equal estimated eigenvalue count on one context")
    ap.add_argument("--checkpoint", action="store_true", help="save every solved slice beside the results")
    ap.add_argument("--resume", action="store_true", help="load the slices an earlier run saved")
    a = ap.parse_args(argv)
    try:
        job = read_global_conf(a.conf)
    except ConfError as e:
        print(e, file=sys.stderr)
        return 2
    grp = Group()
    try:
        run(job, mixed=a.mixed, block=a.block, dry_run=a.dry_run, slices=a.slices, group=grp,
            checkpoint=a.checkpoint, resume=a.resume)
    finally:
        grp.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
