"""CPU tests of the job driver (python -m normalmodes_gb300.run): the
reference's global_conf rules (src/mod_para.f90:79-137, src/mod_string.f90),
dry runs over models in the reference's input files with and without the
reference gravity, and whole jobs, single-interval and sliced, whose GPU
context is replaced by the oracle (the printed tables and the result
files)."""
import io
import json
import os

import numpy as np
import pytest

from normalmodes_gb300 import run as R

# committed copies of the reference's CONST3k / PREM3k P1 inputs and demo
# global_conf (tests/golden/make_ref_inputs.py)
REF_DEMO = os.environ.get("NM_REFERENCE_DEMOS",
                          os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_inputs"))


def _write_conf(path, **kv):
    lines = ["# JOB: normal modes modelling", "# 1 without gravity, 2 with reference gravity"]
    for k, v in kv.items():
        lines.append(f"{k:<11} = {v}   # comment")
    path.write_text("\n".join(lines) + "\n")
    return str(path)


def test_reference_demo_configurations():
    conf = os.path.join(REF_DEMO, "global_conf")
    if not os.path.exists(conf):  # a full demos/models/input checkout keeps it two levels up
        conf = os.path.join(os.path.dirname(os.path.dirname(REF_DEMO)), "global_conf")
    if not os.path.exists(conf):
        pytest.skip("reference demos not present")
    j = R.read_global_conf(conf)
    assert (j.job, j.basename, j.inputdir, j.outputdir, j.porder) == (
        1, "CONST_1L_3k.1", "models/input/CONST3k/", "models/output/CONST3k/", 1)
    assert j.lowfreq == float(np.float32(0.2)) and j.upfreq == 2.0 and not j.gravity


def test_configuration_rules(tmp_path):
    p = tmp_path / "global_conf"
    p.write_text("\n".join([
        "# a comment line",
        "JOB=2",
        "JOB = 1          # the first line of a key wins",
        "basename\tball.1",
        "#basename = other",
        "inputdir   = in/   # trailing comment",
        "outputdir  = out/",
        "lowfreq = 0.1 # mHz",
        "upfreq  = 1.0",
        "pOrder  = 2",
    ]) + "\n")
    j = R.read_global_conf(str(p))
    assert (j.job, j.basename, j.inputdir, j.outputdir, j.porder) == (2, "ball.1", "in/", "out/", 2)
    assert j.lowfreq == float(np.float32(0.1)) and j.gravity and j.base_path == "in/ball.1"
    base = dict(JOB=1, basename="b", inputdir="i/", outputdir="o/", lowfreq=0.1, upfreq=1.0, pOrder=1)
    for bad, msg in ((dict(lowfreq=1.0), "frequencies"), (dict(JOB=20), "not supported"),
                     (dict(pOrder=3), "pOrder")):
        with pytest.raises(R.ConfError, match=msg):
            R.read_global_conf(_write_conf(tmp_path / "c", **{**base, **bad}))
    kv = dict(base)
    del kv["outputdir"]
    with pytest.raises(R.ConfError, match="there is no outputdir"):
        R.read_global_conf(_write_conf(tmp_path / "c", **kv))
    with pytest.raises(R.ConfError, match="does not exist"):
        R.read_global_conf(str(tmp_path / "missing"))
    assert R.main([str(tmp_path / "missing")]) == 2


def _job_files(tmp_path, job, porder=1, **ball):
    from normalmodes_gb300.model import Model
    from tests.test_gravity import _write_reference_files
    src = Model.ball(n_cells=6, porder=porder, fluid_core=0, gravity=True, assemble=False, **ball)
    inp = tmp_path / "input"
    inp.mkdir(exist_ok=True)
    base = _write_reference_files(src, str(inp), "ball.1", porder)
    src.gravity().astype(np.float64).tofile(base + f"_pod_{porder}_potential_acceleration_true.dat")
    return _write_conf(tmp_path / "global_conf", JOB=job, basename="ball.1", inputdir=str(inp) + "/",
                       outputdir=str(tmp_path / "output") + "/", lowfreq=0.1, upfreq=1.0, pOrder=porder)


@pytest.mark.parametrize("job", [1, 2])
def test_dry_run(tmp_path, job):
    conf = _job_files(tmp_path, job)
    out = io.StringIO()
    s = R.run(R.read_global_conf(conf), dry_run=True, out=out)
    assert s["gravity"] == (job == 2) and s["n"] > 0 and s["ntet"] == 1296
    assert "reference gravity" in out.getvalue() or job == 1


class _OracleSolver:
    """Stand-in for the GPU context: the oracle's solve, unscaled vectors."""

    def __init__(self, mats, porder, mixed, device=0):
        from oracle import oracle as O
        self.O, self.op = O, O.setup_operator(mats, porder)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False

    def solve(self, lo, hi, want_vectors, unscale, block):
        from types import SimpleNamespace
        r = self.O.apply_pevsl(self.op, lo, hi)
        return SimpleNamespace(lam=r.lam, vec=r.Y * self.op.D[:, None] if unscale else r.Y, err_ref=r.err_ref,
                               res2=r.res2, xintv=tuple(r.xintv), pol_deg=r.pol.deg, lanczos_steps=r.steps,
                               times=dict(r.times), counts={"amv": self.op.nmatvec["A"]})

    def slice_spectrum(self, lo, hi, n):
        from normalmodes_gb300 import nmgpu
        op = self.op
        lmin, lmax, _ = self.O.lan_bounds(op.amv, op.n, 3000, 1e-5, solve=op.bsolve)
        lmax += 0.005 * (lmax - lmin)
        lam = [float(np.float32(f)) for f in (lo, hi)]
        lam = [(2 * self.O.PI_REF * f) ** 2 * 1e-6 for f in lam]
        deg = nmgpu.kpm_degree(lmin, lmax, lam[0], lam[1], n)

        def apply(X):
            return np.stack([op.bsolve(op.amv(X[:, j])) for j in range(X.shape[1])], axis=1)

        mu = nmgpu.kpm_moments(apply, op.n, lmin, lmax, deg, nvec=8)
        return nmgpu.kpm_slices(mu, op.n, lmin, lmax, lo, hi, n)

    def solve_batched(self, cuts, want_vectors, unscale, block):
        return [self.solve(a, b, want_vectors, unscale, block) for a, b in cuts]


def test_whole_job_with_a_stand_in_solver(tmp_path, monkeypatch):
    from oracle import oracle as O
    conf = _job_files(tmp_path, 2)
    monkeypatch.setattr(R, "make_solver", _OracleSolver)
    out = io.StringIO()
    s = R.run(R.read_global_conf(conf), out=out)
    text = out.getvalue()
    assert s["nev"] > 0
    f, T = O.freq_mhz(s["lam"])
    rows = [ln.split() for ln in text.splitlines() if ln.strip().startswith("Row") and "err." not in ln]
    assert len(rows) == s["nev"]
    assert np.allclose([float(r[2]) for r in rows], f, rtol=1e-12)
    assert np.allclose([float(r[3]) for r in rows], T, rtol=1e-12)
    prefix = s["prefix"]
    assert os.path.basename(prefix).startswith("ball.1_JOB2_pod1_np1_")
    vec1 = np.fromfile(prefix + "_1.dat")
    assert vec1.size == s["n"]
    assert os.path.exists(str(tmp_path / "output" / "ball.1_pod1_np1_vlist.dat"))
    assert not os.path.exists(prefix + f"_{s['nev'] + 1}.dat")
    import json
    rec = json.load(open(prefix + "_run.json"))
    assert rec["config"]["JOB"] == 2 and rec["model"]["gravity"] and rec["model"]["n"] == s["n"]
    assert np.allclose(rec["eigenpairs"]["lambda"], s["lam"]) and np.allclose(rec["eigenpairs"]["f_mhz"], f)
    sl = rec["solver"]["slices"]
    assert len(sl) == 1 and sl[0]["nev"] == s["nev"] and sl[0]["filter_degree"] > 0
    # the reference's run log (src/mod_utility.f90:39-148)
    log = open(str(tmp_path / "output" / "ball.1_0.log")).read().splitlines()
    assert log[0] == "  Start program at time elapsed = 0.0 second."
    assert log[1] == "   1. Starting main program"
    phases = [ln[6:] for ln in log if ln[:4].strip().isdigit() and ln[4:6] == ". "]
    assert phases[-3:] == ["solve the eigenvalue problem", "save eigenvectors", "finalize everything"]
    assert sum("Time elapsed" in ln for ln in log) >= 5


def test_sliced_job_matches_the_single_interval(tmp_path, monkeypatch):
    """--slices: KPM slices solved one after another and merged give the
    eigenvalues of the single-interval solve."""
    conf = _job_files(tmp_path, 2)
    monkeypatch.setattr(R, "make_solver", _OracleSolver)
    whole = R.run(R.read_global_conf(conf), out=io.StringIO())
    out = io.StringIO()
    sliced = R.run(R.read_global_conf(conf), out=out, slices=3)
    assert "spectrum slices" in out.getvalue()
    assert sliced["nev"] == whole["nev"]
    assert np.max(np.abs(sliced["lam"] - whole["lam"]) / whole["lam"]) < 1e-10
    assert np.all(np.diff(sliced["lam"]) >= 0)


def _dist_rank(rank, ws, port, conf, q):
    import sys as _sys
    _sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    from normalmodes_gb300 import run as RR
    from tests.test_run import _OracleSolver as Stand
    RR.make_solver = Stand
    grp = RR.Group()
    try:
        s = RR.run(RR.read_global_conf(conf), out=io.StringIO(), slices=3, group=grp)
        q.put((rank, {k: (v.tolist() if isinstance(v, np.ndarray) else v) for k, v in s.items()}))
    finally:
        grp.close()


def test_slices_across_two_ranks(tmp_path, monkeypatch):
    """torchrun form (one GPU per rank, operator replicated, slices shared
    out, here two gloo ranks with the oracle standing in for the GPU): the
    eigenvalues and eigenvector files are those of the single-rank job, each
    vector written once under its global index."""
    import torch.multiprocessing as mp
    conf = _job_files(tmp_path, 2)
    monkeypatch.setattr(R, "make_solver", _OracleSolver)
    whole = R.run(R.read_global_conf(conf), out=io.StringIO())
    ref_files = {i: np.fromfile(f"{whole['prefix']}_{i + 1}.dat") for i in range(whole["nev"])}
    for i in range(whole["nev"]):
        os.remove(f"{whole['prefix']}_{i + 1}.dat")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29600 + os.getpid() % 1000
    procs = [ctx.Process(target=_dist_rank, args=(r, 2, port, conf, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    lead = out[0]
    assert lead["ranks"] == 2 and lead["nev"] == whole["nev"]
    assert out[0]["prefix"] == out[1]["prefix"] == whole["prefix"]
    assert np.max(np.abs(np.array(lead["lam"]) - whole["lam"]) / whole["lam"]) < 1e-10
    assert 0 < out[1]["nev_local"] < whole["nev"]
    from normalmodes_gb300.model import Model
    m = Model.load(R.read_global_conf(conf).base_path, 1, gravity=True)
    A, B = m.csr("A").to_scipy(), m.csr("B").to_scipy()
    for i in range(whole["nev"]):
        x = np.fromfile(f"{whole['prefix']}_{i + 1}.dat")
        assert x.size == ref_files[i].size
        assert abs((x @ (A @ x)) / (x @ (B @ x)) / whole["lam"][i] - 1) < 1e-9
    assert not os.path.exists(f"{whole['prefix']}_{whole['nev'] + 1}.dat")



def test_checkpoint_and_resume(tmp_path, monkeypatch):
    """--checkpoint saves the slice list and every solved slice; --resume
    loads them and solves only the missing ones, with the same result."""
    conf = _job_files(tmp_path, 2)
    monkeypatch.setattr(R, "make_solver", _OracleSolver)
    first = R.run(R.read_global_conf(conf), out=io.StringIO(), slices=3, checkpoint=True)
    ck = first["prefix"] + "_ckpt"
    assert os.path.exists(ck + "_slices.json")
    assert all(os.path.exists(f"{ck}_slice{j}.npz") for j in range(3))
    os.remove(f"{ck}_slice1.npz")
    solved = []

    class Counting(_OracleSolver):
        def slice_spectrum(self, lo, hi, n):
            raise AssertionError("the slice list must come from the checkpoint")

        def solve_batched(self, cuts, want_vectors, unscale, block):
            solved.extend(cuts)
            return super().solve_batched(cuts, want_vectors, unscale, block)

    monkeypatch.setattr(R, "make_solver", Counting)
    out = io.StringIO()
    again = R.run(R.read_global_conf(conf), out=out, slices=3, resume=True)
    assert len(solved) == 1
    assert out.getvalue().count("resumed from") == 2
    assert again["nev"] == first["nev"]
    assert np.array_equal(again["lam"], first["lam"])


def test_resume_refuses_checkpoints_of_other_settings(tmp_path, monkeypatch):
    """A checkpoint saved with other solver settings (here FP64 against a
    mixed-precision resume) is not merged: the slices are cut again and
    every slice is solved again, with the same result."""
    conf = _job_files(tmp_path, 2)
    monkeypatch.setattr(R, "make_solver", _OracleSolver)
    first = R.run(R.read_global_conf(conf), out=io.StringIO(), slices=3, checkpoint=True)
    ck = first["prefix"] + "_ckpt"
    with open(ck + "_slices.json") as f:
        assert json.load(f)["slices"] == 3
    solved, cut = [], []

    class Counting(_OracleSolver):
        def slice_spectrum(self, lo, hi, n):
            cut.append(n)
            return super().slice_spectrum(lo, hi, n)

        def solve_batched(self, cuts, want_vectors, unscale, block):
            solved.extend(cuts)
            return super().solve_batched(cuts, want_vectors, unscale, block)

    monkeypatch.setattr(R, "make_solver", Counting)
    out = io.StringIO()
    again = R.run(R.read_global_conf(conf), mixed=True, block=0, out=out, slices=3, resume=True)
    assert cut == [3] and len(solved) == 3
    assert "cut again" in out.getvalue() and out.getvalue().count("solved again") == 3
    assert "resumed from" not in out.getvalue()
    assert np.array_equal(again["lam"], first["lam"])
