"""Generate the golden fixtures of tests/golden/ with the CPU FP64 oracle.

    python tests/golden/make_golden.py [name ...]

Each fixture stores, for one seeded synthetic model, the oracle's operator
bounds, the solve interval, the filter, the eigenvalues, the reference-style
RMS residuals and, for the small models, the dense-solver eigenvalues that
pin the oracle independently.  The models are regenerated from their
parameters by the tests (the generator is deterministic).

The reference itself cannot be run here (Fortran/MPI with un-vendored
pEVSL), so these fixtures are the oracle's output, not the reference's.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from normalmodes_gb300.model import Model  # noqa: E402
from oracle import oracle as O  # noqa: E402

SPECS = {
    "solid_p1": dict(model=dict(n_cells=6, porder=1, fluid_core=0), porder=1, interval=(0.2, 1.0), dense=True),
    "fs_p1": dict(model=dict(n_cells=8, porder=1), porder=1, interval=(0.2, 1.0), dense=True),
    "fs_p2": dict(model=dict(n_cells=8, porder=2), porder=2, interval=(0.2, 0.6), dense=False),
    # reference gravity (JOB = 2) of the balls' own density profile
    "solid_p1_grav": dict(model=dict(n_cells=6, porder=1, fluid_core=0, gravity=True), porder=1,
                          interval=(0.1, 1.0), dense=True),
    "fs_p1_grav": dict(model=dict(n_cells=8, porder=1, gravity=True), porder=1, interval=(0.2, 1.0), dense=True),
    # the layered P1 ball of about 10k tetrahedra (jittered) and 0.2-1.0 mHz
    "ball12_p1": dict(model=dict(n_cells=12, porder=1), porder=1, interval=(0.2, 1.0), dense=False),
    # the reference's own demo meshes (P1 inputs copied by make_ref_inputs.py),
    # at the demo global_conf's interval 0.2-2.0 mHz
    "const3k_p1": dict(files="CONST3k/CONST_1L_3k.1", porder=1, interval=(0.2, 2.0), dense=True),
    "prem3k_p1": dict(files="PREM3k/prem_3L_3k.1", porder=1, interval=(0.2, 2.0), dense=True),
}
REF_INPUTS = os.path.join(HERE, "ref_inputs")


def load_model(name: str) -> Model:
    """The model of fixture `name`: a seeded ball, or reference input files."""
    s = SPECS[name]
    if "files" in s:
        return Model.load(os.path.join(REF_INPUTS, s["files"]), s["porder"])
    return Model.ball(**s["model"])


def make(name: str) -> str:
    s = SPECS[name]
    t0 = time.time()
    m = load_model(name)
    mats = m.operators()
    op = O.setup_operator(mats, s["porder"])
    r = O.apply_pevsl(op, *s["interval"])
    out = dict(
        model_kw=repr(s.get("model", s.get("files"))), porder=s["porder"], interval=np.array(s["interval"]),
        b_bounds=np.array(op.bounds["B"]), ap_bounds=np.array(op.bounds.get("Ap", (0.0, 0.0))),
        xintv=np.array(r.xintv, dtype=np.float64), pol_deg=r.pol.deg, pol_bar=r.pol.bar, pol_gam=r.pol.gam,
        lam=r.lam, err_ref=r.err_ref, res2=r.res2, steps=r.steps, n=op.n, np=op.np,
        nnz=np.array([len(v.col) for v in mats.values()]),
    )
    if s["dense"]:
        w, _ = O.dense_reference(op, r.xintv[0], r.xintv[1])
        out["lam_dense"] = w
    path = os.path.join(HERE, f"{name}.npz")
    np.savez(path, **out)
    print(f"{name}: n={op.n} np={op.np} nev={len(r.lam)} deg={r.pol.deg} steps={r.steps} "
          f"{time.time() - t0:.1f}s -> {path}")
    return path


if __name__ == "__main__":
    for nm in (sys.argv[1:] or list(SPECS)):
        make(nm)
