"""Mixed precision against FP64 on one spectrum slice.

    python -m normalmodes_gb300.compare [--cells 24] [--porder 2] [--lateral 0.02]
                                        [--interval 0.1 1.0] [--fp64-block 32|0] [--gravity]

Solves the interval twice on one GPU: the mixed path (FP32 filter SpMMs,
FP64 Lanczos and Rayleigh-Ritz, block of 32) and the FP64 path (block of 32,
or the single-vector ChebLanNr with --fp64-block 0).  Prints one JSON line:
both counts, the per-eigenpair relative eigenvalue difference
|lam_mixed - lam_fp64| / |lam_fp64| (max, median, and the full list), both
residual norms of both paths, and both solve times with their ratio.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=24)
    ap.add_argument("--porder", type=int, default=2)
    ap.add_argument("--lateral", type=float, default=0.02)
    ap.add_argument("--interval", type=float, nargs=2, default=(0.1, 1.0))
    ap.add_argument("--fp64-block", type=int, default=32)
    ap.add_argument("--polish", type=int, default=0, help="mixed path refinement degree (0: default, <0: off)")
    ap.add_argument("--fp64-lam", default=None, help="eigenvalues of an earlier FP64 solve (.npy) instead of solving")
    ap.add_argument("--save-fp64-lam", default=None, help="write the FP64 eigenvalues to this .npy file")
    ap.add_argument("--save-mixed-lam", default=None, help="write the mixed-path eigenvalues to this .npy file")
    ap.add_argument("--gravity", action="store_true", help="operators with the reference gravity (JOB = 2)")
    ap.add_argument("--inner-tol", type=float, default=0.0,
                    help="mixed path: accuracy of the FP32 filter's inner B^-1 solve (0: 2^-24)")
    ap.add_argument("--resid-tol", type=float, default=0.0, help="mixed path: refinement target err_ref (0: 1e-10)")
    ap.add_argument("--refine-sweeps", type=int, default=0)
    ap.add_argument("--refine-maxdeg", type=int, default=0)
    ap.add_argument("--refine-band", type=float, default=0.0)
    ap.add_argument("--refine-purge", type=int, default=0, help="0 auto, 1 every block, -1 none")
    ap.add_argument("--refine-guard", type=float, default=0.0, help="guard range factor g (0: 1.5; <= 1: none)")
    ap.add_argument("--refine-growth", type=float, default=0.0, help="near passes: growth bound (0: 1e3)")
    ap.add_argument("--refine-near", type=float, default=0.0,
                    help="later passes: band from this x the top guarded Ritz value (0: 1.05; < 0: band passes)")
    ap.add_argument("--skip-fp64", action="store_true", help="mixed path only (no comparison)")
    ap.add_argument("--mixed-lam", default=None,
                    help="eigenvalues of an earlier mixed solve (.npy): run the FP64 solve only and compare")
    ap.add_argument("--orth", type=int, default=0,
                    help="mixed Gram-Schmidt: 0 tensor-core projection, 1 FP64, 2 cuBLAS SGEMM")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args(argv)
    from normalmodes_gb300.model import Model
    from normalmodes_gb300.nmgpu import NM_PREC_FP64, NM_PREC_MIXED, Solver
    kw = dict(n_cells=a.cells, porder=a.porder)
    if a.lateral > 0:
        kw.update(lateral_pert=a.lateral, lateral_lmax=8)
    mats = Model.ball(gravity=a.gravity, **kw).operators()
    lo, hi = a.interval
    out = {"cells": a.cells, "porder": a.porder, "lateral": a.lateral, "interval_mhz": [lo, hi], "polish": a.polish,
           "gravity": a.gravity, "inner_tol": a.inner_tol, "resid_tol": a.resid_tol,
           "refine_sweeps": a.refine_sweeps, "refine_maxdeg": a.refine_maxdeg, "refine_band": a.refine_band, "refine_purge": a.refine_purge,
           "refine_guard": a.refine_guard, "refine_near": a.refine_near,
           "refine_growth": a.refine_growth}
    res = {}
    runs = ([] if a.mixed_lam else [("mixed", NM_PREC_MIXED, 32)]) + \
        ([] if (a.fp64_lam or a.skip_fp64) else [("fp64", NM_PREC_FP64, a.fp64_block)])
    for name, prec, block in runs:
        with Solver(mats, a.porder, precision=prec, inner_tol=a.inner_tol, verbose=a.verbose, orth=a.orth) as sv:
            t = time.perf_counter()
            kw = dict(polish=a.polish, resid_tol=a.resid_tol, refine_sweeps=a.refine_sweeps,
                      refine_maxdeg=a.refine_maxdeg, refine_band=a.refine_band,
                      refine_purge=a.refine_purge, refine_guard=a.refine_guard,
                      refine_near=a.refine_near, refine_growth=a.refine_growth) if name == "mixed" else {}
            r = sv.solve(lo, hi, block=block, want_vectors=False, **kw)
            dt = time.perf_counter() - t
        res[name] = r
        out[name] = {"nev": len(r.lam), "seconds": round(dt, 3), "block": block, "lanczos_vectors": r.lanczos_steps,
                     "filter_degree": r.pol_deg, "times_s": {k: round(v, 3) for k, v in r.times.items()},
                     "err_ref_max": float(r.err_ref.max()) if len(r.lam) else None,
                     "err_ref_median": float(np.median(r.err_ref)) if len(r.lam) else None,
                     "res2_max": float(r.res2.max()) if len(r.lam) else None,
                     "res2_median": float(np.median(r.res2)) if len(r.lam) else None,
                     "gated_1e-10": int((r.err_ref <= 1e-10).sum()),
                     "refinement": {k: r.counts[k] for k in ("refine_passes", "refine_blocks", "refine_maxdeg",
                                                             "refine_steps", "res2_before_refine",
                                                             "refine_guards")}}
    m = np.load(a.mixed_lam) if a.mixed_lam else res["mixed"].lam
    if a.save_mixed_lam and "mixed" in res:
        np.save(a.save_mixed_lam, res["mixed"].lam)
    if a.skip_fp64 and not a.fp64_lam:
        print(json.dumps(out))
        return
    f = np.load(a.fp64_lam) if a.fp64_lam else res["fp64"].lam
    if a.save_fp64_lam and "fp64" in res:
        np.save(a.save_fp64_lam, f)
    out["same_count"] = len(m) == len(f)
    if len(m) == len(f) and len(f):
        rel = np.abs(m - f) / np.abs(f)
        out["eig_rel_diff_max"] = float(rel.max())
        out["eig_rel_diff_median"] = float(np.median(rel))
        out["eig_rel_diff"] = [float(x) for x in rel]
    if "fp64" in out and "mixed" in out:
        out["speedup_mixed_over_fp64"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
    print(json.dumps(out))


if __name__ == "__main__":
    main()
