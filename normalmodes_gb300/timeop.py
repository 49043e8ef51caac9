"""Time the eigensolver's operators on a synthetic layered ball.

    python -m normalmodes_gb300.timeop [--cells 36] [--porder 2] [--lateral 0]
                                       [--precision mixed|fp64] [--ops 4,5,6] [--reps 5] [--gravity]

Operators (nm_time_op): 0 A-op, 1 B SpMV, 2 B Chebyshev solve, 3 one filter
degree step (single vector, FP64 SELL); 4 block mass Chebyshev solve, 5
block A-op, 6 one block filter degree step (32 columns, in the context's
precision).  Prints one JSON line: per operator the mean milliseconds, the
algorithmic GB/s and the kernel launches per application.  Also the command
the kernel profiles are taken with (one small case under ncu).
"""
from __future__ import annotations

import argparse
import json
import time


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=36)
    ap.add_argument("--porder", type=int, default=2)
    ap.add_argument("--lateral", type=float, default=0.0)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--ops", default="4,5,6")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--gravity", action="store_true", help="operators with the reference gravity (JOB = 2)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--verbose", action="store_true", help="print every autotuner candidate's time")
    ap.add_argument("--inner-tol", type=float, default=0.0, help="accuracy of the FP32 inner B^-1 solve")
    ap.add_argument("--shape", action="append", default=[],
                    help="pin a launch shape instead of autotuning: KIND:VEC,THREADS,SWEEP with KIND mass|ap|aop "
                         "(e.g. mass:0,1024,1); repeatable")
    a = ap.parse_args(argv)
    from normalmodes_gb300.model import Model
    from normalmodes_gb300.nmgpu import NM_PREC_FP64, NM_PREC_MIXED, Solver
    kw = dict(n_cells=a.cells, porder=a.porder)
    if a.lateral > 0:
        kw.update(lateral_pert=a.lateral, lateral_lmax=8)
    t = time.perf_counter()
    m = Model.ball(gravity=a.gravity, **kw)
    mats = m.operators()
    t_model = time.perf_counter() - t
    with Solver(mats, a.porder, precision=NM_PREC_MIXED if a.precision == "mixed" else NM_PREC_FP64,
                autotune=-1 if a.no_autotune else 0, verbose=a.verbose, inner_tol=a.inner_tol) as sv:
        if a.shape:
            from normalmodes_gb300.nmgpu import lib
            kinds = {"mass": 0, "ap": 1, "aop": 2}
            for spec in a.shape:  # before the first block use, so the autotuner does not run
                k, v = spec.split(":")
                vec, thr, sw = (int(x) for x in v.split(","))
                sv._check(lib().nm_test_gather_shape(sv._h, kinds[k], vec, thr, sw))
        info = sv.info()
        out = {"cells": a.cells, "porder": a.porder, "n": info.n, "np": info.np, "precision": a.precision,
               "model_s": round(t_model, 2)}
        for w in (int(x) for x in a.ops.split(",")):
            ms, by, la = sv.time_op(w, a.reps)
            out[str(w)] = {"ms": round(ms, 4), "GBs": round(by / ms / 1e6, 1), "launches": la,
                           "bytes": by}
        i2 = sv.info()
        out["autotuned"] = {"mass_vec": i2.mass_vec, "mass_threads": i2.mass_threads, "mass_sweep": i2.mass_sweep,
                            "ap_vec": i2.ap_vec, "ap_threads": i2.ap_threads, "ap_sweep": i2.ap_sweep,
                            "aop_threads": i2.aop_threads, "aop_sweep": i2.aop_sweep}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
