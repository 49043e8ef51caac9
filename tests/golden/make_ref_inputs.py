"""Copy the reference's P1 demo model inputs that the tests use into
tests/golden/ref_inputs/ (run once where the reference is checked out).

    python tests/golden/make_ref_inputs.py [/path/to/NormalModes/demos]

The files are the reference's own binary inputs (src/mod_para.f90:286-316
names them): `<base>_mesh.header` (text "Ntet Nvert"), `_ele.dat` (int32
Ntet x 4, 1-based), `_node.dat` (float64 Nvert x 3, km), `_neigh.dat`
(int32 Ntet x 4, -1 = boundary), `_{vp,vs,rho}_pod_1_true.dat` (float64
Ntet x 4) and `_pod_1_potential_acceleration_true.dat` (float64 Ntet x 4 x 3,
the JOB = 2 gravity).  Only the pOrder = 1 files of CONST3k (homogeneous,
solid) and PREM3k (fluid outer core) are copied, with the demo global_conf.
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "ref_inputs")
MODELS = {"CONST3k": "CONST_1L_3k.1", "PREM3k": "prem_3L_3k.1"}
SUFFIXES = ["_mesh.header", "_ele.dat", "_node.dat", "_neigh.dat", "_vp_pod_1_true.dat", "_vs_pod_1_true.dat",
            "_rho_pod_1_true.dat", "_pod_1_potential_acceleration_true.dat"]


def main(demos: str) -> None:
    for d, base in MODELS.items():
        os.makedirs(os.path.join(OUT, d), exist_ok=True)
        for s in SUFFIXES:
            src = os.path.join(demos, "models", "input", d, base + s)
            shutil.copyfile(src, os.path.join(OUT, d, base + s))
    shutil.copyfile(os.path.join(demos, "global_conf"), os.path.join(OUT, "global_conf"))
    print("copied to", OUT)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/demos")
