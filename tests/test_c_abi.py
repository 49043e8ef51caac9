"""The C-ABI from C: tests/c/abi_client.c is compiled against
include/nmgpu.h and linked against libnmgpu.so as a host program would be,
then run (host-side entry points; without a GPU, nm_create's failure)."""
import os
import shutil
import subprocess

import pytest

from tests.conftest import gpu_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_client(tmp_path):
    from normalmodes_gb300 import nmgpu
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    lib = nmgpu.lib_path()
    nmgpu.lib()  # builds the library if this is a fresh tree
    exe = str(tmp_path / "abi_client")
    libdir = os.path.dirname(lib)
    subprocess.run(["gcc", "-std=c11", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "abi_client.c"), "-o", exe, "-L", libdir, "-lnmgpu",
                    f"-Wl,-rpath,{libdir}", "-lm"], check=True, capture_output=True)
    args = [exe] if gpu_available() else [exe, "nogpu"]
    r = subprocess.run(args, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "OK"
