"""The C++ drop-in classes (include/gridfft_gb300.hpp) used the way recon_lib
uses gridFFT, compiled with g++ against libmrg.so and checked against the oracle."""
import os
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT
from tests.helpers import case, rel

pytestmark = pytest.mark.gpu


def test_cxx_gridfft_dropin(mrg_lib, oracle_lib, tmp_path):
    N, C = 32, 3
    c = case(N=N, C=C, nproj=600)
    M = c["kx"].size
    for k in ("kx", "ky", "kz", "kw"):
        c[k].astype(np.float32).tofile(tmp_path / (k + ".bin"))
    c["X"].astype(np.complex64).tofile(tmp_path / "X.bin")
    c["smaps"].astype(np.complex64).tofile(tmp_path / "smaps.bin")
    exe = tmp_path / "shim_demo"
    lib = os.path.join(ROOT, "mri_recon_gb300", "_lib")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "shim_demo.cpp"), "-L", lib, "-lmrg",
                    "-Wl,-rpath," + lib, "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), str(tmp_path), str(N), str(C), str(M)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "caught: mrg:" in r.stdout
    O = oracle_lib.Plan(N, prec=1)
    fr = [dict(kx=c["kx"], ky=c["ky"], kz=c["kz"], kw=c["kw"], data=c["data"])]
    lhs1 = np.fromfile(tmp_path / "lhs_percoil.bin", np.complex64).reshape(N, N, N)
    assert rel(lhs1, O.normal(fr, c["smaps"], 0, c["X"])) < 1e-5
    # gridFFT_CoilThreaded: overgrid 1.375 by default (S = 48 at N = 32) and FFTs without the
    # 1/sqrt(S) per axis, so E is sqrt(Sx Sy Sz) and E^H E Sx Sy Sz times gridFFT's
    assert "coil-threaded: overgrid=1.375 S=48 48 48" in r.stdout
    O2 = oracle_lib.Plan(N, overgrid=1.375, prec=1)
    f = np.sqrt(float(np.prod(O2.gshape)))
    lhs2 = np.fromfile(tmp_path / "lhs_batched.bin", np.complex64).reshape(N, N, N)
    assert rel(lhs2, f * f * O2.normal(fr, c["smaps"], 0, c["X"])) < 1e-5
    y = np.fromfile(tmp_path / "y_batched.bin", np.complex64).reshape(C, M)
    refy = np.stack([O2.forward(c["X"], c["smaps"][k], c["kx"], c["ky"], c["kz"], c["kw"]) for k in range(C)])
    assert rel(y, f * refy) < 1e-5
