"""The C++ drop-in header: build the examples against the library and run them."""
import os
import re
import subprocess

import pytest

from qudrip_gb300 import _capi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu


def test_cpp_spin_example(tmp_path, golden):
    A.lib()  # the library must exist
    exe = str(tmp_path / "spin")
    libdir = os.path.dirname(A.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(ROOT, "examples", "spin.cpp"),
                    "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lqudrip_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    out = subprocess.run([exe, "16"], check=True, capture_output=True, text=True).stdout
    assert "dimension of Hil space = 12870" in out
    assert "nnz = 102960" in out
    ritz = float(re.search(r"ritz = (\S+)", out).group(1))
    E = float(re.search(r"E = (\S+)", out).group(1))
    exact = golden["xy_open_closed_form"]["16"]
    assert abs(ritz - exact) <= 1e-12 * abs(exact)
    assert abs(E - exact) <= 1e-6 * abs(exact)  # raw psi.eval carries the Ritz-vector norm defect


def test_cpp_hubbard_observables_example(tmp_path):
    """Hermitian::LanczosSolver, Arnoldi evolve and McManager through the C++ header."""
    import numpy as np
    import oracle as O
    from qudrip_gb300 import chains
    A.lib()
    exe = str(tmp_path / "hubbard_obs")
    libdir = os.path.dirname(A.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(ROOT, "examples", "hubbard_obs.cpp"),
                    "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lqudrip_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    assert "dim = 36" in out
    spec, ham = chains.hubbard_chain(4, 2, 2, 4.0, -1.0, periodic=True)
    exact = np.linalg.eigvalsh(O.Ham(O.Sector(spec), ham).scipy().toarray())[0]
    E0 = float(re.search(r"E0 = (\S+)", out).group(1))
    assert abs(E0 - exact) <= 1e-10 * abs(exact)
    docc = [float(v) for v in re.findall(r"docc0\(\d\) = (\S+)", out)]
    assert len(docc) == 6 and 0.0 < docc[0] < 1.0
    # an eigenstate is stationary: the double occupancy stays put under evolve
    assert max(abs(d - docc[0]) for d in docc) < 1e-9
