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


@pytest.mark.parametrize("matrix_sum", [0, 1])
def test_cpp_lattice_model_example(tmp_path, matrix_sum):
    """Lattice<2> / Model / params_type / param_finder / McManager.outFile through the C++ headers
    (the way programs/two_liquid_sq.cpp drives a 2D model), against the Python lattice path."""
    import numpy as np
    A.lib()
    exe = str(tmp_path / "heisenberg_2d")
    libdir = os.path.dirname(A.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(ROOT, "examples", "heisenberg_2d.cpp"),
                    "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lqudrip_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    pf = tmp_path / "params.txt"
    pf.write_text(f"# 4x4 periodic Heisenberg\nNx = 4\nNy = 4\nJ = 1\nJz = 1\nkrylov = 100\n"
                  f"matrix_sum = {matrix_sum}\n")
    tsv = tmp_path / "szsz.tsv"
    out = subprocess.run([exe, str(pf), str(tsv)], check=True, capture_output=True, text=True).stdout
    assert "sites = 16 dim = 12870" in out and "bonds = 32" in out
    E0 = float(re.search(r"E0 = (\S+)", out).group(1))
    assert abs(E0 - (-11.228483208428855)) < 1e-8
    rows = tsv.read_text().split("\n")
    assert rows[0] == "#time\tindex\tSzSz"
    vals = [float(r.split("\t")[2]) for r in rows[1:17]]
    assert abs(vals[0] - 0.25) < 1e-6  # (S^z_0)^2 on the Ritz vector (norm 1 to ~1e-8)
    assert abs(sum(vals)) < 1e-5  # total S^z = 0 (the table has 6 decimals)
    szsz01 = float(re.search(r"SzSz\(0,1\) = (\S+)", out).group(1))
    assert abs(szsz01 - vals[1]) < 1e-6 and abs(szsz01 - E0 / 96) < 1e-6  # 32 equivalent bonds x 3 components
    assert np.isfinite(vals).all()
