"""The C++ drop-in header: build the README example against the library and run it."""
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
