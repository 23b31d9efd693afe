"""Lattice / LatticeFunction / Model / params_type (lattice.hpp), param_finder (find_param.hpp) and
McManager.outFile (mc_manager.hpp:147-196): host-side code, checked on the CPU against hand-derived
answers and between the Python module and the C++ headers (include/qudrip_gpu_lattice.hpp,
include/qudrip_gpu_params.hpp), which are compiled here with g++."""
import cmath
import math
import os
import subprocess

import numpy as np
import pytest

import qudrip_gb300 as q
from qudrip_gb300 import lattice as LT
from qudrip_gb300.params import param_finder, stod, stoi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def square(nx, ny):
    return q.Lattice([(i, j) for i in range(nx) for j in range(ny)], [(nx, 0), (0, ny)])


def test_reciprocal_vectors_and_volume():
    rp, vol = LT.get_reci([(5,)])
    assert vol == 25 and list(rp[0]) == [5]
    rp, vol = LT.get_reci([(4, 0), (0, 3)])
    assert [list(v) for v in rp] == [[-3, 0], [0, -4]] and vol == -12
    rp, vol = LT.get_reci([(2, 0, 0), (0, 3, 0), (1, 0, 4)])
    assert [list(v) for v in rp] == [[12, 0, -3], [0, 8, 0], [0, 0, 6]] and vol == 24


def test_reduce_and_index_follow_cpp_integer_division():
    L = square(4, 3)
    assert L.N() == 12 and L.vol() == -12
    assert list(L.reduce((5, -1))) == [1, 2] and L((5, -1)) == 1 * 3 + 2
    assert list(L.reduce((4, 3))) == [0, 0] and L((4, 3)) == 0
    assert list(L.reduce((-1, 0))) == [3, 0] and L((-1, 0)) == 9
    # an exact negative multiple of the period goes one period too far (the reference's rounding)
    assert list(L.reduce((-4, 0))) == [4, 0] and L((-4, 0)) == L.N()
    assert L(7) is L.coords[7] and list(L(7)) == [2, 1]
    # two_liquid_sq.cpp's bonds: site i to c + a0 and c + a1 with wrap-around
    nbr = [(L(L(i) + np.array([1, 0])), L(L(i) + np.array([0, 1]))) for i in range(L.N())]
    assert nbr[11] == (2, 9) and nbr[0] == (3, 1)
    free = q.Lattice([(0,), (1,), (2,)])
    assert free.vol() == 0 and list(free.reduce((7,))) == [7] and free((7,)) == 3


def test_params_type():
    p = q.params_type()
    assert p("Jx") == 0.0  # created on first use
    p["Jx"] = 1.0
    p["phi"] = 30.0
    p["phi"] = p("phi") * math.pi / 180
    assert p.stringize() == "Jx=1.000000,phi=0.523599;"
    with pytest.raises(KeyError, match="undefined params"):
        p.get("nope")
    assert q.params_type().stringize() == ""


def test_lattice_function_dft():
    L = square(4, 3)
    f = q.LatticeFunction(L)
    k = (1, 2)
    th = [sum(float(int(L(i) @ (k[j] * L.rpvec(j)))) / L.vol() for j in range(2)) for i in range(L.N())]
    for i in range(L.N()):
        f[i] = cmath.exp(-1j * th[i])
    assert abs(f.DFT(k) - 1.0) < 1e-14
    g = q.LatticeFunction(L)
    g.data[:] = 2.5
    assert abs(g.DFT((0, 0)) - 2.5) < 1e-15
    h = q.LatticeFunction(L, argn=2)
    h[(3, 4)] = 1.0
    assert h.data[3 * 12 + 4] == 1.0
    ks = [(1, 0), (0, 1)]
    ph = sum(float(int(L(a) @ (ks[ix][j] * L.rpvec(j)))) / L.vol() for ix, a in enumerate((3, 4)) for j in range(2))
    assert abs(h.DFT_multi(ks) - cmath.exp(1j * ph) / 144) < 1e-15


def xy_bond(gc, ga):
    def f(s1, s2, p):
        return p("J") * (gc(s1) * ga(s2)) + p("J") * (gc(s2) * ga(s1))
    return f


def test_model_emits_the_bond_sum():
    L = square(3, 2)
    m = q.Model(L)
    p = q.params_type()
    p["J"] = 0.5
    for i in range(L.N()):
        m.addBond(i, L(L(i) + np.array([1, 0])), p)
    pre = q.getQbits(L.N())
    gc, ga = q.getBoseGate(pre), q.getBoseGate(pre)
    gc << 0.5 * (q.pauli_x + q.II * q.pauli_y)
    ga << 0.5 * (q.pauli_x - q.II * q.pauli_y)
    ham = m.getHamiltonian(xy_bond(gc, ga))
    ref = q.getEmptyOperator()
    for (a, b) in m.bonds:
        ref = ref + 0.5 * (gc(a) * ga(b)) + 0.5 * (gc(b) * ga(a))
    assert ham.size() == ref.size() == 2 * L.N()
    t1, n1, g1, m1 = ham.pack()
    t2, n2, g2, m2 = ref.pack()
    assert (n1, m1) == (n2, m2)
    assert bytes(t1) == bytes(t2) and bytes(g1) == bytes(g2)  # same terms, gates, coefficients, order
    text = m.describe()
    assert text.startswith("Bonds: \n(0,0) and (1,0): J=0.500000;\n")
    with pytest.raises(IndexError):
        m.addBond(0, L.N(), p)


PARAM_FILE = """# a driver's parameter file
Nx = 4
Ny=3
Jx = 1.5e-1 # trailing text is part of the value once spaces are gone
Jz = 2.75abc
phi = 3.9
name = two liquid
Nx = 9
z = (1.5,-2)
vec = --{vecfile}
cvec = --{cvecfile}
noeq
"""


def write_params(tmp_path):
    vf, cf = tmp_path / "v.txt", tmp_path / "c.txt"
    vf.write_text("# header\n0.5\n# skip\n1.25\n2\n")
    cf.write_text("1 2\n# c\n-3 4.5\n")
    pf = tmp_path / "params.txt"
    pf.write_text(PARAM_FILE.format(vecfile=vf, cvecfile=cf))
    return pf


def test_param_finder(tmp_path):
    pf = param_finder(str(write_params(tmp_path)))
    assert pf.find_param("Nx", 0, type=int) == 4  # the first definition wins
    assert pf.find_param("Ny", 0) == 3
    assert pf.find_param("Jx", 0.0) == 0.15  # "1.5e-1#trailing..." -> stod prefix
    assert pf.find_param("Jz", 0.0) == 2.75
    assert pf.find_param("phi", 0, type=int) == 3  # stoi stops at '.'
    assert pf.find_param("name", "", type=str) == "twoliquid"
    assert pf.find_param("z", 0j, type=complex) == complex(1.5, -2)
    assert pf.find_param("missing", 7.0) == 7.0
    with pytest.raises(KeyError):
        pf.find_param("missing", 7.0, warning=1)
    assert pf.find_param_tvec("vec", [0.0] * 3) == [0.5, 1.25, 2.0]
    assert pf.find_param_tvec("Jz", [0.0] * 2) == [2.75, 2.75]
    assert pf.find_param_tvec("cvec", [0j] * 2, type=complex) == [complex(1, 2), complex(-3, 4.5)]
    assert param_finder(str(tmp_path / "absent.txt")).params == {}
    assert stod("  -1.5e3x") == -1500.0 and stoi("+42.9") == 42
    with pytest.raises(ValueError):
        stod("abc")


def test_outfile_table(tmp_path):
    mc = q.McManager(3, None)
    mc.addObs("E", 1, q.MC_REAL)
    mc.addObs("n", 2)
    mc.addObs("c", 1)
    mc.data["E"][:, 0] = [1.0, 0.5, -0.25]
    mc.data["n"][:] = np.array([[1 + 2j, 3], [0.125j, -1], [2, 2]])
    mc.data["c"][:, 0] = [1j, 2, 3]
    f1 = tmp_path / "e.tsv"
    mc.outFile(0.1, str(f1), ["E", "c"])
    assert f1.read_text() == ("#time\tE\tc(real)\tc(imag)\n"
                              "0.000000\t1.000000\t0.000000\t1.000000\n"
                              "0.100000\t0.500000\t2.000000\t0.000000\n"
                              "0.200000\t-0.250000\t3.000000\t0.000000\n")
    f2 = tmp_path / "n.tsv"
    mc.outFile(0.5, str(f2), ["n"])
    lines = f2.read_text().split("\n")
    assert lines[0] == "#time\tindex\tn(real)\tn(imag)"
    assert lines[1:4] == ["0.000000\t0\t1.000000\t2.000000", "0.000000\t1\t3.000000\t0.000000", ""]
    assert lines[4] == "0.500000\t0\t0.000000\t0.125000"
    f3 = tmp_path / "bad.tsv"
    mc.outFile(0.5, str(f3), ["E", "n"])  # mismatched dimensions: nothing written
    assert f3.read_text() == ""
    with pytest.raises(KeyError):
        mc.outFile(0.5, str(f3), ["nope"])
    assert mc.obsValue("n", 1, 0) == 0.125j


CPP = r"""
#include <cstdio>
#include <iostream>
#include "qudrip_gpu_lattice.hpp"
#include "qudrip_gpu_params.hpp"
using namespace qudrip_gpu;
int main(int argc, char** argv) {
  std::vector<c2> coords, pv{c2{4, 0}, c2{0, 3}};
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 3; ++j) coords.push_back(c2{i, j});
  Lattice<2> L(coords, pv);
  std::printf("vol %d rp %d %d %d %d\n", L.vol(), L.rpvec(0)(0), L.rpvec(0)(1), L.rpvec(1)(0), L.rpvec(1)(1));
  for (c2 c : {c2{5, -1}, c2{4, 3}, c2{-1, 0}, c2{-4, 0}})
    std::printf("reduce %d %d -> %d %d idx %zu\n", c(0), c(1), L.reduce(c)(0), L.reduce(c)(1), L(c));
  LatticeFunction<std::complex<double>, 2> f(L);
  for (size_t i = 0; i < L.N(); ++i) f(i) = std::complex<double>(0.1 * i, -0.05 * i * i);
  auto d = f.DFT(c2{1, 2});
  std::printf("dft %.17g %.17g\n", d.real(), d.imag());
  params_type<double> p;
  p("J") = 0.5;
  p("phi") = 30.0;
  Model<double, 2> m(L);
  for (size_t i = 0; i < L.N(); ++i) m.addBond((int)i, (int)L(L(i) + c2{1, 0}), p);
  m.print();
  param_finder pf(argv[1]);
  int nx = 0, phi_i = 0;
  double jx = 0, jz = 0;
  std::string name;
  std::complex<double> z;
  pf.find_param("Nx", nx);
  pf.find_param("phi", phi_i);
  pf.find_param("Jx", jx);
  pf.find_param("Jz", jz);
  pf.find_param("name", name);
  pf.find_param("z", z);
  std::vector<double> v(3);
  pf.find_param_tvec("vec", v);
  std::vector<std::complex<double>> cv(2);
  pf.find_param_tvec("cvec", cv);
  std::printf("params %d %d %.17g %.17g %s %g %g | %g %g %g | %g %g %g %g\n", nx, phi_i, jx, jz, name.c_str(),
              z.real(), z.imag(), v[0], v[1], v[2], cv[0].real(), cv[0].imag(), cv[1].real(), cv[1].imag());
  try {
    pf.find_param("missing", jx, 1);
  } catch (std::string& s) {
    std::printf("missing %s\n", s.c_str());
  }
  return 0;
}
"""


def test_cpp_headers_agree_with_python(tmp_path):
    src, exe = tmp_path / "t.cpp", tmp_path / "t"
    src.write_text(CPP)
    subprocess.run(["g++", "-std=c++17", "-O1", str(src), "-I", os.path.join(ROOT, "include"), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe), str(write_params(tmp_path))], check=True, capture_output=True,
                         text=True).stdout.split("\n")
    L = square(4, 3)
    assert out[0] == "vol -12 rp -3 0 0 -4"
    for line, c in zip(out[1:5], [(5, -1), (4, 3), (-1, 0), (-4, 0)]):
        r = L.reduce(c)
        assert line == f"reduce {c[0]} {c[1]} -> {r[0]} {r[1]} idx {L(c)}"
    f = q.LatticeFunction(L)
    for i in range(L.N()):
        f[i] = complex(0.1 * i, -0.05 * i * i)
    d = f.DFT((1, 2))
    re, im = map(float, out[5].split()[1:])
    assert abs(re - d.real) <= 1e-15 and abs(im - d.imag) <= 1e-15
    m = q.Model(L)
    p = q.params_type()
    p["J"] = 0.5
    p["phi"] = 30.0
    for i in range(L.N()):
        m.addBond(i, L(L(i) + np.array([1, 0])), p)
    assert "\n".join(out[6:6 + 1 + L.N()]) + "\n" == m.describe()
    tail = out[6 + 1 + L.N()]
    assert tail == "params 4 3 0.14999999999999999 2.75 twoliquid 1.5 -2 | 0.5 1.25 2 | 1 2 -3 4.5"
    assert out[7 + 1 + L.N()] == "missing missing"
