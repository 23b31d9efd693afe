// qudrip_gpu_lattice.hpp -- lattices, lattice functions and bond models for the
// drop-in header: the names and behaviour of the reference's lattice.hpp
// (params_type, get_reci, Lattice<N>, LatticeFunction<T, N>, Model<T, N>),
// written over std::array instead of Eigen's fixed-size vectors.  Host code
// only; it needs nothing from the library, so it can be used (and tested)
// without a GPU.  A Model emits its Hamiltonian as an operator sum
// (getHamiltonian: lowered on the device by `>>` like any other operator) or
// as a sum of lowered matrices (getHamiltonianMatrix: device-side sums).
//
// Defined where the reference is undefined: Lattice(coords) with no
// periodicity vectors has vol() == 0, zero reciprocal vectors and reduce() the
// identity; the multi-argument DFT sums over every tuple of sites with one
// momentum per argument; params_type::stringize() of no parameters is "".
#pragma once

#include <array>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace qudrip_gpu {

// ------------------------------------------------------------------ integer vectors
template <int N>
struct IVec {
  std::array<int, N> v{};
  IVec() = default;
  IVec(std::initializer_list<int> l) {
    int i = 0;
    for (int x : l)
      if (i < N) v[i++] = x;
  }
  int& operator()(int i) { return v[i]; }
  int operator()(int i) const { return v[i]; }
  int rows() const { return N; }
  IVec operator+(const IVec& o) const {
    IVec r;
    for (int i = 0; i < N; ++i) r.v[i] = v[i] + o.v[i];
    return r;
  }
  IVec operator-(const IVec& o) const {
    IVec r;
    for (int i = 0; i < N; ++i) r.v[i] = v[i] - o.v[i];
    return r;
  }
  IVec& operator-=(const IVec& o) {
    for (int i = 0; i < N; ++i) v[i] -= o.v[i];
    return *this;
  }
  bool operator==(const IVec& o) const { return v == o.v; }
  bool operator<(const IVec& o) const { return v < o.v; }
};
template <int N>
IVec<N> operator*(int s, const IVec<N>& a) {
  IVec<N> r;
  for (int i = 0; i < N; ++i) r.v[i] = s * a.v[i];
  return r;
}
template <int N>
int StaticInnerProduct(const IVec<N>& a, const IVec<N>& b) {
  int s = 0;
  for (int i = 0; i < N; ++i) s += a.v[i] * b.v[i];
  return s;
}
inline IVec<3> StaticCrossProduct(const IVec<3>& a, const IVec<3>& b) {
  return IVec<3>{a.v[1] * b.v[2] - a.v[2] * b.v[1], a.v[2] * b.v[0] - a.v[0] * b.v[2],
                 a.v[0] * b.v[1] - a.v[1] * b.v[0]};
}
template <int N>
using StaticIVector = IVec<N>;
using c1 = IVec<1>;
using c2 = IVec<2>;
using c3 = IVec<3>;

// ------------------------------------------------------------------ parameters
// Named bond parameters (lattice.hpp:14-52).  The reference keeps an
// unordered_map; here names keep their insertion order.
template <typename T>
class params_type {
 public:
  T& operator()(const std::string& name) {
    for (auto& kv : p_)
      if (kv.first == name) return kv.second;
    p_.emplace_back(name, T{});
    return p_.back().second;
  }
  const T& operator()(const std::string& name) const {
    for (auto& kv : p_)
      if (kv.first == name) return kv.second;
    throw std::string("undefined params");
  }
  std::string stringize() const {
    std::string s;
    for (auto& kv : p_) s += kv.first + "=" + std::to_string(kv.second) + ",";
    if (!s.empty()) s[s.size() - 1] = ';';
    return s;
  }

 private:
  std::vector<std::pair<std::string, T>> p_;
};
template <typename T>
std::ostream& operator<<(std::ostream& os, const params_type<T>& p) {
  return os << p.stringize();
}

// ------------------------------------------------------------------ reciprocal vectors
// Unnormalised reciprocal vectors of the periodicity vectors and the signed
// cell volume (lattice.hpp:62-110).
inline int get_reci(std::vector<IVec<1>>& rp, const std::vector<IVec<1>>& p) {
  rp[0](0) = p[0](0);
  return StaticInnerProduct(p[0], p[0]);
}
inline int get_reci(std::vector<IVec<2>>& rp, const std::vector<IVec<2>>& p) {
  rp[0](0) = -p[1](1);
  rp[0](1) = p[1](0);
  rp[1](0) = p[0](1);
  rp[1](1) = -p[0](0);
  return StaticInnerProduct(rp[0], p[0]);
}
inline int get_reci(std::vector<IVec<3>>& rp, const std::vector<IVec<3>>& p) {
  rp[0] = StaticCrossProduct(p[1], p[2]);
  rp[1] = StaticCrossProduct(p[2], p[0]);
  rp[2] = StaticCrossProduct(p[0], p[1]);
  return StaticInnerProduct(p[0], StaticCrossProduct(p[1], p[2]));
}

// ------------------------------------------------------------------ lattice
template <int NDIM>
class Lattice {
 public:
  using coord_type = IVec<NDIM>;
  using coords_type = std::vector<coord_type>;

  Lattice(const coords_type& coord, const coords_type& pvec) : coord_(coord), pvec_(pvec), rpvec_(NDIM) {
    if (!pvec_.empty()) {
      if ((int)pvec_.size() != NDIM) throw std::invalid_argument("one periodicity vector per dimension");
      vol_ = get_reci(rpvec_, pvec_);
    }
    for (auto& c : coord_)
      for (int i = 0; i < NDIM; ++i)
        if (c(i) < 0) {
          std::cout << "Warning: non-positive coordinates are invalid for periodicity reduction." << std::endl;
          return;
        }
  }
  explicit Lattice(const coords_type& coord) : Lattice(coord, coords_type{}) {}

  size_t N() const { return coord_.size(); }
  int vol() const { return vol_; }

  // For each periodicity vector in turn: ir = (r.rp_i) / vol in C++ integer
  // division, one less when the product is nonzero and its sign differs from
  // vol's, r -= ir p_i (lattice.hpp:163-179).
  coord_type reduce(const coord_type& c) const {
    coord_type r = c;
    if (pvec_.empty()) return r;
    for (int i = 0; i < NDIM; ++i) {
      const int prod = StaticInnerProduct(r, rpvec_[i]);
      int ir = prod / vol_;
      if (prod != 0 && ((prod < 0) != (vol_ < 0))) --ir;
      r -= ir * pvec_[i];
    }
    return r;
  }
  const coord_type& operator()(size_t i) const {
    assert(i < N());
    return coord_[i];
  }
  size_t operator()(const coord_type& c) const { return index(reduce(c)); }
  const coord_type& pvec(size_t i) const { return pvec_.at(i); }
  const coord_type& rpvec(size_t i) const { return rpvec_.at(i); }

 private:
  size_t index(const coord_type& c) const {
    for (size_t i = 0; i < coord_.size(); ++i)
      if (coord_[i] == c) return i;
    return coord_.size();
  }
  coords_type coord_;
  coords_type pvec_, rpvec_;
  int vol_ = 0;
};

// ------------------------------------------------------------------ lattice functions
template <typename T, int NDIM>
class LatticeFunction {
 public:
  using coord_type = IVec<NDIM>;
  using arg_type = std::vector<int>;

  explicit LatticeFunction(const Lattice<NDIM>& latt, int argn = 1)
      : latt_(latt), argn_(argn), data_((size_t)std::llround(std::pow((double)latt.N(), argn))) {}

  const T& operator()(size_t i) const { return data_.at(i); }
  T& operator()(size_t i) { return data_.at(i); }
  const T& operator()(const arg_type& a) const { return data_.at(convert_idx(a)); }
  T& operator()(const arg_type& a) { return data_.at(convert_idx(a)); }

  // (1/N) sum_i f_i exp(i theta_i), theta_i = sum_j <x_i, k_j rp_j> / vol
  // (lattice.hpp:269-283; no factor 2 pi, as in the reference).
  std::complex<double> DFT(const coord_type& k) const {
    std::complex<double> res(0.0, 0.0);
    for (size_t i = 0; i < latt_.N(); ++i) {
      const double th = phase(latt_(i), k);
      res += data_[i] * std::complex<double>(std::cos(th), std::sin(th));
    }
    return res / (double)latt_.N();
  }
  std::complex<double> DFT(const std::vector<coord_type>& ks) const {
    if ((int)ks.size() != argn_) throw std::invalid_argument("one momentum per argument");
    std::complex<double> res(0.0, 0.0);
    arg_type a((size_t)argn_);
    for (size_t idx = 0; idx < data_.size(); ++idx) {
      convert_arg(a, idx);
      double th = 0.0;
      for (int ix = 0; ix < argn_; ++ix) th += phase(latt_((size_t)a[ix]), ks[ix]);
      res += data_[idx] * std::complex<double>(std::cos(th), std::sin(th));
    }
    return res / (double)data_.size();
  }

 private:
  double phase(const coord_type& x, const coord_type& k) const {
    double th = 0.0;
    for (int j = 0; j < NDIM; ++j) th += StaticInnerProduct(x, k(j) * latt_.rpvec(j)) / (double)latt_.vol();
    return th;
  }
  size_t convert_idx(const arg_type& a) const {
    size_t idx = 0;
    for (int x : a) idx = idx * latt_.N() + (size_t)x;
    return idx;
  }
  void convert_arg(arg_type& a, size_t idx) const {
    for (int i = (int)a.size() - 1; i >= 0; --i) {
      a[i] = (int)(idx % latt_.N());
      idx /= latt_.N();
    }
  }
  Lattice<NDIM> latt_;
  int argn_;
  std::vector<T> data_;
};

// ------------------------------------------------------------------ bond models
template <typename T, int NDIM>
class Model {
 public:
  explicit Model(const Lattice<NDIM>& latt) : latt_(latt) {}

  void addBond(int s1, int s2, const params_type<T>& param) {
    if (s1 < 0 || s2 < 0 || (size_t)s1 >= latt_.N() || (size_t)s2 >= latt_.N())
      throw std::out_of_range("bond site outside the lattice");
    bonds_.emplace_back(s1, s2);
    params_.push_back(param);
  }
  size_t nbonds() const { return bonds_.size(); }
  const std::pair<int, int>& bond(size_t i) const { return bonds_.at(i); }
  const params_type<T>& param(size_t i) const { return params_.at(i); }

  // The text of lattice.hpp:327-341 (for 3D it repeats the second coordinate, as there).
  void print(std::ostream& os = std::cout) const {
    os << "Bonds: " << std::endl;
    for (size_t i = 0; i < bonds_.size(); ++i) {
      const auto& a = latt_((size_t)bonds_[i].first);
      const auto& b = latt_((size_t)bonds_[i].second);
      os << "(" + std::to_string(a(0));
      for (int j = 1; j < NDIM; ++j) os << "," + std::to_string(a(1));
      os << ") and (" + std::to_string(b(0));
      for (int j = 1; j < NDIM; ++j) os << "," + std::to_string(b(1));
      os << "): " << params_[i] << std::endl;
    }
  }

  // Sum over the bonds of f(s1, s2, param), from the empty sum R{}
  // (getEmptyOperator() for operator sums), lattice.hpp:370-383.
  template <typename FUNC>
  auto getHamiltonian(FUNC&& f) const -> decltype(f(0, 0, std::declval<const params_type<T>&>())) {
    using R = decltype(f(0, 0, std::declval<const params_type<T>&>()));
    R ham{};
    for (size_t i = 0; i < bonds_.size(); ++i) ham = ham + f(bonds_[i].first, bonds_[i].second, params_[i]);
    return ham;
  }
  // Sum over the bonds of the matrices f(s1, s2, param), starting from `zero`
  // (the reference's SpMatrix(ndim, ndim); pass the empty operator lowered on
  // the sector), lattice.hpp:355-368.
  template <typename FUNC, typename M>
  M getHamiltonianMatrix(FUNC&& f, M zero) const {
    M ham = zero;
    for (size_t i = 0; i < bonds_.size(); ++i) ham = ham + f(bonds_[i].first, bonds_[i].second, params_[i]);
    return ham;
  }

 private:
  std::vector<std::pair<int, int>> bonds_;
  std::vector<params_type<T>> params_;
  Lattice<NDIM> latt_;
};

}  // namespace qudrip_gpu
