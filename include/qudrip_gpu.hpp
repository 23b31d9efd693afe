// qudrip_gpu.hpp -- QuDrip's exact-diagonalization API on the GB300 engine.
//
// Header-only C++17 over the C ABI of qudrip_gb300.h.  The names and their
// meaning follow the reference headers so that a QuDrip program changes its
// include and namespace only:
//
//   getQbits                       index.hpp:80-94,300
//   getNset/getNup/getNdo/getNd/getNh, `cq = value`, cq + cq, cq - cq
//                                  conservation.hpp:89-157,233-256,467-506
//   Constrain / LooseConstrain     conservation.hpp:200-239
//   getBoseGate/getFermiGate, gate << U, gate(site)      operators/bit.hpp:7-45
//   getHopFermiGate/getHopBoseGate, gate(a, b)           operators/hopbit.hpp:7-40
//   Operator * Operator, OperatorSum + - *, append rule  operator.hpp:68-132,
//                                                        operator_abel.hpp:9-158
//   ham >> index  (returns the lowered matrix, on the device)  operator_abel.hpp:25-34
//   getState, psi(t), psi.eval(t, H)                     state.hpp:9-104
//   Arnoldi::getLanczosSolver(index, k).getGroundState   sparse_algorithm.hpp:475-604
//   Arnoldi::getSolver(index, k).evolve                  sparse_algorithm.hpp:548-562
//   SpMatrix + SpMatrix, SpMatrix *= s (device-side)     Eigen sparse sum / scale
//   McManager (addObs, addAux, updateMatrix, incrMatrix, normMatrix, incrAllObs,
//   clearAll, normAll, collectAll, outFile, obsValue)    mc_manager.hpp:14-214
//   Lattice / LatticeFunction / Model / params_type      qudrip_gpu_lattice.hpp
//   param_finder                                         qudrip_gpu_params.hpp
//
// Differences a caller sees: matrices are the small `Matrix` type below
// (2x2 gate matrices) instead of Eigen; the lowered operator is a device
// handle (SpMatrix) instead of an Eigen SparseMatrix; shuffle_state takes a
// seed and draws real uniform[-1, 1] entries; errors throw qudrip_gpu::Error
// instead of aborting.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "qudrip_gb300.h"

namespace qudrip_gpu {

using value_type = std::complex<double>;
const value_type II(0.0, 1.0);
static const double eps = 1e-10;

struct Error : std::runtime_error {
  qd_status code;
  Error(qd_status c, const std::string& where)
      : std::runtime_error(where + ": " + qd_status_string(c) + " (" + qd_last_error() + ")"), code(c) {}
};

inline void check(qd_status s, const char* where) {
  if (s != QD_OK) throw Error(s, where);
}

// ------------------------------------------------------------------ context
class Context {
 public:
  static Context& get() {
    static Context c(0);
    return c;
  }
  qd_ctx* handle() const { return ctx_; }
  ~Context() {
    if (ctx_) qd_ctx_destroy(ctx_);
  }

 private:
  explicit Context(int device) { check(qd_ctx_create(device, &ctx_), "qd_ctx_create"); }
  qd_ctx* ctx_ = nullptr;
};

// ------------------------------------------------------------------ small dense matrices
class Matrix {
 public:
  Matrix(int r = 0, int c = 0) : r_(r), c_(c), a_((size_t)r * c, value_type(0.0, 0.0)) {}
  Matrix(int r, int c, std::initializer_list<value_type> rowmajor) : Matrix(r, c) {
    size_t k = 0;
    for (auto v : rowmajor) {
      a_[k] = v;
      ++k;
    }
  }
  int rows() const { return r_; }
  int cols() const { return c_; }
  value_type& operator()(int i, int j) { return a_[(size_t)i * c_ + j]; }
  value_type operator()(int i, int j) const { return a_[(size_t)i * c_ + j]; }
  Matrix operator+(const Matrix& o) const {
    Matrix m(*this);
    for (size_t k = 0; k < a_.size(); ++k) m.a_[k] += o.a_[k];
    return m;
  }
  Matrix operator-(const Matrix& o) const {
    Matrix m(*this);
    for (size_t k = 0; k < a_.size(); ++k) m.a_[k] -= o.a_[k];
    return m;
  }
  friend Matrix operator*(value_type s, const Matrix& m) {
    Matrix o(m);
    for (auto& v : o.a_) v = s * v;
    return o;
  }
  friend Matrix operator*(const Matrix& m, value_type s) { return s * m; }

 private:
  int r_, c_;
  std::vector<value_type> a_;
};

const Matrix pauli_x(2, 2, {0.0, 1.0, 1.0, 0.0});
const Matrix pauli_y(2, 2, {0.0, -II, II, 0.0});
const Matrix pauli_z(2, 2, {1.0, 0.0, 0.0, -1.0});
const Matrix id(2, 2, {1.0, 0.0, 0.0, 1.0});

// ------------------------------------------------------------------ indices and quantities
class QbitsIndex {
 public:
  explicit QbitsIndex(int n) : n_(n) {}
  int nbits() const { return n_; }
  uint64_t range() const { return 1ull << n_; }

 private:
  int n_;
};
inline QbitsIndex getQbits(int N) { return QbitsIndex(N); }

// A conserved quantity or an integer combination; `cq = v` records the target.
class ConservedQuantity {
 public:
  ConservedQuantity() = default;
  explicit ConservedQuantity(qd_cq_term t) { terms_.push_back(t); }
  ConservedQuantity& operator=(long long v) {
    target_ = v;
    return *this;
  }
  ConservedQuantity operator+(const ConservedQuantity& o) const {
    ConservedQuantity q;
    q.terms_ = terms_;
    q.terms_.insert(q.terms_.end(), o.terms_.begin(), o.terms_.end());
    return q;
  }
  ConservedQuantity operator-(const ConservedQuantity& o) const {
    ConservedQuantity q;
    q.terms_ = terms_;
    for (auto t : o.terms_) {
      t.coef = -t.coef;
      q.terms_.push_back(t);
    }
    return q;
  }
  qd_constraint constraint() const {
    if (terms_.empty() || terms_.size() > 4) throw Error(QD_ERR_INVALID, "constraint needs 1..4 quantities");
    qd_constraint c{};
    c.nterms = (int32_t)terms_.size();
    c.target = target_;
    for (size_t k = 0; k < terms_.size(); ++k) c.term[k] = terms_[k];
    return c;
  }

 private:
  std::vector<qd_cq_term> terms_;
  long long target_ = 0;
};

inline uint64_t bit_range_mask(int lo, int hi_inclusive) {
  uint64_t m = 0;
  for (int i = lo; i <= hi_inclusive && i < 64; ++i) m |= 1ull << i;
  return m;
}
inline ConservedQuantity nset_quantity(uint64_t mask) {
  qd_cq_term t{};
  t.kind = QD_CQ_NSET;
  t.coef = 1;
  t.mask = mask;
  return ConservedQuantity(t);
}
// Nset(index, -1, -1) covers bits 0..popcount(range-1) inclusive (conservation.hpp:417-422)
inline ConservedQuantity getNset(const QbitsIndex& idx) { return nset_quantity(bit_range_mask(0, idx.nbits())); }
inline ConservedQuantity getNup(const QbitsIndex&, int Nsite) { return nset_quantity(bit_range_mask(0, Nsite - 1)); }
inline ConservedQuantity getNdo(const QbitsIndex&, int Nsite) {
  return nset_quantity(bit_range_mask(Nsite, 2 * Nsite - 1));
}
inline ConservedQuantity nd_quantity(int Nsite, int hole) {
  qd_cq_term t{};
  t.kind = QD_CQ_ND;
  t.coef = 1;
  t.nsite = Nsite;
  t.hole = hole;
  return ConservedQuantity(t);
}
inline ConservedQuantity getNd(const QbitsIndex&, int Nsite) { return nd_quantity(Nsite, 0); }
inline ConservedQuantity getNh(const QbitsIndex&, int Nsite) { return nd_quantity(Nsite, 1); }

// The constrained sector (SubIndex), built on the device.
class SubIndex {
 public:
  SubIndex(const QbitsIndex& idx, std::vector<qd_constraint> cons, int tight) {
    auto* raw = (qd_sector*)nullptr;
    check(qd_sector_create(Context::get().handle(), idx.nbits(), cons.empty() ? nullptr : cons.data(),
                           (int)cons.size(), tight, &raw),
          "Constrain");
    sec_.reset(raw, [](qd_sector* s) { qd_sector_destroy(s); });
    check(qd_sector_dim(raw, &dim_), "qd_sector_dim");
  }
  int64_t range() const { return dim_; }
  qd_sector* handle() const { return sec_.get(); }
  std::vector<uint64_t> basis() const {
    std::vector<uint64_t> b((size_t)dim_);
    check(qd_sector_basis(sec_.get(), b.data()), "qd_sector_basis");
    return b;
  }

 private:
  std::shared_ptr<qd_sector> sec_;
  int64_t dim_ = 0;
};

template <typename... CQs>
SubIndex Constrain(const QbitsIndex& idx, const CQs&... cqs) {
  return SubIndex(idx, std::vector<qd_constraint>{cqs.constraint()...}, 0);
}
template <int tight, typename... CQs>
SubIndex LooseConstrain(const QbitsIndex& idx, const CQs&... cqs) {
  return SubIndex(idx, std::vector<qd_constraint>{cqs.constraint()...}, tight);
}

// ------------------------------------------------------------------ operators
class SpMatrix;
class OperatorSum;

class Operator {
 public:
  explicit Operator(std::shared_ptr<const qd_gate> g) { gates_.push_back(std::move(g)); }
  Operator operator*(const Operator& o) const {
    Operator r(*this);
    r.gates_.insert(r.gates_.end(), o.gates_.begin(), o.gates_.end());
    return r;
  }
  bool operator==(const Operator& o) const {  // pointer identity, operator.hpp:123-131
    if (gates_.size() != o.gates_.size()) return false;
    for (size_t i = 0; i < gates_.size(); ++i)
      if (gates_[i] != o.gates_[i]) return false;
    return true;
  }
  const std::vector<std::shared_ptr<const qd_gate>>& gates() const { return gates_; }

 private:
  std::vector<std::shared_ptr<const qd_gate>> gates_;
};

class BitGate {
 public:
  BitGate(const QbitsIndex& idx, int string) : nbits_(idx.nbits()), string_(string) {}
  void operator<<(const Matrix& U) {
    if (U.rows() != 2 || U.cols() != 2) throw Error(QD_ERR_INVALID, "bit gates take a 2x2 matrix");
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) {
        u_[2 * (2 * i + j)] = U(i, j).real();
        u_[2 * (2 * i + j) + 1] = U(i, j).imag();
      }
  }
  Operator operator()(int site) const {
    if (site < 0 || site >= nbits_) throw Error(QD_ERR_INVALID, "gate site out of range");
    auto g = std::make_shared<qd_gate>();
    g->kind = QD_GATE_BIT;
    g->site = site;
    g->string = string_;
    for (int q = 0; q < 8; ++q) g->u[q] = u_[q];
    return Operator(g);
  }

 private:
  int nbits_, string_;
  double u_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

class HopGate {
 public:
  HopGate(const QbitsIndex& idx, int string) : nbits_(idx.nbits()), string_(string) {}
  Operator operator()(int a, int b) const {  // c^dagger_a c_b (hopbit.hpp:102-107)
    if (a < 0 || b < 0 || a >= nbits_ || b >= nbits_) throw Error(QD_ERR_INVALID, "gate site out of range");
    auto g = std::make_shared<qd_gate>();
    g->kind = QD_GATE_HOP;
    g->site = a;
    g->site_b = b;
    g->string = string_;
    return Operator(g);
  }

 private:
  int nbits_, string_;
};

inline BitGate getBoseGate(const QbitsIndex& idx) { return BitGate(idx, 1); }
inline BitGate getFermiGate(const QbitsIndex& idx) { return BitGate(idx, -1); }
inline HopGate getHopBoseGate(const QbitsIndex& idx) { return HopGate(idx, 1); }
inline HopGate getHopFermiGate(const QbitsIndex& idx) { return HopGate(idx, -1); }

class OperatorSum {
 public:
  OperatorSum() = default;
  OperatorSum(const Operator& op, value_type c) {
    ops_.push_back(op);
    coeffs_.push_back(c);
  }
  int size() const { return (int)ops_.size(); }
  OperatorSum& append(const Operator& op, value_type c) {  // operator_abel.hpp:115-127
    for (size_t i = 0; i < ops_.size(); ++i)
      if (ops_[i] == op) {
        coeffs_[i] += c;
        return *this;
      }
    ops_.push_back(op);
    coeffs_.push_back(c);
    return *this;
  }
  OperatorSum operator+(const Operator& op) const { return OperatorSum(*this).append(op, 1.0); }
  OperatorSum operator-(const Operator& op) const { return OperatorSum(*this).append(op, -1.0); }
  OperatorSum operator+(const OperatorSum& o) const {
    OperatorSum r(*this);
    r.ops_.insert(r.ops_.end(), o.ops_.begin(), o.ops_.end());
    r.coeffs_.insert(r.coeffs_.end(), o.coeffs_.begin(), o.coeffs_.end());
    return r;
  }
  OperatorSum operator-(const OperatorSum& o) const {
    OperatorSum r(*this);
    r.ops_.insert(r.ops_.end(), o.ops_.begin(), o.ops_.end());
    for (auto c : o.coeffs_) r.coeffs_.push_back(-c);
    return r;
  }
  OperatorSum operator*(const Operator& op) const {
    OperatorSum r(*this);
    for (auto& o : r.ops_) o = o * op;
    return r;
  }
  OperatorSum operator*(value_type m) const {
    OperatorSum r(*this);
    for (auto& c : r.coeffs_) c *= m;
    return r;
  }
  OperatorSum operator*(const OperatorSum& o) const {
    OperatorSum r;
    for (size_t i = 0; i < ops_.size(); ++i)
      for (size_t j = 0; j < o.ops_.size(); ++j) r.append(ops_[i] * o.ops_[j], coeffs_[i] * o.coeffs_[j]);
    return r;
  }
  SpMatrix operator>>(const SubIndex& index) const;

 private:
  std::vector<Operator> ops_;
  std::vector<value_type> coeffs_;
};

inline OperatorSum operator*(value_type c, const Operator& op) { return OperatorSum(op, c); }
inline OperatorSum operator*(const Operator& op, value_type c) { return OperatorSum(op, c); }
inline OperatorSum operator*(value_type c, const OperatorSum& s) { return s * c; }
inline OperatorSum operator+(const Operator& a, const Operator& b) { return OperatorSum(a, 1.0).append(b, 1.0); }
inline OperatorSum operator-(const Operator& a, const Operator& b) { return OperatorSum(a, 1.0).append(b, -1.0); }
inline OperatorSum getEmptyOperator() { return OperatorSum(); }

// The lowered operator, held on the device (CSR; the reference's CSC on download).
class SpMatrix {
 public:
  SpMatrix() = default;
  explicit SpMatrix(qd_ham* h) : ham_(h, [](qd_ham* p) { qd_ham_destroy(p); }) {
    check(qd_ham_get_info(h, &info_), "qd_ham_get_info");
  }
  int64_t rows() const { return info_.dim; }
  int64_t cols() const { return info_.dim; }
  int64_t nonZeros() const { return info_.nnz; }
  qd_ham* handle() const { return ham_.get(); }
  bool empty() const { return !ham_; }
  // Eigen's sparse sum: union pattern, a + b per value, explicit zeros kept.
  SpMatrix operator+(const SpMatrix& o) const {
    qd_ham* h = nullptr;
    check(qd_ham_add(ham_.get(), o.ham_.get(), &h), "SpMatrix +");
    return SpMatrix(h);
  }
  SpMatrix& operator+=(const SpMatrix& o) { return *this = *this + o; }
  // Value semantics: a copy shares the device matrix until one of them is scaled.
  SpMatrix& operator*=(value_type s) {
    if (ham_.use_count() > 1) {
      qd_ham* h = nullptr;
      check(qd_ham_copy(ham_.get(), &h), "SpMatrix copy");
      *this = SpMatrix(h);
    }
    check(qd_ham_scale(ham_.get(), s.real(), s.imag()), "SpMatrix *=");
    check(qd_ham_get_info(ham_.get(), &info_), "qd_ham_get_info");
    return *this;
  }
  SpMatrix operator*(value_type s) const {
    SpMatrix r = *this;
    r *= s;
    return r;
  }
  // Reference layout: column pointers, row indices, complex values.
  void csc(std::vector<int64_t>& colptr, std::vector<int32_t>& rowidx, std::vector<value_type>& vals) const {
    colptr.resize((size_t)info_.dim + 1);
    rowidx.resize((size_t)info_.nnz);
    vals.resize((size_t)info_.nnz);
    check(qd_ham_download_csc(ham_.get(), colptr.data(), rowidx.data(), reinterpret_cast<double*>(vals.data())),
          "qd_ham_download_csc");
  }

 private:
  std::shared_ptr<qd_ham> ham_;
  qd_ham_info info_{};
};

inline SpMatrix OperatorSum::operator>>(const SubIndex& index) const {
  std::vector<qd_term> terms;
  std::vector<qd_gate> gates;
  for (size_t i = 0; i < ops_.size(); ++i) {
    qd_term t{};
    t.coeff_re = coeffs_[i].real();
    t.coeff_im = coeffs_[i].imag();
    t.gate_offset = (int32_t)gates.size();
    t.ngates = (int32_t)ops_[i].gates().size();
    for (const auto& g : ops_[i].gates()) gates.push_back(*g);
    terms.push_back(t);
  }
  qd_ham* h = nullptr;
  check(qd_ham_lower(index.handle(), terms.data(), (int)terms.size(), gates.data(), (int)gates.size(), &h),
        "operator>>");
  return SpMatrix(h);
}
inline SpMatrix operator>>(const Operator& op, const SubIndex& index) { return OperatorSum(op, 1.0) >> index; }

// ------------------------------------------------------------------ states
class State {
 public:
  State(const SubIndex& idx, int nt) : dim_(idx.range()), nt_(nt) {
    qd_state* raw = nullptr;
    check(qd_state_create(Context::get().handle(), dim_, nt, &raw), "getState");
    st_.reset(raw, [](qd_state* s) { qd_state_destroy(s); });
  }
  State& operator()(int t) {
    if (t < 0 || t >= nt_) throw Error(QD_ERR_INVALID, "time slot out of range");
    t_ = t;
    return *this;
  }
  int t() const { return t_; }
  int nt() const { return nt_; }
  int64_t ndim() const { return dim_; }
  value_type eval(int t, const SpMatrix& H) const {  // state.hpp:33-45
    double e[2];
    check(qd_state_eval(st_.get(), t, H.handle(), e), "State::eval");
    return value_type(e[0], e[1]);
  }
  std::vector<value_type> mat() const {
    std::vector<value_type> v((size_t)dim_);
    check(qd_state_download(st_.get(), t_, reinterpret_cast<double*>(v.data())), "qd_state_download");
    return v;
  }
  void set(const std::vector<value_type>& v) {
    if ((int64_t)v.size() != dim_) throw Error(QD_ERR_INVALID, "state column has the wrong length");
    check(qd_state_upload(st_.get(), t_, reinterpret_cast<const double*>(v.data())), "qd_state_upload");
  }
  qd_state* handle() const { return st_.get(); }

 private:
  std::shared_ptr<qd_state> st_;
  int64_t dim_;
  int nt_;
  int t_ = 0;
};

inline State getState(const SubIndex& idx, int nt) { return State(idx, nt); }

// Seeded real uniform[-1, 1] start vector, normalised (utils.hpp:129-140 draws
// unseeded complex values; a seed makes runs reproducible).
inline void shuffle_state(State& psi, uint64_t seed = 12345) {
  std::mt19937_64 mt(seed);
  std::uniform_real_distribution<double> dice(-1.0, 1.0);
  std::vector<value_type> v((size_t)psi.ndim());
  double n2 = 0.0;
  for (auto& x : v) {
    x = dice(mt);
    n2 += std::norm(x);
  }
  for (auto& x : v) x /= std::sqrt(n2);
  psi.set(v);
}

// ------------------------------------------------------------------ observables
#define MC_REAL 0
#define MC_COMPLEX 1
using functor_type = std::function<value_type(const value_type&)>;

// McManager (mc_manager.hpp:14-214) in one process: named groups of `dim`
// operators with an (nt x dim) table each; incrAllObs evaluates every
// operator on psi(psi_tstp) in one qd_obs_eval pass and adds into row tstp.
// collectAll is the one-process case of the reference's MPI_Reduce (nothing
// to combine; replicas combine their tables on the host).  obsValue(name, t,
// idx) reads row t, column idx.
class McManager {
 public:
  McManager(int nt, State* p_psi) : nt_(nt), p_psi_(p_psi), Nmc_((size_t)nt, 0) {}
  explicit McManager(State* p_psi) : McManager(p_psi->nt(), p_psi) {}

  void addObs(const std::string& name, int dim, int type = MC_COMPLEX) {
    data_[name] = std::vector<value_type>((size_t)nt_ * dim, value_type(0.0, 0.0));
    dims_[name] = dim;
    type_[name] = type;
    obs_[name] = std::vector<SpMatrix>((size_t)dim);
    aux_[name] = {};
  }
  void addAux(const std::string& name, const std::string& name2, const functor_type& func, int dim,
              int aux_type = MC_COMPLEX) {
    if (obs_.find(name2) == obs_.end()) throw std::string{"addAux: wrong dependent variable!"};
    data_[name] = std::vector<value_type>((size_t)nt_ * dim, value_type(0.0, 0.0));
    dims_[name] = dim;
    type_[name] = aux_type;
    func_[name] = func;
    aux_[name2].push_back(name);
  }
  void updateMatrix(const std::string& name, int idx, const SpMatrix& mat) { obs_.at(name).at((size_t)idx) = mat; }
  void incrMatrix(const std::string& name, int idx, const SpMatrix& mat) {
    SpMatrix& m = obs_.at(name).at((size_t)idx);
    if (m.empty()) m = mat;
    else m += mat;
  }
  void normMatrix(const std::string& name, int idx, value_type s) { obs_.at(name).at((size_t)idx) *= s; }
  SpMatrix& matrix(const std::string& name, int idx) { return obs_.at(name).at((size_t)idx); }

  void incrAllObs(int tstp, int psi_tstp = -1) {
    if (psi_tstp == -1) psi_tstp = tstp;
    std::vector<qd_ham*> hs;
    std::vector<std::pair<std::string, size_t>> dst;
    for (auto& o : obs_)
      for (size_t d = 0; d < o.second.size(); ++d) {
        hs.push_back(o.second[d].handle());
        dst.emplace_back(o.first, d);
      }
    if (!hs.empty()) {
      std::vector<double> v(2 * hs.size());
      check(qd_obs_eval(p_psi_->handle(), psi_tstp, (int)hs.size(), hs.data(), v.data()), "incrAllObs");
      for (size_t i = 0; i < hs.size(); ++i) {
        const value_type term(v[2 * i], v[2 * i + 1]);
        const std::string& n = dst[i].first;
        const size_t d = dst[i].second;
        data_[n][(size_t)tstp * dims_[n] + d] += term;
        for (const auto& a : aux_[n]) data_[a][(size_t)tstp * dims_[a] + d] += func_[a](term);
      }
    }
    ++Nmc_[(size_t)tstp];
  }
  void clearAll(int tstp) {
    for (auto& d : data_)
      for (int k = 0; k < dims_[d.first]; ++k) d.second[(size_t)tstp * dims_[d.first] + k] = 0.0;
  }
  void clearAll() {
    for (auto& d : data_) std::fill(d.second.begin(), d.second.end(), value_type(0.0, 0.0));
  }
  void normAll() {
    for (auto& d : data_)
      for (int t = 0; t < nt_; ++t)
        for (int k = 0; k < dims_[d.first]; ++k) d.second[(size_t)t * dims_[d.first] + k] *= 1.0 / Nmc_[(size_t)t];
  }
  void collectAll() {}
  int report() const { return 0; }
  value_type obsValue(const std::string& name, int tstp, int idx) const {
    return data_.at(name).at((size_t)tstp * dims_.at(name) + idx);
  }
  value_type value(const std::string& name, int t, int d) const { return obsValue(name, t, d); }

  // The TSV table of mc_manager.hpp:147-196: "#time[\tindex]", one column per
  // real observable and two (real, imag) per complex one, std::to_string
  // values; with dim > 1 a row per index and a blank line after each time.
  void outFile(double h, const std::string& fname, const std::vector<std::string>& obs_names,
               int precision = 6) const {
    (void)precision;  // the reference takes it and does not use it
    std::ofstream f(fname);
    auto it0 = data_.find(obs_names.at(0));
    if (it0 == data_.end()) throw std::string{"outFile: wrong name!!"};
    const int dim = dims_.at(obs_names[0]);
    std::string label = dim > 1 ? "#time\tindex" : "#time";
    for (const auto& n : obs_names) {
      auto it = type_.find(n);
      if (it == type_.end()) throw std::string{"outFile: wrong name!!"};
      if (it->second == MC_REAL) label += "\t" + n;
      else label += "\t" + n + "(real)" + "\t" + n + "(imag)";
      if (dims_.at(n) != dim) {
        std::cout << "mismatched dimensions" << std::endl;
        return;
      }
    }
    f << label << std::endl;
    for (int t = 0; t < nt_; ++t) {
      for (int idx = 0; idx < dim; ++idx) {
        label = dim > 1 ? std::to_string(t * h) + "\t" + std::to_string(idx) : std::to_string(t * h);
        for (const auto& n : obs_names) {
          const value_type v = data_.at(n)[(size_t)t * dims_.at(n) + idx];
          label += "\t" + std::to_string(v.real());
          if (type_.at(n) == MC_COMPLEX) label += "\t" + std::to_string(v.imag());
        }
        f << label << std::endl;
      }
      if (dim > 1) f << std::endl;
    }
  }

 private:
  int nt_;
  State* p_psi_;
  std::vector<int> Nmc_;
  std::map<std::string, std::vector<value_type>> data_;
  std::map<std::string, int> dims_;
  std::map<std::string, int> type_;
  std::map<std::string, std::vector<SpMatrix>> obs_;
  std::map<std::string, std::vector<std::string>> aux_;
  std::map<std::string, functor_type> func_;
};

// ------------------------------------------------------------------ solvers
namespace Arnoldi {

class LanczosSolver {
 public:
  LanczosSolver(const SubIndex&, int kry_dim) : kry_dim_(kry_dim), evs_(1, 0.0) {}
  // products through the matrix-free form (qd_ham_build_matrix_free) instead of the CSR matrix
  void setMatrixFree(bool on) { spmv_ = on ? QD_SPMV_MATRIX_FREE : QD_SPMV_CSR; }
  // number of tracked eigenvalues and their initial values (sparse_algorithm.hpp:494-500)
  void convergeEV(int N, double iv = 0.0) {
    if (!(N < kry_dim_)) throw Error(QD_ERR_INVALID, "convergeEV: N must be below kry_dim");
    evs_.assign((size_t)N, iv);
  }
  // The first call starts from psi(tstp) and runs add_dim steps (all kry_dim
  // for -1); later calls grow the same Krylov space by add_dim more steps
  // (sparse_algorithm.hpp:564-585); a full space returns at once.
  void getGroundState(const SpMatrix& H, State& psi, int tstp, int add_dim = -1) {
    if (act_ >= kry_dim_) return;
    qd_lanczos_opts o{};
    o.krylov_dim = kry_dim_;
    o.spmv = spmv_;
    o.ritz = QD_RITZ_STORED_BASIS;
    o.add_dim = add_dim > 0 ? add_dim : 0;
    evals_.assign((size_t)kry_dim_, 0.0);
    if (act_ == 0)
      check(qd_lanczos_ground(H.handle(), psi.handle(), tstp, &o, evals_.data(), &res_), "getGroundState");
    else
      check(qd_lanczos_extend(H.handle(), psi.handle(), tstp, &o, evals_.data(), &res_), "getGroundState");
    act_ = res_.act_dim;
    evals_.resize((size_t)act_);
    const size_t m = std::min(evs_.size(), (size_t)act_);
    double e2 = 0.0;
    for (size_t i = 0; i < m; ++i) e2 += (evals_[i] - evs_[i]) * (evals_[i] - evs_[i]);
    err_ = std::sqrt(e2);
    for (size_t i = 0; i < m; ++i) evs_[i] = evals_[i];
  }
  double error() const { return err_; }
  int act_dim() const { return act_; }
  const std::vector<double>& eigenvalues() const { return evals_; }
  void storeE(const std::string& fname) const {
    std::ofstream f(fname);
    for (double e : evals_) f << e << "\n";
  }

 private:
  int kry_dim_;
  int spmv_ = QD_SPMV_CSR;
  int act_ = 0;
  double err_ = 0.0;
  std::vector<double> evs_;
  qd_lanczos_result res_{};
  std::vector<double> evals_;
};

class ArnoldiSolver {
 public:
  ArnoldiSolver(const SubIndex&, int kry_dim) : kry_dim_(kry_dim), evs_(1, 0.0) {}
  void evolve(const SpMatrix& H, State& psi, int tstp, double h, int kry_dim_rt = 0) {
    int act = 0;
    check(qd_arnoldi_evolve(H.handle(), psi.handle(), tstp, tstp + 1, h, kry_dim_rt ? kry_dim_rt : kry_dim_, &act),
          "evolve");
    act_ = act;
  }
  // number of tracked eigenvalues and their initial values (sparse_algorithm.hpp:494-500)
  void convergeEV(int N, double iv = 0.0) {
    if (!(N < kry_dim_)) throw Error(QD_ERR_INVALID, "convergeEV: N must be below kry_dim");
    evs_.assign((size_t)N, iv);
  }
  // Incremental Arnoldi ground state (sparse_algorithm.hpp:564-585): the first call
  // starts from psi(tstp) and runs add_dim steps (all kry_dim for -1); later calls
  // grow the same Krylov space; a full or closed space returns at once.
  void getGroundState(const SpMatrix& H, State& psi, int tstp, int add_dim = -1) {
    if (gs_act_ >= kry_dim_ || gs_closed_) return;
    qd_lanczos_opts o{};
    o.krylov_dim = kry_dim_;
    o.spmv = QD_SPMV_CSR;
    o.ritz = QD_RITZ_STORED_BASIS;
    o.add_dim = add_dim > 0 ? add_dim : 0;
    evals_.assign((size_t)kry_dim_, 0.0);
    if (gs_act_ == 0)
      check(qd_arnoldi_ground(H.handle(), psi.handle(), tstp, &o, evals_.data(), &res_), "getGroundState");
    else
      check(qd_arnoldi_extend(H.handle(), psi.handle(), tstp, &o, evals_.data(), &res_), "getGroundState");
    gs_act_ = act_ = res_.act_dim;
    gs_closed_ = res_.breakdown != 0;
    evals_.resize((size_t)act_);
    const size_t m = std::min(evs_.size(), (size_t)act_);
    double e2 = 0.0;
    for (size_t i = 0; i < m; ++i) e2 += (evals_[i] - evs_[i]) * (evals_[i] - evs_[i]);
    err_ = std::sqrt(e2);
    for (size_t i = 0; i < m; ++i) evs_[i] = evals_[i];
  }
  double error() const { return err_; }
  int act_dim() const { return act_; }
  const std::vector<double>& eigenvalues() const { return evals_; }
  void storeE(const std::string& fname) const {
    std::ofstream f(fname);
    for (double e : evals_) f << e << "\n";
  }

 private:
  int kry_dim_;
  int act_ = 0;
  int gs_act_ = 0;
  bool gs_closed_ = false;
  double err_ = 0.0;
  std::vector<double> evs_;
  qd_lanczos_result res_{};
  std::vector<double> evals_;
};

inline LanczosSolver getLanczosSolver(const SubIndex& index, int kry_dim) { return LanczosSolver(index, kry_dim); }
inline ArnoldiSolver getSolver(const SubIndex& index, int kry_dim) { return ArnoldiSolver(index, kry_dim); }

}  // namespace Arnoldi

// Hermitian::LanczosSolver (sparse_algorithm.hpp:287-301): two-vector Lanczos,
// ground state rebuilt by a second pass.
namespace Hermitian {

class LanczosSolver {
 public:
  LanczosSolver(const SubIndex&, int kry_dim) : kry_dim_(kry_dim) {}
  void getGroundState(const SpMatrix& H, State& psi, int tstp) {
    evals_.assign((size_t)kry_dim_ + 1, 0.0);
    check(qd_hermitian_lanczos_ground(H.handle(), psi.handle(), tstp, kry_dim_, evals_.data(), &res_),
          "getGroundState");
    evals_.resize((size_t)res_.act_dim);
  }
  double error() const { return res_.err; }
  const std::vector<double>& eigenvalues() const { return evals_; }

 private:
  int kry_dim_;
  qd_lanczos_result res_{};
  std::vector<double> evals_;
};

}  // namespace Hermitian
}  // namespace qudrip_gpu
