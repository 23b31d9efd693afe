// qd_oracle.cpp -- CPU restatement of QuDrip's exact-diagonalization path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle for the
// GB300 engine: tests/, __graft_entry__.smoke() and bench.py's CPU baseline
// are its only users.  Nothing in the qudrip_gb300 product links or calls it.
//
// Parity status: parity unpinned against the reference itself.  QuDrip cannot
// be compiled in this environment (it is header-only C++20 on Eigen3 >= 3.3,
// CMakeLists.txt:18, and Eigen is not installed), and QuDrip ships no tests or
// golden vectors, so no output of the reference is available to compare
// with.  The restatement below follows the reference line by line (each
// function cites the file:line it restates) and is checked against
// independent known answers committed under tests/golden/: free-fermion
// closed forms, dense exact diagonalisation with explicit Jordan-Wigner
// strings, scipy eigsh energies, and structural counts (dim, nnz).
//
// Arithmetic: complex products are written out as (ac - bd, ad + bc) with
// separate roundings, which is what GCC emits for std::complex<double> on
// x86-64 (no FMA in the baseline ISA).  Build with -ffp-contract=off so that
// aarch64 hosts give the same bits.
//
// Eigen3 routines the reference calls are restated from their published
// algorithms:
//   * SparseMatrix::setFromTriplets: duplicates summed in insertion order,
//     rows sorted per column; sparse sum keeps the union pattern (explicit
//     zeros stay).
//   * SelfAdjointEigenSolver on the Lanczos matrix: the lower triangle is
//     already real tridiagonal, so it reduces to a symmetric tridiagonal
//     eigenproblem; solved here by implicit QL with Wilkinson shifts
//     (Golub & Van Loan, Matrix Computations, sec. 8.3).
//   * MatrixExp (unsupported/MatrixFunctions): scaling and squaring with
//     Pade approximants of degree 3/5/7/9/13 (Higham, SIAM J. Matrix Anal.
//     Appl. 26 (2005) 1179-1193).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <limits>
#include <unordered_map>
#include <vector>

#include "../include/qudrip_gb300.h"

using cd = std::complex<double>;

namespace {

const double kEps = 1e-10;  // qudrip.hpp:18

inline int popc(uint64_t x) { return __builtin_popcountll(x); }

// Complex product with the rounding sequence of GCC's std::complex<double>
// multiply: re = a.r*b.r - a.i*b.i, im = a.r*b.i + a.i*b.r.
inline cd cmul(cd a, cd b) {
  double rr = a.real() * b.real() - a.imag() * b.imag();
  double ri = a.real() * b.imag() + a.imag() * b.real();
  return cd(rr, ri);
}
inline cd cadd(cd a, cd b) { return cd(a.real() + b.real(), a.imag() + b.imag()); }
inline cd csub(cd a, cd b) { return cd(a.real() - b.real(), a.imag() - b.imag()); }
// real * complex (std::complex operator*(double, complex)): component-wise.
inline cd rmul(double r, cd b) { return cd(r * b.real(), r * b.imag()); }
// conj(a) * b
inline cd cdotmul(cd a, cd b) {
  double rr = a.real() * b.real() + a.imag() * b.imag();
  double ri = a.real() * b.imag() - a.imag() * b.real();
  return cd(rr, ri);
}

}  // namespace

// ===========================================================================
// Sectors: conservation.hpp:89-157 (quantities), 200-231 (LooseConstrain),
// index.hpp:187-261 (SubIndex mapping / inv_mapping).
// ===========================================================================
struct qdo_sector {
  int nbits;
  std::vector<uint64_t> mapping;                   // index.hpp:208
  std::unordered_map<uint64_t, int64_t> inv_mapping;  // index.hpp:209
};

static int64_t cq_value(const qd_cq_term& t, uint64_t s) {
  if (t.kind == QD_CQ_NSET) return popc(s & t.mask);  // conservation.hpp:110-112
  // Nd::eval, conservation.hpp:141-144
  uint64_t mask = t.hole ? ((t.nsite >= 64) ? ~0ull : ((1ull << t.nsite) - 1)) : 0ull;
  uint64_t sh = (t.nsite >= 64) ? 0ull : (s >> t.nsite);
  return popc((sh ^ mask) & (s ^ mask));
}

// Evaluate<tight>, conservation.hpp:209-218: |int(cq - val)| <= tight for all.
static bool cq_accept(const qd_constraint* cons, int ncons, int tight, uint64_t s) {
  for (int c = 0; c < ncons; ++c) {
    int64_t q = 0;
    for (int k = 0; k < cons[c].nterms; ++k)
      q += (int64_t)cons[c].term[k].coef * cq_value(cons[c].term[k], s);
    int d = (int)(q - cons[c].target);
    if (std::abs(d) > tight) return false;
  }
  return true;
}

extern "C" {

qdo_sector* qdo_sector_create(int nbits, const qd_constraint* cons, int ncons, int tight) {
  if (nbits < 1 || nbits > 40) return nullptr;
  auto* s = new qdo_sector();
  s->nbits = nbits;
  const uint64_t range = 1ull << nbits;
  // LooseConstrain scan, conservation.hpp:212-225:
  // ascending over the full index, append every accepted state.
  for (uint64_t x = 0; x < range; ++x) {
    if (ncons == 0 || cq_accept(cons, ncons, tight, x)) {
      s->mapping.push_back(x);
      s->inv_mapping.insert({x, (int64_t)s->mapping.size() - 1});
    }
  }
  return s;
}

int64_t qdo_sector_dim(const qdo_sector* s) { return (int64_t)s->mapping.size(); }

void qdo_sector_basis(const qdo_sector* s, uint64_t* out) {
  std::memcpy(out, s->mapping.data(), s->mapping.size() * sizeof(uint64_t));
}

// SubIndex::operator idxv_type, index.hpp:234-240: range() when absent.
int64_t qdo_sector_rank(const qdo_sector* s, uint64_t state) {
  auto it = s->inv_mapping.find(state);
  return it == s->inv_mapping.end() ? (int64_t)s->mapping.size() : it->second;
}

void qdo_sector_free(qdo_sector* s) { delete s; }

}  // extern "C"

// ===========================================================================
// Tree expansion and lowering.
//   full_branch: operator.hpp:135-206 (ops applied last to first, breadth
//     first; a null node (index 0) only has null children).
//   bitOp::branch: operators/bit.hpp:49-85.
//   hopBitOp::branch: operators/hopbit.hpp:43-84.
//   Operator::operator>>: operator.hpp:235-267 (leaf filter, triplets,
//     setFromTriplets).
//   OperatorSum::operator>>: operator_abel.hpp:25-34 (result += c * M_t).
// ===========================================================================
namespace {

struct Node {
  bool valid;
  uint64_t s;
  cd v;
};

// Expand one product of gates from input state s with root value init.
void expand_term(const qd_gate* g, int ngates, uint64_t s, cd init, std::vector<Node>& cur,
                 std::vector<Node>& nxt) {
  cur.clear();
  cur.push_back({true, s, init});
  for (int ig = ngates - 1; ig >= 0; --ig) {
    const qd_gate& G = g[ig];
    nxt.clear();
    for (const Node& n : cur) {
      if (G.kind == QD_GATE_BIT) {
        if (!n.valid) {
          nxt.push_back({false, 0, cd(0, 0)});
          nxt.push_back({false, 0, cd(0, 0)});
          continue;
        }
        const int site = G.site;
        const int b = (int)((n.s >> site) & 1ull);
        const uint64_t above = (site + 1 >= 64) ? 0ull : (n.s >> (site + 1));
        const cd jw = (popc(above) % 2) ? cd((double)G.string, 0.0) : cd(1.0, 0.0);
        const cd u0(G.u[2 * (b * 2 + 0)], G.u[2 * (b * 2 + 0) + 1]);
        const cd u1(G.u[2 * (b * 2 + 1)], G.u[2 * (b * 2 + 1) + 1]);
        const cd v0 = cmul(cmul(jw, u0), n.v);
        const cd v1 = cmul(cmul(jw, u1), n.v);
        nxt.push_back({true, n.s & ~(1ull << site), v0});
        nxt.push_back({true, n.s | (1ull << site), v1});
      } else {  // QD_GATE_HOP: gate(a, b) = creation at a, annihilation at b
        if (!n.valid) {
          nxt.push_back({false, 0, cd(0, 0)});
          continue;
        }
        const int sa = G.site;    // site2_ in hopBitOp
        const int sb = G.site_b;  // site1_ in hopBitOp
        if (sa == sb) {
          const double occ = (double)((n.s >> sb) & 1ull);
          nxt.push_back({true, n.s, rmul(occ, n.v)});
        } else if (((n.s >> sb) & 1ull) == 1ull && ((n.s >> sa) & 1ull) == 0ull) {
          uint64_t x = n.s;
          const int jw1 = popc((sb + 1 >= 64) ? 0ull : (x >> (sb + 1)));
          x &= ~(1ull << sb);
          const int jw2 = popc((sa + 1 >= 64) ? 0ull : (x >> (sa + 1)));
          x |= (1ull << sa);
          const int jw = ((jw1 % 2) ? G.string : 1) * ((jw2 % 2) ? G.string : 1);
          nxt.push_back({true, x, cmul(cd((double)jw, 0.0), n.v)});
        } else {
          nxt.push_back({false, 0, cd(0, 0)});
        }
      }
    }
    cur.swap(nxt);
  }
}

}  // namespace

struct qdo_ham {
  int64_t dim = 0;
  std::vector<int64_t> colptr;
  std::vector<int32_t> rowidx;
  std::vector<cd> vals;
};

extern "C" {

// Returns nullptr and *status != 0 on invalid input.
qdo_ham* qdo_ham_lower(const qdo_sector* sec, const qd_term* terms, int nterms,
                       const qd_gate* gates, int ngates, int* status) {
  *status = 0;
  for (int t = 0; t < nterms; ++t) {
    if (terms[t].gate_offset < 0 || terms[t].ngates < 0 ||
        terms[t].gate_offset + terms[t].ngates > ngates) {
      *status = QD_ERR_INVALID;
      return nullptr;
    }
  }
  for (int g = 0; g < ngates; ++g) {
    if (gates[g].site < 0 || gates[g].site >= sec->nbits || gates[g].kind < 0 || gates[g].kind > 1 ||
        (gates[g].kind == QD_GATE_HOP && (gates[g].site_b < 0 || gates[g].site_b >= sec->nbits))) {
      *status = QD_ERR_INVALID;
      return nullptr;
    }
  }
  auto* H = new qdo_ham();
  const int64_t dim = (int64_t)sec->mapping.size();
  H->dim = dim;
  H->colptr.assign(dim + 1, 0);
  std::vector<Node> cur, nxt;
  std::vector<std::pair<int64_t, cd>> term_rows;  // setFromTriplets dedupe for one column
  std::vector<std::pair<int64_t, cd>> col;        // union accumulator, unsorted
  for (int64_t i = 0; i < dim; ++i) {
    const uint64_t s = sec->mapping[i];
    col.clear();
    for (int t = 0; t < nterms; ++t) {
      expand_term(gates + terms[t].gate_offset, terms[t].ngates, s, cd(1.0, 0.0), cur, nxt);
      term_rows.clear();
      for (const Node& n : cur) {
        if (!n.valid) continue;
        if (!(std::abs(n.v) > kEps)) continue;  // operator.hpp:255
        const int64_t r = qdo_sector_rank(sec, n.s);
        if (r >= dim) continue;  // leaf outside the sector (operator.hpp:196-199)
        bool found = false;
        for (auto& tr : term_rows)
          if (tr.first == r) {
            tr.second = cadd(tr.second, n.v);  // duplicates: first + next, in leaf order
            found = true;
            break;
          }
        if (!found) term_rows.push_back({r, n.v});
      }
      const cd c(terms[t].coeff_re, terms[t].coeff_im);
      for (const auto& tr : term_rows) {
        const cd p = cmul(c, tr.second);  // coeffs_[i] * (ops_[i] >> index)
        bool found = false;
        for (auto& e : col)
          if (e.first == tr.first) {
            e.second = cadd(e.second, p);  // result + term on the union pattern
            found = true;
            break;
          }
        if (!found) col.push_back({tr.first, cadd(cd(0.0, 0.0), p)});
      }
    }
    std::sort(col.begin(), col.end(),
              [](const std::pair<int64_t, cd>& a, const std::pair<int64_t, cd>& b) { return a.first < b.first; });
    for (const auto& e : col) {
      H->rowidx.push_back((int32_t)e.first);
      H->vals.push_back(e.second);
    }
    H->colptr[i + 1] = (int64_t)H->rowidx.size();
  }
  return H;
}

int64_t qdo_ham_dim(const qdo_ham* H) { return H->dim; }
int64_t qdo_ham_nnz(const qdo_ham* H) { return (int64_t)H->rowidx.size(); }

void qdo_ham_csc(const qdo_ham* H, int64_t* colptr, int32_t* rowidx, double* vals) {
  std::memcpy(colptr, H->colptr.data(), H->colptr.size() * sizeof(int64_t));
  std::memcpy(rowidx, H->rowidx.data(), H->rowidx.size() * sizeof(int32_t));
  std::memcpy(vals, H->vals.data(), H->vals.size() * sizeof(cd));
}

void qdo_ham_free(qdo_ham* H) { delete H; }

}  // extern "C"

// ===========================================================================
// Dense-vector kernels with Eigen's evaluation order where it is observable.
// ===========================================================================
namespace {

// Column-major sparse * dense vector (Eigen sparse_time_dense_product, ColMajor):
// for each column j: rhs_j = 1 * x[j]; for each stored row r: y[r] += v * rhs_j.
void spmv_csc(const qdo_ham* H, const cd* x, cd* y) {
  const int64_t n = H->dim;
  for (int64_t r = 0; r < n; ++r) y[r] = cd(0.0, 0.0);
  for (int64_t j = 0; j < n; ++j) {
    const cd xj = cmul(cd(1.0, 0.0), x[j]);
    for (int64_t k = H->colptr[j]; k < H->colptr[j + 1]; ++k) {
      const int32_t r = H->rowidx[k];
      y[r] = cadd(y[r], cmul(H->vals[k], xj));
    }
  }
}

cd dotc(const cd* a, const cd* b, int64_t n) {  // a^dagger b, sequential sum
  cd s(0.0, 0.0);
  for (int64_t i = 0; i < n; ++i) s = cadd(s, cdotmul(a[i], b[i]));
  return s;
}

double norm2(const cd* a, int64_t n) { return dotc(a, a, n).real(); }  // Hermitian::norm

// State::eval (state.hpp:41-43): (psi^dagger * H) * psi, left to right.  The
// row vector psi^dagger H of a column-major H is formed column by column.
cd eval_left(const qdo_ham* H, const cd* psi) {
  cd e(0.0, 0.0);
  for (int64_t j = 0; j < H->dim; ++j) {
    cd u(0.0, 0.0);
    for (int64_t k = H->colptr[j]; k < H->colptr[j + 1]; ++k)
      u = cadd(u, cdotmul(psi[H->rowidx[k]], H->vals[k]));
    e = cadd(e, cmul(u, psi[j]));
  }
  return e;
}

}  // namespace

// ===========================================================================
// Symmetric tridiagonal eigensolver: implicit QL with Wilkinson shifts.
// d: diagonal (n), e: sub-diagonal (n-1).  Eigenvalues ascending; z (n*n,
// column-major, may be null) receives the eigenvectors as columns.
// ===========================================================================
extern "C" int qdo_tridiag_eig(int n, const double* d_in, const double* e_in, double* evals, double* z_out) {
  std::vector<double> d(d_in, d_in + n), e(n, 0.0), z;
  for (int i = 0; i + 1 < n; ++i) e[i] = e_in[i];
  const bool want = z_out != nullptr;
  if (want) {
    z.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) z[(size_t)i * n + i] = 1.0;
  }
  const double tiny = std::numeric_limits<double>::epsilon();
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    for (;;) {
      int m = l;
      for (; m < n - 1; ++m) {
        const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= tiny * dd) break;
      }
      if (m == l) break;
      if (++iter > 200) return -1;
      // Wilkinson-type shift from the leading 2x2 block at l.
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + (g >= 0 ? r : -r));
      double s = 1.0, c = 1.0, p = 0.0;
      int i = m - 1;
      bool early = false;
      for (; i >= l; --i) {
        const double f = s * e[i];
        const double b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {  // deflation inside the sweep
          d[i + 1] -= p;
          e[m] = 0.0;
          early = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        if (want) {
          for (int k = 0; k < n; ++k) {
            const double zf = z[(size_t)(i + 1) * n + k];
            const double zi = z[(size_t)i * n + k];
            z[(size_t)(i + 1) * n + k] = s * zi + c * zf;
            z[(size_t)i * n + k] = c * zi - s * zf;
          }
        }
      }
      if (early) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  // ascending order (selection sort keeps it simple and stable for small n)
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return d[a] < d[b]; });
  for (int i = 0; i < n; ++i) evals[i] = d[idx[i]];
  if (want)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k) z_out[(size_t)j * n + k] = z[(size_t)idx[j] * n + k];
  return 0;
}

// ===========================================================================
// Lanczos ground state: ArnoldiSolver<T, herm=1> on a fresh solver.
//   initKrylov sparse_algorithm.hpp:514-519, expandBasis<1> :395-425,
//   updateKrylovRepr :521-546, getGroundState :564-585, getState<1> :458-473.
// ===========================================================================
namespace {

// One step of expandBasis<1> with idx = step: V[idx%3] = H V[(idx-1)%3], local
// orthogonalisation against the two previous slots, normalise.  Returns n.
double lanczos_step(const qdo_ham* H, std::vector<cd>* V, int idx, std::vector<cd>& hvals,
                    int64_t& matvecs) {
  const int64_t n = H->dim;
  const int i0 = idx % 3, im1 = (idx - 1) % 3, im2 = (idx - 2) % 3;  // C++ % keeps sign
  spmv_csc(H, V[im1].data(), V[i0].data());
  ++matvecs;
  for (int i = 0; i < idx - 2; ++i) hvals.push_back(cd(0.0, 0.0));
  if (im2 >= 0) {
    const cd hb = dotc(V[im2].data(), V[i0].data(), n);
    for (int64_t k = 0; k < n; ++k) V[i0][k] = csub(V[i0][k], cmul(hb, V[im2][k]));
    hvals.push_back(hb);
  }
  const cd ha = dotc(V[im1].data(), V[i0].data(), n);
  for (int64_t k = 0; k < n; ++k) V[i0][k] = csub(V[i0][k], cmul(ha, V[im1][k]));
  hvals.push_back(ha);
  const double nrm = std::sqrt(norm2(V[i0].data(), n));
  for (int64_t k = 0; k < n; ++k) V[i0][k] = cd(V[i0][k].real() / nrm, V[i0][k].imag() / nrm);
  hvals.push_back(cd(nrm, 0.0));
  return nrm;
}

}  // namespace

extern "C" int qdo_lanczos_ground(const qdo_ham* H, const double* psi0, int kry_dim, double* psi_out,
                                  double* evals_out, int* act_dim_out, double* ritz_out, double* err_out,
                                  int* breakdown_out, int64_t* matvecs_out, double* energy_out) {
  const int64_t n = H->dim;
  if (kry_dim < 1 || n < 1) return QD_ERR_INVALID;
  std::vector<cd> V[3];
  for (auto& v : V) v.assign(n, cd(0.0, 0.0));
  const cd* p0 = reinterpret_cast<const cd*>(psi0);
  // initKrylov
  const double nrm0 = std::sqrt(norm2(p0, n));
  for (int64_t k = 0; k < n; ++k) V[0][k] = cd(p0[k].real() / nrm0, p0[k].imag() / nrm0);
  std::vector<cd> V0 = V[0];
  // updateKrylovRepr(H, -1): add_dim = kry_dim, start = 0
  std::vector<cd> hvals;
  int64_t matvecs = 0;
  int idx;
  int breakdown = 0;
  for (idx = 1; idx <= kry_dim; ++idx) {
    const double nr = lanczos_step(H, V, idx, hvals, matvecs);
    if (nr < kEps) {
      breakdown = 1;
      break;
    }
  }
  const int act = idx - 1;  // expandBasis<1> return value
  if (act < 1) return QD_ERR_BREAKDOWN;
  // Fill KR as updateKrylovRepr does: column i receives h entries j = 0..i+1.
  std::vector<cd> KR((size_t)kry_dim * kry_dim, cd(0.0, 0.0));
  size_t hp = 0;
  for (int i = 0; i < act - 1; ++i)
    for (int j = 0; j <= i + 1; ++j) KR[(size_t)i * kry_dim + j] = hvals[hp++];
  for (int j = 0; j <= act - 1; ++j) KR[(size_t)(act - 1) * kry_dim + j] = hvals[hp++];
  // SelfAdjointEigenSolver reads the lower triangle: real diagonal, sub-diagonal.
  std::vector<double> d(act), e(act > 1 ? act - 1 : 1), ev(act), z((size_t)act * act);
  for (int i = 0; i < act; ++i) d[i] = KR[(size_t)i * kry_dim + i].real();
  for (int i = 0; i + 1 < act; ++i) e[i] = KR[(size_t)i * kry_dim + i + 1].real();
  if (qdo_tridiag_eig(act, d.data(), e.data(), ev.data(), z.data()) != 0) return QD_ERR_INVALID;
  // getState<herm 1>: rebuild the basis one step at a time, psi = sum y_k v_k.
  std::vector<cd> psi(n);
  for (auto& v : V) std::fill(v.begin(), v.end(), cd(0.0, 0.0));
  V[0] = V0;
  for (int64_t k = 0; k < n; ++k) psi[k] = cmul(cd(z[0], 0.0), V[0][k]);
  std::vector<cd> hdummy;
  for (int i = 1; i < act; ++i) {
    lanczos_step(H, V, i, hdummy, matvecs);
    const cd yi(z[i], 0.0);
    for (int64_t k = 0; k < n; ++k) psi[k] = cadd(psi[k], cmul(yi, V[i % 3][k]));
  }
  lanczos_step(H, V, act, hdummy, matvecs);  // the trailing expandBasis of getState<1>
  std::memcpy(psi_out, psi.data(), n * sizeof(cd));
  if (evals_out) std::memcpy(evals_out, ev.data(), act * sizeof(double));
  *act_dim_out = act;
  *ritz_out = ev[0];
  *err_out = std::fabs(ev[0]);  // previous evs_ taken as zero on a fresh solver
  *breakdown_out = breakdown;
  if (matvecs_out) *matvecs_out = matvecs;
  if (energy_out) {
    const cd E = eval_left(H, psi.data());
    energy_out[0] = E.real();
    energy_out[1] = E.imag();
  }
  return 0;
}

// y = H x (complex interleaved) and psi.eval.
extern "C" void qdo_spmv(const qdo_ham* H, const double* x, double* y) {
  spmv_csc(H, reinterpret_cast<const cd*>(x), reinterpret_cast<cd*>(y));
}
extern "C" void qdo_eval(const qdo_ham* H, const double* psi, double* out) {
  const cd e = eval_left(H, reinterpret_cast<const cd*>(psi));
  out[0] = e.real();
  out[1] = e.imag();
}

// ===========================================================================
// Matrix exponential: scaling and squaring with diagonal Pade approximants
// (Higham 2005).  A, E: n x n complex, column-major.
// ===========================================================================
namespace {

using CMat = std::vector<cd>;

CMat mm(const CMat& A, const CMat& B, int n) {
  CMat C((size_t)n * n, cd(0.0, 0.0));
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k) {
      const cd b = B[(size_t)j * n + k];
      for (int i = 0; i < n; ++i) C[(size_t)j * n + i] += A[(size_t)k * n + i] * b;
    }
  return C;
}

// Solve P X = Q (n x n) by LU with partial pivoting.
bool lu_solve(CMat P, CMat Q, int n, CMat& X) {
  for (int k = 0; k < n; ++k) {
    int piv = k;
    double best = std::abs(P[(size_t)k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (std::abs(P[(size_t)k * n + i]) > best) {
        best = std::abs(P[(size_t)k * n + i]);
        piv = i;
      }
    if (best == 0.0) return false;
    if (piv != k) {
      for (int j = 0; j < n; ++j) std::swap(P[(size_t)j * n + k], P[(size_t)j * n + piv]);
      for (int j = 0; j < n; ++j) std::swap(Q[(size_t)j * n + k], Q[(size_t)j * n + piv]);
    }
    const cd inv = 1.0 / P[(size_t)k * n + k];
    for (int i = k + 1; i < n; ++i) {
      const cd f = P[(size_t)k * n + i] * inv;
      P[(size_t)k * n + i] = f;
      for (int j = k + 1; j < n; ++j) P[(size_t)j * n + i] -= f * P[(size_t)j * n + k];
      for (int j = 0; j < n; ++j) Q[(size_t)j * n + i] -= f * Q[(size_t)j * n + k];
    }
  }
  for (int j = 0; j < n; ++j)
    for (int i = n - 1; i >= 0; --i) {
      cd s = Q[(size_t)j * n + i];
      for (int k = i + 1; k < n; ++k) s -= P[(size_t)k * n + i] * Q[(size_t)j * n + k];
      Q[(size_t)j * n + i] = s / P[(size_t)i * n + i];
    }
  X = Q;
  return true;
}

// Coefficients of the [m/m] Pade approximant of exp: c_k = (2m-k)! m! / ((2m)! k! (m-k)!).
std::vector<double> pade_coeffs(int m) {
  std::vector<double> c(m + 1);
  c[0] = 1.0;
  for (int k = 1; k <= m; ++k) c[k] = c[k - 1] * (double)(m - k + 1) / ((double)(2 * m - k + 1) * (double)k);
  return c;
}

}  // namespace

extern "C" int qdo_expm(int n, const double* A_in, double* E_out) {
  const cd* Ain = reinterpret_cast<const cd*>(A_in);
  CMat A(Ain, Ain + (size_t)n * n);
  double nrm1 = 0.0;
  for (int j = 0; j < n; ++j) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += std::abs(A[(size_t)j * n + i]);
    nrm1 = std::max(nrm1, s);
  }
  // theta_m for double precision, Higham 2005 Table 2.3.
  const double th3 = 1.495585217958292e-2, th5 = 2.539398330063230e-1, th7 = 9.504178996162932e-1,
               th9 = 2.097847961257068e0, th13 = 5.371920351148152e0;
  int m, s = 0;
  if (nrm1 <= th3) m = 3;
  else if (nrm1 <= th5) m = 5;
  else if (nrm1 <= th7) m = 7;
  else if (nrm1 <= th9) m = 9;
  else {
    m = 13;
    s = std::max(0, (int)std::ceil(std::log2(nrm1 / th13)));
    const double scale = std::ldexp(1.0, -s);
    for (auto& a : A) a *= scale;
  }
  const std::vector<double> c = pade_coeffs(m);
  CMat I((size_t)n * n, cd(0.0, 0.0));
  for (int i = 0; i < n; ++i) I[(size_t)i * n + i] = 1.0;
  // powers A^2, A^4, A^6 (A^8 for m = 9)
  std::vector<CMat> P(m + 1);
  P[0] = I;
  P[2] = mm(A, A, n);
  for (int k = 4; k <= std::min(m, 8); k += 2) P[k] = mm(P[k - 2], P[2], n);
  CMat U((size_t)n * n, cd(0.0, 0.0)), V((size_t)n * n, cd(0.0, 0.0));
  if (m < 13) {
    CMat Uin((size_t)n * n, cd(0.0, 0.0));
    for (int k = 1; k <= m; k += 2)
      for (size_t q = 0; q < Uin.size(); ++q) Uin[q] += c[k] * P[k - 1][q];
    U = mm(A, Uin, n);
    for (int k = 0; k <= m; k += 2)
      for (size_t q = 0; q < V.size(); ++q) V[q] += c[k] * P[k][q];
  } else {
    const CMat& A2 = P[2];
    const CMat& A4 = P[4];
    const CMat& A6 = P[6];
    CMat t1((size_t)n * n), t2((size_t)n * n);
    for (size_t q = 0; q < t1.size(); ++q) {
      t1[q] = c[13] * A6[q] + c[11] * A4[q] + c[9] * A2[q];
      t2[q] = c[12] * A6[q] + c[10] * A4[q] + c[8] * A2[q];
    }
    CMat u1 = mm(A6, t1, n), v1 = mm(A6, t2, n);
    for (size_t q = 0; q < u1.size(); ++q) {
      u1[q] += c[7] * A6[q] + c[5] * A4[q] + c[3] * A2[q] + c[1] * I[q];
      V[q] = v1[q] + c[6] * A6[q] + c[4] * A4[q] + c[2] * A2[q] + c[0] * I[q];
    }
    U = mm(A, u1, n);
  }
  CMat Pm((size_t)n * n), Qm((size_t)n * n), X;
  for (size_t q = 0; q < Pm.size(); ++q) {
    Pm[q] = V[q] - U[q];
    Qm[q] = V[q] + U[q];
  }
  if (!lu_solve(Pm, Qm, n, X)) return QD_ERR_INVALID;
  for (int k = 0; k < s; ++k) X = mm(X, X, n);
  std::memcpy(E_out, X.data(), X.size() * sizeof(cd));
  return 0;
}

// ===========================================================================
// Krylov real-time step: ArnoldiSolver<T, herm=0>::evolve(H, psi, t, h, m)
//   expandBasis<0> sparse_algorithm.hpp:372-393 (modified Gram-Schmidt over
//   all previous vectors), updateKrylovRepr :521-546, evolve :548-562.
// psi_out = V[:, 0:a] * exp(-i K[0:a,0:a] h)[:, 0]  with a = act_dim.
// ===========================================================================
extern "C" int qdo_arnoldi_evolve(const qdo_ham* H, const double* psi_in, double h, int m, double* psi_out,
                                  int* act_dim_out, int64_t* matvecs_out) {
  const int64_t n = H->dim;
  if (m < 2) return QD_ERR_INVALID;
  const int kdim = m;  // solver kry_dim; V has kry_dim + 1 columns
  std::vector<std::vector<cd>> V(kdim + 1, std::vector<cd>(n, cd(0.0, 0.0)));
  const cd* p = reinterpret_cast<const cd*>(psi_in);
  const double nrm0 = std::sqrt(norm2(p, n));
  for (int64_t k = 0; k < n; ++k) V[0][k] = cd(p[k].real() / nrm0, p[k].imag() / nrm0);
  std::vector<cd> hv;
  int64_t matvecs = 0;
  const int add_dim = m - 1;
  int idx;
  for (idx = 1; idx <= add_dim; ++idx) {
    spmv_csc(H, V[idx - 1].data(), V[idx].data());
    ++matvecs;
    for (int i = 0; i < idx; ++i) {
      const cd nh = dotc(V[i].data(), V[idx].data(), n);
      for (int64_t k = 0; k < n; ++k) V[idx][k] = csub(V[idx][k], cmul(nh, V[i][k]));
      hv.push_back(nh);
    }
    const double nr = std::sqrt(norm2(V[idx].data(), n));
    for (int64_t k = 0; k < n; ++k) V[idx][k] = cd(V[idx][k].real() / nr, V[idx][k].imag() / nr);
    hv.push_back(cd(nr, 0.0));
    if (nr < kEps) {
      ++idx;
      break;
    }
  }
  const int act = idx - 1;
  std::vector<cd> K((size_t)act * act, cd(0.0, 0.0));
  size_t hp = 0;
  for (int i = 0; i < act - 1; ++i)
    for (int j = 0; j <= i + 1; ++j) K[(size_t)i * act + j] = hv[hp++];
  for (int j = 0; j <= act - 1; ++j) K[(size_t)(act - 1) * act + j] = hv[hp++];
  // exp(-i K h)
  std::vector<cd> A((size_t)act * act), E((size_t)act * act);
  const cd mih(0.0, -h);
  for (size_t q = 0; q < A.size(); ++q) A[q] = mih * K[q];
  if (qdo_expm(act, reinterpret_cast<const double*>(A.data()), reinterpret_cast<double*>(E.data())) != 0)
    return QD_ERR_INVALID;
  cd* out = reinterpret_cast<cd*>(psi_out);
  for (int64_t k = 0; k < n; ++k) {
    cd s(0.0, 0.0);
    for (int j = 0; j < act; ++j) s += V[j][k] * E[j];
    out[k] = s;
  }
  *act_dim_out = act;
  if (matvecs_out) *matvecs_out = matvecs;
  return 0;
}

// ===========================================================================
// Arnoldi ground state: Arnoldi::getSolver(index, kry_dim).getGroundState(H,
// psi, t[, add_dim]) -- ArnoldiSolver<T, herm=0> (sparse_algorithm.hpp:475-604):
//   initKrylov :514-519; updateKrylovRepr :521-546 with expandBasis<0>
//   :372-393 (modified Gram-Schmidt of H v_{idx-1} against every previous
//   vector; stop at ||w|| < eps keeping the breaking step); getGroundState
//   :564-585 runs SelfAdjointEigenSolver on KR[0:act, 0:act], which reads the
//   lower triangle only: the real parts of the diagonal <v_i, H v_i> and the
//   sub-diagonal norms (real), i.e. a symmetric tridiagonal matrix (its
//   Householder step is the identity there); getState<herm 0> :447-453 forms
//   psi = V[:, 0:act] z_0 from the lowest eigenvector z_0.
// A solve grown by several calls of add_dim steps each performs the same
// operations in the same order as one call of their total (expandBasis<0>
// continues from the stored basis), so `steps` here is the dimension reached.
// ===========================================================================
extern "C" int qdo_arnoldi_ground(const qdo_ham* H, const double* psi0, int steps, double* psi_out,
                                  double* evals_out, int* act_dim_out, int64_t* matvecs_out, double* energy_out) {
  const int64_t n = H->dim;
  if (steps < 1 || n < 1) return QD_ERR_INVALID;
  std::vector<std::vector<cd>> V(steps + 1, std::vector<cd>(n, cd(0.0, 0.0)));
  const cd* p = reinterpret_cast<const cd*>(psi0);
  const double nrm0 = std::sqrt(norm2(p, n));
  for (int64_t k = 0; k < n; ++k) V[0][k] = cd(p[k].real() / nrm0, p[k].imag() / nrm0);
  std::vector<cd> hv;
  int64_t matvecs = 0;
  int idx;
  for (idx = 1; idx <= steps; ++idx) {
    spmv_csc(H, V[idx - 1].data(), V[idx].data());
    ++matvecs;
    for (int i = 0; i < idx; ++i) {
      const cd nh = dotc(V[i].data(), V[idx].data(), n);
      for (int64_t k = 0; k < n; ++k) V[idx][k] = csub(V[idx][k], cmul(nh, V[i][k]));
      hv.push_back(nh);
    }
    const double nr = std::sqrt(norm2(V[idx].data(), n));
    for (int64_t k = 0; k < n; ++k) V[idx][k] = cd(V[idx][k].real() / nr, V[idx][k].imag() / nr);
    hv.push_back(cd(nr, 0.0));
    if (nr < kEps) {
      ++idx;
      break;
    }
  }
  const int act = idx - 1;
  // KR column i: h entries j = 0..i+1 (j = i+1 is the norm), the last column j = 0..act-1
  std::vector<cd> KR((size_t)act * (act + 1), cd(0.0, 0.0));
  size_t hp = 0;
  for (int i = 0; i < act - 1; ++i)
    for (int j = 0; j <= i + 1; ++j) KR[(size_t)i * (act + 1) + j] = hv[hp++];
  for (int j = 0; j <= act - 1; ++j) KR[(size_t)(act - 1) * (act + 1) + j] = hv[hp++];
  std::vector<double> d(act), e(act > 1 ? act - 1 : 1), ev(act), z((size_t)act * act);
  for (int i = 0; i < act; ++i) d[i] = KR[(size_t)i * (act + 1) + i].real();
  for (int i = 0; i + 1 < act; ++i) e[i] = KR[(size_t)i * (act + 1) + i + 1].real();
  if (qdo_tridiag_eig(act, d.data(), e.data(), ev.data(), z.data()) != 0) return QD_ERR_INVALID;
  cd* out = reinterpret_cast<cd*>(psi_out);
  for (int64_t k = 0; k < n; ++k) {
    cd s(0.0, 0.0);
    for (int j = 0; j < act; ++j) s = cadd(s, cmul(V[j][k], cd(z[j], 0.0)));
    out[k] = s;
  }
  if (evals_out) std::memcpy(evals_out, ev.data(), act * sizeof(double));
  *act_dim_out = act;
  if (matvecs_out) *matvecs_out = matvecs;
  if (energy_out) {
    const cd E = eval_left(H, out);
    energy_out[0] = E.real();
    energy_out[1] = E.imag();
  }
  return 0;
}

// ===========================================================================
// Hermitian::LanczosSolver::getGroundState (sparse_algorithm.hpp:287-301):
// getKrylovReprAd (:72-122) builds tridiag(a, b) with two products per step,
// the dense eigensolver picks the lowest eigenvector, getKrylovGS (:206-238)
// rebuilds psi = sum GS(k) v_k in a second pass.
// ===========================================================================
namespace {

cd vhv(const qdo_ham* H, const std::vector<cd>& v, std::vector<cd>& tmp, int64_t& mv) {
  spmv_csc(H, v.data(), tmp.data());
  ++mv;
  return dotc(v.data(), tmp.data(), H->dim);
}

}  // namespace

extern "C" int qdo_hermitian_lanczos_ground(const qdo_ham* H, const double* psi0, int kry_dim, double* psi_out,
                                            double* evals_out, int* nev_out, double* err_out,
                                            int64_t* matvecs_out) {
  const int64_t n = H->dim;
  const cd* p = reinterpret_cast<const cd*>(psi0);
  std::vector<cd> v(n), w(n, cd(0.0, 0.0)), tmp(n), hv(n);
  int64_t mv = 0;
  const double n0 = std::sqrt(norm2(p, n));
  for (int64_t k = 0; k < n; ++k) v[k] = cd(p[k].real() / n0, p[k].imag() / n0);
  std::vector<cd> a;
  std::vector<double> b;
  a.push_back(vhv(H, v, tmp, mv));
  spmv_csc(H, v.data(), hv.data());
  ++mv;
  for (int64_t k = 0; k < n; ++k) w[k] = hv[k] - a[0] * v[k];
  double nn = norm2(w.data(), n);
  double sq = std::sqrt(nn);
  for (int64_t k = 0; k < n; ++k) w[k] /= sq;
  bool use_v = false;
  int idx = 1;
  while (nn > kEps) {
    if (use_v) {
      a.push_back(vhv(H, v, tmp, mv));
      b.push_back(std::sqrt(nn));
      spmv_csc(H, v.data(), hv.data());
      ++mv;
      const double sn = std::sqrt(nn);
      for (int64_t k = 0; k < n; ++k) w[k] = hv[k] - a.back() * v[k] - sn * w[k];
      nn = norm2(w.data(), n);
      sq = std::sqrt(nn);
      for (int64_t k = 0; k < n; ++k) w[k] /= sq;
    } else {
      a.push_back(vhv(H, w, tmp, mv));
      b.push_back(std::sqrt(nn));
      spmv_csc(H, w.data(), hv.data());
      ++mv;
      const double sn = std::sqrt(nn);
      for (int64_t k = 0; k < n; ++k) v[k] = hv[k] - a.back() * w[k] - sn * v[k];
      nn = norm2(v.data(), n);
      sq = std::sqrt(nn);
      for (int64_t k = 0; k < n; ++k) v[k] /= sq;
    }
    use_v = !use_v;
    ++idx;
    if (idx > kry_dim) break;
  }
  const int K = (int)a.size();
  std::vector<double> d(K), e(K > 1 ? K - 1 : 1), ev(K), z((size_t)K * K);
  for (int i = 0; i < K; ++i) d[i] = a[i].real();
  for (int i = 0; i + 1 < K; ++i) e[i] = b[i];
  if (qdo_tridiag_eig(K, d.data(), e.data(), ev.data(), z.data()) != 0) return QD_ERR_INVALID;
  // getKrylovGS second pass
  for (int64_t k = 0; k < n; ++k) v[k] = cd(p[k].real() / n0, p[k].imag() / n0);
  std::fill(w.begin(), w.end(), cd(0.0, 0.0));
  std::vector<cd> psi(n);
  for (int64_t k = 0; k < n; ++k) psi[k] = z[0] * v[k];
  double alpha = vhv(H, v, tmp, mv).real();
  spmv_csc(H, v.data(), hv.data());
  ++mv;
  for (int64_t k = 0; k < n; ++k) w[k] = hv[k] - alpha * v[k];
  nn = norm2(w.data(), n);
  sq = std::sqrt(nn);
  for (int64_t k = 0; k < n; ++k) w[k] /= sq;
  for (int i = 1; i < K; ++i) {
    const double sn = std::sqrt(nn);
    if (!(i % 2)) {
      for (int64_t k = 0; k < n; ++k) psi[k] += z[i] * v[k];
      alpha = vhv(H, v, tmp, mv).real();
      spmv_csc(H, v.data(), hv.data());
      ++mv;
      for (int64_t k = 0; k < n; ++k) w[k] = hv[k] - alpha * v[k] - sn * w[k];
      nn = norm2(w.data(), n);
      sq = std::sqrt(nn);
      for (int64_t k = 0; k < n; ++k) w[k] /= sq;
    } else {
      for (int64_t k = 0; k < n; ++k) psi[k] += z[i] * w[k];
      alpha = vhv(H, w, tmp, mv).real();
      spmv_csc(H, w.data(), hv.data());
      ++mv;
      for (int64_t k = 0; k < n; ++k) v[k] = hv[k] - alpha * w[k] - sn * v[k];
      nn = norm2(v.data(), n);
      sq = std::sqrt(nn);
      for (int64_t k = 0; k < n; ++k) v[k] /= sq;
    }
  }
  std::memcpy(psi_out, psi.data(), n * sizeof(cd));
  if (evals_out) std::memcpy(evals_out, ev.data(), K * sizeof(double));
  *nev_out = K;
  *err_out = std::sqrt(nn);
  if (matvecs_out) *matvecs_out = mv;
  return 0;
}

// ===========================================================================
// Quantum-jump trajectories: programs/hubbard_diss.cpp:439-482 (loop),
// :520-529 (lindblad_weight), :514-517 (QJ_operator), :565-577 (bsearch),
// for diagonal jump operators L_j = sqrt(gamma) n_{bit_j}.  Random numbers:
// Philox4x32-10 (Salmon et al., SC11) keyed by (seed) with counter
// (step, trajectory, 0, 0): two 53-bit uniforms per step, written out here
// independently of the engine's copy.  Each trajectory starts from psi0.
// The no-jump step evolves with H_eff + (i/2) gamma wtot I exactly as
// QJ_operator builds it; the shift is applied to the Hessenberg diagonal.
// ===========================================================================
namespace {

void philox_round10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t c0 = hi1 ^ c[1] ^ k0, c2 = hi0 ^ c[3] ^ k1;
    c[0] = c0;
    c[1] = lo1;
    c[2] = c2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

void uniform2(uint64_t seed, uint32_t traj, uint32_t step, double& u1, double& u2) {
  uint32_t c[4] = {step, traj, 0u, 0u};
  philox_round10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  u1 = ((double)(c[0] >> 5) * 67108864.0 + (double)(c[1] >> 6)) / 9007199254740992.0;
  u2 = ((double)(c[2] >> 5) * 67108864.0 + (double)(c[3] >> 6)) / 9007199254740992.0;
}

int bsearch_ref(const std::vector<double>& values, double val) {  // hubbard_diss.cpp:565-577
  if (val > values.back() || val < values[0]) return -1;
  int is = 0, ie = (int)values.size();
  while (ie - is > 1) {
    const int imid = is + (ie - is) / 2;
    if (val < values[imid]) ie = imid;
    else is = imid;
  }
  return is;
}

// ArnoldiSolver<T,0>::evolve with a diagonal shift c added to the Hessenberg
// matrix (the operator H + c I).
void evolve_shift(const qdo_ham* H, const cd* psi, double h, int m, cd c, cd* out) {
  const int64_t n = H->dim;
  std::vector<std::vector<cd>> V(m + 1, std::vector<cd>(n));
  const double nrm0 = std::sqrt(norm2(psi, n));
  for (int64_t k = 0; k < n; ++k) V[0][k] = psi[k] / nrm0;
  std::vector<cd> hv;
  int idx;
  for (idx = 1; idx <= m - 1; ++idx) {
    spmv_csc(H, V[idx - 1].data(), V[idx].data());
    for (int i = 0; i < idx; ++i) {
      const cd nh = dotc(V[i].data(), V[idx].data(), n);
      for (int64_t k = 0; k < n; ++k) V[idx][k] -= nh * V[i][k];
      hv.push_back(nh);
    }
    const double nr = std::sqrt(norm2(V[idx].data(), n));
    for (int64_t k = 0; k < n; ++k) V[idx][k] /= nr;
    hv.push_back(nr);
    if (nr < kEps) {
      ++idx;
      break;
    }
  }
  const int act = idx - 1;
  std::vector<cd> K((size_t)act * act, cd(0, 0));
  size_t hp = 0;
  for (int i = 0; i < act - 1; ++i)
    for (int j = 0; j <= i + 1; ++j) K[(size_t)i * act + j] = hv[hp++];
  for (int j = 0; j <= act - 1; ++j) K[(size_t)(act - 1) * act + j] = hv[hp++];
  for (int i = 0; i < act; ++i) K[(size_t)i * act + i] += c;
  std::vector<cd> A((size_t)act * act), E((size_t)act * act);
  for (size_t q = 0; q < A.size(); ++q) A[q] = cd(0.0, -h) * K[q];
  qdo_expm(act, reinterpret_cast<const double*>(A.data()), reinterpret_cast<double*>(E.data()));
  for (int64_t k = 0; k < n; ++k) {
    cd s(0, 0);
    for (int j = 0; j < act; ++j) s += V[j][k] * E[j];
    out[k] = s;
  }
}

}  // namespace

extern "C" int qdo_traj_run(const qdo_ham* Heff, const uint64_t* basis, int ntraj, int nsteps, double dt,
                            double gamma, uint64_t seed, int m, int nchan, const int* chan_bits, int nobs,
                            const int* obs_a, const int* obs_b, const double* psi0, double* obs_mean,
                            int64_t* jumps_out) {
  const int64_t n = Heff->dim;
  const cd* p0 = reinterpret_cast<const cd*>(psi0);
  std::vector<double> sums((size_t)(nsteps + 1) * nobs, 0.0);
  std::vector<cd> psi(n), nxt(n);
  int64_t jumps = 0;
  auto record = [&](int step) {
    const double nn = norm2(psi.data(), n);
    for (int k = 0; k < nobs; ++k) {
      const uint64_t mask = (1ull << obs_a[k]) | (1ull << obs_b[k]);
      double s = 0.0;
      for (int64_t i = 0; i < n; ++i)
        if ((basis[i] & mask) == mask) s += std::norm(psi[i]);
      sums[(size_t)step * nobs + k] += s / nn;
    }
  };
  for (int b = 0; b < ntraj; ++b) {
    const double nrm = std::sqrt(norm2(p0, n));
    for (int64_t i = 0; i < n; ++i) psi[i] = p0[i] / nrm;
    record(0);
    for (int step = 1; step <= nsteps; ++step) {
      std::vector<double> w(nchan, 0.0);
      for (int j = 0; j < nchan; ++j)
        for (int64_t i = 0; i < n; ++i)
          if ((basis[i] >> chan_bits[j]) & 1ull) w[j] += std::norm(psi[i]);
      std::vector<double> wt(nchan + 1, 0.0);
      for (int j = 1; j <= nchan; ++j) wt[j] = wt[j - 1] + w[j - 1];
      const double wtot = wt[nchan];
      for (int j = 0; j <= nchan; ++j) wt[j] /= wt[nchan];
      double u1, u2;
      uniform2(seed, (uint32_t)b, (uint32_t)step, u1, u2);
      if (u1 < gamma * wtot * dt) {
        const int idx = bsearch_ref(wt, u2);
        const uint64_t bit = 1ull << chan_bits[idx];
        for (int64_t i = 0; i < n; ++i) nxt[i] = (basis[i] & bit) ? psi[i] : cd(0, 0);
        ++jumps;
      } else {
        evolve_shift(Heff, psi.data(), dt, m, cd(0.0, 0.5 * gamma * wtot), nxt.data());
      }
      const double nn = std::sqrt(norm2(nxt.data(), n));
      for (int64_t i = 0; i < n; ++i) psi[i] = nxt[i] / nn;
      record(step);
    }
  }
  for (size_t q = 0; q < sums.size(); ++q) obs_mean[q] = sums[q] / ntraj;
  if (jumps_out) *jumps_out = jumps;
  return 0;
}
