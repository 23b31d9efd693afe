// tridiag.cuh -- symmetric tridiagonal eigensolver (implicit QL, Wilkinson
// shifts; Golub & Van Loan, Matrix Computations, sec. 8.3), usable on host
// and device.  Replaces the SelfAdjointEigenSolver call on the Lanczos
// matrix (sparse_algorithm.hpp:571): the matrix's lower triangle is already
// real tridiagonal, so Eigen's Householder step is the identity there.
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

namespace qd {

// d[0..n) diagonal, e[0..n-1) sub-diagonal (both overwritten; on return d
// holds the eigenvalues in ascending order).  If z != nullptr it must hold the
// n x n identity (column-major, leading dimension ldz) and receives the
// eigenvectors as columns, in the same order.  Returns 0 on success.
template <typename Real>
__host__ __device__ inline int tridiag_ql(int n, Real* d, Real* e, Real* z, int ldz) {
  if (n <= 0) return 0;
  e[n - 1] = 0;
  const Real tiny = (Real)2.220446049250313e-16;
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    for (;;) {
      int m = l;
      for (; m < n - 1; ++m) {
        const Real dd = fabs(d[m]) + fabs(d[m + 1]);
        if (fabs(e[m]) <= tiny * dd) break;
      }
      if (m == l) break;
      if (++iter > 300) return -1;
      Real g = (d[l + 1] - d[l]) / ((Real)2 * e[l]);
      Real r = hypot(g, (Real)1);
      g = d[m] - d[l] + e[l] / (g + (g >= 0 ? r : -r));
      Real s = 1, c = 1, p = 0;
      bool deflated = false;
      for (int i = m - 1; i >= l; --i) {
        const Real f = s * e[i];
        const Real b = c * e[i];
        r = hypot(f, g);
        e[i + 1] = r;
        if (r == 0) {
          d[i + 1] -= p;
          e[m] = 0;
          deflated = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + (Real)2 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        if (z) {
          Real* zi = z + (size_t)i * ldz;
          Real* zi1 = z + (size_t)(i + 1) * ldz;
          for (int k = 0; k < n; ++k) {
            const Real a = zi[k], bb = zi1[k];
            zi1[k] = s * a + c * bb;
            zi[k] = c * a - s * bb;
          }
        }
      }
      if (deflated) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0;
    }
  }
  // insertion sort ascending, permuting eigenvector columns along
  for (int i = 1; i < n; ++i) {
    const Real key = d[i];
    int j = i - 1;
    while (j >= 0 && d[j] > key) --j;
    ++j;
    if (j == i) continue;
    for (int q = i; q > j; --q) d[q] = d[q - 1];
    d[j] = key;
    if (z) {
      for (int k = 0; k < n; ++k) {
        const Real t = z[(size_t)i * ldz + k];
        for (int q = i; q > j; --q) z[(size_t)q * ldz + k] = z[(size_t)(q - 1) * ldz + k];
        z[(size_t)j * ldz + k] = t;
      }
    }
  }
  return 0;
}

// Lowest eigenpair only: run the QL sweeps without accumulating vectors,
// recording every plane rotation, then apply the rotations in reverse to the
// unit vector of the lowest eigenvalue's position.  The result equals the
// corresponding column of the accumulated eigenvector matrix (same
// rotations, different association of the products) at O(n^2) cost instead
// of O(n^3).  evals receives all eigenvalues ascending, y the eigenvector.
template <typename Real>
inline int tridiag_lowest(int n, Real* d, Real* e, Real* evals, Real* y) {
  struct Rot {
    int i;
    Real s, c;
  };
  std::vector<Rot> rots;
  rots.reserve((size_t)8 * n * n);
  if (n <= 0) return 0;
  e[n - 1] = 0;
  const Real tiny = (Real)2.220446049250313e-16;
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    for (;;) {
      int m = l;
      for (; m < n - 1; ++m) {
        const Real dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= tiny * dd) break;
      }
      if (m == l) break;
      if (++iter > 300) return -1;
      Real g = (d[l + 1] - d[l]) / ((Real)2 * e[l]);
      Real r = std::hypot(g, (Real)1);
      g = d[m] - d[l] + e[l] / (g + (g >= 0 ? r : -r));
      Real s = 1, c = 1, p = 0;
      bool deflated = false;
      for (int i = m - 1; i >= l; --i) {
        const Real f = s * e[i];
        const Real b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0) {
          d[i + 1] -= p;
          e[m] = 0;
          deflated = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + (Real)2 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        rots.push_back(Rot{i, s, c});
      }
      if (deflated) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0;
    }
  }
  int pos = 0;
  for (int i = 1; i < n; ++i)
    if (d[i] < d[pos]) pos = i;
  for (int i = 0; i < n; ++i) y[i] = (i == pos) ? (Real)1 : (Real)0;
  for (size_t q = rots.size(); q-- > 0;) {
    const Rot& R = rots[q];
    const Real a = y[R.i], b = y[R.i + 1];
    y[R.i] = R.c * a + R.s * b;
    y[R.i + 1] = -R.s * a + R.c * b;
  }
  for (int i = 0; i < n; ++i) evals[i] = d[i];
  std::sort(evals, evals + n);
  return 0;
}

}  // namespace qd
