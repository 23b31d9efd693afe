// dense.h -- small dense complex matrices on the host: products, LU solve and
// the matrix exponential.
//
// The exponential replaces Eigen's MatrixExp (matrix.hpp:20) on the Krylov
// Hessenberg matrix (at most a few dozen rows).  It follows the published
// scaling-and-squaring algorithm with diagonal Pade approximants of degree
// 3, 5, 7, 9 or 13 chosen from the 1-norm (N. J. Higham, SIAM J. Matrix
// Anal. Appl. 26 (2005) 1179-1193); the coefficients are computed from the
// Pade formula c_k = (2m-k)! m! / ((2m)! k! (m-k)!).
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

namespace qd {
namespace dense {

using cd = std::complex<double>;
using Mat = std::vector<cd>;  // column-major n x n

inline Mat identity(int n) {
  Mat I((size_t)n * n, cd(0.0, 0.0));
  for (int i = 0; i < n; ++i) I[(size_t)i * n + i] = 1.0;
  return I;
}

inline Mat matmul(const Mat& A, const Mat& B, int n) {
  Mat C((size_t)n * n, cd(0.0, 0.0));
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k) {
      const cd b = B[(size_t)j * n + k];
      if (b == cd(0.0, 0.0)) continue;
      const cd* a = &A[(size_t)k * n];
      cd* c = &C[(size_t)j * n];
      for (int i = 0; i < n; ++i) c[i] += a[i] * b;
    }
  return C;
}

// Solve P X = Q in place of Q (partial pivoting); false if singular.
inline bool solve(Mat P, Mat& Q, int n) {
  for (int k = 0; k < n; ++k) {
    int piv = k;
    double best = std::abs(P[(size_t)k * n + k]);
    for (int i = k + 1; i < n; ++i) {
      const double v = std::abs(P[(size_t)k * n + i]);
      if (v > best) {
        best = v;
        piv = i;
      }
    }
    if (!(best > 0.0)) return false;
    if (piv != k)
      for (int j = 0; j < n; ++j) {
        std::swap(P[(size_t)j * n + k], P[(size_t)j * n + piv]);
        std::swap(Q[(size_t)j * n + k], Q[(size_t)j * n + piv]);
      }
    const cd inv = 1.0 / P[(size_t)k * n + k];
    for (int i = k + 1; i < n; ++i) {
      const cd f = P[(size_t)k * n + i] * inv;
      if (f == cd(0.0, 0.0)) continue;
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
  return true;
}

inline bool expm(const Mat& A_in, int n, Mat& E) {
  Mat A = A_in;
  double norm1 = 0.0;
  for (int j = 0; j < n; ++j) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += std::abs(A[(size_t)j * n + i]);
    norm1 = std::max(norm1, s);
  }
  // theta_m bounds of the backward error analysis (Higham 2005, Table 2.3)
  static const int degrees[5] = {3, 5, 7, 9, 13};
  static const double theta[5] = {1.495585217958292e-2, 2.539398330063230e-1, 9.504178996162932e-1,
                                  2.097847961257068e0, 5.371920351148152e0};
  int m = 13, squarings = 0;
  for (int q = 0; q < 4; ++q)
    if (norm1 <= theta[q]) {
      m = degrees[q];
      break;
    }
  if (m == 13 && norm1 > theta[4]) {
    squarings = std::max(0, (int)std::ceil(std::log2(norm1 / theta[4])));
    const double f = std::ldexp(1.0, -squarings);
    for (auto& a : A) a *= f;
  }
  std::vector<double> c(m + 1);
  c[0] = 1.0;
  for (int k = 1; k <= m; ++k) c[k] = c[k - 1] * (double)(m - k + 1) / ((double)(2 * m - k + 1) * (double)k);
  const Mat I = identity(n);
  const Mat A2 = matmul(A, A, n);
  Mat U((size_t)n * n, cd(0.0, 0.0)), V((size_t)n * n, cd(0.0, 0.0));
  if (m < 13) {
    // even powers A^0, A^2, ..., A^(m-1)
    std::vector<Mat> P(m / 2 + 1);
    P[0] = I;
    for (int q = 1; q <= m / 2; ++q) P[q] = (q == 1) ? A2 : matmul(P[q - 1], A2, n);
    Mat Uin((size_t)n * n, cd(0.0, 0.0));
    for (int k = 1; k <= m; k += 2)
      for (size_t t = 0; t < Uin.size(); ++t) Uin[t] += c[k] * P[(k - 1) / 2][t];
    U = matmul(A, Uin, n);
    for (int k = 0; k <= m; k += 2)
      for (size_t t = 0; t < V.size(); ++t) V[t] += c[k] * P[k / 2][t];
  } else {
    const Mat A4 = matmul(A2, A2, n);
    const Mat A6 = matmul(A4, A2, n);
    Mat t1((size_t)n * n), t2((size_t)n * n);
    for (size_t t = 0; t < t1.size(); ++t) {
      t1[t] = c[13] * A6[t] + c[11] * A4[t] + c[9] * A2[t];
      t2[t] = c[12] * A6[t] + c[10] * A4[t] + c[8] * A2[t];
    }
    Mat u1 = matmul(A6, t1, n);
    const Mat v1 = matmul(A6, t2, n);
    for (size_t t = 0; t < u1.size(); ++t) {
      u1[t] += c[7] * A6[t] + c[5] * A4[t] + c[3] * A2[t] + c[1] * I[t];
      V[t] = v1[t] + c[6] * A6[t] + c[4] * A4[t] + c[2] * A2[t] + c[0] * I[t];
    }
    U = matmul(A, u1, n);
  }
  Mat P((size_t)n * n), Q((size_t)n * n);
  for (size_t t = 0; t < P.size(); ++t) {
    P[t] = V[t] - U[t];
    Q[t] = V[t] + U[t];
  }
  if (!solve(P, Q, n)) return false;
  for (int s = 0; s < squarings; ++s) Q = matmul(Q, Q, n);
  E = Q;
  return true;
}

}  // namespace dense
}  // namespace qd
