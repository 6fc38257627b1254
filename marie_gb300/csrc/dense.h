// Small dense complex linear algebra on the host (column-major), for the
// projected problems of the Krylov solvers: least squares (MATLAB's A \ b for
// a tall matrix), thin QR (qr(A, 0)), square solves, and eigenpairs of general
// and generalized matrices (eig(A), eig(A, B)).  Sizes are those of a restart
// cycle (tens), so plain O(n^3) algorithms suffice:
//   * Householder QR (Golub & Van Loan, Matrix Computations, 4th ed., 5.2);
//   * LU with partial pivoting (3.4);
//   * eigenvalues by Hessenberg reduction and the shifted QR iteration with
//     Wilkinson shifts, deflating at negligible subdiagonals (7.4-7.5), the
//     eigenvectors from the Schur form by back-substitution (7.6).
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <limits>
#include <vector>

namespace marie {
namespace dense {

using cd = std::complex<double>;

struct Mat {
  int r = 0, c = 0;
  std::vector<cd> a;
  Mat() = default;
  Mat(int rows, int cols) : r(rows), c(cols), a((size_t)rows * cols, cd(0, 0)) {}
  cd& operator()(int i, int j) { return a[(size_t)j * r + i]; }
  const cd& operator()(int i, int j) const { return a[(size_t)j * r + i]; }
  static Mat eye(int n) {
    Mat m(n, n);
    for (int i = 0; i < n; ++i) m(i, i) = 1.0;
    return m;
  }
};

inline Mat mul(const Mat& A, const Mat& B) {
  Mat C(A.r, B.c);
  for (int j = 0; j < B.c; ++j)
    for (int k = 0; k < A.c; ++k) {
      const cd b = B(k, j);
      if (b == cd(0, 0)) continue;
      for (int i = 0; i < A.r; ++i) C(i, j) += A(i, k) * b;
    }
  return C;
}
inline Mat adj(const Mat& A) {
  Mat B(A.c, A.r);
  for (int j = 0; j < A.c; ++j)
    for (int i = 0; i < A.r; ++i) B(j, i) = std::conj(A(i, j));
  return B;
}
inline std::vector<cd> mulv(const Mat& A, const std::vector<cd>& x) {
  std::vector<cd> y(A.r, cd(0, 0));
  for (int j = 0; j < A.c; ++j)
    for (int i = 0; i < A.r; ++i) y[i] += A(i, j) * x[j];
  return y;
}

// Householder QR of an m x n matrix (m >= n): R (n x n) and the reflectors,
// applied through qt_apply.  v_k has v_k[k] = 1 implied by the stored scale.
struct QR {
  Mat F;                 // factored matrix: R on and above the diagonal, reflectors below
  std::vector<cd> beta;  // H_k = I - beta_k v_k v_k^H
  std::vector<cd> diag;  // R diagonal
};

inline QR qr_factor(Mat A) {
  const int m = A.r, n = A.c;
  QR q;
  q.beta.assign(n, cd(0, 0));
  q.diag.assign(n, cd(0, 0));
  for (int k = 0; k < n; ++k) {
    double nx = 0;
    for (int i = k; i < m; ++i) nx += std::norm(A(i, k));
    nx = std::sqrt(nx);
    if (nx == 0) {
      q.diag[k] = 0;
      continue;
    }
    const cd x0 = A(k, k);
    const double ax0 = std::abs(x0);
    const cd ph = ax0 > 0 ? x0 / ax0 : cd(1, 0);
    const cd alpha = -ph * nx;  // R(k,k)
    // v = x - alpha e1, normalised so that v[k] = 1
    const cd v0 = x0 - alpha;
    for (int i = k + 1; i < m; ++i) A(i, k) /= v0;
    double vv = 1.0;
    for (int i = k + 1; i < m; ++i) vv += std::norm(A(i, k));
    const cd beta = 2.0 / vv;
    q.beta[k] = beta;
    q.diag[k] = alpha;
    // apply H_k to the trailing columns
    for (int j = k + 1; j < n; ++j) {
      cd s = A(k, j);
      for (int i = k + 1; i < m; ++i) s += std::conj(A(i, k)) * A(i, j);
      s *= beta;
      A(k, j) -= s;
      for (int i = k + 1; i < m; ++i) A(i, j) -= s * A(i, k);
    }
    A(k, k) = alpha;
  }
  q.F = A;
  return q;
}

// y = Q^H y (Q = H_0 H_1 ... H_{n-1})
inline void qt_apply(const QR& q, std::vector<cd>& y) {
  const int m = q.F.r, n = q.F.c;
  for (int k = 0; k < n; ++k) {
    if (q.beta[k] == cd(0, 0)) continue;
    cd s = y[k];
    for (int i = k + 1; i < m; ++i) s += std::conj(q.F(i, k)) * y[i];
    s *= q.beta[k];
    y[k] -= s;
    for (int i = k + 1; i < m; ++i) y[i] -= s * q.F(i, k);
  }
}
// y = Q y
inline void q_apply(const QR& q, std::vector<cd>& y) {
  const int m = q.F.r, n = q.F.c;
  for (int k = n - 1; k >= 0; --k) {
    if (q.beta[k] == cd(0, 0)) continue;
    cd s = y[k];
    for (int i = k + 1; i < m; ++i) s += std::conj(q.F(i, k)) * y[i];
    s *= q.beta[k];
    y[k] -= s;
    for (int i = k + 1; i < m; ++i) y[i] -= s * q.F(i, k);
  }
}

// least squares min ||A x - b|| for a tall full-rank A
inline std::vector<cd> lstsq(const Mat& A, std::vector<cd> b) {
  const QR q = qr_factor(A);
  qt_apply(q, b);
  const int n = A.c;
  std::vector<cd> x(n, cd(0, 0));
  for (int i = n - 1; i >= 0; --i) {
    cd s = b[i];
    for (int j = i + 1; j < n; ++j) s -= q.F(i, j) * x[j];
    x[i] = s / q.F(i, i);
  }
  return x;
}

// thin QR: A (m x n) = Q (m x n) R (n x n)
inline void qr_thin(const Mat& A, Mat& Q, Mat& R) {
  const QR q = qr_factor(A);
  const int m = A.r, n = A.c;
  R = Mat(n, n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= j; ++i) R(i, j) = q.F(i, j);
  Q = Mat(m, n);
  for (int j = 0; j < n; ++j) {
    std::vector<cd> e(m, cd(0, 0));
    e[j] = 1.0;
    q_apply(q, e);
    for (int i = 0; i < m; ++i) Q(i, j) = e[i];
  }
}

// X = A^{-1} B for square A (LU with partial pivoting)
inline Mat solve(Mat A, Mat B) {
  const int n = A.r;
  std::vector<int> piv(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::abs(A(k, k));
    for (int i = k + 1; i < n; ++i)
      if (std::abs(A(i, k)) > best) {
        best = std::abs(A(i, k));
        p = i;
      }
    piv[k] = p;
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(A(k, j), A(p, j));
      for (int j = 0; j < B.c; ++j) std::swap(B(k, j), B(p, j));
    }
    const cd d = A(k, k);
    if (d == cd(0, 0)) continue;
    for (int i = k + 1; i < n; ++i) {
      const cd l = A(i, k) / d;
      A(i, k) = l;
      for (int j = k + 1; j < n; ++j) A(i, j) -= l * A(k, j);
      for (int j = 0; j < B.c; ++j) B(i, j) -= l * B(k, j);
    }
  }
  for (int j = 0; j < B.c; ++j)
    for (int i = n - 1; i >= 0; --i) {
      cd s = B(i, j);
      for (int k = i + 1; k < n; ++k) s -= A(i, k) * B(k, j);
      B(i, j) = s / A(i, i);
    }
  return B;
}

// X = B R^{-1} for upper-triangular R (MATLAB's B / R)
inline Mat rdiv_upper(const Mat& B, const Mat& R) {
  const int n = R.r;
  Mat X(B.r, n);
  for (int i = 0; i < B.r; ++i)
    for (int j = 0; j < n; ++j) {
      cd s = B(i, j);
      for (int k = 0; k < j; ++k) s -= X(i, k) * R(k, j);
      X(i, j) = s / R(j, j);
    }
  return X;
}

// Eigenpairs of a general complex matrix.  vals[k], vecs column k (unit norm).
inline void eig(Mat A, std::vector<cd>& vals, Mat& vecs) {
  const int n = A.r;
  Mat Z = Mat::eye(n);
  // Hessenberg reduction by Householder reflectors, accumulated in Z
  for (int k = 0; k < n - 2; ++k) {
    double nx = 0;
    for (int i = k + 1; i < n; ++i) nx += std::norm(A(i, k));
    nx = std::sqrt(nx);
    if (nx == 0) continue;
    const cd x0 = A(k + 1, k);
    const double ax0 = std::abs(x0);
    const cd ph = ax0 > 0 ? x0 / ax0 : cd(1, 0);
    const cd alpha = -ph * nx;
    std::vector<cd> v(n, cd(0, 0));
    v[k + 1] = x0 - alpha;
    for (int i = k + 2; i < n; ++i) v[i] = A(i, k);
    double vv = 0;
    for (int i = k + 1; i < n; ++i) vv += std::norm(v[i]);
    if (vv == 0) continue;
    const double beta = 2.0 / vv;
    // A = H A
    for (int j = 0; j < n; ++j) {
      cd s = 0;
      for (int i = k + 1; i < n; ++i) s += std::conj(v[i]) * A(i, j);
      s *= beta;
      for (int i = k + 1; i < n; ++i) A(i, j) -= s * v[i];
    }
    // A = A H, Z = Z H
    for (int i = 0; i < n; ++i) {
      cd s = 0, t = 0;
      for (int j = k + 1; j < n; ++j) {
        s += A(i, j) * v[j];
        t += Z(i, j) * v[j];
      }
      s *= beta;
      t *= beta;
      for (int j = k + 1; j < n; ++j) {
        A(i, j) -= s * std::conj(v[j]);
        Z(i, j) -= t * std::conj(v[j]);
      }
    }
    for (int i = k + 2; i < n; ++i) A(i, k) = 0;
  }
  // shifted QR iteration on the Hessenberg matrix -> upper-triangular Schur form
  const double eps = std::numeric_limits<double>::epsilon();
  int hi = n - 1, iter = 0;
  while (hi > 0) {
    int l = hi;
    for (; l > 0; --l) {
      const double s = std::abs(A(l - 1, l - 1)) + std::abs(A(l, l));
      if (std::abs(A(l, l - 1)) <= eps * (s > 0 ? s : 1.0)) {
        A(l, l - 1) = 0;
        break;
      }
    }
    if (l == hi) {
      --hi;
      iter = 0;
      continue;
    }
    if (++iter > 60 * n) break;  // no convergence: leave the rest as is
    // Wilkinson shift from the trailing 2 x 2 block (exceptional every 11th)
    cd mu;
    if (iter % 11 == 10) {
      mu = A(hi, hi) + std::abs(A(hi, hi - 1));
    } else {
      const cd a = A(hi - 1, hi - 1), b = A(hi - 1, hi), c = A(hi, hi - 1), d = A(hi, hi);
      const cd tr = 0.5 * (a + d);
      const cd disc = std::sqrt((a - tr) * (a - tr) + b * c);
      const cd m1 = tr + disc, m2 = tr - disc;
      mu = std::abs(m1 - d) < std::abs(m2 - d) ? m1 : m2;
    }
    // explicit QR step on rows/columns l..hi with Givens rotations
    std::vector<double> gc(hi - l);
    std::vector<cd> gs(hi - l);
    for (int k = l; k <= hi; ++k) A(k, k) -= mu;
    for (int k = l; k < hi; ++k) {
      const cd x = A(k, k), y = A(k + 1, k);
      const double ax = std::abs(x), ay = std::abs(y);
      double c;
      cd s;
      if (ay == 0) {
        c = 1;
        s = 0;
      } else if (ax == 0) {
        c = 0;
        s = std::conj(y) / ay;
      } else {
        const double r = std::hypot(ax, ay);
        c = ax / r;
        s = (x / ax) * std::conj(y) / r;
      }
      gc[k - l] = c;
      gs[k - l] = s;
      // rows k, k+1: [c s; -conj(s) c]
      for (int j = k; j < n; ++j) {
        const cd u = A(k, j), w = A(k + 1, j);
        A(k, j) = c * u + s * w;
        A(k + 1, j) = -std::conj(s) * u + c * w;
      }
    }
    for (int k = l; k < hi; ++k) {
      const double c = gc[k - l];
      const cd s = gs[k - l];
      // columns k, k+1 times the adjoint rotation
      const int top = std::min(k + 2, hi);
      for (int i = 0; i <= top; ++i) {
        const cd u = A(i, k), w = A(i, k + 1);
        A(i, k) = c * u + std::conj(s) * w;
        A(i, k + 1) = -s * u + c * w;
      }
      for (int i = 0; i < n; ++i) {
        const cd u = Z(i, k), w = Z(i, k + 1);
        Z(i, k) = c * u + std::conj(s) * w;
        Z(i, k + 1) = -s * u + c * w;
      }
    }
    for (int k = l; k <= hi; ++k) A(k, k) += mu;
  }
  vals.assign(n, cd(0, 0));
  for (int i = 0; i < n; ++i) vals[i] = A(i, i);
  // eigenvectors of the triangular T, then back to the original basis
  double tn = 0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= j; ++i) tn = std::max(tn, std::abs(A(i, j)));
  const double small = eps * (tn > 0 ? tn : 1.0);
  vecs = Mat(n, n);
  for (int k = 0; k < n; ++k) {
    std::vector<cd> y(n, cd(0, 0));
    y[k] = 1.0;
    for (int i = k - 1; i >= 0; --i) {
      cd s = 0;
      for (int j = i + 1; j <= k; ++j) s += A(i, j) * y[j];
      cd den = A(i, i) - vals[k];
      if (std::abs(den) < small) den = small;
      y[i] = -s / den;
    }
    double nrm = 0;
    std::vector<cd> v(n, cd(0, 0));
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j <= k; ++j) v[i] += Z(i, j) * y[j];
      nrm += std::norm(v[i]);
    }
    nrm = std::sqrt(nrm);
    for (int i = 0; i < n; ++i) vecs(i, k) = nrm > 0 ? v[i] / nrm : v[i];
  }
}

}  // namespace dense
}  // namespace marie
