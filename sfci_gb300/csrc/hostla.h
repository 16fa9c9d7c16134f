// Small dense host linear algebra of the drivers (no GPU, no library): the
// symmetric tridiagonal eigenproblem of the subspace Lanczos iteration and the
// least-squares solve of the linear Krylov driver.  Header-only so that the host
// tests compile it as it is.
#pragma once

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <limits>
#include <vector>

namespace sfci {
namespace hostla {

// ---- symmetric tridiagonal T (diagonal a[0..m), off-diagonal b[0..m-1)) ----

// number of eigenvalues of T below x (Sturm sequence of the LDL^T pivots)
inline int sturm_below(const std::vector<double>& a, const std::vector<double>& b, int m, double x, double pivmin) {
  int cnt = 0;
  double q = a[0] - x;
  if (std::fabs(q) < pivmin) q = -pivmin;
  if (q < 0) ++cnt;
  for (int i = 1; i < m; ++i) {
    q = a[i] - x - b[i - 1] * b[i - 1] / q;
    if (std::fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++cnt;
  }
  return cnt;
}

// k-th smallest eigenvalue of T by bisection inside the Gershgorin interval
inline double tri_eigval(const std::vector<double>& a, const std::vector<double>& b, int m, int k, double pivmin) {
  double lo = a[0], hi = a[0];
  for (int i = 0; i < m; ++i) {
    const double r = (i ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  const double span = hi - lo;
  lo -= 1e-12 * span + pivmin;
  hi += 1e-12 * span + pivmin;
  for (int it = 0; it < 256; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (hi - lo <= 2.0 * DBL_EPSILON * std::max(std::fabs(lo), std::fabs(hi)) + pivmin) break;
    if (sturm_below(a, b, m, mid, pivmin) > k) hi = mid;
    else lo = mid;
  }
  return 0.5 * (lo + hi);
}

// eigenvector of T for the eigenvalue theta by inverse iteration: Gaussian
// elimination with partial pivoting of T - theta I (upper factor with two
// superdiagonals), three solves, each followed by orthogonalisation against the
// eigenvectors already found
inline void tri_eigvec(const std::vector<double>& a, const std::vector<double>& b, int m, double theta, double tiny,
                const std::vector<std::vector<double>>& prev, std::vector<double>& y) {
  std::vector<double> u0(m), u1(m, 0.0), u2(m, 0.0), L(m, 0.0);
  std::vector<char> sw(m, 0);
  double cd = a[0] - theta, cu = m > 1 ? b[0] : 0.0;
  for (int i = 0; i + 1 < m; ++i) {
    const double bi = b[i], d1 = a[i + 1] - theta, n1 = (i + 2 < m) ? b[i + 1] : 0.0;
    if (std::fabs(cd) >= std::fabs(bi)) {
      if (cd == 0.0) cd = tiny;
      u0[i] = cd;
      u1[i] = cu;
      L[i] = bi / cd;
      cd = d1 - L[i] * cu;
      cu = n1;
    } else {
      sw[i] = 1;
      u0[i] = bi;
      u1[i] = d1;
      u2[i] = n1;
      L[i] = cd / bi;
      const double nd = cu - L[i] * d1;
      cu = -L[i] * n1;
      cd = nd;
    }
  }
  u0[m - 1] = (std::fabs(cd) < tiny) ? (cd < 0 ? -tiny : tiny) : cd;
  for (int i = 0; i < m; ++i)
    if (u0[i] == 0.0) u0[i] = tiny;
  y.assign(m, 0.0);
  for (int i = 0; i < m; ++i) y[i] = 1.0 + 0.01 * (double)((i * 7919) % 101) / 101.0;
  for (int it = 0; it < 3; ++it) {
    for (int i = 0; i + 1 < m; ++i) {
      if (sw[i]) std::swap(y[i], y[i + 1]);
      y[i + 1] -= L[i] * y[i];
    }
    for (int i = m - 1; i >= 0; --i) {
      double s = y[i];
      if (i + 1 < m) s -= u1[i] * y[i + 1];
      if (i + 2 < m) s -= u2[i] * y[i + 2];
      y[i] = s / u0[i];
    }
    for (const auto& p : prev) {
      double dp = 0.0;
      for (int i = 0; i < m; ++i) dp += p[i] * y[i];
      for (int i = 0; i < m; ++i) y[i] -= dp * p[i];
    }
    double nrm = 0.0;
    for (int i = 0; i < m; ++i) nrm += y[i] * y[i];
    nrm = std::sqrt(nrm);
    if (!(nrm > 0.0)) nrm = 1.0;
    for (int i = 0; i < m; ++i) y[i] /= nrm;
  }
}

// the nev lowest eigenpairs of T_m
inline void tri_lowest(const std::vector<double>& a, const std::vector<double>& b, int m, int nev, std::vector<double>& th,
                std::vector<std::vector<double>>& vecs) {
  double tn = 0.0, bmax = 0.0;
  for (int i = 0; i < m; ++i) {
    tn = std::max(tn, std::fabs(a[i]) + (i ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(b[i]) : 0.0));
    if (i + 1 < m) bmax = std::max(bmax, b[i] * b[i]);
  }
  const double pivmin = DBL_MIN * std::max(1.0, bmax);
  const double tiny = DBL_EPSILON * std::max(tn, DBL_MIN);
  th.assign(nev, 0.0);
  vecs.assign(nev, std::vector<double>());
  for (int k = 0; k < nev; ++k) th[k] = tri_eigval(a, b, m, k, pivmin);
  std::vector<std::vector<double>> prev;
  for (int k = 0; k < nev; ++k) {
    tri_eigvec(a, b, m, th[k], tiny, prev, vecs[k]);
    prev.push_back(vecs[k]);
  }
}

// ---- least squares min |A y - e|, A m x n column-major (m >= n) -----------------
// Householder QR with column pivoting, as Eigen's colPivHouseholderQr: columns
// whose remaining norm falls below eps * max(m, n) * |R(0,0)| are left out
// (their y entries are zero).
inline void lstsq_qr(int m, int n, std::vector<double> A, std::vector<double> e, std::vector<double>& y) {
  auto at = [&](int i, int j) -> double& { return A[(size_t)j * m + i]; };
  std::vector<int> perm(n);
  for (int j = 0; j < n; ++j) perm[j] = j;
  std::vector<double> cn(n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) cn[j] += at(i, j) * at(i, j);
  int rank = 0;
  double r00 = 0.0;
  const int kmax = std::min(m, n);
  for (int k = 0; k < kmax; ++k) {
    int p = k;
    for (int j = k + 1; j < n; ++j)
      if (cn[j] > cn[p]) p = j;
    if (p != k) {
      for (int i = 0; i < m; ++i) std::swap(at(i, k), at(i, p));
      std::swap(cn[k], cn[p]);
      std::swap(perm[k], perm[p]);
    }
    double nx = 0.0;
    for (int i = k; i < m; ++i) nx += at(i, k) * at(i, k);
    nx = std::sqrt(nx);
    if (k == 0) r00 = nx;
    if (nx <= std::numeric_limits<double>::epsilon() * std::max(m, n) * r00 || nx == 0.0) break;
    const double alpha = at(k, k) > 0 ? -nx : nx;
    std::vector<double> v(m - k);
    for (int i = k; i < m; ++i) v[i - k] = at(i, k);
    v[0] -= alpha;
    double vn = 0.0;
    for (double t : v) vn += t * t;
    if (vn > 0.0) {
      for (int j = k; j < n; ++j) {
        double d = 0.0;
        for (int i = k; i < m; ++i) d += v[i - k] * at(i, j);
        d = 2.0 * d / vn;
        for (int i = k; i < m; ++i) at(i, j) -= d * v[i - k];
      }
      double d = 0.0;
      for (int i = k; i < m; ++i) d += v[i - k] * e[i];
      d = 2.0 * d / vn;
      for (int i = k; i < m; ++i) e[i] -= d * v[i - k];
    }
    for (int j = k + 1; j < n; ++j) cn[j] -= at(k, j) * at(k, j);
    rank = k + 1;
  }
  std::vector<double> z(n, 0.0);
  for (int k = rank - 1; k >= 0; --k) {
    double s = e[k];
    for (int j = k + 1; j < rank; ++j) s -= at(k, j) * z[j];
    z[k] = s / at(k, k);
  }
  y.assign(n, 0.0);
  for (int k = 0; k < n; ++k) y[perm[k]] = z[k];
}

}  // namespace hostla
}  // namespace sfci
