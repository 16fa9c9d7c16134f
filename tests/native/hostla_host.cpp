// Test harness only: the host linear algebra of the drivers (csrc/hostla.h)
// behind a C ABI for ctypes.
#include <vector>

#include "hostla.h"

extern "C" void hl_tri_lowest(int m, const double* a, const double* b, int nev, double* th, double* vecs) {
  std::vector<double> A(a, a + m), B(m, 0.0);
  for (int i = 0; i + 1 < m; ++i) B[i] = b[i];
  std::vector<double> t;
  std::vector<std::vector<double>> v;
  sfci::hostla::tri_lowest(A, B, m, nev, t, v);
  for (int k = 0; k < nev; ++k) {
    th[k] = t[k];
    for (int i = 0; i < m; ++i) vecs[(size_t)k * m + i] = v[k][i];
  }
}

extern "C" void hl_lstsq(int m, int n, const double* A, const double* e, double* y) {
  std::vector<double> Av(A, A + (size_t)m * n), ev(e, e + m), yv;
  sfci::hostla::lstsq_qr(m, n, Av, ev, yv);
  for (int j = 0; j < n; ++j) y[j] = yv[j];
}
