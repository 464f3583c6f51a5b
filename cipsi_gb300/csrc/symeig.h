// symeig.h -- eigenvalues and eigenvectors of a small dense real symmetric
// matrix by cyclic Jacobi rotations (host).  Used for the Rayleigh-Ritz
// problems of the Davidson iteration (davidson.cu) and for the Gram matrices
// of its orthonormalisation, which are a few tens of rows.
//
// Each rotation zeroes a(p,q): with theta = (a_qq - a_pp) / (2 a_pq),
// t = sign(theta) / (|theta| + sqrt(theta^2 + 1)), c = 1/sqrt(t^2 + 1),
// s = t c, the rotated matrix has a_pp - t a_pq and a_qq + t a_pq on the
// diagonal; sweeps repeat until the off-diagonal norm is below 1e-15 of the
// matrix norm.
#pragma once

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace cipsi_host {

// a: n x n symmetric, row-major (destroyed).  On return w holds the
// eigenvalues in ascending order and v (n x n, row-major) the eigenvectors
// as columns: v[i * n + k] is component i of eigenvector k.
inline void sym_eig(int n, std::vector<double> a, std::vector<double>& w, std::vector<double>& v) {
  v.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
  auto A = [&](int i, int j) -> double& { return a[(size_t)i * n + j]; };
  double norm = 0.0;
  for (double x : a) norm += x * x;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += A(p, q) * A(p, q);
    if (off <= 1e-30 * norm || off == 0.0) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A(p, q);
        if (apq == 0.0) continue;
        const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // columns p, q of A
          const double akp = A(k, p), akq = A(k, q);
          A(k, p) = c * akp - s * akq;
          A(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows p, q
          const double apk = A(p, k), aqk = A(q, k);
          A(p, k) = c * apk - s * aqk;
          A(q, k) = s * apk + c * aqk;
        }
        A(p, q) = A(q, p) = 0.0;
        for (int k = 0; k < n; ++k) {
          const double vkp = v[(size_t)k * n + p], vkq = v[(size_t)k * n + q];
          v[(size_t)k * n + p] = c * vkp - s * vkq;
          v[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return A(x, x) < A(y, y); });
  w.resize(n);
  std::vector<double> vs((size_t)n * n);
  for (int k = 0; k < n; ++k) {
    w[k] = A(ord[k], ord[k]);
    for (int i = 0; i < n; ++i) vs[(size_t)i * n + k] = v[(size_t)i * n + ord[k]];
  }
  v.swap(vs);
}

}  // namespace cipsi_host
