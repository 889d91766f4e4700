#include "dense.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace bgpu {

void jacobi_eigh(int n, const double* a_in, double* w, double* v) {
  std::vector<double> a(a_in, a_in + (size_t)n * n);
  std::fill(v, v + (size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
  auto A = [&](int i, int j) -> double& { return a[(size_t)i * n + j]; };
  double scale = 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) scale = std::max(scale, std::fabs(A(i, j)));
  if (scale == 0.0) scale = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) off += A(i, j) * A(i, j);
    if (std::sqrt(off) <= 1e-15 * scale * n) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A(p, q);
        if (std::fabs(apq) <= 1e-300) continue;
        if (sweep > 3 && std::fabs(apq) < 1e-18 * scale) {
          A(p, q) = A(q, p) = 0.0;
          continue;
        }
        // rotation angle from the classical formula
        const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0);
        const double s = t * c;
        for (int k = 0; k < n; ++k) {  // columns p, q
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
          double* vk = v + (size_t)k * n;
          const double vkp = vk[p], vkq = vk[q];
          vk[p] = c * vkp - s * vkq;
          vk[q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return A(x, x) < A(y, y); });
  std::vector<double> vs(v, v + (size_t)n * n);
  for (int j = 0; j < n; ++j) {
    w[j] = A(idx[j], idx[j]);
    for (int k = 0; k < n; ++k) v[(size_t)k * n + j] = vs[(size_t)k * n + idx[j]];
  }
}

bool orthonormalise_columns(int rows, int cols, double* m) {
  bool ok = true;
  for (int j = 0; j < cols; ++j) {
    for (int pass = 0; pass < 2; ++pass)
      for (int i = 0; i < j; ++i) {
        double d = 0.0;
        for (int r = 0; r < rows; ++r) d += m[(size_t)r * cols + i] * m[(size_t)r * cols + j];
        for (int r = 0; r < rows; ++r) m[(size_t)r * cols + j] -= d * m[(size_t)r * cols + i];
      }
    double nrm = 0.0;
    for (int r = 0; r < rows; ++r) nrm += m[(size_t)r * cols + j] * m[(size_t)r * cols + j];
    nrm = std::sqrt(nrm);
    if (nrm < 1e-12) {
      ok = false;
      nrm = 1.0;
    }
    for (int r = 0; r < rows; ++r) m[(size_t)r * cols + j] /= nrm;
  }
  return ok;
}

}  // namespace bgpu
