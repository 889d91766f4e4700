#include "su2.h"

#include <cmath>
#include <cstdlib>
#include <stdexcept>
#include <unordered_map>

namespace bgpu {

PointGroup PointGroup::from_name(const std::string& s) {
  PointGroup g;
  g.name = s;
  if (s == "c1") g.nirrep = 1;
  else if (s == "ci" || s == "cs" || s == "c2") g.nirrep = 2;
  else if (s == "c2v" || s == "c2h" || s == "d2") g.nirrep = 4;
  else if (s == "d2h") g.nirrep = 8;
  else throw std::runtime_error("unsupported point group: " + s);
  return g;
}

bool quantum_allowed(const Quantum& a, const Quantum& b, const Quantum& c, const PointGroup& g) {
  if (a.n != b.n + c.n) return false;
  if (a.irrep != g.product(b.irrep, c.irrep)) return false;
  if (a.s2 < std::abs(b.s2 - c.s2) || a.s2 > b.s2 + c.s2) return false;
  return ((a.s2 + b.s2 + c.s2) & 1) == 0;
}

// Binomial coefficient by the recursion of new_anglib.C:298-316.
double fbinom(int n, int r) {
  if (n == r || r == 0) return 1.0;
  if (r == 1) return n;
  return 1.0 * n / (n - r) * fbinom(n - 1, r);
}

static inline int mone(int k) { return (k % 2 == 0) ? 1 : -1; }

// Clebsch-Gordan coefficient <j1 m1 j2 m2 | j3 m3>, Racah closed form with
// binomials (new_anglib.C:132-204).
double clebsch(int nj1, int nm1, int nj2, int nm2, int nj3, int nm3) {
  const double j1 = nj1 / 2., j2 = nj2 / 2., j3 = nj3 / 2.;
  const double m1 = nm1 / 2., m2 = nm2 / 2., m3 = nm3 / 2.;
  if (j1 < 0 || j2 < 0 || j3 < 0 || std::fabs(m1) > j1 || std::fabs(m2) > j2 || std::fabs(m3) > j3 ||
      j1 + j2 < j3 || std::fabs(j1 - j2) > j3 || m1 + m2 != m3)
    return 0.0;
  const double num1 = std::pow(2 * j3 + 1, 2);
  const double num2 = fbinom((int)(j1 + j2 + j3 + 1), (int)(j1 + j2 - j3));
  const double num3 = fbinom((int)(2 * j3), (int)(j3 + m3));
  const double den1 = (2 * j1 + 1);
  const double den2 = (2 * j2 + 1);
  const double den3 = fbinom((int)(j1 + j2 + j3 + 1), (int)(j1 - j2 + j3));
  const double den4 = fbinom((int)(j1 + j2 + j3 + 1), (int)(j2 - j1 + j3));
  const double den5 = fbinom((int)(2 * j1), (int)(j1 + m1));
  const double den6 = fbinom((int)(2 * j2), (int)(j2 + m2));
  const double num = num1 * num2 * num3;
  const double den = den1 * den2 * den3 * den4 * den5 * den6;
  const double factor = std::sqrt(num / den);
  const double mint = std::max(std::max(0., j1 - m1 - (j3 - m3)), j2 + m2 - (j3 + m3));
  const double maxt = std::min(std::min(j1 - m1, j2 + m2), j1 + j2 - j3);
  double sum = 0.0;
  for (int t = (int)mint; t <= maxt; t++) {
    const double bin1 = fbinom((int)(j1 + j2 - j3), t);
    const double bin2 = fbinom((int)(j3 - m3), (int)(j1 - m1 - t));
    const double bin3 = fbinom((int)(j3 + m3), (int)(j2 + m2 - t));
    sum = sum + mone(t) * bin1 * bin2 * bin3;
  }
  return factor * sum;
}

static double j6_delta(double a, double b, double c) {
  const double den1 = fbinom((int)(a + b + c + 1), (int)(a + b - c));
  const double den2 = 2 * c + 1;
  const double den3 = fbinom((int)(2 * c), (int)(b + c - a));
  const double den = den1 * den2 * den3;
  return 1 / std::sqrt(den);
}

static double square_six(double a, double b, double c, double d, double e, double f) {
  const int nmin = (int)std::max(std::max(std::max(a + e + f, b + d + f), c + d + e), a + b + c);
  const int nmax = (int)std::min(std::min(a + b + d + e, a + c + d + f), b + c + e + f);
  double sum = 0.0;
  for (int n = nmin; n <= nmax; n++) {
    const double num1 = fbinom(n + 1, (int)(n - a - e - f));
    const double num2 = fbinom((int)(a + e - f), (int)(n - b - d - f));
    const double num3 = fbinom((int)(a - e + f), (int)(n - c - d - e));
    const double num4 = fbinom((int)(-a + e + f), (int)(n - a - b - c));
    sum = sum + mone(n) * num1 * num2 * num3 * num4;
  }
  return sum;
}

// Wigner 6j symbol {a b c; d e f} (new_anglib.C:70-108).
double six_j(int na, int nb, int nc, int nd, int ne, int nf) {
  if ((na + nb) % 2 != nc % 2) return 0.0;
  if ((nc + nd) % 2 != ne % 2) return 0.0;
  if ((na + ne) % 2 != nf % 2) return 0.0;
  if ((nb + nd) % 2 != nf % 2) return 0.0;
  if (na + nb < nc || std::abs(na - nb) > nc) return 0.0;
  if (nc + nd < ne || std::abs(nc - nd) > ne) return 0.0;
  if (na + ne < nf || std::abs(na - ne) > nf) return 0.0;
  if (nb + nd < nf || std::abs(nb - nd) > nf) return 0.0;
  const double a = na / 2., b = nb / 2., c = nc / 2., d = nd / 2., e = ne / 2., f = nf / 2.;
  const double num1 = j6_delta(a, b, c);
  const double num2 = j6_delta(c, d, e);
  const double num3 = j6_delta(b, d, f);
  const double den1 = j6_delta(a, e, f);
  const double pref = num1 * num2 * num3 / den1;
  return pref * square_six(a, b, c, d, e, f);
}

// Wigner 9j symbol as a sum over products of three 6j (new_anglib.C:19-68).
double nine_j(int na, int nb, int nc, int nd, int ne, int nf, int ng, int nh, int ni) {
  if (na + nb < nc || std::abs(na - nb) > nc) return 0.0;
  if (nd + ne < nf || std::abs(nd - ne) > nf) return 0.0;
  if (ng + nh < ni || std::abs(ng - nh) > ni) return 0.0;
  if (na + nd < ng || std::abs(na - nd) > ng) return 0.0;
  if (nb + ne < nh || std::abs(nb - ne) > nh) return 0.0;
  if (nc + nf < ni || std::abs(nc - nf) > ni) return 0.0;
  const int kmin = std::max(std::max(std::abs(nh - nd), std::abs(nb - nf)), std::abs(na - ni));
  const int kmax = std::min(std::min(nh + nd, nb + nf), na + ni);
  double r = 0.0;
  for (int k = kmin; k <= kmax; k++) {
    const double num1 = k + 1;
    const double num2 = six_j(na, nb, nc, nf, ni, k);
    const double num3 = six_j(nd, ne, nf, nb, k, nh);
    const double num4 = six_j(ng, nh, ni, k, na, nd);
    r = r + mone(k) * num1 * num2 * num3 * num4;
  }
  return r;
}

double ninej_norm(int a, int b, int c, int d, int e, int f, int g, int h, int i) {
  return std::pow((g + 1) * (h + 1) * (c + 1) * (f + 1), 0.5) * nine_j(a, b, c, d, e, f, g, h, i);
}

double ninej(int a, int b, int c, int d, int e, int f, int g, int h, int i) {
  // all arguments are small non-negative 2j values; pack 7 bits each.  Each
  // thread keeps its own memo table (no locking on the hot host loops).
  auto ok = [](int x) { return x >= 0 && x < 128; };
  if (!(ok(a) && ok(b) && ok(c) && ok(d) && ok(e) && ok(f) && ok(g) && ok(h) && ok(i)))
    return ninej_norm(a, b, c, d, e, f, g, h, i);
  uint64_t key = 0;
  for (int x : {a, b, c, d, e, f, g, h, i}) key = (key << 7) | (uint64_t)x;
  thread_local std::unordered_map<uint64_t, double> memo;
  auto it = memo.find(key);
  if (it != memo.end()) return it->second;
  const double v = ninej_norm(a, b, c, d, e, f, g, h, i);
  memo.emplace(key, v);
  return v;
}

double transpose_scaling(int l2, int r2, int k2) {
  if (k2 == 0) return 1.0;  // rank-0: clebsch ratio is 1 and (-1)^0 = 1
  for (int lz = -l2; lz < l2 + 1; lz += 2)
    for (int rz = -r2; rz < r2 + 1; rz += 2) {
      const double cleb = clebsch(l2, lz, k2, -k2, r2, rz);
      if (std::fabs(cleb) <= 1e-10) continue;
      const double den = clebsch(r2, rz, k2, k2, l2, lz);
      if (std::fabs(den) <= 1e-10) continue;
      return std::pow(-1.0, k2) * cleb / den;
    }
  throw std::runtime_error("transpose_scaling: no coupling between given spins");
}

double commute_parity(const Quantum& a, const Quantum& b, int c2) {
  const int parity = (is_fermion(a) && is_fermion(b)) ? -1 : 1;
  for (int az = -a.s2; az < a.s2 + 1; az += 2)
    for (int bz = -b.s2; bz < b.s2 + 1; bz += 2) {
      const double cleb = clebsch(a.s2, az, b.s2, bz, c2, c2);
      if (std::fabs(cleb) <= 1e-10) continue;
      return parity * cleb / clebsch(b.s2, bz, a.s2, az, c2, c2);
    }
  throw std::runtime_error("commute_parity: incompatible spins");
}

}  // namespace bgpu
