#include "ops.h"

#include <array>
#include <cmath>
#include <cstdio>
#include <stdexcept>

namespace bgpu {

const char* op_type_name(OpType t) {
  switch (t) {
    case OpType::HAM: return "HAM";
    case OpType::CRE: return "CRE";
    case OpType::CD: return "CRE_DES";
    case OpType::CC: return "CRE_CRE";
    case OpType::CDCOMP: return "CRE_DESCOMP";
    case OpType::DDCOMP: return "DES_DESCOMP";
    case OpType::CCD: return "CRE_CRE_DESCOMP";
    case OpType::OVERLAP: return "OVERLAP";
  }
  return "?";
}

std::string OpKey::str() const {
  char buf[96];
  std::snprintf(buf, sizeof buf, "%s(%d,%d;k2=%d)", op_type_name(type), i, j, k2);
  return buf;
}

static OpKey mk(OpType t, int i, int j, int k2) {
  OpKey k;
  k.type = t;
  k.i = (int16_t)i;
  k.j = (int16_t)j;
  k.k2 = (int8_t)k2;
  return k;
}
OpKey ham_key() { return mk(OpType::HAM, -1, -1, 0); }
OpKey overlap_key() { return mk(OpType::OVERLAP, -1, -1, 0); }
OpKey cre_key(int i) { return mk(OpType::CRE, i, -1, 1); }
OpKey cd_key(int i, int j, int k2) { return mk(OpType::CD, i, j, k2); }
OpKey cc_key(int i, int j, int k2) { return mk(OpType::CC, i, j, k2); }
OpKey cdcomp_key(int i, int j, int k2) { return mk(OpType::CDCOMP, i, j, k2); }
OpKey ddcomp_key(int i, int j, int k2) { return mk(OpType::DDCOMP, i, j, k2); }
OpKey ccd_key(int i) { return mk(OpType::CCD, i, -1, 1); }

Quantum op_dq(const OpKey& k, const std::vector<int>& orbsym) {
  auto sy = [&](int i) { return orbsym[i]; };
  switch (k.type) {
    case OpType::HAM:
    case OpType::OVERLAP: return {0, 0, 0};
    case OpType::CRE: return {1, 1, sy(k.i)};
    case OpType::CCD: return {1, 1, sy(k.i)};
    case OpType::CD: return {0, k.k2, sy(k.i) ^ sy(k.j)};
    case OpType::CDCOMP: return {0, k.k2, sy(k.i) ^ sy(k.j)};
    case OpType::CC: return {2, k.k2, sy(k.i) ^ sy(k.j)};
    case OpType::DDCOMP: return {-2, k.k2, sy(k.i) ^ sy(k.j)};
  }
  return {0, 0, 0};
}

OpLayout make_layout(const StateInfo& si, const Quantum& dq, const PointGroup& g) {
  OpLayout L;
  L.dq = dq;
  L.nq = si.size();
  L.index.assign((size_t)L.nq * L.nq, -1);
  L.by_ket.assign(L.nq, {});
  L.by_bra.assign(L.nq, {});
  for (int b = 0; b < si.size(); ++b)
    for (int k = 0; k < si.size(); ++k) {
      if (!quantum_allowed(si.quanta[b], si.quanta[k], dq, g)) continue;
      OpBlock blk;
      blk.bra = b;
      blk.ket = k;
      blk.rows = si.states[b];
      blk.cols = si.states[k];
      blk.offset = L.size;
      L.index[(size_t)b * L.nq + k] = (int)L.blocks.size();
      L.by_ket[k].push_back((int)L.blocks.size());
      L.by_bra[b].push_back((int)L.blocks.size());
      L.blocks.push_back(blk);
      L.size += (int64_t)blk.rows * blk.cols;
    }
  return L;
}

const OpEntry& OpSet::at(const OpKey& k) const {
  auto it = ops.find(k);
  if (it == ops.end()) throw std::runtime_error("operator not in block: " + k.str());
  return it->second;
}

OpSet make_opset(const StateInfo& si, const std::set<OpKey>& keys, const std::vector<int>& orbsym,
                 const PointGroup& g) {
  OpSet s;
  std::map<std::tuple<int, int, int>, int> by_dq;
  for (const auto& k : keys) {
    Quantum dq = op_dq(k, orbsym);
    auto t = std::make_tuple(dq.n, dq.s2, dq.irrep);
    auto it = by_dq.find(t);
    int li;
    if (it == by_dq.end()) {
      li = (int)s.layouts.size();
      s.layouts.push_back(make_layout(si, dq, g));
      by_dq[t] = li;
    } else {
      li = it->second;
    }
    OpEntry e;
    e.layout = li;
    e.base = s.arena;
    s.arena += s.layouts[li].size;
    s.ops[k] = e;
  }
  return s;
}

std::set<OpKey> catalog_keys(const CatalogSpec& c) {
  std::set<OpKey> k;
  k.insert(ham_key());
  k.insert(overlap_key());
  for (int i : c.sites) k.insert(cre_key(i));
  for (int i : c.ccd_sites) k.insert(ccd_key(i));
  if (c.normal)
    for (int a : c.sites)
      for (int b : c.sites) {
        if (a < b) continue;
        k.insert(cd_key(a, b, 0));
        k.insert(cd_key(a, b, 2));
        k.insert(cc_key(a, b, 0));
        if (a != b) k.insert(cc_key(a, b, 2));
      }
  for (auto& p : c.comp_pairs) {
    const int a = std::max(p.first, p.second), b = std::min(p.first, p.second);
    k.insert(cdcomp_key(a, b, 0));
    k.insert(cdcomp_key(a, b, 2));
    k.insert(ddcomp_key(a, b, 0));
    if (a != b) k.insert(ddcomp_key(a, b, 2));
  }
  for (const OpKey& x : c.extra) k.insert(x);
  return k;
}

CatalogSpec dot_catalog(int x, int norb) {
  CatalogSpec c;
  c.sites = {x};
  c.normal = true;
  for (int i = 0; i < norb; ++i)
    if (i != x) c.ccd_sites.push_back(i);
  for (int i = 0; i < norb; ++i)
    for (int j = 0; j <= i; ++j)
      if (i != x && j != x) c.comp_pairs.push_back({i, j});
  return c;
}

// ---------------------------------------------------------------- recipes

Operand canonical(const Operand& o, double& coef) {
  if (o.identity) return o;
  Operand r = o;
  if ((o.key.type == OpType::CDCOMP || o.key.type == OpType::DDCOMP) && o.key.i < o.key.j) {
    r.key.i = o.key.j;
    r.key.j = o.key.i;
    if (o.key.type == OpType::CDCOMP) {
      // CDcomp^k_ab = e_k T(CDcomp^k_ba), e_0 = +1, e_1 = -1;  T(T(X)) = X
      if (o.key.k2 == 2) coef = -coef;
      r.trans = !o.trans;
    } else {
      if (o.key.k2 == 2) coef = -coef;
    }
  }
  return r;
}

static bool contains(const std::vector<int>& v, int x) {
  for (int y : v)
    if (y == x) return true;
  return false;
}

static void add(std::vector<BuildTerm>& out, double coef, Operand a, Operand b) {
  if (coef == 0.0) return;
  double c = coef;
  a = canonical(a, c);
  b = canonical(b, c);
  BuildTerm t;
  t.coef = c;
  t.a = a;
  t.b = b;
  out.push_back(t);
}

std::vector<BuildTerm> build_terms(const OpKey& T, const std::vector<int>& A, const std::vector<int>& B,
                                   const Integrals& I) {
  std::vector<BuildTerm> out;
  const bool adot = A.size() == 1, bdot = B.size() == 1;
  auto inA = [&](int x) { return contains(A, x); };
  auto inB = [&](int x) { return contains(B, x); };
  const double r3 = std::sqrt(3.0);
  switch (T.type) {
    case OpType::OVERLAP:
      add(out, 1.0, ident(), ident());
      break;
    case OpType::CRE:
      if (inA(T.i)) add(out, 1.0, op(T), ident());
      else add(out, 1.0, ident(), op(T));
      break;
    case OpType::HAM: {
      add(out, 1.0, op(ham_key()), ident());
      add(out, 1.0, ident(), op(ham_key()));
      for (int x : B) {
        add(out, 1.0, op(ccd_key(x)), op(cre_key(x), true));
        add(out, 1.0, op(ccd_key(x), true), op(cre_key(x)));
      }
      for (int i : A) {
        add(out, 1.0, op(cre_key(i), true), op(ccd_key(i)));
        add(out, 1.0, op(cre_key(i)), op(ccd_key(i), true));
      }
      // two-index terms with the single-site sub-block as loop block
      if (bdot) {
        const int x = B[0];
        add(out, 1.0, op(cdcomp_key(x, x, 0)), op(cd_key(x, x, 0)));
        add(out, 1.0, op(cdcomp_key(x, x, 2)), op(cd_key(x, x, 2)));
        add(out, 1.0, op(ddcomp_key(x, x, 0)), op(cc_key(x, x, 0)));
        add(out, 1.0, op(ddcomp_key(x, x, 0), true), op(cc_key(x, x, 0), true));
      } else if (adot) {
        const int x = A[0];
        add(out, 1.0, op(cd_key(x, x, 0)), op(cdcomp_key(x, x, 0)));
        add(out, 1.0, op(cd_key(x, x, 2)), op(cdcomp_key(x, x, 2)));
        add(out, 1.0, op(cc_key(x, x, 0)), op(ddcomp_key(x, x, 0)));
        add(out, 1.0, op(cc_key(x, x, 0), true), op(ddcomp_key(x, x, 0), true));
      } else {
        throw std::runtime_error("HAM build needs a single-site sub-block");
      }
      break;
    }
    case OpType::CD:
    case OpType::CC: {
      const int i = T.i, j = T.j, k2 = T.k2;
      const bool cd = T.type == OpType::CD;
      const double swap = (k2 == 2) ? -1.0 : 1.0;  // (-1)^k for C/D or C/C exchange across blocks
      if (inA(i) && inA(j)) add(out, 1.0, op(T), ident());
      else if (inB(i) && inB(j)) add(out, 1.0, ident(), op(T));
      else if (inA(i) && inB(j)) add(out, 1.0, op(cre_key(i)), op(cre_key(j), cd));
      else add(out, swap, op(cre_key(j), cd), op(cre_key(i)));
      break;
    }
    case OpType::CDCOMP: {
      const int i = T.i, j = T.j, k2 = T.k2;
      add(out, 1.0, op(T), ident());
      add(out, 1.0, ident(), op(T));
      auto w = [&](int p, int q) {
        return k2 == 0 ? 2.0 * I.g(i, j, p, q) - I.g(i, q, p, j) : r3 * I.g(i, q, p, j);
      };
      const double swap = (k2 == 2) ? -1.0 : 1.0;
      for (int p : A)
        for (int q : B) add(out, w(p, q), op(cre_key(p)), op(cre_key(q), true));
      for (int p : B)
        for (int q : A) add(out, swap * w(p, q), op(cre_key(q), true), op(cre_key(p)));
      break;
    }
    case OpType::DDCOMP: {
      const int i = T.i, j = T.j, k2 = T.k2;
      const int S = k2 / 2;
      add(out, 1.0, op(T), ident());
      add(out, 1.0, ident(), op(T));
      const double pre = 0.5 * (S % 2 == 0 ? -1.0 : 1.0) * std::sqrt(2.0 * S + 1.0);
      auto w = [&](int k, int l) { return pre * I.g(i, l, j, k); };
      const double swap = (k2 == 2) ? -1.0 : 1.0;
      for (int k : A)
        for (int l : B) add(out, w(k, l), op(cre_key(k), true), op(cre_key(l), true));
      for (int k : B)
        for (int l : A) add(out, swap * w(k, l), op(cre_key(l), true), op(cre_key(k), true));
      break;
    }
    case OpType::CCD: {
      const int i = T.i;
      add(out, 1.0, op(T), ident());
      add(out, 1.0, ident(), op(T));
      for (int x : B) {
        add(out, 1.0, op(cdcomp_key(x, i, 0)), op(cre_key(x)));
        add(out, 1.0, op(cdcomp_key(x, i, 2)), op(cre_key(x)));
        add(out, -2.0, op(ddcomp_key(x, i, 0), true), op(cre_key(x), true));
        add(out, -2.0, op(ddcomp_key(x, i, 2), true), op(cre_key(x), true));
      }
      for (int r : A) {
        add(out, 1.0, op(cre_key(r)), op(cdcomp_key(r, i, 0)));
        add(out, -1.0, op(cre_key(r)), op(cdcomp_key(r, i, 2)));
        add(out, -2.0, op(cre_key(r), true), op(ddcomp_key(r, i, 0), true));
        add(out, 2.0, op(cre_key(r), true), op(ddcomp_key(r, i, 2), true));
      }
      break;
    }
  }
  return out;
}

static void addp(std::vector<PairTerm>& out, double coef, Operand l, Operand r) {
  double c = coef;
  l = canonical(l, c);
  r = canonical(r, c);
  PairTerm t;
  t.coef = c;
  t.l = l;
  t.r = r;
  out.push_back(t);
}

std::vector<PairTerm> sigma_terms(const std::vector<int>& L, const std::vector<int>& R, bool loop_left) {
  std::vector<PairTerm> out;
  addp(out, 1.0, op(ham_key()), ident());
  addp(out, 1.0, ident(), op(ham_key()));
  for (int i : R) {
    addp(out, 1.0, op(ccd_key(i)), op(cre_key(i), true));
    addp(out, 1.0, op(ccd_key(i), true), op(cre_key(i)));
  }
  for (int i : L) {
    addp(out, 1.0, op(cre_key(i), true), op(ccd_key(i)));
    addp(out, 1.0, op(cre_key(i)), op(ccd_key(i), true));
  }
  const std::vector<int>& loop = loop_left ? L : R;
  for (int a : loop)
    for (int b : loop) {
      if (a < b) continue;
      for (int k2 : {0, 2}) {
        OpKey n = cd_key(a, b, k2), c = cdcomp_key(a, b, k2);
        if (loop_left) addp(out, 1.0, op(n), op(c));
        else addp(out, 1.0, op(c), op(n));
        if (a != b) {
          if (loop_left) addp(out, 1.0, op(n, true), op(c, true));
          else addp(out, 1.0, op(c, true), op(n, true));
        }
      }
      for (int k2 : {0, 2}) {
        if (k2 == 2 && a == b) continue;
        const double f = (a != b) ? 2.0 : 1.0;
        OpKey n = cc_key(a, b, k2), c = ddcomp_key(a, b, k2);
        if (loop_left) {
          addp(out, f, op(n), op(c));
          addp(out, f, op(n, true), op(c, true));
        } else {
          addp(out, f, op(c), op(n));
          addp(out, f, op(c, true), op(n, true));
        }
      }
    }
  return out;
}

// ------------------------------------------------------------------ dot

namespace {
// 4x4 Fock matrices of one spatial orbital, basis |0>, |u>, |d>, |ud>
// with |ud> = a+_u a+_d |0>.
using M4 = std::array<double, 16>;
M4 zero() { M4 m{}; return m; }
M4 mul(const M4& a, const M4& b) {
  M4 c = zero();
  for (int i = 0; i < 4; ++i)
    for (int k = 0; k < 4; ++k)
      for (int j = 0; j < 4; ++j) c[i * 4 + j] += a[i * 4 + k] * b[k * 4 + j];
  return c;
}
M4 tr(const M4& a) {
  M4 c;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) c[i * 4 + j] = a[j * 4 + i];
  return c;
}
M4 axpy(double s, const M4& a, const M4& b) {
  M4 c;
  for (int i = 0; i < 16; ++i) c[i] = s * a[i] + b[i];
  return c;
}
struct Ten {  // tensor components indexed by (q2 + k2)/2
  int k2;
  std::vector<M4> c;
  const M4& at(int q2) const { return c[(q2 + k2) / 2]; }
};
Ten couple(const Ten& A, const Ten& B, int K2) {
  Ten out{K2, std::vector<M4>(K2 + 1, zero())};
  for (int M = -K2; M <= K2; M += 2)
    for (int qa = -A.k2; qa <= A.k2; qa += 2) {
      const int qb = M - qa;
      if (qb < -B.k2 || qb > B.k2) continue;
      const double cg = clebsch(A.k2, qa, B.k2, qb, K2, M);
      if (cg == 0.0) continue;
      out.c[(M + K2) / 2] = axpy(cg, mul(A.at(qa), B.at(qb)), out.c[(M + K2) / 2]);
    }
  return out;
}
Ten scale(double s, const Ten& A) {
  Ten o = A;
  for (auto& m : o.c)
    for (auto& x : m) x *= s;
  return o;
}
Ten sum(const Ten& a, const Ten& b) {
  Ten o = a;
  for (size_t q = 0; q < o.c.size(); ++q) o.c[q] = axpy(1.0, b.c[q], a.c[q]);
  return o;
}
}  // namespace

DotOps make_dot(int x, const Integrals& I, const PointGroup& g) {
  DotOps d;
  const int sx = I.orbsym[x];
  d.si.quanta = {{0, 0, 0}, {1, 1, sx}, {2, 0, 0}};
  d.si.states = {1, 1, 1};
  // the sorted order of StateInfo: (0,0,0) < (1,1,sx) < (2,0,0)
  M4 cu = zero(), cdn = zero();
  cu[1 * 4 + 0] = 1.0;   // |0> -> |u>
  cu[3 * 4 + 2] = 1.0;   // |d> -> |ud>
  cdn[2 * 4 + 0] = 1.0;  // |0> -> |d>
  cdn[3 * 4 + 1] = -1.0; // |u> -> a+_d a+_u|0> = -|ud>
  Ten C{1, {cdn, cu}};                        // q=-1/2: a+_d, q=+1/2: a+_u
  Ten D{1, {tr(cu), scale(-1.0, Ten{1, {tr(cdn), tr(cdn)}}).c[0]}};  // q=-1/2: a_u, q=+1/2: -a_d
  auto cd = [&](int k2) { return couple(C, D, k2); };
  auto cc = [&](int k2) { return couple(C, C, k2); };
  auto dd = [&](int k2) { return couple(D, D, k2); };
  const Ten E = scale(std::sqrt(2.0), cd(0));
  const double t = I.h(x, x), vv = I.g(x, x, x, x);
  // H = t n + 1/2 v sum_st a+_s a+_t a_t a_s
  M4 ham = scale(t, E).c[0];
  {
    const M4 au = tr(cu), ad = tr(cdn);
    const M4* cre[2] = {&cu, &cdn};
    const M4* ann[2] = {&au, &ad};
    for (int s = 0; s < 2; ++s)
      for (int u = 0; u < 2; ++u)
        ham = axpy(0.5 * vv, mul(mul(*cre[s], *cre[u]), mul(*ann[u], *ann[s])), ham);
  }
  std::set<OpKey> keys = catalog_keys(dot_catalog(x, I.norb));
  d.set = make_opset(d.si, keys, I.orbsym, g);
  d.data.assign(d.set.arena, 0.0);
  // state representatives: quantum index -> (basis state, 2m)
  const int rep_state[3][2] = {{0, 0}, {1, 1}, {3, 0}};
  auto project = [&](const OpKey& key, const Ten& op) {
    const OpEntry& e = d.set.at(key);
    const OpLayout& L = d.set.layouts[e.layout];
    for (const auto& blk : L.blocks) {
      const Quantum& qb = d.si.quanta[blk.bra];
      const Quantum& qk = d.si.quanta[blk.ket];
      // find a component with non-zero Clebsch-Gordan coefficient
      const int sb = rep_state[blk.bra][0], mb = rep_state[blk.bra][1];
      const int sk = rep_state[blk.ket][0], mk = rep_state[blk.ket][1];
      double val = 0.0;
      bool found = false;
      const int q2 = mb - mk;
      if (q2 >= -op.k2 && q2 <= op.k2) {
        const double cg = clebsch(qk.s2, mk, op.k2, q2, qb.s2, mb);
        if (std::fabs(cg) > 1e-12) {
          val = op.at(q2)[sb * 4 + sk] / cg;
          found = true;
        }
      }
      if (!found) throw std::runtime_error("dot projection failed for " + key.str());
      d.data[e.base + blk.offset] = val;
    }
  };
  const double r2 = std::sqrt(2.0), r3 = std::sqrt(3.0);
  project(ham_key(), Ten{0, {ham}});
  M4 id = zero();
  for (int i = 0; i < 4; ++i) id[i * 4 + i] = 1.0;
  project(overlap_key(), Ten{0, {id}});
  project(cre_key(x), C);
  project(cd_key(x, x, 0), cd(0));
  project(cd_key(x, x, 2), cd(2));
  project(cc_key(x, x, 0), cc(0));
  for (const auto& kv : d.set.ops) {
    const OpKey& k = kv.first;
    if (k.type == OpType::CCD) {
      const int i = k.i;
      // sqrt(2) (1/2 t_xi C_x + (xi|xx) C_x E_xx)
      Ten z = sum(scale(0.5 * I.h(x, i), C), scale(I.g(x, i, x, x), couple(C, E, 1)));
      project(k, scale(r2, z));
    } else if (k.type == OpType::CDCOMP) {
      const int i = k.i, j = k.j;
      const double w = k.k2 == 0 ? 2.0 * I.g(i, j, x, x) - I.g(i, x, x, j) : r3 * I.g(i, x, x, j);
      project(k, scale(w, cd(k.k2)));
    } else if (k.type == OpType::DDCOMP) {
      const int i = k.i, j = k.j, S = k.k2 / 2;
      const double w = 0.5 * (S % 2 == 0 ? -1.0 : 1.0) * std::sqrt(2.0 * S + 1.0) * I.g(i, x, j, x);
      project(k, scale(w, dd(k.k2)));
    }
  }
  return d;
}

}  // namespace bgpu
