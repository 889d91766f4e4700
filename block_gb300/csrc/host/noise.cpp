// Host-side pieces of the density-matrix noise (DensityMatrix::add_onedot_noise
// with onedot_noise_f, density.C:180-421, and add_twodot_noise,
// density.C:92-165): wavefunction sectors of a total quantum, the quanta of
// the random noise and the operator list of the perturbative noise.
#include <cstdlib>

#include "sweep.h"

namespace bgpu {

std::vector<Superblock::Sector> wave_sectors(const StateInfo& L, const StateInfo& R, const Quantum& q,
                                             const PointGroup& g, int64_t& size) {
  std::vector<Superblock::Sector> out;
  size = 0;
  if (q.n < 0 || q.s2 < 0) return out;
  for (int lq = 0; lq < L.size(); ++lq)
    for (int rq = 0; rq < R.size(); ++rq) {
      if (!quantum_allowed(q, L.quanta[lq], R.quanta[rq], g)) continue;
      Superblock::Sector s;
      s.lq = lq;
      s.rq = rq;
      s.rows = L.states[lq];
      s.cols = R.states[rq];
      s.offset = size;
      size += (int64_t)s.rows * s.cols;
      out.push_back(s);
    }
  return out;
}

// The quanta of add_twodot_noise (density.C:107-134), 2S units: particle
// number +-1 with spin +-1/2, particle number 0, +-2 with spin 0, +-1.
std::vector<Quantum> random_noise_quanta(const Quantum& t) {
  std::vector<Quantum> q;
  auto add = [&](int dn, int ds2) { q.push_back({t.n + dn, t.s2 + ds2, t.irrep}); };
  add(+1, +1);
  add(-1, +1);
  if (t.s2 >= 1) {
    add(+1, -1);
    add(-1, -1);
  }
  add(+2, +2);
  add(0, +2);
  add(-2, +2);
  add(+2, 0);
  add(-2, 0);
  if (t.s2 >= 2) {
    add(+2, -2);
    add(0, -2);
    add(-2, -2);
  }
  return q;
}

// Operators of the perturbative noise on block B (add_onedot_noise,
// density.C:373-399): CRE, then CC and CD when B carries the normal
// two-index operators, else DDCOMP and CDCOMP; each as itself and as its
// adjoint (onedot_noise_f, density.C:228-259), coupled with the target to
// every total spin of target (x) operator.
std::vector<NoiseOp> perturbative_noise_ops(const Block& B, const Quantum& t, const std::vector<int>& orbsym,
                                            const PointGroup& g) {
  bool normal = false;
  for (const auto& kv : B.ops.ops)
    if (kv.first.type == OpType::CC) normal = true;
  const OpType types[3] = {OpType::CRE, normal ? OpType::CC : OpType::DDCOMP, normal ? OpType::CD : OpType::CDCOMP};
  std::vector<NoiseOp> out;
  for (OpType ty : types)
    for (const auto& kv : B.ops.ops) {
      if (kv.first.type != ty) continue;
      const Quantum dq = op_dq(kv.first, orbsym);
      for (int tr = 0; tr < 2; ++tr) {
        const int n = t.n + (tr ? -dq.n : dq.n);
        if (n < 0) continue;
        const int irrep = g.product(t.irrep, dq.irrep);
        for (int s2 = std::abs(t.s2 - dq.s2); s2 <= t.s2 + dq.s2; s2 += 2) out.push_back({kv.first, tr != 0, {n, s2, irrep}});
      }
    }
  return out;
}

}  // namespace bgpu
