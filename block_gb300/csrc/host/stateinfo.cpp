#include "stateinfo.h"

#include <algorithm>
#include <cstdlib>
#include <stdexcept>

namespace bgpu {

long StateInfo::total_states() const {
  long t = 0;
  for (int s : states) t += s;
  return t;
}

int StateInfo::find(const Quantum& q) const {
  auto it = std::lower_bound(quanta.begin(), quanta.end(), q);
  if (it == quanta.end() || !(*it == q)) return -1;
  return (int)(it - quanta.begin());
}

bool QuantumFilter::keep(const Quantum& q, int nsites) const {
  if (q.n < 0 || q.n > nelec) return false;
  const int rest_sites = norb - nsites;
  const int rest_n = nelec - q.n;
  if (rest_n > 2 * rest_sites) return false;
  // spin of the complement must be able to couple q.s2 to the target
  if (std::abs(s2 - q.s2) > rest_n) return false;
  return true;
}

StateInfo product_stateinfo(const StateInfo& a, const StateInfo& b, const PointGroup& g,
                            const QuantumFilter* filter, int nsites, const Quantum* target) {
  struct Unc {
    Quantum q;
    int lq, rq, size;
  };
  std::vector<Unc> unc;
  for (int i = 0; i < a.size(); ++i)
    for (int j = 0; j < b.size(); ++j) {
      const Quantum& qa = a.quanta[i];
      const Quantum& qb = b.quanta[j];
      for (int s2 = std::abs(qa.s2 - qb.s2); s2 <= qa.s2 + qb.s2; s2 += 2) {
        Quantum q{qa.n + qb.n, s2, g.product(qa.irrep, qb.irrep)};
        if (target && !(q == *target)) continue;
        if (!target && filter && !filter->keep(q, nsites)) continue;
        unc.push_back({q, i, j, a.states[i] * b.states[j]});
      }
    }
  StateInfo out;
  std::vector<Quantum> qs;
  for (auto& u : unc) qs.push_back(u.q);
  std::sort(qs.begin(), qs.end());
  qs.erase(std::unique(qs.begin(), qs.end()), qs.end());
  out.quanta = qs;
  out.states.assign(qs.size(), 0);
  out.parts.assign(qs.size(), {});
  out.nleft = a.size();
  out.nright = b.size();
  out.part_index.assign((size_t)out.nleft * out.nright, {});
  for (auto& u : unc) {
    int c = out.find(u.q);
    SectorPart p;
    p.lq = u.lq;
    p.rq = u.rq;
    p.offset = out.states[c];
    p.size = u.size;
    out.part_index[(size_t)u.lq * out.nright + u.rq].push_back({c, (int)out.parts[c].size()});
    out.parts[c].push_back(p);
    out.states[c] += u.size;
  }
  return out;
}

StateInfo truncated_stateinfo(const StateInfo& big, const std::vector<int>& kept, std::vector<int>& index_map) {
  StateInfo out;
  index_map.assign(big.size(), -1);
  for (int q = 0; q < big.size(); ++q) {
    if (kept[q] <= 0) continue;
    index_map[q] = (int)out.quanta.size();
    out.quanta.push_back(big.quanta[q]);
    out.states.push_back(kept[q]);
  }
  return out;
}

}  // namespace bgpu
