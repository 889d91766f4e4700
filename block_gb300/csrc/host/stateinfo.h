// Sector bookkeeping of a block: the quanta it carries, how many multiplets
// each holds, and (for a block made of two sub-blocks) which sub-block
// sectors make up each of its sectors and at which row offset.
//
// Restates StateInfo (StateInfo.h:79-206): TensorProduct of two StateInfos
// (StateInfo.C:123-308) followed by CollectQuanta (StateInfo.C:310-341).
// The uncollected product is enumerated left-quantum major, right-quantum
// minor, then by total spin; collecting sorts the quanta with
// Quantum::operator< and concatenates the uncollected parts of each
// collected quantum in enumeration order, so that each product sector is a
// stack of (left sector x right sector) Kronecker tiles.
#pragma once
#include <map>
#include <vector>

#include "su2.h"

namespace bgpu {

struct SectorPart {
  int lq = 0, rq = 0;  // quantum index in the left / right sub-block
  int offset = 0;      // first row (state) of this part inside the sector
  int size = 0;        // states(lq) * states(rq)
};

struct StateInfo {
  std::vector<Quantum> quanta;  // sorted, unique
  std::vector<int> states;      // number of multiplets per quantum
  // product blocks only: composition of every sector
  std::vector<std::vector<SectorPart>> parts;
  // (lq, rq) -> every (sector, part index) it forms (one per coupled total
  // spin that is kept), dense over left x right quanta
  int nleft = 0, nright = 0;
  std::vector<std::vector<std::pair<int, int>>> part_index;
  const std::vector<std::pair<int, int>>& parts_of(int lq, int rq) const {
    return part_index[(size_t)lq * nright + rq];
  }

  int size() const { return (int)quanta.size(); }
  long total_states() const;
  int find(const Quantum& q) const;  // -1 if absent
  bool is_product() const { return !parts.empty(); }
};

// Filter used when forming a block of `nsites` orbitals out of a system with
// `norb` orbitals, total particle number `nelec` and total spin `s2`:
// keeps quanta that can still be completed to the target by the remaining
// orbitals (SpinQuantum::can_complement, SpinQuantum.C:127-132, plus the
// particle-number range of the complement).
struct QuantumFilter {
  int nelec = 0, s2 = 0, norb = 0;
  bool keep(const Quantum& q, int nsites) const;
};

// Product of two blocks' state spaces.  If `target` is given, only that
// total quantum is kept (superblock); otherwise `filter` prunes quanta.
StateInfo product_stateinfo(const StateInfo& a, const StateInfo& b, const PointGroup& g,
                            const QuantumFilter* filter, int nsites, const Quantum* target);

// Renormalised state space: same quanta as `big`, states[q] = kept[q];
// quanta with kept[q] == 0 are dropped.  `index_map[q_big]` receives the new
// index or -1.
StateInfo truncated_stateinfo(const StateInfo& big, const std::vector<int>& kept, std::vector<int>& index_map);

}  // namespace bgpu
