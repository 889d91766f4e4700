// Spin and point-group bookkeeping for spin-adapted DMRG.
//
// Quantum numbers are (particle number n, twice the total spin s2, abelian irrep).
// Spins are carried as 2j integers throughout, like the reference
// (SpinQuantum.h:25-82, SpinSpace.C:16-33).  The angular-momentum functions
// restate the Racah formulas used by the reference (new_anglib.C:19-316) with
// the same order of floating-point operations so that coupling factors are
// bit-identical; ninej() is the normalised 9j of couplingCoeffs.h:88-97.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace bgpu {

// Abelian point groups supported on the hot path: C1 and D2h (and its
// subgroups of order 2 and 4, which share the XOR product rule).  The product
// table is the XOR of 0-based irrep indices (Symmetry.C:22-120).
struct PointGroup {
  int nirrep = 1;
  std::string name = "c1";
  static PointGroup from_name(const std::string& s);
  int product(int a, int b) const { return a ^ b; }
  int inverse(int a) const { return a; }
};

struct Quantum {
  int n = 0;      // particle number
  int s2 = 0;     // 2S
  int irrep = 0;  // 0-based abelian irrep
  bool operator==(const Quantum& o) const { return n == o.n && s2 == o.s2 && irrep == o.irrep; }
  bool operator!=(const Quantum& o) const { return !(*this == o); }
  // ordering of SpinQuantum::operator< (SpinQuantum.C:120-125)
  bool operator<(const Quantum& o) const {
    if (n != o.n) return n < o.n;
    if (s2 != o.s2) return s2 < o.s2;
    return irrep < o.irrep;
  }
};

inline bool is_fermion(const Quantum& q) { return (q.n & 1) != 0; }

// a in b (x) c  (spin triangle, particle number and irrep product)
bool quantum_allowed(const Quantum& a, const Quantum& b, const Quantum& c, const PointGroup& g);

// Racah-formula restatements (new_anglib.C).  All spin arguments are 2j.
double fbinom(int n, int r);
double clebsch(int j1, int m1, int j2, int m2, int j3, int m3);
double six_j(int a, int b, int c, int d, int e, int f);
double nine_j(int a, int b, int c, int d, int e, int f, int g, int h, int i);
// sqrt((g+1)(h+1)(c+1)(f+1)) * {a b c; d e f; g h i}  (couplingCoeffs.h:88-97)
double ninej_norm(int a, int b, int c, int d, int e, int f, int g, int h, int i);

// Cached normalised 9j (the reference keeps the same values in a table,
// couplingCoeffs.C:131-200); thread-safe for concurrent readers after warm-up.
double ninej(int a, int b, int c, int d, int e, int f, int g, int h, int i);

// Scaling of the reduced element of the adjoint tensor of an operator of
// rank k2 between (bra spin l2, ket spin r2): the stored block is the
// original operator's (r, l) block.  Restates Transposeview::get_scaling
// (BaseOperator.C:56-91) for abelian groups.
double transpose_scaling(int l2, int r2, int k2);

// Sign/phase for re-ordering two coupled tensors [A^a x B^b]^c -> [B^b x A^a]^c
// (getCommuteParity, BaseOperator.C:20-53).
double commute_parity(const Quantum& a, const Quantum& b, int c2);

}  // namespace bgpu
