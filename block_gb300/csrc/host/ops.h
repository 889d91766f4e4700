// Operator catalogue, block-sparse operator layouts and the algebraic
// recipes of the two-site sweep.
//
// Operator types follow the reference's opTypes (BaseOperator.h:35-45) for
// the spin-adapted Hamiltonian path: HAM, CRE (C_i), CRE_DES (CD^k_ij),
// CRE_CRE (CC^S_ij), CRE_DESCOMP (CDcomp^k_ij), DES_DESCOMP (DDcomp^S_ij),
// CRE_CRE_DESCOMP (CCDcomp_i) and OVERLAP.  Every operator is an SU(2)
// tensor whose reduced blocks are stored per allowed (bra, ket) quantum
// pair, row-major (Newmat layout, MatrixBLAS.C:144).
//
// Conventions (checked against a determinant-space model of the operators):
//   D_i = adjoint tensor of C_i (Transposeview, BaseOperator.h:208-243)
//   CD^k_ij     = [C_i x D_j]^k
//   CC^S_ij     = [C_i x C_j]^S
//   CDcomp^0_ij = sum_kl (2(ij|kl) - (il|kj)) CD^0_kl
//   CDcomp^1_ij = sqrt(3) sum_kl (il|kj) CD^1_kl
//   DDcomp^S_ij = 1/2 (-1)^(S+1) sqrt(2S+1) sum_kl (il|jk) [D_k x D_l]^S
//   CCDcomp_i   = sqrt(2) ( 1/2 sum_p t_pi C_p + sum_prs (pi|rs) C_p E_rs )
// so that, for a bipartition L|R,
//   H = H_L + H_R + sum_{i in R} ([CCD_i(L) x D_i(R)]^0 + h.c.)
//       + sum_{i in L} ([D_i(L) x CCD_i(R)]^0 + h.c.)
//       + sum_{ij in loop} sum_k [CD^k_ij x CDcomp^k_ij]^0
//       + sum_{ij in loop} sum_S ([CC^S_ij x DDcomp^S_ij]^0 + h.c.)
// which is the operator-pair form of SpinBlock::multiplyH
// (spinblock.C:722-789, opxop.C:155-285).
#pragma once
#include <cstdint>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "integrals.h"
#include "stateinfo.h"

namespace bgpu {

enum class OpType : uint8_t { HAM = 0, CRE, CD, CC, CDCOMP, DDCOMP, CCD, OVERLAP };

const char* op_type_name(OpType t);

struct OpKey {
  OpType type = OpType::HAM;
  int16_t i = -1, j = -1;
  int8_t k2 = 0;  // twice the tensor rank
  bool operator<(const OpKey& o) const {
    if (type != o.type) return type < o.type;
    if (i != o.i) return i < o.i;
    if (j != o.j) return j < o.j;
    return k2 < o.k2;
  }
  bool operator==(const OpKey& o) const { return type == o.type && i == o.i && j == o.j && k2 == o.k2; }
  std::string str() const;
};

OpKey ham_key();
OpKey overlap_key();
OpKey cre_key(int i);
OpKey cd_key(int i, int j, int k2);
OpKey cc_key(int i, int j, int k2);
OpKey cdcomp_key(int i, int j, int k2);
OpKey ddcomp_key(int i, int j, int k2);
OpKey ccd_key(int i);

// quantum change of an operator (n, 2k, irrep)
Quantum op_dq(const OpKey& k, const std::vector<int>& orbsym);
inline bool op_fermion(const OpKey& k) {
  return k.type == OpType::CRE || k.type == OpType::CCD;
}

// One stored reduced block of an operator.
struct OpBlock {
  int bra = 0, ket = 0;
  int rows = 0, cols = 0;
  int64_t offset = 0;  // element offset inside the operator
};

// Block-sparse structure shared by all operators with the same quantum change
// on one state space (SparseMatrix::allocate, BaseOperator.C:123-145).
struct OpLayout {
  Quantum dq;
  std::vector<OpBlock> blocks;
  int nq = 0;               // quanta of the block's state space
  std::vector<int> index;   // bra * nq + ket -> block, -1 if not allowed
  std::vector<std::vector<int>> by_ket;  // ket -> blocks with that ket
  std::vector<std::vector<int>> by_bra;  // bra -> blocks with that bra
  int64_t size = 0;
  int find(int bra, int ket) const { return index[(size_t)bra * nq + ket]; }
};

OpLayout make_layout(const StateInfo& si, const Quantum& dq, const PointGroup& g);

struct OpEntry {
  int layout = -1;
  int64_t base = 0;  // element offset of the operator inside the block arena
};

// All operators of one block: catalogue, layouts and arena offsets.
struct OpSet {
  std::vector<OpLayout> layouts;
  std::map<OpKey, OpEntry> ops;
  int64_t arena = 0;  // total elements
  bool has(const OpKey& k) const { return ops.count(k) != 0; }
  const OpEntry& at(const OpKey& k) const;
  const OpLayout& layout_of(const OpKey& k) const { return layouts[at(k).layout]; }
};

OpSet make_opset(const StateInfo& si, const std::set<OpKey>& keys, const std::vector<int>& orbsym,
                 const PointGroup& g);

// ---- catalogues ----
// Which operators a block with the given sites carries.
struct CatalogSpec {
  std::vector<int> sites;
  std::vector<int> ccd_sites;                    // CCD_i for these i (outside the block)
  bool normal = false;                           // CD/CC for pairs inside the block
  std::vector<std::pair<int, int>> comp_pairs;   // CDcomp/DDcomp pairs (i >= j), outside the block
  std::vector<OpKey> extra;                      // further operators (density-matrix evaluation)
};
std::set<OpKey> catalog_keys(const CatalogSpec& s);

// The dot (single-site) block carries every operator it could ever be
// asked for (set_spinblock_components.C:331-390).
CatalogSpec dot_catalog(int site, int norb);

// ---- recipes ----
// A factor of a coupled product: an operator of one sub-block, possibly in
// its adjoint-tensor form, or that sub-block's identity.
struct Operand {
  OpKey key;
  bool trans = false;
  bool identity = false;
};
inline Operand ident() { Operand o; o.identity = true; o.key = overlap_key(); return o; }
inline Operand op(const OpKey& k, bool t = false) { Operand o; o.key = k; o.trans = t; return o; }

// target += coef * [a x b]^{rank(target)}
struct BuildTerm {
  double coef = 1.0;
  Operand a, b;
};

// sigma += coef * [l x r]^0 psi
struct PairTerm {
  double coef = 1.0;
  Operand l, r;
};

// Terms that build `target` on the block made of sub-blocks with sites
// `asites` (left) and `bsites` (right); restates the build() of each
// operator class in Operators.C (Cre 453-488, CreDes 624-692,
// CreDesComp 1059-1194, DesDesComp 1472-1615, CreCreDesComp 1905-1967,
// Ham 2322-2395) in the conventions above.
std::vector<BuildTerm> build_terms(const OpKey& target, const std::vector<int>& asites,
                                   const std::vector<int>& bsites, const Integrals& I);

// Operator pairs of sigma = H psi for the superblock L|R with the given loop
// side (SpinBlock::multiplyH, spinblock.C:722-789).
std::vector<PairTerm> sigma_terms(const std::vector<int>& lsites, const std::vector<int>& rsites, bool loop_is_left);

// Canonical (stored) form of a possibly reversed complementary pair operand:
// CDcomp^k_ab (a<b) = e_k T(CDcomp^k_ba), DDcomp^S_ab (a<b) = (-1)^S DDcomp^S_ba.
Operand canonical(const Operand& o, double& coef);

// ---- dot block ----
// Reduced 1x1 blocks of every dot operator of orbital `x` on the single-site
// state space {|0>, |up/dn>, |updn>}; values in layout block order.
struct DotOps {
  StateInfo si;
  OpSet set;
  std::vector<double> data;  // arena of the OpSet
};
DotOps make_dot(int x, const Integrals& I, const PointGroup& g);

}  // namespace bgpu
