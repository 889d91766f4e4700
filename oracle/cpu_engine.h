// TEST INFRASTRUCTURE ONLY.  CPU restatement (FP64) of the sweep hot path,
// used as the oracle the CUDA engine is checked against and as the timed
// CPU baseline.  Nothing in the block_gb300 package may link or call this.
//
// Parity is pinned by the reference's golden energies (dmrg_tests/runtest,
// pydmrg/tests/test_dmrg_simple.py), reproduced by tests/test_oracle_golden.py.
#pragma once
#include <map>
#include <vector>

#include "../block_gb300/csrc/host/sweep.h"

namespace oracle {

using namespace bgpu;

// Row-major C = alpha * op(A) * op(B) + beta * C, op = transpose when t* is true.
void dgemm(bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb,
           double beta, double* C, int ldc);
// the built-in loop of dgemm (used when no tuned BLAS is set)
void dgemm_loop(bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda, const double* B,
                int ldb, double beta, double* C, int ldc);
// Fortran DGEMM (column-major, arguments by reference)
typedef void (*FortranDgemm)(const char* ta, const char* tb, const int* m, const int* n, const int* k,
                             const double* alpha, const double* a, const int* lda, const double* b, const int* ldb,
                             const double* beta, double* c, const int* ldc);
extern FortranDgemm g_blas_dgemm;

class CpuEngine : public Engine {
 public:
  explicit CpuEngine(int threads = 0);
  std::string name() const override { return "cpu-oracle"; }
  void create_block(Block& b) override;
  void release_block(Block& b) override;
  void upload_block(Block& b, const std::vector<double>& arena) override;
  void download_block(const Block& b, std::vector<double>& arena) override;
  void build_block(Block& big, const Block& a, const Block& b,
                   const std::vector<std::pair<OpKey, std::vector<BuildTerm>>>& recipes) override;
  int solve(const Superblock& sb, const DavidsonParams& p, std::vector<double>& energies) override;
  void density(const Superblock& sb, bool left, const std::vector<double>& weights, DensitySpectrum& spec) override;
  void select_rotation(const std::vector<std::vector<int>>& kept) override;
  void set_rotation(const std::vector<std::vector<double>>& rot, const std::vector<int>& kept) override;
  void renormalise(Block& small, const Block& big) override;
  void expectations(const Superblock& sb, const std::vector<PairTerm>& terms, std::vector<double>& out) override;
  // TRANSFORM guess (guess_wavefunction.C:526-620): the last solve's vectors
  // carried to the next step's superblock through the rotation kept with
  // `rotated` and the one kept with `expanded`
  bool transform_guess(const GuessInput& g, const Superblock& sb) override;
  bool get_rotation_record(const Block& b, RotationRecord& r) override;
  void set_rotation_record(const Block& b, const RotationRecord& r) override;
  int64_t block_bytes() const override {
    int64_t n = 0;
    for (const auto& kv : store_) n += 8 * (int64_t)kv.second.size();
    return n;
  }

  // pieces exposed for tests and the bench
  void sigma(const Superblock& sb, const double* psi, double* out);
  void hdiag(const Superblock& sb, double* diag);
  const std::vector<double>& arena(const Block& b) const { return store_.at(b.handle); }
  std::vector<double>& arena(Block& b) { return store_.at(b.handle); }
  const std::vector<std::vector<double>>& wavefunctions() const { return waves_; }
  void set_wavefunctions(const std::vector<std::vector<double>>& w) { waves_ = w; }
  // the last density matrix per sector (row-major), its eigenvectors (row-major,
  // columns in ascending eigenvalue order) and the current rotation (per big
  // sector, rows x kept row-major)
  const std::vector<std::vector<double>>& density_matrices() const { return dm_rho_; }
  const std::vector<std::vector<double>>& density_vectors() const { return dm_vecs_; }
  const std::vector<std::vector<double>>& rotation() const { return rot_; }
  const std::vector<int>& rotation_kept() const { return rot_kept_; }
  // structure only: blocks keep their state spaces and catalogues but no
  // arenas, and builds / renormalisations do no arithmetic (a superblock of
  // the right shape for timing, filled afterwards by fill_random)
  bool structure_only = false;
  void fill_random(Block& b, uint64_t seed);
  double sigma_seconds = 0.0;
  long sigma_calls = 0;
  double last_sigma_flops = 0.0;  // GEMM flops of the last sigma (2mnk per product)
  int threads = 1;

 private:
  void add_noise(const Superblock& sb, bool left, std::vector<std::vector<double>>& rho);
  void apply_one(const Superblock& sb, bool left, const Operand& o, const std::vector<double>& psi,
                 const std::vector<Superblock::Sector>& out, int s2_out, std::vector<double>& phi);
  std::map<int, std::vector<double>> store_;
  int next_handle_ = 0;
  // the rotation each renormalised block was made with, per big-block
  // sector q: u[q] (n[q] x m[q], row-major, m[q] kept states), and the
  // sector maps between the big and the renormalised block
  struct Rot {
    std::vector<int> n, m, small_of_big, big_of_small;
    std::vector<std::vector<double>> u;
  };
  std::map<int, Rot> block_rot_;
  std::vector<std::vector<double>> guess_;  // transformed vectors for the next solve
  std::vector<std::vector<double>> waves_;
  std::vector<std::vector<double>> dm_vecs_;  // eigenvectors per density-matrix sector (columns, ascending)
  std::vector<std::vector<double>> dm_rho_;   // the density matrix per sector
  std::vector<int> dm_dims_;
  std::vector<std::vector<double>> rot_;       // per big sector: rows x kept
  std::vector<int> rot_kept_;
};

}  // namespace oracle
