// Two-site DMRG sweep driver (host side).
//
// Restates the control flow of Sweep::do_one / BlockAndDecimate
// (sweep.C:180-545), InitBlocks (initblocks.C), RenormaliseFrom
// (renormalise.C:39-130) and dmrg() (dmrg.C:600-706) for the spin-adapted,
// two-dot, noise-free hot path.  All floating-point work on operators and
// wavefunctions is delegated to an Engine: the CUDA engine of this library
// in production, and the CPU restatement that serves as the test oracle.
#pragma once
#include <functional>
#include <memory>
#include <string>
#include <map>
#include <vector>

#include "checkpoint.h"
#include "integrals.h"
#include "ops.h"
#include "stateinfo.h"

namespace bgpu {

// A block of consecutive sites with its state space and operator catalogue.
struct Block {
  std::vector<int> sites;
  StateInfo si;
  OpSet ops;
  bool is_dot = false;
  int handle = -1;  // engine-side storage id
};

// The superblock L|R of one sweep step.
struct Superblock {
  const Block* L = nullptr;
  const Block* R = nullptr;
  StateInfo si;       // single target quantum; parts = (lq, rq) sectors of psi
  Quantum target;
  bool loop_left = true;
  std::vector<PairTerm> terms;
  double ecore = 0.0;
  // flattened psi layout: sector s = (lq, rq), offset, rows = states(lq), cols = states(rq)
  struct Sector { int lq, rq, rows, cols; int64_t offset; };
  std::vector<Sector> sectors;
  int64_t size = 0;
};

// Per-step Davidson settings (linear.C:179-385).
struct DavidsonParams {
  int nroots = 1;
  double tol = 1e-8;  // on the squared residual norm
  int max_iter = 200;
  int deflation_min = 2, deflation_max = 20;
  uint64_t seed = 1;
  // engines that iterate in a split precision: leave the FP64 Rayleigh-quotient
  // refinement of the energies to a later refine() call
  bool defer_refine = false;
  // start from the engine's transformed guess (transform_guess) instead of
  // unit vectors on the lowest diagonal elements
  bool use_guess = false;
};

// The previous block step of the same sweep direction, for the wavefunction
// guess transform (GuessWave::transform_previous_wavefunction,
// guess_wavefunction.C:526-620): its enlarged blocks' state spaces and psi
// sectors, the block renormalised at that step (B_L(p-1) in a forward sweep,
// B_R(p+2) in a backward one), the block re-expanded through the rotation
// that made it (B_R(p+1) forward, B_L(p) backward) and the single site
// shared by the old right (forward) or left (backward) enlarged block and the
// new left (forward) or right (backward) one.
struct GuessInput {
  bool forward = true;
  StateInfo old_L, old_R;
  std::vector<Superblock::Sector> old_sectors;
  const Block* rotated = nullptr;
  const Block* expanded = nullptr;
  const StateInfo* dot = nullptr;
};

// Density-matrix spectrum of the block being renormalised: per sector of
// that block, eigenvalues ascending.
struct DensitySpectrum {
  std::vector<std::vector<double>> eig;
};

// Noise added to the density matrices of the next density() calls
// (DensityMatrix::makedensitymatrix, density.C:27-90):
//   perturbative: add_onedot_noise (density.C:330-421): for every root,
//     rho += noise / nroots / tr(N) * N with N = sum over the normalised
//     (O x 1) psi (O x 1)^T psi of the renormalised block's CRE and its
//     two-index operators (CC, CD; or DDCOMP, CDCOMP on a block without
//     them) and their adjoints, over every total spin they couple psi to,
//     when tr(N) > 1;
//   random: add_twodot_noise (density.C:92-165): for every root, normalised
//     random wavefunctions of the quanta next to the target (N +- 1, 2;
//     2S +- 1, 2) each add noise / nroots / (number of quanta) of their
//     outer product; values uniform in [-1, 1) from a counter-based hash of
//     (seed, quantum, element), identical on every engine.
struct NoiseSpec {
  double perturbative = 0.0;
  double random = 0.0;
  uint64_t seed = 0;
  std::vector<int> orbsym;  // orbital irreps (operator quanta)
  PointGroup group;
  bool any() const { return perturbative > 0.0 || random > 0.0; }
};

class Engine {
 public:
  // noise of the following density() calls (none by default)
  virtual void set_noise(const NoiseSpec& n) { noise_ = n; }
  const NoiseSpec& noise() const { return noise_; }
  virtual ~Engine() = default;
  virtual std::string name() const = 0;
  // storage
  virtual void create_block(Block& b) = 0;  // allocates b.ops.arena elements
  virtual void release_block(Block& b) = 0;
  virtual void upload_block(Block& b, const std::vector<double>& arena) = 0;
  virtual void download_block(const Block& b, std::vector<double>& arena) = 0;
  // big = a (x) b built by per-operator recipes
  virtual void build_block(Block& big, const Block& a, const Block& b,
                           const std::vector<std::pair<OpKey, std::vector<BuildTerm>>>& recipes) = 0;
  // Davidson on the superblock; energies of the converged roots.  The
  // wavefunctions stay inside the engine.
  virtual int solve(const Superblock& sb, const DavidsonParams& p, std::vector<double>& energies) = 0;
  // prepares a guess for the next solve on `sb` by transforming the last
  // solve's vectors; false if the engine cannot (the solve then starts from
  // unit vectors)
  virtual bool transform_guess(const GuessInput& g, const Superblock& sb) {
    (void)g;
    (void)sb;
    return false;
  }
  // keeps a copy of the last solve's vectors for a later refine_parked();
  // returns an id, or -1 if the engine does not defer refinements
  virtual int park_vectors() { return -1; }
  // FP64 Rayleigh quotients of parked vectors on their superblock
  virtual bool refine_parked(int id, const Superblock& sb, std::vector<double>& energies) {
    (void)id;
    (void)sb;
    (void)energies;
    return false;
  }
  virtual void drop_parked(int id) { (void)id; }
  // engine-specific timing of the last block step, for verbose logs
  virtual std::string step_stats() { return std::string(); }
  // loads the dense eigensolver of the density-matrix sectors for sectors of
  // up to max_n states (called once by the warm-up, before the first sweep)
  virtual void prepare_density(int max_n) { (void)max_n; }
  // compiles the sigma work lists of the superblock the next solve() gets
  // (engines that run asynchronously overlap this with device work)
  virtual void prepare_plan(const Superblock& sb) { (void)sb; }
  // device seconds of the renormalisations so far (< 0: not measured)
  virtual double device_renorm_seconds() { return -1.0; }
  // FP64-equivalent flops of the renormalisations so far (0 if not counted)
  virtual double renorm_flops() const { return 0.0; }
  // rotation that made a renormalised block (kept by engines that transform
  // wavefunction guesses), read and restored by checkpoints
  virtual bool get_rotation_record(const Block& b, RotationRecord& r) {
    (void)b;
    (void)r;
    return false;
  }
  virtual void set_rotation_record(const Block& b, const RotationRecord& r) {
    (void)b;
    (void)r;
  }
  // FP64 Rayleigh quotients of the last solve's vectors (no-op for engines
  // that solve in FP64); returns true if the energies changed precision
  virtual bool refine(const Superblock& sb, std::vector<double>& energies) {
    (void)sb;
    (void)energies;
    return false;
  }
  // reduced density matrix of the left (forward) or right (backward) block
  // from the engine's current wavefunctions and its eigen-decomposition.
  virtual void density(const Superblock& sb, bool left, const std::vector<double>& weights, DensitySpectrum& spec) = 0;
  // keep eigenvectors `kept[q]` (indices into the ascending spectrum) of
  // every sector as the rotation of the block being renormalised
  virtual void select_rotation(const std::vector<std::vector<int>>& kept) = 0;
  // or use an explicit host rotation (warm-up): per sector, rows x kept, row-major
  virtual void set_rotation(const std::vector<std::vector<double>>& rot, const std::vector<int>& kept) = 0;
  // small = rotation^T big rotation for every operator of small's catalogue
  virtual void renormalise(Block& small, const Block& big) = 0;
  // bytes of block storage (operator arenas) the engine holds now
  virtual int64_t block_bytes() const { return 0; }
  // matrix elements <psi_a| coef * [l x r]^0 |psi_b> of single pair terms
  // between the last solve's vectors (nr of them):
  // out[(a * nr + b) * terms.size() + t]
  virtual void expectations(const Superblock& sb, const std::vector<PairTerm>& terms, std::vector<double>& out) = 0;

 protected:
  NoiseSpec noise_;
};

// Host-side pieces of the noise shared by the engines: the sectors (lq, rq,
// rows, cols, offset) of a wavefunction with total quantum q on L x R, the
// neighbouring quanta of the random noise, its uniform values, and the
// operator list of the perturbative noise.
std::vector<Superblock::Sector> wave_sectors(const StateInfo& L, const StateInfo& R, const Quantum& q,
                                             const PointGroup& g, int64_t& size);
std::vector<Quantum> random_noise_quanta(const Quantum& target);
struct NoiseOp {
  OpKey key;
  bool trans;
  Quantum q;  // total quantum of (O x 1) psi (or (1 x O) psi)
};
std::vector<NoiseOp> perturbative_noise_ops(const Block& B, const Quantum& target, const std::vector<int>& orbsym,
                                            const PointGroup& g);

struct SweepResult {
  std::vector<double> energies;         // final energy per root
  std::vector<double> sweep_energies;   // lowest root, per sweep
  std::vector<double> sweep_seconds;    // wall time per sweep (device work included)
  double warmup_seconds = 0.0;          // wall time of the warm-up (0 on restart)
  // `onepdm`: per root, the spin-summed spatial one-particle density matrix
  // gamma_ij = sum_s <a+_is a_js> (norb x norb row-major, input orbital order)
  std::vector<std::vector<double>> onepdm;
  // with it, between roots a and b (index a * nroots + b): <a|E_ij|b>
  std::vector<std::vector<double>> transition_onepdm;
  double discarded = 0.0;
  int sweeps = 0;
  double sigma_seconds = 0.0;
  long sigma_calls = 0;
  // wall seconds per phase of the block steps: enlarged-block builds and
  // superblock set-up, Davidson solve, density matrix + rotation choice,
  // renormalisation
  double build_seconds = 0.0, solve_seconds = 0.0, density_seconds = 0.0, renorm_seconds = 0.0;
  double renorm_device_seconds = -1.0;  // device time of the renormalisations (< 0: not measured)
  // the same, and their flops, during the sweeps only (warm-up excluded)
  double sweep_renorm_device_seconds = 0.0, sweep_renorm_flops = 0.0;
  // stored blocks copied back to the engine from host memory (`spill`), the
  // bytes copied each way, and the most block storage the engine held at
  // any point of the run (Engine::block_bytes after every block it made)
  long spill_fetches = 0;
  double spill_bytes_up = 0.0, spill_bytes_down = 0.0, peak_block_bytes = 0.0;
};

struct DriverOptions {
  int verbose = 0;
  // > 0: defer the FP64 energy refinement of split-precision solves and
  // refine only steps whose unrefined lowest energy is within this many Eh
  // of the sweep's lowest so far, and every sweep's last step
  double refine_window = 0.0;
  // with refine_window: keep up to this many steps (their enlarged blocks and
  // vectors) whose refinement may still be needed and refine, at the end of
  // the sweep, only those within the window of the sweep's lowest unrefined
  // energy; 0 refines each qualifying step at once
  int deferred_steps = 0;
  // transform the previous step's wavefunction into the next step's guess
  // (TRANSFORM guess); off: unit-vector guesses (BASIC guess) at every step
  bool transform_guess = false;
  // stored blocks that the current step does not read are kept in host
  // memory only (as the `spill` keyword)
  bool spill = false;
  // optional hooks for tests: called after each superblock solve
  std::function<void(const Superblock&, int sweep, int step)> on_step;
};

class SweepDriver {
 public:
  SweepDriver(const Integrals& I, const Config& c, Engine& e, DriverOptions opt = {});
  ~SweepDriver();
  SweepResult run();
  // pieces used by tests and the bench
  void warmup();
  // left blocks [0..q] for q = 1..upto from seeded random rotations
  void warmup_left(int upto);
  double sweep(bool forward, int sweep_index);
  // one sweep that also evaluates the one-particle (transition) density
  // matrices <psi_a|E_ij|psi_b> of the roots a, b at index a * nroots + b,
  // norb x norb in the sweep's orbital order
  std::vector<std::vector<double>> onepdm_sweep(bool forward, int sweep_index);
  // Superblock of partition p (L=[0..p], R=[p+1..N-1]) built from warm-up
  // blocks on both sides: the sector structure and operator catalogue of a
  // mid-sweep step with bond dimension M, without any Davidson solve.
  // L and R receive the enlarged blocks (owned by the caller).
  Superblock prepare_partition(int p, Block& L, Block& R);
  const Integrals& integrals() const { return I_; }
  // builds the superblock of a forward step at partition p (L = [0..p])
  // using current blocks; useful for snapshots.
  Superblock make_superblock(const Block& L, const Block& R) const;
  Block& left_block(int last_site);   // renormalised [0..last_site]
  Block& right_block(int first_site); // renormalised [first_site..N-1]
  Block make_enlarged(const Block& sys, int dot_site, bool dot_on_right, const CatalogSpec& spec);
  bool loop_is_left(int p) const;  // partition L=[0..p], R=[p+1..N-1]
  CatalogSpec sigma_spec(const std::vector<int>& own, const std::vector<int>& other, bool is_loop,
                         const std::vector<int>& loop_sites) const;
  CatalogSpec renorm_spec(const std::vector<int>& own, int next_dot, bool next_big_is_loop) const;
  void merge(CatalogSpec& a, const CatalogSpec& b) const;
  void log(int level, const char* fmt, ...) const;

 private:
  std::vector<int> warmup_rotation(Block& big, int M, uint64_t seed);
  // checkpoint after `sweeps_done` sweeps; restore returns the sweeps done
  void save_checkpoint(const std::string& path, int sweeps_done, bool next_forward, double sweep_energy,
                       const std::vector<double>& sweep_energies);
  int load_checkpoint(const std::string& path, bool& next_forward, double& sweep_energy,
                      std::vector<double>& sweep_energies);
  std::unique_ptr<Block> renormalised(const Block& big, const std::vector<int>& kept, const CatalogSpec& spec);
  double step(bool forward, int p, int sweep_index, std::vector<double>& energies);
  Block make_dot_block(int x);

  Integrals I_;
  Config C_;
  Engine& E_;
  DriverOptions opt_;
  PointGroup g_;
  QuantumFilter filter_;
  Quantum target_;
  int N_;
  std::vector<std::unique_ptr<Block>> left_;   // left_[p] = [0..p]
  std::vector<std::unique_ptr<Block>> right_;  // right_[p] = [p..N-1]
  std::vector<std::unique_ptr<Block>> dots_;
  // spill: host copies of the stored blocks, made once per block (blocks do
  // not change after they are made); a block whose handle is -1 lives only
  // here until resident() gives it engine storage again
  struct HostCopy {
    std::vector<double> arena;
    RotationRecord rot;
    bool has_rot = false;
  };
  std::map<const Block*, HostCopy> host_;
  bool spill_ = false;
  long spill_fetches_ = 0;
  double spill_up_ = 0.0, spill_down_ = 0.0, peak_bytes_ = 0.0;
  void resident(Block* b);       // engine storage for a stored block (from its host copy)
  // every stored block but keep1 / keep2 to host memory (copied once)
  void spill_idle(const Block* keep1 = nullptr, const Block* keep2 = nullptr);
  void drop(std::unique_ptr<Block>& slot);  // releases a stored block and its host copy
  void note_peak();
  int cur_M_ = 0;
  std::vector<double> last_energies_;
  double last_discarded_ = 0.0;
  SweepResult phase_;  // accumulates the per-phase wall times
  // previous block step (guess transform)
  struct PrevStep {
    bool valid = false, forward = true;
    int p = -1;
    StateInfo L, R;
    std::vector<Superblock::Sector> sectors;
  } prev_;
  double sweep_best_unrefined_ = 0.0;
  // steps whose FP64 refinement is deferred (their blocks stay alive)
  struct Candidate {
    std::unique_ptr<Block> L, R;
    Superblock sb;
    int parked = -1;
    int p = 0;
    double e_unrefined = 0.0;
  };
  std::vector<std::unique_ptr<Candidate>> cands_;
  double sweep_refined_min_ = 0.0;
  // density-matrix sweep: the operators each step needs and the elements
  bool rdm_pass_ = false;
  std::vector<std::vector<double>> rdm_;
  // the previous step's cross elements (i, j) -> <r|E_ij|0> per root r, after
  // its phase fix: consecutive steps share the elements (min p, j >= min p + 2)
  std::map<std::pair<int, int>, std::vector<double>> rdm_link_;
  void rdm_extras(int p, CatalogSpec& specL, CatalogSpec& specR) const;
  void rdm_step(int p, const Superblock& sb);
  std::vector<double> sweep_refined_best_;
  void note_refined(const std::vector<double>& e);
  void refine_candidate(Candidate& c);
  void drop_candidate(std::unique_ptr<Candidate>& c);
  void settle_candidates(bool end_of_sweep);
};

}  // namespace bgpu
