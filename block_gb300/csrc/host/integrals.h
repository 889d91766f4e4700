// Molecular Hamiltonian input: the Molpro FCIDUMP reader/writer, the
// dmrg.conf keyword subset of the sweep hot path, the seeded synthetic
// Hamiltonian generator, and orbital reordering.
//
// FCIDUMP layout follows Input::readorbitalsfile (input.C:1407-1681): header
// `&FCI NORB=,NELEC=,MS2=,ORBSYM=,ISYM= &END`, then `value i j k l` lines,
// 1-based; `k=l=0` marks one-electron integrals and `i=j=k=l=0` the core
// energy.  Two-electron integrals are chemist-notation (ij|kl) with 8-fold
// permutational symmetry.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace bgpu {

struct Integrals {
  int norb = 0, nelec = 0, ms2 = 0, isym = 0;  // isym 0-based
  std::vector<int> orbsym;                     // 0-based irreps
  double ecore = 0.0;
  std::vector<double> t;  // norb^2
  std::vector<double> v;  // norb^4, (ij|kl) = v[((i*n+j)*n+k)*n+l]
  // after reorder(): orbital a is orbital order[a] of the input (empty: input order)
  std::vector<int> order;
  double h(int i, int j) const { return t[(size_t)i * norb + j]; }
  double g(int i, int j, int k, int l) const {
    return v[(((size_t)i * norb + j) * norb + k) * norb + l];
  }
  void resize(int n);
  void set_eri(int i, int j, int k, int l, double x);  // sets all 8 permutations
};

Integrals read_fcidump(const std::string& path);
void write_fcidump(const Integrals& I, const std::string& path);
// new orbital i is old orbital perm[i]
Integrals reorder(const Integrals& I, const std::vector<int>& perm);
// Fiedler ordering of the exchange-integral graph (fiedler.C:47-81,
// genetic/ReadIntegral.C:11-62)
std::vector<int> fiedler_order(const Integrals& I);
// Orbital order requested by a configuration (fiedler | noreorder | file:<path>,
// the reorder file holding 1-based orbitals in their new order).
std::vector<int> orbital_order(const Integrals& I, const std::string& reorder);

// Seeded generator of the synthetic Cholesky-factorised Hamiltonian:
// h symmetric, diag linspace(dlo, dhi), off-diagonal N(0, hsd);
// (pq|rs) = sum_k L^k_pq L^k_rs with symmetric L^k_pq ~ N(0, lsd).
// With `d2h_round_robin`, orbital p carries D2h irrep p mod 8 and every
// integral whose irrep product is not totally symmetric is zeroed.
Integrals synthetic_hamiltonian(int norb, int nelec, int nchol, uint64_t seed, bool d2h_round_robin,
                                double dlo = -3.0, double dhi = 1.0, double hsd = 0.05, double lsd = 0.1);

// Small deterministic PRNG (splitmix64 + Box-Muller), identical on every host.
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next();
  double uniform();  // (0,1)
  double normal();
};

struct ScheduleEntry {
  int iter = 0, M = 0;
  double davidson_tol = 1e-8, noise = 0.0;
};

struct Config {
  int nelec = -1, spin = 0, irrep = 0;  // irrep 0-based
  std::string sym = "c1";
  std::string orbitals;  // FCIDUMP path
  std::vector<ScheduleEntry> schedule;
  bool schedule_default = false;
  int startM = 250, maxM = 0;
  int maxiter = 10;
  double sweep_tol = 1e-5;
  int nroots = 1;
  std::vector<double> weights;
  std::string reorder = "fiedler";  // fiedler | noreorder | file:<path>
  int outputlevel = 0;
  int deflation_min = 2, deflation_max = 20;
  // `davidson_max_iter <n>` (a keyword of this library; the reference's
  // Davidson iterates until it converges): iteration limit of every solve
  int davidson_max_iter = 200;
  uint64_t seed = 12345;  // warm-up rotations and Davidson guesses
  std::string warmup = "random";
  // sweep checkpoints (this project's restart format, host/checkpoint.h):
  // `checkpoint <path>` writes one after every completed sweep; `restart`
  // (or `fullrestart`) resumes from it instead of the warm-up, and
  // `reset_iter` then starts the schedule from its first entry again
  std::string checkpoint;
  bool restart = false, reset_iter = false;
  // `spill`: stored blocks that the current block step does not read stay in
  // host memory, copied back to the device when a step needs them (the
  // reference keeps blocks on disk between steps, save_load_block.C:58-110)
  bool spill = false;
  // `onepdm` (or onerdm, ordm): after the sweeps, one more sweep evaluates
  // the spin-summed spatial one-particle density matrix of every root;
  // `prefix <dir>`: where spatial_onepdm.<r>.<r>.txt files are written
  bool onepdm = false;
  // `tran_onepdm`: the same sweep, and also writes the transition matrices
  // <i|E_kl|j> (i > j) as spatial_onepdm.<i>.<j>.txt
  bool tran_onepdm = false;
  std::string prefix;
  // `twodot_noise <amplitude> <gamma>`: random-wavefunction noise of that
  // amplitude in the density matrices of the first sweep (gamma is read and
  // not used); with `schedule default` it replaces the scheduled noise
  double twodot_noise = 0.0;
  // the remaining keywords are recognised and ignored (twodot_to_onedot,
  // hf_occ, onepdm/twopdm, noise columns ...)
  const ScheduleEntry& entry(int sweep) const;
};

Config parse_config(const std::string& path);
// Integrals named by `orbitals`: an FCIDUMP path, or a generated Hamiltonian
// `synthetic:<norb>:<nelec>:<nchol>:<seed>:<d2h 0|1>`; reordered as the
// configuration asks.
Integrals load_integrals(Config& c);
Config parse_config_text(const std::string& text, const std::string& base_dir);
// The reference's default schedule (Schedule.C generateDefaultSchedule) for
// `schedule default` with startM/maxM.
void make_default_schedule(Config& c);

}  // namespace bgpu
