// TEST INFRASTRUCTURE ONLY: C entry points of the CPU oracle for the Python
// tests and the bench's CPU baseline.  Runs the oracle sweep, or stops it at
// a chosen step and exposes that step's superblock (blocks, operator-pair
// list, wavefunction and the oracle's sigma) so the CUDA library can be fed
// the same inputs through its C ABI.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <dlfcn.h>
#include <map>
#include <memory>
#include <random>
#include <string>

#include "cpu_engine.h"

using namespace bgpu;

namespace {
struct Captured {};

struct SnapBlock {
  std::vector<int> quanta, states, keys;
  std::vector<double> arena;
  std::vector<OpKey> order;
  int is_dot = 0;
};

struct Snapshot {
  SnapBlock L, R;
  std::vector<double> coef;
  std::vector<int> ops;
  std::vector<double> psi, sigma, diag;
  int target[3] = {0, 0, 0};
  double ecore = 0.0;
  double energy = 0.0;
  std::vector<int> orbsym;
  std::string group;
  double sigma_seconds = 0.0, sigma_seconds_1t = 0.0;
  double sigma_flops = 0.0;
  int threads = 1;
};

SnapBlock snap_block(const Block& b, oracle::CpuEngine& e) {
  SnapBlock s;
  for (int q = 0; q < b.si.size(); ++q) {
    s.quanta.push_back(b.si.quanta[q].n);
    s.quanta.push_back(b.si.quanta[q].s2);
    s.quanta.push_back(b.si.quanta[q].irrep);
    s.states.push_back(b.si.states[q]);
  }
  for (const auto& kv : b.ops.ops) {
    s.order.push_back(kv.first);
    s.keys.push_back((int)kv.first.type);
    s.keys.push_back(kv.first.i);
    s.keys.push_back(kv.first.j);
    s.keys.push_back(kv.first.k2);
  }
  s.arena = e.arena(b);
  s.is_dot = b.is_dot ? 1 : 0;
  return s;
}

int index_of(const SnapBlock& s, const Operand& o) {
  if (o.identity) return -1;
  for (size_t i = 0; i < s.order.size(); ++i)
    if (s.order[i] == o.key) return (int)i;
  return -2;
}
}  // namespace

extern "C" {

// Routes the oracle's DGEMM through the Fortran DGEMM of the shared library
// at `path` (a tuned BLAS, e.g. the OpenBLAS bundled with SciPy), single-
// threaded (the oracle threads over operator pairs itself).  The library is
// kept only if its products match the built-in loop to 1e-12 on transposed
// and plain operands.  Returns 0 when the BLAS is in use, < 0 otherwise;
// path NULL switches back to the built-in loop.
int oracle_use_blas(const char* path) {
  using oracle::FortranDgemm;
  oracle::g_blas_dgemm = nullptr;
  if (!path) return 0;
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return -1;
  FortranDgemm f = nullptr;
  for (const char* name : {"scipy_dgemm_", "dgemm_"})
    if (!f) f = (FortranDgemm)dlsym(h, name);
  if (!f) return -2;
  typedef void (*SetThreads)(int);
  for (const char* name : {"scipy_openblas_set_num_threads", "openblas_set_num_threads"}) {
    SetThreads st = (SetThreads)dlsym(h, name);
    if (st) {
      st(1);
      break;
    }
  }
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  for (int ta = 0; ta < 2; ++ta)
    for (int tb = 0; tb < 2; ++tb) {
      const int m = 37, n = 29, k = 41, lda = (ta ? m : k) + 3, ldb = (tb ? k : n) + 2, ldc = n + 5;
      std::vector<double> A((size_t)(ta ? k : m) * lda), B((size_t)(tb ? n : k) * ldb), C((size_t)m * ldc), D;
      for (auto& x : A) x = u(rng);
      for (auto& x : B) x = u(rng);
      for (auto& x : C) x = u(rng);
      D = C;
      oracle::g_blas_dgemm = f;
      oracle::dgemm(ta, tb, m, n, k, 0.75, A.data(), lda, B.data(), ldb, 0.5, C.data(), ldc);
      oracle::g_blas_dgemm = nullptr;
      oracle::dgemm_loop(ta, tb, m, n, k, 0.75, A.data(), lda, B.data(), ldb, 0.5, D.data(), ldc);
      for (int i = 0; i < m; ++i)
        for (int j = 0; j < n; ++j)
          if (std::fabs(C[(size_t)i * ldc + j] - D[(size_t)i * ldc + j]) >
              1e-12 * (1.0 + std::fabs(D[(size_t)i * ldc + j])))
            return -3;
    }
  oracle::g_blas_dgemm = f;
  return 0;
}

static std::vector<double> g_last_sweep_energies;  // per sweep, lowest root, of the last oracle_run
static bool g_guess = false;  // oracle_run's Davidson starts from transformed guesses

// Davidson start of the next oracle_run steps: transformed previous
// wavefunctions (on = 1, the TRANSFORM guess) or unit vectors (0, default).
int oracle_set_guess(int on) {
  g_guess = on != 0;
  return 0;
}
static std::vector<std::vector<double>> g_last_onepdm;  // per root, of the last oracle_run with onepdm
static std::vector<std::vector<double>> g_last_tonepdm;  // per root pair (bra * nroots + ket)

// the one-particle density matrix of a root of the last oracle_run (0 on success)
int oracle_onepdm(int root, double* out, int norb) {
  if (root < 0 || root >= (int)g_last_onepdm.size()) return 1;
  if ((size_t)norb * norb != g_last_onepdm[root].size()) return 2;
  std::copy(g_last_onepdm[root].begin(), g_last_onepdm[root].end(), out);
  return 0;
}

// <bra|E_ij|ket> between two roots of the last oracle_run (0 on success)
int oracle_transition_onepdm(int bra, int ket, double* out, int norb) {
  const int nr = (int)g_last_onepdm.size();
  if (bra < 0 || bra >= nr || ket < 0 || ket >= nr) return 1;
  const auto& m = g_last_tonepdm[(size_t)bra * nr + ket];
  if ((size_t)norb * norb != m.size()) return 2;
  std::copy(m.begin(), m.end(), out);
  return 0;
}

// Spin-coupling coefficients of the shared host code (2j arguments), for the
// tests: kind 0 clebsch(j1 m1 j2 m2 j3 m3), 1 six_j(6), 2 nine_j(9),
// 3 ninej (the normalised 9j of the coupling tables, 9), 4
// transpose_scaling(l r k).  Returns 0 on success, 1 for an unknown kind, 2
// when the function refused its arguments.
int oracle_su2(int kind, const int* a, double* out) {
  try {
    switch (kind) {
      case 0: *out = clebsch(a[0], a[1], a[2], a[3], a[4], a[5]); return 0;
      case 1: *out = six_j(a[0], a[1], a[2], a[3], a[4], a[5]); return 0;
      case 2: *out = nine_j(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8]); return 0;
      case 3: *out = ninej(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8]); return 0;
      case 4: *out = transpose_scaling(a[0], a[1], a[2]); return 0;
      default: return 1;
    }
  } catch (const std::exception&) {
    return 2;
  }
}

// the per-sweep energies of the last oracle_run (returns how many; copies up to cap)
int oracle_sweep_energies(double* out, int cap) {
  for (int i = 0; i < cap && i < (int)g_last_sweep_energies.size(); ++i) out[i] = g_last_sweep_energies[i];
  return (int)g_last_sweep_energies.size();
}

// A whole run of dmrg.conf on the CPU engine.  stats (12 entries, may be
// null): sweeps, sigma products, their seconds, 0, wall seconds, discarded
// weight, last sweep energy, roots, blocks copied back from host memory
// (`spill`), bytes copied each way for them, peak bytes of block storage.
int oracle_run(const char* conf, int threads, int verbose, double* energies, int max_roots, double* stats) {
  g_last_onepdm.clear();
  g_last_tonepdm.clear();
  g_last_sweep_energies.clear();
  try {
    auto t0 = std::chrono::steady_clock::now();
    Config c = parse_config(conf);
    Integrals I = load_integrals(c);
    oracle::CpuEngine eng(threads);
    DriverOptions opt;
    opt.verbose = verbose;
    opt.transform_guess = g_guess;
    SweepResult r;
    {
      SweepDriver drv(I, c, eng, opt);
      r = drv.run();
    }
    g_last_sweep_energies = r.sweep_energies;
    g_last_onepdm = r.onepdm;
    g_last_tonepdm = r.transition_onepdm;
    for (int i = 0; i < max_roots && i < (int)r.energies.size(); ++i) energies[i] = r.energies[i];
    if (stats) {
      stats[0] = r.sweeps;
      stats[1] = (double)eng.sigma_calls;
      stats[2] = eng.sigma_seconds;
      stats[3] = 0.0;
      stats[4] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      stats[5] = r.discarded;
      stats[6] = r.sweep_energies.empty() ? 0.0 : r.sweep_energies.back();
      stats[7] = (double)r.energies.size();
      stats[8] = (double)r.spill_fetches;
      stats[9] = r.spill_bytes_up;
      stats[10] = r.spill_bytes_down;
      stats[11] = r.peak_block_bytes;
    }
    return 0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_run: %s\n", e.what());
    return 1;
  }
}

// Run `conf` and capture the superblock of step (sweep, pos); nullptr on error.
void* oracle_snapshot(const char* conf, int sweep, int pos, int threads) {
  auto snap = std::make_unique<Snapshot>();
  try {
    Config c = parse_config(conf);
    Integrals I = load_integrals(c);
    oracle::CpuEngine eng(threads);
    DriverOptions opt;
    snap->orbsym = I.orbsym;
    snap->group = c.sym;
    snap->threads = eng.threads;
    opt.on_step = [&](const Superblock& sb, int s, int p) {
      if (s != sweep || p != pos) return;
      snap->L = snap_block(*sb.L, eng);
      snap->R = snap_block(*sb.R, eng);
      for (const auto& t : sb.terms) {
        snap->coef.push_back(t.coef);
        snap->ops.push_back(index_of(snap->L, t.l));
        snap->ops.push_back(t.l.trans ? 1 : 0);
        snap->ops.push_back(index_of(snap->R, t.r));
        snap->ops.push_back(t.r.trans ? 1 : 0);
      }
      snap->psi = eng.wavefunctions().at(0);
      snap->sigma.assign(sb.size, 0.0);
      auto t0 = std::chrono::steady_clock::now();
      eng.sigma(sb, snap->psi.data(), snap->sigma.data());
      snap->sigma_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      snap->sigma_flops = eng.last_sigma_flops;
      snap->diag.assign(sb.size, 0.0);
      eng.hdiag(sb, snap->diag.data());
      snap->target[0] = sb.target.n;
      snap->target[1] = sb.target.s2;
      snap->target[2] = sb.target.irrep;
      snap->ecore = sb.ecore;
      double e = 0;
      for (size_t i = 0; i < snap->psi.size(); ++i) e += snap->psi[i] * snap->sigma[i];
      snap->energy = e;
      throw Captured{};
    };
    try {
      SweepDriver drv(I, c, eng, opt);
      drv.run();
    } catch (const Captured&) {
      return snap.release();
    }
    std::fprintf(stderr, "oracle_snapshot: step (%d,%d) not reached\n", sweep, pos);
    return nullptr;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_snapshot: %s\n", e.what());
    return nullptr;
  }
}

void oracle_snapshot_free(void* h) { delete static_cast<Snapshot*>(h); }

// sizes: [0]=nquanta L, [1]=nops L, [2]=arena L, [3]=nquanta R, [4]=nops R,
// [5]=arena R, [6]=nterms, [7]=psi size, [8]=norb, [9]=L is dot, [10]=R is dot
void oracle_snapshot_sizes(void* h, int64_t* out) {
  auto* s = static_cast<Snapshot*>(h);
  out[0] = (int64_t)s->L.states.size();
  out[1] = (int64_t)s->L.order.size();
  out[2] = (int64_t)s->L.arena.size();
  out[3] = (int64_t)s->R.states.size();
  out[4] = (int64_t)s->R.order.size();
  out[5] = (int64_t)s->R.arena.size();
  out[6] = (int64_t)s->coef.size();
  out[7] = (int64_t)s->psi.size();
  out[8] = (int64_t)s->orbsym.size();
  out[9] = s->L.is_dot;
  out[10] = s->R.is_dot;
}

void oracle_snapshot_block(void* h, int which, int* quanta, int* states, int* keys, double* arena) {
  auto* s = static_cast<Snapshot*>(h);
  const SnapBlock& b = which == 0 ? s->L : s->R;
  std::memcpy(quanta, b.quanta.data(), b.quanta.size() * sizeof(int));
  std::memcpy(states, b.states.data(), b.states.size() * sizeof(int));
  std::memcpy(keys, b.keys.data(), b.keys.size() * sizeof(int));
  std::memcpy(arena, b.arena.data(), b.arena.size() * sizeof(double));
}

// misc[0..2] target, misc[3] ecore, misc[4] energy <psi|H|psi>, misc[5] oracle sigma seconds,
// misc[6] threads, misc[7] oracle sigma GEMM flops, misc[8] one-thread sigma seconds (0 if not timed)
void oracle_snapshot_data(void* h, double* coef, int* ops, double* psi, double* sigma, double* diag, int* orbsym,
                          double* misc) {
  auto* s = static_cast<Snapshot*>(h);
  std::memcpy(coef, s->coef.data(), s->coef.size() * sizeof(double));
  std::memcpy(ops, s->ops.data(), s->ops.size() * sizeof(int));
  std::memcpy(psi, s->psi.data(), s->psi.size() * sizeof(double));
  std::memcpy(sigma, s->sigma.data(), s->sigma.size() * sizeof(double));
  std::memcpy(diag, s->diag.data(), s->diag.size() * sizeof(double));
  std::memcpy(orbsym, s->orbsym.data(), s->orbsym.size() * sizeof(int));
  misc[0] = s->target[0];
  misc[1] = s->target[1];
  misc[2] = s->target[2];
  misc[3] = s->ecore;
  misc[4] = s->energy;
  misc[5] = s->sigma_seconds;
  misc[6] = s->threads;
  misc[7] = s->sigma_flops;
  misc[8] = s->sigma_seconds_1t;
}

const char* oracle_snapshot_group(void* h) { return static_cast<Snapshot*>(h)->group.c_str(); }

// Time `reps` oracle sigma products on the captured superblock with `threads`
// threads (CPU baseline of the bench); returns seconds per product.
double oracle_time_sigma(const char* conf, int sweep, int pos, int threads, int reps) {
  double per = -1.0;
  try {
    Config c = parse_config(conf);
    Integrals I = load_integrals(c);
    oracle::CpuEngine eng(threads);
    DriverOptions opt;
    opt.on_step = [&](const Superblock& sb, int s, int p) {
      if (s != sweep || p != pos) return;
      std::vector<double> psi = eng.wavefunctions().at(0), out(sb.size);
      auto t0 = std::chrono::steady_clock::now();
      for (int r = 0; r < reps; ++r) eng.sigma(sb, psi.data(), out.data());
      per = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() / reps;
      throw Captured{};
    };
    try {
      SweepDriver drv(I, c, eng, opt);
      drv.run();
    } catch (const Captured&) {
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_time_sigma: %s\n", e.what());
  }
  return per;
}

}  // extern "C"

extern "C" {
// Superblock of `partition` built from seeded warm-up blocks (same
// construction as bgpu_prepare_superblock) captured as a snapshot whose psi
// is a seeded random unit vector.
void* oracle_prepare(const char* conf, int partition, int threads, int reps, int time_single) {
  auto snap = std::make_unique<Snapshot>();
  try {
    Config c = parse_config(conf);
    Integrals I = load_integrals(c);
    oracle::CpuEngine eng(threads);
    snap->orbsym = I.orbsym;
    snap->group = c.sym;
    snap->threads = eng.threads;
    SweepDriver drv(I, c, eng);
    Block L, R;
    Superblock sb = drv.prepare_partition(partition, L, R);
    sb.L = &L;
    sb.R = &R;
    snap->L = snap_block(L, eng);
    snap->R = snap_block(R, eng);
    for (const auto& t : sb.terms) {
      snap->coef.push_back(t.coef);
      snap->ops.push_back(index_of(snap->L, t.l));
      snap->ops.push_back(t.l.trans ? 1 : 0);
      snap->ops.push_back(index_of(snap->R, t.r));
      snap->ops.push_back(t.r.trans ? 1 : 0);
    }
    Rng rng(c.seed + 99991);
    snap->psi.resize(sb.size);
    double nrm = 0;
    for (auto& x : snap->psi) {
      x = rng.normal();
      nrm += x * x;
    }
    for (auto& x : snap->psi) x /= std::sqrt(nrm);
    snap->sigma.assign(sb.size, 0.0);
    if (reps < 1) reps = 1;
    auto t0 = std::chrono::steady_clock::now();
    for (int r = 0; r < reps; ++r) eng.sigma(sb, snap->psi.data(), snap->sigma.data());
    snap->sigma_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() / reps;
    snap->sigma_flops = eng.last_sigma_flops;
    if (time_single) {
      // the same product on one thread
      const int nt = eng.threads;
      eng.threads = 1;
      std::vector<double> tmp(sb.size, 0.0);
      t0 = std::chrono::steady_clock::now();
      eng.sigma(sb, snap->psi.data(), tmp.data());
      snap->sigma_seconds_1t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      eng.threads = nt;
    }
    snap->diag.assign(sb.size, 0.0);
    eng.hdiag(sb, snap->diag.data());
    snap->target[0] = sb.target.n;
    snap->target[1] = sb.target.s2;
    snap->target[2] = sb.target.irrep;
    snap->ecore = sb.ecore;
    double e = 0;
    for (size_t i = 0; i < snap->psi.size(); ++i) e += snap->psi[i] * snap->sigma[i];
    snap->energy = e;
    eng.release_block(L);
    eng.release_block(R);
    return snap.release();
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_prepare: %s\n", e.what());
    return nullptr;
  }
}
}  // extern "C"

// ---------------------------------------------------------------------------
// Block-level case for the element-wise parity tests of the enlarged-block
// build, the density matrix and the renormalisation: at `partition` of a
// configuration's warm-up chain, the system block [0..p-1], the dot p, the
// enlarged block [0..p] built by the oracle (sigma and renormalisation
// catalogues merged, as a forward sweep step builds it), a seeded random
// wavefunction on the superblock [0..p] | [p+1..N-1], its left density
// matrix with eigenvectors, the rotation keeping the M largest weights
// (the truncation rule of the sweep) and the renormalised block U^T O U.
// ---------------------------------------------------------------------------
namespace {
struct BlockCase {
  std::map<std::string, std::vector<int>> ints;
  std::map<std::string, std::vector<double>> reals;
  std::string group;
};

void put_block(BlockCase& c, const std::string& name, const Block& b, oracle::CpuEngine& e, bool with_arena) {
  SnapBlock s = snap_block(b, e);
  c.ints[name + "_quanta"] = s.quanta;
  c.ints[name + "_states"] = s.states;
  c.ints[name + "_keys"] = s.keys;
  c.ints[name + "_sites"] = b.sites;
  if (with_arena) c.reals[name + "_arena"] = s.arena;
}
}  // namespace

extern "C" {
void* oracle_block_case(const char* conf, int partition, int threads, double noise, double random_noise,
                        unsigned long long seed) {
  auto bc = std::make_unique<BlockCase>();
  try {
    Config c = parse_config(conf);
    Integrals I = load_integrals(c);
    oracle::CpuEngine eng(threads);
    bc->group = c.sym;
    SweepDriver drv(I, c, eng);
    const int N = I.norb, p = partition;
    Block L0, R0;
    Superblock sb0 = drv.prepare_partition(p, L0, R0);  // warm-up chain and the environment block
    (void)sb0;
    std::vector<int> Ls, Rs;
    for (int i = 0; i <= p; ++i) Ls.push_back(i);
    for (int i = p + 1; i < N; ++i) Rs.push_back(i);
    const bool loopL = drv.loop_is_left(p);
    CatalogSpec specL = drv.sigma_spec(Ls, Rs, loopL, loopL ? Ls : Rs);
    CatalogSpec keep = drv.renorm_spec(Ls, p + 1, drv.loop_is_left(p + 1));
    drv.merge(specL, keep);
    Block& sys = drv.left_block(p - 1);
    Block big = drv.make_enlarged(sys, p, /*dot_on_right=*/true, specL);
    PointGroup g = PointGroup::from_name(c.sym);
    DotOps dot = make_dot(p, I, g);
    Block dotb;
    dotb.sites = {p};
    dotb.si = dot.si;
    dotb.ops = dot.set;
    dotb.is_dot = true;
    eng.create_block(dotb);
    eng.upload_block(dotb, dot.data);
    put_block(*bc, "sys", sys, eng, true);
    put_block(*bc, "dot", dotb, eng, true);
    put_block(*bc, "big", big, eng, true);
    put_block(*bc, "env", R0, eng, false);
    bc->ints["orbsym"] = I.orbsym;
    int nel = c.nelec >= 0 ? c.nelec : I.nelec;
    bc->ints["filter"] = {nel, c.spin, N};
    Superblock sb = drv.make_superblock(big, R0);
    bc->ints["target"] = {sb.target.n, sb.target.s2, sb.target.irrep};
    Rng rng(c.seed + 424242);
    std::vector<double> psi(sb.size);
    double nrm = 0.0;
    for (auto& x : psi) {
      x = rng.normal();
      nrm += x * x;
    }
    for (auto& x : psi) x /= std::sqrt(nrm);
    bc->reals["psi"] = psi;
    eng.set_wavefunctions({psi});
    NoiseSpec ns;
    ns.perturbative = noise;
    ns.random = random_noise;
    ns.seed = seed;
    ns.orbsym = I.orbsym;
    ns.group = PointGroup::from_name(c.sym);
    eng.set_noise(ns);
    DensitySpectrum spec;
    eng.density(sb, /*left=*/true, {1.0}, spec);
    eng.set_noise(NoiseSpec{});
    std::vector<double> rho, vecs, eig;
    for (const auto& m : eng.density_matrices()) rho.insert(rho.end(), m.begin(), m.end());
    for (const auto& m : eng.density_vectors()) vecs.insert(vecs.end(), m.begin(), m.end());
    for (const auto& v : spec.eig) eig.insert(eig.end(), v.begin(), v.end());
    bc->reals["rho"] = rho;
    bc->reals["vecs"] = vecs;
    bc->reals["eig"] = eig;
    // the M largest weights above 1e-13, eigenvectors of a sector in descending order
    struct W { double w; int q, i; };
    std::vector<W> all;
    for (int q = 0; q < (int)spec.eig.size(); ++q)
      for (int i = 0; i < (int)spec.eig[q].size(); ++i) all.push_back({spec.eig[q][i], q, i});
    std::stable_sort(all.begin(), all.end(), [](const W& a, const W& b) { return a.w > b.w; });
    const int M = c.schedule.empty() ? 100 : c.schedule.front().M;
    std::vector<std::vector<int>> kept_idx(spec.eig.size());
    for (int t = 0; t < std::min<int>(M, (int)all.size()); ++t)
      if (all[t].w > 1e-13) kept_idx[all[t].q].push_back(all[t].i);
    std::vector<int> kept(spec.eig.size());
    for (size_t q = 0; q < kept_idx.size(); ++q) {
      std::sort(kept_idx[q].begin(), kept_idx[q].end(), std::greater<int>());
      kept[q] = (int)kept_idx[q].size();
    }
    eng.select_rotation(kept_idx);
    std::vector<double> rot;
    for (const auto& m : eng.rotation()) rot.insert(rot.end(), m.begin(), m.end());
    bc->ints["kept"] = kept;
    bc->reals["rot"] = rot;
    std::vector<int> map;
    Block small;
    small.sites = big.sites;
    small.si = truncated_stateinfo(big.si, kept, map);
    small.ops = make_opset(small.si, catalog_keys(keep), I.orbsym, g);
    eng.create_block(small);
    eng.renormalise(small, big);
    put_block(*bc, "small", small, eng, true);
    for (Block* b : {&big, &dotb, &small, &L0, &R0}) eng.release_block(*b);
    return bc.release();
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_block_case: %s\n", e.what());
    return nullptr;
  }
}

void oracle_case_free(void* h) { delete static_cast<BlockCase*>(h); }

// length of a named array (-1 if absent); kind 0 = int, 1 = double
int64_t oracle_case_len(void* h, const char* name, int kind) {
  auto* c = static_cast<BlockCase*>(h);
  if (kind == 0) {
    auto it = c->ints.find(name);
    return it == c->ints.end() ? -1 : (int64_t)it->second.size();
  }
  auto it = c->reals.find(name);
  return it == c->reals.end() ? -1 : (int64_t)it->second.size();
}

void oracle_case_get(void* h, const char* name, int kind, void* out) {
  auto* c = static_cast<BlockCase*>(h);
  if (kind == 0) {
    const auto& v = c->ints.at(name);
    std::memcpy(out, v.data(), v.size() * sizeof(int));
  } else {
    const auto& v = c->reals.at(name);
    std::memcpy(out, v.data(), v.size() * sizeof(double));
  }
}

const char* oracle_case_group(void* h) { return static_cast<BlockCase*>(h)->group.c_str(); }
}  // extern "C"

extern "C" {
// Timing sample of the oracle sigma on the superblock of `partition` with
// the sector structure, operator catalogue and operator-pair list of the
// seeded warm-up chain (the superblock bgpu_prepare_superblock builds), but
// with seeded random operator values: the warm-up's renormalisations are
// skipped, which makes a large bond dimension preparable in seconds, and
// sigma's cost does not depend on the values.  out[0] = FP64 flops of one
// product, out[1] = psi elements, out[2] = operator doubles of L and R,
// out[3] = seconds per product over `reps` products, out[4] = norm of the
// last sigma (a checksum), out[5] = threads.  Returns 0 on success.
int oracle_sample_sigma(const char* conf, int partition, int threads, int reps, double* out) {
  try {
    Config c = parse_config(conf);
    Integrals I = load_integrals(c);
    oracle::CpuEngine eng(threads);
    eng.structure_only = true;
    SweepDriver drv(I, c, eng);
    Block L, R;
    Superblock sb = drv.prepare_partition(partition, L, R);
    sb.L = &L;
    sb.R = &R;
    eng.structure_only = false;
    eng.fill_random(L, c.seed + 1);
    eng.fill_random(R, c.seed + 2);
    Rng rng(c.seed + 99991);
    std::vector<double> psi(sb.size), sig(sb.size, 0.0);
    double nrm = 0.0;
    for (auto& x : psi) {
      x = rng.normal();
      nrm += x * x;
    }
    for (auto& x : psi) x /= std::sqrt(nrm);
    if (reps < 1) reps = 1;
    auto t0 = std::chrono::steady_clock::now();
    for (int r = 0; r < reps; ++r) eng.sigma(sb, psi.data(), sig.data());
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() / reps;
    double sn = 0.0;
    for (double x : sig) sn += x * x;
    out[0] = eng.last_sigma_flops;
    out[1] = (double)sb.size;
    out[2] = (double)(L.ops.arena + R.ops.arena);
    out[3] = secs;
    out[4] = std::sqrt(sn);
    out[5] = eng.threads;
    eng.release_block(L);
    eng.release_block(R);
    return 0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_sample_sigma: %s\n", e.what());
    return 1;
  }
}
}  // extern "C"
