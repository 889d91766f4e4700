#include "sweep.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <limits>
#include <numeric>
#include <stdexcept>

#include "dense.h"

namespace bgpu {

SweepDriver::SweepDriver(const Integrals& I, const Config& c, Engine& e, DriverOptions opt)
    : I_(I), C_(c), E_(e), opt_(std::move(opt)) {
  g_ = PointGroup::from_name(C_.sym);
  N_ = I_.norb;
  spill_ = C_.spill || opt_.spill;
  const int nelec = C_.nelec >= 0 ? C_.nelec : I_.nelec;
  filter_.nelec = nelec;
  filter_.s2 = C_.spin;
  filter_.norb = N_;
  target_ = {nelec, C_.spin, C_.irrep};
  left_.resize(N_);
  right_.resize(N_);
  dots_.resize(N_);
  for (int x = 0; x < N_; ++x) {
    dots_[x] = std::make_unique<Block>(make_dot_block(x));
  }
}

SweepDriver::~SweepDriver() {
  for (auto* v : {&left_, &right_, &dots_})
    for (auto& b : *v)
      if (b && b->handle >= 0) E_.release_block(*b);
}

void SweepDriver::log(int level, const char* fmt, ...) const {
  if (opt_.verbose < level) return;
  va_list ap;
  va_start(ap, fmt);
  std::vfprintf(stderr, fmt, ap);
  va_end(ap);
}

Block SweepDriver::make_dot_block(int x) {
  DotOps d = make_dot(x, I_, g_);
  Block b;
  b.sites = {x};
  b.si = d.si;
  b.ops = d.set;
  b.is_dot = true;
  E_.create_block(b);
  E_.upload_block(b, d.data);
  note_peak();
  return b;
}

void SweepDriver::note_peak() { peak_bytes_ = std::max(peak_bytes_, (double)E_.block_bytes()); }

void SweepDriver::resident(Block* b) {
  if (!b || b->handle >= 0) return;
  auto it = host_.find(b);
  if (it == host_.end()) throw std::runtime_error("stored block has neither engine storage nor a host copy");
  E_.create_block(*b);
  E_.upload_block(*b, it->second.arena);
  if (it->second.has_rot) E_.set_rotation_record(*b, it->second.rot);
  ++spill_fetches_;
  spill_up_ += 8.0 * (double)it->second.arena.size();
  note_peak();
}

void SweepDriver::spill_idle(const Block* keep1, const Block* keep2) {
  if (!spill_) return;
  for (auto* v : {&left_, &right_})
    for (auto& up : *v) {
      Block* b = up.get();
      if (!b || b->handle < 0 || b == keep1 || b == keep2) continue;
      if (host_.find(b) == host_.end()) {
        HostCopy hc;
        E_.download_block(*b, hc.arena);
        hc.has_rot = E_.get_rotation_record(*b, hc.rot);
        spill_down_ += 8.0 * (double)hc.arena.size();
        host_.emplace(b, std::move(hc));
      }
      E_.release_block(*b);
    }
}

void SweepDriver::drop(std::unique_ptr<Block>& slot) {
  if (!slot) return;
  if (slot->handle >= 0) E_.release_block(*slot);
  host_.erase(slot.get());
  slot.reset();
}

bool SweepDriver::loop_is_left(int p) const { return (p + 1) <= (N_ - 1 - p); }

CatalogSpec SweepDriver::sigma_spec(const std::vector<int>& own, const std::vector<int>& other, bool is_loop,
                                    const std::vector<int>& loop_sites) const {
  CatalogSpec s;
  s.sites = own;
  s.ccd_sites = other;
  s.normal = is_loop;
  if (!is_loop)
    for (int a : loop_sites)
      for (int b : loop_sites)
        if (a >= b) s.comp_pairs.push_back({a, b});
  return s;
}

CatalogSpec SweepDriver::renorm_spec(const std::vector<int>& own, int /*next_dot*/, bool next_big_is_loop) const {
  CatalogSpec s;
  s.sites = own;
  std::vector<int> comp;
  for (int i = 0; i < N_; ++i)
    if (std::find(own.begin(), own.end(), i) == own.end()) comp.push_back(i);
  s.ccd_sites = comp;
  s.normal = next_big_is_loop;
  for (int a : comp)
    for (int b : comp)
      if (a >= b) s.comp_pairs.push_back({a, b});
  return s;
}

void SweepDriver::merge(CatalogSpec& a, const CatalogSpec& b) const {
  a.normal = a.normal || b.normal;
  for (int x : b.ccd_sites)
    if (std::find(a.ccd_sites.begin(), a.ccd_sites.end(), x) == a.ccd_sites.end()) a.ccd_sites.push_back(x);
  for (auto& p : b.comp_pairs)
    if (std::find(a.comp_pairs.begin(), a.comp_pairs.end(), p) == a.comp_pairs.end()) a.comp_pairs.push_back(p);
  for (const OpKey& k : b.extra)
    if (std::find(a.extra.begin(), a.extra.end(), k) == a.extra.end()) a.extra.push_back(k);
}

Block SweepDriver::make_enlarged(const Block& sys, int x, bool dot_on_right, const CatalogSpec& spec) {
  const Block& dot = *dots_[x];
  const Block& a = dot_on_right ? sys : dot;
  const Block& b = dot_on_right ? dot : sys;
  Block big;
  big.sites = a.sites;
  big.sites.insert(big.sites.end(), b.sites.begin(), b.sites.end());
  big.si = product_stateinfo(a.si, b.si, g_, &filter_, (int)big.sites.size(), nullptr);
  std::set<OpKey> keys = catalog_keys(spec);
  big.ops = make_opset(big.si, keys, I_.orbsym, g_);
  std::vector<std::pair<OpKey, std::vector<BuildTerm>>> recipes;
  for (const auto& kv : big.ops.ops) recipes.push_back({kv.first, build_terms(kv.first, a.sites, b.sites, I_)});
  // check that every operand exists
  for (auto& r : recipes)
    for (auto& t : r.second) {
      if (!t.a.identity && !a.ops.has(t.a.key))
        throw std::runtime_error("build of " + r.first.str() + " needs " + t.a.key.str() + " on left sub-block");
      if (!t.b.identity && !b.ops.has(t.b.key))
        throw std::runtime_error("build of " + r.first.str() + " needs " + t.b.key.str() + " on right sub-block");
    }
  E_.create_block(big);
  note_peak();
  E_.build_block(big, a, b, recipes);
  return big;
}

Superblock SweepDriver::make_superblock(const Block& L, const Block& R) const {
  Superblock sb;
  sb.L = &L;
  sb.R = &R;
  sb.target = target_;
  sb.si = product_stateinfo(L.si, R.si, g_, nullptr, N_, &target_);
  const int p = L.sites.back();
  sb.loop_left = loop_is_left(p);
  sb.terms = sigma_terms(L.sites, R.sites, sb.loop_left);
  sb.ecore = I_.ecore;
  for (int lq = 0; lq < L.si.size(); ++lq)
    for (int rq = 0; rq < R.si.size(); ++rq) {
      if (!quantum_allowed(target_, L.si.quanta[lq], R.si.quanta[rq], g_)) continue;
      Superblock::Sector s;
      s.lq = lq;
      s.rq = rq;
      s.rows = L.si.states[lq];
      s.cols = R.si.states[rq];
      s.offset = sb.size;
      sb.size += (int64_t)s.rows * s.cols;
      sb.sectors.push_back(s);
    }
  for (auto& t : sb.terms) {
    if (!t.l.identity && !L.ops.has(t.l.key)) throw std::runtime_error("sigma needs " + t.l.key.str() + " on L");
    if (!t.r.identity && !R.ops.has(t.r.key)) throw std::runtime_error("sigma needs " + t.r.key.str() + " on R");
  }
  return sb;
}

Block& SweepDriver::left_block(int last) {
  if (last == 0) return *dots_[0];
  if (!left_[last]) throw std::runtime_error("left block missing");
  resident(left_[last].get());
  return *left_[last];
}

Block& SweepDriver::right_block(int first) {
  if (first == N_ - 1) return *dots_[N_ - 1];
  if (!right_[first]) throw std::runtime_error("right block missing");
  resident(right_[first].get());
  return *right_[first];
}

// Heuristic quanta distribution of a warm-up block (the reference guesses a
// distribution too, initblocks.C:229-300): weight of a quantum ~ its size
// times a Gaussian in the particle number around the Hartree-Fock filling of
// the block's orbitals.  Returns the kept count per quantum.
std::vector<int> SweepDriver::warmup_rotation(Block& big, int M, uint64_t seed) {
  const int nsites = (int)big.sites.size();
  std::vector<int> order(N_);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return I_.h(a, a) < I_.h(b, b); });
  std::vector<int> occ(N_, 0);
  int left_e = target_.n;
  for (int o : order) {
    const int k = std::min(2, left_e);
    occ[o] = k;
    left_e -= k;
  }
  double nhf = 0;
  for (int s : big.sites) nhf += occ[s];
  const double sig = std::max(1.0, std::sqrt((double)nsites));
  // spin: low spins favoured for a singlet target; for a target of spin S
  // the block's share of 2S (by its sites) is favoured instead, so that
  // the first superblocks of a high-spin run hold enough states
  const double s2_share = (double)target_.s2 * nsites / std::max(1, N_);
  std::vector<double> w(big.si.size());
  double tot = 0;
  for (int q = 0; q < big.si.size(); ++q) {
    const double dn = big.si.quanta[q].n - nhf;
    const double ds = target_.s2 > 0 ? std::fabs(big.si.quanta[q].s2 - s2_share) : (double)big.si.quanta[q].s2;
    w[q] = big.si.states[q] * std::exp(-dn * dn / (2 * sig * sig)) / (1.0 + ds);
    tot += w[q];
  }
  std::vector<int> kept(big.si.size(), 0);
  const long total = big.si.total_states();
  int budget = (int)std::min<long>(M, total);
  std::vector<int> idx(big.si.size());
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return w[a] > w[b]; });
  for (int q : idx) {
    if (budget <= 0) break;
    if (w[q] <= 1e-12 * tot) continue;
    kept[q] = 1;
    --budget;
  }
  while (budget > 0) {
    bool any = false;
    for (int q : idx) {
      if (budget <= 0) break;
      const int want = (int)std::ceil(M * w[q] / tot);
      if (kept[q] < std::min(want, big.si.states[q])) {
        ++kept[q];
        --budget;
        any = true;
      }
    }
    if (!any) {
      for (int q : idx) {
        if (budget <= 0) break;
        if (kept[q] < big.si.states[q]) {
          ++kept[q];
          --budget;
          any = true;
        }
      }
      if (!any) break;
    }
  }
  Rng rng(seed);
  std::vector<std::vector<double>> rot(big.si.size());
  for (int q = 0; q < big.si.size(); ++q) {
    const int n = big.si.states[q], m = kept[q];
    if (m == 0) continue;
    rot[q].resize((size_t)n * m);
    for (auto& x : rot[q]) x = rng.normal();
    orthonormalise_columns(n, m, rot[q].data());
  }
  E_.set_rotation(rot, kept);
  return kept;
}

std::unique_ptr<Block> SweepDriver::renormalised(const Block& big, const std::vector<int>& kept,
                                                 const CatalogSpec& spec) {
  auto nb = std::make_unique<Block>();
  nb->sites = big.sites;
  std::vector<int> map;
  nb->si = truncated_stateinfo(big.si, kept, map);
  nb->ops = make_opset(nb->si, catalog_keys(spec), I_.orbsym, g_);
  for (const auto& kv : nb->ops.ops)
    if (!big.ops.has(kv.first)) throw std::runtime_error("renormalised block needs " + kv.first.str());
  E_.create_block(*nb);
  note_peak();
  E_.renormalise(*nb, big);
  return nb;
}

void SweepDriver::save_checkpoint(const std::string& path, int sweeps_done, bool next_forward, double sweep_energy,
                                  const std::vector<double>& sweep_energies) {
  CheckpointHeader h;
  h.norb = N_;
  h.nelec = target_.n;
  h.target = target_;
  h.nroots = C_.nroots;
  h.fingerprint = integrals_fingerprint(I_);
  h.sweeps_done = sweeps_done;
  h.next_forward = next_forward ? 1 : 0;
  h.cur_M = cur_M_;
  h.discarded = last_discarded_;
  h.last_sweep_energy = sweep_energy;
  h.energies = last_energies_;
  h.sweep_energies = sweep_energies;
  CheckpointWriter w(path);
  w.header(h);
  int nb = 0;
  std::vector<double> arena;
  for (int side = 0; side < 2; ++side)
    for (int p = 0; p < N_; ++p) {
      const Block* b = side == 0 ? left_[p].get() : right_[p].get();
      if (!b) continue;
      if (b->handle < 0) {  // spilled: its host copy
        auto it = host_.find(b);
        if (it == host_.end()) continue;
        w.block(side, p, b->sites, b->si, b->ops, it->second.arena, it->second.has_rot ? &it->second.rot : nullptr);
        ++nb;
        continue;
      }
      E_.download_block(*b, arena);  // one block at a time on the host
      RotationRecord rr;
      const bool has = E_.get_rotation_record(*b, rr);
      w.block(side, p, b->sites, b->si, b->ops, arena, has ? &rr : nullptr);
      ++nb;
    }
  w.finish(nb);
}

int SweepDriver::load_checkpoint(const std::string& path, bool& next_forward, double& sweep_energy,
                                 std::vector<double>& sweep_energies) {
  CheckpointReader rd(path);
  const CheckpointHeader& h = rd.header();
  if (h.norb != N_ || h.target != target_ || h.nroots != C_.nroots)
    throw std::runtime_error("checkpoint " + path + " was written for another system (orbitals, target or roots)");
  if (h.fingerprint != integrals_fingerprint(I_))
    throw std::runtime_error("checkpoint " + path + " was written for another Hamiltonian");
  CheckpointBlock cb;
  while (rd.next(cb)) {
    if (cb.index < 0 || cb.index >= N_ || (cb.side != 0 && cb.side != 1))
      throw std::runtime_error("checkpoint: block position out of range");
    auto b = std::make_unique<Block>();
    b->sites = cb.sites;
    b->si = cb.si;
    b->ops = make_opset(b->si, std::set<OpKey>(cb.keys.begin(), cb.keys.end()), I_.orbsym, g_);
    if (b->ops.arena != (int64_t)cb.arena.size())
      throw std::runtime_error("checkpoint: operator catalogue does not match its stored arena");
    auto& slot = cb.side == 0 ? left_[cb.index] : right_[cb.index];
    drop(slot);
    E_.create_block(*b);
    E_.upload_block(*b, cb.arena);
    if (cb.has_rot) E_.set_rotation_record(*b, cb.rot);
    note_peak();
    slot = std::move(b);
    spill_idle();
  }
  cur_M_ = h.cur_M;
  last_discarded_ = h.discarded;
  last_energies_ = h.energies;
  next_forward = h.next_forward != 0;
  sweep_energy = h.last_sweep_energy;
  sweep_energies = h.sweep_energies;
  return h.sweeps_done;
}

void SweepDriver::warmup() {
  const int M = C_.schedule.front().M;
  cur_M_ = M;
  int maxM = M;
  for (const auto& e : C_.schedule) maxM = std::max(maxM, e.M);
  E_.prepare_density(maxM);
  for (int p = N_ - 2; p >= 3; --p) {
    Block& sys = right_block(p + 1);
    std::vector<int> own;
    for (int i = p; i < N_; ++i) own.push_back(i);
    CatalogSpec spec = renorm_spec(own, p - 1, !loop_is_left(p - 2));
    Block big = make_enlarged(sys, p, /*dot_on_right=*/false, spec);
    spill_idle();  // the stored blocks are not read again by this step
    std::vector<int> kept = warmup_rotation(big, M, C_.seed + 7919ull * (uint64_t)p);
    drop(right_[p]);
    right_[p] = renormalised(big, kept, spec);
    E_.release_block(big);
    log(2, "warmup right block [%d..%d]: %ld states\n", p, N_ - 1, right_[p]->si.total_states());
  }
}

void SweepDriver::warmup_left(int upto) {
  const int M = C_.schedule.front().M;
  for (int q = 1; q <= upto; ++q) {
    Block& sys = left_block(q - 1);
    std::vector<int> own;
    for (int i = 0; i <= q; ++i) own.push_back(i);
    CatalogSpec spec = renorm_spec(own, q + 1, loop_is_left(q + 1));
    Block big = make_enlarged(sys, q, /*dot_on_right=*/true, spec);
    spill_idle();
    std::vector<int> kept = warmup_rotation(big, M, C_.seed + 6271ull * (uint64_t)q);
    drop(left_[q]);
    left_[q] = renormalised(big, kept, spec);
    E_.release_block(big);
  }
}

Superblock SweepDriver::prepare_partition(int p, Block& L, Block& R) {
  if (p < 1 || p > N_ - 3) throw std::runtime_error("partition out of range");
  warmup();
  warmup_left(p - 1);
  std::vector<int> Ls, Rs;
  for (int i = 0; i <= p; ++i) Ls.push_back(i);
  for (int i = p + 1; i < N_; ++i) Rs.push_back(i);
  const bool loopL = loop_is_left(p);
  const std::vector<int>& loop_sites = loopL ? Ls : Rs;
  L = make_enlarged(left_block(p - 1), p, true, sigma_spec(Ls, Rs, loopL, loop_sites));
  R = make_enlarged(right_block(p + 2), p + 1, false, sigma_spec(Rs, Ls, !loopL, loop_sites));
  return make_superblock(L, R);
}

// Truncation: keep the M largest density-matrix eigenvalues above 1e-13
// (makeRotateMatrix / sort_weights / assign_matrix_by_dm,
// renormalise.C:135-166, rotationmat.C:149-339); returns discarded weight.
static double choose_kept(const DensitySpectrum& spec, int M, std::vector<std::vector<int>>& kept_idx,
                          std::vector<int>& kept, double* cutoff = nullptr) {
  struct W { double w; int q, i; };
  std::vector<W> all;
  double norm = 0.0;
  for (int q = 0; q < (int)spec.eig.size(); ++q)
    for (int i = 0; i < (int)spec.eig[q].size(); ++i) {
      double w = spec.eig[q][i];
      if (w < 1e-14) w = 0.0;
      all.push_back({w, q, i});
      norm += w;
    }
  std::stable_sort(all.begin(), all.end(), [](const W& a, const W& b) { return a.w > b.w; });
  kept_idx.assign(spec.eig.size(), {});
  kept.assign(spec.eig.size(), 0);
  double keptw = 0.0;
  const int nk = std::min<int>(M, (int)all.size());
  for (int t = 0; t < nk; ++t) {
    if (all[t].w <= 1e-13) continue;
    kept_idx[all[t].q].push_back(all[t].i);
    keptw += all[t].w;
  }
  if (cutoff) {  // the last kept and the first discarded weight
    cutoff[0] = nk > 0 ? all[nk - 1].w : 0.0;
    cutoff[1] = nk < (int)all.size() ? all[nk].w : 0.0;
  }
  for (size_t q = 0; q < kept_idx.size(); ++q) {
    // keep the eigenvectors of each sector in descending weight order
    std::sort(kept_idx[q].begin(), kept_idx[q].end(), std::greater<int>());
    kept[q] = (int)kept_idx[q].size();
  }
  return norm - keptw;
}

double SweepDriver::step(bool forward, int p, int sweep_index, std::vector<double>& energies) {
  const ScheduleEntry& se = C_.entry(sweep_index);
  std::vector<int> Ls, Rs;
  for (int i = 0; i <= p; ++i) Ls.push_back(i);
  for (int i = p + 1; i < N_; ++i) Rs.push_back(i);
  const bool loopL = loop_is_left(p);
  const std::vector<int>& loop_sites = loopL ? Ls : Rs;
  CatalogSpec specL = sigma_spec(Ls, Rs, loopL, loop_sites);
  CatalogSpec specR = sigma_spec(Rs, Ls, !loopL, loop_sites);
  CatalogSpec keepspec;
  if (forward) {
    keepspec = renorm_spec(Ls, p + 1, loop_is_left(p + 1));
    merge(specL, keepspec);
  } else {
    keepspec = renorm_spec(Rs, p, !loop_is_left(p - 1));
    merge(specR, keepspec);
  }
  using clk = std::chrono::steady_clock;
  auto secs = [](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
  const SweepResult phase0 = phase_;
  auto t0 = clk::now();
  if (rdm_pass_) rdm_extras(p, specL, specR);
  Block L = make_enlarged(left_block(p - 1), p, true, specL);
  Block R = make_enlarged(right_block(p + 2), p + 1, false, specR);
  Superblock sb = make_superblock(L, R);
  // spill: the stored blocks go to host memory, except the two the guess
  // transform reads (the step's own source on the side it renormalises, and
  // the previous sweep's block it expands)
  if (opt_.transform_guess)
    spill_idle(forward ? left_[p - 1].get() : right_[p + 2].get(), forward ? right_[p + 1].get() : left_[p].get());
  else
    spill_idle();
  phase_.build_seconds += secs(t0);
  t0 = clk::now();
  E_.prepare_plan(sb);
  DavidsonParams dp;
  dp.nroots = C_.nroots;
  dp.tol = se.davidson_tol;
  dp.deflation_min = C_.deflation_min;
  dp.deflation_max = C_.deflation_max;
  dp.max_iter = C_.davidson_max_iter;
  dp.seed = C_.seed + 104729ull * (uint64_t)(sweep_index * N_ + p);
  dp.defer_refine = opt_.refine_window > 0.0;
  if (opt_.transform_guess && prev_.valid && prev_.forward == forward && prev_.p == (forward ? p - 1 : p + 1)) {
    GuessInput g;
    g.forward = forward;
    g.old_L = prev_.L;
    g.old_R = prev_.R;
    g.old_sectors = prev_.sectors;
    g.rotated = forward ? left_[p - 1].get() : right_[p + 2].get();
    g.expanded = forward ? right_[p + 1].get() : left_[p].get();
    g.dot = forward ? &dots_[p]->si : &dots_[p + 1]->si;
    resident(forward ? left_[p - 1].get() : right_[p + 2].get());
    resident(forward ? right_[p + 1].get() : left_[p].get());
    if (g.rotated && g.expanded) dp.use_guess = E_.transform_guess(g, sb);
  }
  spill_idle();
  const int iters = E_.solve(sb, dp, energies);
  char prec_tag[64] = "";
  int parked = -1;
  double e_unrefined = 0.0;
  if (dp.defer_refine && !energies.empty()) {
    const bool last_step = forward ? (p == N_ - 3) : (p == 1);
    e_unrefined = energies[0];
    sweep_best_unrefined_ = std::min(sweep_best_unrefined_, e_unrefined);
    settle_candidates(false);  // steps now too far above the lowest one are dropped
    const bool qualifies = e_unrefined <= sweep_best_unrefined_ + opt_.refine_window;
    if (!last_step && qualifies && opt_.deferred_steps > 0) parked = E_.park_vectors();
    if (parked >= 0) {
      std::snprintf(prec_tag, sizeof(prec_tag), " (unrefined; refinement deferred)");
    } else if (last_step || qualifies) {
      if (E_.refine(sb, energies))
        std::snprintf(prec_tag, sizeof(prec_tag), " (refined; unrefined %+.3e)", e_unrefined - energies[0]);
      note_refined(energies);
    } else {
      std::snprintf(prec_tag, sizeof(prec_tag), " (unrefined)");
    }
  } else {
    note_refined(energies);
  }
  if (rdm_pass_) rdm_step(p, sb);
  phase_.solve_seconds += secs(t0);
  if (opt_.on_step) opt_.on_step(sb, sweep_index, p);
  t0 = clk::now();
  DensitySpectrum spec;
  {
    // the schedule's (perturbative) noise, and the random noise of
    // twodot_noise in the first sweep (DensityMatrix::makedensitymatrix,
    // density.C:27-90, called from renormalise.C:95-104)
    NoiseSpec ns;
    ns.perturbative = se.noise;
    ns.random = sweep_index == 0 ? C_.twodot_noise : 0.0;
    ns.seed = C_.seed + 0x5851F42D4C957F2Dull * (uint64_t)(sweep_index * N_ + p + 1);
    if (ns.any()) {
      ns.orbsym = I_.orbsym;
      ns.group = g_;
    }
    E_.set_noise(ns);
  }
  E_.density(sb, forward, C_.weights, spec);
  std::vector<std::vector<int>> kept_idx;
  std::vector<int> kept;
  double cut[2];
  const double disc = choose_kept(spec, se.M, kept_idx, kept, cut);
  if (opt_.verbose >= 3) {
    std::string s;
    for (size_t q = 0; q < kept.size(); ++q)
      if (kept[q]) s += " " + std::to_string(q) + ":" + std::to_string(kept[q]);
    log(3, "    kept%s  (cutoff %.17g | %.17g)\n", s.c_str(), cut[0], cut[1]);
  }
  if (opt_.verbose >= 4)  // the whole spectrum, sector by sector
    for (size_t q = 0; q < spec.eig.size(); ++q) {
      std::string s;
      char buf[32];
      for (double x : spec.eig[q]) {
        std::snprintf(buf, sizeof(buf), " %.10e", x);
        s += buf;
      }
      log(4, "    rho[%zu]%s\n", q, s.c_str());
    }
  E_.select_rotation(kept_idx);
  phase_.density_seconds += secs(t0);
  t0 = clk::now();
  if (forward) {
    drop(left_[p]);
    left_[p] = renormalised(L, kept, keepspec);
  } else {
    drop(right_[p + 1]);
    right_[p + 1] = renormalised(R, kept, keepspec);
  }
  phase_.renorm_seconds += secs(t0);
  prev_.valid = true;
  prev_.forward = forward;
  prev_.p = p;
  prev_.L = L.si;
  prev_.R = R.si;
  prev_.sectors = sb.sectors;
  log(1, "  %s p=%2d  L=%ld R=%ld psi=%ld  iters=%d  E=%.12f%s  disc=%.3e%s  [build %.3fs solve %.3fs density %.3fs renorm %.3fs]\n",
      forward ? "fwd" : "bwd", p, L.si.total_states(), R.si.total_states(), (long)sb.size, iters,
      energies.empty() ? 0.0 : energies[0], prec_tag, disc, E_.step_stats().c_str(),
      phase_.build_seconds - phase0.build_seconds, phase_.solve_seconds - phase0.solve_seconds,
      phase_.density_seconds - phase0.density_seconds, phase_.renorm_seconds - phase0.renorm_seconds);
  if (parked >= 0) {
    // keep the step's enlarged blocks for a refinement at the end of the sweep
    auto c = std::make_unique<Candidate>();
    c->L = std::make_unique<Block>(std::move(L));
    c->R = std::make_unique<Block>(std::move(R));
    c->sb = std::move(sb);
    c->sb.L = c->L.get();
    c->sb.R = c->R.get();
    c->parked = parked;
    c->p = p;
    c->e_unrefined = e_unrefined;
    cands_.push_back(std::move(c));
    while ((int)cands_.size() > opt_.deferred_steps) {
      // over the limit: refine the highest one now
      size_t hi = 0;
      for (size_t i = 1; i < cands_.size(); ++i)
        if (cands_[i]->e_unrefined > cands_[hi]->e_unrefined) hi = i;
      refine_candidate(*cands_[hi]);
      drop_candidate(cands_[hi]);
      cands_.erase(cands_.begin() + hi);
    }
  } else {
    E_.release_block(L);
    E_.release_block(R);
  }
  return disc;
}

void SweepDriver::note_refined(const std::vector<double>& e) {
  if (!e.empty() && e[0] < sweep_refined_min_) {
    sweep_refined_min_ = e[0];
    sweep_refined_best_ = e;
  }
}

void SweepDriver::refine_candidate(Candidate& c) {
  std::vector<double> e(C_.nroots, 0.0);
  if (E_.refine_parked(c.parked, c.sb, e)) {
    log(1, "  refined p=%2d  E=%.12f (unrefined %+.3e)\n", c.p, e[0], c.e_unrefined - e[0]);
    note_refined(e);
  }
}

void SweepDriver::drop_candidate(std::unique_ptr<Candidate>& c) {
  E_.drop_parked(c->parked);
  E_.release_block(*c->L);
  E_.release_block(*c->R);
  c.reset();
}

// Drops the deferred steps whose unrefined energy is more than the window
// above the sweep's lowest; at the end of the sweep refines the others.
void SweepDriver::settle_candidates(bool end_of_sweep) {
  for (auto& c : cands_) {
    if (!c) continue;
    const bool near = c->e_unrefined <= sweep_best_unrefined_ + opt_.refine_window;
    if (end_of_sweep && near) refine_candidate(*c);
    if (end_of_sweep || !near) drop_candidate(c);
  }
  cands_.erase(std::remove(cands_.begin(), cands_.end(), nullptr), cands_.end());
}

double SweepDriver::sweep(bool forward, int sweep_index) {
  double maxdisc = 0.0;
  sweep_best_unrefined_ = std::numeric_limits<double>::infinity();
  sweep_refined_min_ = std::numeric_limits<double>::infinity();
  sweep_refined_best_.clear();
  auto one = [&](int p) {
    std::vector<double> e;
    maxdisc = std::max(maxdisc, step(forward, p, sweep_index, e));
    last_energies_ = e;  // the last step of a sweep is always refined
  };
  if (forward)
    for (int p = 1; p <= N_ - 3; ++p) one(p);
  else
    for (int p = N_ - 3; p >= 1; --p) one(p);
  settle_candidates(true);
  last_discarded_ = maxdisc;
  // sweep energy: the lowest refined step energy (Sweep::do_one, sweep.C:436-453)
  return sweep_refined_min_;
}

// One-particle density matrix (modules/onepdm, onepdm.C:24-55 and its
// compute_one_pdm_* kernels): gamma_ij = sqrt(2) <[C_i x D_j]^0> with
// [C_i x D_j]^0 = (a+_i,up a_j,up + a+_i,dn a_j,dn) / sqrt(2).  Over one sweep
// every element is taken once, at the step p (L = [0..p], R = [p+1..N-1]):
//   i = p < j, and at p = 1 also i = 0 < j (operators C_i on L, D_j on R);
//   i = j = p for 2 <= p <= N-3 (CD^0_pp on L);
//   i, j in {0, 1} at p = 1 (CD^0 on L) and in {N-2, N-1} at p = N-3 (on R);
// gamma of one root is symmetric (real wavefunctions); between roots a and b
// the sweep takes the transition elements <a|E_ij|b> (tran_onepdm,
// modules/onepdm/onepdm.C with the transition flag) from the same terms.
// Each step's solve fixes every root only up to its sign, so the relative
// sign of two roots may flip from one step to the next: every step also
// takes the cross elements (p-1, j > p), which the neighbouring step takes
// too, and flips root r when its largest shared element <r|E_ij|0>
// changes sign (the phase the reference carries along its sweep through the
// transformed guesses).
void SweepDriver::rdm_extras(int p, CatalogSpec& specL, CatalogSpec& specR) const {
  auto add = [](CatalogSpec& s, const OpKey& k) {
    if (std::find(s.extra.begin(), s.extra.end(), k) == s.extra.end()) s.extra.push_back(k);
  };
  if (p == 1) {
    add(specL, cd_key(0, 0, 0));
    add(specL, cd_key(1, 0, 0));
    add(specL, cd_key(1, 1, 0));
  } else {
    add(specL, cd_key(p, p, 0));
  }
  if (p == N_ - 3) {
    add(specR, cd_key(N_ - 2, N_ - 2, 0));
    add(specR, cd_key(N_ - 1, N_ - 2, 0));
    add(specR, cd_key(N_ - 1, N_ - 1, 0));
  }
}

void SweepDriver::rdm_step(int p, const Superblock& sb) {
  const double r2 = std::sqrt(2.0);
  std::vector<PairTerm> terms;
  std::vector<std::pair<int, int>> at;
  auto cross = [&](int i, int j) {
    PairTerm t;
    t.coef = r2;
    t.l = op(cre_key(i));
    t.r = op(cre_key(j), true);
    terms.push_back(t);
    at.push_back({i, j});
  };
  auto inside = [&](bool left, int a, int b) {  // a >= b
    PairTerm t;
    t.coef = r2;
    if (left) {
      t.l = op(cd_key(a, b, 0));
      t.r = ident();
    } else {
      t.l = ident();
      t.r = op(cd_key(a, b, 0));
    }
    terms.push_back(t);
    at.push_back({a, b});
  };
  for (int j = p + 1; j < N_; ++j) cross(p, j);
  const size_t nfirst = terms.size();
  if (p >= 1)  // the shared elements of the neighbouring step p - 1
    for (int j = p + 1; j < N_; ++j) cross(p - 1, j);
  const size_t nlink = terms.size();
  if (p == 1) {
    for (int j = 2; j < N_; ++j) cross(0, j);
    inside(true, 0, 0);
    inside(true, 1, 0);
    inside(true, 1, 1);
  } else {
    inside(true, p, p);
  }
  if (p == N_ - 3) {
    inside(false, N_ - 2, N_ - 2);
    inside(false, N_ - 1, N_ - 2);
    inside(false, N_ - 1, N_ - 1);
  }
  std::vector<double> v;
  E_.expectations(sb, terms, v);
  const size_t nt = terms.size();
  const int nr = (int)std::lround(std::sqrt((double)(v.size() / std::max<size_t>(nt, 1))));
  if ((int)rdm_.size() < nr * nr) rdm_.resize((size_t)nr * nr, std::vector<double>((size_t)N_ * N_, 0.0));
  auto val = [&](int a, int b, size_t t) { return v[((size_t)a * nr + b) * nt + t]; };
  // phase of every root relative to root 0, from the elements shared with
  // the previous step
  std::vector<double> sgn(nr, 1.0);
  for (int r = 1; r < nr; ++r) {
    double best = 0.0, cur = 0.0;
    for (size_t t = 0; t < nlink; ++t) {
      auto it = rdm_link_.find(at[t]);
      if (it == rdm_link_.end()) continue;
      const double prev = it->second[r];
      if (std::fabs(prev) > std::fabs(best)) {
        best = prev;
        cur = val(r, 0, t);
      }
    }
    if (std::fabs(best) > 1e-8 && (cur < 0.0) != (best < 0.0)) sgn[r] = -1.0;
  }
  rdm_link_.clear();
  for (size_t t = 0; t < nlink; ++t) {
    std::vector<double> col(nr);
    for (int r = 0; r < nr; ++r) col[r] = sgn[r] * val(r, 0, t);
    rdm_link_[at[t]] = col;
  }
  // <a|E_ij|b> from the term (i, j); <a|E_ji|b> = <b|E_ij|a> (real vectors)
  for (int a = 0; a < nr; ++a)
    for (int b = 0; b < nr; ++b)
      for (size_t t = 0; t < nt; ++t) {
        if (t >= nfirst && t < nlink) continue;  // taken by the neighbouring step
        const int i = at[t].first, j = at[t].second;
        const double s = sgn[a] * sgn[b];
        rdm_[(size_t)a * nr + b][(size_t)i * N_ + j] = s * val(a, b, t);
        rdm_[(size_t)a * nr + b][(size_t)j * N_ + i] = s * val(b, a, t);
      }
}

std::vector<std::vector<double>> SweepDriver::onepdm_sweep(bool forward, int sweep_index) {
  if (N_ < 4) throw std::runtime_error("onepdm needs at least 4 orbitals");
  rdm_.clear();
  rdm_link_.clear();
  rdm_pass_ = true;
  try {
    sweep(forward, sweep_index);
  } catch (...) {
    rdm_pass_ = false;
    throw;
  }
  rdm_pass_ = false;
  return std::move(rdm_);
}

SweepResult SweepDriver::run() {
  SweepResult res;
  struct NoiseOff {  // the engine's noise ends with the run
    Engine& e;
    ~NoiseOff() { e.set_noise(NoiseSpec{}); }
  } noise_off{E_};
  double eprev = std::numeric_limits<double>::infinity();
  int s_begin = 0;
  bool first_forward = true;
  if (C_.restart) {
    // resume after the checkpoint's last sweep (dmrg.C:476-560 restarts from
    // the saved blocks the same way); reset_iter starts the schedule over
    int maxM = 0;
    for (const auto& e : C_.schedule) maxM = std::max(maxM, e.M);
    E_.prepare_density(maxM);
    s_begin = load_checkpoint(C_.checkpoint, first_forward, eprev, res.sweep_energies);
    if (C_.reset_iter) s_begin = 0;
    log(1, "restart from %s: %d sweeps done, next sweep %s\n", C_.checkpoint.c_str(), s_begin,
        first_forward ? "forward" : "backward");
  } else {
    const auto tw = std::chrono::steady_clock::now();
    warmup();
    E_.device_renorm_seconds();  // waits for the warm-up's device work
    res.warmup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - tw).count();
  }
  const double rd0 = E_.device_renorm_seconds(), rf0 = E_.renorm_flops();
  const int last_sched = C_.schedule.back().iter;
  for (int s = s_begin; s < C_.maxiter; ++s) {
    const bool forward = ((s - s_begin) % 2 == 0) == first_forward;
    const auto ts = std::chrono::steady_clock::now();
    const double r0 = E_.device_renorm_seconds();
    const double e = sweep(forward, s);
    E_.device_renorm_seconds();  // the sweep's device work is part of its wall time
    res.sweep_seconds.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - ts).count());
    res.sweep_energies.push_back(e);
    res.sweeps = s + 1;
    // phases are host wall times; the renormalisation's device work runs
    // on while the host builds and plans the next step, so its device time
    // is shown beside them
    log(1, "sweep %d (%s) M=%d  E=%.12f  dE=%.3e  maxdisc=%.3e  wall %.2fs  [build %.2fs solve %.2fs density %.2fs renorm %.2fs; renorm on device %.2fs]\n",
        s, forward ? "fwd" : "bwd", C_.entry(s).M, e, e - eprev, last_discarded_,
        std::chrono::duration<double>(std::chrono::steady_clock::now() - ts).count(), phase_.build_seconds,
        phase_.solve_seconds, phase_.density_seconds, phase_.renorm_seconds, E_.device_renorm_seconds() - r0);
    if (!C_.checkpoint.empty()) {
      const auto tc = std::chrono::steady_clock::now();
      save_checkpoint(C_.checkpoint, s + 1, !forward, e, res.sweep_energies);
      log(1, "checkpoint after sweep %d written to %s (%.2fs)\n", s, C_.checkpoint.c_str(),
          std::chrono::duration<double>(std::chrono::steady_clock::now() - tc).count());
    }
    if (s >= last_sched && std::fabs(e - eprev) <= C_.sweep_tol) break;
    eprev = e;
  }
  if (C_.onepdm) {
    // one more sweep, in the next direction, with the final schedule entry
    const int last = std::max(res.sweeps - 1, 0);
    const bool forward = ((res.sweeps - s_begin) % 2 == 0) == first_forward;
    const auto ts = std::chrono::steady_clock::now();
    auto g = onepdm_sweep(forward, last);
    const int nr = (int)std::lround(std::sqrt((double)g.size()));
    res.transition_onepdm.assign(g.size(), std::vector<double>((size_t)N_ * N_, 0.0));
    for (size_t r = 0; r < g.size(); ++r)
      for (int a = 0; a < N_; ++a)
        for (int b = 0; b < N_; ++b) {
          const int A = I_.order.empty() ? a : I_.order[a], B = I_.order.empty() ? b : I_.order[b];
          res.transition_onepdm[r][(size_t)A * N_ + B] = g[r][(size_t)a * N_ + b];
        }
    for (int r = 0; r < nr; ++r) res.onepdm.push_back(res.transition_onepdm[(size_t)r * nr + r]);
    log(1, "onepdm sweep (%s): %.2fs\n", forward ? "fwd" : "bwd",
        std::chrono::duration<double>(std::chrono::steady_clock::now() - ts).count());
    if (!C_.prefix.empty())
      for (int i = 0; i < nr; ++i)
        for (int j = 0; j <= i; ++j) {
          if (i != j && !C_.tran_onepdm) continue;
          // spatial_onepdm.i.j.txt (save_onepdm_spatial_text, onepdm.C:504-528):
          // element (k, l) = <i|E_kl|j>
          const std::vector<double>& m = res.transition_onepdm[(size_t)i * nr + j];
          const std::string path =
              C_.prefix + "/spatial_onepdm." + std::to_string(i) + "." + std::to_string(j) + ".txt";
          FILE* f = std::fopen(path.c_str(), "w");
          if (!f) throw std::runtime_error("cannot write " + path);
          std::fprintf(f, "%d\n", N_);
          for (int a = 0; a < N_; ++a)
            for (int b = 0; b < N_; ++b) std::fprintf(f, "%d %d %20.14e\n", a, b, m[(size_t)a * N_ + b]);
          std::fclose(f);
        }
  }
  res.sweep_renorm_device_seconds = E_.device_renorm_seconds() - rd0;
  res.sweep_renorm_flops = E_.renorm_flops() - rf0;
  res.energies = last_energies_;
  res.discarded = last_discarded_;
  res.build_seconds = phase_.build_seconds;
  res.solve_seconds = phase_.solve_seconds;
  res.density_seconds = phase_.density_seconds;
  res.renorm_seconds = phase_.renorm_seconds;
  res.renorm_device_seconds = E_.device_renorm_seconds();
  res.spill_fetches = spill_fetches_;
  res.spill_bytes_up = spill_up_;
  res.spill_bytes_down = spill_down_;
  res.peak_block_bytes = peak_bytes_;
  return res;
}

}  // namespace bgpu
