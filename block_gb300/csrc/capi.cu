// extern "C" boundary of the library (declarations and reference mapping in
// include/bgpu.h).
#include <cuda_profiler_api.h>

#include <chrono>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>

#include "../../include/bgpu.h"
#include "cuda/gpu_engine.h"
#include "cuda/k_tc.cuh"
#include "host/sweep.h"

using namespace bgpu;

struct bgpu_ctx {
  std::unique_ptr<GpuEngine> eng;
  std::string err;
  int device = 0;
  double refine_window = 1e-3;  // Eh; see bgpu_set_refine_window
  std::vector<double> sweep_energies;  // of the last bgpu_run_dmrg
  std::vector<double> run_stats;       // see bgpu_run_stats
  std::vector<std::vector<double>> onepdm;  // of the last bgpu_run_dmrg with `onepdm`
  std::vector<std::vector<double>> tonepdm;  // per root pair (bra * nroots + ket)
  bool transform_guess = true;  // see bgpu_set_guess
  bool spill = false;           // see bgpu_set_spill
  int deferred_steps = 4;        // see bgpu_set_refine_window
  struct BlockRec {
    Block b;
    std::vector<OpKey> decl;  // declaration order
    std::vector<int> orbsym;
    std::string group = "c1";
    bool filled = false;  // arena uploaded or computed by the library
  };
  std::map<int, std::unique_ptr<BlockRec>> blocks;
  std::map<int, std::unique_ptr<Integrals>> integrals;
  struct SbRec {
    Superblock sb;
    SigmaPlan plan;
    double* psi = nullptr;
    double* sig = nullptr;
    // superblocks prepared from a configuration own their blocks
    std::unique_ptr<Block> ownL, ownR;
    std::unique_ptr<SweepDriver> drv;
    std::vector<int> orbsym;  // orbital irreps and point group (density noise)
    std::string group = "c1";
  };
  NoiseSpec density_noise;  // see bgpu_set_density_noise
  std::map<int, std::unique_ptr<SbRec>> sbs;
  int next = 1;
};

namespace {
template <class F>
int guarded(bgpu_ctx* ctx, F&& f) {
  if (!ctx) return BGPU_ERR_INVALID;
  try {
    f();
    ctx->err.clear();
    return BGPU_OK;
  } catch (const CudaError& e) {
    ctx->err = e.what();
    return BGPU_ERR_CUDA;
  } catch (const std::invalid_argument& e) {
    ctx->err = e.what();
    return BGPU_ERR_INVALID;
  } catch (const std::exception& e) {
    ctx->err = e.what();
    return BGPU_ERR_RUNTIME;
  }
}
void need(bool c, const char* what) {
  if (!c) throw std::invalid_argument(what);
}
void need(bool c, const std::string& what) {
  if (!c) throw std::invalid_argument(what);
}
// operator keys (type, i, j, 2k) of a C-ABI catalogue, in declaration order
std::set<OpKey> read_keys(int nops, const int* op_keys, int norb, std::vector<OpKey>& decl) {
  std::set<OpKey> keys;
  decl.clear();
  for (int o = 0; o < nops; ++o) {
    const int t = op_keys[4 * o], i = op_keys[4 * o + 1], j = op_keys[4 * o + 2], k2 = op_keys[4 * o + 3];
    need(t >= 0 && t <= BGPU_OP_OVERLAP, "bad operator type");
    need(i < norb && j < norb, "orbital index out of range");
    need(k2 >= 0 && k2 <= 4, "bad tensor rank");
    OpKey k;
    k.type = (OpType)t;
    k.i = (int16_t)i;
    k.j = (int16_t)j;
    k.k2 = (int8_t)k2;
    need(keys.insert(k).second, "duplicate operator key");
    decl.push_back(k);
  }
  return keys;
}
}  // namespace

extern "C" {

const char* bgpu_version(void) { return "block_gb300 0.1 (sm_103a)"; }

int bgpu_create(bgpu_ctx** out, int device) {
  if (!out) return BGPU_ERR_INVALID;
  *out = nullptr;
  auto* c = new bgpu_ctx;
  c->device = device;
  int rc = guarded(c, [&] { c->eng = std::make_unique<GpuEngine>(device); });
  if (rc != BGPU_OK) {
    // keep the context so the caller can read the message
    *out = c;
    return rc;
  }
  *out = c;
  return BGPU_OK;
}

int bgpu_destroy(bgpu_ctx* ctx) {
  if (!ctx) return BGPU_ERR_INVALID;
  try {
    if (ctx->eng) {
      for (auto& kv : ctx->sbs) {
        ctx->eng->free_plan(kv.second->plan);
        ctx->eng->free(kv.second->psi);
        ctx->eng->free(kv.second->sig);
      }
      for (auto& kv : ctx->blocks) ctx->eng->release_block(kv.second->b);
      ctx->eng->sync();
    }
  } catch (...) {
  }
  delete ctx;
  return BGPU_OK;
}

const char* bgpu_last_error_string(const bgpu_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int bgpu_set_guess(bgpu_ctx* ctx, int transform) {
  return guarded(ctx, [&] { ctx->transform_guess = transform != 0; });
}

int bgpu_set_spill(bgpu_ctx* ctx, int on) {
  return guarded(ctx, [&] { ctx->spill = on != 0; });
}

int bgpu_set_davidson_graph(bgpu_ctx* ctx, int on) {
  return guarded(ctx, [&] {
    need(ctx->eng != nullptr, "no device");
    ctx->eng->dav_graph = on != 0;
  });
}

int bgpu_set_tc_schedule(bgpu_ctx* ctx, int mode) {
  return guarded(ctx, [&] {
    need(ctx->eng != nullptr, "no device");
    need(mode == 0 || mode == 1, "schedule mode must be 0 (persistent) or 1 (per sector)");
    ctx->eng->tc_schedule_mode = mode;
  });
}

int bgpu_set_tc_tile_width(bgpu_ctx* ctx, int nb) {
  return guarded(ctx, [&] {
    need(ctx->eng != nullptr, "no device");
    need(nb == 0 || nb == dev::kTcRowsB || nb == dev::kTcRowsBWide, "tile width must be 0 (automatic), 64 or 128");
    ctx->eng->tc_nb_mode = nb;
  });
}

int bgpu_set_tc_stacking(bgpu_ctx* ctx, int rows) {
  return guarded(ctx, [&] {
    need(ctx->eng != nullptr, "no device");
    need(rows >= 0 && rows <= dev::kTcRowsA && rows % 8 == 0, "stacking limit must be 0 or a multiple of 8 up to 128");
    ctx->eng->tc_stack_rows = rows;
  });
}

int bgpu_set_autotune(bgpu_ctx* ctx, int on, const char* cache_path) {
  return guarded(ctx, [&] {
    need(ctx->eng != nullptr, "no device");
    ctx->eng->tc_autotune = on != 0;
    if (cache_path) ctx->eng->load_tune_cache(cache_path);
  });
}

int bgpu_autotune_stats(bgpu_ctx* ctx, int64_t* keys_tuned, int64_t* keys_cached, double* seconds) {
  return guarded(ctx, [&] {
    need(ctx->eng != nullptr, "no device");
    if (keys_tuned) *keys_tuned = ctx->eng->tune_runs;
    if (keys_cached) *keys_cached = (int64_t)ctx->eng->tune_cache.size();
    if (seconds) *seconds = ctx->eng->tune_seconds;
  });
}

int bgpu_davidson_graph_launches(bgpu_ctx* ctx, int64_t* launches) {
  return guarded(ctx, [&] {
    need(ctx->eng != nullptr && launches, "bad arguments");
    *launches = ctx->eng->dav_graph_launches_;
  });
}

int bgpu_set_refine_window(bgpu_ctx* ctx, double eh) {
  return guarded(ctx, [&] {
    need(eh >= 0.0, "refine window must be >= 0");
    ctx->refine_window = eh;
  });
}

int bgpu_sweep_energies(bgpu_ctx* ctx, double* e, int cap, int* n) {
  return guarded(ctx, [&] {
    need(n != nullptr && (cap == 0 || e), "null argument");
    *n = (int)ctx->sweep_energies.size();
    for (int i = 0; i < cap && i < *n; ++i) e[i] = ctx->sweep_energies[i];
  });
}

int bgpu_onepdm(bgpu_ctx* ctx, int root, double* gamma, int norb) {
  return guarded(ctx, [&] {
    need(gamma != nullptr, "null argument");
    need(root >= 0 && root < (int)ctx->onepdm.size(),
         "no one-particle density matrix of this root (the last bgpu_run_dmrg needs the onepdm keyword)");
    need((size_t)norb * norb == ctx->onepdm[root].size(), "norb does not match the last run");
    std::copy(ctx->onepdm[root].begin(), ctx->onepdm[root].end(), gamma);
  });
}

int bgpu_transition_onepdm(bgpu_ctx* ctx, int bra, int ket, double* gamma, int norb) {
  return guarded(ctx, [&] {
    need(gamma != nullptr, "null argument");
    const int nr = (int)ctx->onepdm.size();
    need(bra >= 0 && bra < nr && ket >= 0 && ket < nr,
         "no transition density matrix of these roots (the last bgpu_run_dmrg needs the onepdm keyword)");
    const auto& m = ctx->tonepdm[(size_t)bra * nr + ket];
    need((size_t)norb * norb == m.size(), "norb does not match the last run");
    std::copy(m.begin(), m.end(), gamma);
  });
}

int bgpu_run_stats(bgpu_ctx* ctx, double* out, int n) {
  return guarded(ctx, [&] {
    need(out && n >= 0, "null argument");
    for (int i = 0; i < n; ++i) out[i] = i < (int)ctx->run_stats.size() ? ctx->run_stats[i] : 0.0;
  });
}

int bgpu_set_refinement(bgpu_ctx* ctx, int mode) {
  return guarded(ctx, [&] {
    need(ctx->eng != nullptr, "no device");
    need(mode == 0 || mode == 1 || mode == 2,
         "refinement mode must be 0 (energy only), 1 (defect correction) or 2 (defect correction, exact-slice "
         "tensor-core products)");
    ctx->eng->refine_mode = mode;
  });
}

int bgpu_refinement_stats(bgpu_ctx* ctx, int64_t* rounds, int64_t* fp64_products, int* last_verified) {
  return guarded(ctx, [&] {
    need(ctx->eng != nullptr, "no device");
    if (rounds) *rounds = ctx->eng->defect_rounds_;
    if (fp64_products) *fp64_products = ctx->eng->defect_fp64_sigma_;
    if (last_verified)
      *last_verified = ctx->eng->last_fp64_verified_ ? (ctx->eng->last_defect_bounded_ ? 2 : 1) : 0;
  });
}

int bgpu_set_precision(bgpu_ctx* ctx, int p) {
  return guarded(ctx, [&] {
    need(p == BGPU_PREC_FP64 || p == BGPU_PREC_BF16X3 || p == BGPU_PREC_BF16X6 || p == BGPU_PREC_BF16X3_TC ||
             p == BGPU_PREC_FP16X2_TC || p == BGPU_PREC_EXACT_TC,
         "unknown precision");
    need(ctx->eng != nullptr, "no device");
    ctx->eng->precision = (Precision)p;
  });
}

int bgpu_block_define(bgpu_ctx* ctx, int norb, const int* orbsym, const char* group, int nquanta, const int* quanta,
                      const int* states, int nops, const int* op_keys, int is_dot, int* handle, int64_t* arena_elems) {
  return guarded(ctx, [&] {
    need(ctx->eng != nullptr, "no device");
    need(norb > 0 && orbsym && quanta && states && handle && arena_elems, "null argument");
    need(nquanta > 0 && nops >= 0 && (nops == 0 || op_keys), "bad sizes");
    auto rec = std::make_unique<bgpu_ctx::BlockRec>();
    rec->orbsym.assign(orbsym, orbsym + norb);
    rec->group = group ? group : "c1";
    PointGroup g = PointGroup::from_name(rec->group);
    for (int q = 0; q < nquanta; ++q) {
      Quantum Q{quanta[3 * q], quanta[3 * q + 1], quanta[3 * q + 2]};
      need(Q.s2 >= 0 && Q.irrep >= 0 && Q.irrep < g.nirrep, "bad quantum");
      need(states[q] > 0, "sector without states");
      if (q) need(rec->b.si.quanta.back() < Q, "quanta must be sorted ascending and unique");
      rec->b.si.quanta.push_back(Q);
      rec->b.si.states.push_back(states[q]);
    }
    std::set<OpKey> keys = read_keys(nops, op_keys, norb, rec->decl);
    rec->b.ops = make_opset(rec->b.si, keys, rec->orbsym, g);
    rec->b.is_dot = is_dot != 0;
    rec->b.sites.clear();
    ctx->eng->create_block(rec->b);
    *arena_elems = rec->b.ops.arena;
    *handle = ctx->next++;
    ctx->blocks[*handle] = std::move(rec);
  });
}

int bgpu_block_op_offsets(bgpu_ctx* ctx, int handle, int64_t* offsets, int nops) {
  return guarded(ctx, [&] {
    auto it = ctx->blocks.find(handle);
    need(it != ctx->blocks.end() && offsets, "bad block");
    need(nops == (int)it->second->decl.size(), "nops mismatch");
    for (int o = 0; o < nops; ++o) offsets[o] = it->second->b.ops.at(it->second->decl[o]).base;
  });
}

int bgpu_block_upload(bgpu_ctx* ctx, int handle, const double* a, int64_t n) {
  return guarded(ctx, [&] {
    auto it = ctx->blocks.find(handle);
    need(it != ctx->blocks.end() && a, "bad block");
    need(n == it->second->b.ops.arena, "arena size mismatch");
    ctx->eng->upload_block(it->second->b, std::vector<double>(a, a + n));
    it->second->filled = true;
  });
}

int bgpu_block_download(bgpu_ctx* ctx, int handle, double* a, int64_t n) {
  return guarded(ctx, [&] {
    auto it = ctx->blocks.find(handle);
    need(it != ctx->blocks.end() && a, "bad block");
    need(n == it->second->b.ops.arena, "arena size mismatch");
    std::vector<double> h;
    ctx->eng->download_block(it->second->b, h);
    std::memcpy(a, h.data(), n * sizeof(double));
  });
}

int bgpu_block_free(bgpu_ctx* ctx, int handle) {
  return guarded(ctx, [&] {
    auto it = ctx->blocks.find(handle);
    need(it != ctx->blocks.end(), "bad block");
    ctx->eng->release_block(it->second->b);
    ctx->blocks.erase(it);
  });
}

int bgpu_superblock_define(bgpu_ctx* ctx, int left, int right, const int* target, int nterms, const double* coef,
                           const int* term_ops, double ecore, int* sbh, int64_t* psi_elems) {
  return guarded(ctx, [&] {
    auto li = ctx->blocks.find(left), ri = ctx->blocks.find(right);
    need(li != ctx->blocks.end() && ri != ctx->blocks.end(), "bad block handle");
    need(target && sbh && psi_elems && (nterms == 0 || (coef && term_ops)), "null argument");
    auto rec = std::make_unique<bgpu_ctx::SbRec>();
    Superblock& sb = rec->sb;
    sb.L = &li->second->b;
    sb.R = &ri->second->b;
    sb.target = {target[0], target[1], target[2]};
    sb.ecore = ecore;
    const auto& L = *sb.L;
    const auto& R = *sb.R;
    for (int lq = 0; lq < L.si.size(); ++lq)
      for (int rq = 0; rq < R.si.size(); ++rq) {
        const Quantum& a = L.si.quanta[lq];
        const Quantum& b = R.si.quanta[rq];
        // abelian irreps: XOR product
        Quantum t = sb.target;
        if (t.n != a.n + b.n || t.irrep != (a.irrep ^ b.irrep) || t.s2 < std::abs(a.s2 - b.s2) || t.s2 > a.s2 + b.s2 ||
            ((t.s2 + a.s2 + b.s2) & 1))
          continue;
        Superblock::Sector s;
        s.lq = lq;
        s.rq = rq;
        s.rows = L.si.states[lq];
        s.cols = R.si.states[rq];
        s.offset = sb.size;
        sb.size += (int64_t)s.rows * s.cols;
        sb.sectors.push_back(s);
      }
    need(sb.size > 0, "no sector couples to the target");
    for (int t = 0; t < nterms; ++t) {
      PairTerm p;
      p.coef = coef[t];
      const int lo = term_ops[4 * t], lt = term_ops[4 * t + 1], ro = term_ops[4 * t + 2], rt = term_ops[4 * t + 3];
      need(lo >= -1 && lo < (int)li->second->decl.size() && ro >= -1 && ro < (int)ri->second->decl.size(),
           "term operator index out of range");
      p.l = lo < 0 ? ident() : op(li->second->decl[lo], lt != 0);
      p.r = ro < 0 ? ident() : op(ri->second->decl[ro], rt != 0);
      need(!(p.l.identity && p.r.identity), "identity x identity term: use ecore");
      sb.terms.push_back(p);
    }
    ctx->eng->plan_sigma(sb, rec->plan);
    rec->psi = ctx->eng->alloc(sb.size);
    rec->sig = ctx->eng->alloc(sb.size);
    rec->orbsym = li->second->orbsym;
    rec->group = li->second->group;
    *psi_elems = sb.size;
    *sbh = ctx->next++;
    ctx->sbs[*sbh] = std::move(rec);
  });
}

int bgpu_superblock_free(bgpu_ctx* ctx, int sb) {
  return guarded(ctx, [&] {
    auto it = ctx->sbs.find(sb);
    need(it != ctx->sbs.end(), "bad superblock");
    ctx->eng->free_plan(it->second->plan);
    ctx->eng->free(it->second->psi);
    ctx->eng->free(it->second->sig);
    if (it->second->ownL) ctx->eng->release_block(*it->second->ownL);
    if (it->second->ownR) ctx->eng->release_block(*it->second->ownR);
    ctx->sbs.erase(it);
  });
}

int bgpu_superblock_work(bgpu_ctx* ctx, int sb, double* flops, double* bytes) {
  return guarded(ctx, [&] {
    auto it = ctx->sbs.find(sb);
    need(it != ctx->sbs.end(), "bad superblock");
    if (flops) *flops = it->second->plan.flops;
    if (bytes) *bytes = it->second->plan.bytes;
  });
}

int bgpu_sigma(bgpu_ctx* ctx, int sb, const double* psi, double* sigma) {
  return guarded(ctx, [&] {
    auto it = ctx->sbs.find(sb);
    need(it != ctx->sbs.end() && psi && sigma, "bad arguments");
    auto& r = *it->second;
    const int64_t n = r.sb.size;
    cuda_check(cudaMemcpyAsync(r.psi, psi, n * sizeof(double), cudaMemcpyHostToDevice, ctx->eng->stream()), "h2d");
    ctx->eng->sigma_any(r.sb, r.plan, r.psi, r.sig);
    cuda_check(cudaMemcpyAsync(sigma, r.sig, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->eng->stream()), "d2h");
    ctx->eng->sync();
  });
}

int bgpu_host_alloc(bgpu_ctx* ctx, int64_t n, double** p) {
  return guarded(ctx, [&] {
    need(p && n > 0, "bad arguments");
    need(ctx->eng != nullptr, "no device");
    *p = nullptr;
    cuda_check(cudaMallocHost((void**)p, (size_t)n * sizeof(double)), "page-locked host buffer");
  });
}

int bgpu_host_free(bgpu_ctx* ctx, double* p) {
  return guarded(ctx, [&] {
    if (p) cuda_check(cudaFreeHost(p), "free page-locked host buffer");
  });
}

int bgpu_sigma_device(bgpu_ctx* ctx, int sb, const double* psi, double* sigma) {
  return guarded(ctx, [&] {
    auto it = ctx->sbs.find(sb);
    need(it != ctx->sbs.end() && psi && sigma, "bad arguments");
    ctx->eng->sigma_any(it->second->sb, it->second->plan, psi, sigma);
  });
}

int bgpu_sigma_timed(bgpu_ctx* ctx, int sb, const double* psi, double* sigma, int reps, double* ms) {
  return guarded(ctx, [&] {
    auto it = ctx->sbs.find(sb);
    need(it != ctx->sbs.end() && psi && sigma && ms && reps > 0, "bad arguments");
    float t[3] = {0, 0, 0};
    ctx->eng->sigma_timed(it->second->sb, it->second->plan, psi, sigma, reps, t);
    for (int i = 0; i < 3; ++i) ms[i] = t[i];
  });
}

int bgpu_tc_wait_selftest(bgpu_ctx* ctx, double limit_ms, int* gave_up, int* status, double* waited_ms) {
  return guarded(ctx, [&] {
    need(limit_ms > 0 && limit_ms <= 1000 && gave_up && status && waited_ms, "bad arguments");
    cudaStream_t s = ctx->eng->stream();
    int* st = nullptr;
    unsigned long long* out = nullptr;
    cuda_check(cudaMallocAsync((void**)&st, sizeof(int), s), "alloc");
    cuda_check(cudaMallocAsync((void**)&out, 2 * sizeof(unsigned long long), s), "alloc");
    cuda_check(cudaMemsetAsync(st, 0, sizeof(int), s), "memset");
    cuda_check(dev::launch_tc_wait_selftest(st, out, (uint64_t)(limit_ms * 1e6), s), "wait selftest");
    unsigned long long h[2] = {0, 0};
    cuda_check(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, s), "d2h");
    cuda_check(cudaMemcpyAsync(status, st, sizeof(int), cudaMemcpyDeviceToHost, s), "d2h");
    cudaFreeAsync(st, s);
    cudaFreeAsync(out, s);
    ctx->eng->sync();
    *gave_up = (int)h[0];
    *waited_ms = (double)h[1] * 1e-6;
  });
}

int bgpu_superblock_info(bgpu_ctx* ctx, int sb, double* info, int n) {
  return guarded(ctx, [&] {
    auto it = ctx->sbs.find(sb);
    need(it != ctx->sbs.end() && info && n >= 0, "bad arguments");
    auto& r = *it->second;
    if (!r.plan.tc) ctx->eng->plan_tc(r.sb, r.plan);
    const SigmaPlan& p = r.plan;
    const double v[24] = {p.flops,
                          p.bytes,
                          p.tc_mma_flops,
                          (double)p.tc_stats[0],
                          (double)p.tc_stats[1],
                          (double)p.tc_stats[2],
                          (double)p.tc_stats[3],
                          (double)p.tc_stats[4],
                          (double)p.tc_pool_elems[dev::kTcPoolL],
                          (double)p.tc_pool_elems[dev::kTcPoolR],
                          (double)p.tc_pool_elems[dev::kTcPoolPsi],
                          (double)p.tc_pool_elems[dev::kTcPoolS],
                          (double)p.nstage1_units,
                          (double)p.nitems,
                          p.tc_knobs.item_cost,
                          p.tc_knobs.split,
                          (double)p.tc_knobs.group,
                          (double)p.tc_knobs.per_sector,
                          p.tc_tuned ? 1.0 : 0.0,
                          (double)ctx->eng->sigma_launches(p),
                          (double)p.scratch_elems,
                          (double)p.tc_nb,
                          (double)p.tc_stacks,
                          (double)p.tc_stacked_items};
    for (int i = 0; i < n; ++i) info[i] = i < 24 ? v[i] : 0.0;
  });
}

int bgpu_superblock_launches(bgpu_ctx* ctx, int sb, int* launches) {
  return guarded(ctx, [&] {
    auto it = ctx->sbs.find(sb);
    need(it != ctx->sbs.end() && launches, "bad arguments");
    *launches = ctx->eng->sigma_launches(it->second->plan);
  });
}

int bgpu_hdiag(bgpu_ctx* ctx, int sb, double* diag) {
  return guarded(ctx, [&] {
    auto it = ctx->sbs.find(sb);
    need(it != ctx->sbs.end() && diag, "bad arguments");
    auto& r = *it->second;
    ctx->eng->hdiag(r.sb, r.plan, r.sig);
    cuda_check(cudaMemcpyAsync(diag, r.sig, r.sb.size * sizeof(double), cudaMemcpyDeviceToHost, ctx->eng->stream()),
               "d2h");
    ctx->eng->sync();
  });
}

int bgpu_davidson(bgpu_ctx* ctx, int sb, int nroots, double tol, int max_iter, double* energies, double* vectors,
                  int* iterations) {
  return guarded(ctx, [&] {
    auto it = ctx->sbs.find(sb);
    need(it != ctx->sbs.end() && energies && nroots > 0, "bad arguments");
    DavidsonParams p;
    p.nroots = nroots;
    p.tol = tol;
    p.max_iter = max_iter > 0 ? max_iter : 200;
    p.deflation_min = std::max(2, nroots);
    p.deflation_max = std::max(20, nroots + 20);
    if (p.deflation_max + 1 > 32) p.deflation_max = 31;
    std::vector<double> e;
    const int iters = ctx->eng->solve(it->second->sb, p, e);
    for (int r = 0; r < nroots; ++r) energies[r] = e[r];
    if (vectors)
      cuda_check(cudaMemcpyAsync(vectors, ctx->eng->waves(), (size_t)nroots * it->second->sb.size * sizeof(double),
                                 cudaMemcpyDeviceToHost, ctx->eng->stream()),
                 "d2h");
    ctx->eng->sync();
    if (iterations) *iterations = iters;
  });
}

int bgpu_density_eig(bgpu_ctx* ctx, int sb, int left, int nroots, const double* weights, double* eig, int64_t n) {
  return guarded(ctx, [&] {
    auto it = ctx->sbs.find(sb);
    need(it != ctx->sbs.end() && eig, "bad arguments");
    const Block& B = left ? *it->second->sb.L : *it->second->sb.R;
    need(n == B.si.total_states(), "eigenvalue buffer size must equal the block's states");
    std::vector<double> w(weights ? weights : nullptr, weights ? weights + nroots : nullptr);
    DensitySpectrum spec;
    NoiseSpec ns = ctx->density_noise;
    if (ns.any()) {
      ns.orbsym = it->second->orbsym;
      ns.group = PointGroup::from_name(it->second->group);
    }
    ctx->eng->set_noise(ns);
    try {
      ctx->eng->density(it->second->sb, left != 0, w, spec);
    } catch (...) {
      ctx->eng->set_noise(NoiseSpec{});
      throw;
    }
    ctx->eng->set_noise(NoiseSpec{});
    int64_t o = 0;
    for (auto& v : spec.eig)
      for (double x : v) eig[o++] = x;
  });
}

int bgpu_set_density_noise(bgpu_ctx* ctx, double perturbative, double random, uint64_t seed) {
  return guarded(ctx, [&] {
    need(perturbative >= 0.0 && random >= 0.0, "noise amplitudes must be >= 0");
    ctx->density_noise = NoiseSpec{};
    ctx->density_noise.perturbative = perturbative;
    ctx->density_noise.random = random;
    ctx->density_noise.seed = seed;
  });
}

int bgpu_device_alloc(bgpu_ctx* ctx, int64_t n, double** p) {
  return guarded(ctx, [&] {
    need(p && n > 0, "bad arguments");
    *p = ctx->eng->alloc(n);
    ctx->eng->sync();
  });
}
int bgpu_device_free(bgpu_ctx* ctx, double* p) {
  return guarded(ctx, [&] {
    ctx->eng->free(p);
    ctx->eng->sync();
  });
}
int bgpu_copy_to_device(bgpu_ctx* ctx, double* dst, const double* src, int64_t n) {
  return guarded(ctx, [&] {
    cuda_check(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, ctx->eng->stream()), "h2d");
  });
}
int bgpu_copy_to_host(bgpu_ctx* ctx, double* dst, const double* src, int64_t n) {
  return guarded(ctx, [&] {
    cuda_check(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->eng->stream()), "d2h");
    ctx->eng->sync();
  });
}
int bgpu_synchronize(bgpu_ctx* ctx) {
  return guarded(ctx, [&] { ctx->eng->sync(); });
}

int bgpu_profiler_start(bgpu_ctx* ctx) {
  return guarded(ctx, [&] {
    ctx->eng->sync();
    cuda_check(cudaProfilerStart(), "cudaProfilerStart");
  });
}

int bgpu_profiler_stop(bgpu_ctx* ctx) {
  return guarded(ctx, [&] {
    ctx->eng->sync();
    cuda_check(cudaProfilerStop(), "cudaProfilerStop");
  });
}

int bgpu_tc_tile(bgpu_ctx* ctx, const uint16_t* a, const uint16_t* b, float* d, int n, int k, int packed) {
  return guarded(ctx, [&] {
    if (n < 16 || n > 256 || n % 16 || k < 16 || k > (packed ? 256 : 64) || k % 16)
      throw std::runtime_error("bgpu_tc_tile: need 16 <= n <= 256 and 16 <= k <= 64 (256 packed), multiples of 16");
    cudaStream_t s = ctx->eng->stream();
    __nv_bfloat16 *da = nullptr, *db = nullptr;
    float* dd = nullptr;
    int* st = nullptr;
    cuda_check(cudaMallocAsync((void**)&da, (size_t)128 * k * 2, s), "alloc");
    cuda_check(cudaMallocAsync((void**)&db, (size_t)n * k * 2, s), "alloc");
    cuda_check(cudaMallocAsync((void**)&dd, (size_t)128 * n * 4, s), "alloc");
    cuda_check(cudaMallocAsync((void**)&st, sizeof(int), s), "alloc");
    cuda_check(cudaMemsetAsync(st, 0, sizeof(int), s), "memset");
    cuda_check(cudaMemcpyAsync(da, a, (size_t)128 * k * 2, cudaMemcpyHostToDevice, s), "h2d");
    cuda_check(cudaMemcpyAsync(db, b, (size_t)n * k * 2, cudaMemcpyHostToDevice, s), "h2d");
    if (packed)
      cuda_check(dev::launch_tc_tile_bulk(da, db, dd, n, k, st, s), "tc tile bulk");
    else
      cuda_check(dev::launch_tc_tile(da, db, dd, n, k, st, s), "tc tile");
    int hst = 0;
    cuda_check(cudaMemcpyAsync(d, dd, (size_t)128 * n * 4, cudaMemcpyDeviceToHost, s), "d2h");
    cuda_check(cudaMemcpyAsync(&hst, st, sizeof(int), cudaMemcpyDeviceToHost, s), "d2h");
    for (void* p : {(void*)da, (void*)db, (void*)dd, (void*)st}) cudaFreeAsync(p, s);
    ctx->eng->sync();
    if (hst) throw std::runtime_error("bgpu_tc_tile: MMA completion wait ran out");
  });
}

int bgpu_integrals_load(bgpu_ctx* ctx, const char* conf_path, int* handle, int* norb) {
  return guarded(ctx, [&] {
    need(conf_path && handle, "null argument");
    Config c = parse_config(conf_path);
    auto I = std::make_unique<Integrals>(load_integrals(c));
    if (norb) *norb = I->norb;
    *handle = ctx->next++;
    ctx->integrals[*handle] = std::move(I);
  });
}

int bgpu_integrals_define(bgpu_ctx* ctx, int norb, const int* orbsym, const double* h1, const double* eri, double ecore,
                          int* handle) {
  return guarded(ctx, [&] {
    need(norb > 0 && orbsym && h1 && eri && handle, "null argument");
    auto I = std::make_unique<Integrals>();
    I->resize(norb);
    I->orbsym.assign(orbsym, orbsym + norb);
    I->ecore = ecore;
    std::copy(h1, h1 + (size_t)norb * norb, I->t.begin());
    std::copy(eri, eri + (size_t)norb * norb * norb * norb, I->v.begin());
    *handle = ctx->next++;
    ctx->integrals[*handle] = std::move(I);
  });
}

int bgpu_integrals_free(bgpu_ctx* ctx, int handle) {
  return guarded(ctx, [&] { need(ctx->integrals.erase(handle) == 1, "bad integrals handle"); });
}

int bgpu_block_set_sites(bgpu_ctx* ctx, int handle, int nsites, const int* sites) {
  return guarded(ctx, [&] {
    auto it = ctx->blocks.find(handle);
    need(it != ctx->blocks.end(), "bad block");
    need(nsites > 0 && sites, "null argument");
    const int norb = (int)it->second->orbsym.size();
    for (int i = 0; i < nsites; ++i) need(sites[i] >= 0 && sites[i] < norb, "site out of range");
    it->second->b.sites.assign(sites, sites + nsites);
  });
}

int bgpu_block_quanta(bgpu_ctx* ctx, int handle, int* nquanta, int* quanta, int* states) {
  return guarded(ctx, [&] {
    auto it = ctx->blocks.find(handle);
    need(it != ctx->blocks.end() && nquanta, "bad block");
    const StateInfo& si = it->second->b.si;
    const int cap = *nquanta;
    *nquanta = si.size();
    if (!quanta && !states) return;
    need(cap >= si.size(), "quanta buffers smaller than the block's quanta");
    for (int q = 0; q < si.size(); ++q) {
      if (quanta) {
        quanta[3 * q] = si.quanta[q].n;
        quanta[3 * q + 1] = si.quanta[q].s2;
        quanta[3 * q + 2] = si.quanta[q].irrep;
      }
      if (states) states[q] = si.states[q];
    }
  });
}

int bgpu_build_enlarged_ops(bgpu_ctx* ctx, int integrals, int left, int right, const int* filter, int nops,
                            const int* op_keys, int* big, int64_t* arena_elems, int* nquanta) {
  return guarded(ctx, [&] {
    auto ii = ctx->integrals.find(integrals);
    need(ii != ctx->integrals.end(), "bad integrals handle");
    auto li = ctx->blocks.find(left), ri = ctx->blocks.find(right);
    need(li != ctx->blocks.end() && ri != ctx->blocks.end(), "bad block handle");
    need(big && arena_elems && (nops == 0 || op_keys), "null argument");
    const Integrals& I = *ii->second;
    const auto& A = *li->second;
    const auto& B = *ri->second;
    need(!A.b.sites.empty() && !B.b.sites.empty(), "sub-blocks need their sites (bgpu_block_set_sites)");
    need(A.filled && B.filled, "sub-blocks need their operators (bgpu_block_upload)");
    need(A.b.is_dot || B.b.is_dot, "one sub-block must be a single site (is_dot)");
    need((int)A.orbsym.size() == I.norb && A.orbsym == B.orbsym, "orbital irreps of the blocks and integrals differ");
    need(A.group == B.group, "point groups of the sub-blocks differ");
    auto rec = std::make_unique<bgpu_ctx::BlockRec>();
    rec->orbsym = A.orbsym;
    rec->group = A.group;
    PointGroup g = PointGroup::from_name(rec->group);
    Block& nb = rec->b;
    nb.sites = A.b.sites;
    nb.sites.insert(nb.sites.end(), B.b.sites.begin(), B.b.sites.end());
    QuantumFilter qf;
    if (filter) {
      qf.nelec = filter[0];
      qf.s2 = filter[1];
      qf.norb = filter[2];
      need(qf.norb >= (int)nb.sites.size() && qf.nelec >= 0 && qf.s2 >= 0, "bad filter");
    }
    nb.si = product_stateinfo(A.b.si, B.b.si, g, filter ? &qf : nullptr, (int)nb.sites.size(), nullptr);
    need(nb.si.size() > 0, "the product keeps no quantum");
    std::set<OpKey> keys = read_keys(nops, op_keys, I.norb, rec->decl);
    nb.ops = make_opset(nb.si, keys, rec->orbsym, g);
    std::vector<std::pair<OpKey, std::vector<BuildTerm>>> recipes;
    for (const auto& kv : nb.ops.ops) {
      recipes.push_back({kv.first, build_terms(kv.first, A.b.sites, B.b.sites, I)});
      for (const auto& t : recipes.back().second) {
        need(t.a.identity || A.b.ops.has(t.a.key),
             "build of " + kv.first.str() + " needs " + t.a.key.str() + " on the left sub-block");
        need(t.b.identity || B.b.ops.has(t.b.key),
             "build of " + kv.first.str() + " needs " + t.b.key.str() + " on the right sub-block");
      }
    }
    ctx->eng->create_block(nb);
    ctx->eng->build_block(nb, A.b, B.b, recipes);
    ctx->eng->sync();
    rec->filled = true;
    *arena_elems = nb.ops.arena;
    if (nquanta) *nquanta = nb.si.size();
    *big = ctx->next++;
    ctx->blocks[*big] = std::move(rec);
  });
}

int bgpu_diagonalise(bgpu_ctx* ctx, int nmat, const int* dims, const double* a, double* eigvals, double* eigvecs) {
  return guarded(ctx, [&] {
    need(ctx->eng != nullptr, "no device");
    need(nmat > 0 && dims && a && eigvals, "null argument");
    std::vector<int> d(dims, dims + nmat);
    std::vector<int64_t> aoff(nmat), woff(nmat);
    int64_t ta = 0, tw = 0;
    for (int j = 0; j < nmat; ++j) {
      need(d[j] >= 1 && d[j] <= dev::kEigMaxN, "matrix order out of range (1 .. 4096)");
      aoff[j] = ta;
      woff[j] = tw;
      ta += (int64_t)d[j] * d[j];
      tw += d[j];
    }
    GpuEngine& e = *ctx->eng;
    double* da = e.alloc(ta);
    double* dz = e.alloc(ta);
    double* dw = e.alloc(tw);
    cuda_check(cudaMemcpyAsync(da, a, ta * sizeof(double), cudaMemcpyHostToDevice, e.stream()), "h2d");
    int* st = e.eigh_batched(d, da, aoff, /*copy_inputs=*/false, dz, aoff, dw, woff);
    std::vector<int> hs(nmat);
    std::vector<double> z(eigvecs ? ta : 0);
    cuda_check(cudaMemcpyAsync(eigvals, dw, tw * sizeof(double), cudaMemcpyDeviceToHost, e.stream()), "d2h");
    if (eigvecs) cuda_check(cudaMemcpyAsync(z.data(), dz, ta * sizeof(double), cudaMemcpyDeviceToHost, e.stream()), "d2h");
    cuda_check(cudaMemcpyAsync(hs.data(), st, nmat * sizeof(int), cudaMemcpyDeviceToHost, e.stream()), "d2h");
    e.sync();
    cudaFreeAsync(st, e.stream());
    e.free(da);
    e.free(dz);
    e.free(dw);
    for (int j = 0; j < nmat; ++j)
      if (hs[j] < 0) throw std::runtime_error("bgpu_diagonalise: tridiagonal solver did not converge for matrix " +
                                              std::to_string(j));
    if (eigvecs)  // column-major per matrix -> row-major with the eigenvectors as columns
      for (int j = 0; j < nmat; ++j) {
        const int n = d[j];
        const double* src = z.data() + aoff[j];
        double* dst = eigvecs + aoff[j];
        for (int r = 0; r < n; ++r)
          for (int c = 0; c < n; ++c) dst[(int64_t)r * n + c] = src[(int64_t)c * n + r];
      }
  });
}

int bgpu_set_wavefunctions(bgpu_ctx* ctx, int sb, int nroots, const double* vectors) {
  return guarded(ctx, [&] {
    auto it = ctx->sbs.find(sb);
    need(it != ctx->sbs.end() && vectors && nroots > 0, "bad arguments");
    ctx->eng->set_waves(nroots, it->second->sb.size, vectors);
  });
}

int bgpu_density_download(bgpu_ctx* ctx, double* rho, double* vecs, int64_t n) {
  return guarded(ctx, [&] {
    need(rho || vecs, "null argument");
    std::vector<double> r, v;
    ctx->eng->density_download(r, v);
    need(n == (int64_t)r.size(), "buffer size must be the sum of the squared sector sizes (" +
                                     std::to_string(r.size()) + ")");
    if (rho) std::copy(r.begin(), r.end(), rho);
    if (vecs) std::copy(v.begin(), v.end(), vecs);
  });
}

int bgpu_renormalise(bgpu_ctx* ctx, int big, const int* kept, const double* rotations, int nops, const int* op_keys,
                     int* small, int64_t* arena_elems, int* nquanta) {
  return guarded(ctx, [&] {
    auto bi = ctx->blocks.find(big);
    need(bi != ctx->blocks.end(), "bad block handle");
    need(kept && small && arena_elems && (nops == 0 || op_keys), "null argument");
    const auto& B = *bi->second;
    need(B.filled, "the block has no operators yet (bgpu_block_upload or bgpu_build_enlarged_ops)");
    const StateInfo& si = B.b.si;
    const int nq = si.size();
    std::vector<int> k(kept, kept + nq);
    int64_t total = 0;
    for (int q = 0; q < nq; ++q) {
      need(k[q] >= 0 && k[q] <= si.states[q], "kept states out of range");
      total += k[q];
    }
    need(total > 0, "no state kept");
    if (rotations) {
      std::vector<std::vector<double>> rot(nq);
      int64_t o = 0;
      for (int q = 0; q < nq; ++q) {
        const int64_t sz = (int64_t)si.states[q] * k[q];
        rot[q].assign(rotations + o, rotations + o + sz);
        o += sz;
      }
      ctx->eng->set_rotation(rot, k);
    } else {
      need(ctx->eng->density_dims() == si.states,
           "no density matrix of this block: call bgpu_density_eig first or pass rotations");
      std::vector<std::vector<int>> idx(nq);
      for (int q = 0; q < nq; ++q)
        for (int c = 0; c < k[q]; ++c) idx[q].push_back(si.states[q] - 1 - c);  // descending eigenvalues
      ctx->eng->select_rotation(idx);
    }
    auto rec = std::make_unique<bgpu_ctx::BlockRec>();
    rec->orbsym = B.orbsym;
    rec->group = B.group;
    PointGroup g = PointGroup::from_name(rec->group);
    Block& nb = rec->b;
    nb.sites = B.b.sites;
    std::vector<int> map;
    nb.si = truncated_stateinfo(si, k, map);
    std::set<OpKey> keys = read_keys(nops, op_keys, (int)rec->orbsym.size(), rec->decl);
    for (const OpKey& key : keys) need(B.b.ops.has(key), "the enlarged block has no operator " + key.str());
    nb.ops = make_opset(nb.si, keys, rec->orbsym, g);
    ctx->eng->create_block(nb);
    ctx->eng->renormalise(nb, B.b);
    ctx->eng->sync();
    rec->filled = true;
    *arena_elems = nb.ops.arena;
    if (nquanta) *nquanta = nb.si.size();
    *small = ctx->next++;
    ctx->blocks[*small] = std::move(rec);
  });
}

int bgpu_rotation_download(bgpu_ctx* ctx, int small, double* rot, int64_t n) {
  return guarded(ctx, [&] {
    auto it = ctx->blocks.find(small);
    need(it != ctx->blocks.end() && rot, "bad arguments");
    RotationRecord r;
    need(ctx->eng->get_rotation_record(it->second->b, r), "the block was not made by bgpu_renormalise");
    int64_t tot = 0;
    for (size_t q = 0; q < r.off.size(); ++q) tot += (int64_t)r.n[q] * r.m[q];
    need(n == tot, "buffer size must be the sum of rows x kept over the sectors (" + std::to_string(tot) + ")");
    int64_t o = 0;
    for (size_t q = 0; q < r.off.size(); ++q) {
      const int64_t sz = (int64_t)r.n[q] * r.m[q];
      std::copy(r.data.begin() + r.off[q], r.data.begin() + r.off[q] + sz, rot + o);
      o += sz;
    }
  });
}

int bgpu_prepare_superblock(bgpu_ctx* ctx, const char* conf_path, int partition, int* sbh, int64_t* psi_elems) {
  return guarded(ctx, [&] {
    need(conf_path && sbh && psi_elems, "null argument");
    Config c = parse_config(conf_path);
    Integrals I = load_integrals(c);
    need(partition >= 1 && partition <= I.norb - 3, "partition out of range");
    auto rec = std::make_unique<bgpu_ctx::SbRec>();
    rec->drv = std::make_unique<SweepDriver>(I, c, *ctx->eng);
    rec->ownL = std::make_unique<Block>();
    rec->ownR = std::make_unique<Block>();
    rec->sb = rec->drv->prepare_partition(partition, *rec->ownL, *rec->ownR);
    rec->sb.L = rec->ownL.get();
    rec->sb.R = rec->ownR.get();
    rec->drv.reset();  // warm-up blocks are no longer needed
    rec->orbsym = I.orbsym;
    rec->group = c.sym;
    ctx->eng->plan_sigma(rec->sb, rec->plan);
    rec->psi = ctx->eng->alloc(rec->sb.size);
    rec->sig = ctx->eng->alloc(rec->sb.size);
    *psi_elems = rec->sb.size;
    *sbh = ctx->next++;
    ctx->sbs[*sbh] = std::move(rec);
  });
}

int bgpu_run_dmrg(bgpu_ctx* ctx, const char* conf_path, int verbose, double* energies, int max_roots,
                  double* stats) {
  return guarded(ctx, [&] {
    need(conf_path && energies && max_roots > 0, "bad arguments");
    ctx->onepdm.clear();  // results of a run that fails are not kept
    ctx->tonepdm.clear();
    ctx->sweep_energies.clear();
    auto t0 = std::chrono::steady_clock::now();
    Config c = parse_config(conf_path);
    Integrals I = load_integrals(c);
    DriverOptions opt;
    opt.verbose = verbose;
    if (precision_slices(ctx->eng->precision) && ctx->eng->refine_mode == 0) {
      // energy-only refinement: deferred to the steps that may set the sweep energy
      opt.refine_window = ctx->refine_window;
      opt.deferred_steps = ctx->deferred_steps;
    }
    opt.transform_guess = ctx->transform_guess;
    opt.spill = ctx->spill;
    const double s0 = ctx->eng->sigma_seconds, f0 = ctx->eng->sigma_flops, p0 = ctx->eng->plan_seconds;
    const double d0 = ctx->eng->renorm_device_seconds;
    const long c0 = ctx->eng->sigma_calls;
    GpuEngine& E = *ctx->eng;
    const long sc0 = E.split_calls, fc0 = E.fp64_calls, dr0 = E.defect_rounds_, db0 = E.defect_bounded_,
               xc0 = E.exact_calls;
    const double xs0 = E.exact_seconds;
    const double ss0 = E.split_seconds, fs0 = E.fp64_seconds, dv0 = E.derived_fp64_sigma_seconds;
    SweepResult r;
    {
      SweepDriver drv(I, c, *ctx->eng, opt);
      r = drv.run();
    }
    ctx->eng->sync();  // the last renormalisation and block releases
    ctx->sweep_energies = r.sweep_energies;
    ctx->onepdm = r.onepdm;
    ctx->tonepdm = r.transition_onepdm;
    ctx->run_stats = {(double)(E.split_calls - sc0), E.split_seconds - ss0, (double)(E.fp64_calls - fc0),
                      E.fp64_seconds - fs0, (double)(E.defect_rounds_ - dr0), E.derived_fp64_sigma_seconds - dv0,
                      r.warmup_seconds, (double)(E.defect_bounded_ - db0), (double)(E.exact_calls - xc0),
                      E.exact_seconds - xs0, r.sweep_renorm_flops, E.fp64_rate_, (double)E.renorm_exact(),
                      r.sweep_renorm_device_seconds, (double)r.spill_fetches, r.spill_bytes_up,
                      r.spill_bytes_down, r.peak_block_bytes};
    for (double t : r.sweep_seconds) ctx->run_stats.push_back(t);
    for (int i = 0; i < max_roots && i < (int)r.energies.size(); ++i) energies[i] = r.energies[i];
    if (stats) {
      stats[0] = r.sweeps;
      stats[1] = (double)(ctx->eng->sigma_calls - c0);
      stats[2] = ctx->eng->sigma_seconds - s0;
      stats[3] = ctx->eng->sigma_flops - f0;
      stats[4] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      stats[5] = r.discarded;
      stats[6] = r.sweep_energies.empty() ? 0.0 : r.sweep_energies.back();
      stats[7] = (double)r.energies.size();
      stats[8] = r.build_seconds;
      stats[9] = r.solve_seconds;
      stats[10] = r.density_seconds;
      stats[11] = ctx->eng->renorm_device_seconds - d0;
      stats[12] = ctx->eng->plan_seconds - p0;
    }
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free sigma (bgpu_sigma_noalloc).  The stage-1 intermediates go
// to a fixed device array instead of the superblock's scratch buffer.  Host
// code only ever sees the array's name as a host-side stand-in, never as a
// device address: its device address is looked up once per device with
// cudaGetSymbolAddress (with that device current) and passed to the kernels.
// ---------------------------------------------------------------------------
namespace {
static __device__ __align__(256) double g_noalloc_scratch[BGPU_NOALLOC_SCRATCH_DOUBLES];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on `device` (set-up on first use).
cudaError_t noalloc_scratch(int device, double** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) return e;
    if (cur != device && (e = cudaSetDevice(device)) != cudaSuccess) return e;
    double* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (cur != device) cudaSetDevice(cur);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[device] = p;
  }
  *out = g_noalloc_ptr[device];
  return cudaSuccess;
}
}  // namespace

extern "C" int bgpu_sigma_noalloc(bgpu_ctx* ctx, int sb, const double* psi, double* sigma) {
  return guarded(ctx, [&] {
    need(ctx->eng != nullptr, "no device");
    auto it = ctx->sbs.find(sb);
    need(it != ctx->sbs.end() && psi && sigma, "bad arguments");
    const SigmaPlan& plan = it->second->plan;
    if (plan.scratch_elems > (int64_t)BGPU_NOALLOC_SCRATCH_DOUBLES)
      throw std::invalid_argument("bgpu_sigma_noalloc: superblock needs " + std::to_string(plan.scratch_elems) +
                                  " doubles of intermediates, more than the fixed " +
                                  std::to_string((long long)BGPU_NOALLOC_SCRATCH_DOUBLES) +
                                  "; use bgpu_sigma_device");
    double* scratch = nullptr;
    cuda_check(noalloc_scratch(ctx->device, &scratch), "noalloc scratch address");
    // always the FP64 plan, whatever bgpu_set_precision chose: the split
    // paths keep packed operand pools that are allocated on first use
    ctx->eng->sigma_fp64(it->second->sb, plan, psi, sigma, scratch);
  });
}
