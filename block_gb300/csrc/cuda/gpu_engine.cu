// Host side of the CUDA engine: compiles the operator algebra of a sweep
// step into device work lists and drives the kernels of kernels.cu.
#include "gpu_engine.h"
#include "k_dc.cuh"
#include "k_noise.cuh"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "../host/dense.h"

#include <deque>
#include <functional>
#include <mutex>
#include <queue>
#include <set>
#include <unordered_map>

#include "../host/parallel.h"


namespace bgpu {

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// ------------------------------------------------------------------ staging
//
// A host-to-device copy from pageable memory waits for the stream, so every
// work-list upload would stall the host until the device caught up.  Uploads
// are therefore staged through a pinned ring buffer per stream: the data is
// copied into the ring, the device copy is queued behind the work already on
// the stream, and a ring region is reused only after the event recorded
// behind its copy has completed.  The host thus compiles the next step's
// work lists while the device still runs the current step.
namespace {
struct StageRing {
  char* ring = nullptr;
  size_t cap = 0, head = 0;
  struct Span {
    size_t beg, end;
    cudaEvent_t ev;
  };
  std::deque<Span> inflight;
  std::vector<cudaEvent_t> spare;
  void drain() {
    for (auto& sp : inflight) {
      cudaEventSynchronize(sp.ev);
      spare.push_back(sp.ev);
    }
    inflight.clear();
  }
};
std::mutex g_stage_mu;
std::map<cudaStream_t, StageRing> g_stage;
}  // namespace

cudaError_t stage_h2d(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return cudaSuccess;
  // block arenas (restarts) are copied directly: a ring for them would pin
  // several times their size
  constexpr size_t kStageMax = size_t(256) << 20;
  if (bytes > kStageMax) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
  std::lock_guard<std::mutex> lk(g_stage_mu);
  StageRing& st = g_stage[s];
  const size_t need = (bytes + 255) & ~(size_t)255;
  if (need > st.cap / 4) {  // the ring holds at least four of the largest copy
    st.drain();
    if (st.ring) cudaFreeHost(st.ring);
    st.ring = nullptr;
    st.cap = std::max<size_t>(size_t(64) << 20, 4 * need);
    st.head = 0;
    if (cudaMallocHost((void**)&st.ring, st.cap) != cudaSuccess) {
      cudaGetLastError();
      st.ring = nullptr;
      st.cap = 0;
      return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);  // unstaged
    }
  }
  size_t p = st.head;
  if (p + need > st.cap) p = 0;
  // wait for the newest copy still reading [p, p + need); copies on one
  // stream complete in order, so every older span is free as well
  int last = -1;
  for (int i = 0; i < (int)st.inflight.size(); ++i)
    if (st.inflight[i].beg < p + need && p < st.inflight[i].end) last = i;
  if (last >= 0) {
    cudaError_t e = cudaEventSynchronize(st.inflight[last].ev);
    if (e != cudaSuccess) return e;
    for (int i = 0; i <= last; ++i) {
      st.spare.push_back(st.inflight.front().ev);
      st.inflight.pop_front();
    }
  }
  std::memcpy(st.ring + p, src, bytes);
  cudaError_t e = cudaMemcpyAsync(dst, st.ring + p, bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  cudaEvent_t ev;
  if (!st.spare.empty()) {
    ev = st.spare.back();
    st.spare.pop_back();
  } else if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) {
    return e;
  }
  if ((e = cudaEventRecord(ev, s)) != cudaSuccess) return e;
  st.inflight.push_back({p, p + need, ev});
  st.head = p + need;
  return cudaSuccess;
}

void release_staging(cudaStream_t s) {
  std::lock_guard<std::mutex> lk(g_stage_mu);
  auto it = g_stage.find(s);
  if (it == g_stage.end()) return;
  it->second.drain();
  for (cudaEvent_t ev : it->second.spare) cudaEventDestroy(ev);
  if (it->second.ring) cudaFreeHost(it->second.ring);
  g_stage.erase(it);
}

template <class T>
void DevArray<T>::upload(const std::vector<T>& h, cudaStream_t s) {
  release(s);
  n = h.size();
  if (n == 0) return;
  cuda_check(cudaMallocAsync((void**)&d, n * sizeof(T), s), "cudaMallocAsync(desc)");
  cuda_check(stage_h2d(d, h.data(), n * sizeof(T), s), "upload desc");
}
template <class T>
void DevArray<T>::release(cudaStream_t s) {
  if (d) cudaFreeAsync(d, s);
  d = nullptr;
  n = 0;
}

GpuEngine::GpuEngine(int device) : device_(device) {
  cuda_check(cudaSetDevice(device_), "cudaSetDevice");
  cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
  cudaMemPool_t pool;
  cuda_check(cudaDeviceGetDefaultMemPool(&pool, device_), "mempool");
  uint64_t thr = UINT64_MAX;
  cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  cuda_check(cudaEventCreate(&ev0_), "event");
  cuda_check(cudaEventCreate(&ev1_), "event");
  cuda_check(cudaMalloc((void**)&tc_status_, sizeof(int)), "alloc status");
  cuda_check(cudaMemset(tc_status_, 0, sizeof(int)), "memset status");
  cuda_check(cudaMallocHost((void**)&tc_status_host_, sizeof(int)), "alloc status");
  *tc_status_host_ = 0;
  cuda_check(cudaMallocHost((void**)&dav_host_, sizeof(dev::DavCtl)), "alloc davidson header");
  const char* g = std::getenv("BGPU_DAVIDSON_GRAPH");
  dav_graph = !(g && g[0] == '0');
  const char* at = std::getenv("BGPU_AUTOTUNE");
  tc_autotune = at && at[0] == '1';
  const char* tcp = std::getenv("BGPU_TUNE_CACHE");
  if (tcp && *tcp) load_tune_cache(tcp);
}

GpuEngine::~GpuEngine() {
  if (have_plan_) free_plan(plan_);
  for (auto& kv : blocks_)
    if (kv.second.d) cudaFreeAsync(kv.second.d, stream_);
  if (waves_) cudaFreeAsync(waves_, stream_);
  if (dm_vecs_) cudaFreeAsync(dm_vecs_, stream_);
  if (dm_rho_) cudaFreeAsync(dm_rho_, stream_);
  if (rot_) cudaFreeAsync(rot_, stream_);
  for (auto& kv : block_rot_)
    if (kv.second.d) cudaFreeAsync(kv.second.d, stream_);
  for (auto& kv : parked_)
    if (kv.second.d) cudaFreeAsync(kv.second.d, stream_);
  if (guess_) cudaFreeAsync(guess_, stream_);
  for (auto* q : pool_cache_)
    if (q) cudaFreeAsync(q, stream_);
  cudaStreamSynchronize(stream_);
  release_staging(stream_);
  cudaEventDestroy(ev0_);
  cudaEventDestroy(ev1_);
  cudaFree(tc_status_);
  cudaFreeHost(tc_status_host_);
  cudaFreeHost(dav_host_);
  cudaStreamDestroy(stream_);
}

double* GpuEngine::alloc(int64_t elems) {
  double* p = nullptr;
  if (elems <= 0) elems = 1;
  cuda_check(cudaMallocAsync((void**)&p, (size_t)elems * sizeof(double), stream_), "cudaMallocAsync");
  return p;
}
void GpuEngine::free(double* p) {
  if (p) cudaFreeAsync(p, stream_);
}
void GpuEngine::sync() {
  cuda_check(cudaStreamSynchronize(stream_), "stream sync");
  for (auto& ev : pending_renorm_) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev.first, ev.second) == cudaSuccess) renorm_device_seconds += ms * 1e-3;
    cudaEventDestroy(ev.first);
    cudaEventDestroy(ev.second);
  }
  pending_renorm_.clear();
  if (*tc_status_host_) {
    *tc_status_host_ = 0;
    cudaMemset(tc_status_, 0, sizeof(int));
    throw std::runtime_error("tensor-core sigma: a pipeline wait ran out (results discarded)");
  }
}

void GpuEngine::create_block(Block& b) {
  b.handle = next_handle_++;
  DevBlock& d = blocks_[b.handle];
  d.n = b.ops.arena;
  d.d = alloc(d.n);
  d.dot = b.is_dot;
  block_bytes_ += 8 * d.n;
  cuda_check(cudaMemsetAsync(d.d, 0, (size_t)std::max<int64_t>(d.n, 1) * sizeof(double), stream_), "memset");
}

void GpuEngine::release_block(Block& b) {
  auto sl = slices_.find(b.handle);
  if (sl != slices_.end()) {
    for (auto* p : sl->second.s)
      if (p) cudaFreeAsync(p, stream_);
    slices_.erase(sl);
  }
  auto it = blocks_.find(b.handle);
  if (it != blocks_.end()) {
    free(it->second.d);
    block_bytes_ -= 8 * it->second.n;
    blocks_.erase(it);
  }
  auto rr = block_rot_.find(b.handle);
  if (rr != block_rot_.end()) {
    free(rr->second.d);
    block_rot_.erase(rr);
  }
  b.handle = -1;
}

void GpuEngine::upload_block(Block& b, const std::vector<double>& a) {
  DevBlock& d = blocks_.at(b.handle);
  if ((int64_t)a.size() != d.n) throw std::runtime_error("upload_block: size mismatch");
  cuda_check(stage_h2d(d.d, a.data(), a.size() * sizeof(double), stream_), "upload");
  if (b.is_dot || d.dot) d.host = a;
  sync();
}

void GpuEngine::download_block(const Block& b, std::vector<double>& a) {
  const DevBlock& d = blocks_.at(b.handle);
  a.resize(d.n);
  cuda_check(cudaMemcpyAsync(a.data(), d.d, a.size() * sizeof(double), cudaMemcpyDeviceToHost, stream_), "download");
  sync();
}

double* GpuEngine::arena(const Block& b) const { return blocks_.at(b.handle).d; }

int GpuEngine::sm_count() {
  if (sm_count_ <= 0) cuda_check(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device_), "sm count");
  return sm_count_;
}

// ------------------------------------------------------------------ views

namespace {
struct HostView {
  bool ok = false, identity = false, trans = false;
  int64_t off = 0;  // element offset of the stored block in its arena
  int rows = 0, cols = 0, ld = 0;
  double scale = 1.0;
};

HostView hview(const Block& B, const Operand& o, int bra, int ket) {
  HostView v;
  if (o.identity) {
    if (bra != ket) return v;
    v.ok = v.identity = true;
    v.rows = v.cols = B.si.states[bra];
    return v;
  }
  const OpEntry& e = B.ops.at(o.key);
  const OpLayout& L = B.ops.layouts[e.layout];
  if (!o.trans) {
    const int i = L.find(bra, ket);
    if (i < 0) return v;
    const OpBlock& b = L.blocks[i];
    v.ok = true;
    v.off = e.base + b.offset;
    v.rows = b.rows;
    v.cols = b.cols;
    v.ld = b.cols;
  } else {
    const int i = L.find(ket, bra);
    if (i < 0) return v;
    const OpBlock& b = L.blocks[i];
    v.ok = true;
    v.trans = true;
    v.off = e.base + b.offset;
    v.rows = b.cols;
    v.cols = b.rows;
    v.ld = b.cols;
    v.scale = transpose_scaling(B.si.quanta[bra].s2, B.si.quanta[ket].s2, o.key.k2);
  }
  return v;
}
inline int rank2(const Operand& o) { return o.identity ? 0 : o.key.k2; }
inline bool fermion(const Operand& o) { return !o.identity && op_fermion(o.key); }

// (bra, ket) pairs of the blocks of an operand view
void view_pairs(const Block& B, const Operand& o, std::vector<std::pair<int, int>>& out) {
  out.clear();
  if (o.identity) {
    for (int q = 0; q < B.si.size(); ++q) out.push_back({q, q});
    return;
  }
  const OpLayout& L = B.ops.layout_of(o.key);
  for (const OpBlock& b : L.blocks) out.push_back(o.trans ? std::make_pair(b.ket, b.bra) : std::make_pair(b.bra, b.ket));
}

// One TensorMultiply coupling of a pair term (operatorfunctions.C:506-533):
// sigma(lQ, rQ) += f * A(lQ, lQ') psi(lQ', rQ') B(rQ, rQ')^T
struct Coupling {
  int lQ, lQp, rQ, rQp, cs, vs;
  HostView va, vb;
  double f;
};

// Enumerates the couplings of `t`, driven by the operator's own block list.
template <class F>
void for_each_coupling(const Superblock& sb, const PairTerm& t, const std::vector<std::vector<std::pair<int, int>>>& by_l,
                       F&& fn) {
  const Block& L = *sb.L;
  const Block& R = *sb.R;
  const int J = sb.target.s2;
  const int kL = t.l.identity ? 0 : t.l.key.k2, kR = t.r.identity ? 0 : t.r.key.k2;
  const bool fR = !t.r.identity && op_fermion(t.r.key);
  std::vector<std::pair<int, int>> lp;
  view_pairs(L, t.l, lp);
  for (auto& pr : lp) {
    const int lQ = pr.first, lQp = pr.second;
    HostView va = hview(L, t.l, lQ, lQp);
    if (!va.ok) continue;
    for (auto& cp : by_l[lQp]) {
      const int rQp = cp.first, cs = cp.second;
      for (auto& vp : by_l[lQ]) {
        const int rQ = vp.first, vs = vp.second;
        HostView vb = hview(R, t.r, rQ, rQp);
        if (!vb.ok) continue;
        double f = t.coef * ninej(L.si.quanta[lQp].s2, R.si.quanta[rQp].s2, J, kL, kR, 0, L.si.quanta[lQ].s2,
                                  R.si.quanta[rQ].s2, J);
        if (fR && is_fermion(L.si.quanta[lQp])) f = -f;
        if (f == 0.0) continue;
        fn(Coupling{lQ, lQp, rQ, rQp, cs, vs, va, vb, f});
      }
    }
  }
}

std::vector<std::vector<std::pair<int, int>>> sectors_by_left(const Superblock& sb) {
  std::vector<std::vector<std::pair<int, int>>> by_l(sb.L->si.size());
  for (int s = 0; s < (int)sb.sectors.size(); ++s) by_l[sb.sectors[s].lq].push_back({sb.sectors[s].rq, s});
  return by_l;
}

double env_double(const char* name, double dflt) {
  const char* e = std::getenv(name);
  if (!e || !*e) return dflt;
  char* end = nullptr;
  const double v = std::strtod(e, &end);
  return (end && end != e && v > 0) ? v : dflt;
}

// Prints the host time of the stages of a plan compiler (BGPU_PLAN_TIMING=1).
struct PlanLaps {
  const char* name;
  bool on = env_double("BGPU_PLAN_TIMING", 0.0) > 0.5;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void lap(const char* what) {
    if (!on) return;
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "[plan %s] %-24s %8.1f ms\n", name, what,
                 std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
};

// adds the wall time of its scope to a counter
struct PlanTimer {
  double& acc;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  explicit PlanTimer(double& a) : acc(a) {}
  ~PlanTimer() { acc += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

// Longest-processing-time assignment of tasks to `nblocks` persistent
// blocks; block j runs order[ranges[j].x .. ranges[j].y), in task order.
// Tasks with the same bundle id (contiguous in task order; for instance the
// column tiles of one row of an output sector, which read the same A
// operands) stay together on one block, consecutive, unless a bundle costs
// more than a block's fair share, in which case it is cut into pieces of at
// most that share.
void schedule_lpt(const std::vector<double>& cost, const std::vector<int64_t>& bundle, int nblocks,
                  std::vector<int>& order, std::vector<int2>& ranges) {
  const int n = (int)cost.size();
  order.clear();
  ranges.clear();
  if (n == 0) return;
  nblocks = std::max(1, std::min(nblocks, n));
  double total = 0.0;
  for (double c : cost) total += c;
  const double share = total / nblocks;
  // units: contiguous task ranges
  std::vector<std::pair<int, int>> units;
  std::vector<double> ucost;
  int b0 = 0;
  double acc = 0.0;
  for (int i = 0; i < n; ++i) {
    const bool split = i > b0 && (bundle[i] != bundle[i - 1] || acc + cost[i] > share);
    if (split) {
      units.push_back({b0, i});
      ucost.push_back(acc);
      b0 = i;
      acc = 0.0;
    }
    acc += cost[i];
  }
  units.push_back({b0, n});
  ucost.push_back(acc);
  std::vector<int> idx(units.size());
  for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int)i;
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return ucost[a] > ucost[b]; });
  nblocks = std::max(1, std::min(nblocks, (int)units.size()));
  std::vector<std::vector<int>> per(nblocks);
  std::priority_queue<std::pair<double, int>, std::vector<std::pair<double, int>>, std::greater<>> load;
  for (int j = 0; j < nblocks; ++j) load.push({0.0, j});
  for (int u : idx) {
    auto [l, j] = load.top();
    load.pop();
    per[j].push_back(u);
    load.push({l + ucost[u], j});
  }
  for (auto& v : per) {
    std::sort(v.begin(), v.end());
    const int b = (int)order.size();
    for (int u : v)
      for (int i = units[u].first; i < units[u].second; ++i) order.push_back(i);
    ranges.push_back(make_int2(b, (int)order.size()));
  }
}

// Wave assignment: the tasks, in task order, cut into waves of `nblocks`;
// within a wave the longest-processing-time rule places each task (longest
// first) on the least-loaded block, so that all blocks work through the
// waves together; block j runs order[ranges[j].x .. ranges[j].y) in task
// order.
void schedule_waves(const std::vector<double>& cost, int nblocks, std::vector<int>& order,
                    std::vector<int2>& ranges) {
  const int n = (int)cost.size();
  order.clear();
  ranges.clear();
  if (n == 0) return;
  nblocks = std::max(1, std::min(nblocks, n));
  std::vector<std::vector<int>> per(nblocks);
  std::vector<double> load(nblocks, 0.0);
  std::vector<int> wave;
  for (int w0 = 0; w0 < n; w0 += nblocks) {
    const int w1 = std::min(n, w0 + nblocks);
    wave.clear();
    for (int i = w0; i < w1; ++i) wave.push_back(i);
    std::stable_sort(wave.begin(), wave.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::priority_queue<std::pair<double, int>, std::vector<std::pair<double, int>>, std::greater<>> q;
    for (int j = 0; j < nblocks; ++j) q.push({load[j], j});
    for (int i : wave) {
      auto [l, j] = q.top();
      q.pop();
      per[j].push_back(i);
      load[j] = l + cost[i];
      q.push({load[j], j});
    }
  }
  for (auto& v : per) {
    const int b = (int)order.size();
    for (int i : v) order.push_back(i);
    ranges.push_back(make_int2(b, (int)order.size()));
  }
}

void add_tasks(std::vector<dev::GemmTask>& t, int unit, int m, int n) {
  for (int a = 0; a < (m + 63) / 64; ++a)
    for (int b = 0; b < (n + 63) / 64; ++b) t.push_back({unit, a, b});
}
}  // namespace

// ------------------------------------------------------------------ build

void GpuEngine::build_block(Block& big, const Block& a, const Block& b,
                            const std::vector<std::pair<OpKey, std::vector<BuildTerm>>>& recipes) {
  const DevBlock& da = blocks_.at(a.handle);
  const DevBlock& db = blocks_.at(b.handle);
  // which factor is the single-site one whose values fold into the factors
  const bool a_scalar = da.dot && !db.dot;
  const bool b_scalar = !a_scalar;  // if both are dots, b folds
  if (b_scalar && !db.dot) throw std::runtime_error("build_block: one sub-block must be a single site");
  const DevBlock& dsc = a_scalar ? da : db;
  if ((int64_t)dsc.host.size() != dsc.n) throw std::runtime_error("build_block: the single-site block was never uploaded");
  // per recipe: rectangles keyed by (target block, row part, column part)
  struct Rect {
    int64_t key;
    dev::CopyUnit u;
    std::vector<dev::CopyItem> items;
    int64_t block_off;  // arena offset of the operator block
    int r0, c0;         // rectangle origin inside the block
  };
  std::vector<std::vector<Rect>> per(recipes.size());
  parallel_for((int)recipes.size(), [&](int ri) {
    const OpKey& tk = recipes[ri].first;
    const OpEntry& te = big.ops.at(tk);
    const OpLayout& TL = big.ops.layouts[te.layout];
    const int kC = tk.k2;
    std::unordered_map<int64_t, int> where;
    std::vector<Rect>& rects = per[ri];
    std::vector<std::pair<int, int>> ap, bp;
    for (const BuildTerm& t : recipes[ri].second) {
      view_pairs(a, t.a, ap);
      view_pairs(b, t.b, bp);
      for (auto& x : ap)
        for (auto& y : bp) {
          const auto& rows = big.si.parts_of(x.first, y.first);
          const auto& cols = big.si.parts_of(x.second, y.second);
          for (auto& rp : rows)
            for (auto& cp : cols) {
              const int tbi = TL.find(rp.first, cp.first);
              if (tbi < 0) continue;
              const OpBlock& tb = TL.blocks[tbi];
              const SectorPart& pr = big.si.parts[rp.first][rp.second];
              const SectorPart& pc = big.si.parts[cp.first][cp.second];
              HostView va = hview(a, t.a, pr.lq, pc.lq);
              HostView vb = hview(b, t.b, pr.rq, pc.rq);
              if (!va.ok || !vb.ok) continue;
              double f = t.coef * ninej(a.si.quanta[pc.lq].s2, b.si.quanta[pc.rq].s2, big.si.quanta[tb.ket].s2,
                                        rank2(t.a), rank2(t.b), kC, a.si.quanta[pr.lq].s2, b.si.quanta[pr.rq].s2,
                                        big.si.quanta[tb.bra].s2);
              if (fermion(t.b) && is_fermion(a.si.quanta[pc.lq])) f = -f;
              if (f == 0.0) continue;
              const HostView& vs = a_scalar ? va : vb;  // single-site factor
              const HostView& vg = a_scalar ? vb : va;  // factor copied from HBM
              if (!vs.identity) f *= vs.scale * dsc.host[vs.off];  // 1x1 block
              if (f == 0.0) continue;
              dev::CopyItem it{};
              it.alpha = f * (vg.identity ? 1.0 : vg.scale);
              it.trans = vg.trans ? 1 : 0;
              it.lds = vg.ld;
              it.s_off = vg.off;
              it.s_buf = vg.identity ? -1 : (a_scalar ? 1 : 0);
              const int64_t key = ((int64_t)tbi << 32) | ((int64_t)rp.second << 16) | (int64_t)cp.second;
              auto w = where.find(key);
              if (w == where.end()) {
                Rect r;
                r.key = key;
                r.u.c_off = te.base + tb.offset + (int64_t)pr.offset * tb.cols + pc.offset;
                r.u.ldc = tb.cols;
                r.u.m = pr.size;
                r.u.n = pc.size;
                r.block_off = te.base + tb.offset;
                r.r0 = pr.offset;
                r.c0 = pc.offset;
                where.emplace(key, (int)rects.size());
                rects.push_back(std::move(r));
                rects.back().items.push_back(it);
              } else {
                rects[w->second].items.push_back(it);
              }
            }
        }
    }
  });
  std::vector<dev::CopyUnit> units;
  std::vector<dev::CopyItem> items;
  DevBlock& dt = blocks_.at(big.handle);
  dt.nz.clear();
  for (auto& rv : per)
    for (auto& r : rv) {
      dev::CopyUnit u = r.u;
      u.ibeg = (int)items.size();
      items.insert(items.end(), r.items.begin(), r.items.end());
      u.iend = (int)items.size();
      units.push_back(u);
      dt.nz[r.block_off].push_back({r.r0, r.c0, r.u.m, r.u.n});
    }
  cuda_check(cudaMemsetAsync(dt.d, 0, (size_t)std::max<int64_t>(dt.n, 1) * sizeof(double), stream_), "memset");
  DevArray<dev::CopyUnit> du;
  DevArray<dev::CopyItem> di;
  du.upload(units, stream_);
  di.upload(items, stream_);
  dev::Bufs bufs{};
  bufs.p[0] = da.d;
  bufs.p[1] = db.d;
  cuda_check(dev::launch_copy(bufs, dt.d, du.d, di.d, (int)units.size(), stream_), "build copy");
  du.release(stream_);
  di.release(stream_);
  if (big.is_dot) {
    dt.host.resize(dt.n);
    cuda_check(cudaMemcpyAsync(dt.host.data(), dt.d, dt.n * sizeof(double), cudaMemcpyDeviceToHost, stream_), "d2h");
    sync();
  }
  // otherwise stream-ordered: the host goes on planning while the copies run
}

// ------------------------------------------------------------------ sigma

// Compiles TensorMultiply (operatorfunctions.C:485-537) over all operator
// pairs of SpinBlock::multiplyH into two grouped-GEMM launches:
//   stage 1: M[t,lQ,lQ',rQ'] = s_L * A(lQ,lQ') * psi(lQ',rQ')
//   stage 2: sigma(lQ,rQ) = sum over (t, rQ') of f * M * B(rQ,rQ')^T
// plus direct products for pairs with one identity factor.  Every output
// sector is owned by one unit (no atomics).
void GpuEngine::plan_sigma(const Superblock& sb, SigmaPlan& plan) {
  PlanTimer timer_(plan_seconds);
  PlanLaps laps{"fp64"};
  const Block& L = *sb.L;
  const Block& R = *sb.R;
  const int J = sb.target.s2;
  const auto by_l = sectors_by_left(sb);
  // buffers: 0 = L arena, 1 = R arena, 2 = psi, 3 = sigma, 4 = scratch
  std::vector<dev::GemmUnit> u1;
  std::vector<dev::GemmItem> i1;
  std::vector<std::vector<dev::GemmItem>> per_sector(sb.sectors.size());
  int64_t scratch = 0;
  double flops = 0.0, bytes = 0.0;
  std::set<std::pair<int, OpKey>> used;
  for (const PairTerm& t : sb.terms) {
    if (!t.l.identity && used.insert({0, t.l.key}).second) bytes += 8.0 * L.ops.layout_of(t.l.key).size;
    if (!t.r.identity && used.insert({1, t.r.key}).second) bytes += 8.0 * R.ops.layout_of(t.r.key).size;
    // group the couplings of a term by (lQ, lQ', rQ'): one stage-1 product each
    int cur_l = -1, cur_lp = -1, cur_rp = -1;
    int64_t cur_m = -1;
    for_each_coupling(sb, t, by_l, [&](const Coupling& c) {
      const auto& S = sb.sectors[c.cs];
      const auto& SV = sb.sectors[c.vs];
      const int mr = L.si.states[c.lQ], mc = R.si.states[c.rQp];
      if (c.va.identity && c.vb.identity) throw std::runtime_error("identity x identity pair term");
      if (c.va.identity) {
        // L identity: sigma(lQ,rQ) += f psi(lQ,rQ') B^T
        dev::GemmItem g{};
        g.a_buf = 2;
        g.a_off = S.offset;
        g.lda = S.cols;
        g.b_buf = 1;
        g.b_off = c.vb.off;
        g.ldb = c.vb.ld;
        g.tb = c.vb.trans ? 0 : 1;
        g.k = mc;
        g.alpha = c.f * c.vb.scale;
        per_sector[c.vs].push_back(g);
        flops += 2.0 * SV.rows * SV.cols * mc;
        return;
      }
      if (c.vb.identity) {
        // R identity: sigma(lQ,rQ') += f s_L A psi(lQ',rQ')
        dev::GemmItem g{};
        g.a_buf = 0;
        g.a_off = c.va.off;
        g.lda = c.va.ld;
        g.ta = c.va.trans ? 1 : 0;
        g.b_buf = 2;
        g.b_off = S.offset;
        g.ldb = S.cols;
        g.k = S.rows;
        g.alpha = c.f * c.va.scale;
        per_sector[c.vs].push_back(g);
        flops += 2.0 * mr * mc * S.rows;
        return;
      }
      if (!(c.lQ == cur_l && c.lQp == cur_lp && c.rQp == cur_rp)) {
        // stage 1: M = s_L A psi
        dev::GemmUnit u{};
        u.c_buf = 4;
        u.c_off = scratch;
        u.ldc = mc;
        u.m = mr;
        u.n = mc;
        u.ibeg = (int)i1.size();
        dev::GemmItem g{};
        g.a_buf = 0;
        g.a_off = c.va.off;
        g.lda = c.va.ld;
        g.ta = c.va.trans ? 1 : 0;
        g.b_buf = 2;
        g.b_off = S.offset;
        g.ldb = S.cols;
        g.k = S.rows;
        g.alpha = c.va.scale;
        i1.push_back(g);
        u.iend = (int)i1.size();
        u1.push_back(u);
        flops += 2.0 * mr * mc * S.rows;
        cur_l = c.lQ;
        cur_lp = c.lQp;
        cur_rp = c.rQp;
        cur_m = scratch;
        scratch += (int64_t)mr * mc;
      }
      dev::GemmItem h{};
      h.a_buf = 4;
      h.a_off = cur_m;
      h.lda = mc;
      h.b_buf = 1;
      h.b_off = c.vb.off;
      h.ldb = c.vb.ld;
      h.tb = c.vb.trans ? 0 : 1;
      h.k = mc;
      h.alpha = c.f * c.vb.scale;
      per_sector[c.vs].push_back(h);
      flops += 2.0 * SV.rows * SV.cols * mc;
    });
  }
  laps.lap("stage-1 and items");
  // stage 2: one unit per sector; a sector whose 64x64 tiles carry more K
  // than a fair share of the FP64 pipe is split along its item list into
  // units writing partial sectors after the stage-1 intermediates, summed
  // into sigma in a fixed order by the build-copy kernel
  std::vector<dev::GemmUnit> u2;
  std::vector<dev::GemmItem> i2;
  std::vector<dev::GemmTask> t1, t2;
  std::vector<dev::CopyUnit> ru;
  std::vector<dev::CopyItem> ri;
  double tile_k_total = 0.0;
  for (size_t s = 0; s < sb.sectors.size(); ++s) {
    const auto& S = sb.sectors[s];
    double k = 0.0;
    for (auto& g : per_sector[s]) k += g.k;
    tile_k_total += k * ((S.rows + 63) / 64) * ((S.cols + 63) / 64);
  }
  const double tile_k_share = std::max(tile_k_total / (4.0 * sm_count()), 4096.0);
  int64_t partial = scratch;  // partial sectors follow the stage-1 intermediates
  for (size_t s = 0; s < sb.sectors.size(); ++s) {
    const auto& S = sb.sectors[s];
    const auto& items = per_sector[s];
    double k = 0.0;
    for (auto& g : items) k += g.k;
    const int ntiles = ((S.rows + 63) / 64) * ((S.cols + 63) / 64);
    const int nchunks = std::max(1, std::min((int)items.size(), (int)std::ceil(k * ntiles / tile_k_share / ntiles)));
    if (nchunks <= 1) {
      dev::GemmUnit u{};
      u.c_buf = 3;
      u.c_off = S.offset;
      u.ldc = S.cols;
      u.m = S.rows;
      u.n = S.cols;
      u.beta_one = 0;
      u.ibeg = (int)i2.size();
      for (auto& g : items) i2.push_back(g);
      u.iend = (int)i2.size();
      u2.push_back(u);
      continue;
    }
    dev::CopyUnit cu{};
    cu.c_off = S.offset;
    cu.ldc = S.cols;
    cu.m = S.rows;
    cu.n = S.cols;
    cu.ibeg = (int)ri.size();
    const double per = k / nchunks;
    size_t a = 0;
    for (int c = 0; c < nchunks && a < items.size(); ++c) {
      size_t e = a;
      double acc = 0.0;
      while (e < items.size() && (acc < per || e == a || c == nchunks - 1)) acc += items[e++].k;
      dev::GemmUnit u{};
      u.c_buf = 4;
      u.c_off = partial;
      u.ldc = S.cols;
      u.m = S.rows;
      u.n = S.cols;
      u.beta_one = 0;
      u.ibeg = (int)i2.size();
      for (size_t x = a; x < e; ++x) i2.push_back(items[x]);
      u.iend = (int)i2.size();
      u2.push_back(u);
      dev::CopyItem ci{};
      ci.s_off = partial;
      ci.lds = S.cols;
      ci.s_buf = 4;
      ci.alpha = 1.0;
      ri.push_back(ci);
      partial += (int64_t)S.rows * S.cols;
      a = e;
    }
    cu.iend = (int)ri.size();
    ru.push_back(cu);
  }
  scratch = partial;
  for (int u = 0; u < (int)u1.size(); ++u) add_tasks(t1, u, u1[u].m, u1[u].n);
  // heavier output tiles first
  std::vector<std::pair<double, int>> cost;
  for (int u = 0; u < (int)u2.size(); ++u) {
    double c = 0;
    for (int i = u2[u].ibeg; i < u2[u].iend; ++i) c += i2[i].k;
    cost.push_back({-c, u});
  }
  std::stable_sort(cost.begin(), cost.end());
  for (auto& c : cost) add_tasks(t2, c.second, u2[c.second].m, u2[c.second].n);
  laps.lap("stage-2 units");
  plan.u1.upload(u1, stream_);
  plan.i1.upload(i1, stream_);
  plan.t1.upload(t1, stream_);
  plan.u2.upload(u2, stream_);
  plan.i2.upload(i2, stream_);
  plan.t2.upload(t2, stream_);
  plan.ru.upload(ru, stream_);
  plan.ri.upload(ri, stream_);
  plan.scratch_elems = scratch;
  plan.scratch = nullptr;  // allocated by the first FP64 product
  plan.flops = flops;
  plan.bytes = bytes + 2.0 * 8.0 * sb.size;
  plan.n = sb.size;
  plan.ecore = sb.ecore;
  plan.nstage1_units = (int)u1.size();
  plan.nstage2_units = (int)u2.size();
  plan.nitems = (int)(i1.size() + i2.size());
  laps.lap("uploads");
  // diagonal work list (diagonalH, spinblock.C:855-899)
  std::vector<dev::DiagUnit> du;
  std::vector<dev::DiagItem> di;
  for (const auto& S : sb.sectors) {
    dev::DiagUnit u{};
    u.d_off = S.offset;
    u.rows = S.rows;
    u.cols = S.cols;
    u.ibeg = (int)di.size();
    for (const PairTerm& t : sb.terms) {
      HostView va = hview(L, t.l, S.lq, S.lq);
      if (!va.ok) continue;
      HostView vb = hview(R, t.r, S.rq, S.rq);
      if (!vb.ok) continue;
      double f = t.coef * ninej(L.si.quanta[S.lq].s2, R.si.quanta[S.rq].s2, J, rank2(t.l), rank2(t.r), 0,
                                L.si.quanta[S.lq].s2, R.si.quanta[S.rq].s2, J);
      if (fermion(t.r) && is_fermion(L.si.quanta[S.lq])) f = -f;
      if (f == 0.0) continue;
      dev::DiagItem it{};
      it.a_off = va.identity ? -1 : va.off;
      it.a_stride = va.ld + 1;
      it.a_buf = 0;
      it.b_off = vb.identity ? -1 : vb.off;
      it.b_stride = vb.ld + 1;
      it.b_buf = 1;
      it.alpha = f * va.scale * vb.scale;
      di.push_back(it);
    }
    u.iend = (int)di.size();
    du.push_back(u);
  }
  std::vector<dev::GemmTask> dtask;
  for (int u = 0; u < (int)du.size(); ++u) add_tasks(dtask, u, du[u].rows, du[u].cols);
  laps.lap("diagonal lists");
  plan.du.upload(du, stream_);
  plan.di.upload(di, stream_);
  plan.dtask.upload(dtask, stream_);
}

void GpuEngine::free_tc(SigmaPlan& p) {
  for (int i = 0; i < dev::kTcPools; ++i) {
    if (p.tc_pool[i] && p.reuse_pools) {
      if (pool_cache_[i]) cudaFreeAsync(pool_cache_[i], stream_);
      pool_cache_[i] = p.tc_pool[i];
      pool_cache_cap_[i] = p.tc_pool_cap[i];
    } else if (p.tc_pool[i]) {
      cudaFreeAsync(p.tc_pool[i], stream_);
    }
    p.tc_pool[i] = nullptr;
    p.tc_pool_elems[i] = 0;
    p.tc_pool_cap[i] = 0;
  }
  p.tc_psi_pack.release(stream_);
  p.tc_w1.release(stream_);
  p.tc_w2.release(stream_);
  p.tc_r1.release(stream_);
  p.tc_r2.release(stream_);
  p.tc_tiles.release(stream_);
  p.tc_slots.release(stream_);
  p.tc_rows.release(stream_);
  p.tc_stacks = p.tc_stacked_items = 0;
  if (p.tc_partials) cudaFreeAsync(p.tc_partials, stream_);
  p.tc_partials = nullptr;
  p.tc_partial_cap = 0;
  p.tc_host.reset();
  for (int i = 0; i < dev::kTcPools; ++i) {
    if (p.tcx_ex[i]) cudaFreeAsync(p.tcx_ex[i], stream_);
    p.tcx_ex[i] = nullptr;
    p.tcx_ex_n[i] = 0;
  }
  if (p.tcx_t) cudaFreeAsync(p.tcx_t, stream_);
  p.tcx_t = nullptr;
  p.tcx_t_n = 0;
  p.tcx_tpack.release(stream_);
  p.tcx_w1.release(stream_);
  p.tcx_w2.release(stream_);
  p.tc_l1.clear();
  p.tc_l2.clear();
  p.tc_tuned = false;
  p.tc = false;
}

void GpuEngine::free_plan(SigmaPlan& p) {
  for (int i = 0; i < 3; ++i) {
    if (p.psi_s[i]) cudaFreeAsync(p.psi_s[i], stream_);
    p.psi_s[i] = nullptr;
  }
  p.ns = 0;
  p.fi.release(stream_);
  p.ft.release(stream_);
  p.ftile.release(stream_);
  if (p.partials) cudaFreeAsync(p.partials, stream_);
  p.partials = nullptr;
  p.fused = false;
  free_tc(p);
  p.u1.release(stream_);
  p.u2.release(stream_);
  p.i1.release(stream_);
  p.i2.release(stream_);
  p.t1.release(stream_);
  p.t2.release(stream_);
  p.du.release(stream_);
  p.di.release(stream_);
  p.dtask.release(stream_);
  p.ru.release(stream_);
  p.ri.release(stream_);
  free(p.scratch);
  p.scratch = nullptr;
}

void GpuEngine::sigma(const Superblock& sb, const SigmaPlan& p, const double* psi, double* out) {
  if (!p.scratch) p.scratch = alloc(p.scratch_elems);
  sigma_fp64(sb, p, psi, out, p.scratch);
}

void GpuEngine::sigma_fp64(const Superblock& sb, const SigmaPlan& p, const double* psi, double* out,
                           double* scratch) {
  dev::Bufs bufs{};
  bufs.p[0] = arena(*sb.L);
  bufs.p[1] = arena(*sb.R);
  bufs.p[2] = const_cast<double*>(psi);
  bufs.p[3] = out;
  bufs.p[4] = scratch;
  cuda_check(dev::launch_gemm(bufs, p.u1.d, p.i1.d, p.t1.d, (int)p.t1.n, stream_), "sigma stage 1");
  cuda_check(dev::launch_gemm(bufs, p.u2.d, p.i2.d, p.t2.d, (int)p.t2.n, stream_), "sigma stage 2");
  cuda_check(dev::launch_copy(bufs, out, p.ru.d, p.ri.d, (int)p.ru.n, stream_), "sigma stage-2 partial sums");
  if (p.ecore != 0.0) cuda_check(dev::launch_axpy(p.ecore, psi, out, p.n, stream_), "ecore");
  sigma_flops += p.flops;
  ++sigma_calls;
}

const GpuEngine::Slices& GpuEngine::block_slices(const Block& b, int ns) {
  Slices& sl = slices_[b.handle];
  if (sl.ns >= ns) return sl;
  for (auto*& p : sl.s)
    if (p) {
      cudaFreeAsync(p, stream_);
      p = nullptr;
    }
  const DevBlock& d = blocks_.at(b.handle);
  for (int i = 0; i < ns; ++i)
    cuda_check(cudaMallocAsync((void**)&sl.s[i], std::max<int64_t>(d.n, 1) * sizeof(__nv_bfloat16), stream_),
               "slices");
  cuda_check(dev::launch_slices(d.d, d.n, ns, sl.s[0], sl.s[1], ns > 2 ? sl.s[2] : nullptr, stream_), "slice op");
  sl.ns = ns;
  return sl;
}

// Work lists of the fused split-precision kernel: the same couplings as
// plan_sigma, grouped by output sector; every 64 x 64 tile of a sector gets
// its coupling list cut into chunks of similar cost (one thread block each)
// and a fixed-order reduction of the chunks' partial tiles.
void GpuEngine::plan_fused(const Superblock& sb, SigmaPlan& plan) {
  PlanTimer timer_(plan_seconds);
  const auto by_l = sectors_by_left(sb);
  std::vector<std::vector<std::vector<dev::FusedItem>>> per_t(sb.terms.size());
  parallel_for((int)sb.terms.size(), [&](int ti) {
    auto& per = per_t[ti];
    per.assign(sb.sectors.size(), {});
    for_each_coupling(sb, sb.terms[ti], by_l, [&](const Coupling& c) {
      const auto& C = sb.sectors[c.cs];
      dev::FusedItem it{};
      it.n1 = C.cols;
      it.k1 = C.rows;
      it.c_off = C.offset;
      it.ldc = C.cols;
      if (c.va.identity && c.vb.identity) throw std::runtime_error("identity x identity pair term");
      if (c.va.identity) {
        it.kind = dev::kFusedLIdent;
        it.a_off = C.offset;  // psi(lQ, rQ') with lQ' = lQ
        it.lda = C.cols;
        it.b_off = c.vb.off;
        it.ldb = c.vb.ld;
        it.tb = c.vb.trans;
        it.alpha = (float)(c.f * c.vb.scale);
      } else if (c.vb.identity) {
        it.kind = dev::kFusedRIdent;
        it.a_off = c.va.off;
        it.lda = c.va.ld;
        it.ta = c.va.trans;
        it.alpha = (float)(c.f * c.va.scale);
      } else {
        it.kind = dev::kFusedFull;
        it.a_off = c.va.off;
        it.lda = c.va.ld;
        it.ta = c.va.trans;
        it.b_off = c.vb.off;
        it.ldb = c.vb.ld;
        it.tb = c.vb.trans;
        it.alpha = (float)(c.f * c.va.scale * c.vb.scale);
      }
      per[c.vs].push_back(it);
    });
  });
  std::vector<std::vector<dev::FusedItem>> per(sb.sectors.size());
  for (auto& pt : per_t)
    for (size_t s2 = 0; s2 < pt.size(); ++s2) per[s2].insert(per[s2].end(), pt[s2].begin(), pt[s2].end());
  auto cost = [](const dev::FusedItem& it) {
    const double n1 = ((it.n1 + 15) / 16) * 16.0, k1 = ((it.k1 + 15) / 16) * 16.0;
    double c = 2048.0;
    if (it.kind != dev::kFusedLIdent) c += k1 * (it.kind == dev::kFusedRIdent ? 64.0 : n1);
    if (it.kind != dev::kFusedRIdent) c += n1 * 64.0;
    return c;
  };
  double total = 0.0;
  std::vector<double> sec_cost(sb.sectors.size(), 0.0);
  for (size_t s = 0; s < per.size(); ++s) {
    for (auto& it : per[s]) sec_cost[s] += cost(it);
    const auto& S = sb.sectors[s];
    total += sec_cost[s] * ((S.rows + 63) / 64) * ((S.cols + 63) / 64);
  }
  const double chunk = std::max(total / (152.0 * 12.0), 64.0 * 1024.0);
  std::vector<dev::FusedItem> items;
  std::vector<dev::FusedTask> tasks;
  std::vector<dev::FusedTile> tiles;
  for (size_t s = 0; s < per.size(); ++s) {
    const auto& S = sb.sectors[s];
    const int ib = (int)items.size();
    for (auto& it : per[s]) items.push_back(it);
    const int ie = (int)items.size();
    for (int tm = 0; tm < (S.rows + 63) / 64; ++tm)
      for (int tn = 0; tn < (S.cols + 63) / 64; ++tn) {
        dev::FusedTile tl{};
        tl.s_off = S.offset;
        tl.lds = S.cols;
        tl.m = S.rows;
        tl.n = S.cols;
        tl.tm = tm;
        tl.tn = tn;
        tl.pbeg = (int)tasks.size();
        int a = ib;
        while (a < ie) {
          double acc = 0.0;
          int b = a;
          while (b < ie && (acc < chunk || b == a)) acc += cost(items[b++]);
          tasks.push_back({S.rows, S.cols, tm, tn, a, b});
          a = b;
        }
        tl.pend = (int)tasks.size();
        tiles.push_back(tl);
      }
  }
  plan.fi.upload(items, stream_);
  plan.ft.upload(tasks, stream_);
  plan.ftile.upload(tiles, stream_);
  cuda_check(cudaMallocAsync((void**)&plan.partials, std::max<size_t>(tasks.size(), 1) * 4096 * sizeof(float), stream_),
             "partials");
  plan.fused = true;
  sync();
}

// Split-precision sigma with the fused two-stage kernel: operator arenas
// are sliced once per block, psi per call.
void GpuEngine::sigma_split(const Superblock& sb, SigmaPlan& p, int ns, const double* psi, double* out,
                            cudaEvent_t* marks) {
  if (!p.fused) plan_fused(sb, p);
  const Slices& Ls = block_slices(*sb.L, ns);
  const Slices& Rs = block_slices(*sb.R, ns);
  if (p.ns < ns) {
    for (int i = 0; i < 3; ++i) {
      if (p.psi_s[i]) cudaFreeAsync(p.psi_s[i], stream_);
      p.psi_s[i] = nullptr;
    }
    for (int i = 0; i < ns; ++i)
      cuda_check(cudaMallocAsync((void**)&p.psi_s[i], std::max<int64_t>(p.n, 1) * 2, stream_), "psi slices");
    p.ns = ns;
  }
  cuda_check(dev::launch_slices(psi, p.n, ns, p.psi_s[0], p.psi_s[1], ns > 2 ? p.psi_s[2] : nullptr, stream_),
             "slice psi");
  dev::FusedBufs fb{};
  for (int i = 0; i < 3; ++i) {
    fb.L[i] = Ls.s[i];
    fb.R[i] = Rs.s[i];
    fb.psi[i] = p.psi_s[i];
  }
  fb.psi64 = psi;
  fb.partials = p.partials;
  if (marks) cuda_check(cudaEventRecord(marks[0], stream_), "record");
  cuda_check(dev::launch_fused_sigma(ns, fb, p.fi.d, p.ft.d, (int)p.ft.n, stream_), "fused sigma");
  if (marks) cuda_check(cudaEventRecord(marks[1], stream_), "record");
  cuda_check(dev::launch_fused_reduce(fb, p.ftile.d, (int)p.ftile.n, out, stream_), "fused reduce");
  if (p.ecore != 0.0) cuda_check(dev::launch_axpy(p.ecore, psi, out, p.n, stream_), "ecore");
  sigma_flops += p.flops;
  ++sigma_calls;
}

// Tensor-core plan.  Stage-1 products S = s_L A psi (one per (term, lQ, lQ',
// rQ') as in plan_sigma) become phase-1 tasks writing S as packed bf16
// (hi, lo) operands; every sigma sector tile then sums its items
// alpha * X * Y^T (X = S, psi or an L operator; Y = an R operator or psi^T)
// in phase 2, in the same order as the FP64 plan.
// Host side of a tensor-core plan: phase-1 items and tasks (with the psi
// sector each task reads), and the phase-2 items of every sigma sector.
struct TcHostPlan {
  std::vector<dev::TcItem> i1;
  std::vector<dev::TcTask> t1;
  std::vector<int> sec1;
  std::vector<int64_t> bundle1;
  std::vector<std::vector<dev::TcItem>> per_sector;
  double mma1 = 0.0;  // tensor-core flops of phase 1
};

// Output-tile width of a new plan: BGPU_TC_NB or tc_nb_mode when set, else
// 128 when most of sigma's stage-2 work lies in sectors at least 128 columns
// wide (there a 128 x 128 tile reads each A piece once for twice the MMA
// work), otherwise 64 (two pipelines per SM hide the per-item latency of
// small sectors).
int GpuEngine::tc_choose_nb(const Superblock& sb) const {
  const int env = (int)env_double("BGPU_TC_NB", 0.0);
  if (env == 64 || env == 128) return env;
  if (tc_nb_mode == 64 || tc_nb_mode == 128) return tc_nb_mode;
  double wide = 0.0, all = 0.0;
  for (const auto& S : sb.sectors) {
    const double w = (double)S.rows * S.cols * S.cols;
    all += w;
    if (S.cols >= 128) wide += w;
  }
  return all > 0.0 && wide >= 0.5 * all ? dev::kTcRowsBWide : dev::kTcRowsB;
}

void GpuEngine::plan_tc(const Superblock& sb, SigmaPlan& plan) {
  PlanTimer timer_(plan_seconds);
  PlanLaps laps{"tc"};
  using namespace dev;
  const Block& L = *sb.L;
  const Block& R = *sb.R;
  if (!plan.tc_nb_set) plan.tc_nb = tc_choose_nb(sb);
  if (plan.tc_nb != kTcRowsB && plan.tc_nb != kTcRowsBWide) plan.tc_nb = kTcRowsB;
  if (plan.tcx) plan.tc_nb = kTcxNB;
  const int nb = plan.tc_nb;
  // slices per packed element: bf16 hi and lo, or six exact digits
  const int64_t nsl = plan.tcx ? kTcxSlices : 2;
  int64_t ex_n[kTcPools] = {0, 0, 0, 0, 0};  // rows of each pool (row exponents)
  std::vector<TcPack> t_packs;                // exact: T -> pool S, per stage-1 product
  int64_t t_n = 0;
  const auto by_l = sectors_by_left(sb);
  const int nsec = (int)sb.sectors.size();
  std::vector<std::vector<Coupling>> per_t(sb.terms.size());
  parallel_for((int)sb.terms.size(), [&](int ti) {
    for_each_coupling(sb, sb.terms[ti], by_l, [&](const Coupling& c) { per_t[ti].push_back(c); });
  });
  laps.lap("couplings");
  int64_t pool_n[kTcPools] = {0, 0, 0, 0, 0};
  // Every item is checked against the packed operands it reads (rows and K
  // of its output sector), so that no bulk copy can leave its operand.
  auto fail = []() { throw std::runtime_error("tensor-core plan: operand shape does not match its sector"); };
  std::vector<TcPack> ops_packs, psi_packs;
  std::unordered_map<int64_t, int> lmap, rmap;  // (block offset, transposed) -> index in ops_packs
  lmap.reserve(1 << 16);
  rmap.reserve(1 << 16);
  auto pack_view = [&](int pool, const HostView& v, std::unordered_map<int64_t, int>& m) -> TcPack {
    const int64_t key = v.off * 2 + (v.trans ? 1 : 0);
    auto it = m.find(key);
    if (it != m.end()) return ops_packs[it->second];
    TcPack p{};
    p.src_off = v.off;
    p.ld = v.ld;
    p.rows_v = v.rows;
    p.cols_v = v.cols;
    p.rows_p = tc_round8(v.rows);
    p.kp = tc_round16(v.cols);
    p.trans = v.trans ? 1 : 0;
    p.rt = pool == kTcPoolL ? kTcRowsA : nb;  // L blocks are A operands, R blocks B operands
    p.src = (uint8_t)pool;  // 0: L arena, 1: R arena
    p.pool = (uint8_t)pool;
    p.dst_off = pool_n[pool];
    pool_n[pool] += nsl * (int64_t)p.rows_p * p.kp;  // all slices
    p.ex_off = (int32_t)ex_n[pool];
    ex_n[pool] += p.rows_p;
    m.emplace(key, (int)ops_packs.size());
    ops_packs.push_back(p);
    return p;
  };
  std::vector<int64_t> psi_off(nsec), psit_off(nsec);
  std::vector<int32_t> psi_ex(nsec), psit_ex(nsec);
  for (int s = 0; s < nsec; ++s) {
    const auto& S = sb.sectors[s];
    TcPack a{};
    a.src = 2;
    a.pool = kTcPoolPsi;
    a.src_off = S.offset;
    a.ld = S.cols;
    a.rows_v = S.rows;
    a.cols_v = S.cols;
    a.rows_p = tc_round8(S.rows);
    a.kp = tc_round16(S.cols);
    a.rt = kTcRowsA;
    a.dst_off = psi_off[s] = pool_n[kTcPoolPsi];
    pool_n[kTcPoolPsi] += nsl * (int64_t)a.rows_p * a.kp;
    a.ex_off = psi_ex[s] = (int32_t)ex_n[kTcPoolPsi];
    ex_n[kTcPoolPsi] += a.rows_p;
    psi_packs.push_back(a);
    TcPack t = a;
    t.pool = kTcPoolPsiT;
    t.trans = 1;
    t.rows_v = S.cols;
    t.cols_v = S.rows;
    t.rows_p = tc_round8(S.cols);
    t.kp = tc_round16(S.rows);
    t.rt = nb;
    t.dst_off = psit_off[s] = pool_n[kTcPoolPsiT];
    pool_n[kTcPoolPsiT] += nsl * (int64_t)t.rows_p * t.kp;
    t.ex_off = psit_ex[s] = (int32_t)ex_n[kTcPoolPsiT];
    ex_n[kTcPoolPsiT] += t.rows_p;
    psi_packs.push_back(t);
  }
  std::vector<TcItem> i1;
  std::vector<TcTask> t1;
  std::vector<int> sec1;          // psi sector read by each phase-1 task
  std::vector<int64_t> bundle1;  // tasks reading the same A row tile
  std::vector<std::vector<TcItem>> per_sector(nsec);
  std::vector<std::vector<int>> per_sector_s(nsec);  // phase-1 item of a stage-1 operand, else -1
  double mma = 0.0;
  for (auto& cl : per_t) {
    int cur_l = -1, cur_lp = -1, cur_rp = -1, cur_kp = 0, cur_item = -1;
    int64_t cur_s = -1;
    int32_t cur_ex = 0;
    for (const Coupling& c : cl) {
      if (c.va.identity && c.vb.identity) throw std::runtime_error("identity x identity pair term");
      const auto& SV = sb.sectors[c.vs];
      const int out_rows_p = tc_round8(SV.rows), out_cols_p = tc_round8(SV.cols);
      TcItem it{};
      if (c.va.identity) {  // sigma(lQ,rQ) += f psi(lQ,rQ') B^T
        const TcPack pb = pack_view(1, c.vb, rmap);
        it.a_pool = kTcPoolPsi;
        it.a_off = psi_off[c.cs];
        it.b_pool = kTcPoolR;
        it.b_off = pb.dst_off;
        it.kp = tc_round16(R.si.states[c.rQp]);
        it.alpha = (float)(c.f * c.vb.scale);
        it.alpha64 = c.f * c.vb.scale;
        it.a_ex = psi_ex[c.cs];
        it.b_ex = pb.ex_off;
        const auto& C = sb.sectors[c.cs];
        if (tc_round8(C.rows) != out_rows_p || tc_round16(C.cols) != it.kp || pb.rows_p != out_cols_p ||
            pb.kp != it.kp)
          fail();
        per_sector[c.vs].push_back(it);
        per_sector_s[c.vs].push_back(-1);
        continue;
      }
      if (c.vb.identity) {  // sigma(lQ,rQ') += f s_L A psi(lQ',rQ')
        const TcPack pa = pack_view(0, c.va, lmap);
        it.a_pool = kTcPoolL;
        it.a_off = pa.dst_off;
        it.b_pool = kTcPoolPsiT;
        it.b_off = psit_off[c.cs];
        it.kp = tc_round16(L.si.states[c.lQp]);
        it.alpha = (float)(c.f * c.va.scale);
        it.alpha64 = c.f * c.va.scale;
        it.a_ex = pa.ex_off;
        it.b_ex = psit_ex[c.cs];
        const auto& C = sb.sectors[c.cs];
        if (pa.rows_p != out_rows_p || pa.kp != it.kp || tc_round8(C.cols) != out_cols_p ||
            tc_round16(C.rows) != it.kp)
          fail();
        per_sector[c.vs].push_back(it);
        per_sector_s[c.vs].push_back(-1);
        continue;
      }
      if (!(c.lQ == cur_l && c.lQp == cur_lp && c.rQp == cur_rp)) {
        const int mr = L.si.states[c.lQ], mc = R.si.states[c.rQp], k1 = L.si.states[c.lQp];
        const int rows_p = tc_round8(mr), skp = tc_round16(mc);
        cur_s = pool_n[kTcPoolS];
        pool_n[kTcPoolS] += nsl * (int64_t)rows_p * skp;
        cur_ex = (int32_t)ex_n[kTcPoolS];
        ex_n[kTcPoolS] += rows_p;
        if (plan.tcx) {  // the FP64 product T, packed into pool S after phase 1
          TcPack tp{};
          tp.src = 3;
          tp.src_off = t_n;
          tp.ld = skp;
          tp.rows_v = mr;
          tp.cols_v = mc;
          tp.rows_p = rows_p;
          tp.kp = skp;
          tp.rt = kTcRowsA;
          tp.pool = kTcPoolS;
          tp.dst_off = cur_s;
          tp.ex_off = cur_ex;
          t_packs.push_back(tp);
          t_n += (int64_t)rows_p * skp;
        }
        const TcPack pa = pack_view(0, c.va, lmap);
        TcItem a{};
        a.a_pool = kTcPoolL;
        a.a_off = pa.dst_off;
        a.b_pool = kTcPoolPsiT;
        a.b_off = psit_off[c.cs];
        a.kp = tc_round16(k1);
        a.alpha = (float)c.va.scale;
        a.alpha64 = c.va.scale;
        a.a_ex = pa.ex_off;
        a.b_ex = psit_ex[c.cs];
        a.o_ex = cur_ex;
        const auto& C = sb.sectors[c.cs];
        if (pa.rows_p != rows_p || pa.kp != a.kp || tc_round8(C.cols) != tc_round8(mc) ||
            tc_round16(C.rows) != a.kp)
          fail();
        const int idx = (int)i1.size();
        i1.push_back(a);
        for (int tm = 0; tm < (mr + 127) / 128; ++tm)
          for (int tn = 0; tn < (mc + nb - 1) / nb; ++tn) {
            TcTask t{};
            t.a_rows = rows_p;
            t.b_rows = tc_round8(mc);
            t.tm = tm;
            t.tn = tn;
            t.ibeg = idx;
            t.iend = idx + 1;
            t.out_off = cur_s;
            t.out_kp = skp;
            t1.push_back(t);
            sec1.push_back(c.cs);
            bundle1.push_back((cur_s << 8) | tm);
            mma += 3.0 * 2.0 * 128 * tc_round16(std::min(nb, t.b_rows - nb * tn)) * a.kp;
          }
        cur_l = c.lQ;
        cur_lp = c.lQp;
        cur_rp = c.rQp;
        cur_kp = skp;
        cur_item = idx;
        if (rows_p != out_rows_p) fail();
      }
      const TcPack pb = pack_view(1, c.vb, rmap);
      it.a_pool = kTcPoolS;
      it.a_off = cur_s;
      it.b_pool = kTcPoolR;
      it.b_off = pb.dst_off;
      it.kp = cur_kp;
      it.alpha = (float)(c.f * c.vb.scale);
      it.alpha64 = c.f * c.vb.scale;
      it.a_ex = cur_ex;
      it.b_ex = pb.ex_off;
      if (pb.rows_p != out_cols_p || pb.kp != it.kp) fail();
      per_sector[c.vs].push_back(it);
      per_sector_s[c.vs].push_back(cur_item);
    }
  }
  laps.lap("items");
  // alpha of a stage-1 product read by exactly one item moves into phase 1,
  // so that such items (alpha = 1) can share a tensor-core accumulator
  {
    std::vector<int> consumers(i1.size(), 0);
    for (auto& v : per_sector_s)
      for (int u : v)
        if (u >= 0) ++consumers[u];
    for (int s = 0; s < nsec; ++s) {
      auto& v = per_sector[s];
      const auto& us = per_sector_s[s];
      for (size_t k = 0; k < v.size(); ++k)
        if (us[k] >= 0 && consumers[us[k]] == 1) {
          TcItem& u = i1[us[k]];
          u.alpha = (float)((double)u.alpha * (double)v[k].alpha);
          v[k].alpha = 1.0f;
          u.alpha64 *= v[k].alpha64;
          v[k].alpha64 = 1.0;
        }
    }
    // items with alpha = 1 first, so that they form long accumulation runs
    for (auto& v : per_sector)
      std::stable_partition(v.begin(), v.end(), [](const TcItem& it) { return it.alpha == 1.0f; });
  }
  laps.lap("alpha folding");
  // Stacks: phase-1 products of small operator blocks (at most tc_stack_rows
  // rows) that read the same psi^T block (same B operand, same K) share one
  // 128-row A tile.  Each member is packed again at its row offset of a
  // stacked operand in pool L, and the phase-1 epilogue sends every row of
  // the stacked tile, scaled by its member's alpha, to that member's
  // stage-1 operand (TcRow).  Every row is the same dot product as in the
  // unstacked tile; a stack takes one pass through the pipeline instead of
  // one per member.
  std::vector<TcRow> rows_tab;
  int64_t n_stacks = 0, n_stacked = 0;
  if (!plan.tcx && tc_stack_rows > 0) {
    std::unordered_map<int64_t, int> lpack;  // pool-L offset -> its pack unit
    for (size_t i = 0; i < ops_packs.size(); ++i)
      if (ops_packs[i].pool == kTcPoolL) lpack.emplace(ops_packs[i].dst_off, (int)i);
    const size_t ni = i1.size();
    std::vector<std::vector<int>> tasks_of(ni);
    for (size_t k = 0; k < t1.size(); ++k) tasks_of[t1[k].ibeg].push_back((int)k);
    auto task_mma = [&](const TcTask& t) {
      return 3.0 * 2.0 * 128 * tc_round16(std::min(nb, t.b_rows - nb * t.tn)) * i1[t.ibeg].kp;
    };
    // candidates grouped by (psi^T block, K), each group in item order
    std::map<std::pair<int64_t, int>, std::vector<int>> groups;
    for (size_t u = 0; u < ni; ++u) {
      if (tasks_of[u].empty() || i1[u].a_pool != kTcPoolL) continue;
      if (t1[tasks_of[u][0]].a_rows > std::min(tc_stack_rows, kTcRowsA)) continue;
      groups[{i1[u].b_off, i1[u].kp}].push_back((int)u);
    }
    std::vector<char> drop(t1.size(), 0);
    std::vector<TcTask> t_new;
    std::vector<int> sec_new;
    std::vector<int64_t> bun_new;
    for (const auto& g : groups) {
      const std::vector<int>& us = g.second;
      size_t x = 0;
      while (x < us.size()) {
        size_t y = x;
        int H = 0;
        while (y < us.size() && H + t1[tasks_of[us[y]][0]].a_rows <= kTcRowsA) H += t1[tasks_of[us[y++]][0]].a_rows;
        if (y - x < 2) {
          x = y;
          continue;
        }
        const int kp = i1[us[x]].kp;
        const int64_t st_off = pool_n[kTcPoolL];
        pool_n[kTcPoolL] += 2 * (int64_t)H * kp;
        const int64_t base = (int64_t)rows_tab.size();
        rows_tab.resize(base + kTcRowsA, TcRow{0, 0, 0, 0.f});
        int r0 = 0;
        for (size_t m = x; m < y; ++m) {
          const int u = us[m];
          const TcTask& T = t1[tasks_of[u][0]];
          auto it = lpack.find(i1[u].a_off);
          if (it == lpack.end() || i1[u].kp != kp || T.tm != 0) fail();
          TcPack pk = ops_packs[it->second];
          pk.dst_off = st_off;
          pk.row0 = r0;
          pk.dst_rows = H;
          ops_packs.push_back(pk);
          for (int lr = 0; lr < T.a_rows; ++lr)
            rows_tab[base + r0 + lr] = TcRow{T.out_off, (int16_t)T.a_rows, (int16_t)lr, i1[u].alpha};
          for (int k : tasks_of[u]) {
            drop[k] = 1;
            mma -= task_mma(t1[k]);
          }
          r0 += T.a_rows;
        }
        TcItem si = i1[us[x]];
        si.a_off = st_off;
        si.alpha = 1.0f;
        si.alpha64 = 1.0;
        const int idx = (int)i1.size();
        i1.push_back(si);
        for (int k : tasks_of[us[x]]) {
          TcTask t = t1[k];
          t.a_rows = H;
          t.ibeg = idx;
          t.iend = idx + 1;
          t.out_off = base;
          t.stacked = 1;
          t_new.push_back(t);
          sec_new.push_back(sec1[k]);
          bun_new.push_back(((int64_t)1 << 50) + (n_stacks << 8));
          mma += task_mma(t);
        }
        ++n_stacks;
        n_stacked += (int64_t)(y - x);
        x = y;
      }
    }
    if (n_stacks > 0) {
      std::vector<TcTask> tk;
      std::vector<int> sk;
      std::vector<int64_t> bk;
      for (size_t k = 0; k < t1.size(); ++k)
        if (!drop[k]) {
          tk.push_back(t1[k]);
          sk.push_back(sec1[k]);
          bk.push_back(bundle1[k]);
        }
      tk.insert(tk.end(), t_new.begin(), t_new.end());
      sk.insert(sk.end(), sec_new.begin(), sec_new.end());
      bk.insert(bk.end(), bun_new.begin(), bun_new.end());
      t1 = std::move(tk);
      sec1 = std::move(sk);
      bundle1 = std::move(bk);
    }
  }
  plan.tc_stacks = n_stacks;
  plan.tc_stacked_items = n_stacked;
  plan.tc_stack_used = tc_stack_rows;
  laps.lap("stacks");
  // the item lists stay on the host, so that the device work lists can be
  // rebuilt for other schedule knobs (autotuner, per-sector baseline)
  auto host = std::make_shared<TcHostPlan>();
  host->i1 = std::move(i1);
  host->t1 = std::move(t1);
  host->sec1 = std::move(sec1);
  host->bundle1 = std::move(bundle1);
  host->per_sector = std::move(per_sector);
  host->mma1 = mma;
  plan.tc_host = host;
  for (int i = 0; i < kTcPools; ++i) {
    plan.tc_pool_elems[i] = pool_n[i];
    const size_t bytes = (size_t)std::max<int64_t>(pool_n[i], 8) * sizeof(__nv_bfloat16);
    if (plan.reuse_pools && pool_cache_[i] && pool_cache_cap_[i] >= bytes) {
      plan.tc_pool[i] = pool_cache_[i];
      plan.tc_pool_cap[i] = pool_cache_cap_[i];
      pool_cache_[i] = nullptr;
      pool_cache_cap_[i] = 0;
      continue;
    }
    if (plan.reuse_pools && pool_cache_[i]) {
      cudaFreeAsync(pool_cache_[i], stream_);
      pool_cache_[i] = nullptr;
      pool_cache_cap_[i] = 0;
    }
    // pools handed from solve to solve get 1/8 slack for the next superblock
    const size_t cap = plan.reuse_pools ? bytes + bytes / 8 : bytes;
    cuda_check(cudaMallocAsync((void**)&plan.tc_pool[i], cap, stream_), "tc pool");
    plan.tc_pool_cap[i] = cap;
  }
  plan.tc_psi_pack.upload(psi_packs, stream_);
  plan.tc_rows.upload(rows_tab, stream_);
  // operator blocks are packed once per plan
  DevArray<TcPack> dops;
  dops.upload(ops_packs, stream_);
  if (plan.tcx) {
    for (int i = 0; i < kTcPools; ++i) {
      plan.tcx_ex_n[i] = ex_n[i];
      cuda_check(cudaMallocAsync((void**)&plan.tcx_ex[i], (size_t)std::max<int64_t>(ex_n[i], 1) * sizeof(int), stream_),
                 "tcx row exponents");
    }
    plan.tcx_t_n = t_n;
    cuda_check(cudaMallocAsync((void**)&plan.tcx_t, (size_t)std::max<int64_t>(t_n, 1) * sizeof(double), stream_),
               "tcx stage-1 products");
    plan.tcx_tpack.upload(t_packs, stream_);
    TcxBufs xb{};
    xb.src[0] = arena(L);
    xb.src[1] = arena(R);
    for (int i = 0; i < kTcPools; ++i) {
      xb.pool[i] = plan.tc_pool[i];
      xb.ex[i] = plan.tcx_ex[i];
    }
    cuda_check(launch_tcx_rowexp(xb, dops.d, (int)ops_packs.size(), stream_), "tcx operator exponents");
    cuda_check(launch_tcx_pack(xb, dops.d, (int)ops_packs.size(), stream_), "tcx pack operators");
    plan.tc_fp16 = false;
  } else {
    TcBufs b{};
    b.src[0] = arena(L);
    b.src[1] = arena(R);
    for (int i = 0; i < kTcPools; ++i) {
      b.pool[i] = plan.tc_pool[i];
    }
    b.fp16 = precision == Precision::FP16X2_TC ? 1 : 0;
    plan.tc_fp16 = b.fp16 != 0;
    cuda_check(launch_tc_pack(b, dops.d, (int)ops_packs.size(), stream_), "tc pack operators");
  }
  dops.release(stream_);
  laps.lap("pools + pack operators");
  TcKnobs kn = tc_default_knobs();
  kn.per_sector = tc_schedule_mode == 1 ? 1 : 0;
  plan.tc_tuned = false;
  schedule_tc(sb, plan, kn);
  plan.tc = true;
  if (laps.on) sync();
  laps.lap("schedule");
}

TcKnobs GpuEngine::tc_default_knobs() const {
  // defaults measured near-optimal on the 24-orbital M=500 superblock;
  // BGPU_TC_ITEM_COST, BGPU_TC_SPLIT and BGPU_TC_GROUP override them
  TcKnobs k;
  k.item_cost = env_double("BGPU_TC_ITEM_COST", 400.0);
  k.split = env_double("BGPU_TC_SPLIT", 3.0);
  k.group = (int)env_double("BGPU_TC_GROUP", 16.0);
  k.waves = (int)env_double("BGPU_TC_WAVES", 0.0);
  k.pairs = (int)env_double("BGPU_TC_PAIRS", 0.0);
  return k;
}

// Phase-2 tasks, cost model, block assignment and flattened work records of
// a tensor-core plan for one set of knobs.  Persistent schedule: two blocks
// per SM, longest-processing-time assignment; tiles costing more than
// total / (2 split SMs) are cut into pieces summed by the reduce kernel.
// Per-sector schedule (baseline): no cut tiles, one block per task, one
// launch per psi sector (phase 1) and per sigma sector (phase 2).
void GpuEngine::schedule_tc(const Superblock& sb, SigmaPlan& plan, const TcKnobs& kn) {
  PlanTimer timer_(plan_seconds);
  PlanLaps laps{"tc schedule"};
  using namespace dev;
  const TcHostPlan& H = *plan.tc_host;
  const auto& i1 = H.i1;
  const auto& t1 = H.t1;
  const auto& per_sector = H.per_sector;
  const int nsec = (int)sb.sectors.size();
  const int nsm = sm_count();
  const int nb = plan.tc_nb;  // fixed by the packing of the B-role pools
  const bool seq = kn.per_sector != 0;
  const double item_fixed = kn.item_cost;
  auto item_cost = [&](const TcItem& it, int hb) { return item_fixed + (double)it.kp * tc_round16(hb) / 8.0; };
  auto fail = []() { throw std::runtime_error("tensor-core plan: operand shape does not match its sector"); };
  double mma = H.mma1;
  std::vector<TcItem> i2;
  std::vector<TcTask> t2;
  std::vector<double> c2;
  std::vector<int> sec2;
  std::vector<int64_t> bundle2;
  std::vector<TcTile> tiles;
  std::vector<int64_t> slots;
  int64_t partial_n = 0;
  double total = 0.0;
  for (int s = 0; s < nsec; ++s) {
    const auto& S = sb.sectors[s];
    for (int tn = 0; tn < (S.cols + nb - 1) / nb; ++tn) {
      const int hb = std::min(nb, tc_round8(S.cols) - nb * tn);
      for (const TcItem& it : per_sector[s]) total += item_cost(it, hb) * ((S.rows + 127) / 128);
    }
  }
  const double chunk = seq ? 1e300 : std::max(total / (2.0 * kn.split * nsm), 20000.0);
  // cluster pairs (phase 2 with 128-column tiles): the column tiles tn and
  // tn + 1 of a sigma row tile run on the two blocks of a cluster, which
  // read the same items; a row tile with an odd number of column tiles
  // pairs its last one with a ghost copy that writes nothing.  Split tiles
  // cut every column tile of a row tile at the same items.  t2 holds the
  // pairs' tasks one after the other (2p, 2p + 1), c2 their pair costs.
  const bool pairs = kn.pairs != 0 && nb == kTcRowsBWide && !seq && !plan.tcx;
  std::vector<double> cp;  // cost per pair
  std::vector<int64_t> bundle_p;
  if (pairs) {
    for (int s = 0; s < nsec; ++s) {
      const auto& S = sb.sectors[s];
      const int ib = (int)i2.size();
      i2.insert(i2.end(), per_sector[s].begin(), per_sector[s].end());
      const int ie = (int)i2.size();
      const int rows_p = tc_round8(S.rows), cols_p = tc_round8(S.cols);
      const int ntn = (S.cols + nb - 1) / nb;
      for (int tm = 0; tm < (S.rows + 127) / 128; ++tm) {
        const int ha = std::min(128, rows_p - 128 * tm);
        const int hb0 = std::min(nb, cols_p);  // the widest column tile
        double tile_cost = 0.0;
        for (int x = ib; x < ie; ++x) tile_cost += item_cost(i2[x], hb0);
        // item cuts shared by every column tile of this row tile
        std::vector<int2> cuts;
        if (tile_cost <= chunk || ie - ib <= 1) {
          cuts.push_back(make_int2(ib, ie));
        } else {
          int x0 = ib;
          while (x0 < ie) {
            double acc = 0.0;
            int x1 = x0;
            while (x1 < ie && (acc < chunk || x1 == x0)) acc += item_cost(i2[x1++], hb0);
            cuts.push_back(make_int2(x0, x1));
            x0 = x1;
          }
        }
        const bool direct = cuts.size() == 1;
        // per column tile: its tasks (one per cut), partial slots and tile
        std::vector<std::vector<TcTask>> col(ntn);
        std::vector<std::vector<double>> colc(ntn);
        for (int tn = 0; tn < ntn; ++tn) {
          const int hb = std::min(nb, cols_p - nb * tn);
          TcTask t{};
          t.a_rows = rows_p;
          t.b_rows = cols_p;
          t.tm = tm;
          t.tn = tn;
          t.valid_rows = std::min(128, S.rows - 128 * tm);
          t.valid_cols = std::min(nb, S.cols - nb * tn);
          for (int x = ib; x < ie; ++x) mma += 3.0 * 2.0 * 128 * tc_round16(hb) * i2[x].kp;
          TcTile tl{};
          if (!direct) {
            tl.s_off = S.offset;
            tl.lds = S.cols;
            tl.h = t.valid_rows;
            tl.w = t.valid_cols;
            tl.r0 = 128 * tm;
            tl.c0 = nb * tn;
            tl.pad = hb;
            tl.pbeg = (int)slots.size();
          }
          for (const int2& ct : cuts) {
            TcTask u = t;
            u.ibeg = ct.x;
            u.iend = ct.y;
            double acc = 0.0;
            for (int x = ct.x; x < ct.y; ++x) acc += item_cost(i2[x], hb);
            if (direct) {
              u.direct = 1;
              u.out_off = S.offset;
              u.out_kp = S.cols;
            } else {
              u.direct = 0;
              u.out_off = partial_n;
              slots.push_back(partial_n);
              partial_n += (int64_t)ha * hb;
            }
            col[tn].push_back(u);
            colc[tn].push_back(acc);
          }
          if (!direct) {
            tl.pend = (int)slots.size();
            tiles.push_back(tl);
          }
        }
        for (int tn = 0; tn < ntn; tn += 2)
          for (size_t k = 0; k < cuts.size(); ++k) {
            const TcTask& a = col[tn][k];
            TcTask g = a;  // ghost partner of a last odd column tile
            g.ghost = 1;
            const TcTask& bt = tn + 1 < ntn ? col[tn + 1][k] : g;
            t2.push_back(a);
            t2.push_back(bt);
            sec2.push_back(s);
            sec2.push_back(s);
            c2.push_back(colc[tn][k]);
            c2.push_back(tn + 1 < ntn ? colc[tn + 1][k] : colc[tn][k]);
            cp.push_back(std::max(c2[c2.size() - 2], c2.back()));
            bundle_p.push_back(direct ? (((int64_t)s << 8) | tm) : -(int64_t)cp.size());
          }
      }
    }
  } else {
    for (int s = 0; s < nsec; ++s) {
      const auto& S = sb.sectors[s];
      const int ib = (int)i2.size();
      i2.insert(i2.end(), per_sector[s].begin(), per_sector[s].end());
      const int ie = (int)i2.size();
      const int rows_p = tc_round8(S.rows), cols_p = tc_round8(S.cols);
      for (int tm = 0; tm < (S.rows + 127) / 128; ++tm)
        for (int tn = 0; tn < (S.cols + nb - 1) / nb; ++tn) {
          const int ha = std::min(128, rows_p - 128 * tm), hb = std::min(nb, cols_p - nb * tn);
          double tile_cost = 0.0;
          for (int x = ib; x < ie; ++x) tile_cost += item_cost(i2[x], hb);
          TcTask t{};
          t.a_rows = rows_p;
          t.b_rows = cols_p;
          t.tm = tm;
          t.tn = tn;
          t.valid_rows = std::min(128, S.rows - 128 * tm);
          t.valid_cols = std::min(nb, S.cols - nb * tn);
          for (int x = ib; x < ie; ++x) mma += 3.0 * 2.0 * 128 * tc_round16(hb) * i2[x].kp;
          if (tile_cost <= chunk || ie - ib <= 1) {
            t.ibeg = ib;
            t.iend = ie;
            t.direct = 1;
            t.out_off = S.offset;
            t.out_kp = S.cols;
            t2.push_back(t);
            c2.push_back(tile_cost);
            sec2.push_back(s);
            bundle2.push_back(((int64_t)s << 8) | tm);
            continue;
          }
          TcTile tl{};
          tl.s_off = S.offset;
          tl.lds = S.cols;
          tl.h = t.valid_rows;
          tl.w = t.valid_cols;
          tl.r0 = 128 * tm;
          tl.c0 = nb * tn;
          tl.pad = hb;  // row stride of the partial slots
          tl.pbeg = (int)slots.size();
          int x0 = ib;
          while (x0 < ie) {
            double acc = 0.0;
            int x1 = x0;
            while (x1 < ie && (acc < chunk || x1 == x0)) acc += item_cost(i2[x1++], hb);
            TcTask u = t;
            u.ibeg = x0;
            u.iend = x1;
            u.direct = 0;
            u.out_off = partial_n;
            slots.push_back(partial_n);
            partial_n += (int64_t)ha * hb;
            t2.push_back(u);
            c2.push_back(acc);
            sec2.push_back(s);
            bundle2.push_back(-(int64_t)t2.size());  // pieces of a split tile spread over blocks
            x0 = x1;
          }
          tl.pend = (int)slots.size();
          tiles.push_back(tl);
        }
    }
  }
  std::vector<double> c1;
  for (const TcTask& t : t1)
    c1.push_back(item_cost(i1[t.ibeg], std::min(nb, t.b_rows - nb * t.tn)) + 200.0);
  laps.lap("phase-2 tasks");
  // tiles inside their operands (item shapes were checked against their
  // sectors when the items were made)
  for (const TcTask& t : t1)
    if (kTcRowsA * t.tm >= t.a_rows || nb * t.tn >= t.b_rows || nb * t.tn >= t.out_kp) fail();
  for (const TcTask& t : t2)
    if (kTcRowsA * t.tm >= t.a_rows || nb * t.tn >= t.b_rows ||
        (t.direct && (t.valid_rows > std::min(kTcRowsA, t.a_rows - kTcRowsA * t.tm) ||
                      t.valid_cols > std::min(nb, t.b_rows - nb * t.tn))))
      fail();
  std::vector<int> o1, o2;
  std::vector<int2> r1, r2, l1, l2;
  if (!seq) {
    // persistent blocks: two per SM with 64-column tiles, one with 128 (and
    // one for the exact kernels)
    const int bps = plan.tcx ? tcx_blocks_per_sm() : tc_blocks_per_sm(nb);
    if (kn.waves) {
      schedule_waves(c1, bps * nsm, o1, r1);
    } else {
      schedule_lpt(c1, H.bundle1, bps * nsm, o1, r1);
    }
    if (pairs) {
      // pairs to clusters of two blocks; block 2c runs the first task of
      // each of cluster c's pairs, block 2c + 1 the second
      std::vector<int> op;
      std::vector<int2> rp;
      schedule_lpt(cp, bundle_p, bps * nsm / 2, op, rp);
      o2.clear();
      r2.clear();
      for (const int2& g : rp)
        for (int rank = 0; rank < 2; ++rank) {
          const int b0 = (int)o2.size();
          for (int k = g.x; k < g.y; ++k) o2.push_back(2 * op[k] + rank);
          r2.push_back(make_int2(b0, (int)o2.size()));
        }
    } else if (kn.waves) {
      schedule_waves(c2, bps * nsm, o2, r2);
    } else {
      schedule_lpt(c2, bundle2, bps * nsm, o2, r2);
    }
  } else {
    // one block per task, tasks grouped by sector, one launch per group
    auto by_sector = [](const std::vector<int>& sec, std::vector<int>& o, std::vector<int2>& r,
                        std::vector<int2>& l) {
      o.resize(sec.size());
      for (size_t i = 0; i < o.size(); ++i) o[i] = (int)i;
      std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return sec[a] < sec[b]; });
      for (size_t i = 0; i < o.size(); ++i) {
        r.push_back(make_int2((int)i, (int)i + 1));
        if (i == 0 || sec[o[i]] != sec[o[i - 1]]) l.push_back(make_int2((int)i, 0));
        ++l.back().y;
      }
    };
    by_sector(H.sec1, o1, r1, l1);
    by_sector(sec2, o2, r2, l2);
  }
  laps.lap("assignment");
  if (partial_n > plan.tc_partial_cap || !plan.tc_partials) {
    if (plan.tc_partials) cudaFreeAsync(plan.tc_partials, stream_);
    plan.tc_partial_cap = std::max<int64_t>(partial_n, 1);
    cuda_check(cudaMallocAsync((void**)&plan.tc_partials, (size_t)plan.tc_partial_cap * sizeof(float2), stream_),
               "tc partials");
  }
  // flatten every block's tasks into its stream of work records; within a
  // task, runs of items with alpha = 1 form accumulation groups of at most
  // kn.group items and kGroupK summed K (f32 accumulation length)
  const int group_items = std::max(1, kn.group);
  constexpr int kGroupK = 1024;
  // blocks are flattened in parallel, each into its own slice of records
  auto flatten = [&](int phase, const std::vector<TcTask>& tasks, const std::vector<TcItem>& items,
                     const std::vector<int>& order, const std::vector<int2>& ranges, std::vector<TcWork>& w,
                     std::vector<int2>& wr) {
    wr.assign(ranges.size(), make_int2(0, 0));
    int64_t nrec = 0;
    for (size_t j = 0; j < ranges.size(); ++j) {
      wr[j].x = (int)nrec;
      for (int k = ranges[j].x; k < ranges[j].y; ++k) {
        const TcTask& T = tasks[order[k]];
        nrec += std::max(1, T.iend - T.ibeg);
      }
      wr[j].y = (int)nrec;
    }
    if (nrec > INT32_MAX) throw std::runtime_error("tensor-core plan: too many work records");
    w.assign(nrec, TcWork{});
    parallel_for((int)ranges.size(), [&](int j) {
      const int2& rg = ranges[j];
      int64_t pos = wr[j].x;
      for (int k = rg.x; k < rg.y; ++k) {
        const TcTask& T = tasks[order[k]];
        TcWork base{};
        base.h_a = (int16_t)std::min(kTcRowsA, T.a_rows - kTcRowsA * T.tm);
        base.h_b = (int16_t)std::min(nb, T.b_rows - nb * T.tn);
        base.valid_rows = (int16_t)T.valid_rows;
        base.valid_cols = (int16_t)T.valid_cols;
        if (phase == 1) {
          base.out_base = T.out_off + 2 * (int64_t)kTcRowsA * T.tm * T.out_kp;
          base.out_ld = T.out_kp;
          base.col0 = nb * T.tn;
        } else if (T.direct) {
          base.out_base = T.out_off + (int64_t)kTcRowsA * T.tm * T.out_kp + nb * T.tn;
          base.out_ld = T.out_kp;
        } else {
          base.out_base = T.out_off;
          base.out_ld = base.h_b;
        }
        const uint8_t f0 = (uint8_t)((T.direct ? kTcDirect : 0) | (phase == 1 && T.stacked ? kTcStacked : 0) |
                                     (phase == 2 && T.ghost ? kTcGhost : 0));
        if (T.ibeg == T.iend) {
          TcWork x = base;
          x.flags = (uint8_t)(f0 | kTcFirst | kTcLast | kTcEmpty);
          w[pos++] = x;
          continue;
        }
        int gn = 0, gk = 0;  // items and K in the open group
        for (int i = T.ibeg; i < T.iend; ++i) {
          const TcItem& it = items[i];
          TcWork x = base;
          x.a_base = it.a_off + 2 * (int64_t)kTcRowsA * T.tm * it.kp;
          x.b_base = it.b_off + 2 * (int64_t)nb * T.tn * it.kp;
          x.kp = it.kp;
          x.alpha = it.alpha;
          x.a_pool = it.a_pool;
          x.b_pool = it.b_pool;
          uint32_t f = f0 | (i == T.ibeg ? kTcFirst : 0) | (i + 1 == T.iend ? kTcLast : 0);
          const bool foldable = phase == 2 && it.alpha == 1.0f;
          if (gn == 0) f |= kTcGStart;
          ++gn;
          gk += it.kp;
          const bool next_joins = foldable && i + 1 < T.iend && items[i + 1].alpha == 1.0f && gn < group_items &&
                                  gk + items[i + 1].kp <= kGroupK;
          if (!next_joins) {
            f |= kTcGEnd;
            gn = gk = 0;
          }
          x.flags = (uint8_t)f;
          w[pos++] = x;
        }
      }
    });
  };
  // exact records: every item its own read-out (no accumulation groups:
  // each item has its own row and column scales), FP64 alpha, pool
  // offsets of six-slice blocks, row-exponent offsets; phase-1 outputs go to
  // the FP64 T buffer (element offset = pool-S offset / kTcxSlices)
  auto flatten_x = [&](int phase, const std::vector<TcTask>& tasks, const std::vector<TcItem>& items,
                       const std::vector<int>& order, const std::vector<int2>& ranges, std::vector<TcxWork>& w,
                       std::vector<int2>& wr) {
    wr.assign(ranges.size(), make_int2(0, 0));
    int64_t nrec = 0;
    for (size_t j = 0; j < ranges.size(); ++j) {
      wr[j].x = (int)nrec;
      for (int k = ranges[j].x; k < ranges[j].y; ++k) {
        const TcTask& T = tasks[order[k]];
        nrec += std::max(1, T.iend - T.ibeg);
      }
      wr[j].y = (int)nrec;
    }
    if (nrec > INT32_MAX) throw std::runtime_error("tensor-core plan: too many work records");
    w.assign(nrec, TcxWork{});
    parallel_for((int)ranges.size(), [&](int j) {
      const int2& rg = ranges[j];
      int64_t pos = wr[j].x;
      for (int k = rg.x; k < rg.y; ++k) {
        const TcTask& T = tasks[order[k]];
        TcxWork base{};
        base.h_a = (int16_t)std::min(kTcRowsA, T.a_rows - kTcRowsA * T.tm);
        base.h_b = (int16_t)std::min(nb, T.b_rows - nb * T.tn);
        base.valid_rows = (int16_t)T.valid_rows;
        base.valid_cols = (int16_t)T.valid_cols;
        if (phase == 1) {
          base.out_base = T.out_off / kTcxSlices + (int64_t)kTcRowsA * T.tm * T.out_kp;
          base.out_ld = T.out_kp;
          base.col0 = nb * T.tn;
        } else if (T.direct) {
          base.out_base = T.out_off + (int64_t)kTcRowsA * T.tm * T.out_kp + nb * T.tn;
          base.out_ld = T.out_kp;
        } else {
          base.out_base = T.out_off;
          base.out_ld = base.h_b;
        }
        const uint8_t f0 = (uint8_t)(T.direct ? kTcDirect : 0);
        if (T.ibeg == T.iend) {
          TcxWork x = base;
          x.flags = (uint8_t)(f0 | kTcFirst | kTcLast | kTcEmpty);
          w[pos++] = x;
          continue;
        }
        for (int i = T.ibeg; i < T.iend; ++i) {
          const TcItem& it = items[i];
          TcxWork x = base;
          x.a_base = it.a_off + (int64_t)kTcxSlices * kTcRowsA * T.tm * it.kp;
          x.b_base = it.b_off + (int64_t)kTcxSlices * nb * T.tn * it.kp;
          x.a_ex = it.a_ex + kTcRowsA * T.tm;
          x.b_ex = it.b_ex + nb * T.tn;
          x.o_ex = it.o_ex + kTcRowsA * T.tm;
          x.kp = it.kp;
          x.alpha = it.alpha64;
          x.a_pool = it.a_pool;
          x.b_pool = it.b_pool;
          x.flags = (uint8_t)(f0 | (i == T.ibeg ? kTcFirst : 0) | (i + 1 == T.iend ? kTcLast : 0) | kTcGStart | kTcGEnd);
          w[pos++] = x;
        }
      }
    });
  };
  std::vector<TcWork> w1, w2;
  std::vector<int2> wr1, wr2;
  if (plan.tcx) {
    std::vector<TcxWork> x1, x2;
    flatten_x(1, t1, i1, o1, r1, x1, wr1);
    flatten_x(2, t2, i2, o2, r2, x2, wr2);
    plan.tcx_w1.release(stream_);
    plan.tcx_w2.release(stream_);
    plan.tcx_w1.upload(x1, stream_);
    plan.tcx_w2.upload(x2, stream_);
  } else {
    flatten(1, t1, i1, o1, r1, w1, wr1);
    flatten(2, t2, i2, o2, r2, w2, wr2);
    if (pairs) {
      // the two blocks of a cluster must stream the same A pieces in the
      // same order (their stages are filled for each other)
      if (wr2.size() % 2) throw std::runtime_error("tensor-core plan: odd number of blocks for cluster pairs");
      for (size_t c = 0; c + 1 < wr2.size(); c += 2) {
        const int2 a = wr2[c], bq = wr2[c + 1];
        if (a.y - a.x != bq.y - bq.x) throw std::runtime_error("tensor-core plan: cluster pair streams differ");
        for (int i = 0; i < a.y - a.x; ++i) {
          const TcWork& x = w2[a.x + i];
          const TcWork& y = w2[bq.x + i];
          const int fx = x.flags & ~(kTcGhost | kTcDirect), fy = y.flags & ~(kTcGhost | kTcDirect);
          if (x.a_base != y.a_base || x.kp != y.kp || x.h_a != y.h_a || x.a_pool != y.a_pool || fx != fy)
            throw std::runtime_error("tensor-core plan: cluster pair streams differ");
        }
      }
    }
  }
  for (auto* d : {&plan.tc_w1, &plan.tc_w2}) d->release(stream_);
  for (auto* d : {&plan.tc_r1, &plan.tc_r2}) d->release(stream_);
  plan.tc_tiles.release(stream_);
  plan.tc_slots.release(stream_);
  plan.tc_w1.upload(w1, stream_);
  plan.tc_w2.upload(w2, stream_);
  plan.tc_r1.upload(wr1, stream_);
  plan.tc_r2.upload(wr2, stream_);
  plan.tc_tiles.upload(tiles, stream_);
  plan.tc_slots.upload(slots, stream_);
  plan.tc_mma_flops = mma;
  plan.tc_l1 = std::move(l1);
  plan.tc_l2 = std::move(l2);
  plan.tc_knobs = kn;
  plan.tc_knobs.nb = nb;
  plan.tc_pairs = pairs;
  {
    int64_t full = 0;
    for (const TcItem& it : i2) full += it.a_pool == kTcPoolS ? 1 : 0;
    const int64_t st[5] = {(int64_t)t1.size(), (int64_t)t2.size(), (int64_t)i2.size(), full, (int64_t)tiles.size()};
    for (int i = 0; i < 5; ++i) plan.tc_stats[i] = st[i];
  }
  laps.lap("flatten + upload");
}

// Autotuner key: slice format, octave of the plan's tensor-core work and the
// histogram of psi-sector shapes (octaves of rows and columns, octave of the
// count per bin), so that superblocks with the same sector structure share
// their tuned knobs.
std::string GpuEngine::tc_tune_key(const Superblock& sb, const SigmaPlan& p) const {
  auto oct = [](double x) {
    int b = 0;
    while (x >= 2.0 && b < 80) {
      x *= 0.5;
      ++b;
    }
    return b;
  };
  std::map<std::pair<int, int>, int> hist;
  for (const auto& S : sb.sectors) ++hist[{oct(S.rows), oct(S.cols)}];
  std::string k = std::string(p.tc_fp16 ? "fp16" : "bf16") + "/w" + std::to_string(oct(p.flops));
  for (const auto& h : hist)
    k += "/" + std::to_string(h.first.first) + "x" + std::to_string(h.first.second) + ":" + std::to_string(oct(h.second));
  return k;
}

// Tile shape and schedule knobs: for each output-tile width (64 columns with
// two pipelines per SM, 128 with one; the pools are packed again for each),
// a coordinate search over the schedule knobs (LPT item cost, phase-2 split,
// accumulation group), each candidate timed by CUDA events over three
// products on the plan's own operators; a candidate replaces the best one
// when it is at least 2 % faster.  Keys seen before reuse their choice.
void GpuEngine::autotune_tc(const Superblock& sb, SigmaPlan& p) {
  p.tc_tuned = true;  // also stops sigma_tc from re-entering
  const std::string key = tc_tune_key(sb, p);
  auto use_nb = [&](int nb) {
    if (p.tc_nb == nb && p.tc) return;
    free_tc(p);
    p.tc_nb = nb;
    p.tc_nb_set = true;
    plan_tc(sb, p);
    p.tc_tuned = true;
  };
  auto it = tune_cache.find(key);
  if (it != tune_cache.end()) {
    TcKnobs k = it->second;
    k.per_sector = 0;
    use_nb(k.nb);
    if (!(k == p.tc_knobs)) schedule_tc(sb, p, k);
    return;
  }
  const auto t0 = std::chrono::steady_clock::now();
  const double f0 = sigma_flops;
  const long c0 = sigma_calls;
  double* x = alloc(p.n);
  double* y = alloc(p.n);
  cuda_check(dev::launch_fill(x, 1.0 / std::sqrt((double)std::max<int64_t>(p.n, 1)), p.n, stream_), "fill");
  cudaEvent_t e[2];
  for (auto& v : e) cuda_check(cudaEventCreate(&v), "event");
  auto measure = [&]() {
    sigma_tc(sb, p, x, y);
    cuda_check(cudaEventRecord(e[0], stream_), "record");
    for (int r = 0; r < 3; ++r) sigma_tc(sb, p, x, y);
    cuda_check(cudaEventRecord(e[1], stream_), "record");
    sync();
    float ms = 0.f;
    cuda_check(cudaEventElapsedTime(&ms, e[0], e[1]), "elapsed");
    return (double)ms;
  };
  const double costs[] = {150.0, 400.0, 1000.0};
  const double splits[] = {1.5, 3.0, 6.0};
  const int groups[] = {8, 16, 32};
  TcKnobs best;
  double tbest = 1e300;
  const int first_nb = p.tc_nb;
  for (int nb : {first_nb, first_nb == dev::kTcRowsB ? dev::kTcRowsBWide : dev::kTcRowsB}) {
    use_nb(nb);
    TcKnobs b = p.tc_knobs;
    b.per_sector = 0;
    if (!(b == p.tc_knobs)) schedule_tc(sb, p, b);
    double tb = measure();
    for (int axis = 0; axis < 3; ++axis)
      for (int v = 0; v < 3; ++v) {
        TcKnobs c = b;
        if (axis == 0) c.item_cost = costs[v];
        if (axis == 1) c.split = splits[v];
        if (axis == 2) c.group = groups[v];
        if (c == b) continue;
        schedule_tc(sb, p, c);
        const double t = measure();
        if (t < 0.98 * tb) {
          b = c;
          tb = t;
        }
      }
    if (tb < 0.98 * tbest || nb == first_nb) {
      best = b;
      tbest = tb;
    }
  }
  use_nb(best.nb);
  if (!(best == p.tc_knobs)) schedule_tc(sb, p, best);
  for (auto& v : e) cudaEventDestroy(v);
  free(x);
  free(y);
  sync();
  sigma_flops = f0;
  sigma_calls = c0;
  tune_cache[key] = best;
  if (!tune_cache_path.empty()) {
    if (FILE* f = std::fopen(tune_cache_path.c_str(), "a")) {
      std::fprintf(f, "%s %.17g %.17g %d %d\n", key.c_str(), best.item_cost, best.split, best.group, best.nb);
      std::fclose(f);
    }
  }
  ++tune_runs;
  tune_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void GpuEngine::load_tune_cache(const std::string& path) {
  tune_cache_path = path;
  tune_cache.clear();  // a cache file replaces the choices held so far
  if (path.empty()) return;
  FILE* f = std::fopen(path.c_str(), "r");
  if (!f) return;
  char line[8192], key[4096];
  while (std::fgets(line, sizeof(line), f)) {
    TcKnobs k;
    const int got = std::sscanf(line, "%4095s %lf %lf %d %d", key, &k.item_cost, &k.split, &k.group, &k.nb);
    if (got < 4) continue;
    if (got == 4) k.nb = dev::kTcRowsB;  // files written before the tile width was tuned
    if (k.item_cost > 0 && k.split > 0 && k.group > 0 && (k.nb == dev::kTcRowsB || k.nb == dev::kTcRowsBWide))
      tune_cache[key] = k;
  }
  std::fclose(f);
}

void GpuEngine::sigma_tc(const Superblock& sb, SigmaPlan& p, const double* psi, double* out, cudaEvent_t* marks) {
  if (p.tc && p.tcx) {  // packed for the exact kernels
    free_tc(p);
    p.tc_nb_set = false;
  }
  p.tcx = false;
  const bool fp16 = precision == Precision::FP16X2_TC;
  if (p.tc && p.tc_fp16 != fp16) free_tc(p);  // operators packed in the other format
  if (p.tc && tc_nb_mode && tc_nb_mode != p.tc_nb) {  // packed for the other tile width
    free_tc(p);
    p.tc_nb_set = false;
  }
  if (p.tc && p.tc_stack_used != tc_stack_rows) free_tc(p);  // stacked for another limit
  if (!p.tc) plan_tc(sb, p);
  if (p.tc_knobs.per_sector != (tc_schedule_mode == 1 ? 1 : 0)) {
    TcKnobs k = tc_default_knobs();
    k.per_sector = tc_schedule_mode == 1 ? 1 : 0;
    schedule_tc(sb, p, k);
    p.tc_tuned = false;
  }
  if (tc_autotune && !p.tc_knobs.per_sector && !p.tc_tuned) autotune_tc(sb, p);
  dev::TcBufs b{};
  b.src[0] = arena(*sb.L);
  b.src[1] = arena(*sb.R);
  b.src[2] = psi;
  for (int i = 0; i < dev::kTcPools; ++i) {
    b.pool[i] = p.tc_pool[i];
  }
  b.rows = p.tc_rows.d;
  b.partials = p.tc_partials;
  b.status = tc_status_;
  b.fp16 = fp16 ? 1 : 0;
  constexpr uint64_t kWaitLimitNs = 1000000000ull;
  cuda_check(dev::launch_tc_pack(b, p.tc_psi_pack.d, (int)p.tc_psi_pack.n, stream_), "tc pack psi");
  if (marks) cuda_check(cudaEventRecord(marks[0], stream_), "record");
  if (p.tc_knobs.per_sector) {
    // baseline: one launch per psi sector (phase 1) and per sigma sector
    // (phase 2), one block per task
    for (const int2& g : p.tc_l1)
      cuda_check(dev::launch_tc_sigma(1, p.tc_nb, b, p.tc_w1.d, p.tc_r1.d + g.x, g.y, out, kWaitLimitNs, stream_),
                 "tc phase 1");
    for (const int2& g : p.tc_l2)
      cuda_check(dev::launch_tc_sigma(2, p.tc_nb, b, p.tc_w2.d, p.tc_r2.d + g.x, g.y, out, kWaitLimitNs, stream_),
                 "tc phase 2");
  } else {
    cuda_check(dev::launch_tc_sigma(1, p.tc_nb, b, p.tc_w1.d, p.tc_r1.d, (int)p.tc_r1.n, out, kWaitLimitNs, stream_),
               "tc phase 1");
    if (p.tc_pairs)
      cuda_check(dev::launch_tc_sigma_pairs(b, p.tc_w2.d, p.tc_r2.d, (int)p.tc_r2.n, out, kWaitLimitNs, stream_),
                 "tc phase 2 (cluster pairs)");
    else
      cuda_check(dev::launch_tc_sigma(2, p.tc_nb, b, p.tc_w2.d, p.tc_r2.d, (int)p.tc_r2.n, out, kWaitLimitNs, stream_),
                 "tc phase 2");
  }
  if (marks) cuda_check(cudaEventRecord(marks[1], stream_), "record");
  cuda_check(dev::launch_tc_reduce(b, p.tc_tiles.d, p.tc_slots.d, (int)p.tc_tiles.n, out, stream_), "tc reduce");
  if (p.ecore != 0.0) cuda_check(dev::launch_axpy(p.ecore, psi, out, p.n, stream_), "ecore");
  cuda_check(cudaMemcpyAsync(tc_status_host_, tc_status_, sizeof(int), cudaMemcpyDeviceToHost, stream_), "status");
  sigma_flops += p.flops;
  ++sigma_calls;
}

// Exact-slice product (plan p.tcx): psi's row exponents and digits, phase 1
// (T in FP64, its row exponents reduced by the kernel), T's digits into pool
// S, phase 2, FP64 sum of split tiles.
void GpuEngine::sigma_tcx(const Superblock& sb, SigmaPlan& p, const double* psi, double* out) {
  if (!p.tcx) throw std::logic_error("sigma_tcx: not an exact-slice plan");
  if (!p.tc) plan_tc(sb, p);
  dev::TcxBufs b{};
  b.src[0] = arena(*sb.L);
  b.src[1] = arena(*sb.R);
  b.src[2] = psi;
  b.src[3] = p.tcx_t;
  for (int i = 0; i < dev::kTcPools; ++i) {
    b.pool[i] = p.tc_pool[i];
    b.ex[i] = p.tcx_ex[i];
  }
  b.t = p.tcx_t;
  b.partials = reinterpret_cast<double*>(p.tc_partials);
  b.status = tc_status_;
  constexpr uint64_t kWaitLimitNs = 1000000000ull;
  cuda_check(dev::launch_tcx_rowexp(b, p.tc_psi_pack.d, (int)p.tc_psi_pack.n, stream_), "tcx psi exponents");
  cuda_check(dev::launch_tcx_pack(b, p.tc_psi_pack.d, (int)p.tc_psi_pack.n, stream_), "tcx pack psi");
  cuda_check(dev::launch_fill_int(p.tcx_ex[dev::kTcPoolS], p.tcx_ex_n[dev::kTcPoolS], dev::kTcxNoExp, stream_),
             "tcx T exponents");
  cuda_check(dev::launch_tcx_sigma(1, b, p.tcx_w1.d, p.tc_r1.d, (int)p.tc_r1.n, out, kWaitLimitNs, stream_),
             "tcx phase 1");
  cuda_check(dev::launch_tcx_pack(b, p.tcx_tpack.d, (int)p.tcx_tpack.n, stream_), "tcx pack T");
  cuda_check(dev::launch_tcx_sigma(2, b, p.tcx_w2.d, p.tc_r2.d, (int)p.tc_r2.n, out, kWaitLimitNs, stream_),
             "tcx phase 2");
  cuda_check(dev::launch_tcx_reduce(b, p.tc_tiles.d, p.tc_slots.d, (int)p.tc_tiles.n, out, stream_), "tcx reduce");
  if (p.ecore != 0.0) cuda_check(dev::launch_axpy(p.ecore, psi, out, p.n, stream_), "ecore");
  cuda_check(cudaMemcpyAsync(tc_status_host_, tc_status_, sizeof(int), cudaMemcpyDeviceToHost, stream_), "status");
  sigma_flops += p.flops;
  ++sigma_calls;
}

void GpuEngine::sigma_exact(const Superblock& sb, const SigmaPlan& ref, const double* psi, double* out) {
  // device bytes of one exact plan: six digit slices (12 B) per packed
  // element of every pool, and the FP64 stage-1 products (8 B each); the
  // split plan's pools hold two bf16 slices (4 B) per packed element
  int64_t split_elems = 0;
  for (int i = 0; i < dev::kTcPools; ++i) split_elems += ref.tc_pool_elems[i];
  double need = 6.0 * (double)split_elems + 4.0 * (double)ref.tc_pool_elems[dev::kTcPoolS];
  if (split_elems == 0) need = 0.0;  // no split plan to size from: one chunk
  sync();
  size_t free_b = 0, total_b = 0;
  cuda_check(cudaMemGetInfo(&free_b, &total_b), "memory info");
  const int nterm = (int)sb.terms.size();
  int nchunks = need > 0.0 ? (int)std::ceil(need / (0.8 * (double)free_b)) : 1;
  nchunks = std::max(1, std::min(nchunks, std::max(1, nterm)));
  for (;;) {
    bool ok = true;
    double* tmp = nullptr;
    try {
      if (nchunks > 1) tmp = alloc(sb.size);
      for (int c = 0; c < nchunks && ok; ++c) {
        Superblock part = sb;
        const int t0 = (int)((int64_t)nterm * c / nchunks), t1 = (int)((int64_t)nterm * (c + 1) / nchunks);
        part.terms.assign(sb.terms.begin() + t0, sb.terms.begin() + t1);
        part.ecore = c == 0 ? sb.ecore : 0.0;
        SigmaPlan xp;
        xp.tcx = true;
        xp.n = ref.n;
        xp.ecore = part.ecore;
        xp.flops = ref.flops * (double)(t1 - t0) / std::max(1, nterm);
        try {
          plan_tc(part, xp);
          sigma_tcx(part, xp, psi, nchunks > 1 ? tmp : out);
          sync();
        } catch (const CudaError&) {
          cudaGetLastError();
          free_plan(xp);
          sync();
          ok = false;
          break;
        }
        free_plan(xp);
        if (nchunks > 1) {
          if (c == 0) cuda_check(cudaMemcpyAsync(out, tmp, sb.size * sizeof(double), cudaMemcpyDeviceToDevice, stream_), "copy");
          else cuda_check(dev::launch_axpy(1.0, tmp, out, sb.size, stream_), "sum of chunks");
        }
      }
    } catch (const CudaError&) {  // the chunk buffer itself
      cudaGetLastError();
      ok = false;
    }
    if (tmp) free(tmp);
    sync();
    if (ok) break;
    if (nchunks >= std::max(1, nterm) || nchunks >= 64) throw CudaError("exact product: device memory too small");
    nchunks = std::min(std::max(1, nterm), nchunks * 2);
    ++exact_fallbacks_;
  }
  last_exact_chunks_ = nchunks;
}

void GpuEngine::gemm_exact(const dev::Bufs& bufs, const std::vector<dev::GemmUnit>& units,
                           const std::vector<dev::GemmItem>& items) {
  using namespace dev;
  if (units.empty()) return;
  const int c_buf = units[0].c_buf;
  std::vector<TcPack> packs;
  packs.reserve(2 * items.size());
  int64_t pool_n[2] = {0, 0}, ex_n[2] = {0, 0};
  struct Ref {
    int64_t off;
    int32_t ex;
  };
  std::vector<Ref> aref(items.size()), bref(items.size());
  for (const GemmUnit& u : units) {
    if (u.c_buf != c_buf || u.beta_one) throw std::logic_error("gemm_exact: one output buffer, overwritten");
    for (int i = u.ibeg; i < u.iend; ++i) {
      const GemmItem& g = items[i];
      TcPack a{};  // A view: u.m x k
      a.src = g.a_buf;
      a.src_off = g.a_off;
      a.ld = g.lda;
      a.trans = g.ta;
      a.rows_v = u.m;
      a.cols_v = g.k;
      a.rows_p = tc_round8(u.m);
      a.kp = tc_round16(g.k);
      a.rt = kTcRowsA;
      a.pool = kTcPoolL;
      a.dst_off = pool_n[0];
      a.ex_off = (int32_t)ex_n[0];
      pool_n[0] += (int64_t)kTcxSlices * a.rows_p * a.kp;
      ex_n[0] += a.rows_p;
      aref[i] = {a.dst_off, a.ex_off};
      packs.push_back(a);
      TcPack b{};  // B^T view: u.n x k (element (j, kk) = op(B)(kk, j))
      b.src = g.b_buf;
      b.src_off = g.b_off;
      b.ld = g.ldb;
      b.trans = g.tb ? 0 : 1;
      b.rows_v = u.n;
      b.cols_v = g.k;
      b.rows_p = tc_round8(u.n);
      b.kp = tc_round16(g.k);
      b.rt = kTcxNB;
      b.pool = kTcPoolR;
      b.dst_off = pool_n[1];
      b.ex_off = (int32_t)ex_n[1];
      pool_n[1] += (int64_t)kTcxSlices * b.rows_p * b.kp;
      ex_n[1] += b.rows_p;
      bref[i] = {b.dst_off, b.ex_off};
      packs.push_back(b);
    }
  }
  if (ex_n[0] > INT32_MAX || ex_n[1] > INT32_MAX) throw std::runtime_error("gemm_exact: too many rows");
  // tasks: 128 x 64 tiles of every unit, with the unit's items
  struct Task {
    int u, tm, tn;
  };
  std::vector<Task> tasks;
  std::vector<double> cost;
  for (int u = 0; u < (int)units.size(); ++u) {
    const GemmUnit& U = units[u];
    for (int tm = 0; tm < (U.m + kTcRowsA - 1) / kTcRowsA; ++tm)
      for (int tn = 0; tn < (U.n + kTcxNB - 1) / kTcxNB; ++tn) {
        tasks.push_back({u, tm, tn});
        double c = 400.0;
        for (int i = U.ibeg; i < U.iend; ++i) c += 400.0 + tc_round16(items[i].k);
        cost.push_back(c);
      }
  }
  std::vector<int64_t> bundle(tasks.size());
  for (size_t t = 0; t < tasks.size(); ++t) bundle[t] = -(int64_t)t - 1;
  std::vector<int> order;
  std::vector<int2> ranges;
  schedule_lpt(cost, bundle, tcx_blocks_per_sm() * sm_count(), order, ranges);
  std::vector<TcxWork> w;
  std::vector<int2> wr(ranges.size());
  for (size_t j = 0; j < ranges.size(); ++j) {
    wr[j].x = (int)w.size();
    for (int k = ranges[j].x; k < ranges[j].y; ++k) {
      const Task& T = tasks[order[k]];
      const GemmUnit& U = units[T.u];
      TcxWork base{};
      base.h_a = (int16_t)std::min(kTcRowsA, tc_round8(U.m) - kTcRowsA * T.tm);
      base.h_b = (int16_t)std::min(kTcxNB, tc_round8(U.n) - kTcxNB * T.tn);
      base.valid_rows = (int16_t)std::min(kTcRowsA, U.m - kTcRowsA * T.tm);
      base.valid_cols = (int16_t)std::min(kTcxNB, U.n - kTcxNB * T.tn);
      base.out_base = U.c_off + (int64_t)kTcRowsA * T.tm * U.ldc + kTcxNB * T.tn;
      base.out_ld = U.ldc;
      if (U.ibeg == U.iend) {
        TcxWork x = base;
        x.flags = (uint8_t)(kTcDirect | kTcFirst | kTcLast | kTcEmpty);
        w.push_back(x);
        continue;
      }
      for (int i = U.ibeg; i < U.iend; ++i) {
        const GemmItem& g = items[i];
        TcxWork x = base;
        const int kp = tc_round16(g.k);
        x.a_base = aref[i].off + (int64_t)kTcxSlices * kTcRowsA * T.tm * kp;
        x.b_base = bref[i].off + (int64_t)kTcxSlices * kTcxNB * T.tn * kp;
        x.a_ex = aref[i].ex + kTcRowsA * T.tm;
        x.b_ex = bref[i].ex + kTcxNB * T.tn;
        x.kp = kp;
        x.alpha = g.alpha;
        x.a_pool = kTcPoolL;
        x.b_pool = kTcPoolR;
        x.flags = (uint8_t)(kTcDirect | (i == U.ibeg ? kTcFirst : 0) | (i + 1 == U.iend ? kTcLast : 0) |
                            kTcGStart | kTcGEnd);
        w.push_back(x);
      }
    }
    wr[j].y = (int)w.size();
  }
  TcxBufs xb{};
  for (int i = 0; i < 4; ++i) xb.src[i] = bufs.p[i];
  __nv_bfloat16* pools[2] = {nullptr, nullptr};
  int* exs[2] = {nullptr, nullptr};
  auto release = [&]() {
    for (int i = 0; i < 2; ++i) {
      if (pools[i]) cudaFreeAsync(pools[i], stream_);
      if (exs[i]) cudaFreeAsync(exs[i], stream_);
      pools[i] = nullptr;
      exs[i] = nullptr;
    }
  };
  DevArray<TcPack> dp;
  DevArray<TcxWork> dw;
  DevArray<int2> dr;
  try {
    for (int i = 0; i < 2; ++i) {
      cuda_check(cudaMallocAsync((void**)&pools[i], (size_t)std::max<int64_t>(pool_n[i], 8) * sizeof(__nv_bfloat16),
                                 stream_),
                 "exact gemm pool");
      cuda_check(cudaMallocAsync((void**)&exs[i], (size_t)std::max<int64_t>(ex_n[i], 1) * sizeof(int), stream_),
                 "exact gemm exponents");
    }
    dp.upload(packs, stream_);
    dw.upload(w, stream_);
    dr.upload(wr, stream_);
  } catch (...) {
    // nothing was launched: the caller may run the FP64 path instead
    dp.release(stream_);
    dw.release(stream_);
    dr.release(stream_);
    release();
    throw;
  }
  xb.pool[kTcPoolL] = pools[0];
  xb.pool[kTcPoolR] = pools[1];
  xb.ex[kTcPoolL] = exs[0];
  xb.ex[kTcPoolR] = exs[1];
  xb.status = tc_status_;
  constexpr uint64_t kWaitLimitNs = 1000000000ull;
  cuda_check(launch_tcx_rowexp(xb, dp.d, (int)packs.size(), stream_), "exact gemm exponents");
  cuda_check(launch_tcx_pack(xb, dp.d, (int)packs.size(), stream_), "exact gemm pack");
  cuda_check(launch_tcx_sigma(2, xb, dw.d, dr.d, (int)wr.size(), bufs.p[c_buf], kWaitLimitNs, stream_),
             "exact gemm");
  dp.release(stream_);
  dw.release(stream_);
  dr.release(stream_);
  release();
}

void GpuEngine::sigma_any(const Superblock& sb, SigmaPlan& p, const double* psi, double* out) {
  if (precision == Precision::EXACT_TC) {
    p.reuse_pools = false;
    if (p.tc && !p.tcx) free_tc(p);  // packed for the split kernels
    if (p.scratch) {  // FP64 intermediates (allocated again by an FP64 product)
      free(p.scratch);
      p.scratch = nullptr;
    }
    p.tcx = true;
    sigma_tcx(sb, p, psi, out);
    return;
  }
  const int ns = precision_slices(precision);
  if (precision_tc(precision)) sigma_tc(sb, p, psi, out);
  else if (ns) sigma_split(sb, p, ns, psi, out);
  else sigma(sb, p, psi, out);
}

int GpuEngine::sigma_launches(const SigmaPlan& p) const {
  if (precision_tc(precision)) {  // pack psi, phase 1, phase 2, reduce of split tiles
    const int phases = (p.tc && p.tc_knobs.per_sector) ? (int)(p.tc_l1.size() + p.tc_l2.size()) : 2;
    return 1 + phases + (p.tc && p.tc_tiles.n == 0 ? 0 : 1) + (p.ecore != 0.0 ? 1 : 0);
  }
  if (precision_slices(precision)) return 3 + (p.ecore != 0.0 ? 1 : 0);  // slice psi, fused, reduce (+ecore)
  return (p.t1.n ? 1 : 0) + (p.t2.n ? 1 : 0) + (p.ru.n ? 1 : 0) + (p.ecore != 0.0 ? 1 : 0);
}

void GpuEngine::sigma_timed(const Superblock& sb, const SigmaPlan& p, const double* psi, double* out, int reps,
                            float* ms) {
  ms[0] = ms[1] = ms[2] = 0.f;
  if (precision == Precision::EXACT_TC) {
    SigmaPlan& pm = const_cast<SigmaPlan&>(p);
    sigma_any(sb, pm, psi, out);  // plans and packs the operators outside the timed region
    sync();
    cudaEvent_t e0, e1;
    cuda_check(cudaEventCreate(&e0), "event");
    cuda_check(cudaEventCreate(&e1), "event");
    for (int r = 0; r < reps; ++r) {
      cuda_check(cudaEventRecord(e0, stream_), "record");
      sigma_any(sb, pm, psi, out);
      cuda_check(cudaEventRecord(e1, stream_), "record");
      cuda_check(cudaEventSynchronize(e1), "sync");
      float a;
      cudaEventElapsedTime(&a, e0, e1);
      ms[0] += a;
      ms[1] += a;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    sync();  // raises if a pipeline wait ran out
    return;
  }
  if (!precision_slices(precision) && !p.scratch) p.scratch = alloc(p.scratch_elems);
  dev::Bufs bufs{};
  bufs.p[0] = arena(*sb.L);
  bufs.p[1] = arena(*sb.R);
  bufs.p[2] = const_cast<double*>(psi);
  bufs.p[3] = out;
  bufs.p[4] = p.scratch;
  cudaEvent_t e[4];
  for (auto& x : e) cuda_check(cudaEventCreate(&x), "event");
  ms[0] = ms[1] = ms[2] = 0.f;
  const int ns = precision_slices(precision);
  if (ns) {
    SigmaPlan& pm = const_cast<SigmaPlan&>(p);
    auto call = [&](cudaEvent_t* marks) {
      if (precision_tc(precision)) sigma_tc(sb, pm, psi, out, marks);
      else sigma_split(sb, pm, ns, psi, out, marks);
    };
    call(nullptr);  // slices / packs operators and buffers outside the timed region
    sync();
    for (int r = 0; r < reps; ++r) {
      cuda_check(cudaEventRecord(e[0], stream_), "record");
      call(e + 1);
      cuda_check(cudaEventRecord(e[3], stream_), "record");
      cuda_check(cudaEventSynchronize(e[3]), "sync");
      float a, b;
      cudaEventElapsedTime(&a, e[0], e[3]);
      cudaEventElapsedTime(&b, e[1], e[2]);
      ms[0] += a;
      ms[1] += b;  // tensor-core kernels alone
      ms[2] += a - b;
    }
    for (auto& x : e) cudaEventDestroy(x);
    sync();
    return;
  }
  for (int r = 0; r < reps; ++r) {
    cuda_check(cudaEventRecord(e[0], stream_), "record");
    cuda_check(dev::launch_gemm(bufs, p.u1.d, p.i1.d, p.t1.d, (int)p.t1.n, stream_), "sigma stage 1");
    cuda_check(cudaEventRecord(e[1], stream_), "record");
    cuda_check(dev::launch_gemm(bufs, p.u2.d, p.i2.d, p.t2.d, (int)p.t2.n, stream_), "sigma stage 2");
    cuda_check(dev::launch_copy(bufs, out, p.ru.d, p.ri.d, (int)p.ru.n, stream_), "sigma stage-2 partial sums");
    cuda_check(cudaEventRecord(e[2], stream_), "record");
    if (p.ecore != 0.0) cuda_check(dev::launch_axpy(p.ecore, psi, out, p.n, stream_), "ecore");
    cuda_check(cudaEventRecord(e[3], stream_), "record");
    cuda_check(cudaEventSynchronize(e[3]), "sync");
    float a, b, c;
    cudaEventElapsedTime(&a, e[0], e[3]);
    cudaEventElapsedTime(&b, e[0], e[1]);
    cudaEventElapsedTime(&c, e[1], e[2]);
    ms[0] += a;
    ms[1] += b;
    ms[2] += c;
    sigma_flops += p.flops;
    ++sigma_calls;
  }
  for (auto& x : e) cudaEventDestroy(x);
}

void GpuEngine::hdiag(const Superblock& sb, const SigmaPlan& p, double* d) {
  dev::Bufs bufs{};
  bufs.p[0] = arena(*sb.L);
  bufs.p[1] = arena(*sb.R);
  cuda_check(dev::launch_fill(d, sb.ecore, sb.size, stream_), "fill");
  cuda_check(dev::launch_diag_tiles(bufs, d, p.du.d, p.di.d, p.dtask.d, (int)p.dtask.n, stream_), "hdiag");
}

// ------------------------------------------------------------------ Davidson

// Linear::block_davidson (linear.C:179-385) with the vectors, every O(n)
// pass and every steering scalar on the GPU.  The first iteration's sigma
// vectors and subspace matrix are formed eagerly; every later iteration is
// one launch of a captured CUDA graph (the sigma of the newest basis vector,
// its subspace row, the subspace eigenproblem, Ritz rotation, residual with
// Olsen correction, convergence / deflation decisions, Gram-Schmidt and the
// append), after which the host reads a 296-byte header to stop the loop.
// dav_graph = false (BGPU_DAVIDSON_GRAPH=0) issues the same launches without
// capture.
//
// After a Ritz rotation the basis diagonalises the projected Hamiltonian, so
// the subspace matrix of the next iteration is diag(Ritz values) bordered by
// the row of the new vector (b_new . sigma_j), instead of the reference's
// full recomputation of b_i . sigma_j: the same matrix up to rounding, at
// O(k n) instead of O(k^2 n) memory traffic per iteration.
void GpuEngine::prepare_plan(const Superblock& sb) {
  if (have_plan_) free_plan(plan_);
  plan_.reuse_pools = true;
  plan_sigma(sb, plan_);
  if (precision_tc(precision)) plan_tc(sb, plan_);
  have_plan_ = true;
  prepared_ = true;
}

int GpuEngine::solve(const Superblock& sb, const DavidsonParams& p, std::vector<double>& energies) {
  // work lists compiled by prepare_plan for this superblock, else now
  if (!prepared_ || !have_plan_ || plan_.n != sb.size) prepare_plan(sb);
  prepared_ = false;
  const int64_t n = sb.size;
  const int nroots = p.nroots;
  if (n < nroots) throw std::runtime_error("superblock smaller than number of roots");
  const int kmax = std::max(p.deflation_max, nroots) + 1;
  if (kmax > dev::kDavMax) throw std::runtime_error("Davidson subspace larger than 32 vectors");
  if (p.deflation_min < nroots || p.deflation_min >= p.deflation_max)
    throw std::runtime_error("Davidson deflation sizes must satisfy nroots <= min < max");
  // buffers and graphs of this solve, released on every exit
  struct Scope {
    GpuEngine& e;
    std::vector<double*> bufs;
    dev::DavCtl* ctl = nullptr;
    cudaGraphExec_t gx[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    ~Scope() {
      cudaStreamSynchronize(e.stream_);
      for (auto& g : gx)
        if (g) cudaGraphExecDestroy(g);
      for (auto& x : ev)
        if (x) cudaEventDestroy(x);
      for (double* q : bufs) e.free(q);
      if (ctl) cudaFreeAsync(ctl, e.stream_);
    }
  } sc{*this};
  auto buf = [&](int64_t elems) {
    sc.bufs.push_back(alloc(elems));
    return sc.bufs.back();
  };
  double* diag = buf(n);
  double* B = buf((int64_t)kmax * n);
  double* S = buf((int64_t)kmax * n);
  double* r = buf(n);
  double* y = buf(n);
  double* work = buf((int64_t)dev::kDavBlocks * dev::kDavMax);
  double* red = buf(dev::kDavMax);
  cuda_check(cudaMallocAsync((void**)&sc.ctl, sizeof(dev::DavCtl), stream_), "alloc");
  for (auto& x : sc.ev) cuda_check(cudaEventCreate(&x), "event");
  PlanLaps laps{"davidson"};
  laps.lap("plan");
  hdiag(sb, plan_, diag);
  if (p.use_guess && guess_ && guess_n_ == n && nguess_ >= nroots) {
    // transformed previous wavefunctions (orthonormalised below)
    cuda_check(cudaMemcpyAsync(B, guess_, (size_t)nroots * n * sizeof(double), cudaMemcpyDeviceToDevice, stream_),
               "guess");
  } else {
    // basic guess (as the oracle): unit vectors on the lowest diagonal + small noise
    std::vector<double> hd(n);
    cuda_check(cudaMemcpyAsync(hd.data(), diag, n * sizeof(double), cudaMemcpyDeviceToHost, stream_), "d2h diag");
    sync();
    std::vector<int64_t> order(n);
    for (int64_t i = 0; i < n; ++i) order[i] = i;
    std::partial_sort(order.begin(), order.begin() + nroots, order.end(),
                      [&](int64_t a, int64_t b) { return hd[a] < hd[b]; });
    Rng rng(p.seed);
    std::vector<double> g((size_t)nroots * n);
    for (int rr = 0; rr < nroots; ++rr) {
      for (int64_t i = 0; i < n; ++i) g[(size_t)rr * n + i] = 1e-3 * (rng.uniform() - 0.5);
      g[(size_t)rr * n + order[rr]] = 1.0;
    }
    cuda_check(cudaMemcpyAsync(B, g.data(), g.size() * sizeof(double), cudaMemcpyHostToDevice, stream_), "guess");
    sync();
  }
  auto row = [&](double* M, int i) { return M + (int64_t)i * n; };
  auto dots = [&](const double* X, int nx, const double* v, double* out) {
    cuda_check(dev::launch_gram(X, nx, v, 1, n, n, work, red, stream_), "dot");
    cuda_check(cudaMemcpyAsync(out, red, nx * sizeof(double), cudaMemcpyDeviceToHost, stream_), "d2h");
    sync();
  };
  laps.lap("diag + guess");
  for (int i = 0; i < nroots; ++i) {
    double h;
    for (int j = 0; j < i; ++j) {
      dots(row(B, j), 1, row(B, i), &h);
      cuda_check(dev::launch_axpy(-h, row(B, j), row(B, i), n, stream_), "gs");
    }
    dots(row(B, i), 1, row(B, i), &h);
    cuda_check(dev::launch_scale(1.0 / std::sqrt(h), row(B, i), n, stream_), "norm");
  }
  auto count_sigma = [&](double dt) {
    sigma_seconds += dt;
    if (precision_slices(precision)) {
      split_seconds += dt;
      ++split_calls;
    } else {
      fp64_seconds += dt;
      ++fp64_calls;
    }
  };
  if (precision_tc(precision) && !plan_.tc) {
    plan_tc(sb, plan_);
    laps.lap("tensor-core plan");
  }
  // first iteration: sigma of every start vector, whole subspace matrix
  // h_ij = b_i . sigma_j (j <= i, symmetrised as linear.C:268-272)
  for (int i = 0; i < nroots; ++i) {
    auto t0 = std::chrono::steady_clock::now();
    sigma_any(sb, plan_, row(B, i), row(S, i));
    sync();
    count_sigma(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
  }
  dev::DavCtl c0{};
  {
    std::vector<double> col(nroots);
    for (int j = 0; j < nroots; ++j) {
      dots(B, nroots, row(S, j), col.data());  // b_i . sigma_j
      for (int i = j; i < nroots; ++i) c0.h[i * nroots + j] = c0.h[j * nroots + i] = col[i];
    }
  }
  c0.k = nroots;
  c0.mode = 2;
  cuda_check(cudaMemcpyAsync(sc.ctl, &c0, sizeof(c0), cudaMemcpyHostToDevice, stream_), "h2d ctl");
  sync();
  laps.lap("first sigma + subspace");
  dev::DavBufs db{B, S, r, diag, y, work, sc.ctl, n, nroots, p.deflation_min, p.deflation_max, p.tol};
  // one iteration; with_sigma: the newest basis vector (left in r) has no sigma yet
  // (event records inside a capture become external event nodes; outside a
  // capture the external flag is refused)
  auto enqueue = [&](bool with_sigma, bool capturing) {
    const unsigned rec = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    if (with_sigma) {
      cuda_check(cudaEventRecordWithFlags(sc.ev[0], stream_, rec), "record");
      sigma_any(sb, plan_, r, y);
      cuda_check(cudaEventRecordWithFlags(sc.ev[1], stream_, rec), "record");
      cuda_check(dev::launch_dav_new_row(db, stream_), "davidson row");
    }
    cuda_check(dev::launch_dav_update(db, stream_), "davidson update");
    cuda_check(cudaMemcpyAsync(dav_host_, sc.ctl, dev::kDavHeaderBytes, cudaMemcpyDeviceToHost, stream_), "d2h ctl");
  };
  const bool use_graph = dav_graph;
  auto capture = [&](bool with_sigma) {
    const double f0 = sigma_flops;
    const long c0n = sigma_calls;
    cudaGraph_t g = nullptr;
    cuda_check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeRelaxed), "begin capture");
    try {
      enqueue(with_sigma, true);
    } catch (...) {
      cudaStreamEndCapture(stream_, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    cuda_check(cudaStreamEndCapture(stream_, &g), "end capture");
    cudaGraphExec_t x = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&x, g, 0);
    cudaGraphDestroy(g);
    cuda_check(e, "instantiate");
    sigma_flops = f0;  // the captured launches ran nothing
    sigma_calls = c0n;
    return x;
  };
  bool with_sigma = false;
  int iter = 0, total_iter = 0;
  dav_graph_launches_ = 0;
  // iterations until every root converged or max_iter; returns how many of
  // them computed a sigma (expanded the basis)
  auto iterate = [&]() {
    int expansions = 0;
    with_sigma = false;
    while (true) {
      const int w = with_sigma ? 1 : 0;
      auto t0 = std::chrono::steady_clock::now();
      if (use_graph) {
        if (!sc.gx[w]) sc.gx[w] = capture(with_sigma);
        cuda_check(cudaGraphLaunch(sc.gx[w], stream_), "graph launch");
        ++dav_graph_launches_;
        if (with_sigma) {
          sigma_flops += plan_.flops;
          ++sigma_calls;
        }
      } else {
        enqueue(with_sigma, false);
      }
      sync();
      if (with_sigma) {
        ++expansions;
        float ms = 0.f;
        double dt;
        if (cudaEventElapsedTime(&ms, sc.ev[0], sc.ev[1]) == cudaSuccess) dt = ms * 1e-3;
        else dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        count_sigma(dt);
      }
      const dev::DavCtl& h = *dav_host_;
      if (h.status < 0) throw std::runtime_error("subspace eigensolver did not converge");
      iter = h.iter;
      if (h.done || iter >= p.max_iter) break;
      with_sigma = h.expand != 0;
    }
    total_iter += iter;
    return expansions;
  };
  iterate();
  laps.lap("iterations");
  // Defect correction of split-precision solves: the Ritz vectors get FP64
  // products, the Davidson restarts from them with their exact FP64
  // subspace matrix and residuals, and every further basis vector (a
  // correction, small next to the vectors) gets a split-precision product.
  // The split error then enters only through the corrections, scaled by
  // their size, and each round shrinks the FP64 residual by about the split
  // precision; the solve ends when a restart's FP64 residuals of every root
  // are below tol without any new basis vector (linear.C:301-335 applied to
  // the FP64 residual).
  //
  // After a restart every sigma row carries a bound of its difference from
  // the FP64 product (DavCtl::eb): 0 for the restart vectors, eps for each
  // correction, carried through the Ritz rotations.  eps is kEpsSafety times
  // the largest difference |S_i - H_64 x_i| seen on this superblock when the
  // split-precision Ritz vectors x_i got their FP64 products (each a sum of
  // split products of unit vectors).  A restart that converges after adding
  // corrections is accepted without another FP64 product when
  // (|r_i| + eb_i)^2 <= tol for every root: the FP64 residual of a vector
  // sum_j y_j b_j is the subspace residual plus sum_j y_j (H_64 b_j - S_j).
  bool fp64_verified = false;
  last_defect_rounds_ = 0;
  last_defect_bounded_ = false;
  last_plan_flops_ = plan_.flops;
  if (precision_slices(precision) && (refine_mode == 1 || refine_mode == 2)) {
    constexpr double kEpsSafety = 4.0;
    double eps = 0.0;
    double* prev = alloc((int64_t)nroots * n);  // split-precision sigma rows
    // mode 2: the FP64-level products on the tensor cores (exact slices),
    // except until the FP64 product rate of this context is known: the
    // first solve with a product of at least kRateFlops measures it on FP64
    // products (the rate prices the FP64 solves that these products stand
    // in for; smaller products run below the FP64 pipe's rate)
    constexpr double kRateFlops = 1e11;
    const bool exact = refine_mode == 2 && (fp64_rate_ > 0.0 || plan_.flops < kRateFlops);
    for (int round = 0; round < kDefectRounds; ++round) {
      if (round == 0)
        cuda_check(cudaMemcpyAsync(prev, S, (size_t)nroots * n * sizeof(double), cudaMemcpyDeviceToDevice, stream_),
                   "copy sigma rows");
      for (int i = 0; i < nroots; ++i) {
        auto t0 = std::chrono::steady_clock::now();
        if (exact) sigma_exact(sb, plan_, row(B, i), row(S, i));
        else sigma(sb, plan_, row(B, i), row(S, i));
        sync();
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        sigma_seconds += dt;
        if (exact) {
          exact_seconds += dt;
          ++exact_calls;
        } else {
          fp64_seconds += dt;
          ++fp64_calls;
          if (plan_.flops >= kRateFlops && dt > 0.0) fp64_rate_ = plan_.flops / dt;
        }
        ++defect_fp64_sigma_;
      }
      if (round == 0) {
        for (int i = 0; i < nroots; ++i) {
          double d2;
          cuda_check(dev::launch_axpy(-1.0, row(S, i), prev + (int64_t)i * n, n, stream_), "sigma difference");
          dots(prev + (int64_t)i * n, 1, prev + (int64_t)i * n, &d2);
          eps = std::max(eps, kEpsSafety * std::sqrt(std::max(d2, 0.0)));
        }
        last_split_eps_ = eps;
      }
      dev::DavCtl c1{};
      std::vector<double> col(nroots);
      for (int j = 0; j < nroots; ++j) {
        dots(B, nroots, row(S, j), col.data());
        for (int i = j; i < nroots; ++i) c1.h[i * nroots + j] = c1.h[j * nroots + i] = col[i];
      }
      c1.k = nroots;
      c1.mode = 2;
      c1.eps = eps;
      cuda_check(cudaMemcpyAsync(sc.ctl, &c1, sizeof(c1), cudaMemcpyHostToDevice, stream_), "h2d ctl");
      sync();
      ++last_defect_rounds_;
      ++defect_rounds_;
      const int expansions = iterate();
      if (expansions == 0 && dav_host_->done) {
        fp64_verified = true;
        break;
      }
      if (dav_host_->done && eps > 0.0) {
        double rn[dev::kDavMax], eb[dev::kDavMax];
        const dev::DavCtl* dc = sc.ctl;
        cuda_check(cudaMemcpyAsync(rn, dc->rn, nroots * sizeof(double), cudaMemcpyDeviceToHost, stream_), "d2h");
        cuda_check(cudaMemcpyAsync(eb, dc->eb, nroots * sizeof(double), cudaMemcpyDeviceToHost, stream_), "d2h");
        sync();
        bool ok = true;
        for (int i = 0; i < nroots; ++i) {
          const double bound = std::sqrt(std::max(rn[i], 0.0)) + eb[i];
          ok = ok && bound * bound <= p.tol;
        }
        if (ok) {
          fp64_verified = true;
          last_defect_bounded_ = true;
          ++defect_bounded_;
          break;
        }
      }
    }
    free(prev);
    laps.lap("defect correction");
  }
  energies.assign(dav_host_->lam, dav_host_->lam + nroots);
  if (waves_) free(waves_);
  waves_ = alloc((int64_t)nroots * n);
  cuda_check(cudaMemcpyAsync(waves_, B, (size_t)nroots * n * sizeof(double), cudaMemcpyDeviceToDevice, stream_), "waves");
  wave_n_ = n;
  nwaves_ = nroots;
  last_fp64_verified_ = fp64_verified;
  // without a verified FP64 restart (energy-only mode, or rounds / iterations
  // exhausted): FP64 Rayleigh quotients of the final vectors
  if (precision_slices(precision) && !fp64_verified && (!p.defer_refine || refine_mode >= 1)) refine(sb, energies);
  sync();
  return total_iter;
}

// <psi_r| T |psi_r> of single pair terms T for the last solve's vectors: one
// FP64 product per term and root, each followed by a deterministic dot
// product (one-particle density matrix, SweepDriver::rdm_step).
void GpuEngine::expectations(const Superblock& sb, const std::vector<PairTerm>& terms, std::vector<double>& out) {
  if (!waves_ || wave_n_ != sb.size) throw std::runtime_error("expectations: no wavefunction of this superblock");
  const int64_t n = sb.size;
  const int nt = (int)terms.size(), nr = nwaves_;
  out.assign((size_t)nr * nr * nt, 0.0);
  if (nt == 0) return;
  const double f0 = sigma_flops;
  const long c0 = sigma_calls;
  double* y = alloc(n);
  double* work = alloc((int64_t)dev::kGramBlocks);
  double* red = alloc((int64_t)nr * nr * nt);
  for (int t = 0; t < nt; ++t) {
    Superblock one = sb;
    one.terms.assign(1, terms[t]);
    one.ecore = 0.0;
    SigmaPlan p;
    plan_sigma(one, p);
    for (int b = 0; b < nr; ++b) {
      sigma(one, p, waves_ + (int64_t)b * n, y);
      for (int a = 0; a < nr; ++a)
        cuda_check(dev::launch_gram(waves_ + (int64_t)a * n, 1, y, 1, n, n, work,
                                    red + ((int64_t)a * nr + b) * nt + t, stream_),
                   "dot");
    }
    free_plan(p);
  }
  cuda_check(cudaMemcpyAsync(out.data(), red, out.size() * sizeof(double), cudaMemcpyDeviceToHost, stream_), "d2h");
  sync();
  free(y);
  free(work);
  free(red);
  sigma_flops = f0;  // density-matrix products are not sigma products of the solve
  sigma_calls = c0;
}

// Defect correction: energies of the split-precision Ritz vectors from one
// FP64 product each (Rayleigh quotient, second order in the vector error).
bool GpuEngine::refine(const Superblock& sb, std::vector<double>& energies) {
  if (!precision_slices(precision) || !have_plan_ || !waves_) return false;
  const int64_t n = wave_n_;
  double* r = alloc(n);
  double* work = alloc((int64_t)dev::kGramBlocks);
  double* red = alloc(8);
  for (int rr = 0; rr < nwaves_ && rr < (int)energies.size(); ++rr) {
    auto t0 = std::chrono::steady_clock::now();
    const double* b = waves_ + (int64_t)rr * n;
    sigma(sb, plan_, b, r);
    cuda_check(dev::launch_gram(b, 1, r, 1, n, n, work, red, stream_), "dot");
    double h;
    cuda_check(cudaMemcpyAsync(&h, red, sizeof(double), cudaMemcpyDeviceToHost, stream_), "d2h");
    sync();
    energies[rr] = h;
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    sigma_seconds += dt;
    fp64_seconds += dt;
    ++fp64_calls;
  }
  free(r);
  free(work);
  free(red);
  sync();
  return true;
}

// Guess transform (GuessWave::transform_previous_wavefunction with
// TransformLeftBlock / onedot_shufflesysdot / TransformRightBlock,
// guess_wavefunction.C:17-53, 434-486, 526-620) of the last solve's vectors
// into the state space of `sb`:
//   forward (previous step p-1, this step p):
//     phi[a, r]   = U^T psi           U: rotation that made B_L(p-1)
//     chi[(a d) J_L, b] = sum_{J_R} W(a, d, b; J_L, J_R) phi[a, (d b) J_R]
//     guess[., e] = chi V^T           V: rotation that made B_R(p+1), e in dot(p+1) x B_R(p+2)
//   backward (previous step p+1, this step p): the mirror image, with
//     phi = psi V, the recoupling ((a d) J_L, r) -> (a, (d r) J_R) and
//     guess = U chi.
// W = (-1)^{(j_a + j_d + j_b + J)/2} sqrt((2J_L+1)(2J_R+1)) {j_a j_d J_L; j_b J J_R}
// is the recoupling coefficient of three spins (no fermion signs: the site
// order does not change).  Stages are grouped FP64 GEMMs and one build-copy.
bool GpuEngine::transform_guess(const GuessInput& g, const Superblock& sb) {
  PlanLaps laps{"guess"};
  if (!waves_ || nwaves_ < 1 || !g.rotated || !g.expanded || !g.dot) return false;
  auto ri = block_rot_.find(g.rotated->handle);
  auto ei = block_rot_.find(g.expanded->handle);
  if (ri == block_rot_.end() || ei == block_rot_.end()) return false;
  const RotRecord& rot = ri->second;  // U (forward) / V (backward)
  const RotRecord& exp = ei->second;  // V (forward) / U (backward)
  int64_t old_n = 0;
  for (const auto& S : g.old_sectors) old_n = std::max<int64_t>(old_n, S.offset + (int64_t)S.rows * S.cols);
  if (old_n != wave_n_) return false;
  const StateInfo& newL = sb.L->si;
  const StateInfo& newR = sb.R->si;
  const int J = sb.target.s2;
  // the rotations must belong to the state spaces they are applied to
  const StateInfo& rot_big = g.forward ? g.old_L : g.old_R;
  const StateInfo& exp_big = g.forward ? newR : newL;
  if ((int)rot.n.size() != rot_big.size() || (int)exp.n.size() != exp_big.size()) return false;
  for (int q = 0; q < rot_big.size(); ++q)
    if (rot.m[q] > 0 && rot.n[q] != rot_big.states[q]) return false;
  for (int q = 0; q < exp_big.size(); ++q)
    if (exp.m[q] > 0 && exp.n[q] != exp_big.states[q]) return false;
  if (!g.forward && !(g.old_L.is_product() && newR.is_product())) return false;
  if (g.forward && !(g.old_R.is_product() && newL.is_product())) return false;
  auto W = [&](int ja, int jd, int jb, int jl, int jr) {
    const int ph = (ja + jd + jb + J) / 2;
    return ((ph & 1) ? -1.0 : 1.0) * std::sqrt((double)(jl + 1) * (jr + 1)) * six_j(ja, jd, jl, jb, J, jr);
  };
  // stage A: phi per old sector
  std::map<std::pair<int, int>, std::pair<int64_t, int>> phi;  // (row q, col q) -> (offset, cols)
  std::vector<dev::GemmUnit> ua;
  std::vector<dev::GemmItem> ia;
  int64_t phi_n = 0;
  for (const auto& S : g.old_sectors) {
    dev::GemmUnit u{};
    dev::GemmItem it{};
    u.c_buf = 3;
    u.beta_one = 0;
    it.alpha = 1.0;
    if (g.forward) {
      const int a = rot.small_of_big[S.lq];
      if (a < 0) continue;
      const int m = rot.m[S.lq];
      u.m = m;
      u.n = S.cols;
      u.ldc = S.cols;
      it.a_buf = 0;  // U^T
      it.a_off = rot.off[S.lq];
      it.lda = m;
      it.ta = 1;
      it.b_buf = 2;  // psi
      it.b_off = S.offset;
      it.ldb = S.cols;
      it.k = S.rows;
      phi[{a, S.rq}] = {phi_n, S.cols};
    } else {
      const int r = rot.small_of_big[S.rq];
      if (r < 0) continue;
      const int m = rot.m[S.rq];
      u.m = S.rows;
      u.n = m;
      u.ldc = m;
      it.a_buf = 2;  // psi
      it.a_off = S.offset;
      it.lda = S.cols;
      it.b_buf = 0;  // V
      it.b_off = rot.off[S.rq];
      it.ldb = m;
      it.k = S.cols;
      phi[{S.lq, r}] = {phi_n, m};
    }
    u.c_off = phi_n;
    u.ibeg = (int)ia.size();
    ia.push_back(it);
    u.iend = (int)ia.size();
    ua.push_back(u);
    phi_n += (int64_t)u.m * u.n;
  }
  // stage B (chi, scaled copies) and stage C (GEMM into the new sectors)
  std::vector<dev::CopyUnit> ub;
  std::vector<dev::CopyItem> ib;
  std::vector<dev::GemmUnit> uc;
  std::vector<dev::GemmItem> ic;
  int64_t chi_n = 0;
  for (const auto& S : sb.sectors) {
    if (g.forward) {
      const int b = exp.small_of_big[S.rq];  // B_R(p+1) quantum behind the new right sector
      if (b < 0) continue;
      const int mb = exp.m[S.rq];
      const int64_t chi0 = chi_n;
      chi_n += (int64_t)S.rows * mb;
      bool any = false;
      for (const SectorPart& pt : newL.parts[S.lq]) {  // (a in B_L(p-1), d in dot(p))
        dev::CopyUnit cu{};
        cu.c_off = chi0 + (int64_t)pt.offset * mb;
        cu.ldc = mb;
        cu.m = pt.size;
        cu.n = mb;
        cu.ibeg = (int)ib.size();
        const int ja = g.old_L.quanta[rot.big_of_small[pt.lq]].s2;
        const int jd = g.dot->quanta[pt.rq].s2;
        const int jb = g.expanded->si.quanta[b].s2;
        for (const auto& jp : g.old_R.parts_of(pt.rq, b)) {  // old right quantum J_R with part (d, b)
          auto f = phi.find({pt.lq, jp.first});
          if (f == phi.end()) continue;
          const double c = W(ja, jd, jb, newL.quanta[S.lq].s2, g.old_R.quanta[jp.first].s2);
          if (c == 0.0) continue;
          dev::CopyItem ci{};
          ci.s_buf = 3;
          ci.s_off = f->second.first + g.old_R.parts[jp.first][jp.second].offset;
          ci.lds = f->second.second;
          ci.alpha = c;
          ib.push_back(ci);
        }
        cu.iend = (int)ib.size();
        ub.push_back(cu);  // also when empty: the rectangle is zero-filled
        any = any || cu.iend > cu.ibeg;
      }
      if (!any) continue;
      dev::GemmUnit u{};
      u.c_buf = 5;
      u.c_off = S.offset;
      u.ldc = S.cols;
      u.m = S.rows;
      u.n = S.cols;
      u.beta_one = 0;
      u.ibeg = (int)ic.size();
      dev::GemmItem it{};
      it.alpha = 1.0;
      it.a_buf = 4;  // chi
      it.a_off = chi0;
      it.lda = mb;
      it.b_buf = 1;  // V^T
      it.b_off = exp.off[S.rq];
      it.ldb = mb;
      it.tb = 1;
      it.k = mb;
      ic.push_back(it);
      u.iend = (int)ic.size();
      uc.push_back(u);
    } else {
      const int a = exp.small_of_big[S.lq];  // B_L(p) quantum behind the new left sector
      if (a < 0) continue;
      const int ma = exp.m[S.lq];
      const int64_t chi0 = chi_n;
      chi_n += (int64_t)ma * S.cols;
      bool any = false;
      for (const SectorPart& pt : newR.parts[S.rq]) {  // (d in dot(p+1), r in B_R(p+2))
        dev::CopyUnit cu{};
        cu.c_off = chi0 + pt.offset;
        cu.ldc = S.cols;
        cu.m = ma;
        cu.n = pt.size;
        cu.ibeg = (int)ib.size();
        const int ja = g.expanded->si.quanta[a].s2;
        const int jd = g.dot->quanta[pt.lq].s2;
        const int jr = g.old_R.quanta[rot.big_of_small[pt.rq]].s2;
        for (const auto& jp : g.old_L.parts_of(a, pt.lq)) {  // old left quantum J_L with part (a, d)
          auto f = phi.find({jp.first, pt.rq});
          if (f == phi.end()) continue;
          const double c = W(ja, jd, jr, g.old_L.quanta[jp.first].s2, newR.quanta[S.rq].s2);
          if (c == 0.0) continue;
          dev::CopyItem ci{};
          ci.s_buf = 3;
          ci.s_off = f->second.first + (int64_t)g.old_L.parts[jp.first][jp.second].offset * f->second.second;
          ci.lds = f->second.second;
          ci.alpha = c;
          ib.push_back(ci);
        }
        cu.iend = (int)ib.size();
        ub.push_back(cu);
        any = any || cu.iend > cu.ibeg;
      }
      if (!any) continue;
      dev::GemmUnit u{};
      u.c_buf = 5;
      u.c_off = S.offset;
      u.ldc = S.cols;
      u.m = S.rows;
      u.n = S.cols;
      u.beta_one = 0;
      u.ibeg = (int)ic.size();
      dev::GemmItem it{};
      it.alpha = 1.0;
      it.a_buf = 1;  // U
      it.a_off = exp.off[S.lq];
      it.lda = ma;
      it.b_buf = 4;  // chi
      it.b_off = chi0;
      it.ldb = S.cols;
      it.k = ma;
      ic.push_back(it);
      u.iend = (int)ic.size();
      uc.push_back(u);
    }
  }
  if (uc.empty()) return false;
  std::vector<dev::GemmTask> ta, tc;
  for (int u = 0; u < (int)ua.size(); ++u) add_tasks(ta, u, ua[u].m, ua[u].n);
  for (int u = 0; u < (int)uc.size(); ++u) add_tasks(tc, u, uc[u].m, uc[u].n);
  DevArray<dev::GemmUnit> dua, duc;
  DevArray<dev::GemmItem> dia, dic;
  DevArray<dev::GemmTask> dta, dtc;
  DevArray<dev::CopyUnit> dub;
  DevArray<dev::CopyItem> dib;
  dua.upload(ua, stream_);
  dia.upload(ia, stream_);
  dta.upload(ta, stream_);
  dub.upload(ub, stream_);
  dib.upload(ib, stream_);
  duc.upload(uc, stream_);
  dic.upload(ic, stream_);
  dtc.upload(tc, stream_);
  double* phi_d = alloc(phi_n);
  double* chi_d = alloc(chi_n);
  const int nr = nwaves_;
  if (guess_) free(guess_);
  guess_ = alloc((int64_t)nr * sb.size);
  cuda_check(cudaMemsetAsync(guess_, 0, (size_t)nr * sb.size * sizeof(double), stream_), "memset guess");
  cuda_check(cudaMemsetAsync(chi_d, 0, (size_t)std::max<int64_t>(chi_n, 1) * sizeof(double), stream_), "memset chi");
  for (int r = 0; r < nr; ++r) {
    dev::Bufs bufs{};
    bufs.p[0] = rot.d;
    bufs.p[1] = exp.d;
    bufs.p[2] = waves_ + (int64_t)r * wave_n_;
    bufs.p[3] = phi_d;
    bufs.p[4] = chi_d;
    bufs.p[5] = guess_ + (int64_t)r * sb.size;
    cuda_check(dev::launch_gemm(bufs, dua.d, dia.d, dta.d, (int)ta.size(), stream_), "guess stage A");
    cuda_check(dev::launch_copy(bufs, chi_d, dub.d, dib.d, (int)ub.size(), stream_), "guess stage B");
    cuda_check(dev::launch_gemm(bufs, duc.d, dic.d, dtc.d, (int)tc.size(), stream_), "guess stage C");
  }
  free(phi_d);
  free(chi_d);
  for (auto* a : {&dua, &duc}) a->release(stream_);
  for (auto* a : {&dia, &dic}) a->release(stream_);
  for (auto* a : {&dta, &dtc}) a->release(stream_);
  dub.release(stream_);
  dib.release(stream_);
  // usable only if every root keeps a sizeable norm
  double* work = alloc((int64_t)dev::kGramBlocks);
  double* red = alloc(8);
  bool ok = true;
  for (int r = 0; r < nr && ok; ++r) {
    const double* x = guess_ + (int64_t)r * sb.size;
    cuda_check(dev::launch_gram(x, 1, x, 1, sb.size, sb.size, work, red, stream_), "guess norm");
    double h = 0.0;
    cuda_check(cudaMemcpyAsync(&h, red, sizeof(double), cudaMemcpyDeviceToHost, stream_), "d2h");
    sync();
    ok = std::isfinite(h) && h > 1e-4;
  }
  free(work);
  free(red);
  guess_n_ = sb.size;
  nguess_ = ok ? nr : 0;
  sync();
  laps.lap("transform");
  return ok;
}

bool GpuEngine::get_rotation_record(const Block& b, RotationRecord& r) {
  auto it = block_rot_.find(b.handle);
  if (it == block_rot_.end() || !it->second.d) return false;
  const RotRecord& rec = it->second;
  r.off = rec.off;
  r.n = rec.n;
  r.m = rec.m;
  r.small_of_big = rec.small_of_big;
  r.big_of_small = rec.big_of_small;
  int64_t tot = 0;
  for (size_t q = 0; q < rec.off.size(); ++q) tot = std::max<int64_t>(tot, rec.off[q] + (int64_t)rec.n[q] * rec.m[q]);
  r.data.assign(std::max<int64_t>(tot, 1), 0.0);
  cuda_check(cudaMemcpyAsync(r.data.data(), rec.d, r.data.size() * sizeof(double), cudaMemcpyDeviceToHost, stream_),
             "d2h rotation");
  sync();
  return true;
}

void GpuEngine::set_rotation_record(const Block& b, const RotationRecord& r) {
  const size_t nq = r.off.size();
  if (r.n.size() != nq || r.m.size() != nq || r.small_of_big.size() != nq)
    throw std::runtime_error("rotation record: inconsistent sizes");
  for (size_t q = 0; q < nq; ++q)
    if (r.off[q] < 0 || r.off[q] + (int64_t)r.n[q] * r.m[q] > (int64_t)r.data.size())
      throw std::runtime_error("rotation record: sector outside its data");
  RotRecord rec;
  rec.off = r.off;
  rec.n = r.n;
  rec.m = r.m;
  rec.small_of_big = r.small_of_big;
  rec.big_of_small = r.big_of_small;
  rec.d = alloc((int64_t)std::max<size_t>(r.data.size(), 1));
  cuda_check(stage_h2d(rec.d, r.data.data(), r.data.size() * sizeof(double), stream_), "h2d rotation");
  auto old = block_rot_.find(b.handle);
  if (old != block_rot_.end()) free(old->second.d);
  block_rot_[b.handle] = std::move(rec);
}

int GpuEngine::park_vectors() {
  if (!precision_slices(precision) || !waves_ || nwaves_ < 1) return -1;
  Parked pk;
  pk.nroots = nwaves_;
  pk.n = wave_n_;
  pk.d = alloc((int64_t)nwaves_ * wave_n_);
  cuda_check(cudaMemcpyAsync(pk.d, waves_, (size_t)nwaves_ * wave_n_ * sizeof(double), cudaMemcpyDeviceToDevice,
                             stream_),
             "park vectors");
  const int id = next_parked_++;
  parked_[id] = pk;
  return id;
}

// FP64 Rayleigh quotients of parked vectors, with a temporary FP64 plan of
// their superblock (whose blocks the caller kept alive).
bool GpuEngine::refine_parked(int id, const Superblock& sb, std::vector<double>& energies) {
  auto it = parked_.find(id);
  if (it == parked_.end() || it->second.n != sb.size) return false;
  const Parked& pk = it->second;
  SigmaPlan plan;
  plan_sigma(sb, plan);
  double* r = alloc(pk.n);
  double* work = alloc((int64_t)dev::kGramBlocks);
  double* red = alloc(8);
  energies.assign(pk.nroots, 0.0);
  for (int rr = 0; rr < pk.nroots; ++rr) {
    auto t0 = std::chrono::steady_clock::now();
    const double* b = pk.d + (int64_t)rr * pk.n;
    sigma(sb, plan, b, r);
    cuda_check(dev::launch_gram(b, 1, r, 1, pk.n, pk.n, work, red, stream_), "dot");
    double h;
    cuda_check(cudaMemcpyAsync(&h, red, sizeof(double), cudaMemcpyDeviceToHost, stream_), "d2h");
    sync();
    energies[rr] = h;
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    sigma_seconds += dt;
    fp64_seconds += dt;
    ++fp64_calls;
  }
  free(r);
  free(work);
  free(red);
  free_plan(plan);
  sync();
  return true;
}

void GpuEngine::drop_parked(int id) {
  auto it = parked_.find(id);
  if (it == parked_.end()) return;
  free(it->second.d);
  parked_.erase(it);
}

std::string GpuEngine::step_stats() {
  char buf[320];
  char exact_part[64] = "";
  if (exact_calls > last_exact_calls_)
    std::snprintf(exact_part, sizeof(exact_part), ", exact sigma %ld x %.4fs", exact_calls - last_exact_calls_,
                  (exact_seconds - last_exact_seconds_) / (exact_calls - last_exact_calls_));
  std::snprintf(buf, sizeof(buf), "  [split sigma %ld x %.4fs, fp64 sigma %ld x %.4fs%s%s]", split_calls - last_split_calls_,
                split_calls > last_split_calls_ ? (split_seconds - last_split_seconds_) / (split_calls - last_split_calls_)
                                                : 0.0,
                fp64_calls - last_fp64_calls_,
                fp64_calls > last_fp64_calls_ ? (fp64_seconds - last_fp64_seconds_) / (fp64_calls - last_fp64_calls_)
                                              : 0.0,
                exact_part,
                precision_slices(precision) && (refine_mode == 1 || refine_mode == 2)
                    ? (last_fp64_verified_ ? (last_defect_bounded_ ? ", FP64 residual bounds met tol"
                                                                   : ", FP64 residuals met tol")
                                           : ", FP64 residuals NOT verified")
                    : "");
  // what the step's Davidson products would have cost in FP64: every product
  // of the step (split, exact or FP64) at the step's measured FP64 product
  // time, or, without one, at the context's measured FP64 product rate
  const long ds = split_calls - last_split_calls_, df = fp64_calls - last_fp64_calls_,
             dx = exact_calls - last_exact_calls_;
  if (df > 0) derived_fp64_sigma_seconds += (double)(ds + df + dx) * ((fp64_seconds - last_fp64_seconds_) / df);
  else if (dx > 0 && fp64_rate_ > 0.0) derived_fp64_sigma_seconds += (double)(ds + dx) * (last_plan_flops_ / fp64_rate_);
  last_split_seconds_ = split_seconds;
  last_fp64_seconds_ = fp64_seconds;
  last_split_calls_ = split_calls;
  last_fp64_calls_ = fp64_calls;
  last_exact_calls_ = exact_calls;
  last_exact_seconds_ = exact_seconds;
  return buf;
}

// ------------------------------------------------------------------ density

void GpuEngine::density(const Superblock& sb, bool left, const std::vector<double>& weights, DensitySpectrum& spec) {
  PlanLaps laps{"density"};
  const Block& B = left ? *sb.L : *sb.R;
  const int nq = B.si.size();
  std::vector<int64_t> off(nq);
  int64_t tot = 0;
  int maxn = 0;
  dm_dims_.assign(nq, 0);
  for (int q = 0; q < nq; ++q) {
    off[q] = tot;
    dm_dims_[q] = B.si.states[q];
    tot += (int64_t)B.si.states[q] * B.si.states[q];
    maxn = std::max(maxn, B.si.states[q]);
  }
  // the matrix is kept (until the next density) for density_download
  if (dm_rho_) free(dm_rho_);
  dm_rho_ = alloc(tot);
  double* rho = dm_rho_;
  cuda_check(cudaMemsetAsync(rho, 0, std::max<int64_t>(tot, 1) * sizeof(double), stream_), "memset");
  // rho(q) = sum_r w_r sum_sectors psi psi^T (or psi^T psi for the right block)
  std::vector<dev::GemmUnit> units;
  std::vector<dev::GemmItem> items;
  std::vector<dev::GemmTask> tasks;
  for (int q = 0; q < nq; ++q) {
    dev::GemmUnit u{};
    u.c_buf = 1;
    u.c_off = off[q];
    u.ldc = B.si.states[q];
    u.m = u.n = B.si.states[q];
    u.beta_one = 0;
    u.ibeg = (int)items.size();
    for (int rr = 0; rr < nwaves_; ++rr) {
      const double w = rr < (int)weights.size() ? weights[rr] : 1.0 / nwaves_;
      for (const auto& S : sb.sectors) {
        if ((left ? S.lq : S.rq) != q) continue;
        dev::GemmItem g{};
        g.a_buf = g.b_buf = 0;
        g.a_off = g.b_off = (int64_t)rr * wave_n_ + S.offset;
        g.lda = g.ldb = S.cols;
        if (left) {
          g.ta = 0;
          g.tb = 1;
          g.k = S.cols;
        } else {
          g.ta = 1;
          g.tb = 0;
          g.k = S.rows;
        }
        g.alpha = w;
        items.push_back(g);
      }
    }
    u.iend = (int)items.size();
    units.push_back(u);
  }
  for (int u = 0; u < (int)units.size(); ++u) add_tasks(tasks, u, units[u].m, units[u].n);
  DevArray<dev::GemmUnit> du;
  DevArray<dev::GemmItem> di;
  DevArray<dev::GemmTask> dt;
  du.upload(units, stream_);
  di.upload(items, stream_);
  dt.upload(tasks, stream_);
  dev::Bufs bufs{};
  bufs.p[0] = waves_;
  bufs.p[1] = rho;
  cuda_check(dev::launch_gemm(bufs, du.d, di.d, dt.d, (int)tasks.size(), stream_), "density");
  if (noise_.any()) add_noise(sb, left, rho, off);
  if (laps.on) sync();
  laps.lap("rho gemm");
  // eigen-decomposition of every sector (diagonalise_dm): sectors up to
  // kJacobiMax states in one batched Jacobi launch, larger ones with the
  // dense divide-and-conquer solver (eigenvectors column-major)
  constexpr int kJacobiMax = 48;
  if (dm_vecs_) free(dm_vecs_);
  dm_vecs_ = alloc(tot);
  dm_off_ = off;
  dm_colmajor_.assign(nq, 0);
  double* w = alloc(std::max<int64_t>(B.si.total_states(), 1));
  std::vector<int64_t> woff(nq);
  int64_t wt = 0;
  std::vector<int> small_dims(nq, 0), large;
  int small_max = 0;
  for (int q = 0; q < nq; ++q) {
    woff[q] = wt;
    wt += B.si.states[q];
    if (dm_dims_[q] > kJacobiMax) {
      large.push_back(q);
      dm_colmajor_[q] = 1;
    } else {
      small_dims[q] = dm_dims_[q];
      small_max = std::max(small_max, dm_dims_[q]);
    }
  }
  DevArray<int64_t> doff, dwoff;
  DevArray<int> ddims, dstat;
  doff.upload(off, stream_);
  dwoff.upload(woff, stream_);
  ddims.upload(small_dims, stream_);
  dstat.upload(std::vector<int>(nq, 0), stream_);
  double* jac = nullptr;  // the Jacobi sweeps overwrite their matrices: a copy of rho
  if (small_max > 0) {
    jac = alloc(tot);
    cuda_check(cudaMemcpyAsync(jac, rho, tot * sizeof(double), cudaMemcpyDeviceToDevice, stream_), "copy rho");
    cuda_check(dev::launch_jacobi(jac, doff.d, ddims.d, w, dwoff.d, dm_vecs_, doff.d, dstat.d, nq, small_max, stream_),
               "density eig");
  }
  int* eig_status = nullptr;
  if (!large.empty()) {
    // the batched Householder / QL solver (k_eig.cu) on a copy of the large
    // sectors (it overwrites its inputs); eigenvectors column-major
    std::vector<int> dims;
    std::vector<int64_t> aoff, zoff, wo;
    for (int q : large) {
      dims.push_back(dm_dims_[q]);
      aoff.push_back(off[q]);
      zoff.push_back(off[q]);
      wo.push_back(woff[q]);
    }
    eig_status = eigh_batched(dims, rho, aoff, /*copy_inputs=*/true, dm_vecs_, zoff, w, wo);
  }
  {
    // eigenvector signs as on every engine (the basis of the renormalised
    // block, and so the random noise of later steps, depends on them)
    DevArray<int> dall, dcm;
    dall.upload(dm_dims_, stream_);
    dcm.upload(std::vector<int>(dm_colmajor_.begin(), dm_colmajor_.end()), stream_);
    cuda_check(dev::launch_canon_signs(dm_vecs_, doff.d, dall.d, dcm.d, nq, stream_), "eigenvector signs");
    dall.release(stream_);
    dcm.release(stream_);
  }
  if (laps.on) {
    sync();
    char what[64];
    std::snprintf(what, sizeof(what), "eig (%zu dense, max n %d)", large.size(), maxn);
    laps.lap(what);
  }
  std::vector<double> hw(wt);
  std::vector<int> st(nq), info(large.size());
  cuda_check(cudaMemcpyAsync(hw.data(), w, wt * sizeof(double), cudaMemcpyDeviceToHost, stream_), "d2h");
  cuda_check(cudaMemcpyAsync(st.data(), dstat.d, nq * sizeof(int), cudaMemcpyDeviceToHost, stream_), "d2h");
  if (!large.empty())
    cuda_check(cudaMemcpyAsync(info.data(), eig_status, large.size() * sizeof(int), cudaMemcpyDeviceToHost, stream_),
               "d2h");
  sync();
  if (eig_status) cudaFreeAsync(eig_status, stream_);
  for (int q = 0; q < nq; ++q)
    if (st[q] < 0) throw std::runtime_error("density-matrix eigensolver did not converge");
  for (int x : info)
    if (x != 0) throw std::runtime_error("density-matrix eigensolver (tridiagonal divide and conquer) did not converge");
  spec.eig.assign(nq, {});
  for (int q = 0; q < nq; ++q) spec.eig[q].assign(hw.begin() + woff[q], hw.begin() + woff[q] + B.si.states[q]);
  du.release(stream_);
  di.release(stream_);
  dt.release(stream_);
  doff.release(stream_);
  dwoff.release(stream_);
  ddims.release(stream_);
  dstat.release(stream_);
  free(w);
  if (jac) free(jac);
  sync();
}

// Noise of the density matrix (add_onedot_noise, density.C:330-421, with
// the single-operator TensorMultiply of operatorfunctions.C:331-404;
// add_twodot_noise, density.C:92-165); see NoiseSpec.  Every
// phi = (O x 1) psi (or (1 x O) psi) is one grouped FP64 GEMM unit per
// output sector, normalised on the device, and its outer products are summed
// into the sectors of the noise matrix N by a second grouped GEMM; the trace
// condition and scale are applied on the device.  Operators are processed in
// chunks of at most 64 M doubles of phi.
void GpuEngine::add_noise(const Superblock& sb, bool left, double* rho, const std::vector<int64_t>& off) {
  const Block& L = *sb.L;
  const Block& R = *sb.R;
  const Block& B = left ? L : R;
  const int nq = B.si.size();
  const int nroots = std::max(nwaves_, 1);
  const PointGroup& g = noise_.group;
  int64_t tot = 0;
  for (int q = 0; q < nq; ++q) tot += (int64_t)B.si.states[q] * B.si.states[q];
  // psi sector of each (lq, rq)
  std::vector<int> index((size_t)L.si.size() * R.si.size(), -1);
  for (int s = 0; s < (int)sb.sectors.size(); ++s) index[(size_t)sb.sectors[s].lq * R.si.size() + sb.sectors[s].rq] = s;
  DevArray<int64_t> doff;
  DevArray<int> ddims;
  doff.upload(off, stream_);
  ddims.upload(B.si.states, stream_);
  const int64_t chunk_limit = 64ll << 20;
  double* scal = alloc(2);  // trace of N
  // one chunk of wavefunctions phi_j (ranges of `phi`), each added to `target`
  // as phi_j phi_j^T with weight alpha (after normalisation on the device)
  struct Wave {
    std::vector<Superblock::Sector> sec;
    int64_t base = 0;
  };
  auto add_outer = [&](const std::vector<Wave>& waves, double* phi, double* target, double alpha) {
    std::vector<dev::GemmUnit> units;
    std::vector<dev::GemmItem> items;
    std::vector<dev::GemmTask> tasks;
    for (int q = 0; q < nq; ++q) {
      dev::GemmUnit u{};
      u.c_buf = 1;
      u.c_off = off[q];
      u.ldc = u.m = u.n = B.si.states[q];
      u.beta_one = 1;
      u.ibeg = (int)items.size();
      for (const Wave& w : waves)
        for (const auto& S : w.sec) {
          if ((left ? S.lq : S.rq) != q) continue;
          dev::GemmItem it{};
          it.a_buf = it.b_buf = 0;
          it.a_off = it.b_off = w.base + S.offset;
          it.lda = it.ldb = S.cols;
          it.ta = left ? 0 : 1;
          it.tb = left ? 1 : 0;
          it.k = left ? S.cols : S.rows;
          it.alpha = alpha;
          items.push_back(it);
        }
      u.iend = (int)items.size();
      if (u.iend > u.ibeg) units.push_back(u);
    }
    for (int u = 0; u < (int)units.size(); ++u) add_tasks(tasks, u, units[u].m, units[u].n);
    DevArray<dev::GemmUnit> du;
    DevArray<dev::GemmItem> di;
    DevArray<dev::GemmTask> dt;
    du.upload(units, stream_);
    di.upload(items, stream_);
    dt.upload(tasks, stream_);
    dev::Bufs bufs{};
    bufs.p[0] = phi;
    bufs.p[1] = target;
    cuda_check(dev::launch_gemm(bufs, du.d, di.d, dt.d, (int)tasks.size(), stream_), "noise outer products");
    du.release(stream_);
    di.release(stream_);
    dt.release(stream_);
  };
  auto normalise = [&](const std::vector<Wave>& waves, double* phi, int64_t total) {
    std::vector<longlong2> ranges;
    for (const Wave& w : waves) {
      int64_t sz = 0;
      for (const auto& S : w.sec) sz += (int64_t)S.rows * S.cols;
      ranges.push_back(make_longlong2(w.base, w.base + sz));
    }
    (void)total;
    DevArray<longlong2> dr;
    dr.upload(ranges, stream_);
    double* nrm = alloc((int64_t)ranges.size());
    cuda_check(dev::launch_range_norm2(phi, dr.d, (int)ranges.size(), nrm, stream_), "noise norms");
    cuda_check(dev::launch_range_normalise(phi, dr.d, (int)ranges.size(), nrm, stream_), "noise normalise");
    dr.release(stream_);
    free(nrm);
  };
  if (noise_.perturbative > 0.0) {
    const std::vector<NoiseOp> ops = perturbative_noise_ops(B, sb.target, noise_.orbsym, g);
    const int J = sb.target.s2;
    double* N = alloc(tot);
    for (int r = 0; r < nroots; ++r) {
      cuda_check(cudaMemsetAsync(N, 0, std::max<int64_t>(tot, 1) * sizeof(double), stream_), "memset");
      size_t i0 = 0;
      while (i0 < ops.size()) {
        // the next chunk of operators and its phi layout
        std::vector<Wave> waves;
        std::vector<size_t> which;
        int64_t total = 0;
        size_t i1 = i0;
        for (; i1 < ops.size(); ++i1) {
          Wave w;
          int64_t size = 0;
          w.sec = wave_sectors(L.si, R.si, ops[i1].q, g, size);
          if (total > 0 && total + size > chunk_limit) break;
          w.base = total;
          total += size;
          waves.push_back(std::move(w));
          which.push_back(i1);
        }
        i0 = i1;
        if (total == 0) continue;
        double* phi = alloc(total);
        std::vector<dev::GemmUnit> units;
        std::vector<dev::GemmItem> items;
        std::vector<dev::GemmTask> tasks;
        for (size_t x = 0; x < waves.size(); ++x) {
          const NoiseOp& no = ops[which[x]];
          const Operand o = op(no.key, no.trans);
          const int k = no.key.k2;
          for (const auto& S : waves[x].sec) {
            dev::GemmUnit u{};
            u.c_buf = 2;
            u.c_off = waves[x].base + S.offset;
            u.ldc = S.cols;
            u.m = S.rows;
            u.n = S.cols;
            u.beta_one = 0;
            u.ibeg = (int)items.size();
            if (left) {
              for (int lqp = 0; lqp < L.si.size(); ++lqp) {
                const int s = index[(size_t)lqp * R.si.size() + S.rq];
                if (s < 0) continue;
                const HostView v = hview(L, o, S.lq, lqp);
                if (!v.ok) continue;
                const double f = ninej(L.si.quanta[lqp].s2, R.si.quanta[S.rq].s2, J, k, 0, k, L.si.quanta[S.lq].s2,
                                       R.si.quanta[S.rq].s2, no.q.s2) *
                                 v.scale;
                if (f == 0.0) continue;
                const auto& P = sb.sectors[s];
                dev::GemmItem it{};
                it.a_buf = 0;
                it.a_off = v.off;
                it.lda = v.ld;
                it.ta = v.trans ? 1 : 0;
                it.b_buf = 1;
                it.b_off = (int64_t)r * wave_n_ + P.offset;
                it.ldb = P.cols;
                it.tb = 0;
                it.k = P.rows;
                it.alpha = f;
                items.push_back(it);
              }
            } else {
              for (int rqp = 0; rqp < R.si.size(); ++rqp) {
                const int s = index[(size_t)S.lq * R.si.size() + rqp];
                if (s < 0) continue;
                const HostView v = hview(R, o, S.rq, rqp);
                if (!v.ok) continue;
                double f = ninej(L.si.quanta[S.lq].s2, R.si.quanta[rqp].s2, J, 0, k, k, L.si.quanta[S.lq].s2,
                                 R.si.quanta[S.rq].s2, no.q.s2) *
                           v.scale;
                if (op_fermion(no.key) && is_fermion(L.si.quanta[S.lq])) f = -f;
                if (f == 0.0) continue;
                const auto& P = sb.sectors[s];
                dev::GemmItem it{};
                it.a_buf = 1;  // psi(lq, rq')
                it.a_off = (int64_t)r * wave_n_ + P.offset;
                it.lda = P.cols;
                it.ta = 0;
                it.b_buf = 0;  // O(rq, rq')^T
                it.b_off = v.off;
                it.ldb = v.ld;
                it.tb = v.trans ? 0 : 1;
                it.k = P.cols;
                it.alpha = f;
                items.push_back(it);
              }
            }
            u.iend = (int)items.size();
            units.push_back(u);  // (units without items write zeros)
          }
        }
        for (int u = 0; u < (int)units.size(); ++u) add_tasks(tasks, u, units[u].m, units[u].n);
        DevArray<dev::GemmUnit> du;
        DevArray<dev::GemmItem> di;
        DevArray<dev::GemmTask> dt;
        du.upload(units, stream_);
        di.upload(items, stream_);
        dt.upload(tasks, stream_);
        dev::Bufs bufs{};
        bufs.p[0] = arena(B);
        bufs.p[1] = waves_;
        bufs.p[2] = phi;
        cuda_check(dev::launch_gemm(bufs, du.d, di.d, dt.d, (int)tasks.size(), stream_), "noise O psi");
        du.release(stream_);
        di.release(stream_);
        dt.release(stream_);
        normalise(waves, phi, total);
        add_outer(waves, phi, N, 1.0);
        free(phi);
      }
      cuda_check(dev::launch_block_trace(N, doff.d, ddims.d, nq, scal, stream_), "noise trace");
      cuda_check(dev::launch_noise_update(rho, N, tot, scal, noise_.perturbative / nroots, stream_), "noise update");
    }
    free(N);
  }
  if (noise_.random > 0.0) {
    const std::vector<Quantum> qs = random_noise_quanta(sb.target);
    for (int r = 0; r < nroots; ++r) {
      const uint64_t seed = noise_.seed + 0x632BE59BD9B4E019ull * (uint64_t)r;
      for (int i = 0; i < (int)qs.size(); ++i) {
        Wave w;
        int64_t size = 0;
        w.sec = wave_sectors(L.si, R.si, qs[i], g, size);
        if (size == 0) continue;
        double* phi = alloc(size);
        cuda_check(dev::launch_noise_fill(phi, size, seed, i, stream_), "noise fill");
        std::vector<Wave> one{w};
        normalise(one, phi, size);
        add_outer(one, phi, rho, noise_.random / nroots / (double)qs.size());
        free(phi);
      }
    }
  }
  free(scal);
  doff.release(stream_);
  ddims.release(stream_);
}

void GpuEngine::density_download(std::vector<double>& rho, std::vector<double>& vecs) {
  if (!dm_rho_ || !dm_vecs_) throw std::invalid_argument("no density matrix has been formed");
  int64_t tot = 0;
  for (int n : dm_dims_) tot += (int64_t)n * n;
  rho.resize(tot);
  vecs.resize(tot);
  cuda_check(cudaMemcpyAsync(rho.data(), dm_rho_, tot * sizeof(double), cudaMemcpyDeviceToHost, stream_), "d2h rho");
  cuda_check(cudaMemcpyAsync(vecs.data(), dm_vecs_, tot * sizeof(double), cudaMemcpyDeviceToHost, stream_), "d2h vecs");
  sync();
  // every sector row-major with the eigenvectors as columns
  for (size_t q = 0; q < dm_dims_.size(); ++q) {
    if (q >= dm_colmajor_.size() || !dm_colmajor_[q]) continue;
    const int n = dm_dims_[q];
    double* v = vecs.data() + dm_off_[q];
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) std::swap(v[(int64_t)i * n + j], v[(int64_t)j * n + i]);
  }
}

void GpuEngine::set_waves(int nroots, int64_t n, const double* host) {
  if (nroots < 1 || n < 1) throw std::invalid_argument("set_waves: empty");
  if (waves_) free(waves_);
  waves_ = alloc((int64_t)nroots * n);
  cuda_check(stage_h2d(waves_, host, (size_t)nroots * n * sizeof(double), stream_), "h2d waves");
  wave_n_ = n;
  nwaves_ = nroots;
  sync();
}

// The eigensolver of the large density-matrix sectors is the library's own
// (eigh_batched); it needs no loading ahead of the first sweep.
void GpuEngine::prepare_density(int max_n) { (void)max_n; }

// Symmetric eigendecomposition of a batch of matrices (k_eig.cu): matrix j
// of order dims[j] at a + a_off[j] (row-major, lower triangle read; copied
// first when copy_inputs, else overwritten), eigenvectors column-major at
// z + z_off[j] and eigenvalues ascending at w + w_off[j].  Stream-ordered;
// returns a device array of per-matrix status words (< 0: the QL iteration
// did not converge) that the caller reads and frees (cudaFreeAsync).
int* GpuEngine::eigh_batched(const std::vector<int>& dims, double* a, const std::vector<int64_t>& a_off,
                             bool copy_inputs, double* z, const std::vector<int64_t>& z_off, double* w,
                             const std::vector<int64_t>& w_off) {
  const int nj = (int)dims.size();
  std::vector<dev::EigJob> jobs(nj);
  int64_t work = 0;
  int tiles = 0, bt = 0, max_n = 0;
  for (int j = 0; j < nj; ++j) max_n = std::max(max_n, dims[j]);
  if (max_n > dev::kEigMaxN)
    throw std::runtime_error("eigensolver: matrix of order " + std::to_string(max_n) + " above the limit " +
                             std::to_string(dev::kEigMaxN));
  const int bt_cols = dev::eig_bt_cols(max_n);
  for (int j = 0; j < nj; ++j) {
    dev::EigJob& J = jobs[j];
    const int n = dims[j];
    J.n = n;
    J.nt = (n + dev::kEigTile - 1) / dev::kEigTile;
    J.z_off = z_off[j];
    J.w_off = w_off[j];
    J.a_off = copy_inputs ? work : a_off[j];
    if (copy_inputs) work += (int64_t)n * n;
    J.v_off = work;
    work += (int64_t)n * n;
    J.q_off = work;
    work += (int64_t)n * n;
    J.s_off = work;
    work += dev::eig_scalar_elems(n);
    J.tile0 = tiles;
    tiles += J.nt * (J.nt + 1) / 2;
    J.bt0 = bt;
    bt += (n + bt_cols - 1) / bt_cols;
  }
  double* wk = alloc(work);
  if (copy_inputs)
    for (int j = 0; j < nj; ++j)
      cuda_check(cudaMemcpyAsync(wk + jobs[j].a_off, a + a_off[j], (size_t)dims[j] * dims[j] * sizeof(double),
                                 cudaMemcpyDeviceToDevice, stream_),
                 "copy eigensolver input");
  int* status = nullptr;
  cuda_check(cudaMallocAsync((void**)&status, std::max(nj, 1) * sizeof(int), stream_), "alloc status");
  cuda_check(cudaMemsetAsync(status, 0, std::max(nj, 1) * sizeof(int), stream_), "memset");
  DevArray<dev::EigJob> dj;
  dj.upload(jobs, stream_);
  dev::EigBufs eb{copy_inputs ? wk : a, z, w, wk, status};
  cuda_check(dev::launch_eig_tridiag(eb, dj.d, nj, max_n, tiles, stream_), "eigensolver tridiagonalisation");
  tridiagonal_dc(jobs, dj.d, wk, status);
  cuda_check(dev::launch_eig_backtransform(eb, dj.d, nj, max_n, bt, stream_), "eigensolver back-transformation");
  dj.release(stream_);
  free(wk);
  return status;
}

// Divide and conquer on the tridiagonal matrices of an eigensolver batch
// (k_dc.cuh): the tree of every job (halves down to leaves of at most
// kDcLeaf rows), the tears, the leaves, then the merges level by level
// (a merge's level is its height in its tree, so that both its children are
// done).  Each level reads back its merges' pole counts to lay out the
// eigenvector GEMM.
void GpuEngine::tridiagonal_dc(const std::vector<dev::EigJob>& jobs, const dev::EigJob* djobs, double* wk,
                               int* status) {
  std::vector<dev::DcLeaf> leaves;
  std::vector<std::vector<dev::DcMerge>> levels;
  std::function<int(int, int, int)> tree = [&](int job, int o, int len) -> int {
    if (len <= dev::kDcLeaf) {
      leaves.push_back({job, o, len, 0});
      return 0;
    }
    const int n1 = len / 2;
    const int h = 1 + std::max(tree(job, o, n1), tree(job, o + n1, len - n1));
    if ((int)levels.size() < h) levels.resize(h);
    dev::DcMerge m{};
    m.job = job;
    m.o = o;
    m.n1 = n1;
    m.nm = len;
    levels[h - 1].push_back(m);
    return h;
  };
  for (int j = 0; j < (int)jobs.size(); ++j) {
    // the merges write only the diagonal blocks of Z: the rest stays zero
    cuda_check(cudaMemsetAsync(wk + jobs[j].q_off, 0, (size_t)jobs[j].n * jobs[j].n * sizeof(double), stream_),
               "memset Z");
    if (jobs[j].n > 0) tree(j, 0, jobs[j].n);
  }
  std::vector<dev::DcMerge> all;
  for (const auto& lv : levels) all.insert(all.end(), lv.begin(), lv.end());
  DevArray<dev::DcMerge> dall;
  DevArray<dev::DcLeaf> dleaves;
  dall.upload(all, stream_);
  dleaves.upload(leaves, stream_);
  cuda_check(dev::launch_dc_tear(wk, djobs, dall.d, (int)all.size(), stream_), "tears");
  cuda_check(dev::launch_dc_leaves(wk, djobs, dleaves.d, (int)leaves.size(), status, stream_), "leaves");
  for (auto& lv : levels) {
    int64_t slots = 0, sq = 0;
    int max_nm = 0;
    for (auto& m : lv) {
      m.x_off = slots;
      m.u_off = m.g_off = sq;
      slots += m.nm;
      sq += (int64_t)m.nm * m.nm;
      max_nm = std::max(max_nm, m.nm);
    }
    const int nm_ = (int)lv.size();
    DevArray<dev::DcMerge> dm;
    dm.upload(lv, stream_);
    // doubles: rotation values (2 per slot), U, G, per slot dk, zk, tau,
    // zhat, per merge rho; ints: rotation columns (2 per slot), per slot
    // col, org, per merge K, nrot (vector members first and 16-byte aligned)
    const int64_t sq2 = (sq + 1) & ~1ll;
    double* dbl = alloc(2 * slots + 2 * sq2 + 4 * slots + nm_);
    int* ints = nullptr;
    cuda_check(cudaMallocAsync((void**)&ints, (size_t)(4 * slots + 2 * nm_) * sizeof(int), stream_), "alloc");
    dev::DcLevel L{};
    L.merges = dm.d;
    L.nmerges = nm_;
    L.nslots = slots;
    L.rot_cs = reinterpret_cast<double2*>(dbl);
    L.U = dbl + 2 * slots;
    L.G = L.U + sq2;
    L.dk = L.G + sq2;
    L.zk = L.dk + slots;
    L.tau = L.zk + slots;
    L.zhat = L.tau + slots;
    L.rho = L.zhat + slots;
    L.rot_cols = reinterpret_cast<int2*>(ints);
    L.col = ints + 2 * slots;
    L.org = L.col + slots;
    L.K = L.org + slots;
    L.nrot = L.K + nm_;
    cuda_check(dev::launch_dc_deflate(wk, djobs, L, max_nm, stream_), "merge deflation");
    std::vector<int> K(nm_);
    cuda_check(cudaMemcpyAsync(K.data(), L.K, nm_ * sizeof(int), cudaMemcpyDeviceToHost, stream_), "d2h K");
    cuda_check(dev::launch_dc_roots(wk, djobs, L, status, stream_), "merge roots");
    sync();
    std::vector<dev::GemmUnit> units;
    std::vector<dev::GemmItem> items;
    std::vector<dev::GemmTask> tasks;
    for (int i = 0; i < nm_; ++i) {
      if (K[i] <= 0) continue;
      const dev::DcMerge& m = lv[i];
      const dev::EigJob& J = jobs[m.job];
      // Z columns [o, o+K) of rows [o, o+nm) = (G[:, 0:K) U)^T as rows:
      // C (K x nm) = U^T (K x K, row-major view of column-major U) G^T
      dev::GemmUnit u{};
      u.c_buf = 2;
      u.c_off = J.q_off + (int64_t)m.o * J.n + m.o;
      u.ldc = J.n;
      u.m = K[i];
      u.n = m.nm;
      u.beta_one = 0;
      u.ibeg = (int)items.size();
      dev::GemmItem it{};
      it.a_buf = 0;
      it.a_off = m.u_off;
      it.lda = K[i];
      it.ta = 0;
      it.b_buf = 1;
      it.b_off = m.g_off;
      it.ldb = m.nm;
      it.tb = 0;
      it.k = K[i];
      it.alpha = 1.0;
      items.push_back(it);
      u.iend = (int)items.size();
      units.push_back(u);
    }
    for (int u = 0; u < (int)units.size(); ++u) add_tasks(tasks, u, units[u].m, units[u].n);
    if (!tasks.empty()) {
      DevArray<dev::GemmUnit> du;
      DevArray<dev::GemmItem> di;
      DevArray<dev::GemmTask> dt;
      du.upload(units, stream_);
      di.upload(items, stream_);
      dt.upload(tasks, stream_);
      dev::Bufs bufs{};
      bufs.p[0] = L.U;
      bufs.p[1] = L.G;
      bufs.p[2] = wk;
      cuda_check(dev::launch_gemm(bufs, du.d, di.d, dt.d, (int)tasks.size(), stream_), "merge eigenvectors");
      du.release(stream_);
      di.release(stream_);
      dt.release(stream_);
    }
    cuda_check(dev::launch_dc_finish(wk, djobs, L, stream_), "merge deflated columns");
    dm.release(stream_);
    free(dbl);
    cudaFreeAsync(ints, stream_);
  }
  dall.release(stream_);
  dleaves.release(stream_);
}

void GpuEngine::select_rotation(const std::vector<std::vector<int>>& kept) {
  const int nq = (int)kept.size();
  rot_off_.assign(nq, 0);
  rot_kept_.assign(nq, 0);
  rot_rows_.assign(nq, 0);
  int64_t tot = 0;
  std::vector<dev::GatherUnit> units;
  std::vector<int> cols;
  for (int q = 0; q < nq; ++q) {
    rot_off_[q] = tot;
    rot_kept_[q] = (int)kept[q].size();
    rot_rows_[q] = dm_dims_[q];
    dev::GatherUnit g{};
    g.u_off = tot;
    g.v_off = dm_off_[q];
    g.colmajor = dm_colmajor_.empty() ? 0 : dm_colmajor_[q];
    g.n = dm_dims_[q];
    g.m = rot_kept_[q];
    g.c_off = (int)cols.size();
    for (int c : kept[q]) cols.push_back(c);
    if (g.m > 0) units.push_back(g);
    tot += (int64_t)dm_dims_[q] * rot_kept_[q];
  }
  if (rot_) free(rot_);
  rot_ = alloc(tot);
  DevArray<dev::GatherUnit> du;
  DevArray<int> dc;
  du.upload(units, stream_);
  dc.upload(cols, stream_);
  cuda_check(dev::launch_gather_cols(dm_vecs_, rot_, du.d, dc.d, (int)units.size(), stream_), "gather");
  du.release(stream_);
  dc.release(stream_);
}

void GpuEngine::set_rotation(const std::vector<std::vector<double>>& rot, const std::vector<int>& kept) {
  const int nq = (int)kept.size();
  rot_off_.assign(nq, 0);
  rot_kept_ = kept;
  rot_rows_.assign(nq, 0);
  int64_t tot = 0;
  for (int q = 0; q < nq; ++q) {
    rot_off_[q] = tot;
    rot_rows_[q] = kept[q] > 0 ? (int)(rot[q].size() / kept[q]) : 0;
    tot += (int64_t)rot[q].size();
  }
  std::vector<double> h(std::max<int64_t>(tot, 1));
  for (int q = 0; q < nq; ++q) std::copy(rot[q].begin(), rot[q].end(), h.begin() + rot_off_[q]);
  if (rot_) free(rot_);
  rot_ = alloc(tot);
  cuda_check(stage_h2d(rot_, h.data(), tot * sizeof(double), stream_), "rot");
}

// O'(b',k') = U_b^T O(b,k) U_k in two grouped-GEMM launches per chunk of
// operators (renormalise_transform, BaseOperator.C:341-363; MatrixRotate,
// MatrixBLAS.C:553-572).
void GpuEngine::renormalise(Block& small, const Block& big) {
  PlanLaps laps{"renormalise"};
  double rflops = 0.0;
  const DevBlock& dbig = blocks_.at(big.handle);
  double* dst = arena(small);
  std::pair<cudaEvent_t, cudaEvent_t> ev{};
  cuda_check(cudaEventCreate(&ev.first), "event");
  cuda_check(cudaEventCreate(&ev.second), "event");
  cuda_check(cudaEventRecord(ev.first, stream_), "record");
  const double* src = arena(big);
  const int64_t chunk_limit = 64ll << 20;  // scratch elements per chunk (512 MB)
  std::vector<dev::GemmUnit> ua, ub;
  std::vector<dev::GemmItem> ia, ib;
  int64_t scratch = 0;
  double* tmp = nullptr;
  auto flush = [&]() {
    if (ua.empty()) return;
    std::vector<dev::GemmTask> ta, tb;
    for (int u = 0; u < (int)ua.size(); ++u) add_tasks(ta, u, ua[u].m, ua[u].n);
    for (int u = 0; u < (int)ub.size(); ++u) add_tasks(tb, u, ub[u].m, ub[u].n);
    tmp = alloc(scratch);
    DevArray<dev::GemmUnit> dua, dub;
    DevArray<dev::GemmItem> dia, dib;
    DevArray<dev::GemmTask> dta, dtb;
    dua.upload(ua, stream_);
    dub.upload(ub, stream_);
    dia.upload(ia, stream_);
    dib.upload(ib, stream_);
    dta.upload(ta, stream_);
    dtb.upload(tb, stream_);
    dev::Bufs bufs{};
    bufs.p[0] = const_cast<double*>(src);
    bufs.p[1] = dst;
    bufs.p[2] = rot_;
    bufs.p[3] = tmp;
    // exact-slice products where their pools fit, else the FP64 pipe
    auto stage = [&](const std::vector<dev::GemmUnit>& u, const std::vector<dev::GemmItem>& it,
                     DevArray<dev::GemmUnit>& du, DevArray<dev::GemmItem>& di, DevArray<dev::GemmTask>& dt,
                     size_t ntask, const char* what) {
      if (renorm_exact()) {
        try {
          gemm_exact(bufs, u, it);
          return;
        } catch (const CudaError&) {
          cudaGetLastError();
          ++renorm_exact_fallbacks_;
        }
      }
      cuda_check(dev::launch_gemm(bufs, du.d, di.d, dt.d, (int)ntask, stream_), what);
    };
    stage(ua, ia, dua, dia, dta, ta.size(), "rotate A");
    stage(ub, ib, dub, dib, dtb, tb.size(), "rotate B");
    for (auto* a : {&dua, &dub}) a->release(stream_);
    for (auto* a : {&dia, &dib}) a->release(stream_);
    for (auto* a : {&dta, &dtb}) a->release(stream_);
    free(tmp);
    ua.clear();
    ub.clear();
    ia.clear();
    ib.clear();
    scratch = 0;
  };
  cuda_check(cudaMemsetAsync(dst, 0, std::max<int64_t>(small.ops.arena, 1) * sizeof(double), stream_), "memset");
  for (const auto& kv : small.ops.ops) {
    const OpEntry& se = kv.second;
    const OpLayout& SL = small.ops.layouts[se.layout];
    const OpEntry& be = big.ops.at(kv.first);
    const OpLayout& BL = big.ops.layouts[be.layout];
    for (const OpBlock& sbk : SL.blocks) {
      const int b = big.si.find(small.si.quanta[sbk.bra]);
      const int k = big.si.find(small.si.quanta[sbk.ket]);
      const int bi = BL.find(b, k);
      if (bi < 0) continue;
      const OpBlock& bb = BL.blocks[bi];
      const int mb = rot_kept_[b], mk = rot_kept_[k];
      // T = O U_k; for a built block only its nonzero rectangles take part:
      // one unit per row band (rows without a rectangle are written as zero),
      // one item per rectangle in column order
      auto nzit = dbig.nz.find(be.base + bb.offset);
      if (nzit == dbig.nz.end()) {
        dev::GemmUnit u{};
        u.c_buf = 3;
        u.c_off = scratch;
        u.ldc = mk;
        u.m = bb.rows;
        u.n = mk;
        u.beta_one = 0;
        u.ibeg = (int)ia.size();
        dev::GemmItem g{};
        g.a_buf = 0;
        g.a_off = be.base + bb.offset;
        g.lda = bb.cols;
        g.ta = 0;
        g.b_buf = 2;
        g.b_off = rot_off_[k];
        g.ldb = mk;
        g.tb = 0;
        g.k = bb.cols;
        g.alpha = 1.0;
        ia.push_back(g);
        u.iend = (int)ia.size();
        ua.push_back(u);
        rflops += 2.0 * bb.rows * bb.cols * mk;
      } else {
        auto rects = nzit->second;  // (r0, c0, rows, cols)
        std::sort(rects.begin(), rects.end());
        auto band = [&](int r0, int rows) {
          dev::GemmUnit u{};
          u.c_buf = 3;
          u.c_off = scratch + (int64_t)r0 * mk;
          u.ldc = mk;
          u.m = rows;
          u.n = mk;
          u.beta_one = 0;
          u.ibeg = u.iend = (int)ia.size();
          ua.push_back(u);
        };
        int next_row = 0;
        for (size_t x = 0; x < rects.size();) {
          const int r0 = rects[x][0], rows = rects[x][2];
          if (r0 < next_row || r0 + rows > bb.rows) throw std::runtime_error("renormalise: overlapping rectangles");
          if (r0 > next_row) band(next_row, r0 - next_row);
          band(r0, rows);
          for (; x < rects.size() && rects[x][0] == r0; ++x) {
            if (rects[x][2] != rows || rects[x][1] + rects[x][3] > bb.cols)
              throw std::runtime_error("renormalise: ragged rectangle band");
            dev::GemmItem g{};
            g.a_buf = 0;
            g.a_off = be.base + bb.offset + (int64_t)r0 * bb.cols + rects[x][1];
            g.lda = bb.cols;
            g.ta = 0;
            g.b_buf = 2;
            g.b_off = rot_off_[k] + (int64_t)rects[x][1] * mk;
            g.ldb = mk;
            g.tb = 0;
            g.k = rects[x][3];
            g.alpha = 1.0;
            ia.push_back(g);
            rflops += 2.0 * rows * rects[x][3] * mk;
          }
          ua.back().iend = (int)ia.size();
          next_row = r0 + rows;
        }
        if (next_row < bb.rows) band(next_row, bb.rows - next_row);
      }
      // O' = U_b^T T
      dev::GemmUnit v{};
      v.c_buf = 1;
      v.c_off = se.base + sbk.offset;
      v.ldc = sbk.cols;
      v.m = mb;
      v.n = mk;
      v.beta_one = 0;
      v.ibeg = (int)ib.size();
      dev::GemmItem h{};
      h.a_buf = 2;
      h.a_off = rot_off_[b];
      h.lda = mb;
      h.ta = 1;
      h.b_buf = 3;
      h.b_off = scratch;
      h.ldb = mk;
      h.tb = 0;
      h.k = bb.rows;
      h.alpha = 1.0;
      ib.push_back(h);
      v.iend = (int)ib.size();
      ub.push_back(v);
      scratch += (int64_t)bb.rows * mk;
      rflops += 2.0 * mb * mk * bb.rows;
      if (scratch > chunk_limit) flush();
    }
  }
  flush();
  renorm_flops_ += rflops;
  if (laps.on) {
    sync();
    char what[64];
    std::snprintf(what, sizeof(what), "U^T O U %.3g flops", rflops);
    laps.lap(what);
  }
  // keep the rotation with the block (guess transform of later steps)
  {
    RotRecord rec;
    const int nq = (int)rot_kept_.size();
    rec.off = rot_off_;
    rec.n = rot_rows_;
    rec.m = rot_kept_;
    rec.small_of_big.assign(nq, -1);
    int64_t tot = 0;
    for (int q = 0; q < nq; ++q) {
      tot = std::max<int64_t>(tot, rot_off_[q] + (int64_t)rot_rows_[q] * rot_kept_[q]);
      if (rot_kept_[q] > 0) {
        rec.small_of_big[q] = (int)rec.big_of_small.size();
        rec.big_of_small.push_back(q);
      }
    }
    if (nq == big.si.size() && (int)rec.big_of_small.size() == small.si.size()) {
      rec.d = alloc(tot);
      cuda_check(cudaMemcpyAsync(rec.d, rot_, std::max<int64_t>(tot, 1) * sizeof(double), cudaMemcpyDeviceToDevice,
                                 stream_),
                 "keep rotation");
      auto old = block_rot_.find(small.handle);
      if (old != block_rot_.end()) free(old->second.d);
      block_rot_[small.handle] = std::move(rec);
    }
  }
  // stream-ordered: the host goes on with the next step's block builds and
  // work-list compilation while the products run; their device time is
  // read from the events at the next synchronisation
  cuda_check(cudaEventRecord(ev.second, stream_), "record");
  pending_renorm_.push_back(ev);
}

}  // namespace bgpu
