// CUDA engine of the sweep hot path: operator arenas in HBM, host-compiled
// work lists, FP64 grouped-GEMM sigma, GPU Davidson, density matrix,
// batched Jacobi eigensolver and U^T O U renormalisation.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <map>
#include <unordered_map>
#include <stdexcept>
#include <set>
#include <memory>
#include <string>
#include <vector>

#include "../host/sweep.h"
#include "k_dav.cuh"
#include "k_eig.cuh"
#include "k_fused.cuh"
#include "k_split.cuh"
#include "k_tc.cuh"
#include "kernels.cuh"

namespace bgpu {

// FP64, or split precision: bf16 slices on the tensor cores with f32
// accumulation (BF16X3 / BF16X6: warp-level MMA kernel with 2 / 3 slices;
// BF16X3_TC: tcgen05 / TMEM kernels with 2 slices)
// (FP16X2_TC: the tcgen05 kernels with 2 fp16 slices, 3 products)
// EXACT_TC: the exact-slice tensor-core products (k_tc.cuh), about 1e-12
// relative; treated as FP64 by the solver (no defect correction)
enum class Precision : int { FP64 = 0, BF16X3 = 1, BF16X6 = 2, BF16X3_TC = 3, FP16X2_TC = 4, EXACT_TC = 5 };
inline int precision_slices(Precision p) {
  return (p == Precision::BF16X3 || p == Precision::BF16X3_TC || p == Precision::FP16X2_TC) ? 2
         : p == Precision::BF16X6                                                        ? 3
                                                                                         : 0;
}
inline bool precision_tc(Precision p) { return p == Precision::BF16X3_TC || p == Precision::FP16X2_TC; }

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
void cuda_check(cudaError_t e, const char* what);
// host-to-device copy queued on stream s without waiting for it (staged
// through a pinned ring buffer of that stream); release_staging frees the ring
cudaError_t stage_h2d(void* dst, const void* src, size_t bytes, cudaStream_t s);
void release_staging(cudaStream_t s);

// Device array of trivially-copyable descriptors.
template <class T>
struct DevArray {
  T* d = nullptr;
  size_t n = 0;
  void upload(const std::vector<T>& h, cudaStream_t s);
  void release(cudaStream_t s);
};

// Knobs of the tensor-core work-list schedule (the tile shapes follow the
// sectors: 128-row A tiles and up to 64-column B tiles, cut to each sector).
struct TcKnobs {
  double item_cost = 400.0;  // LPT cost of an item on top of its K x N work
  double split = 3.0;        // phase-2 pieces per persistent block (tile splitting)
  int group = 16;            // items per tensor-core accumulation group
  int per_sector = 0;        // 1: one launch per sector, one block per task (baseline)
  int nb = 64;               // output-tile width: 64 (two pipelines per SM) or 128 (one, wider MMAs)
  // task order across the persistent blocks: 0 longest-processing-time
  // assignment (column tiles of a row kept on one block), 1 waves (task
  // order cut into waves of one task per block, balanced within each wave,
  // so that the blocks work on neighbouring tiles of a sector together and
  // share its operand tiles in L2)
  int waves = 0;
  // 1: phase 2 of 128-column plans on pairs of blocks in clusters of two,
  // each A piece copied once for both column tiles (cluster multicast)
  int pairs = 0;
  bool operator==(const TcKnobs& o) const {
    return item_cost == o.item_cost && split == o.split && group == o.group && per_sector == o.per_sector &&
           nb == o.nb && waves == o.waves && pairs == o.pairs;
  }
};
struct TcHostPlan;  // item lists of a tensor-core plan, kept for rescheduling

// Compiled sigma = H psi work lists of one superblock.
struct SigmaPlan {
  DevArray<dev::GemmUnit> u1, u2;
  DevArray<dev::GemmItem> i1, i2;
  DevArray<dev::GemmTask> t1, t2;
  DevArray<dev::DiagUnit> du;
  DevArray<dev::DiagItem> di;
  DevArray<dev::GemmTask> dtask;  // 64 x 64 tiles of the diagonal units
  DevArray<dev::CopyUnit> ru;  // FP64 sum of split stage-2 partial sectors into sigma
  DevArray<dev::CopyItem> ri;
  // stage-1 intermediates, then split stage-2 partial sectors (FP64 path;
  // allocated on the first FP64 product)
  mutable double* scratch = nullptr;
  int64_t scratch_elems = 0;
  double flops = 0.0;         // FP64-equivalent flops of one sigma
  double bytes = 0.0;         // algorithmic bytes of one sigma (operator blocks + psi + sigma)
  int64_t n = 0;
  double ecore = 0.0;
  int nstage1_units = 0, nstage2_units = 0, nitems = 0;
  // split-precision fused work lists and buffers (built on first use)
  bool fused = false;
  DevArray<dev::FusedItem> fi;
  DevArray<dev::FusedTask> ft;
  DevArray<dev::FusedTile> ftile;
  float* partials = nullptr;
  int ns = 0;
  __nv_bfloat16* psi_s[3] = {nullptr, nullptr, nullptr};
  // tensor-core (tcgen05) split-precision work lists and packed operand
  // pools (built on first use): L / R operator blocks packed once, psi and
  // psi^T packed per product, S = stage-1 products written by phase 1
  bool tc = false;
  bool tc_fp16 = false;  // slices of the packed pools are fp16 (else bf16)
  int tc_nb = 64;        // output-tile width the pools were packed for (row tile of the B-role pools)
  bool tc_nb_set = false;  // tc_nb chosen by the autotuner (else plan_tc chooses it)
  __nv_bfloat16* tc_pool[dev::kTcPools] = {};  // packed operands, hi and lo per block
  int64_t tc_pool_elems[dev::kTcPools] = {};
  DevArray<dev::TcPack> tc_psi_pack;
  DevArray<dev::TcWork> tc_w1, tc_w2;  // work records of phases 1 and 2, grouped by block
  DevArray<int2> tc_r1, tc_r2;         // per persistent block: its range of records
  DevArray<dev::TcTile> tc_tiles;
  DevArray<int64_t> tc_slots;
  DevArray<dev::TcRow> tc_rows;  // row maps of the stacked phase-1 tiles (128 per stack)
  bool tc_pairs = false;         // phase 2 runs on cluster pairs (TcKnobs::pairs)
  int64_t tc_stacks = 0, tc_stacked_items = 0;  // stacks and the stage-1 products they replace
  int tc_stack_used = 0;  // the engine's tc_stack_rows when the plan was built
  float2* tc_partials = nullptr;
  double tc_mma_flops = 0.0;  // tensor-core flops issued per product (3 bf16 products per logical one)
  // plan statistics: phase-1 tasks, phase-2 tasks, phase-2 items, phase-2
  // items reading a stage-1 product, split tiles
  int64_t tc_stats[5] = {};
  std::shared_ptr<TcHostPlan> tc_host;
  TcKnobs tc_knobs;                // knobs of the current schedule
  bool tc_tuned = false;           // knobs chosen by the autotuner
  std::vector<int2> tc_l1, tc_l2;  // per-sector launches: (first block range, blocks)
  int64_t tc_partial_cap = 0;      // float2 capacity of tc_partials
  size_t tc_pool_cap[dev::kTcPools] = {};  // bytes of each packed pool
  // the pools come from (and return to) the engine's pool cache: set for the
  // plan of the sweep's consecutive solves, whose pools have similar sizes
  bool reuse_pools = false;
  // exact-slice plans (dev::TcxWork; six digit slices per pool block,
  // 64-column output tiles): row-exponent arrays of the pools, the FP64
  // stage-1 products T and their packing units into pool S
  bool tcx = false;
  int* tcx_ex[dev::kTcPools] = {};
  int64_t tcx_ex_n[dev::kTcPools] = {};
  double* tcx_t = nullptr;
  int64_t tcx_t_n = 0;
  DevArray<dev::TcPack> tcx_tpack;
  DevArray<dev::TcxWork> tcx_w1, tcx_w2;
};

class GpuEngine : public Engine {
 public:
  explicit GpuEngine(int device = 0);
  ~GpuEngine() override;
  std::string name() const override { return "cuda"; }
  void create_block(Block& b) override;
  void release_block(Block& b) override;
  void upload_block(Block& b, const std::vector<double>& arena) override;
  void download_block(const Block& b, std::vector<double>& arena) override;
  void build_block(Block& big, const Block& a, const Block& b,
                   const std::vector<std::pair<OpKey, std::vector<BuildTerm>>>& recipes) override;
  int solve(const Superblock& sb, const DavidsonParams& p, std::vector<double>& energies) override;
  bool refine(const Superblock& sb, std::vector<double>& energies) override;
  bool transform_guess(const GuessInput& g, const Superblock& sb) override;
  int park_vectors() override;
  bool refine_parked(int id, const Superblock& sb, std::vector<double>& energies) override;
  void drop_parked(int id) override;
  std::string step_stats() override;
  void prepare_density(int max_n) override;
  void prepare_plan(const Superblock& sb) override;
  bool get_rotation_record(const Block& b, RotationRecord& r) override;
  void set_rotation_record(const Block& b, const RotationRecord& r) override;
  // (synchronises, so that every renormalisation issued so far is counted)
  double renorm_flops() const override { return renorm_flops_; }
  int64_t block_bytes() const override { return block_bytes_; }
  double device_renorm_seconds() override {
    sync();
    return renorm_device_seconds;
  }
  double renorm_device_seconds = 0.0;  // device time of the renormalisations (events)
  void density(const Superblock& sb, bool left, const std::vector<double>& weights, DensitySpectrum& spec) override;
  void select_rotation(const std::vector<std::vector<int>>& kept) override;
  void set_rotation(const std::vector<std::vector<double>>& rot, const std::vector<int>& kept) override;
  void renormalise(Block& small, const Block& big) override;
  void expectations(const Superblock& sb, const std::vector<PairTerm>& terms, std::vector<double>& out) override;

  // pieces used by the C ABI, the tests and the bench
  void plan_sigma(const Superblock& sb, SigmaPlan& plan);
  void free_plan(SigmaPlan& plan);
  void free_tc(SigmaPlan& plan);  // tensor-core lists and pools only
  // device pointers, stream-ordered on stream()
  void sigma(const Superblock& sb, const SigmaPlan& plan, const double* psi_d, double* out_d);
  // the FP64 product's launches with the stage-1 intermediates in `scratch`
  // (plan.scratch_elems doubles), whoever owns it; counts the product
  void sigma_fp64(const Superblock& sb, const SigmaPlan& plan, const double* psi_d, double* out_d, double* scratch);
  // split-precision product with `ns` bf16 slices (2 or 3)
  void sigma_split(const Superblock& sb, SigmaPlan& plan, int ns, const double* psi_d, double* out_d,
                   cudaEvent_t* marks = nullptr);
  void plan_fused(const Superblock& sb, SigmaPlan& plan);
  // split-precision product on tcgen05 (pack psi, phase 1, phase 2, reduce)
  void plan_tc(const Superblock& sb, SigmaPlan& plan);
  void sigma_tc(const Superblock& sb, SigmaPlan& plan, const double* psi_d, double* out_d,
                cudaEvent_t* marks = nullptr);
  // exact-slice product on tcgen05 (plan.tcx; see k_tc.cuh): pack psi,
  // phase 1, pack T, phase 2, reduce
  void sigma_tcx(const Superblock& sb, SigmaPlan& plan, const double* psi_d, double* out_d);
  // one exact-slice product of sb with plans built and freed on the spot:
  // the pair terms are cut into as many chunks as the free device memory
  // needs (each chunk's plan packs only its own operators), the chunks'
  // products summed; `ref` is a plan of sb (sizes of its split pools, flops)
  void sigma_exact(const Superblock& sb, const SigmaPlan& ref, const double* psi_d, double* out_d);
  // grouped GEMM of gemm_fp64_kernel's work lists (units written, not
  // accumulated) with the exact-slice kernels: every item's A and B^T views
  // packed into six-digit pools, 128 x 64 output tiles, FP64 tile sums;
  // stream-ordered (no host wait)
  void gemm_exact(const dev::Bufs& bufs, const std::vector<dev::GemmUnit>& units,
                  const std::vector<dev::GemmItem>& items);
  // renormalisation products: 0 FP64 pipe, 1 exact-slice tensor cores for
  // split-precision runs (default), 2 exact-slice always
  int renorm_mode = 1;
  long renorm_exact_fallbacks_ = 0;  // renormalisation stages run on the FP64 pipe for want of memory
  double renorm_flops_ = 0.0;        // FP64-equivalent flops of all renormalisations
  bool renorm_exact() const { return renorm_mode == 2 || (renorm_mode == 1 && precision_slices(precision) > 0); }
  // (re)builds the device work lists of a tensor-core plan for the knobs
  void schedule_tc(const Superblock& sb, SigmaPlan& plan, const TcKnobs& knobs);
  // chooses the knobs of a tensor-core plan by timing candidate schedules;
  // the choice is cached under the superblock's sector-size histogram
  void autotune_tc(const Superblock& sb, SigmaPlan& plan);
  std::string tc_tune_key(const Superblock& sb, const SigmaPlan& plan) const;
  TcKnobs tc_default_knobs() const;
  // tensor-core schedule of new plans: 0 persistent blocks (LPT), 1 one
  // launch per sector (baseline); autotune: tune the knobs of persistent plans
  int tc_schedule_mode = 0;
  // output-tile width of new plans: 0 chosen from the sector sizes (or by the
  // autotuner), else 64 or 128
  int tc_nb_mode = 0;
  int tc_choose_nb(const Superblock& sb) const;
  // stage-1 products of operator blocks with at most this many rows that
  // share their psi block are stacked into one 128-row tensor-core tile
  // (0: no stacking)
  int tc_stack_rows = 64;
  bool tc_autotune = false;
  std::map<std::string, TcKnobs> tune_cache;
  std::string tune_cache_path;  // file the cache is read from and appended to
  void load_tune_cache(const std::string& path);
  double tune_seconds = 0.0;    // time spent tuning
  long tune_runs = 0;           // keys tuned
  // product at the engine's current precision
  void sigma_any(const Superblock& sb, SigmaPlan& plan, const double* psi_d, double* out_d);
  void hdiag(const Superblock& sb, const SigmaPlan& plan, double* diag_d);
  // reps products timed by events on stream(): ms[0] total, ms[1] stage 1, ms[2] stage 2
  void sigma_timed(const Superblock& sb, const SigmaPlan& plan, const double* psi_d, double* out_d, int reps,
                   float* ms);
  int sigma_launches(const SigmaPlan& plan) const;
  double* arena(const Block& b) const;
  int sm_count();
  cudaStream_t stream() const { return stream_; }
  double* alloc(int64_t elems);
  void free(double* p);
  void sync();
  // last Davidson wavefunctions (device, nroots x n)
  const double* waves() const { return waves_; }
  // replaces them with caller vectors (host, nroots x n), e.g. for density()
  void set_waves(int nroots, int64_t n, const double* host);
  // the last density matrix, per sector row-major, and its eigenvectors
  // (per sector row-major, column c = eigenvector of the c-th smallest
  // eigenvalue); sectors back to back in quantum order
  void density_download(std::vector<double>& rho, std::vector<double>& vecs);
  // adds the noise of noise() to the density matrix rho (sectors at off)
  void add_noise(const Superblock& sb, bool left, double* rho, const std::vector<int64_t>& off);
  // sector sizes of the last density matrix
  const std::vector<int>& density_dims() const { return dm_dims_; }
  // batched symmetric eigendecomposition (k_eig.cu); returns a device array
  // of per-matrix status words for the caller to read and free
  int* eigh_batched(const std::vector<int>& dims, double* a, const std::vector<int64_t>& a_off, bool copy_inputs,
                    double* z, const std::vector<int64_t>& z_off, double* w, const std::vector<int64_t>& w_off);
  // divide and conquer on the tridiagonal matrices of an eigensolver batch
  void tridiagonal_dc(const std::vector<dev::EigJob>& jobs, const dev::EigJob* djobs, double* wk, int* status);
  int64_t wave_size() const { return wave_n_; }
  Precision precision = Precision::FP64;
  // split-precision solves: defect correction against FP64 residuals with
  // restart products on the FP64 pipe (1) or exact-slice products on the
  // tensor cores (2, default); 0 only FP64 Rayleigh quotients of the
  // converged split vectors
  int refine_mode = 2;
  static constexpr int kDefectRounds = 8;  // FP64 restarts per solve at most
  int last_defect_rounds_ = 0;             // FP64 restarts of the last solve
  bool last_fp64_verified_ = false;        // its roots met tol on FP64 residuals
  long defect_rounds_ = 0, defect_fp64_sigma_ = 0;  // totals over all solves
  // the last solve was accepted on the error bound of its corrections'
  // sigma rows (no FP64 product after its last restart); solves so accepted
  bool last_defect_bounded_ = false;
  long defect_bounded_ = 0;
  double last_split_eps_ = 0.0;  // the bound eps of one split product (last solve)
  // exact-slice products of defect correction (refinement mode 2), the FP64
  // product rate measured in this context (flops / s), the last solve's
  // FP64-equivalent flops per product
  long exact_calls = 0;
  long exact_fallbacks_ = 0;  // exact products retried with more term chunks after running out of memory
  int last_exact_chunks_ = 0;  // term chunks of the last exact product
  double exact_seconds = 0.0;
  long last_exact_calls_ = 0;
  double last_exact_seconds_ = 0.0;
  double fp64_rate_ = 0.0;
  double last_plan_flops_ = 0.0;
  double sigma_seconds = 0.0;
  long sigma_calls = 0;
  double sigma_flops = 0.0;
  long split_calls = 0, fp64_calls = 0;
  double split_seconds = 0.0, fp64_seconds = 0.0;
  double plan_seconds = 0.0;  // host time compiling sigma work lists
  // sum over block steps of (products of the step) x (its mean FP64 product
  // time): the FP64 sigma time of the same solves, for steps with an FP64 product
  double derived_fp64_sigma_seconds = 0.0;
  // counters at the previous step_stats() call
  double last_split_seconds_ = 0.0, last_fp64_seconds_ = 0.0;
  long last_split_calls_ = 0, last_fp64_calls_ = 0;

 private:
  struct Slices {
    int ns = 0;
    __nv_bfloat16* s[3] = {nullptr, nullptr, nullptr};
  };
  const Slices& block_slices(const Block& b, int ns);
  std::map<int, Slices> slices_;
  int device_ = 0;
  cudaStream_t stream_ = nullptr;
  struct DevBlock {
    double* d = nullptr;
    int64_t n = 0;
    std::vector<double> host;  // dot blocks keep a host copy (their 1x1 blocks fold into factors)
    bool dot = false;
    // blocks built by build_block: the nonzero rectangles (row, column,
    // rows, columns) of every operator block, keyed by the block's arena
    // offset; everything outside them is zero
    std::unordered_map<int64_t, std::vector<std::array<int, 4>>> nz;
  };
  std::map<int, DevBlock> blocks_;
  int next_handle_ = 0;
  int64_t block_bytes_ = 0;  // bytes of the operator arenas held (blocks_)
  // current superblock plan (solve)
  SigmaPlan plan_;
  bool have_plan_ = false;
  bool prepared_ = false;  // plan_ was compiled by prepare_plan for the next solve
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending_renorm_;
  double* waves_ = nullptr;
  int64_t wave_n_ = 0;
  int nwaves_ = 0;
  // density / rotation state
  double* dm_vecs_ = nullptr;
  double* dm_rho_ = nullptr;
  std::vector<int64_t> dm_off_;
  std::vector<int> dm_dims_;
  std::vector<char> dm_colmajor_;  // sector eigenvectors stored column-major (dense solver)
  double* rot_ = nullptr;
  std::vector<int64_t> rot_off_;
  std::vector<int> rot_kept_, rot_rows_;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  // rotation that made each renormalised block (big-block quantum q: n[q] x m[q]
  // row-major at off[q]), kept for the wavefunction guess transform
  struct RotRecord {
    double* d = nullptr;
    std::vector<int64_t> off;
    std::vector<int> n, m, small_of_big, big_of_small;
  };
  std::map<int, RotRecord> block_rot_;
  struct Parked {
    double* d = nullptr;
    int nroots = 0;
    int64_t n = 0;
  };
  std::map<int, Parked> parked_;  // vectors kept for deferred energy refinement
  int next_parked_ = 0;
  double* guess_ = nullptr;  // transformed guess vectors (nguess_ x guess_n_)
  int64_t guess_n_ = 0;
  int nguess_ = 0;
  // pipeline-wait status of the tensor-core kernels (device flag, pinned copy)
  int* tc_status_ = nullptr;
  int sm_count_ = 0;
  int* tc_status_host_ = nullptr;
  // header of the Davidson control record, read back after every iteration
  dev::DavCtl* dav_host_ = nullptr;
  // packed-operand pools of the last solve's plan, handed to the next one
  __nv_bfloat16* pool_cache_[dev::kTcPools] = {};
  size_t pool_cache_cap_[dev::kTcPools] = {};

 public:
  // Davidson iterations as launches of a captured CUDA graph (else the same
  // launches issued one by one); graph launches of the last solve
  bool dav_graph = true;
  long dav_graph_launches_ = 0;
};

}  // namespace bgpu
