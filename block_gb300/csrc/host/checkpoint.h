// Sweep checkpoints: this project's own binary restart format for the
// renormalised blocks of a sweep (the reference keeps its blocks in Boost
// archives on disk, save_load_block.C:29-110, and restarts from them with
// the `restart` keyword, dmrg.C:476-560).  A checkpoint is written after a
// completed sweep and holds everything the next sweep reads: the block
// bookkeeping (sites, quanta, multiplicities, operator catalogue), every
// block's FP64 operator arena, the rotation that made each block (for the
// wavefunction guess transform) and the sweep counters and energies.
//
// Layout (little-endian): "BGPUCKPT", u32 version, then the header fields in
// the order of CheckpointHeader, then per block: side, index, sites,
// quanta, multiplicities, catalogue, arena, optional rotation record; a
// trailing end marker.  Vectors are an i64 length followed by the elements.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "integrals.h"
#include "ops.h"
#include "stateinfo.h"

namespace bgpu {

constexpr uint32_t kCheckpointVersion = 1;

struct CheckpointHeader {
  int32_t norb = 0, nelec = 0;
  Quantum target;
  int32_t nroots = 1;
  uint64_t fingerprint = 0;  // of the Hamiltonian (integrals_fingerprint)
  int32_t sweeps_done = 0;   // sweeps completed
  int32_t next_forward = 1;  // direction of the next sweep
  int32_t cur_M = 0;
  double discarded = 0.0;
  double last_sweep_energy = 0.0;
  std::vector<double> energies;        // per root, of the last step
  std::vector<double> sweep_energies;  // lowest root, per completed sweep
};

// Rotation that made a renormalised block (big-block quantum q: n[q] x m[q]
// rows x kept states, row-major at off[q] of data).
struct RotationRecord {
  std::vector<int64_t> off;
  std::vector<int> n, m, small_of_big, big_of_small;
  std::vector<double> data;
};

// FNV-1a over the integrals, orbital irreps and core energy.
uint64_t integrals_fingerprint(const Integrals& I);

class CheckpointWriter {
 public:
  explicit CheckpointWriter(const std::string& path);  // writes to path + ".tmp"
  ~CheckpointWriter();
  void header(const CheckpointHeader& h);
  void block(int side, int index, const std::vector<int>& sites, const StateInfo& si, const OpSet& ops,
             const std::vector<double>& arena, const RotationRecord* rot);
  void finish(int nblocks);  // end marker, then renames the file into place
 private:
  void raw(const void* p, size_t n);
  template <class T>
  void vec(const std::vector<T>& v);
  std::string path_, tmp_;
  FILE* f_ = nullptr;
};

struct CheckpointBlock {
  int side = 0, index = 0;  // side 0: left block [0..index], 1: right block [index..N-1]
  std::vector<int> sites;
  StateInfo si;
  std::vector<OpKey> keys;
  std::vector<double> arena;
  bool has_rot = false;
  RotationRecord rot;
};

class CheckpointReader {
 public:
  explicit CheckpointReader(const std::string& path);
  ~CheckpointReader();
  const CheckpointHeader& header() const { return h_; }
  // next block; false after the last one (the end marker is checked)
  bool next(CheckpointBlock& b);

 private:
  void raw(void* p, size_t n);
  template <class T>
  void vec(std::vector<T>& v);
  std::string path_;
  FILE* f_ = nullptr;
  CheckpointHeader h_;
};

}  // namespace bgpu
