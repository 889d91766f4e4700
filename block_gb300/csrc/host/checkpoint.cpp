#include "checkpoint.h"

#include <cstring>
#include <stdexcept>

namespace bgpu {

namespace {
constexpr char kMagic[8] = {'B', 'G', 'P', 'U', 'C', 'K', 'P', 'T'};
constexpr int32_t kBlockTag = 1, kEndTag = 0;
constexpr uint32_t kEndMarker = 0x21444e45u;  // "END!"
// sanity bound on element counts read back (2^40 doubles = 8 TB)
constexpr int64_t kMaxElems = int64_t(1) << 40;

void fnv(uint64_t& h, const void* p, size_t n) {
  const unsigned char* c = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= c[i];
    h *= 1099511628211ull;
  }
}
}  // namespace

uint64_t integrals_fingerprint(const Integrals& I) {
  uint64_t h = 1469598103934665603ull;
  fnv(h, &I.norb, sizeof(I.norb));
  fnv(h, &I.nelec, sizeof(I.nelec));
  fnv(h, &I.ecore, sizeof(I.ecore));
  fnv(h, I.orbsym.data(), I.orbsym.size() * sizeof(int));
  fnv(h, I.t.data(), I.t.size() * sizeof(double));
  fnv(h, I.v.data(), I.v.size() * sizeof(double));
  return h;
}

// ---------------------------------------------------------------- writer

CheckpointWriter::CheckpointWriter(const std::string& path) : path_(path), tmp_(path + ".tmp") {
  f_ = std::fopen(tmp_.c_str(), "wb");
  if (!f_) throw std::runtime_error("checkpoint: cannot write " + tmp_);
  raw(kMagic, sizeof(kMagic));
  raw(&kCheckpointVersion, sizeof(kCheckpointVersion));
}

CheckpointWriter::~CheckpointWriter() {
  if (f_) {  // not finished: leave no partial file behind
    std::fclose(f_);
    std::remove(tmp_.c_str());
  }
}

void CheckpointWriter::raw(const void* p, size_t n) {
  if (n && std::fwrite(p, 1, n, f_) != n) throw std::runtime_error("checkpoint: write failed: " + tmp_);
}

template <class T>
void CheckpointWriter::vec(const std::vector<T>& v) {
  const int64_t n = (int64_t)v.size();
  raw(&n, sizeof(n));
  raw(v.data(), v.size() * sizeof(T));
}

void CheckpointWriter::header(const CheckpointHeader& h) {
  const int32_t ints[9] = {h.norb, h.nelec, h.target.n, h.target.s2, h.target.irrep, h.nroots,
                           h.sweeps_done, h.next_forward, h.cur_M};
  raw(ints, sizeof(ints));
  raw(&h.fingerprint, sizeof(h.fingerprint));
  raw(&h.discarded, sizeof(double));
  raw(&h.last_sweep_energy, sizeof(double));
  vec(h.energies);
  vec(h.sweep_energies);
}

void CheckpointWriter::block(int side, int index, const std::vector<int>& sites, const StateInfo& si,
                             const OpSet& ops, const std::vector<double>& arena, const RotationRecord* rot) {
  if ((int64_t)arena.size() != ops.arena) throw std::runtime_error("checkpoint: arena size does not match catalogue");
  raw(&kBlockTag, sizeof(kBlockTag));
  const int32_t si2[2] = {side, index};
  raw(si2, sizeof(si2));
  vec(sites);
  std::vector<int32_t> q;
  for (const Quantum& x : si.quanta) {
    q.push_back(x.n);
    q.push_back(x.s2);
    q.push_back(x.irrep);
  }
  vec(q);
  vec(si.states);
  std::vector<int32_t> keys;
  for (const auto& kv : ops.ops) {
    keys.push_back((int32_t)kv.first.type);
    keys.push_back(kv.first.i);
    keys.push_back(kv.first.j);
    keys.push_back(kv.first.k2);
  }
  vec(keys);
  vec(arena);
  const int32_t has = rot ? 1 : 0;
  raw(&has, sizeof(has));
  if (rot) {
    vec(rot->off);
    vec(rot->n);
    vec(rot->m);
    vec(rot->small_of_big);
    vec(rot->big_of_small);
    vec(rot->data);
  }
}

void CheckpointWriter::finish(int nblocks) {
  raw(&kEndTag, sizeof(kEndTag));
  const int32_t nb = nblocks;
  raw(&nb, sizeof(nb));
  raw(&kEndMarker, sizeof(kEndMarker));
  const bool ok = std::fflush(f_) == 0;
  std::fclose(f_);
  f_ = nullptr;
  if (!ok || std::rename(tmp_.c_str(), path_.c_str()) != 0) {
    std::remove(tmp_.c_str());
    throw std::runtime_error("checkpoint: cannot move " + tmp_ + " to " + path_);
  }
}

// ---------------------------------------------------------------- reader

CheckpointReader::CheckpointReader(const std::string& path) : path_(path) {
  f_ = std::fopen(path.c_str(), "rb");
  if (!f_) throw std::runtime_error("checkpoint: cannot open " + path);
  char magic[8];
  uint32_t version = 0;
  raw(magic, sizeof(magic));
  raw(&version, sizeof(version));
  if (std::memcmp(magic, kMagic, sizeof(kMagic)) != 0) throw std::runtime_error("checkpoint: not a checkpoint: " + path);
  if (version != kCheckpointVersion)
    throw std::runtime_error("checkpoint: version " + std::to_string(version) + " not supported");
  int32_t ints[9];
  raw(ints, sizeof(ints));
  h_.norb = ints[0];
  h_.nelec = ints[1];
  h_.target = Quantum{ints[2], ints[3], ints[4]};
  h_.nroots = ints[5];
  h_.sweeps_done = ints[6];
  h_.next_forward = ints[7];
  h_.cur_M = ints[8];
  raw(&h_.fingerprint, sizeof(h_.fingerprint));
  raw(&h_.discarded, sizeof(double));
  raw(&h_.last_sweep_energy, sizeof(double));
  vec(h_.energies);
  vec(h_.sweep_energies);
}

CheckpointReader::~CheckpointReader() {
  if (f_) std::fclose(f_);
}

void CheckpointReader::raw(void* p, size_t n) {
  if (n && std::fread(p, 1, n, f_) != n) throw std::runtime_error("checkpoint: truncated file " + path_);
}

template <class T>
void CheckpointReader::vec(std::vector<T>& v) {
  int64_t n = 0;
  raw(&n, sizeof(n));
  if (n < 0 || n > kMaxElems) throw std::runtime_error("checkpoint: corrupt length in " + path_);
  v.resize((size_t)n);
  raw(v.data(), v.size() * sizeof(T));
}

bool CheckpointReader::next(CheckpointBlock& b) {
  int32_t tag = 0;
  raw(&tag, sizeof(tag));
  if (tag == kEndTag) {
    int32_t nb = 0;
    uint32_t end = 0;
    raw(&nb, sizeof(nb));
    raw(&end, sizeof(end));
    if (end != kEndMarker) throw std::runtime_error("checkpoint: missing end marker in " + path_);
    return false;
  }
  if (tag != kBlockTag) throw std::runtime_error("checkpoint: corrupt block tag in " + path_);
  int32_t si2[2];
  raw(si2, sizeof(si2));
  b.side = si2[0];
  b.index = si2[1];
  vec(b.sites);
  std::vector<int32_t> q;
  vec(q);
  if (q.size() % 3) throw std::runtime_error("checkpoint: corrupt quanta in " + path_);
  b.si = StateInfo{};
  for (size_t i = 0; i < q.size(); i += 3) b.si.quanta.push_back(Quantum{q[i], q[i + 1], q[i + 2]});
  vec(b.si.states);
  if (b.si.states.size() != b.si.quanta.size()) throw std::runtime_error("checkpoint: corrupt states in " + path_);
  std::vector<int32_t> keys;
  vec(keys);
  if (keys.size() % 4) throw std::runtime_error("checkpoint: corrupt catalogue in " + path_);
  b.keys.clear();
  for (size_t i = 0; i < keys.size(); i += 4) {
    OpKey k;
    k.type = (OpType)keys[i];
    k.i = (int16_t)keys[i + 1];
    k.j = (int16_t)keys[i + 2];
    k.k2 = (int8_t)keys[i + 3];
    b.keys.push_back(k);
  }
  vec(b.arena);
  int32_t has = 0;
  raw(&has, sizeof(has));
  b.has_rot = has != 0;
  if (b.has_rot) {
    vec(b.rot.off);
    vec(b.rot.n);
    vec(b.rot.m);
    vec(b.rot.small_of_big);
    vec(b.rot.big_of_small);
    vec(b.rot.data);
  }
  return true;
}

}  // namespace bgpu
