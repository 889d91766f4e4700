// Descriptors of the fused two-stage split-precision sigma kernel (k_fused.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace bgpu {
namespace dev {

enum : uint8_t { kFusedFull = 0, kFusedLIdent = 1, kFusedRIdent = 2 };

// One coupling of an output sector: sigma(lQ,rQ) += alpha * A psi(lQ',rQ') B^T.
struct FusedItem {
  int64_t a_off;  // L-operator block (kFusedLIdent: FP64 psi block (lQ, rQ'))
  int64_t c_off;  // psi block (lQ', rQ')
  int64_t b_off;  // R-operator block
  int32_t lda, ldc, ldb;
  int32_t k1, n1;  // n_lQ', n_rQ'
  uint8_t ta;      // A stored transposed (block (lQ', lQ))
  uint8_t tb;      // B stored transposed (block (rQ', rQ))
  uint8_t kind;
  uint8_t pad;
  float alpha;
};

// One thread block: a 64 x 64 tile of a sector and a range of its items.
struct FusedTask {
  int32_t m, n;    // sector rows / cols
  int32_t tm, tn;  // tile
  int32_t ibeg, iend;
};

// Sum of the partial tiles [pbeg, pend) into the FP64 sector tile.
struct FusedTile {
  int64_t s_off;
  int32_t lds, m, n, tm, tn, pbeg, pend;
};

struct FusedBufs {
  const __nv_bfloat16* L[3];
  const __nv_bfloat16* R[3];
  const __nv_bfloat16* psi[3];
  const double* psi64;
  float* partials;  // ntasks x 4096
};

cudaError_t launch_fused_sigma(int ns, const FusedBufs& fb, const FusedItem* items, const FusedTask* tasks,
                               int ntasks, cudaStream_t s);
cudaError_t launch_fused_reduce(const FusedBufs& fb, const FusedTile* tiles, int ntiles, double* sigma,
                                cudaStream_t s);

}  // namespace dev
}  // namespace bgpu
