// Tensor-core (tcgen05 / TMEM) kernels of the split-precision path.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace bgpu {
namespace dev {

// One 128 x N tile: D = A * B^T with A (128 x K) and B (N x K) row-major
// bf16, D row-major f32; 16 <= N <= 256 and 16 <= K <= 64, both multiples of
// 16.  status is set to 1 if the MMA completion wait ran out.
cudaError_t launch_tc_tile(const __nv_bfloat16* A, const __nv_bfloat16* B, float* D, int N, int K, int* status,
                           cudaStream_t s);

// Same product from operands pre-packed as K-chunks of 64 columns in the
// K-major core-matrix order (chunk c of an R-row operand starts at element
// R * 64 * c), moved by bulk copies; 16 <= K <= 256, multiple of 16.
cudaError_t launch_tc_tile_bulk(const __nv_bfloat16* Ap, const __nv_bfloat16* Bp, float* D, int N, int K,
                                int* status, cudaStream_t s);

// ---------------------------------------------------------------- sigma
//
// Packed operand: `rows` (multiple of 8) x `kp` (multiple of 16) values split
// into bf16 hi = bf16(x) and lo = bf16(x - hi), cut into row tiles of `rt`
// rows (128 for operands in the MMA A role, 64 for the B role) and K-chunks
// of kTcKC columns.  Block (row tile t, chunk c), h rows x w columns, starts
// at element 2 * tc_block_off(rows, kp, t, c, rt) of its pool and holds the
// h x w hi values followed by the h x w lo values, each in the K-major
// core-matrix order (byte (j/8)*h*16 + (i/8)*128 + (i%8)*16 + (j%8)*2), so
// that one bulk copy moves both slices.  Rows beyond the operand's own rows
// and columns beyond its own K are zero.
constexpr int kTcKC = 32;
constexpr int kTcRowsA = 128;  // output tile rows (MMA M)
constexpr int kTcRowsB = 64;   // output tile columns (MMA N at most) of the narrow tiles
constexpr int kTcRowsBWide = 128;  // the same for wide tiles (one pipeline per SM)
__host__ __device__ inline int64_t tc_block_off(int rows, int kp, int t, int c, int rt) {
  const int rest = rows - rt * t;
  const int h = rest < rt ? rest : rt;
  return (int64_t)rt * t * kp + (int64_t)h * kTcKC * c;
}
__host__ __device__ inline int tc_round8(int x) { return (x + 7) & ~7; }
__host__ __device__ inline int tc_round16(int x) { return (x + 15) & ~15; }

enum : int { kTcPoolL = 0, kTcPoolR = 1, kTcPoolPsi = 2, kTcPoolPsiT = 3, kTcPoolS = 4, kTcPools = 5 };

// One packed operand filled from an FP64 block: view element (r, k) is
// src[src_off + (trans ? k * ld + r : r * ld + k)] for r < rows_v, k < cols_v;
// row tiles of rt rows; dst_off in elements of the pool.  The rows_p rows
// written are rows row0.. of a packed operand of dst_rows rows at dst_off
// (row0 = 0 and dst_rows = rows_p, or 0, for a standalone operand; a stack
// of small operators shares one operand, each member at its own row0).
struct TcPack {
  int64_t src_off, dst_off;
  int32_t ld, rows_v, cols_v, rows_p, kp, rt;
  int32_t ex_off;  // exact pools: first row of this operand in the pool's row-exponent array
  uint8_t src, pool, trans, pad;
  int32_t row0, dst_rows;
};

// out (+)= alpha * A * B^T over K = kp, A and B packed operands (host plan);
// a_ex / b_ex: the operands' first rows in their pools' row-exponent arrays,
// o_ex: a stage-1 product's first row in pool S's (exact path)
struct TcItem {
  int64_t a_off, b_off;
  int32_t kp;
  uint8_t a_pool, b_pool;
  uint16_t pad;
  float alpha;
  double alpha64;
  int32_t a_ex, b_ex, o_ex, pad2;
};

// One task of the host plan: output tile (tm, tn) -- rows 128 tm.. of the A
// operands, rows 64 tn.. of the B operands -- and the items [ibeg, iend).
//   phase 1 (one item): writes alpha * A B^T as the packed S operand at
//     out_off of pool S (rows a_rows, K out_kp);
//   phase 2: sum of the items with a compensated (hi, lo) f32 accumulation;
//     direct: the FP64 tile (valid_rows x valid_cols) goes to sigma at
//     out_off + (128 tm + r) * out_kp + 64 tn + c; otherwise the h_a x h_b
//     (hi, lo) pairs go to partials + out_off for the reduce kernel.
//   phase 1, stacked (A is a stack of small operators sharing the B
//     operand): out_off is the first of the 128 TcRow entries that give each
//     row's stage-1 operand.
struct TcTask {
  int32_t a_rows, b_rows;
  int32_t tm, tn;
  int32_t ibeg, iend;
  int64_t out_off;
  int32_t out_kp, direct;
  int32_t valid_rows, valid_cols;
  int32_t stacked;
  int32_t ghost;  // cluster pairs: repeats its partner's tile, writes nothing
};

// Row r of a stacked phase-1 tile: row lrow of the packed stage-1 operand S
// at s_off of pool S (h rows, K = the task's out_ld), scaled by alpha; h = 0
// for rows past the stack.
struct __align__(16) TcRow {
  int64_t s_off;
  int16_t h, lrow;
  float alpha;
};
static_assert(sizeof(TcRow) == 16, "TcRow is 16 bytes");

// sigma tile (rows r0.., cols c0.., h x w) = sum of the partial slots
// slots[pbeg..pend) (each with row stride pad, the tile's padded width)
struct TcTile {
  int64_t s_off;
  int32_t lds, h, w, r0, c0, pbeg, pend, pad;
};

// One item as the persistent kernel streams it (64 bytes): the items of a
// block's tasks, flattened in processing order, each carrying what the
// producer, MMA and epilogue roles need, so that a warp loads 32 of them
// with one coalesced access and no role chases task -> item pointers.
//   a_base / b_base: pool elements of the row tile (128 rows of A, 64 of B)
//   out_base: phase 1: S row-tile base (pool S); phase 2 direct: sigma
//     element of tile (0, 0); phase 2 partial: partial slot (float2)
//   out_ld: phase 1: kp of S; phase 2 direct: sigma row stride; partial: h_b
//   col0: phase 1: S column of tile column 0
// Consecutive items of a task form accumulation groups (kTcGStart ..
// kTcGEnd) summed by the tensor core in one TMEM accumulator; alpha is
// applied to the group sum (groups of several items have alpha = 1).
enum : uint32_t {
  kTcFirst = 1,    // first record of a task
  kTcLast = 2,     // last record of a task: write the result
  kTcDirect = 4,   // phase 2: result straight into sigma
  kTcEmpty = 8,    // task without items (writes zeros)
  kTcGStart = 16,  // first item of an accumulation group
  kTcGEnd = 32,    // last item of an accumulation group
  kTcStacked = 64,  // phase 1: A is a stack of operators; out_base indexes TcBufs::rows
  kTcGhost = 128    // cluster pairs: this block repeats its partner's tile and writes nothing
};
struct __align__(16) TcWork {
  int64_t a_base, b_base, out_base;
  int32_t kp;
  float alpha;
  int16_t h_a, h_b, valid_rows, valid_cols;
  int32_t out_ld, col0;
  uint8_t a_pool, b_pool, flags, pad;
  int32_t pad2[3];
};
static_assert(sizeof(TcWork) == 64, "TcWork is 64 bytes");

struct TcBufs {
  const double* src[3];  // FP64 sources of packing: L arena, R arena, psi
  __nv_bfloat16* pool[kTcPools];
  const TcRow* rows;  // row maps of the stacked phase-1 tiles
  float2* partials;
  int* status;  // set to 1 when a pipeline wait ran out
  int fp16;     // slices are fp16 (else bf16)
};

cudaError_t launch_tc_pack(const TcBufs& b, const TcPack* units, int nunits, cudaStream_t s);
// phase 1 or 2 on nblocks persistent blocks: block j runs the work records
// work[ranges[j].x .. ranges[j].y); nb = output-tile width (kTcRowsB or
// kTcRowsBWide, the row tile of the B-role pools); limit_ns bounds every
// pipeline wait
cudaError_t launch_tc_sigma(int phase, int nb, const TcBufs& b, const TcWork* work, const int2* ranges, int nblocks,
                            double* sigma, uint64_t limit_ns, cudaStream_t s);
// persistent blocks per SM of the kernels with tile width nb
int tc_blocks_per_sm(int nb);
// Phase 2 with 128-column tiles on pairs of blocks in thread-block clusters
// of two (blocks 2c and 2c + 1): the two blocks of a pair run record streams
// of the same items (the column tiles tn and tn + 1, or a ghost copy, of one
// sigma row tile); each copies half of every A piece into both blocks'
// stages with a cluster-multicast bulk copy and its own B piece, and a stage
// is refilled once both blocks' MMAs released it.  nblocks is even.
cudaError_t launch_tc_sigma_pairs(const TcBufs& b, const TcWork* work, const int2* ranges, int nblocks, double* sigma,
                                  uint64_t limit_ns, cudaStream_t s);
// Bounded-wait self-check: one thread waits, with the sigma kernels' wait,
// on an mbarrier that nothing arrives at; out[0] = 1 when the wait gave up,
// out[1] = nanoseconds waited; *status is set by the wait.
cudaError_t launch_tc_wait_selftest(int* status, unsigned long long* out, uint64_t limit_ns, cudaStream_t s);
cudaError_t launch_tc_reduce(const TcBufs& b, const TcTile* tiles, const int64_t* slots, int ntiles, double* sigma,
                             cudaStream_t s);

// ---------------------------------------------------------------- exact
//
// Products exact to about 2^-42 of each operand row's largest element, on
// the same tensor cores (the splitting of Ozaki et al., "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59 (2012) 95-118,
// with fixed-point slices so that the f32 accumulation is exact).  Every
// operand row r is scaled by 2^-e_r, e_r = 1 + the largest binary exponent
// of its elements, and written as six balanced base-128 digits
//   x = 2^e_r sum_{s=0..5} a_s 2^-7(s+1),  |a_0| <= 128, |a_s| <= 64 (the
//   balanced digits of |x|, a_s in [-64, 63], times the sign of x),
// one bf16 slice per digit (integers of at most 8 bits are exact in bf16).
// The 21 digit products with s + u <= 5 go to six f32 TMEM accumulators
// J_q (q = s + u); every term is an integer of at most 2^15 per K element, so
// that J_q is exact for K <= 512.  After each 512 K (and at the end of an
// item) sum_q J_q 2^(7(5-q)) is formed exactly in int64 and added, times
// alpha 2^(e_r + f_c - 49), to an FP64 accumulator of the output tile.
// The pools hold six slices per block (tc_block_off times kTcxSlices; each
// 16-column half of a block holds its six h x 16 slices together) and an
// int32 row-exponent array each (the largest unbiased exponent of the row,
// kTcxNoExp for a zero row).  Output tiles are 128 x 64.
constexpr int kTcxSlices = 6;
constexpr int kTcxKBlock = 512;
constexpr int kTcxKS = 16;  // K per pipeline stage (half of a K-chunk)
constexpr int kTcxNoExp = -100000;
constexpr int kTcxNB = kTcRowsB;

struct TcxBufs {
  const double* src[4];  // packing sources: L arena, R arena, psi, T (phase-1 output)
  __nv_bfloat16* pool[kTcPools];
  int* ex[kTcPools];
  double* t;         // phase-1 output T (FP64, the S operands before packing)
  double* partials;  // phase-2 partial tiles (FP64)
  int* status;
};

// One record of the exact kernels (80 bytes): as TcWork, with the FP64
// alpha and the row-exponent offsets of A, B and (phase 1) of the T rows.
struct __align__(16) TcxWork {
  int64_t a_base, b_base, out_base;
  double alpha;
  int32_t kp, out_ld, col0;
  int32_t a_ex, b_ex, o_ex;
  int16_t h_a, h_b, valid_rows, valid_cols;
  uint8_t a_pool, b_pool, flags, pad;
  int32_t pad2[3];
};
static_assert(sizeof(TcxWork) == 80, "TcxWork is 80 bytes");

// row exponents of the units' rows (not needed for units whose exponents
// the phase-1 kernel has already reduced)
cudaError_t launch_tcx_rowexp(const TcxBufs& b, const TcPack* units, int nunits, cudaStream_t s);
// digit slices of the units
cudaError_t launch_tcx_pack(const TcxBufs& b, const TcPack* units, int nunits, cudaStream_t s);
// phase 1: T tiles (FP64) and the largest exponent of every T row
// (atomicMax into ex[kTcPoolS], which must start at kTcxNoExp); phase 2:
// sigma tiles or FP64 partial tiles
cudaError_t launch_tcx_sigma(int phase, const TcxBufs& b, const TcxWork* work, const int2* ranges, int nblocks,
                             double* sigma, uint64_t limit_ns, cudaStream_t s);
int tcx_blocks_per_sm();
cudaError_t launch_tcx_reduce(const TcxBufs& b, const TcTile* tiles, const int64_t* slots, int ntiles, double* sigma,
                              cudaStream_t s);
// every element of x (n ints) = v
cudaError_t launch_fill_int(int* x, int64_t n, int v, cudaStream_t s);

}  // namespace dev
}  // namespace bgpu
