// tcgen05 building blocks: a single-tile GEMM used to check the operand
// layout, descriptors and TMEM read-back against a host product.
#include "k_tc.cuh"
#include "tc.cuh"

namespace bgpu {
namespace dev {

using namespace tc;

// D (128 x N, row-major f32) = A (128 x K, row-major bf16) * B (N x K, row-major bf16)^T
__global__ void __launch_bounds__(128) tc_tile_kernel(const __nv_bfloat16* __restrict__ A,
                                                       const __nv_bfloat16* __restrict__ B, float* __restrict__ D,
                                                       int N, int K, int* status) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, warp = tid >> 5;
  uint8_t* sA = smem;
  uint8_t* sB = smem + 128 * K * 2;
  if (warp == 0) {
    tmem_alloc(&tbase, 256);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  for (int idx = tid; idx < 128 * K; idx += 128)
    *(__nv_bfloat16*)(sA + kmajor_off(idx / K, idx % K, 128)) = A[idx];
  for (int idx = tid; idx < N * K; idx += 128) *(__nv_bfloat16*)(sB + kmajor_off(idx / K, idx % K, N)) = B[idx];
  fence_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t d = tbase;
  if (tid == 0) {
    const uint32_t idesc = idesc_bf16(128, N);
    for (int j = 0; j < K / 16; ++j) {
      const uint64_t ad = smem_desc(smem_u32(sA) + j * 2 * 128 * 16, 128 * 16, 128);
      const uint64_t bd = smem_desc(smem_u32(sB) + j * 2 * N * 16, N * 16, 128);
      mma_bf16(d, ad, bd, idesc, j > 0 ? 1u : 0u);
    }
    mma_commit(&bar);
  }
  __syncwarp();
  bool ok = mbar_wait_bounded(&bar, 0, 1000000000ull);
  ok = __syncthreads_and(ok) != 0;
  fence_after_sync();
  if (ok) {
    const int row = warp * 32 + (tid & 31);
    for (int c = 0; c < N; c += 16) {
      float v[16];
      tmem_ld16(d + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[(int64_t)row * N + c + i] = v[i];
    }
  } else {
    if (tid == 0) atomicExch(status, 1);
    mbar_wait_bounded(&bar, 0, 1000000000ull);  // let the MMAs drain before freeing TMEM
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tbase, 256);
}

// Same product with both operands pre-packed in global memory as K-chunks of
// 64 columns in the K-major core-matrix order (chunk c of a R-row operand at
// element R * 64 * c), each chunk moved to shared memory by one bulk copy.
__global__ void __launch_bounds__(128) tc_tile_bulk_kernel(const __nv_bfloat16* __restrict__ Ap,
                                                            const __nv_bfloat16* __restrict__ Bp,
                                                            float* __restrict__ D, int N, int K, int* status) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t full, done;
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, warp = tid >> 5;
  uint8_t* sA = smem;              // 128 x 64
  uint8_t* sB = smem + 128 * 128;  // N x 64
  if (warp == 0) {
    tmem_alloc(&tbase, 256);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(&full, 1);
    mbar_init(&done, 1);
    mbar_fence_init();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t d = tbase;
  bool ok = true;
  if (tid == 0) {
    const uint32_t idesc = idesc_bf16(128, N);
    const int nck = (K + 63) / 64;
    for (int c = 0; c < nck && ok; ++c) {
      const int w = min(64, K - 64 * c);
      mbar_expect_tx(&full, (uint32_t)(128 + N) * w * 2);
      bulk_g2s(sA, Ap + (int64_t)128 * 64 * c, 128 * w * 2, &full);
      bulk_g2s(sB, Bp + (int64_t)N * 64 * c, N * w * 2, &full);
      ok = mbar_wait_bounded(&full, c & 1, 1000000000ull);
      if (!ok) break;
      fence_after_sync();
      for (int j = 0; j < w / 16; ++j) {
        const uint64_t ad = smem_desc(smem_u32(sA) + j * 2 * 128 * 16, 128 * 16, 128);
        const uint64_t bd = smem_desc(smem_u32(sB) + j * 2 * N * 16, N * 16, 128);
        mma_bf16(d, ad, bd, idesc, (c > 0 || j > 0) ? 1u : 0u);
      }
      mma_commit(&done);
      ok = mbar_wait_bounded(&done, c & 1, 1000000000ull);  // stage reused by the next chunk
    }
    if (!ok) atomicExch(status, 1);
  }
  ok = __syncthreads_and(ok) != 0;
  fence_after_sync();
  if (ok) {
    const int row = warp * 32 + (tid & 31);
    for (int c = 0; c < N; c += 16) {
      float v[16];
      tmem_ld16(d + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[(int64_t)row * N + c + i] = v[i];
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tbase, 256);
}

cudaError_t launch_tc_tile_bulk(const __nv_bfloat16* Ap, const __nv_bfloat16* Bp, float* D, int N, int K,
                                int* status, cudaStream_t s) {
  if (N < 16 || N > 256 || N % 16 || K < 16 || K > 256 || K % 16) return cudaErrorInvalidValue;
  const size_t smem = 200 * 1024;  // operands use (128 + N) * 128 bytes
  cudaError_t e = cudaFuncSetAttribute(tc_tile_bulk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  tc_tile_bulk_kernel<<<1, 128, smem, s>>>(Ap, Bp, D, N, K, status);
  return cudaGetLastError();
}

cudaError_t launch_tc_tile(const __nv_bfloat16* A, const __nv_bfloat16* B, float* D, int N, int K, int* status,
                           cudaStream_t s) {
  if (N < 16 || N > 256 || N % 16 || K < 16 || K > 64 || K % 16) return cudaErrorInvalidValue;
  // the operands need (128 + N) * K * 2 bytes; the allocation is larger so
  // that every address the descriptors can form stays inside it
  const size_t smem = 200 * 1024;
  cudaError_t e = cudaFuncSetAttribute(tc_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  tc_tile_kernel<<<1, 128, smem, s>>>(A, B, D, N, K, status);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- sigma

// p[i] for a small kernel-parameter array, by selects (dynamic indexing
// would copy the parameter block to local memory)
template <class T, int N>
__device__ __forceinline__ T pick(const T (&p)[N], int i) {
  T r = p[0];
#pragma unroll
  for (int k = 1; k < N; ++k)
    if (i == k) r = p[k];
  return r;
}

// Packs FP64 blocks into split bf16 operands.  Each thread writes one
// 16-byte core-matrix row (8 consecutive K values of one operand row) of the
// hi and of the lo slice; for transposed views consecutive threads take
// consecutive rows so that the FP64 reads stay coalesced.
__global__ void __launch_bounds__(256) tc_pack_kernel(TcBufs b, const TcPack* __restrict__ units) {
  const TcPack u = units[blockIdx.x];
  const double* src = pick(b.src, u.src) + u.src_off;
  __nv_bfloat16* dst = pick(b.pool, u.pool) + u.dst_off;
  const int kg = u.kp >> 3;
  const int64_t total = (int64_t)u.rows_p * kg;
  for (int64_t g = (int64_t)blockIdx.y * blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.y * blockDim.x) {
    int r, k0;
    if (u.trans) {
      r = (int)(g % u.rows_p);
      k0 = (int)(g / u.rows_p) * 8;
    } else {
      r = (int)(g / kg);
      k0 = (int)(g % kg) * 8;
    }
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int k = k0 + e;
      double x = 0.0;
      if (r < u.rows_v && k < u.cols_v) x = u.trans ? src[(int64_t)k * u.ld + r] : src[(int64_t)r * u.ld + k];
      uint32_t bh, bl;
      split16(x, b.fp16 != 0, bh, bl);
      if (e & 1) {
        hw[e >> 1] |= bh << 16;
        lw[e >> 1] |= bl << 16;
      } else {
        hw[e >> 1] = bh;
        lw[e >> 1] = bl;
      }
    }
    // row R of the destination operand (of H rows; a stack member starts at row0)
    const int H = u.dst_rows > 0 ? u.dst_rows : u.rows_p, R = u.row0 + r;
    const int t = R / u.rt, c = k0 / kTcKC;
    const int rest = H - u.rt * t;
    const int h = rest < u.rt ? rest : u.rt;
    const int w = min(kTcKC, u.kp - kTcKC * c);
    const int64_t off = 2 * tc_block_off(H, u.kp, t, c, u.rt) + (kmajor_off(R - u.rt * t, k0 % kTcKC, h) >> 1);
    *(uint4*)(dst + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    *(uint4*)(dst + off + (int64_t)h * w) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
}

cudaError_t launch_tc_pack(const TcBufs& b, const TcPack* units, int nunits, cudaStream_t s) {
  if (nunits > 0) tc_pack_kernel<<<dim3(nunits, 4), 256, 0, s>>>(b, units);
  return cudaGetLastError();
}

namespace {

// Pipeline shape by output-tile width NB (the B operands' row tile): with
// NB = 64 two independent blocks share an SM (256 TMEM columns and a
// 4-stage ring each); with NB = 128 one block owns the SM (512 TMEM
// columns, a 6-stage ring of 32 KB stages).  One stage holds the largest
// piece: A (128 rows) and B (NB rows) x 32 columns, hi and lo.
template <int NB>
struct TcCfg {
  static constexpr int kSlots = NB == 64 ? 4 : 6;
  static constexpr uint32_t kStageBytes = 2u * (kTcRowsA + NB) * kTcKC * 2;
  static constexpr int kSmem = kSlots * (int)kStageBytes;
  static constexpr uint32_t kTmemCols = 4 * NB;     // two accumulators, then the (hi, lo) sums
  static constexpr uint32_t kVh = 2 * NB, kVl = 3 * NB;
  static constexpr int kBlocksPerSm = NB == 64 ? 2 : 1;
};
constexpr int kTcMaxSlots = 6;
constexpr int kTcThreads = 192;  // warps 0-3 epilogue, 4 bulk-copy producer, 5 MMA issuer
constexpr int kTcProducer = 4, kTcIssuer = 5;
constexpr int kTcAcc = 2;        // accumulators of NB TMEM columns

struct TcShared {
  uint64_t full[kTcMaxSlots], empty[kTcMaxSlots], acc_full[kTcAcc], acc_empty[kTcAcc], drain;
  uint32_t tbase;
  int abort_flag;
};

// bounded wait that also gives up when another role gave up
__device__ bool tc_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, int* status, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (*abort_flag) return false;
    if (globaltimer_ns() - t0 > limit_ns) {
      *abort_flag = 1;
      atomicExch(status, 1);
      return false;
    }
  }
  return true;
}

// hi + lo += x, with the rounding error of the sum kept in lo (TwoSum)
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bp = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
  hi = s;
  lo = __fadd_rn(lo, err);
}

}  // namespace

// A warp's batch of up to 32 work records: lane l holds record base + l.
struct WorkRegs {
  int4 q[4];
};
__device__ __forceinline__ void load_work(const TcWork* __restrict__ w, int idx, int end, WorkRegs& r) {
  if (idx < end) {
    const int4* p = reinterpret_cast<const int4*>(w + idx);
#pragma unroll
    for (int i = 0; i < 4; ++i) r.q[i] = __ldg(p + i);
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) r.q[i] = make_int4(0, 0, 0, 0);
  }
}
__device__ __forceinline__ int64_t shfl64(int lo, int hi, int j) {
  const uint32_t l = (uint32_t)__shfl_sync(0xffffffffu, lo, j), h = (uint32_t)__shfl_sync(0xffffffffu, hi, j);
  return (int64_t)(((uint64_t)h << 32) | l);
}
__device__ __forceinline__ int shfl32(int v, int j) { return __shfl_sync(0xffffffffu, v, j); }

// Grouped split-precision GEMM over packed operands on tcgen05: per K=16
// step three MMAs (hi*hi + hi*lo + lo*hi) into an f32 TMEM accumulator of
// 128 x 64; the items of an accumulation group share the accumulator, eight
// accumulators rotate between groups.  Operand pieces are streamed by bulk
// copies through an 8-stage shared-memory ring.  Persistent: block j walks the work records [ranges[j].x,
// ranges[j].y), each role loading them 32 at a time, and the pipeline runs
// across task boundaries.  The epilogue folds each group sum into a
// compensated (hi, lo) f32 pair held in registers.
template <int PHASE, int NB, bool PAIR = false>
__global__ void __launch_bounds__(kTcThreads, TcCfg<NB>::kBlocksPerSm)
    tc_sigma_kernel(TcBufs b, const TcWork* __restrict__ work, const int2* __restrict__ ranges,
                    double* __restrict__ sigma, uint64_t limit_ns) {
  using Cfg = TcCfg<NB>;
  constexpr int kTcSlots = Cfg::kSlots;
  constexpr uint32_t kTcStageBytes = Cfg::kStageBytes;
  constexpr uint32_t kTcVh = Cfg::kVh, kTcVl = Cfg::kVl;
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ TcShared sh;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int2 rg = ranges[blockIdx.x];
  // TMEM: two accumulators of NB columns, then the phase-2 (hi, lo) sums
  if (warp == kTcIssuer) {
    tmem_alloc(&sh.tbase, Cfg::kTmemCols);
    tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < kTcSlots; ++i) {
      mbar_init(&sh.full[i], 1);
      mbar_init(&sh.empty[i], PAIR ? 2 : 1);  // pairs: released by both blocks' MMAs
    }
    for (int i = 0; i < kTcAcc; ++i) {
      mbar_init(&sh.acc_full[i], 1);
      mbar_init(&sh.acc_empty[i], 4);
    }
    mbar_init(&sh.drain, 1);
    sh.abort_flag = 0;
    mbar_fence_init();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  // pairs: both blocks' barriers exist before either block copies or commits into the other
  if (PAIR) cluster_sync();
  const uint32_t rank = PAIR ? cluster_ctarank() : 0u;
  const uint32_t tmem = sh.tbase;
  volatile int* abort_flag = &sh.abort_flag;

  if (warp == kTcProducer) {
    // ---- producer: lane 0 streams the operand pieces (one K-chunk of one
    // item: A hi, A lo, B hi, B lo) of every item through the stages
    uint32_t k = 0;  // pieces issued
    bool ok = true;
    for (int base = rg.x; base < rg.y && ok; base += 32) {
      WorkRegs r;
      load_work(work, base + lane, rg.y, r);
      const int cnt = min(32, rg.y - base);
      for (int j = 0; j < cnt && ok; ++j) {
        const int64_t a_base = shfl64(r.q[0].x, r.q[0].y, j);
        const int64_t b_base = shfl64(r.q[0].z, r.q[0].w, j);
        const int kp = shfl32(r.q[1].z, j);
        const int hw = shfl32(r.q[2].x, j);
        const int pf = shfl32(r.q[3].x, j);
        if (lane == 0 && !((pf >> 16) & kTcEmpty)) {
          const int h_a = hw & 0xffff, h_b = (hw >> 16) & 0xffff;
          const __nv_bfloat16* pa = pick(b.pool, pf & 0xff) + a_base;
          const __nv_bfloat16* pb = pick(b.pool, (pf >> 8) & 0xff) + b_base;
          const int nck = (kp + kTcKC - 1) / kTcKC;
          for (int c = 0; c < nck; ++c, ++k) {
            const int w = min(kTcKC, kp - kTcKC * c);
            const uint32_t abytes = 2u * h_a * w * 2, bbytes = 2u * h_b * w * 2;
            const int slot = (int)(k % kTcSlots);
            if (!tc_wait(&sh.empty[slot], ((k / kTcSlots) & 1u) ^ 1u, abort_flag, b.status, limit_ns)) {
              ok = false;
              break;
            }
            uint8_t* dst = smem + slot * kTcStageBytes;
            mbar_expect_tx(&sh.full[slot], abytes + bbytes);
            if constexpr (PAIR) {
              // this block's half of the A piece's 8-column groups (hi and
              // lo slices), into the same stage of both blocks of the pair
              const int ng = w / 8;
              const int g0 = rank ? (ng + 1) / 2 : 0, g1 = rank ? ng : (ng + 1) / 2;
              if (g1 > g0) {
                const uint32_t slice = (uint32_t)h_a * w * 2;
                const uint32_t off = (uint32_t)g0 * h_a * 16, len = (uint32_t)(g1 - g0) * h_a * 16;
                const uint8_t* src = reinterpret_cast<const uint8_t*>(pa + 2 * (int64_t)h_a * kTcKC * c);
                bulk_g2s_mc(dst + off, src + off, len, &sh.full[slot], (uint16_t)3);
                bulk_g2s_mc(dst + slice + off, src + slice + off, len, &sh.full[slot], (uint16_t)3);
              }
            } else {
              bulk_g2s(dst, pa + 2 * (int64_t)h_a * kTcKC * c, abytes, &sh.full[slot]);
            }
            bulk_g2s(dst + abytes, pb + 2 * (int64_t)h_b * kTcKC * c, bbytes, &sh.full[slot]);
          }
        }
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      }
    }
    if (lane == 0 && !ok) {
      // copies already issued still land in shared memory: wait for them
      for (uint32_t i = (k > kTcSlots ? k - kTcSlots : 0); i < k; ++i)
        mbar_wait_bounded(&sh.full[i % kTcSlots], (i / kTcSlots) & 1u, limit_ns);
    }
    if (PAIR && lane == 0 && ok) {
      // the last stages released by both blocks: every multicast copy of
      // this block has landed in the partner and been read there
      for (uint32_t i = (k > kTcSlots ? k - kTcSlots : 0); i < k; ++i)
        tc_wait(&sh.empty[i % kTcSlots], (i / kTcSlots) & 1u, abort_flag, b.status, limit_ns);
    }
  } else if (warp == kTcIssuer) {
    // ---- MMA issuer (lane 0)
    uint32_t k = 0;
    int ab = 0;
    uint32_t aph = 0;
    bool ok = true;
    for (int base = rg.x; base < rg.y && ok; base += 32) {
      WorkRegs r;
      load_work(work, base + lane, rg.y, r);
      const int cnt = min(32, rg.y - base);
      for (int j = 0; j < cnt && ok; ++j) {
        const int kp = shfl32(r.q[1].z, j);
        const int hw = shfl32(r.q[2].x, j);
        const int pf = shfl32(r.q[3].x, j);
        const int flags = (pf >> 16) & 0xff;
        if (lane == 0 && !(flags & kTcEmpty)) {
          const int h_a = hw & 0xffff, h_b = (hw >> 16) & 0xffff;
          const uint32_t idesc = b.fp16 ? idesc_f16(128, (h_b + 15) & ~15) : idesc_bf16(128, (h_b + 15) & ~15);
          if ((flags & kTcGStart) &&
              !tc_wait(&sh.acc_empty[ab], aph ^ 1u, abort_flag, b.status, limit_ns))
            ok = false;
          if (ok) {
            fence_after_sync();
            const uint32_t d = tmem + (uint32_t)ab * (uint32_t)NB;
            const int nck = (kp + kTcKC - 1) / kTcKC;
            for (int c = 0; c < nck; ++c, ++k) {
              const int w = min(kTcKC, kp - kTcKC * c);
              const uint32_t abytes = 2u * h_a * w * 2;
              const int slot = (int)(k % kTcSlots);
              if (!tc_wait(&sh.full[slot], (k / kTcSlots) & 1u, abort_flag, b.status, limit_ns)) {
                ok = false;
                break;
              }
              fence_after_sync();
              const uint32_t sa = smem_u32(smem + slot * kTcStageBytes);
              const uint32_t a_lo = (uint32_t)h_a * w * 2, b0 = abytes, b_lo = abytes + (uint32_t)h_b * w * 2;
              for (int jj = 0; jj < w / 16; ++jj) {
                const uint32_t ao = (uint32_t)(32 * jj * h_a), bo = (uint32_t)(32 * jj * h_b);
                const uint64_t dah = smem_desc(sa + ao, h_a * 16, 128);
                const uint64_t dal = smem_desc(sa + a_lo + ao, h_a * 16, 128);
                const uint64_t dbh = smem_desc(sa + b0 + bo, h_b * 16, 128);
                const uint64_t dbl = smem_desc(sa + b_lo + bo, h_b * 16, 128);
                const uint32_t acc = ((flags & kTcGStart) && c == 0 && jj == 0) ? 0u : 1u;
                mma_bf16(d, dah, dbh, idesc, acc);
                mma_bf16(d, dah, dbl, idesc, 1u);
                mma_bf16(d, dal, dbh, idesc, 1u);
              }
              if (PAIR) mma_commit_mc(&sh.empty[slot], (uint16_t)3);
              else mma_commit(&sh.empty[slot]);
            }
            if (ok && (flags & kTcGEnd)) {
              mma_commit(&sh.acc_full[ab]);
              if (++ab == kTcAcc) {
                ab = 0;
                aph ^= 1u;
              }
            }
          }
        }
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      }
    }
  } else {
    // ---- epilogue: warp w owns TMEM lanes 32 w.., all NB columns, read in
    // halves of 64 columns
    const int row = 32 * warp + lane;
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
    const uint32_t vh_t = tmem + kTcVh + lane_base, vl_t = tmem + kTcVl + lane_base;
    int ab = 0;
    uint32_t aph = 0;
    bool ok = true, first = true;
    for (int base = rg.x; base < rg.y && ok; base += 32) {
      WorkRegs r;
      load_work(work, base + lane, rg.y, r);
      const int cnt = min(32, rg.y - base);
      for (int j = 0; j < cnt && ok; ++j) {
        const int pf = shfl32(r.q[3].x, j);
        const int flags = (pf >> 16) & 0xff;
        if (!(flags & (kTcFirst | kTcLast | kTcGEnd))) continue;
        const float alpha = __int_as_float(shfl32(r.q[1].w, j));
        const int hw = shfl32(r.q[2].x, j);
        const int h_a = hw & 0xffff, h_b = (hw >> 16) & 0xffff;
        const int ng = ((h_b + 15) & ~15) >> 4;  // 16-column groups of the accumulator
        const int64_t out_base = shfl64(r.q[1].x, r.q[1].y, j);
        const int vrc = shfl32(r.q[2].y, j);
        const int out_ld = shfl32(r.q[2].z, j);
        const int col0 = shfl32(r.q[2].w, j);
        if (flags & kTcFirst) first = true;
        const bool have = (flags & kTcGEnd) && !(flags & kTcEmpty);
        const bool last = (flags & kTcLast) != 0;
        // phase 1: the stage-1 operand, row and scale this thread's row goes to
        int64_t s_base = out_base;
        int s_h = h_a, s_row = row;
        float s_alpha = alpha;
        if (PHASE == 1 && (flags & kTcStacked) && have && row < h_a) {
          const int4 e = __ldg(reinterpret_cast<const int4*>(b.rows + out_base + row));
          s_base = (int64_t)(((uint64_t)(uint32_t)e.y << 32) | (uint32_t)e.x);
          s_h = e.z & 0xffff;
          s_row = (e.z >> 16) & 0xffff;
          s_alpha = __int_as_float(e.w);
        }
        if (have) {
          ok = __all_sync(0xffffffffu, tc_wait(&sh.acc_full[ab], aph, abort_flag, b.status, limit_ns));
          if (!ok) break;  // TMEM loads below need the whole warp
          fence_after_sync();
        }
        const uint32_t dacc = tmem + (uint32_t)ab * (uint32_t)NB + lane_base;
#pragma unroll 1
        for (int hh = 0; hh < NB / 64; ++hh) {
          const int ngh = min(max(ng - 4 * hh, 0), 4);  // 16-column groups of this half
          float v[64];
          if (have) {
#pragma unroll
            for (int e = 0; e < 64; ++e) v[e] = 0.f;
            const uint32_t d = dacc + 64u * (uint32_t)hh;
            if (ngh > 2) {
              tmem_ld32(d, v);
              if (ngh == 4) tmem_ld32(d + 32u, v + 32);
              else tmem_ld16(d + 32u, v + 32);
            } else if (ngh == 2) {
              tmem_ld32(d, v);
            } else if (ngh == 1) {
              tmem_ld16(d, v);
            }
            if (hh == NB / 64 - 1) {
              // accumulator read: the MMA issuer may reuse it
              fence_before_sync();
              __syncwarp();
              if (lane == 0) mbar_arrive(&sh.acc_empty[ab]);
            }
          }
          if (PHASE == 2) {
            if (!have && !last) continue;
#pragma unroll
            for (int g = 0; g < 4; ++g) {
              if (g < ngh) {
                const int cb = 64 * hh + 16 * g;  // first column of this group
                float vh[16], vl[16];
                if (first) {
#pragma unroll
                  for (int e = 0; e < 16; ++e) {
                    vh[e] = have ? __fmul_rn(alpha, v[16 * g + e]) : 0.f;
                    vl[e] = 0.f;
                  }
                } else {
                  tmem_ld16x2(vh_t + (uint32_t)cb, vl_t + (uint32_t)cb, vh, vl);
                  if (have) {
#pragma unroll
                    for (int e = 0; e < 16; ++e) two_sum_acc(vh[e], vl[e], __fmul_rn(alpha, v[16 * g + e]));
                  }
                }
                if (!last) {
                  tmem_st16(vh_t + (uint32_t)cb, vh);
                  tmem_st16(vl_t + (uint32_t)cb, vl);
                } else if (PAIR && (flags & kTcGhost)) {
                  // the partner's tile repeated for the pair: no output
                } else if (flags & kTcDirect) {
                  const int vrows = vrc & 0xffff, vcols = (vrc >> 16) & 0xffff;
                  if (row < vrows) {
                    double* out = sigma + out_base + (int64_t)row * out_ld;
#pragma unroll
                    for (int e = 0; e < 16; ++e) {
                      const int col = cb + e;
                      if (col < vcols) out[col] = (double)vh[e] + (double)vl[e];
                    }
                  }
                } else if (row < h_a) {
                  float2* out = b.partials + out_base + (int64_t)row * h_b;
#pragma unroll
                  for (int e = 0; e < 16; ++e) {
                    const int col = cb + e;
                    if (col < h_b) out[col] = make_float2(vh[e], vl[e]);
                  }
                }
              }
            }
          } else if (have && row < h_a && s_h > 0) {
            // phase 1: S tile written as a packed operand (rows of this tile,
            // K columns col0.. of S; row s_row of an s_h-row operand)
            const int ncols = min(NB, out_ld - col0);
            __nv_bfloat16* sp = b.pool[kTcPoolS] + s_base;
#pragma unroll
            for (int g8 = 0; g8 < 8; ++g8) {
              const int c0 = 64 * hh + 8 * g8;
              if (c0 < ncols) {
                uint32_t hw4[4], lw4[4];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                  const float x = (c0 + e) < h_b ? __fmul_rn(s_alpha, v[8 * g8 + e]) : 0.f;
                  uint32_t bh, bl;
                  split16(x, b.fp16 != 0, bh, bl);
                  if (e & 1) {
                    hw4[e >> 1] |= bh << 16;
                    lw4[e >> 1] |= bl << 16;
                  } else {
                    hw4[e >> 1] = bh;
                    lw4[e >> 1] = bl;
                  }
                }
                const int C = col0 + c0;  // S column
                const int cc = C / kTcKC, wc = min(kTcKC, out_ld - kTcKC * cc);
                const int64_t off = 2 * (int64_t)s_h * kTcKC * cc + (kmajor_off(s_row, C % kTcKC, s_h) >> 1);
                *(uint4*)(sp + off) = make_uint4(hw4[0], hw4[1], hw4[2], hw4[3]);
                *(uint4*)(sp + off + (int64_t)s_h * wc) = make_uint4(lw4[0], lw4[1], lw4[2], lw4[3]);
              }
            }
          }
        }
        if (have && ++ab == kTcAcc) {
          ab = 0;
          aph ^= 1u;
        }
        if (PHASE == 2 && (have || last)) first = false;
      }
    }
  }
  __syncthreads();
  if (warp == kTcIssuer) {
    // every MMA of this block has completed before TMEM is released
    if (lane == 0) {
      mma_commit(&sh.drain);
      mbar_wait_bounded(&sh.drain, 0, limit_ns);
    }
    __syncwarp();
    fence_after_sync();
    tmem_dealloc(tmem, TcCfg<NB>::kTmemCols);
  }
  // pairs: neither block leaves while the other may still copy into it
  if (PAIR) cluster_sync();
}

template <int PHASE, int NB>
static cudaError_t launch_tc_sigma_nb(const TcBufs& b, const TcWork* work, const int2* ranges, int nblocks,
                                      double* sigma, uint64_t limit_ns, cudaStream_t s) {
  constexpr int smem = TcCfg<NB>::kSmem;
  cudaError_t e = cudaFuncSetAttribute(tc_sigma_kernel<PHASE, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  tc_sigma_kernel<PHASE, NB><<<nblocks, kTcThreads, smem, s>>>(b, work, ranges, sigma, limit_ns);
  return cudaGetLastError();
}

cudaError_t launch_tc_sigma(int phase, int nb, const TcBufs& b, const TcWork* work, const int2* ranges, int nblocks,
                            double* sigma, uint64_t limit_ns, cudaStream_t s) {
  if (nblocks <= 0) return cudaGetLastError();
  if (phase == 1 && nb == 64) return launch_tc_sigma_nb<1, 64>(b, work, ranges, nblocks, sigma, limit_ns, s);
  if (phase == 2 && nb == 64) return launch_tc_sigma_nb<2, 64>(b, work, ranges, nblocks, sigma, limit_ns, s);
  if (phase == 1 && nb == 128) return launch_tc_sigma_nb<1, 128>(b, work, ranges, nblocks, sigma, limit_ns, s);
  if (phase == 2 && nb == 128) return launch_tc_sigma_nb<2, 128>(b, work, ranges, nblocks, sigma, limit_ns, s);
  return cudaErrorInvalidValue;
}

int tc_blocks_per_sm(int nb) { return nb == 64 ? TcCfg<64>::kBlocksPerSm : TcCfg<128>::kBlocksPerSm; }

cudaError_t launch_tc_sigma_pairs(const TcBufs& b, const TcWork* work, const int2* ranges, int nblocks, double* sigma,
                                  uint64_t limit_ns, cudaStream_t s) {
  if (nblocks <= 0) return cudaGetLastError();
  if (nblocks % 2) return cudaErrorInvalidValue;
  constexpr int smem = TcCfg<128>::kSmem;
  auto kern = tc_sigma_kernel<2, 128, true>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblocks);
  cfg.blockDim = dim3(kTcThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, kern, b, work, ranges, sigma, limit_ns);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

__global__ void __launch_bounds__(256) tc_reduce_kernel(const float2* __restrict__ partials,
                                                         const TcTile* __restrict__ tiles,
                                                         const int64_t* __restrict__ slots, double* __restrict__ sigma) {
  const TcTile t = tiles[blockIdx.x];
  const int n = t.h * t.w;
  for (int e = blockIdx.y * blockDim.x + threadIdx.x; e < n; e += gridDim.y * blockDim.x) {
    double acc = 0.0;
    const int r = e / t.w, c = e % t.w;
    for (int p = t.pbeg; p < t.pend; ++p) {
      const float2 v = partials[slots[p] + (int64_t)r * t.pad + c];  // slots are h_a x h_b, row stride pad
      acc += (double)v.x + (double)v.y;
    }
    sigma[t.s_off + (int64_t)(t.r0 + r) * t.lds + t.c0 + c] = acc;
  }
}

cudaError_t launch_tc_reduce(const TcBufs& b, const TcTile* tiles, const int64_t* slots, int ntiles, double* sigma,
                             cudaStream_t s) {
  if (ntiles > 0) tc_reduce_kernel<<<dim3(ntiles, 16), 256, 0, s>>>(b.partials, tiles, slots, sigma);
  return cudaGetLastError();
}

// Waits on an mbarrier that nothing arrives at, through the same bounded
// wait the sigma kernels use; the wait must give up after limit_ns and set
// *status.  out[0] = 1 if the wait reported failure, out[1] = elapsed ns.
__global__ void tc_wait_selftest_kernel(int* status, unsigned long long* out, uint64_t limit_ns) {
  __shared__ uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
    abort_flag = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint64_t t0 = globaltimer_ns();
    const bool ok = tc_wait(&bar, 0, &abort_flag, status, limit_ns);
    out[0] = ok ? 0ull : 1ull;
    out[1] = globaltimer_ns() - t0;
  }
}

cudaError_t launch_tc_wait_selftest(int* status, unsigned long long* out, uint64_t limit_ns, cudaStream_t s) {
  tc_wait_selftest_kernel<<<1, 32, 0, s>>>(status, out, limit_ns);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bgpu
