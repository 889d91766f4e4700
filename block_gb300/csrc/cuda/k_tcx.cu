// Exact-slice products on tcgen05 (see k_tc.cuh, "exact"): row exponents,
// six-digit packing, the two sigma phases and the FP64 reduction of split
// tiles.
#include "k_tc.cuh"
#include "tc.cuh"

namespace bgpu {
namespace dev {

using namespace tc;

namespace {

template <class T, int N>
__device__ __forceinline__ T pick_x(const T (&p)[N], int i) {
  T r = p[0];
#pragma unroll
  for (int k = 1; k < N; ++k)
    if (i == k) r = p[k];
  return r;
}

// unbiased binary exponent of a normal FP64 number (kTcxNoExp for zero and
// subnormal values, which the digits treat as zero)
__device__ __forceinline__ int exp_of(double x) {
  const int e = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
  return e == 0 ? kTcxNoExp : e - 1023;
}

// the six balanced base-128 digits of x / 2^e (e > exponent of x), most
// significant first: x = 2^e sum_s d[s] 2^-7(s+1) up to 2^(e-43)
__device__ __forceinline__ void digits6(double x, int e, int (&d)[kTcxSlices]) {
  const uint64_t bits = (uint64_t)__double_as_longlong(x);
  const int be = (int)((bits >> 52) & 0x7ff);
  uint64_t M = 0;
  if (be != 0) {
    const uint64_t mant = (bits & ((1ull << 52) - 1)) | (1ull << 52);
    // |x| = mant 2^(be-1023-52);  M = round(|x| 2^(42-e)) = mant >> sh
    const int sh = e - (be - 1023) + 10;  // >= 11
    if (sh < 64) M = (mant + (1ull << (sh - 1))) >> sh;
  }
  // offset 64 in each of the five lower digits makes them balanced
  constexpr uint64_t C = 64ull * (1ull + (1ull << 7) + (1ull << 14) + (1ull << 21) + (1ull << 28));
  const uint64_t Mp = M + C;
  const int sg = (bits >> 63) ? -1 : 1;
  d[0] = sg * (int)(Mp >> 35);
#pragma unroll
  for (int s = 1; s < kTcxSlices; ++s) d[s] = sg * ((int)((Mp >> (7 * (5 - s))) & 127) - 64);
}

__device__ __forceinline__ uint32_t bf16_bits(int v) {
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn((float)v));
}

// x 2^k, by the exponent field where the result stays normal
__device__ __forceinline__ double scale_pow2(double x, int k) {
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e != 0 && e + k >= 1 && e + k <= 2046) return __longlong_as_double(b + ((long long)k << 52));
  return ldexp(x, k);
}

// Row exponents of one packed operand per block: rows of a row-major view
// one warp each (lanes along K), rows of a transposed view one thread each
// (threads along the source's contiguous rows).
__global__ void __launch_bounds__(256) tcx_rowexp_kernel(TcxBufs b, const TcPack* __restrict__ units) {
  const TcPack u = units[blockIdx.x];
  const double* src = pick_x(b.src, u.src) + u.src_off;
  int* ex = pick_x(b.ex, u.pool) + u.ex_off;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (!u.trans) {
    for (int r = warp; r < u.rows_p; r += 8) {
      int m = kTcxNoExp;
      if (r < u.rows_v)
        for (int k = lane; k < u.cols_v; k += 32) m = max(m, exp_of(src[(int64_t)r * u.ld + k]));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
      if (lane == 0) ex[r] = m;
    }
  } else {
    for (int r = tid; r < u.rows_p; r += 256) {
      int m = kTcxNoExp;
      if (r < u.rows_v)
        for (int k = 0; k < u.cols_v; ++k) m = max(m, exp_of(src[(int64_t)k * u.ld + r]));
      ex[r] = m;
    }
  }
}

// Six digit slices per element; each thread writes one 16-byte core-matrix
// row (8 consecutive K of one row) of every slice.  Within the block of a
// K-chunk (h rows x w columns, six slices), each 16-column half holds the six
// slices of h x 16 one after another (slice s of half p at element
// (6 p + s) h 16), each in the K-major core-matrix order, so that one bulk
// copy moves the operand piece of one K=16 step.
__global__ void __launch_bounds__(256) tcx_pack_kernel(TcxBufs b, const TcPack* __restrict__ units) {
  const TcPack u = units[blockIdx.x];
  const double* src = pick_x(b.src, u.src) + u.src_off;
  __nv_bfloat16* dst = pick_x(b.pool, u.pool) + u.dst_off;
  const int* ex = pick_x(b.ex, u.pool) + u.ex_off;
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
    const int em = ex[r];
    const bool zero_row = em <= kTcxNoExp / 2;
    uint32_t w[kTcxSlices][4];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int k = k0 + e;
      double x = 0.0;
      if (!zero_row && r < u.rows_v && k < u.cols_v) x = u.trans ? src[(int64_t)k * u.ld + r] : src[(int64_t)r * u.ld + k];
      int d[kTcxSlices];
      digits6(x, zero_row ? 0 : em + 1, d);
#pragma unroll
      for (int s = 0; s < kTcxSlices; ++s) {
        const uint32_t v = bf16_bits(d[s]);
        if (e & 1) w[s][e >> 1] |= v << 16;
        else w[s][e >> 1] = v;
      }
    }
    const int t = r / u.rt, c = k0 / kTcKC, kk = k0 % kTcKC;
    const int rest = u.rows_p - u.rt * t;
    const int h = rest < u.rt ? rest : u.rt;
    // half kk / 16 of the chunk: six slices of h x 16, one after another
    const int64_t off = (int64_t)kTcxSlices * tc_block_off(u.rows_p, u.kp, t, c, u.rt) +
                        (int64_t)(kk / kTcxKS) * kTcxSlices * h * kTcxKS + (kmajor_off(r - u.rt * t, kk % kTcxKS, h) >> 1);
#pragma unroll
    for (int s = 0; s < kTcxSlices; ++s)
      *(uint4*)(dst + off + (int64_t)s * h * kTcxKS) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
  }
}

constexpr int kTcxSlots = 4;  // stages of one K=16 step
constexpr uint32_t kTcxStageBytes = (uint32_t)kTcxSlices * (kTcRowsA + kTcxNB) * kTcxKS * 2;
constexpr int kTcxAccBytes = kTcRowsA * kTcxNB * 8;  // FP64 tile accumulator, column-major
constexpr int kTcxSmem = kTcxSlots * (int)kTcxStageBytes + kTcxAccBytes;
constexpr uint32_t kTcxTmemCols = 512;  // six accumulators of 64 columns
// warps 0-7 epilogue (warp w: TMEM lanes 32 (w % 4).., tile columns
// 32 (w / 4)..), 8 producer, 9 MMA issuer
constexpr int kTcxEpiWarps = 8;
constexpr int kTcxThreads = 32 * (kTcxEpiWarps + 2);
constexpr int kTcxProducer = kTcxEpiWarps, kTcxIssuer = kTcxEpiWarps + 1;
constexpr int kTcxHalf = kTcxNB / 2;  // tile columns per epilogue warp
constexpr int kTcxStepsPerBlock = kTcxKBlock / kTcxKS;

struct TcxShared {
  uint64_t full[kTcxSlots], empty[kTcxSlots], acc_full, acc_empty, drain;
  uint32_t tbase;
  int abort_flag;
};

__device__ bool tcx_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, int* status, uint64_t limit_ns) {
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

struct XRegs {
  int4 q[5];
};
__device__ __forceinline__ void load_xwork(const TcxWork* __restrict__ w, int idx, int end, XRegs& r) {
  if (idx < end) {
    const int4* p = reinterpret_cast<const int4*>(w + idx);
#pragma unroll
    for (int i = 0; i < 5; ++i) r.q[i] = __ldg(p + i);
  } else {
#pragma unroll
    for (int i = 0; i < 5; ++i) r.q[i] = make_int4(0, 0, 0, 0);
  }
}
__device__ __forceinline__ int64_t xshfl64(int lo, int hi, int j) {
  const uint32_t l = (uint32_t)__shfl_sync(0xffffffffu, lo, j), h = (uint32_t)__shfl_sync(0xffffffffu, hi, j);
  return (int64_t)(((uint64_t)h << 32) | l);
}
__device__ __forceinline__ int xshfl(int v, int j) { return __shfl_sync(0xffffffffu, v, j); }

// field access of a record held as five int4 (layout of TcxWork)
struct XRec {
  int64_t a_base, b_base, out_base;
  double alpha;
  int kp, out_ld, col0, a_ex, b_ex, o_ex;
  int h_a, h_b, valid_rows, valid_cols;
  int a_pool, b_pool, flags;
};
__device__ __forceinline__ XRec xrec(const XRegs& r, int j) {
  XRec x;
  x.a_base = xshfl64(r.q[0].x, r.q[0].y, j);
  x.b_base = xshfl64(r.q[0].z, r.q[0].w, j);
  x.out_base = xshfl64(r.q[1].x, r.q[1].y, j);
  x.alpha = __longlong_as_double(xshfl64(r.q[1].z, r.q[1].w, j));
  x.kp = xshfl(r.q[2].x, j);
  x.out_ld = xshfl(r.q[2].y, j);
  x.col0 = xshfl(r.q[2].z, j);
  x.a_ex = xshfl(r.q[2].w, j);
  x.b_ex = xshfl(r.q[3].x, j);
  x.o_ex = xshfl(r.q[3].y, j);
  const int hw = xshfl(r.q[3].z, j), vv = xshfl(r.q[3].w, j), pf = xshfl(r.q[4].x, j);
  x.h_a = hw & 0xffff;
  x.h_b = (hw >> 16) & 0xffff;
  x.valid_rows = vv & 0xffff;
  x.valid_cols = (vv >> 16) & 0xffff;
  x.a_pool = pf & 0xff;
  x.b_pool = (pf >> 8) & 0xff;
  x.flags = (pf >> 16) & 0xff;
  return x;
}

// 32 lanes x 16 columns of six accumulators, one wait
__device__ __forceinline__ void tmem_ld16x6(uint32_t t, uint32_t (&r)[kTcxSlices][16]) {
#pragma unroll
  for (int q = 0; q < kTcxSlices; ++q) {
    const uint32_t a = t + (uint32_t)(q * kTcxNB);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[q][0]), "=r"(r[q][1]), "=r"(r[q][2]), "=r"(r[q][3]), "=r"(r[q][4]), "=r"(r[q][5]), "=r"(r[q][6]),
          "=r"(r[q][7]), "=r"(r[q][8]), "=r"(r[q][9]), "=r"(r[q][10]), "=r"(r[q][11]), "=r"(r[q][12]),
          "=r"(r[q][13]), "=r"(r[q][14]), "=r"(r[q][15])
        : "r"(a));
  }
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace

// Persistent grouped exact-slice GEMM: per K=16 step the 21 digit products
// (s, u), s + u <= 5, into accumulator s + u; accumulators are read out after
// every kTcxKBlock K of an item and at its end (the MMA issuer waits for
// the read-out before the next K block).  Phase 1 writes the T tiles (FP64)
// and reduces their row exponents; phase 2 sums the items of a task in an
// FP64 shared-memory tile and writes sigma or a partial tile.
template <int PHASE>
__global__ void __launch_bounds__(kTcxThreads, 1)
    tcx_sigma_kernel(TcxBufs b, const TcxWork* __restrict__ work, const int2* __restrict__ ranges,
                     double* __restrict__ sigma, uint64_t limit_ns) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ TcxShared sh;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int2 rg = ranges[blockIdx.x];
  if (warp == kTcxIssuer) {
    tmem_alloc(&sh.tbase, kTcxTmemCols);
    tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < kTcxSlots; ++i) {
      mbar_init(&sh.full[i], 1);
      mbar_init(&sh.empty[i], 1);
    }
    mbar_init(&sh.acc_full, 1);
    mbar_init(&sh.acc_empty, kTcxEpiWarps);
    mbar_init(&sh.drain, 1);
    sh.abort_flag = 0;
    mbar_fence_init();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = sh.tbase;
  volatile int* abort_flag = &sh.abort_flag;
  double* accs = reinterpret_cast<double*>(smem + kTcxSlots * kTcxStageBytes);

  if (warp == kTcxProducer) {
    uint32_t k = 0;
    bool ok = true;
    for (int base = rg.x; base < rg.y && ok; base += 32) {
      XRegs r;
      load_xwork(work, base + lane, rg.y, r);
      const int cnt = min(32, rg.y - base);
      for (int j = 0; j < cnt && ok; ++j) {
        const XRec x = xrec(r, j);
        if (lane == 0 && !(x.flags & kTcEmpty)) {
          const __nv_bfloat16* pa = pick_x(b.pool, x.a_pool) + x.a_base;
          const __nv_bfloat16* pb = pick_x(b.pool, x.b_pool) + x.b_base;
          // one stage per K=16 step: half st % 2 of chunk st / 2
          const int nst = x.kp / kTcxKS;
          const uint32_t abytes = (uint32_t)kTcxSlices * x.h_a * kTcxKS * 2;
          const uint32_t bbytes = (uint32_t)kTcxSlices * x.h_b * kTcxKS * 2;
          for (int st = 0; st < nst; ++st, ++k) {
            const int slot = (int)(k % kTcxSlots);
            if (!tcx_wait(&sh.empty[slot], ((k / kTcxSlots) & 1u) ^ 1u, abort_flag, b.status, limit_ns)) {
              ok = false;
              break;
            }
            uint8_t* dst = smem + slot * kTcxStageBytes;
            const int64_t ha = (int64_t)kTcxSlices * x.h_a * kTcxKS, hb = (int64_t)kTcxSlices * x.h_b * kTcxKS;
            mbar_expect_tx(&sh.full[slot], abytes + bbytes);
            bulk_g2s(dst, pa + ha * st, abytes, &sh.full[slot]);
            bulk_g2s(dst + abytes, pb + hb * st, bbytes, &sh.full[slot]);
          }
        }
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      }
    }
    if (lane == 0 && !ok)
      for (uint32_t i = (k > kTcxSlots ? k - kTcxSlots : 0); i < k; ++i)
        mbar_wait_bounded(&sh.full[i % kTcxSlots], (i / kTcxSlots) & 1u, limit_ns);
  } else if (warp == kTcxIssuer) {
    uint32_t k = 0, nblk = 0;
    bool ok = true;
    for (int base = rg.x; base < rg.y && ok; base += 32) {
      XRegs r;
      load_xwork(work, base + lane, rg.y, r);
      const int cnt = min(32, rg.y - base);
      for (int j = 0; j < cnt && ok; ++j) {
        const XRec x = xrec(r, j);
        if (lane == 0 && !(x.flags & kTcEmpty)) {
          const uint32_t idesc = idesc_bf16(128, (x.h_b + 15) & ~15);
          const int nst = x.kp / kTcxKS;
          for (int st = 0; st < nst && ok; ++st, ++k) {
            const bool blk_first = (st % kTcxStepsPerBlock) == 0;
            const bool blk_last = (st % kTcxStepsPerBlock) == kTcxStepsPerBlock - 1 || st == nst - 1;
            if (blk_first && !tcx_wait(&sh.acc_empty, (nblk & 1u) ^ 1u, abort_flag, b.status, limit_ns)) {
              ok = false;
              break;
            }
            const int slot = (int)(k % kTcxSlots);
            if (!tcx_wait(&sh.full[slot], (k / kTcxSlots) & 1u, abort_flag, b.status, limit_ns)) {
              ok = false;
              break;
            }
            fence_after_sync();
            const uint32_t sa = smem_u32(smem + slot * kTcxStageBytes);
            const uint32_t sa_slice = (uint32_t)x.h_a * kTcxKS * 2, sb_slice = (uint32_t)x.h_b * kTcxKS * 2;
            const uint32_t sb = sa + (uint32_t)kTcxSlices * sa_slice;
#pragma unroll
            for (int q = 0; q < kTcxSlices; ++q) {
              const uint32_t d = tmem + (uint32_t)(q * kTcxNB);
#pragma unroll
              for (int s = 0; s <= q; ++s) {
                const int u = q - s;
                const uint64_t da = smem_desc(sa + (uint32_t)s * sa_slice, x.h_a * 16, 128);
                const uint64_t db = smem_desc(sb + (uint32_t)u * sb_slice, x.h_b * 16, 128);
                mma_bf16(d, da, db, idesc, (blk_first && s == 0) ? 0u : 1u);
              }
            }
            mma_commit(&sh.empty[slot]);
            if (blk_last) {
              mma_commit(&sh.acc_full);
              ++nblk;
            }
          }
        }
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      }
    }
  } else {
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4).. and owns tile
    // columns 32 (w / 4).. of its rows in the column-major FP64 tile
    // accumulator; thread `row` owns row `row` of those columns
    const int row = 32 * (warp & 3) + lane;
    const int cb0 = kTcxHalf * (warp >> 2);
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
    uint32_t nblk = 0;
    bool ok = true;
    for (int base = rg.x; base < rg.y && ok; base += 32) {
      XRegs r;
      load_xwork(work, base + lane, rg.y, r);
      const int cnt = min(32, rg.y - base);
      for (int j = 0; j < cnt && ok; ++j) {
        const XRec x = xrec(r, j);
        if (x.flags & kTcFirst)
          for (int c = cb0; c < cb0 + kTcxHalf; ++c) accs[c * kTcRowsA + row] = 0.0;
        if (!(x.flags & kTcEmpty)) {
          // row exponent of this thread's row, column exponent of the
          // warp's column cb0 + lane (read before the wait, so that the
          // loads overlap the MMAs)
          const int* exa = pick_x(b.ex, x.a_pool) + x.a_ex;
          const int* exb = pick_x(b.ex, x.b_pool) + x.b_ex;
          const int ea = row < x.h_a ? __ldg(exa + row) : kTcxNoExp;
          const int eb_l = cb0 + lane < x.h_b ? __ldg(exb + cb0 + lane) : kTcxNoExp;
          const bool live_a = ea > kTcxNoExp / 2;
          const int nkb = (x.kp + kTcxKBlock - 1) / kTcxKBlock;
          for (int kb = 0; kb < nkb; ++kb) {
            ok = __all_sync(0xffffffffu, tcx_wait(&sh.acc_full, nblk & 1u, abort_flag, b.status, limit_ns));
            if (!ok) break;
            fence_after_sync();
#pragma unroll 1
            for (int g = 0; g < kTcxHalf / 16; ++g) {
              const int cb = cb0 + 16 * g;
              if (cb >= x.h_b) break;  // warp-uniform
              uint32_t v[kTcxSlices][16];
              tmem_ld16x6(tmem + lane_base + (uint32_t)cb, v);
              double y[16];
#pragma unroll
              for (int e = 0; e < 16; ++e) {
                const int eb = __shfl_sync(0xffffffffu, eb_l, 16 * g + e);  // kTcxNoExp beyond h_b
                // the accumulators hold integers below 2^24 in magnitude:
                // 32-bit conversions (not the FP64 pipe's 64-bit ones)
                long long a = 0;
#pragma unroll
                for (int q = 0; q < kTcxSlices; ++q)
                  a += (long long)__float2int_rn(__uint_as_float(v[q][e])) * (1ll << (7 * (kTcxSlices - 1 - q)));
                const bool live = live_a && eb > kTcxNoExp / 2 && a != 0;
                y[e] = live ? scale_pow2((double)a, (ea + 1) + (eb + 1) - 7 * (kTcxSlices + 1)) : 0.0;
              }
              if (live_a) {
                double* p = accs + cb * kTcRowsA + row;
                double acc[16];
#pragma unroll
                for (int e = 0; e < 16; ++e) acc[e] = p[e * kTcRowsA];
#pragma unroll
                for (int e = 0; e < 16; ++e) p[e * kTcRowsA] = fma(y[e], x.alpha, acc[e]);
              }
            }
            // accumulators read: the MMA issuer may start the next K block
            fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(&sh.acc_empty);
            ++nblk;
          }
          if (!ok) break;
        }
        if (!(x.flags & kTcLast)) continue;
        // the task's tile is complete in this thread's row and columns
        const int ce = cb0 + kTcxHalf;
        if (PHASE == 1) {
          if (row < x.h_a) {
            const int ncols = min(kTcxNB, x.out_ld - x.col0);
            double* out = b.t + x.out_base + (int64_t)row * x.out_ld + x.col0;
            int m = kTcxNoExp;
            for (int c = cb0; c < min(ncols, ce); ++c) {
              const double v = c < x.h_b ? accs[c * kTcRowsA + row] : 0.0;
              out[c] = v;
              m = max(m, exp_of(v));
            }
            if (m > kTcxNoExp / 2) atomicMax(b.ex[kTcPoolS] + x.o_ex + row, m);
          }
        } else if (x.flags & kTcDirect) {
          if (row < x.valid_rows) {
            double* out = sigma + x.out_base + (int64_t)row * x.out_ld;
            for (int c = cb0; c < min(x.valid_cols, ce); ++c) out[c] = accs[c * kTcRowsA + row];
          }
        } else if (row < x.h_a) {
          double* out = b.partials + x.out_base + (int64_t)row * x.h_b;
          for (int c = cb0; c < min(x.h_b, ce); ++c) out[c] = accs[c * kTcRowsA + row];
        }
      }
    }
  }
  __syncthreads();
  if (warp == kTcxIssuer) {
    if (lane == 0) {
      mma_commit(&sh.drain);
      mbar_wait_bounded(&sh.drain, 0, limit_ns);
    }
    __syncwarp();
    fence_after_sync();
    tmem_dealloc(tmem, kTcxTmemCols);
  }
}

__global__ void __launch_bounds__(256) tcx_reduce_kernel(const double* __restrict__ partials,
                                                          const TcTile* __restrict__ tiles,
                                                          const int64_t* __restrict__ slots, double* __restrict__ sigma) {
  const TcTile t = tiles[blockIdx.x];
  const int n = t.h * t.w;
  for (int e = blockIdx.y * blockDim.x + threadIdx.x; e < n; e += gridDim.y * blockDim.x) {
    double acc = 0.0;
    const int r = e / t.w, c = e % t.w;
    for (int p = t.pbeg; p < t.pend; ++p) acc += partials[slots[p] + (int64_t)r * t.pad + c];
    sigma[t.s_off + (int64_t)(t.r0 + r) * t.lds + t.c0 + c] = acc;
  }
}

__global__ void fill_int_kernel(int* x, int64_t n, int v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] = v;
}

cudaError_t launch_tcx_rowexp(const TcxBufs& b, const TcPack* units, int nunits, cudaStream_t s) {
  if (nunits > 0) tcx_rowexp_kernel<<<nunits, 256, 0, s>>>(b, units);
  return cudaGetLastError();
}

cudaError_t launch_tcx_pack(const TcxBufs& b, const TcPack* units, int nunits, cudaStream_t s) {
  if (nunits > 0) tcx_pack_kernel<<<dim3(nunits, 4), 256, 0, s>>>(b, units);
  return cudaGetLastError();
}

template <int PHASE>
static cudaError_t launch_tcx_phase(const TcxBufs& b, const TcxWork* work, const int2* ranges, int nblocks,
                                    double* sigma, uint64_t limit_ns, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(tcx_sigma_kernel<PHASE>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcxSmem);
  if (e != cudaSuccess) return e;
  tcx_sigma_kernel<PHASE><<<nblocks, kTcxThreads, kTcxSmem, s>>>(b, work, ranges, sigma, limit_ns);
  return cudaGetLastError();
}

cudaError_t launch_tcx_sigma(int phase, const TcxBufs& b, const TcxWork* work, const int2* ranges, int nblocks,
                             double* sigma, uint64_t limit_ns, cudaStream_t s) {
  if (nblocks <= 0) return cudaGetLastError();
  if (phase == 1) return launch_tcx_phase<1>(b, work, ranges, nblocks, sigma, limit_ns, s);
  if (phase == 2) return launch_tcx_phase<2>(b, work, ranges, nblocks, sigma, limit_ns, s);
  return cudaErrorInvalidValue;
}

int tcx_blocks_per_sm() { return 1; }

cudaError_t launch_tcx_reduce(const TcxBufs& b, const TcTile* tiles, const int64_t* slots, int ntiles, double* sigma,
                              cudaStream_t s) {
  if (ntiles > 0) tcx_reduce_kernel<<<dim3(ntiles, 16), 256, 0, s>>>(b.partials, tiles, slots, sigma);
  return cudaGetLastError();
}

cudaError_t launch_fill_int(int* x, int64_t n, int v, cudaStream_t s) {
  if (n > 0) fill_int_kernel<<<(int)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, s>>>(x, n, v);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bgpu
