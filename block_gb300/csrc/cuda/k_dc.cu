// Divide and conquer for the tridiagonal eigenproblems of the batched
// eigensolver; see k_dc.cuh for the method and the data layout.
#include <cmath>

#include "k_dc.cuh"

namespace bgpu {
namespace dev {
namespace {

constexpr double kEps = 2.220446049250313e-16;
constexpr int kLeafWarps = 4;
constexpr int kDefThreads = 256;
constexpr int kWarpThreads = 256;  // warps-per-slot kernels: 8 warps per CTA
constexpr int kColThreads = 128;   // CTA-per-column kernels
constexpr int kSecularIters = 256;
constexpr int kLeafIters = 60;     // QL sweeps per eigenvalue of a leaf

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ double warp_prod(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x *= __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ double warp_max(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// scalar work area of a job (k_eig.cu): d, e, tau, unsorted eigenvalues, ...
__device__ __forceinline__ double* diag_of(double* work, const EigJob& J) { return work + J.s_off; }
__device__ __forceinline__ double* offd_of(double* work, const EigJob& J) { return work + J.s_off + J.n; }
__device__ __forceinline__ double* eig_of(double* work, const EigJob& J) { return work + J.s_off + 3ll * J.n; }

// the merge that owns a level slot
__device__ __forceinline__ int find_merge(const DcLevel& L, int64_t slot) {
  int lo = 0, hi = L.nmerges - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (L.merges[mid].x_off <= slot) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void dc_tear_kernel(double* work, const EigJob* __restrict__ jobs, const DcMerge* __restrict__ merges,
                               int nmerges) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nmerges) return;
  const DcMerge M = merges[i];
  const EigJob J = jobs[M.job];
  double* d = diag_of(work, J);
  const int t = M.o + M.n1;
  const double b = fabs(offd_of(work, J)[t - 1]);
  d[t - 1] -= b;
  d[t] -= b;
}

// One warp per leaf: implicit QL with Wilkinson shifts (the iteration of
// the large solver, k_eig.cu, in one warp): lane 0 runs the scalar
// recurrence of one sweep and leaves its rotations in shared memory, then
// every lane applies them to its row of the leaf's Z.
__global__ void __launch_bounds__(32 * kLeafWarps) dc_leaf_kernel(double* work, const EigJob* __restrict__ jobs,
                                                                  const DcLeaf* __restrict__ leaves, int nleaves,
                                                                  int* status) {
  __shared__ double zs[kLeafWarps][kDcLeaf * kDcLeaf];
  __shared__ double dd[kLeafWarps][kDcLeaf], ee[kLeafWarps][kDcLeaf];
  __shared__ double2 rb[kLeafWarps][kDcLeaf];
  __shared__ int ctl[kLeafWarps][3];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int li = blockIdx.x * kLeafWarps + w;
  if (li >= nleaves) return;  // the whole warp leaves; the CTA never synchronises
  const DcLeaf Lf = leaves[li];
  const EigJob J = jobs[Lf.job];
  const int n = J.n, len = Lf.len, o = Lf.o;
  double* __restrict__ z = zs[w];
  double* __restrict__ d = dd[w];
  double* __restrict__ e = ee[w];
  for (int c = 0; c < kDcLeaf; ++c) z[c * kDcLeaf + lane] = c == lane ? 1.0 : 0.0;
  if (lane < len) {
    d[lane] = diag_of(work, J)[o + lane];
    e[lane] = lane < len - 1 ? offd_of(work, J)[o + lane] : 0.0;
  }
  __syncwarp();
  int l = 0, it = 0;
  bool fail = false;
  double tiny = 0.0;
  if (lane == 0) {
    double tn = 0.0;
    for (int i = 0; i < len; ++i) tn = fmax(tn, fabs(d[i]) + fabs(e[i]));
    tiny = kEps * tn;
  }
  while (true) {
    if (lane == 0) {
      int m = -1, cnt = 0;
      while (l < len) {
        m = l;
        while (m < len - 1) {
          if (fabs(e[m]) <= tiny) break;
          ++m;
        }
        if (m == l) {
          ++l;
          it = 0;
          continue;
        }
        if (++it > kLeafIters) {
          fail = true;
          l = len;
          m = -1;
          break;
        }
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        double r = hypot(g, 1.0);
        g = d[m] - d[l] + e[l] / (g + copysign(r, g));
        double s = 1.0, c = 1.0, p = 0.0;
        bool early = false;
        for (int i = m - 1; i >= l; --i) {
          const double f = s * e[i], bb = c * e[i];
          r = hypot(f, g);
          e[i + 1] = r;
          if (r == 0.0) {
            d[i + 1] -= p;
            e[m] = 0.0;
            early = true;
            break;
          }
          s = f / r;
          c = g / r;
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0 * c * bb;
          p = s * r;
          d[i + 1] = g + p;
          g = c * r - bb;
          rb[w][cnt++] = make_double2(c, s);
        }
        if (!early) {
          d[l] -= p;
          e[l] = g;
          e[m] = 0.0;
        }
        if (cnt > 0) break;
        m = -1;
      }
      ctl[w][0] = m;
      ctl[w][1] = cnt;
      ctl[w][2] = (m < 0 || cnt == 0) ? 1 : 0;
    }
    __syncwarp();
    if (ctl[w][2]) break;
    {
      const int m = ctl[w][0], cnt = ctl[w][1], r = lane;
      double zi1 = z[m * kDcLeaf + r];
      for (int x = 0; x < cnt; ++x) {
        const int i = m - 1 - x;
        const double2 cs = rb[w][x];
        const double zi = z[i * kDcLeaf + r];
        z[(i + 1) * kDcLeaf + r] = cs.y * zi + cs.x * zi1;
        zi1 = cs.x * zi - cs.y * zi1;
      }
      z[(m - cnt) * kDcLeaf + r] = zi1;
    }
    __syncwarp();
  }
  double* __restrict__ Z = work + J.q_off;
  if (lane < len) eig_of(work, J)[o + lane] = d[lane];
  for (int c = 0; c < len; ++c)
    if (lane < len) Z[(int64_t)(o + c) * n + o + lane] = z[c * kDcLeaf + lane];
  if (lane == 0 && fail) status[Lf.job] = -1;
}

// One CTA per merge: the sorted poles, their weights z, the deflation of
// small weights and of close pairs (whose Givens rotations are applied to the
// block's columns of Z here), and the poles that remain.
__global__ void __launch_bounds__(kDefThreads) dc_deflate_kernel(double* work, const EigJob* __restrict__ jobs,
                                                                 DcLevel L) {
  extern __shared__ double sm[];
  __shared__ double red[kDefThreads / 32];
  __shared__ int nrot_s;
  const int tid = threadIdx.x;
  const DcMerge M = L.merges[blockIdx.x];
  const EigJob J = jobs[M.job];
  const int n = J.n, o = M.o, n1 = M.n1, nm = M.nm;
  int P = 1;
  while (P < nm) P <<= 1;
  double* key = sm;
  double* zs = sm + P;
  int* idx = reinterpret_cast<int*>(sm + 2 * P);
  double* __restrict__ Z = work + J.q_off;
  const double* eu = eig_of(work, J);
  const double beta = offd_of(work, J)[o + n1 - 1];
  const double sg = beta < 0.0 ? -1.0 : 1.0;
  for (int c = tid; c < P; c += kDefThreads) {
    key[c] = c < nm ? eu[o + c] : 1.7e308;
    idx[c] = c;
  }
  for (int c = tid; c < nm; c += kDefThreads)
    zs[c] = c < n1 ? Z[(int64_t)(o + c) * n + (o + n1 - 1)] : sg * Z[(int64_t)(o + c) * n + (o + n1)];
  __syncthreads();
  // bitonic sort of (key, idx), ascending, ties by index
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < P; i += kDefThreads) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const double a = key[i], b = key[ixj];
          const int ia = idx[i], ib = idx[ixj];
          const bool gt = a > b || (a == b && ia > ib);
          if (gt == ((i & k) == 0)) {
            key[i] = b;
            key[ixj] = a;
            idx[i] = ib;
            idx[ixj] = ia;
          }
        }
      }
      __syncthreads();
    }
  // |Q^T v|^2 and max |z| (fixed-order reductions)
  double s2 = 0.0, zm = 0.0;
  for (int c = tid; c < nm; c += kDefThreads) {
    s2 += zs[c] * zs[c];
    zm = fmax(zm, fabs(zs[c]));
  }
  s2 = warp_sum(s2);
  zm = warp_max(zm);
  if ((tid & 31) == 0) red[tid >> 5] = s2;
  __syncthreads();
  double zn2 = 0.0;
  for (int i = 0; i < kDefThreads / 32; ++i) zn2 += red[i];
  __syncthreads();
  if ((tid & 31) == 0) red[tid >> 5] = zm;
  __syncthreads();
  double zmax = 0.0;
  for (int i = 0; i < kDefThreads / 32; ++i) zmax = fmax(zmax, red[i]);
  if (tid == 0) {
    const int64_t x = M.x_off;
    const double zsc = zn2 > 0.0 ? 1.0 / sqrt(zn2) : 0.0;
    const double rho = fabs(beta) * zn2;
    const double tol = 8.0 * kEps * fmax(fmax(fabs(key[0]), fabs(key[nm - 1])), zmax * zsc);
    int K = 0, nd = 0, nrot = 0;
    auto pole = [&](double dv, double zv, int cv) {
      L.dk[x + K] = dv;
      L.zk[x + K] = zv;
      L.col[x + K] = cv;
      ++K;
    };
    auto deflate = [&](double dv, int cv) {  // from the end of the slots
      ++nd;
      L.dk[x + nm - nd] = dv;
      L.col[x + nm - nd] = cv;
    };
    bool have = false;
    double pd = 0.0, pz = 0.0;
    int pc = -1;
    for (int t = 0; t < nm; ++t) {
      const double dt = key[t];
      const int ct = idx[t];
      const double zt = zs[ct] * zsc;
      if (rho * fabs(zt) <= tol) {
        deflate(dt, ct);
        continue;
      }
      if (!have) {
        have = true;
        pd = dt;
        pz = zt;
        pc = ct;
        continue;
      }
      // close pair: |(d_t - d_p) c s| <= tol for the rotation that zeroes z_p
      const double r2 = zt * zt + pz * pz;
      if (fabs((dt - pd) * zt * pz) <= tol * r2) {
        const double tau = sqrt(r2), c = zt / tau, s = -pz / tau;
        L.rot_cols[x + nrot] = make_int2(pc, ct);
        L.rot_cs[x + nrot] = make_double2(c, s);
        ++nrot;
        deflate(pd * c * c + dt * s * s, pc);
        pd = pd * s * s + dt * c * c;
        pz = tau;
        pc = ct;
      } else {
        pole(pd, pz, pc);
        pd = dt;
        pz = zt;
        pc = ct;
      }
    }
    if (have) pole(pd, pz, pc);
    L.K[blockIdx.x] = K;
    L.nrot[blockIdx.x] = nrot;
    L.rho[blockIdx.x] = rho;
    nrot_s = nrot;
  }
  __syncthreads();
  // the rotations, in order, on the block's rows (each thread owns its rows):
  // column p <- c p + s q, column q <- -s p + c q
  const int nrot = nrot_s;
  for (int r = tid; r < nm; r += kDefThreads)
    for (int t = 0; t < nrot; ++t) {
      const int2 pq = L.rot_cols[M.x_off + t];
      const double2 cs = L.rot_cs[M.x_off + t];
      double* zp = Z + (int64_t)(o + pq.x) * n + o + r;
      double* zq = Z + (int64_t)(o + pq.y) * n + o + r;
      const double a = *zp, b = *zq;
      *zp = cs.x * a + cs.y * b;
      *zq = -cs.y * a + cs.x * b;
    }
}

// One warp per root j of a merge's secular equation
//   f(lambda) = 1/rho + sum_i z_i^2 / (d_i - lambda) = 0,
// root j in (d_j, d_{j+1}) (the last one in (d_{K-1}, d_{K-1} + rho)), kept
// as lambda = d_o + tau with o the nearer pole, so that every d_i - lambda is
// formed as (d_i - d_o) - tau without cancellation.  Each step models the
// poles left and right of the root by one pole each, matching the value and
// derivative of their sums, solves the model exactly and falls back to
// bisection of the bracket when the model leaves it.
__global__ void __launch_bounds__(kWarpThreads) dc_secular_kernel(DcLevel L, const EigJob* __restrict__ jobs,
                                                                  int* status) {
  const int64_t s = ((int64_t)blockIdx.x * kWarpThreads + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= L.nslots) return;
  const int mi = find_merge(L, s);
  const DcMerge M = L.merges[mi];
  const int j = (int)(s - M.x_off);
  const int K = L.K[mi];
  if (j >= K) return;
  const double* __restrict__ dd = L.dk + M.x_off;
  const double* __restrict__ z = L.zk + M.x_off;
  const double rho = L.rho[mi], rr = 1.0 / rho;
  double tau;
  int org;
  bool conv = true;
  if (K == 1) {
    tau = rho * z[0] * z[0];
    org = 0;
  } else {
    double lo, hi;
    if (j < K - 1) {
      const double del = dd[j + 1] - dd[j];
      double f = 0.0;
      for (int i = lane; i < K; i += 32) f += z[i] * z[i] / ((dd[i] - dd[j]) - 0.5 * del);
      f = warp_sum(f) + rr;
      if (f >= 0.0) {  // the root lies in the left half
        org = j;
        lo = 0.0;
        hi = 0.5 * del;
      } else {
        org = j + 1;
        lo = -0.5 * del;
        hi = 0.0;
      }
      tau = org == j ? 0.5 * del : -0.5 * del;
      if (f == 0.0) {
        L.tau[s] = tau;  // the midpoint itself
        L.org[s] = org;
        return;
      }
    } else {
      org = K - 1;
      lo = 0.0;
      hi = rho;
      tau = 0.5 * rho;
    }
    const double d0 = dd[org];
    conv = false;
    for (int it = 0; it < kSecularIters; ++it) {
      double p1 = 0.0, q1 = 0.0, p2 = 0.0, q2 = 0.0;
      for (int i = lane; i < K; i += 32) {
        const double t = z[i] / ((dd[i] - d0) - tau);
        if (i <= j) {
          p1 += z[i] * t;
          q1 += t * t;
        } else {
          p2 += z[i] * t;
          q2 += t * t;
        }
      }
      p1 = warp_sum(p1);
      q1 = warp_sum(q1);
      p2 = warp_sum(p2);
      q2 = warp_sum(q2);
      const double f = rr + p1 + p2;
      if (f == 0.0) {
        conv = true;
        break;
      }
      if (f > 0.0) hi = tau;
      else lo = tau;
      const double err = 8.0 * kEps * (rr + fabs(p1) + fabs(p2)) + kEps * fabs(tau) * (q1 + q2);
      if (fabs(f) <= err) {
        conv = true;
        break;
      }
      const double dj = (dd[j] - d0) - tau;  // < 0
      double eta;
      if (j < K - 1) {
        const double dj1 = (dd[j + 1] - d0) - tau;  // > 0
        const double b1 = q1 * dj * dj, b2 = q2 * dj1 * dj1;
        const double c0 = rr + (p1 - q1 * dj) + (p2 - q2 * dj1);
        // c0 (dj - eta)(dj1 - eta) + b1 (dj1 - eta) + b2 (dj - eta) = 0
        const double qa = c0, qb = -(c0 * (dj + dj1) + b1 + b2), qc = c0 * dj * dj1 + b1 * dj1 + b2 * dj;
        if (qa == 0.0) {
          eta = -qc / qb;
        } else {
          const double disc = fmax(qb * qb - 4.0 * qa * qc, 0.0);
          const double qq = -0.5 * (qb + copysign(sqrt(disc), qb));
          const double r1 = qq / qa, r2 = qq != 0.0 ? qc / qq : r1;
          eta = (r1 > dj && r1 < dj1) ? r1 : r2;
        }
      } else {
        const double b1 = q1 * dj * dj;
        const double c0 = rr + (p1 - q1 * dj);
        eta = c0 > 0.0 ? dj + b1 / c0 : hi - tau;
      }
      double nt = tau + eta;
      if (!(nt > lo && nt < hi)) nt = 0.5 * (lo + hi);
      if (nt == tau) {
        conv = true;
        break;
      }
      tau = nt;
    }
  }
  if (lane == 0) {
    L.tau[s] = tau;
    L.org[s] = org;
    if (!conv) status[M.job] = -2;
  }
}

// One warp per pole i: zhat_i^2 = prod_j (lambda_j - d_i) / prod_{j != i}
// (d_j - d_i) (the weights for which the computed roots are exact), as a
// product of ratios.
__global__ void __launch_bounds__(kWarpThreads) dc_zhat_kernel(DcLevel L) {
  const int64_t s = ((int64_t)blockIdx.x * kWarpThreads + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= L.nslots) return;
  const int mi = find_merge(L, s);
  const DcMerge M = L.merges[mi];
  const int i = (int)(s - M.x_off);
  const int K = L.K[mi];
  if (i >= K) return;
  const int64_t x = M.x_off;
  const double* __restrict__ dd = L.dk + x;
  const double di = dd[i];
  double prod = 1.0;
  for (int j = lane; j < K; j += 32) {
    const double num = (dd[L.org[x + j]] - di) + L.tau[x + j];
    prod *= j == i ? num : num / (dd[j] - di);
  }
  prod = warp_prod(prod);
  if (lane == 0) L.zhat[s] = copysign(sqrt(fmax(prod, 0.0)), L.zk[s]);
}

// One warp per root j: column j of U, zhat_i / (d_i - lambda_j) normalised,
// and lambda_j as the eigenvalue of the block's column j.
__global__ void __launch_bounds__(kWarpThreads) dc_vectors_kernel(double* work, const EigJob* __restrict__ jobs,
                                                                  DcLevel L) {
  const int64_t s = ((int64_t)blockIdx.x * kWarpThreads + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= L.nslots) return;
  const int mi = find_merge(L, s);
  const DcMerge M = L.merges[mi];
  const int j = (int)(s - M.x_off);
  const int K = L.K[mi];
  if (j >= K) return;
  const int64_t x = M.x_off;
  const double* __restrict__ dd = L.dk + x;
  const double* __restrict__ zh = L.zhat + x;
  const double d0 = dd[L.org[s]], tj = L.tau[s];
  double acc = 0.0;
  for (int i = lane; i < K; i += 32) {
    const double v = zh[i] / ((dd[i] - d0) - tj);
    acc += v * v;
  }
  const double inv = 1.0 / sqrt(warp_sum(acc));
  double* __restrict__ u = L.U + M.u_off + (int64_t)j * K;
  for (int i = lane; i < K; i += 32) u[i] = inv * (zh[i] / ((dd[i] - d0) - tj));
  if (lane == 0) eig_of(work, jobs[M.job])[M.o + j] = d0 + tj;
}

// One CTA per block column k: G[:, k] = the block column of slot k (poles
// first, then the deflated ones).
__global__ void __launch_bounds__(kColThreads) dc_gather_kernel(double* work, const EigJob* __restrict__ jobs,
                                                                DcLevel L) {
  const int64_t s = blockIdx.x;
  const int mi = find_merge(L, s);
  const DcMerge M = L.merges[mi];
  const EigJob J = jobs[M.job];
  const int k = (int)(s - M.x_off), nm = M.nm, n = J.n;
  const double* __restrict__ src = work + J.q_off + (int64_t)(M.o + L.col[s]) * n + M.o;
  double* __restrict__ dst = L.G + M.g_off + (int64_t)k * nm;
  for (int r = threadIdx.x; r < nm; r += kColThreads) dst[r] = src[r];
}

// One CTA per deflated slot: its column back into the block and its
// eigenvalue.
__global__ void __launch_bounds__(kColThreads) dc_finish_kernel(double* work, const EigJob* __restrict__ jobs,
                                                                DcLevel L) {
  const int64_t s = blockIdx.x;
  const int mi = find_merge(L, s);
  const DcMerge M = L.merges[mi];
  const int k = (int)(s - M.x_off);
  if (k < L.K[mi]) return;
  const EigJob J = jobs[M.job];
  const int nm = M.nm, n = J.n;
  const double* __restrict__ src = L.G + M.g_off + (int64_t)k * nm;
  double* __restrict__ dst = work + J.q_off + (int64_t)(M.o + k) * n + M.o;
  for (int r = threadIdx.x; r < nm; r += kColThreads) dst[r] = src[r];
  if (threadIdx.x == 0) eig_of(work, J)[M.o + k] = L.dk[s];
}

inline int warp_grid(int64_t nslots) { return (int)((nslots * 32 + kWarpThreads - 1) / kWarpThreads); }

}  // namespace

cudaError_t launch_dc_tear(double* work, const EigJob* jobs, const DcMerge* merges, int nmerges, cudaStream_t s) {
  if (nmerges <= 0) return cudaSuccess;
  dc_tear_kernel<<<(nmerges + 127) / 128, 128, 0, s>>>(work, jobs, merges, nmerges);
  return cudaGetLastError();
}

cudaError_t launch_dc_leaves(double* work, const EigJob* jobs, const DcLeaf* leaves, int nleaves, int* status,
                             cudaStream_t s) {
  if (nleaves <= 0) return cudaSuccess;
  dc_leaf_kernel<<<(nleaves + kLeafWarps - 1) / kLeafWarps, 32 * kLeafWarps, 0, s>>>(work, jobs, leaves, nleaves,
                                                                                    status);
  return cudaGetLastError();
}

cudaError_t launch_dc_deflate(double* work, const EigJob* jobs, const DcLevel& L, int max_nm, cudaStream_t s) {
  if (L.nmerges <= 0) return cudaSuccess;
  if (max_nm < 2 || max_nm > kEigMaxN) return cudaErrorInvalidValue;
  int P = 1;
  while (P < max_nm) P <<= 1;
  const size_t smem = (size_t)P * (2 * sizeof(double) + sizeof(int));
  cudaError_t e = cudaFuncSetAttribute(dc_deflate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dc_deflate_kernel<<<L.nmerges, kDefThreads, smem, s>>>(work, jobs, L);
  return cudaGetLastError();
}

cudaError_t launch_dc_roots(double* work, const EigJob* jobs, const DcLevel& L, int* status, cudaStream_t s) {
  if (L.nslots <= 0) return cudaSuccess;
  const int g = warp_grid(L.nslots);
  dc_secular_kernel<<<g, kWarpThreads, 0, s>>>(L, jobs, status);
  dc_zhat_kernel<<<g, kWarpThreads, 0, s>>>(L);
  dc_vectors_kernel<<<g, kWarpThreads, 0, s>>>(work, jobs, L);
  dc_gather_kernel<<<(unsigned)L.nslots, kColThreads, 0, s>>>(work, jobs, L);
  return cudaGetLastError();
}

cudaError_t launch_dc_finish(double* work, const EigJob* jobs, const DcLevel& L, cudaStream_t s) {
  if (L.nslots <= 0) return cudaSuccess;
  dc_finish_kernel<<<(unsigned)L.nslots, kColThreads, 0, s>>>(work, jobs, L);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bgpu
