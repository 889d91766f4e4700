// TEST INFRASTRUCTURE ONLY: CPU oracle of the sweep hot path (see cpu_engine.h).
#include "cpu_engine.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "../block_gb300/csrc/host/dense.h"
#include "../block_gb300/csrc/host/noise_rng.h"
#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

// ------------------------------------------------------------------ dgemm
// Optional Fortran DGEMM of a tuned BLAS (set by oracle_use_blas after a
// self-check); the reference links one the same way (CMakeLists.txt:31-47).
FortranDgemm g_blas_dgemm = nullptr;

// Row-major DGEMM used where the reference calls MatrixMultiply -> DGEMM
// (MatrixBLAS.C:438-498): through the tuned BLAS when one is set (row-major
// C = op(A) op(B) is column-major C^T = op(B)^T op(A)^T, as MatrixMultiply
// maps it, MatrixBLAS.C:456-483), else operands are packed to row-major
// non-transposed panels and an i-k-j loop with a 64-column tile keeps B rows
// in cache.
void dgemm(bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb,
           double beta, double* C, int ldc) {
  if (m <= 0 || n <= 0) return;
  if (g_blas_dgemm && k > 0) {
    const char tra = tb ? 'T' : 'N', trb = ta ? 'T' : 'N';
    g_blas_dgemm(&tra, &trb, &n, &m, &k, &alpha, B, &ldb, A, &lda, &beta, C, &ldc);
    return;
  }
  dgemm_loop(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

void dgemm_loop(bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda, const double* B,
                int ldb, double beta, double* C, int ldc) {
  if (m <= 0 || n <= 0) return;
  if (beta != 1.0)
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < n; ++j) C[(size_t)i * ldc + j] = (beta == 0.0) ? 0.0 : beta * C[(size_t)i * ldc + j];
  if (k <= 0 || alpha == 0.0) return;
  std::vector<double> Ap, Bp;
  const double* a = A;
  int la = lda;
  if (ta) {
    Ap.resize((size_t)m * k);
    for (int p = 0; p < k; ++p)
      for (int i = 0; i < m; ++i) Ap[(size_t)i * k + p] = A[(size_t)p * lda + i];
    a = Ap.data();
    la = k;
  }
  const double* b = B;
  int lb = ldb;
  if (tb) {
    Bp.resize((size_t)k * n);
    for (int j = 0; j < n; ++j)
      for (int p = 0; p < k; ++p) Bp[(size_t)p * n + j] = B[(size_t)j * ldb + p];
    b = Bp.data();
    lb = n;
  }
  const int JT = 256, KT = 128;
  for (int j0 = 0; j0 < n; j0 += JT) {
    const int j1 = std::min(n, j0 + JT);
    for (int p0 = 0; p0 < k; p0 += KT) {
      const int p1 = std::min(k, p0 + KT);
      for (int i = 0; i < m; ++i) {
        double* c = C + (size_t)i * ldc;
        const double* ai = a + (size_t)i * la;
        for (int p = p0; p < p1; ++p) {
          const double s = alpha * ai[p];
          if (s == 0.0) continue;
          const double* bp = b + (size_t)p * lb;
          for (int j = j0; j < j1; ++j) c[j] += s * bp[j];
        }
      }
    }
  }
}

// ------------------------------------------------------------- helpers

namespace {

// A reduced block of an operand: element (r, c) = scale * (trans ? p[c*ld + r] : p[r*ld + c]).
struct View {
  const double* p = nullptr;  // nullptr for the identity
  int rows = 0, cols = 0, ld = 0;
  bool trans = false;
  double scale = 1.0;
  double at(int r, int c) const {
    if (!p) return r == c ? 1.0 : 0.0;
    return scale * (trans ? p[(size_t)c * ld + r] : p[(size_t)r * ld + c]);
  }
};

bool view(const Block& B, const double* arena, const Operand& o, int bra, int ket, View& v) {
  if (o.identity) {
    if (bra != ket) return false;
    v.p = nullptr;
    v.rows = v.cols = B.si.states[bra];
    v.scale = 1.0;
    return true;
  }
  const OpEntry& e = B.ops.at(o.key);
  const OpLayout& L = B.ops.layouts[e.layout];
  if (!o.trans) {
    const int i = L.find(bra, ket);
    if (i < 0) return false;
    const OpBlock& b = L.blocks[i];
    v.p = arena + e.base + b.offset;
    v.rows = b.rows;
    v.cols = b.cols;
    v.ld = b.cols;
    v.trans = false;
    v.scale = 1.0;
  } else {
    const int i = L.find(ket, bra);
    if (i < 0) return false;
    const OpBlock& b = L.blocks[i];
    v.p = arena + e.base + b.offset;
    v.rows = b.cols;
    v.cols = b.rows;
    v.ld = b.cols;
    v.trans = true;
    v.scale = transpose_scaling(B.si.quanta[bra].s2, B.si.quanta[ket].s2, o.key.k2);
  }
  return true;
}

int rank2(const Operand& o) { return o.identity ? 0 : o.key.k2; }
bool fermion(const Operand& o) { return !o.identity && op_fermion(o.key); }

}  // namespace

// ------------------------------------------------------------- engine

CpuEngine::CpuEngine(int t) {
#ifdef _OPENMP
  threads = t > 0 ? t : omp_get_max_threads();
#else
  threads = 1;
  (void)t;
#endif
}

void CpuEngine::create_block(Block& b) {
  b.handle = next_handle_++;
  if (structure_only && !b.is_dot) store_[b.handle].clear();
  else store_[b.handle].assign(b.ops.arena, 0.0);
}

void CpuEngine::fill_random(Block& b, uint64_t seed) {
  std::vector<double>& a = store_.at(b.handle);
  a.resize(b.ops.arena);
  Rng rng(seed);
  for (auto& x : a) x = 0.1 * rng.normal();
}

void CpuEngine::release_block(Block& b) {
  store_.erase(b.handle);
  block_rot_.erase(b.handle);
  b.handle = -1;
}

void CpuEngine::upload_block(Block& b, const std::vector<double>& a) {
  if ((int64_t)a.size() != b.ops.arena) throw std::runtime_error("upload size mismatch");
  if (structure_only && !b.is_dot) return;
  store_.at(b.handle) = a;
}

void CpuEngine::download_block(const Block& b, std::vector<double>& a) { a = store_.at(b.handle); }

// TensorProduct of two sub-block operators into an operator of the block
// made of both (operatorfunctions.C:146-254; MatrixTensorProduct,
// MatrixBLAS.C:125-291).  Reduced factor: scale * 9j * transpose scalings *
// fermion sign of the right operator passing the left ket.
static void tensor_product(const Block& big, const OpKey& tk, double* T, const Block& A, const double* Aar,
                           const Operand& oa, const Block& B, const double* Bar, const Operand& ob, double coef) {
  const OpLayout& TL = big.ops.layout_of(tk);
  const int kA = rank2(oa), kB = rank2(ob), kC = tk.k2;
  const bool fB = fermion(ob);
  for (const OpBlock& tb : TL.blocks) {
    const int cq = tb.bra, cqp = tb.ket;
    const Quantum& Q = big.si.quanta[cq];
    const Quantum& Qp = big.si.quanta[cqp];
    double* Tblk = T + TL.blocks[TL.find(cq, cqp)].offset;
    const int ldT = tb.cols;
    for (const SectorPart& pr : big.si.parts[cq])
      for (const SectorPart& pc : big.si.parts[cqp]) {
        View va, vb;
        if (!view(A, Aar, oa, pr.lq, pc.lq, va)) continue;
        if (!view(B, Bar, ob, pr.rq, pc.rq, vb)) continue;
        double f = coef * ninej(A.si.quanta[pc.lq].s2, B.si.quanta[pc.rq].s2, Qp.s2, kA, kB, kC,
                                A.si.quanta[pr.lq].s2, B.si.quanta[pr.rq].s2, Q.s2);
        if (fB && is_fermion(A.si.quanta[pc.lq])) f = -f;
        if (f == 0.0) continue;
        const int br = vb.rows, bc = vb.cols;
        for (int ia = 0; ia < va.rows; ++ia)
          for (int ja = 0; ja < va.cols; ++ja) {
            const double fa = f * va.at(ia, ja);
            if (fa == 0.0) continue;
            for (int ib = 0; ib < br; ++ib) {
              double* trow = Tblk + (size_t)(pr.offset + ia * br + ib) * ldT + pc.offset + ja * bc;
              for (int jb = 0; jb < bc; ++jb) trow[jb] += fa * vb.at(ib, jb);
            }
          }
      }
  }
}

void CpuEngine::build_block(Block& big, const Block& a, const Block& b,
                            const std::vector<std::pair<OpKey, std::vector<BuildTerm>>>& recipes) {
  if (structure_only) return;
  std::vector<double>& T = store_.at(big.handle);
  std::fill(T.begin(), T.end(), 0.0);
  const double* Aar = store_.at(a.handle).data();
  const double* Bar = store_.at(b.handle).data();
#pragma omp parallel for schedule(dynamic) num_threads(threads)
  for (int r = 0; r < (int)recipes.size(); ++r) {
    const OpKey& tk = recipes[r].first;
    double* Tp = T.data() + big.ops.at(tk).base;
    for (const BuildTerm& t : recipes[r].second) tensor_product(big, tk, Tp, a, Aar, t.a, b, Bar, t.b, t.coef);
  }
}

// sigma = H psi by operator pairs: TensorMultiply (operatorfunctions.C:485-537)
// over the pair list of SpinBlock::multiplyH (spinblock.C:722-789), with
// per-thread sigma copies reduced at the end (distribute.h:128-224).
void CpuEngine::sigma(const Superblock& sb, const double* psi, double* out) {
  auto t0 = std::chrono::steady_clock::now();
  const Block& L = *sb.L;
  const Block& R = *sb.R;
  const double* Lar = store_.at(L.handle).data();
  const double* Rar = store_.at(R.handle).data();
  const int nL = L.si.size(), nR = R.si.size();
  std::vector<int> sec((size_t)nL * nR, -1);
  for (int s = 0; s < (int)sb.sectors.size(); ++s) sec[(size_t)sb.sectors[s].lq * nR + sb.sectors[s].rq] = s;
  const int J = sb.target.s2;
  const int nth = threads;
  std::vector<std::vector<double>> part(nth, std::vector<double>(sb.size, 0.0));
  std::vector<double> fl(nth, 0.0);
#pragma omp parallel num_threads(nth)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double* V = part[tid].data();
    std::vector<double> m, bufA, bufB;
#pragma omp for schedule(dynamic)
    for (int ti = 0; ti < (int)sb.terms.size(); ++ti) {
      const PairTerm& t = sb.terms[ti];
      const int kL = rank2(t.l), kR = rank2(t.r);
      const bool fR = fermion(t.r);
      for (int lQ = 0; lQ < nL; ++lQ)
        for (int rQp = 0; rQp < nR; ++rQp)
          for (int lQp = 0; lQp < nL; ++lQp) {
            const int cs = sec[(size_t)lQp * nR + rQp];
            if (cs < 0) continue;
            View va;
            if (!view(L, Lar, t.l, lQ, lQp, va)) continue;
            const auto& S = sb.sectors[cs];
            const int mr = L.si.states[lQ], mc = R.si.states[rQp];
            // m = A(lQ,lQ') C(lQ',rQ')
            m.assign((size_t)mr * mc, 0.0);
            if (!va.p) {
              std::memcpy(m.data(), psi + S.offset, sizeof(double) * mr * mc);
            } else {
              dgemm(va.trans, false, mr, mc, S.rows, va.scale, va.p, va.ld, psi + S.offset, S.cols, 0.0, m.data(), mc);
              fl[tid] += 2.0 * mr * mc * S.rows;
            }
            for (int rQ = 0; rQ < nR; ++rQ) {
              const int vs = sec[(size_t)lQ * nR + rQ];
              if (vs < 0) continue;
              View vb;
              if (!view(R, Rar, t.r, rQ, rQp, vb)) continue;
              double f = t.coef * ninej(L.si.quanta[lQp].s2, R.si.quanta[rQp].s2, J, kL, kR, 0, L.si.quanta[lQ].s2,
                                        R.si.quanta[rQ].s2, J);
              if (fR && is_fermion(L.si.quanta[lQp])) f = -f;
              if (f == 0.0) continue;
              const auto& SV = sb.sectors[vs];
              if (!vb.p) {
                double* v = V + SV.offset;
                for (size_t e = 0; e < m.size(); ++e) v[e] += f * m[e];
              } else {
                // V += f * m * B(rQ,rQ')^T
                dgemm(false, !vb.trans, mr, SV.cols, mc, f * vb.scale, m.data(), mc, vb.p, vb.ld, 1.0, V + SV.offset,
                      SV.cols);
                fl[tid] += 2.0 * mr * SV.cols * mc;
              }
            }
          }
    }
  }
  last_sigma_flops = 0.0;
  for (int t = 0; t < nth; ++t) last_sigma_flops += fl[t];
  std::fill(out, out + sb.size, 0.0);
  for (int t = 0; t < nth; ++t)
    for (int64_t i = 0; i < sb.size; ++i) out[i] += part[t][i];
  if (sb.ecore != 0.0)
    for (int64_t i = 0; i < sb.size; ++i) out[i] += sb.ecore * psi[i];
  sigma_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  ++sigma_calls;
}

// Diagonal of H (SpinBlock::diagonalH, spinblock.C:855-899; diagonal
// TensorTrace / TensorProduct, operatorfunctions.C:653-762).
void CpuEngine::hdiag(const Superblock& sb, double* d) {
  const Block& L = *sb.L;
  const Block& R = *sb.R;
  const double* Lar = store_.at(L.handle).data();
  const double* Rar = store_.at(R.handle).data();
  const int J = sb.target.s2;
  std::fill(d, d + sb.size, sb.ecore);
  for (const PairTerm& t : sb.terms) {
    const int kL = rank2(t.l), kR = rank2(t.r);
    const bool fR = fermion(t.r);
    for (const auto& S : sb.sectors) {
      View va, vb;
      if (!view(L, Lar, t.l, S.lq, S.lq, va)) continue;
      if (!view(R, Rar, t.r, S.rq, S.rq, vb)) continue;
      double f = t.coef * ninej(L.si.quanta[S.lq].s2, R.si.quanta[S.rq].s2, J, kL, kR, 0, L.si.quanta[S.lq].s2,
                                R.si.quanta[S.rq].s2, J);
      if (fR && is_fermion(L.si.quanta[S.lq])) f = -f;
      if (f == 0.0) continue;
      for (int i = 0; i < S.rows; ++i) {
        const double a = f * va.at(i, i);
        if (a == 0.0) continue;
        for (int j = 0; j < S.cols; ++j) d[S.offset + (int64_t)i * S.cols + j] += a * vb.at(j, j);
      }
    }
  }
}

static double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}
static void axpy(double s, const std::vector<double>& x, std::vector<double>& y) {
  for (size_t i = 0; i < x.size(); ++i) y[i] += s * x[i];
}
static void scal(double s, std::vector<double>& x) {
  for (auto& v : x) v *= s;
}

// Davidson preconditioner r_i /= (e - diag_i) (Linear::precondition, linear.C:27-47)
static void precondition(std::vector<double>& r, double e, const std::vector<double>& d) {
  for (size_t i = 0; i < r.size(); ++i)
    if (std::fabs(e - d[i]) > 1e-12) r[i] /= (e - d[i]);
}

// Block Davidson (Linear::block_davidson, linear.C:179-385) with the Olsen
// correction (linear.C:50-60), deflation and the squared-residual test.
int CpuEngine::solve(const Superblock& sb, const DavidsonParams& p, std::vector<double>& energies) {
  const int64_t n = sb.size;
  std::vector<double> diag(n);
  hdiag(sb, diag.data());
  const int nroots = p.nroots;
  if (n < nroots) throw std::runtime_error("superblock smaller than number of roots");
  // basic guess: unit vectors on the lowest diagonal elements, slightly perturbed
  std::vector<int64_t> order(n);
  for (int64_t i = 0; i < n; ++i) order[i] = i;
  std::partial_sort(order.begin(), order.begin() + nroots, order.end(),
                    [&](int64_t a, int64_t b) { return diag[a] < diag[b]; });
  Rng rng(p.seed);
  std::vector<std::vector<double>> b(nroots, std::vector<double>(n, 0.0)), sigma;
  if (p.use_guess && (int)guess_.size() >= nroots && (int64_t)guess_[0].size() == n) {
    // transformed previous wavefunctions (orthonormalised below)
    for (int r = 0; r < nroots; ++r) b[r] = guess_[r];
  } else {
    for (int r = 0; r < nroots; ++r) {
      for (int64_t i = 0; i < n; ++i) b[r][i] = 1e-3 * (rng.uniform() - 0.5);
      b[r][order[r]] = 1.0;
    }
  }
  for (int i = 0; i < nroots; ++i) {
    for (int j = 0; j < i; ++j) axpy(-dot(b[j], b[i]), b[j], b[i]);
    scal(1.0 / std::sqrt(dot(b[i], b[i])), b[i]);
  }
  int converged = 0, iter = 0;
  std::vector<double> lam;
  while (true) {
    ++iter;
    for (size_t i = sigma.size(); i < b.size(); ++i) {
      sigma.emplace_back(n);
      this->sigma(sb, b[i].data(), sigma.back().data());
    }
    const int k = (int)b.size();
    std::vector<double> h((size_t)k * k), alpha((size_t)k * k);
    lam.assign(k, 0.0);
    for (int i = 0; i < k; ++i)
      for (int j = 0; j <= i; ++j) h[(size_t)i * k + j] = h[(size_t)j * k + i] = dot(b[i], sigma[j]);
    jacobi_eigh(k, h.data(), lam.data(), alpha.data());
    {
      std::vector<std::vector<double>> bt = b, st = sigma;
      for (int j = 0; j < k; ++j) {
        std::fill(b[j].begin(), b[j].end(), 0.0);
        std::fill(sigma[j].begin(), sigma[j].end(), 0.0);
        for (int i = 0; i < k; ++i) {
          axpy(alpha[(size_t)i * k + j], bt[i], b[j]);
          axpy(alpha[(size_t)i * k + j], st[i], sigma[j]);
        }
      }
    }
    std::vector<double> r;
    for (int i = 0; i < converged; ++i) {
      r = sigma[i];
      axpy(-lam[i], b[i], r);
      if (dot(r, r) > p.tol) {
        converged = i;
        break;
      }
    }
    r = sigma[converged];
    axpy(-lam[converged], b[converged], r);
    const double rnorm = dot(r, r);
    {  // Olsen preconditioning
      std::vector<double> c0 = b[converged];
      precondition(c0, lam[converged], diag);
      const double num = dot(c0, r), den = dot(b[converged], c0);
      axpy(-num / den, b[converged], r);
      precondition(r, lam[converged], diag);
    }
    if (rnorm < p.tol) {
      ++converged;
      if (converged == nroots) break;
    } else {
      if ((int)b.size() >= p.deflation_max) {
        b.resize(p.deflation_min);
        sigma.resize(p.deflation_min);
      }
      for (size_t j = 0; j < b.size(); ++j) {
        scal(1.0 / std::sqrt(dot(r, r)), r);
        axpy(-dot(r, b[j]), b[j], r);
      }
      // a correction that lies almost inside the subspace (few states left
      // outside it, e.g. many roots of a small superblock) loses its
      // orthogonality in the pass above: a second pass restores it (twice
      // is enough, Kahan); the reference's single pass is kept otherwise
      if (dot(r, r) < 1e-2)
        for (size_t j = 0; j < b.size(); ++j) axpy(-dot(r, b[j]), b[j], r);
      scal(1.0 / std::sqrt(dot(r, r)), r);
      b.push_back(r);
    }
    if (iter >= p.max_iter) break;
  }
  energies.assign(lam.begin(), lam.begin() + nroots);
  waves_.assign(b.begin(), b.begin() + nroots);
  return iter;
}

// Reduced density matrix sum_r w_r psi_r psi_r^T of the block being
// renormalised (DensityMatrix::makedensitymatrix, density.C:27-90;
// MultiplyProduct, operatorfunctions.C:630-650) and its per-sector
// eigen-decomposition (diagonalise_dm, rotationmat.C:258-279).
void CpuEngine::density(const Superblock& sb, bool left, const std::vector<double>& weights, DensitySpectrum& spec) {
  const Block& B = left ? *sb.L : *sb.R;
  const int nq = B.si.size();
  std::vector<std::vector<double>> rho(nq);
  for (int q = 0; q < nq; ++q) rho[q].assign((size_t)B.si.states[q] * B.si.states[q], 0.0);
  for (size_t r = 0; r < waves_.size(); ++r) {
    const double w = r < weights.size() ? weights[r] : 1.0 / waves_.size();
    for (const auto& S : sb.sectors) {
      const double* psi = waves_[r].data() + S.offset;
      if (left)
        dgemm(false, true, S.rows, S.rows, S.cols, w, psi, S.cols, psi, S.cols, 1.0, rho[S.lq].data(), S.rows);
      else
        dgemm(true, false, S.cols, S.cols, S.rows, w, psi, S.cols, psi, S.cols, 1.0, rho[S.rq].data(), S.cols);
    }
  }
  if (noise_.any()) add_noise(sb, left, rho);
  dm_rho_ = rho;  // kept for the element-wise parity tests
  spec.eig.assign(nq, {});
  dm_vecs_.assign(nq, {});
  dm_dims_.assign(nq, 0);
  for (int q = 0; q < nq; ++q) {
    const int d = B.si.states[q];
    dm_dims_[q] = d;
    spec.eig[q].resize(d);
    dm_vecs_[q].resize((size_t)d * d);
    jacobi_eigh(d, rho[q].data(), spec.eig[q].data(), dm_vecs_[q].data());
    // every eigenvector's largest component (the first of equal ones)
    // positive, as on the GPU: the renormalised basis, and so the random
    // noise of later steps, depends on the signs
    double* v = dm_vecs_[q].data();
    for (int j = 0; j < d; ++j) {
      int bi = 0;
      for (int i = 1; i < d; ++i)
        if (std::fabs(v[(size_t)i * d + j]) > std::fabs(v[(size_t)bi * d + j])) bi = i;
      if (v[(size_t)bi * d + j] < 0.0)
        for (int i = 0; i < d; ++i) v[(size_t)i * d + j] = -v[(size_t)i * d + j];
    }
  }
}

// phi = (O x 1) psi (left) or (1 x O) psi (right) onto total quantum q, in
// the sectors `out` of L x R (single-operator TensorMultiply,
// operatorfunctions.C:331-404, in the conventions of sigma's couplings).
void CpuEngine::apply_one(const Superblock& sb, bool left, const Operand& o, const std::vector<double>& psi,
                          const std::vector<Superblock::Sector>& out, int s2_out, std::vector<double>& phi) {
  const Block& L = *sb.L;
  const Block& R = *sb.R;
  const Block& B = left ? L : R;
  const std::vector<double>& ar = store_.at(B.handle);
  const int k = o.key.k2, J = sb.target.s2;
  std::vector<int> index((size_t)L.si.size() * R.si.size(), -1);
  for (int s = 0; s < (int)sb.sectors.size(); ++s) index[(size_t)sb.sectors[s].lq * R.si.size() + sb.sectors[s].rq] = s;
  std::fill(phi.begin(), phi.end(), 0.0);
  for (const auto& S : out) {
    double* dst = phi.data() + S.offset;
    if (left) {
      for (int lqp = 0; lqp < L.si.size(); ++lqp) {
        const int s = index[(size_t)lqp * R.si.size() + S.rq];
        if (s < 0) continue;
        View v;
        if (!view(L, ar.data(), o, S.lq, lqp, v)) continue;
        const double f = ninej(L.si.quanta[lqp].s2, R.si.quanta[S.rq].s2, J, k, 0, k, L.si.quanta[S.lq].s2,
                               R.si.quanta[S.rq].s2, s2_out) * v.scale;
        if (f == 0.0) continue;
        const auto& P = sb.sectors[s];
        dgemm(v.trans, false, S.rows, S.cols, P.rows, f, v.p, v.ld, psi.data() + P.offset, P.cols, 1.0, dst, S.cols);
      }
    } else {
      for (int rqp = 0; rqp < R.si.size(); ++rqp) {
        const int s = index[(size_t)S.lq * R.si.size() + rqp];
        if (s < 0) continue;
        View v;
        if (!view(R, ar.data(), o, S.rq, rqp, v)) continue;
        double f = ninej(L.si.quanta[S.lq].s2, R.si.quanta[rqp].s2, J, 0, k, k, L.si.quanta[S.lq].s2,
                         R.si.quanta[S.rq].s2, s2_out) * v.scale;
        if (op_fermion(o.key) && is_fermion(L.si.quanta[S.lq])) f = -f;
        if (f == 0.0) continue;
        const auto& P = sb.sectors[s];
        // psi(lq, rq') O(rq, rq')^T
        dgemm(false, !v.trans, S.rows, S.cols, P.cols, f, psi.data() + P.offset, P.cols, v.p, v.ld, 1.0, dst, S.cols);
      }
    }
  }
}

// rho(b) += alpha * phi phi^T restricted to the sectors of the block (left:
// rows, right: columns)
static void add_outer(bool left, const std::vector<Superblock::Sector>& sec, const double* phi, double alpha,
                      std::vector<std::vector<double>>& rho) {
  for (const auto& S : sec) {
    const double* p = phi + S.offset;
    if (left)
      dgemm(false, true, S.rows, S.rows, S.cols, alpha, p, S.cols, p, S.cols, 1.0, rho[S.lq].data(), S.rows);
    else
      dgemm(true, false, S.cols, S.cols, S.rows, alpha, p, S.cols, p, S.cols, 1.0, rho[S.rq].data(), S.cols);
  }
}

// Noise of the density matrix (add_onedot_noise, density.C:330-421;
// add_twodot_noise, density.C:92-165); see NoiseSpec.
void CpuEngine::add_noise(const Superblock& sb, bool left, std::vector<std::vector<double>>& rho) {
  const Block& B = left ? *sb.L : *sb.R;
  const int nq = B.si.size();
  const int nroots = (int)waves_.size();
  const PointGroup& g = noise_.group;
  if (noise_.perturbative > 0.0) {
    const std::vector<NoiseOp> ops = perturbative_noise_ops(B, sb.target, noise_.orbsym, g);
    for (int r = 0; r < nroots; ++r) {
      std::vector<std::vector<double>> nm(nq);
      for (int q = 0; q < nq; ++q) nm[q].assign((size_t)B.si.states[q] * B.si.states[q], 0.0);
      for (const NoiseOp& no : ops) {
        int64_t size = 0;
        const auto sec = wave_sectors(sb.L->si, sb.R->si, no.q, g, size);
        if (size == 0) continue;
        std::vector<double> phi(size);
        apply_one(sb, left, op(no.key, no.trans), waves_[r], sec, no.q.s2, phi);
        double nrm = 0.0;
        for (double x : phi) nrm += x * x;
        if (std::fabs(nrm) > 1e-15) add_outer(left, sec, phi.data(), 1.0 / nrm, nm);
      }
      double tr = 0.0;
      for (int q = 0; q < nq; ++q)
        for (int i = 0; i < B.si.states[q]; ++i) tr += nm[q][(size_t)i * B.si.states[q] + i];
      if (tr > 1.0) {
        const double a = noise_.perturbative / nroots / tr;
        for (int q = 0; q < nq; ++q)
          for (size_t e = 0; e < nm[q].size(); ++e) rho[q][e] += a * nm[q][e];
      }
    }
  }
  if (noise_.random > 0.0) {
    const std::vector<Quantum> qs = random_noise_quanta(sb.target);
    for (int r = 0; r < nroots; ++r)
      for (int i = 0; i < (int)qs.size(); ++i) {
        int64_t size = 0;
        const auto sec = wave_sectors(sb.L->si, sb.R->si, qs[i], g, size);
        if (size == 0) continue;
        std::vector<double> phi(size);
        const uint64_t seed = noise_.seed + 0x632BE59BD9B4E019ull * (uint64_t)r;
        double nrm = 0.0;
        for (int64_t e = 0; e < size; ++e) {
          phi[e] = noise_uniform(seed, i, e);
          nrm += phi[e] * phi[e];
        }
        if (std::fabs(nrm) > 1e-15)
          add_outer(left, sec, phi.data(), noise_.random / nroots / (double)qs.size() / nrm, rho);
      }
  }
}

// <psi_r| T |psi_r> of single pair terms: the product of one term
// (TensorMultiply over its couplings) dotted with the wavefunction.
void CpuEngine::expectations(const Superblock& sb, const std::vector<PairTerm>& terms, std::vector<double>& out) {
  const size_t nt = terms.size(), nr = waves_.size();
  out.assign(nr * nr * nt, 0.0);
  std::vector<double> y(sb.size);
  for (size_t t = 0; t < nt; ++t) {
    Superblock one = sb;
    one.terms.assign(1, terms[t]);
    one.ecore = 0.0;
    for (size_t b = 0; b < nr; ++b) {
      std::fill(y.begin(), y.end(), 0.0);
      sigma(one, waves_[b].data(), y.data());
      for (size_t a = 0; a < nr; ++a) {
        double d = 0.0;
        for (int64_t e = 0; e < sb.size; ++e) d += waves_[a][e] * y[e];
        out[(a * nr + b) * nt + t] = d;
      }
    }
  }
}

void CpuEngine::select_rotation(const std::vector<std::vector<int>>& kept) {
  const int nq = (int)kept.size();
  rot_.assign(nq, {});
  rot_kept_.assign(nq, 0);
  for (int q = 0; q < nq; ++q) {
    const int d = dm_dims_[q], m = (int)kept[q].size();
    rot_kept_[q] = m;
    rot_[q].resize((size_t)d * m);
    for (int c = 0; c < m; ++c)
      for (int r = 0; r < d; ++r) rot_[q][(size_t)r * m + c] = dm_vecs_[q][(size_t)r * d + kept[q][c]];
  }
}

void CpuEngine::set_rotation(const std::vector<std::vector<double>>& rot, const std::vector<int>& kept) {
  rot_ = rot;
  rot_kept_ = kept;
}

// O'(b',k') = U_b^T O(b,k) U_k for every operator of the new block
// (SparseMatrix::renormalise_transform, BaseOperator.C:341-363;
// MatrixRotate, MatrixBLAS.C:553-572).
void CpuEngine::renormalise(Block& small, const Block& big) {
  if (structure_only) return;
  std::vector<double>& S = store_.at(small.handle);
  const std::vector<double>& Bg = store_.at(big.handle);
  std::vector<std::pair<const OpKey*, const OpEntry*>> list;
  for (const auto& kv : small.ops.ops) list.push_back({&kv.first, &kv.second});
#pragma omp parallel for schedule(dynamic) num_threads(threads)
  for (int oi = 0; oi < (int)list.size(); ++oi) {
    const OpKey& k = *list[oi].first;
    const OpEntry& se = *list[oi].second;
    const OpLayout& SL = small.ops.layouts[se.layout];
    const OpEntry& be = big.ops.at(k);
    const OpLayout& BL = big.ops.layouts[be.layout];
    std::vector<double> tmp;
    for (const OpBlock& sbk : SL.blocks) {
      const int b = big.si.find(small.si.quanta[sbk.bra]);
      const int kk = big.si.find(small.si.quanta[sbk.ket]);
      const int bi = BL.find(b, kk);
      double* dst = S.data() + se.base + sbk.offset;
      if (bi < 0) {
        std::fill(dst, dst + (size_t)sbk.rows * sbk.cols, 0.0);
        continue;
      }
      const OpBlock& bb = BL.blocks[bi];
      const double* O = Bg.data() + be.base + bb.offset;
      const int mb = rot_kept_[b], mk = rot_kept_[kk];
      // tmp = O U_k  (rows(b) x mk), dst = U_b^T tmp
      tmp.assign((size_t)bb.rows * mk, 0.0);
      dgemm(false, false, bb.rows, mk, bb.cols, 1.0, O, bb.cols, rot_[kk].data(), mk, 0.0, tmp.data(), mk);
      dgemm(true, false, mb, mk, bb.rows, 1.0, rot_[b].data(), mb, tmp.data(), mk, 0.0, dst, sbk.cols);
    }
  }
  // keep the rotation with the block (guess transform of later steps)
  Rot rec;
  const int nq = (int)rot_kept_.size();
  rec.m = rot_kept_;
  rec.n.assign(nq, 0);
  rec.small_of_big.assign(nq, -1);
  rec.u.resize(nq);
  for (int q = 0; q < nq; ++q) {
    const int m = rot_kept_[q];
    rec.n[q] = m > 0 ? (int)(rot_[q].size() / m) : (q < big.si.size() ? big.si.states[q] : 0);
    if (m > 0) {
      rec.small_of_big[q] = (int)rec.big_of_small.size();
      rec.big_of_small.push_back(q);
      rec.u[q] = rot_[q];
    }
  }
  if (nq == big.si.size() && (int)rec.big_of_small.size() == small.si.size())
    block_rot_[small.handle] = std::move(rec);
}

bool CpuEngine::get_rotation_record(const Block& b, RotationRecord& r) {
  auto it = block_rot_.find(b.handle);
  if (it == block_rot_.end()) return false;
  const Rot& x = it->second;
  r.n = x.n;
  r.m = x.m;
  r.small_of_big = x.small_of_big;
  r.big_of_small = x.big_of_small;
  r.off.assign(x.n.size(), 0);
  r.data.clear();
  for (size_t q = 0; q < x.n.size(); ++q) {
    r.off[q] = (int64_t)r.data.size();
    r.data.insert(r.data.end(), x.u[q].begin(), x.u[q].end());
  }
  if (r.data.empty()) r.data.push_back(0.0);
  return true;
}

void CpuEngine::set_rotation_record(const Block& b, const RotationRecord& r) {
  const size_t nq = r.off.size();
  if (r.n.size() != nq || r.m.size() != nq || r.small_of_big.size() != nq)
    throw std::runtime_error("rotation record: inconsistent sizes");
  Rot x;
  x.n = r.n;
  x.m = r.m;
  x.small_of_big = r.small_of_big;
  x.big_of_small = r.big_of_small;
  x.u.resize(nq);
  for (size_t q = 0; q < nq; ++q) {
    const int64_t sz = (int64_t)r.n[q] * r.m[q];
    if (r.off[q] < 0 || r.off[q] + sz > (int64_t)r.data.size())
      throw std::runtime_error("rotation record: sector outside its data");
    if (r.m[q] > 0) x.u[q].assign(r.data.begin() + r.off[q], r.data.begin() + r.off[q] + sz);
  }
  block_rot_[b.handle] = std::move(x);
}

// The previous step's vectors in the next step's superblock (GuessWave::
// transform_previous_wavefunction, guess_wavefunction.C:526-620, onto the
// spin-adapted two-site blocks).  Forward (the dot moves right): the old
// left big block is rotated to its kept states, phi = U^T psi per old
// sector; each new sector (l, r) with l = (a, d) collects, for every old
// right quantum J_R made of (d, b), the columns of phi(a, J_R) that belong
// to (d, b), times the recoupling of (a d) l with (d b) J_R,
//   W = (-1)^((j_a + j_d + j_b + J)/2) sqrt((2 j_l + 1)(2 j_R + 1))
//       {j_a j_d j_l; j_b J j_R},
// into chi (rows of l x kept states of b), and expands the right side with
// the rotation V that made b: psi'(l, r) = chi V^T.  Backward is the mirror
// image (psi V on the right, U chi on the left).
bool CpuEngine::transform_guess(const GuessInput& g, const Superblock& sb) {
  guess_.clear();
  if (waves_.empty() || !g.rotated || !g.expanded || !g.dot) return false;
  auto ri = block_rot_.find(g.rotated->handle);
  auto ei = block_rot_.find(g.expanded->handle);
  if (ri == block_rot_.end() || ei == block_rot_.end()) return false;
  const Rot& rot = ri->second;
  const Rot& exq = ei->second;
  int64_t old_n = 0;
  for (const auto& S : g.old_sectors) old_n = std::max<int64_t>(old_n, S.offset + (int64_t)S.rows * S.cols);
  if (old_n != (int64_t)waves_[0].size()) return false;
  const StateInfo& newL = sb.L->si;
  const StateInfo& newR = sb.R->si;
  const int J = sb.target.s2;
  const StateInfo& rot_big = g.forward ? g.old_L : g.old_R;
  const StateInfo& exp_big = g.forward ? newR : newL;
  if ((int)rot.n.size() != rot_big.size() || (int)exq.n.size() != exp_big.size()) return false;
  for (int q = 0; q < rot_big.size(); ++q)
    if (rot.m[q] > 0 && rot.n[q] != rot_big.states[q]) return false;
  for (int q = 0; q < exp_big.size(); ++q)
    if (exq.m[q] > 0 && exq.n[q] != exp_big.states[q]) return false;
  if (!g.forward && !(g.old_L.is_product() && newR.is_product())) return false;
  if (g.forward && !(g.old_R.is_product() && newL.is_product())) return false;
  auto W = [&](int ja, int jd, int jb, int jl, int jr) {
    const int ph = (ja + jd + jb + J) / 2;
    return ((ph & 1) ? -1.0 : 1.0) * std::sqrt((double)(jl + 1) * (jr + 1)) * six_j(ja, jd, jl, jb, J, jr);
  };
  const int nr = (int)waves_.size();
  guess_.assign(nr, std::vector<double>(sb.size, 0.0));
  for (int r = 0; r < nr; ++r) {
    const std::vector<double>& psi = waves_[r];
    std::map<std::pair<int, int>, std::pair<std::vector<double>, int>> phi;  // -> (block, its columns)
    for (const auto& S : g.old_sectors) {
      if (g.forward) {
        const int a = rot.small_of_big[S.lq];
        if (a < 0) continue;
        const int m = rot.m[S.lq];
        std::vector<double> P((size_t)m * S.cols);
        dgemm(true, false, m, S.cols, S.rows, 1.0, rot.u[S.lq].data(), m, psi.data() + S.offset, S.cols, 0.0,
              P.data(), S.cols);
        phi[{a, S.rq}] = {std::move(P), S.cols};
      } else {
        const int b = rot.small_of_big[S.rq];
        if (b < 0) continue;
        const int m = rot.m[S.rq];
        std::vector<double> P((size_t)S.rows * m);
        dgemm(false, false, S.rows, m, S.cols, 1.0, psi.data() + S.offset, S.cols, rot.u[S.rq].data(), m, 0.0,
              P.data(), m);
        phi[{S.lq, b}] = {std::move(P), m};
      }
    }
    for (const auto& S : sb.sectors) {
      double* out = guess_[r].data() + S.offset;
      if (g.forward) {
        const int b = exq.small_of_big[S.rq];  // kept quantum of the expanded right block
        if (b < 0) continue;
        const int mb = exq.m[S.rq];
        std::vector<double> chi((size_t)S.rows * mb, 0.0);
        bool any = false;
        for (const SectorPart& pt : newL.parts[S.lq]) {  // (a, d)
          const int ja = g.old_L.quanta[rot.big_of_small[pt.lq]].s2;
          const int jd = g.dot->quanta[pt.rq].s2;
          const int jb = g.expanded->si.quanta[b].s2;
          for (const auto& jp : g.old_R.parts_of(pt.rq, b)) {  // old right quantum made of (d, b)
            auto f = phi.find({pt.lq, jp.first});
            if (f == phi.end()) continue;
            const double c = W(ja, jd, jb, newL.quanta[S.lq].s2, g.old_R.quanta[jp.first].s2);
            if (c == 0.0) continue;
            const std::vector<double>& P = f->second.first;
            const int lds = f->second.second, c0 = g.old_R.parts[jp.first][jp.second].offset;
            for (int i = 0; i < pt.size; ++i)
              for (int j = 0; j < mb; ++j) chi[(size_t)(pt.offset + i) * mb + j] += c * P[(size_t)i * lds + c0 + j];
            any = true;
          }
        }
        if (any)
          dgemm(false, true, S.rows, S.cols, mb, 1.0, chi.data(), mb, exq.u[S.rq].data(), mb, 0.0, out, S.cols);
      } else {
        const int a = exq.small_of_big[S.lq];  // kept quantum of the expanded left block
        if (a < 0) continue;
        const int ma = exq.m[S.lq];
        std::vector<double> chi((size_t)ma * S.cols, 0.0);
        bool any = false;
        for (const SectorPart& pt : newR.parts[S.rq]) {  // (d, b)
          const int ja = g.expanded->si.quanta[a].s2;
          const int jd = g.dot->quanta[pt.lq].s2;
          const int jb = g.old_R.quanta[rot.big_of_small[pt.rq]].s2;
          for (const auto& jp : g.old_L.parts_of(a, pt.lq)) {  // old left quantum made of (a, d)
            auto f = phi.find({jp.first, pt.rq});
            if (f == phi.end()) continue;
            const double c = W(ja, jd, jb, g.old_L.quanta[jp.first].s2, newR.quanta[S.rq].s2);
            if (c == 0.0) continue;
            const std::vector<double>& P = f->second.first;
            const int lds = f->second.second, r0 = g.old_L.parts[jp.first][jp.second].offset;
            for (int i = 0; i < ma; ++i)
              for (int j = 0; j < pt.size; ++j)
                chi[(size_t)i * S.cols + pt.offset + j] += c * P[(size_t)(r0 + i) * lds + j];
            any = true;
          }
        }
        if (any)
          dgemm(false, false, S.rows, S.cols, ma, 1.0, exq.u[S.lq].data(), ma, chi.data(), S.cols, 0.0, out, S.cols);
      }
    }
  }
  // usable only if every root keeps a sizeable norm
  for (const auto& v : guess_) {
    double h = 0.0;
    for (double x : v) h += x * x;
    if (!std::isfinite(h) || h <= 1e-4) {
      guess_.clear();
      return false;
    }
  }
  return true;
}

}  // namespace oracle
