/*
 * C ABI of the GB300 sweep hot path of spin-adapted two-site DMRG.
 *
 * Everything is plain pointers and sizes; device memory is owned by the
 * library; one host thread per context; calls are stream-ordered on the
 * context's stream and return when their results are ready (host buffers)
 * unless stated otherwise.  Every entry point returns BGPU_OK or an error
 * code, with the message available from bgpu_last_error_string().
 *
 * The reference has no plugin API for this path; its call sites are
 * internal C++ functions.  Each entry point below names the reference
 * function whose work it replaces (file:line in sanshar/Block).
 *
 * Conventions shared with the reference:
 *  - quanta are (particle number, 2S, irrep) triples; irreps are 0-based
 *    abelian indices with XOR products (Symmetry.C:22-120);
 *  - an operator is an SU(2) tensor stored as reduced dense blocks for every
 *    allowed (bra quantum, ket quantum) pair, enumerated bra-major then
 *    ket, each block row-major (SparseMatrix::allocate, BaseOperator.C:123-145;
 *    Newmat row-major storage, MatrixBLAS.C:144); operators of a block are
 *    laid out back to back in the order of their keys (type, i, j, 2k)
 *    sorted ascending;
 *  - a wavefunction is block-sparse over the (left quantum, right quantum)
 *    sectors coupling to the target, left-major, each sector row-major
 *    (Wavefunction::initialise, wavefunction.C:17-52).
 */
#ifndef BGPU_H
#define BGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BGPU_OK 0
#define BGPU_ERR_INVALID 1
#define BGPU_ERR_CUDA 2
#define BGPU_ERR_RUNTIME 3

/* operator types (BaseOperator.h:35-45) */
#define BGPU_OP_HAM 0
#define BGPU_OP_CRE 1
#define BGPU_OP_CRE_DES 2
#define BGPU_OP_CRE_CRE 3
#define BGPU_OP_CRE_DESCOMP 4
#define BGPU_OP_DES_DESCOMP 5
#define BGPU_OP_CRE_CRE_DESCOMP 6
#define BGPU_OP_OVERLAP 7

/* arithmetic of the sigma product: FP64, or bf16 slices on the tensor cores
 * with FP32 accumulation -- 2 slices / 3 products per logical product
 * (BF16X3) or 3 slices / 6 products (BF16X6) with warp-level MMAs, or
 * 2 slices / 3 products on tcgen05 with TMEM accumulators and bulk-copy
 * staged operands (BF16X3_TC), or the same kernels with 2 fp16 slices
 * (11-bit significands, values within +-65504; FP16X2_TC).  With a split
 * precision, bgpu_davidson and bgpu_run_dmrg iterate with split-precision
 * sigma and then correct the roots against FP64 residuals (see
 * bgpu_set_refinement). */
#define BGPU_PREC_FP64 0
#define BGPU_PREC_BF16X3 1
#define BGPU_PREC_BF16X6 2
#define BGPU_PREC_BF16X3_TC 3
#define BGPU_PREC_FP16X2_TC 4
/* products of six-digit integer slices on the tensor cores, accumulated
 * exactly and summed in FP64: about 1e-12 relative to FP64 */
#define BGPU_PREC_EXACT_TC 5

typedef struct bgpu_ctx bgpu_ctx;

/* Context on CUDA device `device`. */
int bgpu_create(bgpu_ctx** ctx, int device);
int bgpu_destroy(bgpu_ctx* ctx);
const char* bgpu_last_error_string(const bgpu_ctx* ctx);
/* Library version string. */
const char* bgpu_version(void);
/* Arithmetic of sigma products (BGPU_PREC_*). */
int bgpu_set_precision(bgpu_ctx* ctx, int precision);
/*
 * Refinement of split-precision Davidson solves (no reference counterpart;
 * the reference iterates in FP64 throughout, linear.C:179-385):
 *   mode 1, defect correction: after the split-precision solve
 *     converges, its Ritz vectors get FP64 products and the Davidson
 *     restarts from them with their FP64 subspace matrix and residuals;
 *     further basis vectors (corrections) get split-precision products.
 *     Rounds repeat until a restart finds every root's squared FP64
 *     residual norm below the solve's tolerance without expanding, or a
 *     restart converges with corrections whose split-precision error bound
 *     keeps (|r| + bound)^2 below the tolerance for every root (at most 8
 *     rounds; otherwise the energies are FP64 Rayleigh quotients of the
 *     final vectors).  The bound of one split product of a unit vector is 4
 *     times the largest difference between the split and FP64 products of
 *     the first round's Ritz vectors; it is carried through the Ritz
 *     rotations.  Energies are then FP64 Ritz values and the vectors meet
 *     the FP64 convergence test of an FP64 solve.
 *   mode 2 (default): mode 1 with the restart products on the tensor cores
 *     (BGPU_PREC_EXACT_TC, about 1e-12 relative to FP64) instead of the FP64
 *     pipe, with the pair terms cut into as many chunks as the free device
 *     memory needs; until this context has measured its FP64 product rate, a
 *     solve whose product has at least 1e11 flops still uses FP64 products
 *     (the rate prices the FP64 solves in bgpu_run_stats).
 *   mode 0, energy only: one FP64 Rayleigh quotient per converged root, and
 *     in bgpu_run_dmrg only for the steps bgpu_set_refine_window selects.
 */
int bgpu_set_refinement(bgpu_ctx* ctx, int mode);
/* FP64 restarts and FP64 products spent by defect correction in this
 * context, and whether the last solve's roots met the tolerance on FP64
 * residuals (1), on FP64 residual bounds (2), or not (0). */
int bgpu_refinement_stats(bgpu_ctx* ctx, int64_t* rounds, int64_t* fp64_products, int* last_verified);
/* Split-precision sweeps with energy-only refinement (bgpu_set_refinement
 * mode 0; no reference counterpart): bgpu_run_dmrg refines
 * a step's energies with FP64 Rayleigh quotients only when its unrefined
 * lowest energy is within `eh` of the lowest one seen so far in the sweep,
 * and always at the last step of every sweep (so that sweep and final
 * energies are FP64-refined).  Qualifying steps are kept (their enlarged
 * blocks and vectors, at most 4 at a time) and refined at the end of the
 * sweep only if they are still within `eh` of the sweep's lowest unrefined
 * energy.  0 refines every step.  Default 1e-3 Eh. */
int bgpu_set_refine_window(bgpu_ctx* ctx, double eh);
/* Davidson start of bgpu_run_dmrg's block steps: transform = 1 (default)
 * transforms the previous step's wavefunction into the next step's state
 * space when the two steps are consecutive in one sweep direction
 * (TRANSFORM guess, guess_wavefunction.C:526-620), otherwise and with
 * transform = 0 unit vectors on the lowest diagonal elements (BASIC guess,
 * guess_wavefunction.C:258-273). */
int bgpu_set_guess(bgpu_ctx* ctx, int transform);
/* Block store of bgpu_run_dmrg (replaces the reference's block files,
 * save_load_block.C:58-110): on = 1 keeps every stored block that the
 * current block step does not read in host memory only (copied there once,
 * copied back when a step needs it), so that the device holds the step's
 * own blocks; 0 (default) keeps all blocks on the device.  The `spill`
 * keyword of dmrg.conf does the same.  bgpu_run_stats reports the copies
 * and the peak block storage. */
int bgpu_set_spill(bgpu_ctx* ctx, int on);
/* Davidson iterations (bgpu_davidson, bgpu_run_dmrg) as launches of a
 * captured CUDA graph: on = 1 (default, unless the environment sets
 * BGPU_DAVIDSON_GRAPH=0) captures one iteration (the sigma of the newest
 * basis vector, subspace eigenproblem, Ritz rotation, Olsen residual,
 * convergence and deflation decisions, Gram-Schmidt) once per solve and
 * launches it per iteration; on = 0 issues the same launches one by one.
 * Results are identical.  No reference counterpart (the reference steps
 * Linear::block_davidson, linear.C:179-385, on the host). */
int bgpu_set_davidson_graph(bgpu_ctx* ctx, int on);
/* Graph launches of the last Davidson solve (0 when it ran without capture). */
int bgpu_davidson_graph_launches(bgpu_ctx* ctx, int64_t* launches);
/* Work-list schedule of the tensor-core sigma (no reference counterpart; the
 * reference calls one DGEMM per sector pair, operatorfunctions.C:515,530):
 * mode 0 (default) runs every sigma as two persistent launches (two blocks
 * per SM, longest-processing-time assignment of the sector tiles); mode 1 is
 * the per-sector baseline: one launch per psi sector (stage-1 products) and
 * per sigma sector (stage-2 tiles), one block per tile.  Applies to the next
 * product of every superblock. */
int bgpu_set_tc_schedule(bgpu_ctx* ctx, int mode);
/* Output-tile width of the tensor-core sigma (no reference counterpart):
 * 64 columns (two pipelines per SM, 128 x 64 MMAs) or 128 (one pipeline per
 * SM, 128 x 128 MMAs reading each A piece once for twice the work); 0
 * (default) chooses 128 when most of the stage-2 work lies in sectors at
 * least 128 columns wide, or lets the autotuner choose.  Applies to the next
 * product of every superblock (its operands are packed again). */
int bgpu_set_tc_tile_width(bgpu_ctx* ctx, int nb);
/* Stacking of small stage-1 products in the tensor-core sigma (no reference
 * counterpart; the reference multiplies every operator block separately,
 * operatorfunctions.C:515): the products of operator blocks of at most
 * `rows` rows (0, or a multiple of 8 up to 128; default 64) that read the
 * same psi block are stacked into one 128-row MMA tile, each row sent to its
 * own stage-1 operand.  0 multiplies every block separately.  Results are the
 * same dot products either way.  Applies to the next product of every
 * superblock (its operators are packed again). */
int bgpu_set_tc_stacking(bgpu_ctx* ctx, int rows);
/* Autotuner of the persistent tensor-core schedule (no reference
 * counterpart): on = 1 times candidate tile widths (64, 128 columns) and,
 * for each, candidate knobs (cost model of the block assignment, splitting
 * of heavy tiles, accumulation group length) on the first product of every
 * superblock whose sector-size histogram was not seen before and keeps the
 * fastest; superblocks with a known histogram reuse the choice.  cache_path
 * (may be NULL: the choices made so far are kept) is a text file the
 * choices are read from and appended to; it replaces the choices held so
 * far. */
int bgpu_set_autotune(bgpu_ctx* ctx, int on, const char* cache_path);
/* Histograms tuned by this context, histograms in the cache, seconds spent tuning. */
int bgpu_autotune_stats(bgpu_ctx* ctx, int64_t* keys_tuned, int64_t* keys_cached, double* seconds);

/*
 * Declare a block: its state space and operator catalogue.
 * Replaces the SpinBlock state (spinblock.h:104-259) and the operator
 * containers Op_component / SparseMatrix::allocate (op_components.h:161-210,
 * BaseOperator.C:123-145).
 *   norb, orbsym[norb]: orbital irreps (0-based), group: "c1", "d2h", ...
 *   quanta[3*nquanta]: (n, 2S, irrep) sorted ascending; states[nquanta]
 *   op_keys[4*nops]: (type, i, j, 2k) per operator
 *   is_dot: 1 for single-site blocks
 * Returns a block handle and the number of doubles of its operator arena.
 */
int bgpu_block_define(bgpu_ctx* ctx, int norb, const int* orbsym, const char* group, int nquanta, const int* quanta,
                      const int* states, int nops, const int* op_keys, int is_dot, int* handle,
                      int64_t* arena_elems);
/* Element offset of every operator of a block inside its arena (nops values,
 * in the order the operators were declared). */
int bgpu_block_op_offsets(bgpu_ctx* ctx, int handle, int64_t* offsets, int nops);
/* Copy a whole operator arena in / out (host buffers, `n` doubles). */
int bgpu_block_upload(bgpu_ctx* ctx, int handle, const double* arena, int64_t n);
int bgpu_block_download(bgpu_ctx* ctx, int handle, double* arena, int64_t n);
int bgpu_block_free(bgpu_ctx* ctx, int handle);

/* Orbitals of a block, in order (SpinBlock::sites, spinblock.h:104-259);
 * the enlarged-block build needs them for its integral-weighted terms. */
int bgpu_block_set_sites(bgpu_ctx* ctx, int handle, int nsites, const int* sites);
/* State space of a block (StateInfo::quanta / quantaStates, StateInfo.h:79-206):
 * *nquanta is the capacity of quanta[3*cap] / states[cap] on entry (both may
 * be NULL to query the count) and the block's number of quanta on return. */
int bgpu_block_quanta(bgpu_ctx* ctx, int handle, int* nquanta, int* quanta, int* states);

/*
 * Hamiltonian integrals read by the operator builds (Input::readorbitalsfile,
 * input.C:1407-1681; the integral-weighted sums of the complementary
 * operators, Operators.C:87-137, 1059-1194).  _load takes the `orbitals` of
 * a dmrg.conf (an FCIDUMP, or synthetic:<norb>:<nelec>:<nchol>:<seed>:<d2h>)
 * reordered as the configuration asks and returns norb; _define takes
 * h1[norb*norb] row-major and the chemist-notation eri[norb^4] with (ij|kl)
 * at ((i*norb+j)*norb+k)*norb+l, both in the block orbitals' order.
 */
int bgpu_integrals_load(bgpu_ctx* ctx, const char* conf_path, int* handle, int* norb);
int bgpu_integrals_define(bgpu_ctx* ctx, int norb, const int* orbsym, const double* h1, const double* eri, double ecore,
                          int* handle);
int bgpu_integrals_free(bgpu_ctx* ctx, int handle);

/*
 * Enlarged block left (x) right built on the GPU, one of the two a single
 * site (is_dot): SpinBlock::BuildSumBlock (spinblock.C:194-260) with every
 * operator made by TensorProduct (operatorfunctions.h:34,
 * operatorfunctions.C:146-254) as Op::build does it (Operators.C:453-2395).
 * Both sub-blocks must be defined with their sites and uploaded.
 *   filter[3] = (nelec, 2S, norb) of the whole system: quanta the remaining
 *     orbitals cannot complete to that target are dropped
 *     (PARTICLE_SPIN_NUMBER_CONSTRAINT, StateInfo.C:123-308); NULL keeps all
 *   op_keys[4*nops]: catalogue of the enlarged block (type, i, j, 2k)
 * Returns the new block, the doubles of its arena and its number of quanta
 * (read them with bgpu_block_quanta; download with bgpu_block_download).
 */
int bgpu_build_enlarged_ops(bgpu_ctx* ctx, int integrals, int left, int right, const int* filter, int nops,
                            const int* op_keys, int* big, int64_t* arena_elems, int* nquanta);

/*
 * Superblock L|R with its operator-pair list; compiles the sigma work lists.
 * Replaces the set-up of SpinBlock::multiplyH (spinblock.C:722-789) and the
 * opxop pair loops (opxop.C:155-285).
 *   target[3]: (n, 2S, irrep) of the wavefunction
 *   nterms, coef[nterms], term_ops[4*nterms] = (left op index | -1 identity,
 *   left transpose flag, right op index | -1, right transpose flag); op
 *   indices refer to the op_keys order of the blocks' declarations; every
 *   term is coef * [left x right]^0 applied to psi (TensorMultiply,
 *   operatorfunctions.C:485-537).
 *   ecore: constant added as ecore * psi
 * Returns a superblock handle and the number of doubles of a wavefunction.
 */
int bgpu_superblock_define(bgpu_ctx* ctx, int left, int right, const int* target, int nterms, const double* coef,
                           const int* term_ops, double ecore, int* sb, int64_t* psi_elems);
int bgpu_superblock_free(bgpu_ctx* ctx, int sb);
/* Algorithmic work of one sigma: FP64-equivalent flops and bytes. */
int bgpu_superblock_work(bgpu_ctx* ctx, int sb, double* flops, double* bytes);
/* Bounded-wait self-check of the tensor-core kernels (no reference
 * counterpart): one GPU thread waits, with the kernels' own bounded mbarrier
 * wait, on a barrier that nothing arrives at, for limit_ms (0 < limit_ms <=
 * 1000).  gave_up = 1 when the wait returned failure, status = the status
 * word the wait sets, waited_ms = time spent waiting. */
int bgpu_tc_wait_selftest(bgpu_ctx* ctx, double limit_ms, int* gave_up, int* status, double* waited_ms);
/* Work-list statistics of one sigma (no reference counterpart), info[n]:
 *   FP64-equivalent flops, algorithmic bytes, tensor-core flops issued by the
 *   tcgen05 path (3 bf16 products, padded tiles), phase-1 tasks, phase-2
 *   tasks, phase-2 items, phase-2 items reading a stage-1 product, split
 *   tiles, packed elements of the L-operator / R-operator / psi / stage-1
 *   pools, FP64 stage-1 units, FP64 items, the schedule knobs (item cost,
 *   split, group, per-sector flag, 1 when chosen by the autotuner), the
 *   launches of one sigma at the current precision and the doubles of
 *   stage-1 intermediates the FP64 product needs (compare with
 *   BGPU_NOALLOC_SCRATCH_DOUBLES), the output-tile width of the
 *   tensor-core plan, its stacked phase-1 tiles and the stage-1 products
 *   they hold.  Builds the tensor-core plan if needed. */
int bgpu_superblock_info(bgpu_ctx* ctx, int sb, double* info, int n);
/* Kernel launches of one sigma product. */
int bgpu_superblock_launches(bgpu_ctx* ctx, int sb, int* launches);

/*
 * sigma = H psi on host buffers (copies in and out are part of the call), in
 * the context's precision (bgpu_set_precision).
 * Replaces SpinBlock::multiplyH (spinblock.C:722-789) as called by the
 * Davidson functor (davidson.C:19-22).
 */
int bgpu_sigma(bgpu_ctx* ctx, int sb, const double* psi, double* sigma);
/* Same on device pointers (stream-ordered, asynchronous). */
int bgpu_sigma_device(bgpu_ctx* ctx, int sb, const double* psi_dev, double* sigma_dev);
/* n doubles of page-locked host memory (no reference counterpart): host
 * buffers for bgpu_sigma whose copies to and from the device run at the
 * host link's rate instead of through a pageable staging copy.  Release
 * with bgpu_host_free. */
int bgpu_host_alloc(bgpu_ctx* ctx, int64_t n, double** p);
int bgpu_host_free(bgpu_ctx* ctx, double* p);
/*
 * `reps` back-to-back sigma products on device buffers timed with CUDA
 * events on the context's stream; ms[0] = total.  FP64: ms[1] = first GEMM
 * stage, ms[2] = second stage.  Split precision: ms[1] = the fused two-stage
 * tensor-core kernel, ms[2] = the rest (psi slicing, partial-tile
 * reduction).  All summed over the repetitions.
 */
int bgpu_sigma_timed(bgpu_ctx* ctx, int sb, const double* psi_dev, double* sigma_dev, int reps, double* ms);
/*
 * sigma = H psi on device buffers without allocating any memory.  This entry
 * point has no counterpart in the reference; it exists for callers that may
 * not allocate device memory while they run -- for example code recorded
 * into a CUDA graph, code running under a fixed memory budget, or a host
 * application whose own allocator owns the GPU -- and therefore cannot let
 * the library call cudaMalloc on their behalf.  Instead of a per-superblock
 * scratch buffer, the stage-1 intermediates of the product live in one
 * fixed array of BGPU_NOALLOC_SCRATCH_DOUBLES doubles (32 MiB) that every
 * GPU loading the library holds until the process exits.  The superblock
 * must already be defined (bgpu_superblock_define / _prepare_superblock);
 * superblocks whose intermediates do not fit are rejected with
 * BGPU_ERR_INVALID.  The first call on a device looks up the array's
 * address and should therefore come before any stream capture.  All calls
 * share the array: calls whose work overlaps on the GPU (other streams,
 * other contexts on the same device) race and must be serialised by the
 * caller.  Stream-ordered and asynchronous like bgpu_sigma_device.  The
 * product is always the FP64 one, whatever bgpu_set_precision chose: the
 * split-precision paths need packed operand pools that the library
 * allocates on first use, so they are not available here.  Counted in the
 * context's sigma statistics like every other product.
 */
#define BGPU_NOALLOC_SCRATCH_DOUBLES (4 * 1024 * 1024)
int bgpu_sigma_noalloc(bgpu_ctx* ctx, int sb, const double* psi_dev, double* sigma_dev);
/* Diagonal of H (SpinBlock::diagonalH, spinblock.C:855-899). */
int bgpu_hdiag(bgpu_ctx* ctx, int sb, double* diag);
/*
 * Block Davidson for the lowest `nroots` states (Linear::block_davidson,
 * linear.C:179-385): tol bounds the squared residual norm.  energies[nroots];
 * vectors (nroots x psi_elems, may be NULL) receive the eigenvectors.
 */
int bgpu_davidson(bgpu_ctx* ctx, int sb, int nroots, double tol, int max_iter, double* energies, double* vectors,
                  int* iterations);
/*
 * Reduced density matrix of the left (left=1) or right block from the last
 * Davidson vectors with root weights[nroots] and its per-sector
 * eigenvalues, ascending within each sector, concatenated in sector order
 * (DensityMatrix::makedensitymatrix, density.C:27-90; diagonalise_dm,
 * rotationmat.C:258-279).
 */
int bgpu_density_eig(bgpu_ctx* ctx, int sb, int left, int nroots, const double* weights, double* eigvals,
                     int64_t n_eigvals);

/*
 * Symmetric eigendecomposition of a batch of dense matrices (diagonalise,
 * MatrixBLAS.h:105 / MatrixBLAS.C:381-414, which calls LAPACK DSYEV), with
 * the library's own GPU solver (Householder tridiagonalisation, implicit QL
 * with accumulated rotations, back-transformation; the same solver runs on
 * every density-matrix sector above 48 states).  Matrix j has order
 * dims[j] (1 .. 4096) and is stored row-major in a, matrices back to back;
 * eigvals receive the eigenvalues of each matrix in ascending order and
 * eigvecs (may be NULL) the eigenvectors, row-major per matrix with column c
 * the eigenvector of the c-th eigenvalue.  Host buffers.
 */
int bgpu_diagonalise(bgpu_ctx* ctx, int nmat, const int* dims, const double* a, double* eigvals, double* eigvecs);
/*
 * Noise added by the following bgpu_density_eig calls (the `noise` and
 * `additional_noise` of DensityMatrix::makedensitymatrix, density.C:27-90):
 *   perturbative > 0: add_onedot_noise (density.C:330-421) -- for every
 *     root, rho += perturbative / nroots / tr(N) * N when tr(N) > 1, N the
 *     sum of the normalised outer products of (O x 1) psi (the block's CRE
 *     and two-index operators and their adjoints, coupled to every total
 *     spin);
 *   random > 0: add_twodot_noise (density.C:92-165) -- for every root,
 *     normalised random wavefunctions of the quanta next to the target each
 *     add random / nroots / (number of quanta) of their outer product; the
 *     values are uniform in [-1, 1) from a counter-based generator seeded
 *     with `seed` (the same values on every run and engine).
 * 0, 0 (the default) adds none.  bgpu_run_dmrg takes its noise from the
 * dmrg.conf instead (schedule noise column; twodot_noise).
 */
int bgpu_set_density_noise(bgpu_ctx* ctx, double perturbative, double random, uint64_t seed);
/*
 * Wavefunctions the next bgpu_density_eig reads (host, nroots x psi_elems in
 * the superblock's sector order), in place of the last Davidson vectors:
 * the `wave_solutions` argument of DensityMatrix::makedensitymatrix
 * (density.C:27-90).
 */
int bgpu_set_wavefunctions(bgpu_ctx* ctx, int sb, int nroots, const double* vectors);
/*
 * The last density matrix and its eigenvectors (the matrices diagonalise_dm
 * fills, rotationmat.C:258-279): per sector of the block, back to back in
 * quantum order, rho row-major and the eigenvectors row-major with column c
 * the eigenvector of the c-th smallest eigenvalue.  n = sum of the squared
 * sector sizes; either pointer may be NULL.
 */
int bgpu_density_download(bgpu_ctx* ctx, double* rho, double* vecs, int64_t n);
/*
 * Renormalised block small = U^T big U for every operator of its catalogue
 * (SpinBlock::transform_operators, spinblock.h:253, save_load_block.C:267-319;
 * SparseMatrix::renormalise_transform, BaseOperator.h:199-204 /
 * BaseOperator.C:341-363; MatrixRotate, MatrixBLAS.C:553-572).
 *   kept[nquanta of big]: states kept per quantum (0 drops the quantum)
 *   rotations: per quantum with kept > 0, states x kept row-major, back to
 *     back in quantum order (the rotation matrices of makeRotateMatrix,
 *     renormalise.C:135-166); NULL takes, per quantum, the eigenvectors of
 *     the kept[q] largest eigenvalues of the last bgpu_density_eig of this
 *     block, in descending order, without leaving the GPU
 *   op_keys[4*nops]: catalogue of the renormalised block (each present in big)
 * Returns the new block, the doubles of its arena and its number of quanta.
 */
int bgpu_renormalise(bgpu_ctx* ctx, int big, const int* kept, const double* rotations, int nops, const int* op_keys,
                     int* small, int64_t* arena_elems, int* nquanta);
/* The rotation that made a block returned by bgpu_renormalise, in the layout
 * of its `rotations` argument (n doubles): the rotation matrices a Block
 * caller stores for its later steps (rotationmat.C:21-60). */
int bgpu_rotation_download(bgpu_ctx* ctx, int small, double* rot, int64_t n);

/*
 * Device-memory accounting: pointer to a device buffer of `n` doubles owned
 * by the context (for callers that drive bgpu_sigma_device).
 */
int bgpu_device_alloc(bgpu_ctx* ctx, int64_t n, double** ptr);
int bgpu_device_free(bgpu_ctx* ctx, double* ptr);
int bgpu_copy_to_device(bgpu_ctx* ctx, double* dst, const double* src, int64_t n);
int bgpu_copy_to_host(bgpu_ctx* ctx, double* dst, const double* src, int64_t n);
int bgpu_synchronize(bgpu_ctx* ctx);
/* Start / stop the CUDA profiler's collection range (cudaProfilerStart/Stop),
 * so that a profiler run with collection off at start sees only the calls in
 * between. */
int bgpu_profiler_start(bgpu_ctx* ctx);
int bgpu_profiler_stop(bgpu_ctx* ctx);
/* Tensor-core self-check (no reference counterpart): one 128 x n tile
 * d = a * b^T on tcgen05 with a TMEM accumulator, d row-major f32.  With
 * packed = 0, a (128 x k) and b (n x k) are row-major bf16 bit patterns
 * (16 <= k <= 64); with packed = 1 they are K-chunks of 64 columns in the
 * K-major core-matrix order (chunk c of an r-row operand at element
 * r * 64 * c; element (i, j) of a chunk at byte (j/8)*r*16 + (i/8)*128 +
 * (i%8)*16 + (j%8)*2), moved by bulk copies (16 <= k <= 256).
 * 16 <= n <= 256; n and k multiples of 16. */
int bgpu_tc_tile(bgpu_ctx* ctx, const uint16_t* a, const uint16_t* b, float* d, int n, int k, int packed);

/*
 * Superblock of the bipartition after orbital `partition` (left block
 * [0..partition], right block [partition+1..norb-1]) for the system of a
 * dmrg.conf, built from warm-up blocks of bond dimension M (the first
 * schedule entry) made by seeded random rotations: the sector structure and
 * operator catalogue of a mid-sweep step (InitBlocks / BlockAndDecimate,
 * sweep.C:91-178) without the Davidson solves.  The superblock owns its
 * blocks; use it with bgpu_sigma / bgpu_davidson / bgpu_hdiag.
 */
int bgpu_prepare_superblock(bgpu_ctx* ctx, const char* conf_path, int partition, int* sb, int64_t* psi_elems);

/*
 * Full two-site sweep DMRG from a dmrg.conf and its FCIDUMP (the
 * `block.spin_adapted dmrg.conf` entry, main.C:25-52 / dmrg.C:600-706), with
 * all operator and wavefunction arithmetic on the GPU.  `orbitals` may also
 * name a generated Hamiltonian: synthetic:<norb>:<nelec>:<nchol>:<seed>:<d2h>.
 * energies[max_roots] receive the final energies; stats[13] (may be NULL):
 *   sweeps, sigma calls, sigma seconds, sigma flops, total seconds, max
 *   discarded weight, last-sweep energy, number of roots, then wall seconds
 *   of the block-build, Davidson and density/rotation phases, the device
 *   seconds of the renormalisations (they run while the host builds and
 *   plans the next step, so the phases overlap), and the host seconds spent
 *   compiling sigma work lists (part of the Davidson phase).
 */
int bgpu_run_dmrg(bgpu_ctx* ctx, const char* conf_path, int verbose, double* energies, int max_roots,
                  double* stats);
/* Spin-summed spatial one-particle density matrix gamma_ij =
 * sum_s <a+_is a_js> of root `root` (norb x norb row-major, the FCIDUMP's
 * orbital order) from the last bgpu_run_dmrg whose dmrg.conf had `onepdm`
 * (modules/onepdm, onepdm.C:24-55; the same values as its
 * spatial_onepdm.<root>.<root>.txt, which the run also writes under
 * `prefix <dir>` when given).  The run evaluates it in one more sweep after
 * the last one. */
int bgpu_onepdm(bgpu_ctx* ctx, int root, double* gamma, int norb);
/* Transition one-particle density matrix gamma_ij = sum_s <bra| a+_is a_js
 * |ket> between two state-averaged roots of the same run (norb x norb
 * row-major, the FCIDUMP's orbital order); bra == ket gives bgpu_onepdm's
 * matrix.  The reference's `tran_onepdm` writes the same values as
 * spatial_onepdm.<bra>.<ket>.txt (bra > ket); this run does so under
 * `prefix <dir>` with that keyword. */
int bgpu_transition_onepdm(bgpu_ctx* ctx, int bra, int ket, double* gamma, int norb);
/* Arithmetic of the last bgpu_run_dmrg (no reference counterpart), out[n]:
 * split-precision products and their seconds, FP64 products and their
 * seconds, defect-correction rounds, the FP64 product time the same
 * solves would have taken (every product of a block step at that step's
 * measured FP64 product time, summed over the steps with an FP64 product),
 * the warm-up's wall seconds, the solves accepted on the error bound of
 * their corrections (no FP64 product after the last restart; see
 * bgpu_refinement_stats), the exact-slice restart products and their
 * seconds (refinement mode 2), the FP64-equivalent flops of the sweeps'
 * renormalisations (warm-up excluded), the FP64 product rate measured in
 * this context (flops per second, 0 if none), whether the renormalisations
 * ran on the exact-slice kernels (1) or the FP64 pipe (0), their device
 * seconds during the sweeps, the blocks copied back from host memory
 * (bgpu_set_spill), the bytes copied to the device and to the host for
 * them, the most operator-arena bytes the device held at once, then the
 * wall seconds of each sweep. */
int bgpu_run_stats(bgpu_ctx* ctx, double* out, int n);
/* Sweep energies (lowest root per sweep, Sweep::do_one's return value,
 * sweep.C:436-453) of the last bgpu_run_dmrg: *n = number of sweeps, up to
 * cap of them copied to e. */
int bgpu_sweep_energies(bgpu_ctx* ctx, double* e, int cap, int* n);

#ifdef __cplusplus
}
#endif

#endif /* BGPU_H */
