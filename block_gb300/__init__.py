"""GB300-native sweep hot path of spin-adapted two-site DMRG (sanshar/Block).

Python mirror of the library's C ABI (include/bgpu.h).  The compute path is
the in-tree CUDA library block_gb300/_build/libblockgb300.so; importing the
package never falls back to anything else, and every call raises if the
library or a GPU is missing.
"""
import ctypes
import os

import numpy as np

__all__ = ["Context", "BgpuError", "load_library", "LIB_PATH", "OP", "PREC"]

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libblockgb300.so")

OP = dict(HAM=0, CRE=1, CRE_DES=2, CRE_CRE=3, CRE_DESCOMP=4, DES_DESCOMP=5, CRE_CRE_DESCOMP=6, OVERLAP=7)
PREC = dict(fp64=0, bf16x3=1, bf16x6=2, bf16x3tc=3, fp16x2tc=4, exacttc=5)
# BGPU_NOALLOC_SCRATCH_DOUBLES: doubles of the fixed array behind bgpu_sigma_noalloc
NOALLOC_SCRATCH_DOUBLES = 4 * 1024 * 1024

_lib = None

_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double
_P = ctypes.c_void_p
_IP = ctypes.POINTER(ctypes.c_int)
_I64P = ctypes.POINTER(ctypes.c_int64)
_DP = ctypes.POINTER(ctypes.c_double)
_CP = ctypes.c_char_p

_SIGS = {
    "bgpu_create": (_I, [ctypes.POINTER(_P), _I]),
    "bgpu_destroy": (_I, [_P]),
    "bgpu_last_error_string": (_CP, [_P]),
    "bgpu_version": (_CP, []),
    "bgpu_set_precision": (_I, [_P, _I]),
    "bgpu_block_define": (_I, [_P, _I, _IP, _CP, _I, _IP, _IP, _I, _IP, _I, _IP, _I64P]),
    "bgpu_block_op_offsets": (_I, [_P, _I, _I64P, _I]),
    "bgpu_block_upload": (_I, [_P, _I, _DP, _I64]),
    "bgpu_block_download": (_I, [_P, _I, _DP, _I64]),
    "bgpu_block_free": (_I, [_P, _I]),
    "bgpu_superblock_define": (_I, [_P, _I, _I, _IP, _I, _DP, _IP, _D, _IP, _I64P]),
    "bgpu_superblock_free": (_I, [_P, _I]),
    "bgpu_superblock_work": (_I, [_P, _I, _DP, _DP]),
    "bgpu_sigma": (_I, [_P, _I, _DP, _DP]),
    "bgpu_sigma_device": (_I, [_P, _I, _P, _P]),
    "bgpu_host_alloc": (_I, [_P, _I64, ctypes.POINTER(_DP)]),
    "bgpu_host_free": (_I, [_P, _DP]),
    "bgpu_hdiag": (_I, [_P, _I, _DP]),
    "bgpu_sigma_timed": (_I, [_P, _I, _P, _P, _I, _DP]),
    "bgpu_superblock_launches": (_I, [_P, _I, _IP]),
    "bgpu_sigma_noalloc": (_I, [_P, _I, _P, _P]),
    "bgpu_davidson": (_I, [_P, _I, _I, _D, _I, _DP, _DP, _IP]),
    "bgpu_density_eig": (_I, [_P, _I, _I, _I, _DP, _DP, _I64]),
    "bgpu_device_alloc": (_I, [_P, _I64, ctypes.POINTER(_P)]),
    "bgpu_device_free": (_I, [_P, _P]),
    "bgpu_copy_to_device": (_I, [_P, _P, _DP, _I64]),
    "bgpu_copy_to_host": (_I, [_P, _DP, _P, _I64]),
    "bgpu_synchronize": (_I, [_P]),
    "bgpu_profiler_start": (_I, [_P]),
    "bgpu_profiler_stop": (_I, [_P]),
    "bgpu_tc_tile": (_I, [_P, _P, _P, _P, _I, _I, _I]),
    "bgpu_superblock_info": (_I, [_P, _I, _DP, _I]),
    "bgpu_set_refine_window": (_I, [_P, ctypes.c_double]),
    "bgpu_set_guess": (_I, [_P, _I]),
    "bgpu_set_spill": (_I, [_P, _I]),
    "bgpu_set_davidson_graph": (_I, [_P, _I]),
    "bgpu_set_tc_schedule": (_I, [_P, _I]),
    "bgpu_set_tc_tile_width": (_I, [_P, _I]),
    "bgpu_set_tc_stacking": (_I, [_P, _I]),
    "bgpu_set_autotune": (_I, [_P, _I, _CP]),
    "bgpu_autotune_stats": (_I, [_P, _I64P, _I64P, _DP]),
    "bgpu_davidson_graph_launches": (_I, [_P, _I64P]),
    "bgpu_tc_wait_selftest": (_I, [_P, ctypes.c_double, _IP, _IP, _DP]),
    "bgpu_prepare_superblock": (_I, [_P, _CP, _I, _IP, _I64P]),
    "bgpu_run_dmrg": (_I, [_P, _CP, _I, _DP, _I, _DP]),
    "bgpu_set_refinement": (_I, [_P, _I]),
    "bgpu_sweep_energies": (_I, [_P, _DP, _I, _IP]),
    "bgpu_run_stats": (_I, [_P, _DP, _I]),
    "bgpu_onepdm": (_I, [_P, _I, _DP, _I]),
    "bgpu_transition_onepdm": (_I, [_P, _I, _I, _DP, _I]),
    "bgpu_refinement_stats": (_I, [_P, _I64P, _I64P, _IP]),
    "bgpu_block_set_sites": (_I, [_P, _I, _I, _IP]),
    "bgpu_block_quanta": (_I, [_P, _I, _IP, _IP, _IP]),
    "bgpu_integrals_load": (_I, [_P, _CP, _IP, _IP]),
    "bgpu_integrals_define": (_I, [_P, _I, _IP, _DP, _DP, _D, _IP]),
    "bgpu_integrals_free": (_I, [_P, _I]),
    "bgpu_build_enlarged_ops": (_I, [_P, _I, _I, _I, _IP, _I, _IP, _IP, _I64P, _IP]),
    "bgpu_set_wavefunctions": (_I, [_P, _I, _I, _DP]),
    "bgpu_diagonalise": (_I, [_P, _I, _IP, _DP, _DP, _DP]),
    "bgpu_set_density_noise": (_I, [_P, _D, _D, ctypes.c_uint64]),
    "bgpu_density_download": (_I, [_P, _DP, _DP, _I64]),
    "bgpu_renormalise": (_I, [_P, _I, _IP, _DP, _I, _IP, _IP, _I64P, _IP]),
    "bgpu_rotation_download": (_I, [_P, _I, _DP, _I64]),
}

EXPORTED = sorted(_SIGS)


class BgpuError(RuntimeError):
    pass


def load_library(path=LIB_PATH):
    """Load the CUDA library; raises if it was not built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise BgpuError("native library missing: %s (run __graft_entry__.build())" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _ip(a):
    return a.ctypes.data_as(_IP)


def _dp(a):
    return a.ctypes.data_as(_DP)


def pack_kmajor(x):
    """Rows x k matrix (rows % 8 == 0, k % 16 == 0) as K-chunks of 64 columns,
    each in the K-major core-matrix order of the tensor-core kernels."""
    r, k = x.shape
    out = np.zeros(r * k, dtype=x.dtype)
    for c in range(0, k, 64):
        w = min(64, k - c)
        blk = x[:, c:c + w].reshape(r // 8, 8, w // 8, 8).transpose(2, 0, 1, 3)  # [k/8][r/8][8][8]
        out[r * c:r * c + r * w] = blk.reshape(-1)
    return out


class Context:
    """One CUDA context of the library (bgpu_create / bgpu_destroy)."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = _P()
        rc = self.lib.bgpu_create(ctypes.byref(h), device)
        self.h = h
        if rc != 0:
            msg = self.lib.bgpu_last_error_string(h).decode() if h else "bgpu_create failed"
            if h:
                self.lib.bgpu_destroy(h)
            self.h = None
            raise BgpuError(msg)

    def close(self):
        if self.h:
            self.lib.bgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise BgpuError(self.lib.bgpu_last_error_string(self.h).decode())

    def set_precision(self, prec):
        self._check(self.lib.bgpu_set_precision(self.h, PREC[prec] if isinstance(prec, str) else int(prec)))

    # ---- blocks and superblocks (SpinBlock / SpinBlock::multiplyH boundary)
    def block_define(self, orbsym, group, quanta, states, op_keys, is_dot=False):
        orbsym = np.ascontiguousarray(orbsym, dtype=np.int32)
        quanta = np.ascontiguousarray(quanta, dtype=np.int32).reshape(-1)
        states = np.ascontiguousarray(states, dtype=np.int32)
        op_keys = np.ascontiguousarray(op_keys, dtype=np.int32).reshape(-1)
        h = _I()
        n = _I64()
        self._check(self.lib.bgpu_block_define(self.h, len(orbsym), _ip(orbsym), group.encode(), len(states),
                                               _ip(quanta), _ip(states), len(op_keys) // 4, _ip(op_keys),
                                               int(is_dot), ctypes.byref(h), ctypes.byref(n)))
        return h.value, n.value

    def block_upload(self, handle, arena):
        arena = np.ascontiguousarray(arena, dtype=np.float64)
        self._check(self.lib.bgpu_block_upload(self.h, handle, _dp(arena), arena.size))

    def block_download(self, handle, n):
        out = np.empty(n, dtype=np.float64)
        self._check(self.lib.bgpu_block_download(self.h, handle, _dp(out), n))
        return out

    def block_set_sites(self, handle, sites):
        sites = np.ascontiguousarray(sites, dtype=np.int32)
        self._check(self.lib.bgpu_block_set_sites(self.h, handle, len(sites), _ip(sites)))

    def block_quanta(self, handle):
        """(quanta as an (n, 3) array of (n, 2S, irrep), states per quantum)."""
        nq = _I(0)
        self._check(self.lib.bgpu_block_quanta(self.h, handle, ctypes.byref(nq), None, None))
        q = np.zeros(3 * nq.value, dtype=np.int32)
        st = np.zeros(nq.value, dtype=np.int32)
        self._check(self.lib.bgpu_block_quanta(self.h, handle, ctypes.byref(nq), _ip(q), _ip(st)))
        return q.reshape(-1, 3), st

    # ---- operator builds and renormalisation (TensorProduct / transform_operators boundary)
    def integrals_load(self, conf_path):
        """Integrals of a dmrg.conf's `orbitals`: (handle, norb)."""
        h, n = _I(), _I()
        self._check(self.lib.bgpu_integrals_load(self.h, conf_path.encode(), ctypes.byref(h), ctypes.byref(n)))
        return h.value, n.value

    def integrals_define(self, orbsym, h1, eri, ecore=0.0):
        orbsym = np.ascontiguousarray(orbsym, dtype=np.int32)
        h1 = np.ascontiguousarray(h1, dtype=np.float64).reshape(-1)
        eri = np.ascontiguousarray(eri, dtype=np.float64).reshape(-1)
        h = _I()
        self._check(self.lib.bgpu_integrals_define(self.h, len(orbsym), _ip(orbsym), _dp(h1), _dp(eri), float(ecore),
                                                   ctypes.byref(h)))
        return h.value

    def integrals_free(self, handle):
        self._check(self.lib.bgpu_integrals_free(self.h, handle))

    def build_enlarged_ops(self, integrals, left, right, op_keys, filt=None):
        """Enlarged block left (x) right with catalogue op_keys; filt =
        (nelec, 2S, norb) of the system or None.  Returns (handle, arena
        doubles, quanta)."""
        op_keys = np.ascontiguousarray(op_keys, dtype=np.int32).reshape(-1)
        f = np.ascontiguousarray(filt, dtype=np.int32) if filt is not None else None
        h, n, nq = _I(), _I64(), _I()
        self._check(self.lib.bgpu_build_enlarged_ops(self.h, integrals, left, right, _ip(f) if f is not None else None,
                                                     len(op_keys) // 4, _ip(op_keys), ctypes.byref(h),
                                                     ctypes.byref(n), ctypes.byref(nq)))
        return h.value, n.value, nq.value

    def diagonalise(self, matrices, vectors=True):
        """Eigenpairs of a list of symmetric matrices on the GPU solver:
        [(eigenvalues ascending, eigenvectors as columns or None)]."""
        dims = np.array([m.shape[0] for m in matrices], dtype=np.int32)
        a = np.concatenate([np.ascontiguousarray(m, dtype=np.float64).reshape(-1) for m in matrices])
        w = np.empty(int(dims.sum()))
        z = np.empty(a.size) if vectors else None
        self._check(self.lib.bgpu_diagonalise(self.h, len(dims), _ip(dims), _dp(a), _dp(w),
                                              _dp(z) if z is not None else None))
        out, oa, ow = [], 0, 0
        for n in dims:
            n = int(n)
            out.append((w[ow:ow + n].copy(), z[oa:oa + n * n].reshape(n, n).copy() if z is not None else None))
            oa += n * n
            ow += n
        return out

    def set_density_noise(self, perturbative=0.0, random=0.0, seed=0):
        """Noise of the following density_eig calls (see bgpu_set_density_noise)."""
        self._check(self.lib.bgpu_set_density_noise(self.h, float(perturbative), float(random), int(seed)))

    def set_wavefunctions(self, sb, vectors):
        v = np.ascontiguousarray(np.atleast_2d(vectors), dtype=np.float64)
        self._check(self.lib.bgpu_set_wavefunctions(self.h, sb, v.shape[0], _dp(v)))

    def density_download(self, n):
        """(rho, eigenvectors) of the last density matrix, n doubles each."""
        rho = np.empty(n, dtype=np.float64)
        vec = np.empty(n, dtype=np.float64)
        self._check(self.lib.bgpu_density_download(self.h, _dp(rho), _dp(vec), n))
        return rho, vec

    def renormalise(self, big, kept, op_keys, rotations=None):
        """U^T big U with kept states per quantum; rotations (concatenated
        states x kept blocks) or None for the last density's eigenvectors.
        Returns (handle, arena doubles, quanta)."""
        kept = np.ascontiguousarray(kept, dtype=np.int32)
        op_keys = np.ascontiguousarray(op_keys, dtype=np.int32).reshape(-1)
        r = np.ascontiguousarray(rotations, dtype=np.float64) if rotations is not None else None
        h, n, nq = _I(), _I64(), _I()
        self._check(self.lib.bgpu_renormalise(self.h, big, _ip(kept), _dp(r) if r is not None else None,
                                              len(op_keys) // 4, _ip(op_keys), ctypes.byref(h), ctypes.byref(n),
                                              ctypes.byref(nq)))
        return h.value, n.value, nq.value

    def rotation_download(self, small, n):
        out = np.empty(n, dtype=np.float64)
        self._check(self.lib.bgpu_rotation_download(self.h, small, _dp(out), n))
        return out

    def superblock_define(self, left, right, target, coef, term_ops, ecore=0.0):
        target = np.ascontiguousarray(target, dtype=np.int32)
        coef = np.ascontiguousarray(coef, dtype=np.float64)
        term_ops = np.ascontiguousarray(term_ops, dtype=np.int32).reshape(-1)
        sb = _I()
        n = _I64()
        self._check(self.lib.bgpu_superblock_define(self.h, left, right, _ip(target), len(coef), _dp(coef),
                                                    _ip(term_ops), float(ecore), ctypes.byref(sb), ctypes.byref(n)))
        return sb.value, n.value

    def prepare_superblock(self, conf_path, partition):
        sb = _I()
        n = _I64()
        self._check(self.lib.bgpu_prepare_superblock(self.h, conf_path.encode(), partition, ctypes.byref(sb),
                                                     ctypes.byref(n)))
        return sb.value, n.value

    def superblock_work(self, sb):
        f = _D()
        b = _D()
        self._check(self.lib.bgpu_superblock_work(self.h, sb, ctypes.byref(f), ctypes.byref(b)))
        return f.value, b.value

    def sigma(self, sb, psi, out=None):
        """sigma = H psi on host arrays; `out` (optional): a contiguous
        float64 array of psi's size that receives sigma (for example a
        page-locked one from host_array)."""
        psi = np.ascontiguousarray(psi, dtype=np.float64)
        if out is None:
            out = np.empty_like(psi)
        elif out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or out.size != psi.size:
            raise ValueError("out must be a contiguous float64 array of psi's size")
        self._check(self.lib.bgpu_sigma(self.h, sb, _dp(psi), _dp(out)))
        return out

    def host_array(self, n):
        """n doubles of page-locked host memory (bgpu_host_alloc) as a numpy
        array; release it with host_free before the context closes."""
        p = _DP()
        self._check(self.lib.bgpu_host_alloc(self.h, int(n), ctypes.byref(p)))
        return np.ctypeslib.as_array(p, shape=(int(n),))

    def host_free(self, arr):
        self._check(self.lib.bgpu_host_free(self.h, _dp(arr)))

    def sigma_device(self, sb, psi_ptr, out_ptr):
        self._check(self.lib.bgpu_sigma_device(self.h, sb, _P(psi_ptr), _P(out_ptr)))

    def sigma_timed(self, sb, psi_ptr, out_ptr, reps):
        """Device-timed products: (total ms, stage-1 ms, stage-2 ms) summed over reps."""
        ms = np.zeros(3)
        self._check(self.lib.bgpu_sigma_timed(self.h, sb, _P(psi_ptr), _P(out_ptr), reps, _dp(ms)))
        return ms

    def sigma_noalloc(self, sb, psi_ptr, out_ptr):
        """FP64 sigma on device buffers using only the library's fixed device
        array for intermediates (no device allocation during the call),
        whatever precision the context is set to."""
        self._check(self.lib.bgpu_sigma_noalloc(self.h, sb, _P(psi_ptr), _P(out_ptr)))

    def superblock_launches(self, sb):
        n = _I()
        self._check(self.lib.bgpu_superblock_launches(self.h, sb, ctypes.byref(n)))
        return n.value

    def hdiag(self, sb, n):
        out = np.empty(n, dtype=np.float64)
        self._check(self.lib.bgpu_hdiag(self.h, sb, _dp(out)))
        return out

    def davidson(self, sb, n, nroots=1, tol=1e-10, max_iter=200, vectors=False):
        e = np.empty(nroots, dtype=np.float64)
        v = np.empty((nroots, n), dtype=np.float64) if vectors else None
        it = _I()
        self._check(self.lib.bgpu_davidson(self.h, sb, nroots, tol, max_iter, _dp(e),
                                           _dp(v) if v is not None else None, ctypes.byref(it)))
        return e, v, it.value

    def density_eig(self, sb, left, nstates, weights):
        w = np.ascontiguousarray(weights, dtype=np.float64)
        out = np.empty(nstates, dtype=np.float64)
        self._check(self.lib.bgpu_density_eig(self.h, sb, int(left), len(w), _dp(w), _dp(out), nstates))
        return out

    def device_alloc(self, n):
        p = _P()
        self._check(self.lib.bgpu_device_alloc(self.h, n, ctypes.byref(p)))
        return p.value

    def device_free(self, p):
        self._check(self.lib.bgpu_device_free(self.h, _P(p)))

    def to_device(self, dst, src):
        src = np.ascontiguousarray(src, dtype=np.float64)
        self._check(self.lib.bgpu_copy_to_device(self.h, _P(dst), _dp(src), src.size))

    def to_host(self, src, n):
        out = np.empty(n, dtype=np.float64)
        self._check(self.lib.bgpu_copy_to_host(self.h, _dp(out), _P(src), n))
        return out

    def profiler_start(self):
        self._check(self.lib.bgpu_profiler_start(self.h))

    def profiler_stop(self):
        self._check(self.lib.bgpu_profiler_stop(self.h))

    INFO_KEYS = ("flops", "bytes", "tc_mma_flops", "tc_phase1_tasks", "tc_phase2_tasks", "tc_phase2_items",
                 "tc_phase2_stage1_items", "tc_split_tiles", "tc_pool_L", "tc_pool_R", "tc_pool_psi",
                 "tc_pool_S", "fp64_stage1_units", "fp64_items", "tc_item_cost", "tc_split", "tc_group",
                 "tc_per_sector", "tc_tuned", "launches", "fp64_scratch", "tc_nb", "tc_stacks",
                 "tc_stacked_items")

    def tc_wait_selftest(self, limit_ms=20.0):
        """Bounded mbarrier wait on a barrier nothing arrives at: returns
        (gave_up, status, waited_ms)."""
        g = np.zeros(1, dtype=np.int32)
        st = np.zeros(1, dtype=np.int32)
        w = np.zeros(1)
        self._check(self.lib.bgpu_tc_wait_selftest(self.h, float(limit_ms), _ip(g), _ip(st), _dp(w)))
        return int(g[0]), int(st[0]), float(w[0])

    def set_guess(self, transform=True):
        """Davidson start of run_dmrg steps: transformed previous wavefunction
        (True) or unit vectors (False)."""
        self._check(self.lib.bgpu_set_guess(self.h, int(bool(transform))))

    def set_spill(self, on=True):
        """run_dmrg keeps the stored blocks that the current step does not
        read in host memory only (True) or all blocks on the device (False)."""
        self._check(self.lib.bgpu_set_spill(self.h, int(bool(on))))

    def set_davidson_graph(self, on=True):
        """Davidson iterations as launches of a captured CUDA graph (True) or
        as the same launches issued one by one (False)."""
        self._check(self.lib.bgpu_set_davidson_graph(self.h, int(bool(on))))

    def set_tc_schedule(self, per_sector=False):
        """Tensor-core sigma as two persistent launches (False) or as the
        per-sector baseline, one launch per sector (True)."""
        self._check(self.lib.bgpu_set_tc_schedule(self.h, int(bool(per_sector))))

    def set_tc_tile_width(self, nb=0):
        """Output-tile width of the tensor-core sigma: 64, 128 or 0 (automatic)."""
        self._check(self.lib.bgpu_set_tc_tile_width(self.h, int(nb)))

    def set_tc_stacking(self, rows=64):
        """Stack the stage-1 products of operator blocks of at most `rows`
        rows (multiple of 8, up to 128) that share a psi block into one
        128-row tensor-core tile; 0 turns stacking off."""
        self._check(self.lib.bgpu_set_tc_stacking(self.h, int(rows)))

    def set_autotune(self, on=True, cache_path=None):
        """Autotuner of the persistent tensor-core schedule, keyed on the
        sector-size histogram; cache_path: text file of tuned knobs."""
        self._check(self.lib.bgpu_set_autotune(self.h, int(bool(on)),
                                               cache_path.encode() if cache_path else None))

    def autotune_stats(self):
        """(histograms tuned, histograms cached, seconds spent tuning)."""
        a, b, c = _I64(), _I64(), ctypes.c_double()
        self._check(self.lib.bgpu_autotune_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def davidson_graph_launches(self):
        """Graph launches of the last Davidson solve."""
        v = _I64()
        self._check(self.lib.bgpu_davidson_graph_launches(self.h, ctypes.byref(v)))
        return v.value

    def set_refinement(self, mode):
        """Split-precision solves: "exact" (FP64-residual defect correction
        with exact-slice tensor-core restart products, the default),
        "defect" (the same with FP64 products) or "energy" (FP64 Rayleigh
        quotients only)."""
        self._check(self.lib.bgpu_set_refinement(self.h, {"energy": 0, "defect": 1, "exact": 2}[mode]))

    def refinement_stats(self):
        """(FP64 restarts, FP64 products, how the last solve was verified:
        0 not, 1 on FP64 residuals, 2 on FP64 residual bounds)."""
        a, b, c = _I64(), _I64(), _I()
        self._check(self.lib.bgpu_refinement_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def onepdm(self, root, norb):
        """Spatial one-particle density matrix of a root from the last
        run_dmrg with the onepdm keyword (norb x norb)."""
        g = np.zeros((norb, norb))
        self._check(self.lib.bgpu_onepdm(self.h, int(root), _dp(g), int(norb)))
        return g

    def transition_onepdm(self, bra, ket, norb):
        """<bra|E_ij|ket> between two roots of the last run_dmrg with the
        onepdm (or tran_onepdm) keyword (norb x norb)."""
        g = np.zeros((norb, norb))
        self._check(self.lib.bgpu_transition_onepdm(self.h, int(bra), int(ket), _dp(g), int(norb)))
        return g

    def set_refine_window(self, eh):
        """FP64 energy refinement window of split-precision sweeps (Eh)."""
        self._check(self.lib.bgpu_set_refine_window(self.h, float(eh)))

    def superblock_info(self, sb):
        """Work-list statistics of one sigma (see bgpu_superblock_info)."""
        v = np.zeros(len(self.INFO_KEYS))
        self._check(self.lib.bgpu_superblock_info(self.h, sb, _dp(v), len(v)))
        return dict(zip(self.INFO_KEYS, v.tolist()))

    def tc_tile(self, a_bits, b_bits, packed=False):
        """d = a * b^T on one tcgen05 tile; a (128 x k) and b (n x k) are
        uint16 arrays of bf16 bit patterns, d is float32 (128 x n).  With
        packed=True the operands are staged through the K-chunk core-matrix
        packing and bulk copies."""
        a = np.ascontiguousarray(a_bits, dtype=np.uint16)
        b = np.ascontiguousarray(b_bits, dtype=np.uint16)
        n, k = b.shape
        if a.shape != (128, k):
            raise ValueError("a must be 128 x k")
        if packed:
            a, b = pack_kmajor(a), pack_kmajor(b)
        d = np.zeros((128, n), dtype=np.float32)
        self._check(self.lib.bgpu_tc_tile(self.h, a.ctypes.data, b.ctypes.data, d.ctypes.data, n, k, int(packed)))
        return d

    def synchronize(self):
        self._check(self.lib.bgpu_synchronize(self.h))

    # ---- full sweep (block.spin_adapted dmrg.conf)
    def run_dmrg(self, conf_path, verbose=0, max_roots=32):
        e = np.zeros(max_roots, dtype=np.float64)
        st = np.zeros(13, dtype=np.float64)
        self._check(self.lib.bgpu_run_dmrg(self.h, conf_path.encode(), verbose, _dp(e), max_roots, _dp(st)))
        nroots = int(st[7])
        stats = dict(sweeps=int(st[0]), sigma_calls=int(st[1]), sigma_seconds=st[2], sigma_flops=st[3],
                     seconds=st[4], discarded=st[5], last_sweep_energy=st[6], build_seconds=st[8],
                     solve_seconds=st[9], density_seconds=st[10], renorm_seconds=st[11],
                     plan_seconds=st[12])
        sw = np.zeros(256)
        ns = _I()
        self._check(self.lib.bgpu_sweep_energies(self.h, _dp(sw), len(sw), ctypes.byref(ns)))
        stats["sweep_energies"] = sw[:min(ns.value, len(sw))].copy()
        nsw = len(stats["sweep_energies"])
        rs = np.zeros(18 + nsw)
        self._check(self.lib.bgpu_run_stats(self.h, _dp(rs), len(rs)))
        stats.update(split_sigma_calls=int(rs[0]), split_sigma_seconds=rs[1], fp64_sigma_calls=int(rs[2]),
                     fp64_sigma_seconds=rs[3], defect_rounds=int(rs[4]), derived_fp64_sigma_seconds=rs[5],
                     warmup_seconds=rs[6], bounded_verifications=int(rs[7]), exact_sigma_calls=int(rs[8]),
                     exact_sigma_seconds=rs[9], sweep_renorm_flops=rs[10], fp64_rate=rs[11],
                     renorm_exact=bool(rs[12]), sweep_renorm_device_seconds=rs[13],
                     spill_fetches=int(rs[14]), spill_bytes_up=rs[15], spill_bytes_down=rs[16],
                     peak_block_bytes=rs[17], sweep_seconds=rs[18:18 + nsw].copy())
        return e[:nroots].copy(), stats
