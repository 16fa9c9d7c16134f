"""sfci_gb300 — GB300-native truncated-Krylov hot path of SFCI.

Python mirror of the reference's operator interface, over the C ABI of
``libsfci_gb300.so`` (``include/sfci_gb300.h``):

* :class:`Context` — integrals + options; ``SpMVMtply_bucket`` (src/functions.cpp:511),
  ``calc_energy`` (:1272), ``DiagCal_bit`` (src/bitstr.cpp:433),
  ``sparse_krylov_solve_eigenval`` (src/sparse_solver.cpp:246), ``minres_sp``
  (src/minres.cpp:73), ``calc_CISD`` (src/sparse_solver.cpp:15), ``fci``
  (src/dense_algo.cpp:77);
* :class:`SpVec` — a device-resident ``dynVec`` (src/all.h:150) with the
  reference's method names (``dot``, ``addTwo``, ``addThree``, ``shrinkFrom``,
  ``norm``, ``normalize``, ``scalarMtply``, ``naiveCopy``, ``setZeroVec``).

Keys are numpy ``uint64`` arrays: shape ``(n,)`` for up to 64 spin orbitals,
``(n, 2)`` (low word first) for up to 128.  There is no CPU fallback: if the
library is missing or its CUDA calls fail, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

__all__ = ["Context", "SpVec", "SfciError", "load_library", "gsaes", "keys_from_ints", "ints_from_keys"]


class SfciError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (status, msg))
        self.status = status


_LIB = None


class Opts(C.Structure):
    _fields_ = [("Nd", C.c_uint64), ("hpsi_cap", C.c_uint64), ("coeff_cut", C.c_double),
                ("bucket_unit", C.c_uint64), ("mem_budget", C.c_uint64), ("verbose", C.c_int),
                ("reserved", C.c_int * 7)]


_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_vp = C.c_void_p


def _sigs(L):
    L.sfci_last_error.restype = C.c_char_p
    L.sfci_status_name.restype = C.c_char_p
    L.sfci_status_name.argtypes = [C.c_int]
    L.sfci_ctx_create.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(Opts), C.POINTER(_vp)]
    L.sfci_ctx_destroy.argtypes = [_vp]
    L.sfci_key_words.argtypes = [_vp]
    L.sfci_ctx_stream.argtypes = [_vp, C.POINTER(_vp)]
    L.sfci_ctx_set_nd.argtypes = [_vp, C.c_uint64]
    L.sfci_ctx_trim.argtypes = [_vp]
    L.sfci_ctx_launch_count.argtypes = [_vp, C.POINTER(C.c_uint64)]
    L.sfci_ctx_event_record.argtypes = [_vp, C.c_int]
    L.sfci_ctx_event_elapsed.argtypes = [_vp, C.c_int, C.c_int, C.POINTER(C.c_float)]
    L.sfci_ctx_profile.argtypes = [_vp, C.c_int]
    L.sfci_ctx_profile_read.argtypes = [_vp, C.c_char_p, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
    L.sfci_ctx_profile_reset.argtypes = [_vp]
    L.sfci_ctx_last_stats.argtypes = [_vp, C.POINTER(C.c_uint64)]
    L.sfci_vec_create.argtypes = [_vp, C.c_uint64, C.POINTER(_vp)]
    L.sfci_vec_destroy.argtypes = [_vp]
    L.sfci_vec_len.argtypes = [_vp, C.POINTER(C.c_uint64)]
    L.sfci_vec_cap.argtypes = [_vp, C.POINTER(C.c_uint64)]
    L.sfci_vec_upload.argtypes = [_vp, _vp, _vp, C.c_uint64]
    L.sfci_vec_download.argtypes = [_vp, _vp, _vp, C.c_uint64, C.POINTER(C.c_uint64)]
    L.sfci_vec_copy.argtypes = [_vp, _vp]
    L.sfci_vec_clear.argtypes = [_vp]
    L.sfci_spmspv.argtypes = [_vp, _vp, _vp, C.c_double, C.c_double, C.POINTER(C.c_double)]
    L.sfci_diag_elements.argtypes = [_vp, _vp, C.c_uint64, _vp]
    L.sfci_energy.argtypes = [_vp, _vp, C.POINTER(C.c_double)]
    L.sfci_dot.argtypes = [_vp, _vp, _vp, C.POINTER(C.c_double)]
    L.sfci_norm.argtypes = [_vp, _vp, C.POINTER(C.c_double)]
    L.sfci_scale.argtypes = [_vp, _vp, C.c_double]
    L.sfci_normalize.argtypes = [_vp, _vp]
    L.sfci_add_two.argtypes = [_vp, _vp, _vp, C.c_double]
    L.sfci_add_three.argtypes = [_vp, _vp, _vp, _vp, _vp, C.c_double, C.c_double, C.c_double]
    L.sfci_shrink_from.argtypes = [_vp, _vp, _vp]
    L.sfci_combine.argtypes = [_vp, _vp, C.POINTER(_vp), _vp, C.c_int]
    L.sfci_lanczos_ground.argtypes = [_vp, _vp, C.c_int, C.c_int, _vp, C.POINTER(C.c_double)]
    L.sfci_minres.argtypes = [_vp, _vp, _vp, _vp, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_int)]
    L.sfci_gsaes.argtypes = [C.c_int, _vp, _vp, _vp, _vp]
    L.sfci_vec_save.argtypes = [_vp, C.c_char_p]
    L.sfci_vec_load.argtypes = [_vp, C.c_char_p]
    L.sfci_psi_write.argtypes = [_vp, _vp, C.c_uint64, C.c_int, C.c_char_p]
    L.sfci_psi_read.argtypes = [C.c_char_p, C.c_int, C.c_int, _vp, _vp, C.c_uint64, C.POINTER(C.c_uint64)]
    L.sfci_cisd.argtypes = [_vp, _vp, C.c_int, C.c_int, _vp, _vp, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
    L.sfci_fci.argtypes = [_vp, C.c_int, _vp, _vp, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
    L.sfci_spmspv_linear.argtypes = [_vp, _vp, _vp, C.c_double, C.POINTER(_vp), C.c_int, _vp]
    L.sfci_res_norm.argtypes = [_vp, _vp, _vp, _vp, C.c_double, C.POINTER(C.c_double)]
    L.sfci_krylov_linear.argtypes = [_vp, _vp, _vp, C.c_double, C.c_int, C.c_int, _vp]
    L.sfci_shift_invert.argtypes = [_vp, _vp, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_double)]
    _u64p = C.POINTER(C.c_uint64)
    L.sfci_batch_create.argtypes = [C.c_int, C.POINTER(C.c_char_p), _vp, _vp, C.POINTER(Opts), C.POINTER(_vp)]
    L.sfci_batch_lanczos.argtypes = [_vp, C.POINTER(_vp), C.c_int, C.c_int, C.c_int, _vp, _vp]
    L.sfci_ctx_set_tuning.argtypes = [_vp, _vp]
    L.sfci_ctx_set_class_passes.argtypes = [_vp, C.c_int]
    L.sfci_ctx_get_tuning.argtypes = [_vp, _vp]
    L.sfci_autotune.argtypes = [_vp, _vp, _vp, _vp, C.POINTER(C.c_double)]
    L.sfci_screen_create.argtypes = [_vp, C.c_uint64, C.POINTER(_vp)]
    L.sfci_screen_destroy.argtypes = [_vp]
    L.sfci_screen_log.argtypes = [_vp, _vp, _vp, C.c_double, _u64p, _u64p]
    L.sfci_screen_train.argtypes = [_vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_double)]
    L.sfci_screen_stats.argtypes = [_vp, _u64p, _u64p, _u64p, _u64p]
    L.sfci_screen_predict.argtypes = [_vp, _vp, C.c_double, _u64p, _u64p, _u64p, _vp, C.c_uint64]
    L.sfci_screen_param_count.restype = C.c_uint64
    L.sfci_screen_params.argtypes = [_vp, _vp, _vp, C.c_uint64]
    L.sfci_screen_grads.argtypes = [_vp, _vp, C.c_uint64]
    L.sfci_ctx_set_screen.argtypes = [_vp, _vp, C.c_double]
    L.sfci_ctx_set_screen_guard.argtypes = [_vp, C.c_double]
    L.sfci_ctx_set_screen_floor.argtypes = [_vp, C.c_double]
    L.sfci_ctx_screen_stats.argtypes = [_vp, _u64p]
    return L


def load_library(path: str | None = None, build: bool = True):
    """Load libsfci_gb300.so (building it in-tree first when ``build``)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = path or os.environ.get("SFCI_GB300_LIB")
    if p is None:
        p = _build.build() if build else _build.LIB
    if not os.path.exists(p):
        raise ImportError("libsfci_gb300.so not found at %s; run sfci_gb300.build.build()" % p)
    L = C.CDLL(p)
    for fn in ("sfci_ctx_create", "sfci_last_error", "sfci_status_name", "sfci_ctx_destroy", "sfci_key_words",
               "sfci_ctx_stream", "sfci_ctx_set_nd", "sfci_ctx_launch_count", "sfci_ctx_event_record",
               "sfci_ctx_event_elapsed", "sfci_ctx_profile", "sfci_ctx_profile_read", "sfci_ctx_profile_reset",
               "sfci_ctx_last_stats", "sfci_vec_create", "sfci_vec_destroy", "sfci_vec_len", "sfci_vec_cap",
               "sfci_vec_upload", "sfci_vec_download", "sfci_vec_copy", "sfci_vec_clear", "sfci_spmspv",
               "sfci_diag_elements", "sfci_energy", "sfci_dot", "sfci_norm", "sfci_scale", "sfci_normalize",
               "sfci_add_two", "sfci_add_three", "sfci_shrink_from", "sfci_combine", "sfci_lanczos_ground",
               "sfci_minres", "sfci_gsaes", "sfci_cisd", "sfci_fci", "sfci_spmspv_linear", "sfci_res_norm",
               "sfci_krylov_linear", "sfci_shift_invert", "sfci_screen_create", "sfci_screen_train",
               "sfci_ctx_set_screen", "sfci_ctx_set_screen_guard", "sfci_ctx_set_screen_floor"):
        getattr(L, fn)
    _LIB = _sigs(L)
    return _LIB


def _check(st):
    if st != 0:
        L = _LIB
        raise SfciError(L.sfci_status_name(st).decode(), L.sfci_last_error().decode())


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None and a.size else None


def keys_from_ints(ints, words: int) -> np.ndarray:
    """Python ints (determinant bitstrings) -> key array for ``words`` words."""
    ints = [int(x) for x in ints]
    if words == 1:
        return np.array(ints, dtype=np.uint64)
    a = np.zeros((len(ints), 2), dtype=np.uint64)
    m = (1 << 64) - 1
    for i, x in enumerate(ints):
        a[i, 0] = x & m
        a[i, 1] = x >> 64
    return a


def ints_from_keys(keys: np.ndarray):
    keys = np.asarray(keys, dtype=np.uint64)
    if keys.ndim == 1:
        return [int(x) for x in keys]
    return [int(lo) | (int(hi) << 64) for lo, hi in keys]


def gsaes(K, S):
    """FP64 generalised symmetric eigensolve K c = E S c (ascending, S-orthonormal)."""
    L = load_library()
    K = np.asfortranarray(np.asarray(K, dtype=np.float64))
    S = np.asfortranarray(np.asarray(S, dtype=np.float64))
    n = K.shape[0]
    ev = np.zeros(n)
    X = np.zeros((n, n), order="F")
    _check(L.sfci_gsaes(n, K.ctypes.data_as(C.c_void_p), S.ctypes.data_as(C.c_void_p),
                        ev.ctypes.data_as(C.c_void_p), X.ctypes.data_as(C.c_void_p)))
    return ev, X


def psi_write(path: str, keys, amps, key_words: int = 1):
    """Write a restart-vector file from host arrays (no GPU): the length, then
    "key amplitude" lines, keys in decimal, amplitudes with 12 significant digits."""
    L = load_library()
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    amps = np.ascontiguousarray(amps, dtype=np.float64)
    _check(L.sfci_psi_write(_ptr(keys), _ptr(amps), len(amps), int(key_words), os.fsencode(path)))


def psi_read(path: str, num_orb: int, key_words: int = 1):
    """Read a restart-vector file into host arrays (no GPU); keys are checked
    against num_orb.  Returns (keys, amps), keys of shape (n, 2) for two words."""
    L = load_library()
    n = C.c_uint64()
    _check(L.sfci_psi_read(os.fsencode(path), int(key_words), int(num_orb), None, None, 0, C.byref(n)))
    keys = np.zeros((n.value, 2) if key_words == 2 else n.value, dtype=np.uint64)
    amps = np.zeros(n.value)
    _check(L.sfci_psi_read(os.fsencode(path), int(key_words), int(num_orb), _ptr(keys), _ptr(amps), n.value,
                           C.byref(n)))
    return keys, amps



INST_SHIFT = 59  # instance tag: the top five bits of a batched context's two-word keys


def tag_keys(keys, inst: int):
    """Two-word keys (n, 2) of batched instance `inst` (bits 123..127 of the key).
    ValueError for an instance outside 0..31 or a key that already sets one of
    the tag bits."""
    inst = int(inst)
    if not 0 <= inst < 32:
        raise ValueError("batched instance %d outside 0..31" % inst)
    k = np.array(keys, dtype=np.uint64, copy=True).reshape(-1, 2)
    if k.size and np.any(k[:, 1] >> np.uint64(INST_SHIFT)):
        raise ValueError("keys already use the instance bits 123..127")
    k[:, 1] |= np.uint64(inst << INST_SHIFT)
    return k


class Context:
    """Integrals + options + one CUDA stream (the reference's global state, made explicit)."""

    def __init__(self, in_path: str, num_orb: int, num_e: int, Nd: int = 200000, hpsi_cap: int = 60000000,
                 coeff_cut: float = 1e-5, mem_budget: int = 0, verbose: bool = False, _batch=None):
        self.L = load_library()
        o = Opts()
        o.Nd = int(Nd)
        o.hpsi_cap = int(hpsi_cap)
        o.coeff_cut = float(coeff_cut)
        o.mem_budget = int(mem_budget)
        o.verbose = 1 if verbose else 0
        h = _vp()
        if _batch is None:
            _check(self.L.sfci_ctx_create(in_path.encode(), int(num_orb), int(num_e), C.byref(o), C.byref(h)))
        else:
            paths, orbs, nes = _batch
            n = len(paths)
            pa = (C.c_char_p * n)(*[p.encode() for p in paths])
            oa = np.ascontiguousarray(orbs, np.int32)
            ea = np.ascontiguousarray(nes, np.int32)
            _check(self.L.sfci_batch_create(n, pa, _ptr(oa), _ptr(ea), C.byref(o), C.byref(h)))
            self.instances = n
        self.h = h
        self.num_orb, self.num_e = num_orb, num_e
        self.words = self.L.sfci_key_words(h)
        self.Nd = int(Nd)
        self.hpsi_cap = int(hpsi_cap)

    @classmethod
    def batch(cls, in_paths, num_orbs, num_es, Nd: int = 200000, hpsi_cap: int = 60000000, **kw):
        """A batched context: one Hamiltonian per instance (<= 32 instances, <= 120 spin
        orbitals each); keys carry their instance in their top bits (tag_keys).
        In batch_lanczos, hpsi_cap caps each instance's products, as in its own run."""
        return cls(None, 128, max(num_es), Nd=Nd, hpsi_cap=hpsi_cap, _batch=(list(in_paths), num_orbs, num_es), **kw)

    def batch_lanczos(self, vecs, Nl: int, num_restart: int):
        """sparse_krylov_solve_eigenval on every instance, one batched product per Krylov step."""
        n = len(vecs)
        arr = (_vp * n)(*[v.h for v in vecs])
        en = np.full(n * num_restart, np.nan)
        fe = np.zeros(n)
        _check(self.L.sfci_batch_lanczos(self.h, arr, n, int(Nl), int(num_restart), _ptr(en), _ptr(fe)))
        return en.reshape(n, num_restart), fe

    def tuning(self):
        t = np.zeros(4, np.int32)
        _check(self.L.sfci_ctx_get_tuning(self.h, _ptr(t)))
        return dict(zip(["l1_bits", "digit_bits", "leaf_keys", "gen_ctas_per_sm"], [int(x) for x in t]))

    def set_tuning(self, l1_bits=9, digit_bits=9, leaf_keys=120, gen_ctas_per_sm=2):
        t = np.array([l1_bits, digit_bits, leaf_keys, gen_ctas_per_sm], np.int32)
        _check(self.L.sfci_ctx_set_tuning(self.h, _ptr(t)))

    def set_class_passes(self, mode: int):
        """Generation passes by target alpha class: 0 when needed, 1 always, -1 never."""
        _check(self.L.sfci_ctx_set_class_passes(self.h, int(mode)))

    def autotune(self, vin: "SpVec", vout: "SpVec"):
        """Time the candidate product plans on vin and keep the fastest (results never depend on the plan)."""
        t = np.zeros(4, np.int32)
        ms = C.c_double()
        _check(self.L.sfci_autotune(self.h, vin.h, vout.h, _ptr(t), C.byref(ms)))
        return dict(zip(["l1_bits", "digit_bits", "leaf_keys", "gen_ctas_per_sm"], [int(x) for x in t])), ms.value

    def close(self):
        if getattr(self, "h", None):
            self.L.sfci_ctx_destroy(self.h)
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

    # --- vectors
    def vec(self, cap: int) -> "SpVec":
        return SpVec(self, cap)

    def vec_from(self, keys, amps, cap: int | None = None) -> "SpVec":
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        amps = np.ascontiguousarray(amps, dtype=np.float64)
        v = SpVec(self, cap if cap is not None else max(1, len(amps)))
        v.upload(keys, amps)
        return v

    def trim(self):
        """Free the device scratch this context's products keep between calls."""
        _check(self.L.sfci_ctx_trim(self.h))

    def set_Nd(self, Nd: int):
        _check(self.L.sfci_ctx_set_nd(self.h, int(Nd)))
        self.Nd = int(Nd)

    # --- hot path (reference names)
    def SpMVMtply_bucket(self, vin: "SpVec", vout: "SpVec", lam: float, coeff: float, diag: float = 0.0) -> float:
        d = C.c_double(diag)
        _check(self.L.sfci_spmspv(self.h, vin.h, vout.h, float(lam), float(coeff), C.byref(d)))
        return d.value

    spmspv = SpMVMtply_bucket

    def calc_energy(self, psi: "SpVec") -> float:
        e = C.c_double()
        _check(self.L.sfci_energy(self.h, psi.h, C.byref(e)))
        return e.value

    def DiagCal_bit(self, keys) -> np.ndarray:
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        n = keys.shape[0]
        out = np.zeros(n)
        _check(self.L.sfci_diag_elements(self.h, _ptr(keys), n, _ptr(out)))
        return out

    def sparse_krylov_solve_eigenval(self, v: "SpVec", Nl: int, num_restart: int):
        en = np.full(num_restart, np.nan)
        fe = C.c_double()
        _check(self.L.sfci_lanczos_ground(self.h, v.h, int(Nl), int(num_restart), _ptr(en), C.byref(fe)))
        return en, fe.value

    def minres_sp(self, rhs: "SpVec", guess: "SpVec", result: "SpVec", iters: int, tol: float, lam: float) -> int:
        done = C.c_int()
        _check(self.L.sfci_minres(self.h, rhs.h, guess.h, result.h, int(iters), float(tol), float(lam),
                                  C.byref(done)))
        return done.value

    def calc_CISD(self, ref_det, state_idx: int = 0, n_evals: int = 10):
        """calc_CISD (src/sparse_solver.cpp:15-114): eigenvector ``state_idx`` of H on
        the block of ``ref_det`` and every determinant it connects to, keys
        ascending, largest component positive.  Returns (SpVec, the n_evals lowest
        eigenvalues, norm of the residual H x - E x)."""
        key = keys_from_ints([int(ref_det)], self.words).reshape(-1)
        occ = [b for b in range(self.num_orb) if int(ref_det) >> b & 1]
        M = self.num_orb // 2
        na = sum(1 for b in occ if b % 2 == 0)
        nb = len(occ) - na
        c2 = lambda x: x * (x - 1) // 2
        size = (1 + na * (M - na) + nb * (M - nb) + c2(na) * c2(M - na) + c2(nb) * c2(M - nb)
                + na * (M - na) * nb * (M - nb))
        out = SpVec(self, max(1, size))
        ev = np.full(max(0, int(n_evals)), np.nan)
        r = C.c_double()
        bs = C.c_uint64()
        _check(self.L.sfci_cisd(self.h, _ptr(key), int(state_idx), int(n_evals), _ptr(ev), out.h, C.byref(r),
                                C.byref(bs)))
        return out, ev, r.value

    def fci(self, n_evals: int = 1, ground: bool = True):
        """fci (src/dense_algo.cpp:77-124): the n_evals lowest eigenvalues of H on
        every determinant with num_e/2 electrons of each spin.  Returns (eigenvalues,
        ground state as an SpVec or None, residual norm of the ground state)."""
        import math
        n = math.comb(self.num_orb // 2, self.num_e // 2) ** 2
        g = SpVec(self, max(1, n)) if ground else None
        ev = np.full(max(0, int(n_evals)), np.nan)
        r = C.c_double()
        d = C.c_uint64()
        _check(self.L.sfci_fci(self.h, int(n_evals), _ptr(ev), g.h if g is not None else None, C.byref(r),
                               C.byref(d)))
        return ev, g, r.value

    def spmspvm_bucket_linear(self, vin: "SpVec", vout: "SpVec", lam: float, basis) -> np.ndarray:
        """spmspvm_bucket_linear (src/functions.cpp:858): returns Hij[0..len(basis))."""
        arr = (_vp * len(basis))(*[v.h for v in basis])
        h = np.zeros(len(basis))
        _check(self.L.sfci_spmspv_linear(self.h, vin.h, vout.h, float(lam), arr, len(basis), _ptr(h)))
        return h

    def spmspvm_bucket_res_norm(self, x: "SpVec", r: "SpVec", b: "SpVec", lam: float) -> float:
        """spmspvm_bucket_res_norm (src/functions.cpp:1096): r = cut, capped A x - b;
        returns |A x - b| before the cut."""
        res = C.c_double()
        _check(self.L.sfci_res_norm(self.h, x.h, r.h, b.h, float(lam), C.byref(res)))
        return res.value

    def sparse_krylov_solve_linear(self, b: "SpVec", result: "SpVec", target_energy: float, num_iter: int,
                                   num_restart: int) -> np.ndarray:
        """sparse_krylov_solve_linear (src/sparse_solver.cpp:561): returns |A x - b| per restart."""
        res = np.zeros(int(num_restart))
        _check(self.L.sfci_krylov_linear(self.h, b.h, result.h, float(target_energy), int(num_iter), int(num_restart),
                                         _ptr(res)))
        return res

    def sparse_solve_SI(self, b: "SpVec", target_energy: float, num_iter: int, num_restart: int) -> float:
        """sparse_solve_SI (src/sparse_solver.cpp:732): b becomes the normalised
        shift-invert iterate; returns its energy."""
        e = C.c_double()
        _check(self.L.sfci_shift_invert(self.h, b.h, float(target_energy), int(num_iter), int(num_restart),
                                        C.byref(e)))
        return e.value

    def combine(self, dst: "SpVec", vecs, coef):
        coef = np.ascontiguousarray(coef, dtype=np.float64)
        arr = (_vp * len(vecs))(*[v.h for v in vecs])
        _check(self.L.sfci_combine(self.h, dst.h, arr, _ptr(coef), len(vecs)))

    # --- instrumentation
    def launches(self) -> int:
        n = C.c_uint64()
        _check(self.L.sfci_ctx_launch_count(self.h, C.byref(n)))
        return n.value

    def stream(self) -> int:
        s = _vp()
        _check(self.L.sfci_ctx_stream(self.h, C.byref(s)))
        return s.value or 0

    def event_record(self, slot: int):
        _check(self.L.sfci_ctx_event_record(self.h, int(slot)))

    def event_elapsed(self, a: int, b: int) -> float:
        ms = C.c_float()
        _check(self.L.sfci_ctx_event_elapsed(self.h, int(a), int(b), C.byref(ms)))
        return ms.value

    def profile(self, enable: bool = True):
        _check(self.L.sfci_ctx_profile(self.h, 1 if enable else 0))

    def profile_read(self) -> dict:
        out = {}
        for ph in ("count", "scatter", "partition", "merge", "select", "sort", "other"):
            ms = C.c_double()
            n = C.c_uint64()
            _check(self.L.sfci_ctx_profile_read(self.h, ph.encode(), C.byref(ms), C.byref(n)))
            out[ph] = (ms.value, n.value)
        return out

    def profile_reset(self):
        _check(self.L.sfci_ctx_profile_reset(self.h))

    def last_stats(self) -> dict:
        a = (C.c_uint64 * 8)()
        _check(self.L.sfci_ctx_last_stats(self.h, a))
        names = ["input_dets", "terms", "unique", "survivors", "out_len", "passes", "leaves", "big_leaves"]
        return dict(zip(names, [int(x) for x in a]))

    # learned excitation screen
    def set_screen(self, screen: "Screen | None", threshold: float = 0.5, guard: float = 0.0, floor: float = 0.0):
        """Screen this context's products (None: plain products).  A group whose
        largest possible term |c_j| * max|V| reaches `guard` is always kept, one
        below `floor` is skipped without the network (0: neither)."""
        _check(self.L.sfci_ctx_set_screen(self.h, screen.h if screen is not None else None, float(threshold)))
        _check(self.L.sfci_ctx_set_screen_guard(self.h, float(guard)))
        _check(self.L.sfci_ctx_set_screen_floor(self.h, float(floor)))
        self._screen = screen

    def screen_stats(self) -> dict:
        a = (C.c_uint64 * 5)()
        _check(self.L.sfci_ctx_screen_stats(self.h, a))
        return dict(zip(["groups", "kept_groups", "kept_terms", "products", "all_terms"], [int(x) for x in a]))


class Screen:
    """Learned excitation screen: a BF16 MLP on the tensor cores predicting which
    term groups of a product survive its cut (see include/sfci_gb300.h)."""

    def __init__(self, ctx: Context, seed: int = 1):
        self.ctx = ctx
        self.L = ctx.L
        h = _vp()
        _check(self.L.sfci_screen_create(ctx.h, int(seed), C.byref(h)))
        self.h = h
        self.nparam = int(self.L.sfci_screen_param_count())

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.L.sfci_screen_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def log(self, vin: "SpVec", vout: "SpVec", min_term: float = 0.0):
        """Label the groups of vin's determinants by vout (the product of vin): alive when
        a term of magnitude above min_term lands on a determinant of vout."""
        ne, npos = C.c_uint64(), C.c_uint64()
        _check(self.L.sfci_screen_log(self.h, vin.h, vout.h, float(min_term), C.byref(ne), C.byref(npos)))
        return ne.value, npos.value

    def train(self, steps: int, batch_tiles: int = 64, lr: float = 1e-3, pos_weight: float = 1.0,
              sequential: bool = False) -> float:
        loss = C.c_double()
        _check(self.L.sfci_screen_train(self.h, int(steps), int(batch_tiles), float(lr), float(pos_weight),
                                        1 if sequential else 0, C.byref(loss)))
        return loss.value

    def stats(self) -> dict:
        a = [C.c_uint64() for _ in range(4)]
        _check(self.L.sfci_screen_stats(self.h, *[C.byref(x) for x in a]))
        return dict(zip(["sources", "examples", "positives", "steps"], [x.value for x in a]))

    def predict(self, vin: "SpVec", threshold: float = 0.5, probs: bool = False):
        g, kg, kt = C.c_uint64(), C.c_uint64(), C.c_uint64()
        buf = None
        cap = 0
        if probs:
            cap = self.groups_of(vin)
            buf = np.zeros(max(cap, 1), np.float32)
        _check(self.L.sfci_screen_predict(self.h, vin.h, float(threshold), C.byref(g), C.byref(kg), C.byref(kt),
                                          _ptr(buf) if probs else None, cap))
        out = {"groups": g.value, "kept_groups": kg.value, "kept_terms": kt.value}
        if probs:
            out["prob"] = buf[: g.value]
        return out

    def groups_of(self, vin: "SpVec") -> int:
        g, kg, kt = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(self.L.sfci_screen_predict(self.h, vin.h, 0.5, C.byref(g), C.byref(kg), C.byref(kt), None, 0))
        return g.value

    def params(self) -> np.ndarray:
        a = np.zeros(self.nparam, np.float32)
        _check(self.L.sfci_screen_params(self.h, _ptr(a), None, self.nparam))
        return a

    def set_params(self, a):
        a = np.ascontiguousarray(a, np.float32)
        _check(self.L.sfci_screen_params(self.h, None, _ptr(a), self.nparam))

    def grads(self) -> np.ndarray:
        a = np.zeros(self.nparam, np.float32)
        _check(self.L.sfci_screen_grads(self.h, _ptr(a), self.nparam))
        return a


class SpVec:
    """Device-resident sparse vector (dynVec): keys ascending, FP64 amplitudes."""

    def __init__(self, ctx: Context, cap: int):
        self.ctx = ctx
        self.L = ctx.L
        h = _vp()
        _check(self.L.sfci_vec_create(ctx.h, int(cap), C.byref(h)))
        self.h = h
        self.cap = int(cap)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.L.sfci_vec_destroy(self.h)
                self.h = None
        except Exception:
            pass

    @property
    def len(self) -> int:
        n = C.c_uint64()
        _check(self.L.sfci_vec_len(self.h, C.byref(n)))
        return n.value

    def __len__(self):
        return self.len

    def upload(self, keys, amps):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        amps = np.ascontiguousarray(amps, dtype=np.float64)
        if self.ctx.words == 2 and keys.ndim != 2:
            raise ValueError("128-bit keys need shape (n, 2)")
        _check(self.L.sfci_vec_upload(self.h, _ptr(keys), _ptr(amps), len(amps)))
        return self

    def download(self):
        n = self.len
        w = self.ctx.words
        keys = np.zeros((n, 2) if w == 2 else n, dtype=np.uint64)
        amps = np.zeros(n)
        got = C.c_uint64()
        _check(self.L.sfci_vec_download(self.h, _ptr(keys), _ptr(amps), n, C.byref(got)))
        return keys, amps

    # restart-vector text file, wf_self_as_guess.out format (src/minres.cpp:59-70, src/main.cpp:288-307)
    def writePsi(self, path: str):
        _check(self.L.sfci_vec_save(self.h, os.fsencode(path)))

    def readPsi(self, path: str):
        _check(self.L.sfci_vec_load(self.h, os.fsencode(path)))
        return self

    # dynVec method names (src/all.h)
    def naiveCopy(self, src: "SpVec"):
        _check(self.L.sfci_vec_copy(self.h, src.h))

    def setZeroVec(self):
        _check(self.L.sfci_vec_clear(self.h))

    def dot(self, other: "SpVec") -> float:
        d = C.c_double()
        _check(self.L.sfci_dot(self.ctx.h, self.h, other.h, C.byref(d)))
        return d.value

    def norm(self) -> float:
        d = C.c_double()
        _check(self.L.sfci_norm(self.ctx.h, self.h, C.byref(d)))
        return d.value

    def scalarMtply(self, a: float):
        _check(self.L.sfci_scale(self.ctx.h, self.h, float(a)))

    def normalize(self):
        _check(self.L.sfci_normalize(self.ctx.h, self.h))

    def addTwo(self, w: "SpVec", a: float):
        _check(self.L.sfci_add_two(self.ctx.h, self.h, w.h, float(a)))

    def addThree(self, x: "SpVec", y: "SpVec", z: "SpVec", a: float, b: float, c: float):
        _check(self.L.sfci_add_three(self.ctx.h, self.h, x.h, y.h, z.h, float(a), float(b), float(c)))

    def shrinkFrom(self, src: "SpVec"):
        _check(self.L.sfci_shrink_from(self.ctx.h, self.h, src.h))
