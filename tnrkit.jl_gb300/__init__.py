"""GB300-native coarse-graining engine with TNRKit.jl's API (host side, Python).

Mirrors the reference's user-facing interface for the hot path:

    T = classical_ising()                 # src/models/ising.jl
    scheme = BTRG(T)                      # src/schemes/btrg.jl
    data = run(scheme, truncrank(16), maxiter(25))      # run! (tnrscheme.jl:33-59)
    f = free_energy(data, ising_βc)       # src/utility/free_energy.jl

Schemes: TRG, BTRG, HOTRG, HOTRG_3D (the hot path), ATRG, ATRG_3D, ImpurityHOTRG,
ImpurityTRG and CorrelationHOTRG.  Stopping criteria: maxiter, convcrit, trivial_convcrit
and ``a & b``.  Finalizers: the default one, two_by_two_Finalizer, and the fixed-point
functions cft_data, ground_state_degeneracy, gu_wen_ratio and central_charge.

Every step runs as sm_103a CUDA inside ``libtnr_gb300.so`` behind the C ABI of
``include/tnr_gb300.h``; the tensor stays resident in GPU memory between calls.
There is no CPU fallback: without the library or a GPU the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from .models import (SymTensor, classical_clock, classical_ising, classical_ising_3D, classical_ising_impurity,  # noqa: F401
                     classical_potts, f_onsager, ising_beta_c, ising_beta_c_3D, ising_βc, ising_βc_3D, phi4_complex, phi4_real,
                     phi4_real_imp1, phi4_real_imp2, potts_beta_c, potts_βc, random_hotrg_tensor, sixvertex)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("TNR_GB300_LIB") or os.path.join(HERE, "libtnr_gb300.so")

(TNR_TRG, TNR_BTRG, TNR_HOTRG, TNR_HOTRG_3D, TNR_IMPURITY_HOTRG, TNR_IMPURITY_TRG, TNR_CORRELATION_HOTRG, TNR_ATRG,
 TNR_ATRG_3D) = range(1, 10)
PREC_F64, PREC_SPLIT = 0, 1
STATUS = {0: "ok", 1: "invalid argument", 2: "out of device memory", 3: "iteration cap reached",
          4: "CUDA error", 5: "admission refused", 6: "non-finite value", 7: "unsupported", 8: "no device"}

EXPORTS = ["tnr_default_options", "tnr_create", "tnr_create_device", "tnr_step", "tnr_finalize", "tnr_run",
           "tnr_free_energy", "tnr_get_tensor", "tnr_singular_values", "tnr_truncation_errors", "tnr_btrg_bonds",
           "tnr_device_bytes", "tnr_decomposition_stats", "tnr_destroy", "tnr_last_error", "tnr_status_string", "tnr_timer_start",
           "tnr_timer_stop", "tnr_run_batch", "tnr_device_info", "tnr_version", "tnr_kernel_launches",
           "tnr_profile_enable", "tnr_profile_reset", "tnr_profile_read", "tnr_debug_gemm", "tnr_gemm_time",
           "tnr_gemm_split_noalloc", "tnr_server_create", "tnr_server_submit", "tnr_server_submit_sym",
           "tnr_server_poll", "tnr_debug_chol",
           "tnr_server_stats", "tnr_server_destroy", "tnr_footprint_bytes", "tnr_create_impurity_hotrg",
           "tnr_create_impurity_trg", "tnr_finalize_impurity", "tnr_run_impurity", "tnr_create_correlation_hotrg",
           "tnr_run_correlation", "tnr_correlation_ratio", "tnr_set_finalizer", "tnr_transfer_eigvals",
           "tnr_gu_wen_ratio", "tnr_central_charge", "tnr_get_impurity_tensor"]


class TNRError(RuntimeError):
    """A non-zero status from the C ABI (the reference raises a Julia exception here)."""

    def __init__(self, status, msg):
        super().__init__("%s (status %d): %s" % (STATUS.get(status, "?"), status, msg))
        self.status = status


class Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("btrg_k", C.c_double), ("symmetry_n", C.c_int),
                ("leg_charges", C.POINTER(C.c_int32)), ("seed", C.c_uint64), ("stream", C.c_void_p)]


_lib = None


def lib():
    """Load the in-tree shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libtnr_gb300.so is not built: run tnrkit.jl_gb300/build.py (nvcc, sm_103a)")
    L = C.CDLL(LIB_PATH)
    P, I, D, Z = C.c_void_p, C.c_int, C.c_double, C.c_size_t
    pd, pi64, pz = C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_size_t)
    sig = {
        "tnr_default_options": (None, [C.POINTER(Options)]),
        "tnr_create": (I, [C.POINTER(P), I, I, pi64, pd, C.POINTER(Options)]),
        "tnr_create_device": (I, [C.POINTER(P), I, I, pi64, P, C.POINTER(Options)]),
        "tnr_step": (I, [P, I]),
        "tnr_finalize": (I, [P, pd]),
        "tnr_run": (I, [P, I, I, I, pd, Z, pz]),
        "tnr_create_impurity_hotrg": (I, [C.POINTER(P), pi64, pd, pd, pd, pd, C.c_void_p]),
        "tnr_create_impurity_trg": (I, [C.POINTER(P), pi64, pd, pd, pd, pd, pd, C.c_void_p]),
        "tnr_finalize_impurity": (I, [P, pd]),
        "tnr_create_correlation_hotrg": (I, [C.POINTER(P), pi64, pd, pd, pd, I, C.c_void_p]),
        "tnr_run_correlation": (I, [P, I, I, pd, Z, pz]),
        "tnr_correlation_ratio": (I, [P, pd]),
        "tnr_set_finalizer": (I, [P, I]),
        "tnr_transfer_eigvals": (I, [P, I, pd, pd, Z, pz]),
        "tnr_gu_wen_ratio": (I, [P, pd, pd]),
        "tnr_central_charge": (I, [P, C.c_double, pd]),
        "tnr_get_impurity_tensor": (I, [P, I, pd, Z, pi64, C.POINTER(I)]),
        "tnr_run_impurity": (I, [P, I, I, I, pd, Z, pz]),
        "tnr_free_energy": (D, [pd, Z, D, D, D]),
        "tnr_get_tensor": (I, [P, pd, Z, pi64, C.POINTER(I)]),
        "tnr_singular_values": (I, [P, pd, Z, pz, C.POINTER(C.c_int32), Z, pz]),
        "tnr_truncation_errors": (I, [P, pd, Z, pz]),
        "tnr_btrg_bonds": (I, [P, pd, Z, pz, pd, Z, pz]),
        "tnr_device_bytes": (I, [P, pz]),
        "tnr_decomposition_stats": (I, [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(I)]),
        "tnr_destroy": (I, [P]),
        "tnr_last_error": (I, [P, C.c_char_p, Z]),
        "tnr_status_string": (C.c_char_p, [I]),
        "tnr_timer_start": (I, [P]),
        "tnr_timer_stop": (I, [P, pd]),
        "tnr_run_batch": (I, [C.POINTER(P), I, C.POINTER(I), C.POINTER(I), I, pd, Z, pz, pd, pd]),
        "tnr_profile_enable": (I, [I]),
        "tnr_profile_reset": (I, []),
        "tnr_profile_read": (I, [I, C.POINTER(C.c_uint64), pd, pd]),
        "tnr_debug_gemm": (I, [I, I, I, C.c_int64, C.c_int64, C.c_int64, pd, C.c_int64, C.c_int64, pd, C.c_int64,
                               C.c_int64, pd, C.c_int64, C.c_int64, I]),
        "tnr_gemm_time": (I, [I, I, I, C.c_int64, C.c_int64, C.c_int64, I, I, I, pd]),
        "tnr_debug_chol": (I, [I, I, D, I, pd, pd, C.POINTER(I)]),
        "tnr_gemm_split_noalloc": (I, [I, I, C.c_int64, C.c_int64, C.c_int64, D, P, C.c_int64, P, C.c_int64, D, P,
                                       C.c_int64, P, C.c_char_p, Z]),
        "tnr_server_create": (I, [C.POINTER(P), Z, I, I]),
        "tnr_server_submit": (I, [P, I, I, pi64, pd, I, I, D, C.POINTER(C.c_uint64)]),
        "tnr_server_submit_sym": (I, [P, I, I, pi64, pd, I, C.POINTER(C.c_int32), I, I, D, C.POINTER(C.c_uint64)]),
        "tnr_server_poll": (I, [P, C.c_uint64, I, C.POINTER(I), pd, Z, pz, pd, pd]),
        "tnr_server_stats": (I, [P, C.POINTER(I), C.POINTER(I), pz]),
        "tnr_server_destroy": (I, [P]),
        "tnr_footprint_bytes": (Z, [I, I, I, pi64]),
        "tnr_device_info": (I, [C.POINTER(I), C.POINTER(I), C.POINTER(I), pz]),
        "tnr_version": (C.c_char_p, []),
        "tnr_kernel_launches": (C.c_uint64, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _err(h=None):
    buf = C.create_string_buffer(1024)
    lib().tnr_last_error(h, buf, 1024)
    return buf.value.decode(errors="replace")


def _check(st, h=None):
    if st != 0:
        raise TNRError(st, _err(h))


@dataclass
class truncrank:
    """MatrixAlgebraKit ``truncrank(howmany)``: keep the ``howmany`` largest values."""
    howmany: int


class stopcrit:
    """A stopping criterion of run! (src/utility/stopping.jl): called with (steps, data), it
    returns whether to continue; ``a & b`` continues while both do (MultipleCrit)."""

    def __and__(self, other):
        return MultipleCrit([self, other])


@dataclass
class maxiter(stopcrit):
    """``maxiter(n)`` (src/utility/stopping.jl:3-5,18): continue while steps < n."""
    n: int

    def __call__(self, steps, data):
        return steps < self.n


@dataclass
class convcrit(stopcrit):
    """``convcrit(Δ, f)`` (src/utility/stopping.jl:7-10,19): continue while Δ < f(steps, data)."""
    delta: float
    f: object

    def __call__(self, steps, data):
        return self.delta < self.f(steps, data)


@dataclass
class MultipleCrit(stopcrit):
    """``MultipleCrit(crits)`` (src/utility/stopping.jl:12-22): continue while every criterion does."""
    crits: list

    def __call__(self, steps, data):
        return all(c(steps, data) for c in self.crits)


def trivial_convcrit(delta):
    """``trivial_convcrit(Δ)`` (src/utility/stopping.jl:42): continue while Δ < data[end]."""
    return convcrit(delta, lambda steps, data: data[-1])


def ATRG_3D_convcrit(steps, data):
    """``ATRG_3D_convcrit`` (src/schemes/atrg3d.jl:98): |log(data[end]) 8^(1 - steps)|."""
    return abs(np.log(data[-1]) * 8.0 ** (1 - steps))


def _as_sym(T):
    if isinstance(T, SymTensor):
        return T
    return SymTensor(np.asarray(T, dtype=np.float64), None, 1)


class _Scheme:
    kind = 0
    nlegs = 4
    scalefactor = 2.0

    def __init__(self, T, precision=PREC_F64, k=-0.5, seed=0, stream=None):
        T = _as_sym(T)
        a = np.asarray(T.array, dtype=np.float64)
        if a.ndim != self.nlegs:
            raise ValueError("%s needs a %d-leg tensor" % (type(self).__name__, self.nlegs))
        L = lib()
        o = Options()
        L.tnr_default_options(C.byref(o))
        o.precision = precision
        o.btrg_k = k
        o.seed = seed
        o.stream = stream
        keep = None
        if T.charges is not None and T.N > 1:
            keep = np.ascontiguousarray(np.concatenate([np.asarray(c, dtype=np.int32) for c in T.charges]))
            o.symmetry_n = T.N
            o.leg_charges = keep.ctypes.data_as(C.POINTER(C.c_int32))
        dims = (C.c_int64 * a.ndim)(*a.shape)
        data = np.asfortranarray(a)                     # column-major, first leg fastest
        h = C.c_void_p()
        st = L.tnr_create(C.byref(h), self.kind, a.ndim, dims, data.ctypes.data_as(C.POINTER(C.c_double)),
                          C.byref(o))
        _check(st)
        self._h = h
        self.precision = precision
        self.symmetry_n = T.N

    # --- reference fields -------------------------------------------------
    def dims(self):
        """The current tensor's leg dimensions (no data copy)."""
        dims = (C.c_int64 * 8)()
        n = C.c_int()
        _check(lib().tnr_get_tensor(self._h, None, 0, dims, C.byref(n)), self._h)
        return tuple(dims[i] for i in range(n.value))

    @property
    def T(self):
        """Current tensor as a host array indexed like the reference (T[i1, i2, ...])."""
        L = lib()
        dims = (C.c_int64 * 8)()
        n = C.c_int()
        shape = self.dims()
        out = np.empty(int(np.prod(shape)), dtype=np.float64)
        _check(L.tnr_get_tensor(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), out.size, dims, C.byref(n)),
               self._h)
        return out.reshape(shape, order="F")

    def singular_values(self):
        """Kept singular values / Gram eigenvalues of the last step, one array per decomposition."""
        L = lib()
        n, nd = C.c_size_t(), C.c_size_t()
        _check(L.tnr_singular_values(self._h, None, 0, C.byref(n), None, 0, C.byref(nd)), self._h)
        vals = np.empty(max(n.value, 1))
        cnt = (C.c_int32 * max(nd.value, 1))()
        _check(L.tnr_singular_values(self._h, vals.ctypes.data_as(C.POINTER(C.c_double)), vals.size, C.byref(n),
                                     cnt, nd.value, C.byref(nd)), self._h)
        out, at = [], 0
        for i in range(nd.value):
            out.append(vals[at:at + cnt[i]].copy())
            at += cnt[i]
        return out

    def truncation_errors(self):
        L = lib()
        n = C.c_size_t()
        _check(L.tnr_truncation_errors(self._h, None, 0, C.byref(n)), self._h)
        out = np.empty(max(n.value, 1))
        _check(L.tnr_truncation_errors(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), out.size, C.byref(n)),
               self._h)
        return out[:n.value]

    def device_bytes(self):
        b = C.c_size_t()
        _check(lib().tnr_device_bytes(self._h, C.byref(b)), self._h)
        return b.value

    def decomposition_stats(self):
        """(decompositions, gap fallbacks decomposed in full FP64, most subspace iterations)."""
        nd, nf, mi = C.c_uint64(), C.c_uint64(), C.c_int()
        _check(lib().tnr_decomposition_stats(self._h, C.byref(nd), C.byref(nf), C.byref(mi)), self._h)
        return nd.value, nf.value, mi.value

    def close(self):
        if getattr(self, "_h", None):
            lib().tnr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TRG(_Scheme):
    """Tensor Renormalization Group (src/schemes/trg.jl:26-41); rescales by sqrt(2)."""
    kind = TNR_TRG


class BTRG(_Scheme):
    """Bond-weighted TRG (src/schemes/btrg.jl:26-94); ``BTRG(T, k=-0.5)``."""
    kind = TNR_BTRG

    def __init__(self, T, k=-0.5, **kw):
        super().__init__(T, k=k, **kw)
        self.k = k

    @property
    def S1(self):
        return self._bonds()[0]

    @property
    def S2(self):
        return self._bonds()[1]

    def _bonds(self):
        L = lib()
        n1, n2 = C.c_size_t(), C.c_size_t()
        _check(L.tnr_btrg_bonds(self._h, None, 0, C.byref(n1), None, 0, C.byref(n2)), self._h)
        a, b = np.empty(n1.value), np.empty(n2.value)
        _check(L.tnr_btrg_bonds(self._h, a.ctypes.data_as(C.POINTER(C.c_double)), a.size, C.byref(n1),
                                b.ctypes.data_as(C.POINTER(C.c_double)), b.size, C.byref(n2)), self._h)
        return a, b


class HOTRG(_Scheme):
    """Higher-Order TRG (src/schemes/hotrg.jl:27-160); rescales by 2 (area factor 4)."""
    kind = TNR_HOTRG
    scalefactor = 4.0


class ATRG(_Scheme):
    """Anisotropic TRG (src/schemes/atrg.jl:26-81): two anisotropic half steps per step, each a
    linear rescaling by sqrt(2) (area factor 4 per step)."""
    kind = TNR_ATRG
    scalefactor = 4.0


class ATRG_3D(_Scheme):
    """3D anisotropic TRG (src/schemes/atrg3d.jl:26-90): three half steps per step (volume
    factor 8); on the device up to truncrank(12) (its QR factors have at most chi^2 columns)."""
    kind = TNR_ATRG_3D
    nlegs = 6
    scalefactor = 8.0


class HOTRG_3D(_Scheme):
    """3D HOTRG (src/schemes/hotrg3d.jl:27-135); volume factor 8 per step."""
    kind = TNR_HOTRG_3D
    nlegs = 6
    scalefactor = 8.0


class _ImpurityScheme(_Scheme):
    """A pure tensor and impurity tensors of the same spaces, stepped together on the device;
    finalize!/run! return a tuple of ``norms`` norms per entry."""
    norms = 1
    _create = ""

    def _make(self, tensors, precision, seed, stream, *extra):
        arrs = [np.asfortranarray(np.asarray(_as_sym(t).array, dtype=np.float64)) for t in tensors]
        if any(a.ndim != 4 or a.shape != arrs[0].shape for a in arrs):
            raise ValueError(f"{type(self).__name__} needs {len(arrs)} 4-leg tensors of the same dims")
        L = lib()
        o = Options()
        L.tnr_default_options(C.byref(o))
        o.precision = precision
        o.seed = seed
        o.stream = stream
        dims = (C.c_int64 * 4)(*arrs[0].shape)
        pp = [a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs]
        h = C.c_void_p()
        _check(getattr(L, self._create)(C.byref(h), dims, *pp, *extra, C.byref(o)))
        self._h = h
        self.precision = precision
        self.symmetry_n = 1


def _impurity_tensor(scheme, which):
    """Impurity tensor ``which`` of an impurity scheme as a host array (tnr_get_impurity_tensor)."""
    L = lib()
    dims = (C.c_int64 * 8)()
    n = C.c_int()
    _check(L.tnr_get_impurity_tensor(scheme._h, int(which), None, 0, dims, C.byref(n)), scheme._h)
    shape = tuple(dims[i] for i in range(n.value))
    out = np.empty(int(np.prod(shape)), dtype=np.float64)
    _check(L.tnr_get_impurity_tensor(scheme._h, int(which), out.ctypes.data_as(C.POINTER(C.c_double)), out.size,
                                     dims, C.byref(n)), scheme._h)
    return out.reshape(shape, order="F")


class ImpurityHOTRG(_ImpurityScheme):
    """``ImpurityHOTRG(T, T_imp_order1_1, T_imp_order1_2, T_imp_order2)``
    (src/schemes/impurityhotrg.jl:26-84): four tensors of the same spaces; ``run`` returns
    the (pure, +1, -1, second-order) norm tuples of finalize!(::ImpurityHOTRG)."""
    kind = TNR_IMPURITY_HOTRG
    scalefactor = 4.0
    norms = 4
    _create = "tnr_create_impurity_hotrg"

    def __init__(self, T, T_imp_order1_1, T_imp_order1_2, T_imp_order2, precision=PREC_F64, seed=0, stream=None):
        self._make((T, T_imp_order1_1, T_imp_order1_2, T_imp_order2), precision, seed, stream)

    T_imp_order1_1 = property(lambda self: _impurity_tensor(self, 0))
    T_imp_order1_2 = property(lambda self: _impurity_tensor(self, 1))
    T_imp_order2 = property(lambda self: _impurity_tensor(self, 2))


class ImpurityTRG(_ImpurityScheme):
    """``ImpurityTRG(T, T_imp1, T_imp2, T_imp3, T_imp4)`` (src/schemes/impuritytrg.jl:38-61):
    the pure tensor and the four sites of an impurity plaquette; ``run`` returns the
    (pure, plaquette) norm tuples of finalize!(::ImpurityTRG) (src/utility/finalize.jl:75-88)."""
    kind = TNR_IMPURITY_TRG
    scalefactor = 2.0
    norms = 2
    _create = "tnr_create_impurity_trg"

    def __init__(self, T, T_imp1, T_imp2, T_imp3, T_imp4, precision=PREC_F64, seed=0, stream=None):
        self._make((T, T_imp1, T_imp2, T_imp3, T_imp4), precision, seed, stream)

    T_imp1 = property(lambda self: _impurity_tensor(self, 0))
    T_imp2 = property(lambda self: _impurity_tensor(self, 1))
    T_imp3 = property(lambda self: _impurity_tensor(self, 2))
    T_imp4 = property(lambda self: _impurity_tensor(self, 3))


class CorrelationHOTRG(_ImpurityScheme):
    """``CorrelationHOTRG(Tpure, Timp1, Timp2, dist)`` (src/schemes/correlationhotrg.jl:29-71): two
    first-order impurities 2^dist sites apart, merged into one at step dist.  ``run`` returns the
    (n, n_1, n_2) / (n, n_imp, n_imp) tuple of every step (correlationhotrg.jl:138-162); ``step``
    runs step! with its phase finalizer; ``correlation()`` is |tr Timp_final| / |tr Tpure|."""
    kind = TNR_CORRELATION_HOTRG
    scalefactor = 4.0
    norms = 3
    _create = "tnr_create_correlation_hotrg"

    def __init__(self, Tpure, Timp1, Timp2, dist, precision=PREC_F64, seed=0, stream=None):
        if int(dist) < 0:
            raise ValueError("Distance must be non-negative")
        self.dist = int(dist)
        self._make((Tpure, Timp1, Timp2), precision, seed, stream, self.dist)

    Tpure = property(lambda self: self.T)
    Timp1 = property(lambda self: _impurity_tensor(self, 0))
    Timp2 = property(lambda self: _impurity_tensor(self, 1))
    Timp_final = property(lambda self: _impurity_tensor(self, 2))

    def correlation(self):
        out = C.c_double()
        _check(lib().tnr_correlation_ratio(self._h, C.byref(out)), self._h)
        return out.value


def step(scheme, trunc):
    """``step!(scheme, truncrank(chi))``"""
    _check(lib().tnr_step(scheme._h, int(trunc.howmany)), scheme._h)
    return scheme


def finalize(scheme):
    """``finalize!(scheme)``: trace norm n, T /= n; returns n (impurity schemes: a tuple of norms)."""
    if isinstance(scheme, CorrelationHOTRG):
        raise TypeError("CorrelationHOTRG finalizes inside step!; use run or step")
    if isinstance(scheme, _ImpurityScheme):
        out = np.empty(scheme.norms)
        _check(lib().tnr_finalize_impurity(scheme._h, out.ctypes.data_as(C.POINTER(C.c_double))), scheme._h)
        return tuple(out)
    n = C.c_double()
    _check(lib().tnr_finalize(scheme._h, C.byref(n)), scheme._h)
    return n.value


class Finalizer:
    """A finalizer of run! (src/utility/finalize.jl); ``code`` is its C-ABI constant."""

    def __init__(self, name, code):
        self.name, self.code = name, code

    def __repr__(self):
        return self.name


default_Finalizer = Finalizer("default_Finalizer", 0)          # finalize! (tnrscheme.jl:26)
two_by_two_Finalizer = Finalizer("two_by_two_Finalizer", 1)    # finalize_two_by_two! (finalize.jl:17-41,151)


def set_finalizer(scheme, finalizer):
    """The finalizer that ``finalize`` and ``run`` use for this scheme."""
    _check(lib().tnr_set_finalizer(scheme._h, int(finalizer.code)), scheme._h)
    scheme.finalizer = finalizer


def finalize_two_by_two(scheme):
    """``finalize_two_by_two!(scheme)`` (src/utility/finalize.jl:17-41): the 2 x 2 plaquette norm
    n, T /= n^(1/4); returns n^(1/4)."""
    old = getattr(scheme, "finalizer", default_Finalizer)
    set_finalizer(scheme, two_by_two_Finalizer)
    try:
        return finalize(scheme)
    finally:
        set_finalizer(scheme, old)


def transfer_eigvals(scheme, unitcell=1):
    """``eig_full`` of the unit-cell column transfer matrix (src/utility/cft.jl:7-16), on the device."""
    n = int(scheme.dims()[1]) ** unitcell
    re, im = np.empty(n), np.empty(n)
    k = C.c_size_t()
    _check(lib().tnr_transfer_eigvals(scheme._h, int(unitcell), re.ctypes.data_as(C.POINTER(C.c_double)),
                                      im.ctypes.data_as(C.POINTER(C.c_double)), n, C.byref(k)), scheme._h)
    return re[:k.value] + 1j * im[:k.value]


def cft_data(scheme, v=1, unitcell=1, is_real=True):
    """``cft_data(scheme; v, unitcell, is_real)`` (src/utility/cft.jl:5-73): the transfer
    matrix's eigenvalues sorted by magnitude, real part > 0 and magnitude > 1e-12 kept, as
    unitcell / (2 pi v) log(lambda_1 / lambda)."""
    lam = transfer_eigvals(scheme, unitcell)
    lam = lam[np.argsort(-np.abs(lam), kind="stable")]
    lam = lam[lam.real > 0]
    lam = lam[np.abs(lam) > 1e-12]
    if is_real:
        lam = lam.real
    return unitcell * (1.0 / (2.0 * np.pi * v)) * np.log(lam[0] / lam)


def ground_state_degeneracy(scheme, unitcell=1):
    """``ground_state_degeneracy(scheme)`` (src/utility/cft.jl:278-340): exp of the Shannon
    entropy of |lambda / tr D| over the transfer matrix's nonzero eigenvalues."""
    lam = transfer_eigvals(scheme, unitcell)
    p = np.abs(lam / lam.sum())
    p = p[p != 0]
    return float(np.exp(-np.sum(p * np.log(p))))


def gu_wen_ratio(scheme):
    """``gu_wen_ratio(scheme)`` (src/utility/cft.jl:374-396): (X1, X2), on the device."""
    x1, x2 = C.c_double(), C.c_double()
    _check(lib().tnr_gu_wen_ratio(scheme._h, C.byref(x1), C.byref(x2)), scheme._h)
    return x1.value, x2.value


def central_charge(scheme, n):
    """``central_charge(scheme, n)`` (src/utility/cft.jl:256-269), on the device."""
    out = C.c_double()
    _check(lib().tnr_central_charge(scheme._h, float(n), C.byref(out)), scheme._h)
    return out.value


def run(scheme, trunc, crit, finalizer=None, finalize_beginning=True, verbosity=0):
    """``run!(scheme, trunc, maxiter(n)[, finalizer]; finalize_beginning)``; the default
    Finalizer unless ``finalizer`` is given (it then stays selected for the scheme).

    Returns the list of norms (n + 1 with ``finalize_beginning``).  With maxiter(n) the whole
    loop runs in the library and the norms come back once; any other criterion (convcrit,
    MultipleCrit) is evaluated on the host after every step, as run! does
    (src/schemes/tnrscheme.jl:39-52), from the norm that step's finalize! returns."""
    if not isinstance(crit, stopcrit):
        raise TypeError("crit must be a stopping criterion (maxiter, convcrit, a & b)")
    if finalizer is not None:
        set_finalizer(scheme, finalizer)
    if not isinstance(crit, maxiter):
        if isinstance(scheme, CorrelationHOTRG):
            raise TypeError("CorrelationHOTRG's run! takes maxiter(n)")
        data = [finalize(scheme)] if finalize_beginning else []
        steps = 0
        while True:
            step(scheme, trunc)
            data.append(finalize(scheme))
            steps += 1
            if not crit(steps, data):
                return data
    nsteps = max(crit.n, 1)
    cap = nsteps + 1
    if isinstance(scheme, CorrelationHOTRG):
        if crit.n <= scheme.dist:
            raise ValueError("niter must be larger than dist")
        out = np.empty(3 * crit.n)
        n = C.c_size_t()
        _check(lib().tnr_run_correlation(scheme._h, int(trunc.howmany), int(crit.n),
                                         out.ctypes.data_as(C.POINTER(C.c_double)), out.size, C.byref(n)), scheme._h)
        return [tuple(out[3 * i:3 * i + 3]) for i in range(n.value)]
    if isinstance(scheme, _ImpurityScheme):
        k = scheme.norms
        out = np.empty(k * cap)
        n = C.c_size_t()
        _check(lib().tnr_run_impurity(scheme._h, int(trunc.howmany), int(crit.n), 1 if finalize_beginning else 0,
                                      out.ctypes.data_as(C.POINTER(C.c_double)), out.size, C.byref(n)), scheme._h)
        return [tuple(out[k * i:k * i + k]) for i in range(n.value)]
    out = np.empty(cap)
    n = C.c_size_t()
    _check(lib().tnr_run(scheme._h, int(trunc.howmany), int(crit.n), 1 if finalize_beginning else 0,
                         out.ctypes.data_as(C.POINTER(C.c_double)), cap, C.byref(n)), scheme._h)
    return list(out[:n.value])


run_ = run   # run! in Julia


def run_batch(schemes, chis, maxiters, finalize_beginning=True, timing=None):
    """Runs ``run!`` on many independent schemes concurrently; returns one norm list per scheme.

    If ``timing`` is a dict it receives ``device_ms`` (CUDA-event span of the batch) and
    ``latency_ms`` (per-instance completion times from batch start)."""
    n = len(schemes)
    if len(chis) != n or len(maxiters) != n:
        raise ValueError("one chi and one maxiter per scheme")
    if n == 0:
        if timing is not None:
            timing["device_ms"] = 0.0
            timing["latency_ms"] = np.zeros(0)
        return []
    stride = max(max(int(m), 1) for m in maxiters) + 1
    out = np.empty(n * stride)
    cnt = (C.c_size_t * n)()
    hs = (C.c_void_p * n)(*[s._h for s in schemes])
    ch = (C.c_int * n)(*[int(x) for x in chis])
    mi = (C.c_int * n)(*[int(x) for x in maxiters])
    dev_ms = C.c_double()
    lat = np.zeros(n)
    st = lib().tnr_run_batch(hs, n, ch, mi, 1 if finalize_beginning else 0,
                             out.ctypes.data_as(C.POINTER(C.c_double)), stride, cnt,
                             C.byref(dev_ms), lat.ctypes.data_as(C.POINTER(C.c_double)))
    _check(st)
    if timing is not None:
        timing["device_ms"] = dev_ms.value
        timing["latency_ms"] = lat
    return [list(out[i * stride:i * stride + cnt[i]]) for i in range(n)]


PROFILE_CLASSES = {"gemm_bulk": 0, "gemm_f64": 1, "jacobi": 2, "chol": 3, "permute": 4, "split": 5, "jacobi32": 6,
                   "tc": 7, "chol32": 8}


def profile_enable(on=True):
    _check(lib().tnr_profile_enable(1 if on else 0))


def profile_reset():
    _check(lib().tnr_profile_reset())


def profile_read():
    """{class: (launches, total_ms, work)} of the launches recorded since the last reset."""
    out = {}
    for name, cls in PROFILE_CLASSES.items():
        n, ms, w = C.c_uint64(), C.c_double(), C.c_double()
        _check(lib().tnr_profile_read(cls, C.byref(n), C.byref(ms), C.byref(w)))
        out[name] = (n.value, ms.value, w.value)
    return out


class Server:
    """Serving loop: submit run! requests, admitted by HBM footprint, solved concurrently.

    ``submit(T, scheme, chi, maxiter)`` returns a request id; ``result(id)`` blocks and
    returns (norms, latency_ms, queue_ms)."""

    KINDS = {"TRG": TNR_TRG, "BTRG": TNR_BTRG, "HOTRG": TNR_HOTRG, "HOTRG_3D": TNR_HOTRG_3D, "ATRG": TNR_ATRG,
             "ATRG_3D": TNR_ATRG_3D}

    def __init__(self, hbm_budget_bytes, max_active=32, precision=PREC_F64):
        h = C.c_void_p()
        _check(lib().tnr_server_create(C.byref(h), int(hbm_budget_bytes), int(max_active), int(precision)))
        self._h = h
        self.maxiter = {}

    def submit(self, T, scheme, chi, maxiter, k=-0.5):
        """Queue a run!(scheme(T), truncrank(chi), maxiter(maxiter)) request; a Z_N tensor (its
        charges given) runs block by block over its charge sectors."""
        T = _as_sym(T)
        a = np.asfortranarray(T.array, dtype=np.float64)
        kind = self.KINDS[scheme if isinstance(scheme, str) else scheme.__name__]
        dims = (C.c_int64 * a.ndim)(*a.shape)
        rid = C.c_uint64()
        if T.charges is not None and T.N > 1:
            q = np.ascontiguousarray(np.concatenate([np.asarray(c, dtype=np.int32) for c in T.charges]))
            st = lib().tnr_server_submit_sym(self._h, kind, a.ndim, dims, a.ctypes.data_as(C.POINTER(C.c_double)),
                                             int(T.N), q.ctypes.data_as(C.POINTER(C.c_int32)), int(chi),
                                             int(maxiter), float(k), C.byref(rid))
        else:
            st = lib().tnr_server_submit(self._h, kind, a.ndim, dims, a.ctypes.data_as(C.POINTER(C.c_double)),
                                         int(chi), int(maxiter), float(k), C.byref(rid))
        _check(st)
        self.maxiter[rid.value] = maxiter
        return rid.value

    def result(self, rid, wait=True):
        cap = max(self.maxiter[rid], 1) + 1
        out = np.empty(cap)
        done, n, lat, q = C.c_int(), C.c_size_t(), C.c_double(), C.c_double()
        st = lib().tnr_server_poll(self._h, rid, 1 if wait else 0, C.byref(done),
                                   out.ctypes.data_as(C.POINTER(C.c_double)), cap, C.byref(n), C.byref(lat),
                                   C.byref(q))
        _check(st)
        if not done.value:
            return None
        return list(out[:n.value]), lat.value, q.value

    def stats(self):
        a, qd, b = C.c_int(), C.c_int(), C.c_size_t()
        _check(lib().tnr_server_stats(self._h, C.byref(a), C.byref(qd), C.byref(b)))
        return {"active": a.value, "queued": qd.value, "bytes_in_use": b.value}

    def close(self):
        if getattr(self, "_h", None):
            lib().tnr_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def footprint_bytes(scheme, chi, dims):
    kind = Server.KINDS[scheme if isinstance(scheme, str) else scheme.__name__]
    d = (C.c_int64 * len(dims))(*dims)
    return int(lib().tnr_footprint_bytes(kind, int(chi), len(dims), d))


def free_energy(data, beta, scalefactor=2.0, initial_size=1.0):
    """``free_energy(data, β; scalefactor, initial_size)`` (src/utility/free_energy.jl:13-20)."""
    a = np.ascontiguousarray(np.asarray(data, dtype=np.float64))
    return lib().tnr_free_energy(a.ctypes.data_as(C.POINTER(C.c_double)), a.size, float(beta), float(scalefactor),
                                 float(initial_size))


def debug_gemm(A, B, ta=False, tb=False, precision=PREC_SPLIT):
    """op(A) @ op(B) through the engine's GEMM kernel (batched if A, B are 3-D: [batch, rows, cols])."""
    A3 = np.atleast_3d(A) if A.ndim == 3 else A[None]
    B3 = np.atleast_3d(B) if B.ndim == 3 else B[None]
    batch = A3.shape[0]
    # column-major storage of each stored matrix, batches contiguous
    Af = np.ascontiguousarray(np.transpose(A3, (0, 2, 1)))
    Bf = np.ascontiguousarray(np.transpose(B3, (0, 2, 1)))
    ar, ac = A3.shape[1:]
    br, bc = B3.shape[1:]
    m, k = (ac, ar) if ta else (ar, ac)
    kb, n = (bc, br) if tb else (br, bc)
    assert k == kb
    Cf = np.zeros((batch, n, m))
    st = lib().tnr_debug_gemm(precision, int(ta), int(tb), m, n, k, Af.ctypes.data_as(C.POINTER(C.c_double)), ar,
                              ar * ac if batch > 1 else 0, Bf.ctypes.data_as(C.POINTER(C.c_double)), br,
                              br * bc if batch > 1 else 0, Cf.ctypes.data_as(C.POINTER(C.c_double)), m, m * n, batch)
    _check(st)
    out = np.transpose(Cf, (0, 2, 1))
    return out if A.ndim == 3 else out[0]


def debug_chol(G, shift=0.0, precision=PREC_F64):
    """L^-1 of the Cholesky factor of G + shift I through the engine's kernel (G: [batch,] r x r);
    returns (Linv, breakdown)."""
    G3 = np.asarray(G, dtype=np.float64)
    G3 = G3 if G3.ndim == 3 else G3[None]
    batch, r = G3.shape[0], G3.shape[1]
    Gf = np.ascontiguousarray(np.transpose(G3, (0, 2, 1)))
    out = np.zeros_like(Gf)
    bd = C.c_int()
    _check(lib().tnr_debug_chol(precision, r, float(shift), batch, Gf.ctypes.data_as(C.POINTER(C.c_double)),
                                out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(bd)))
    L = np.transpose(out, (0, 2, 1))
    return (L if np.ndim(G) == 3 else L[0]), bool(bd.value)


def gemm_time(m, n, k, batch=1, ta=False, tb=False, precision=PREC_SPLIT, reps=5, contraction=False):
    """Average device milliseconds of one batched GEMM of this shape on seeded device operands
    (contraction=True: the contraction path, K accumulated in chunks)."""
    ms = C.c_double()
    _check(lib().tnr_gemm_time(precision, int(ta), int(tb), m, n, k, batch, reps, int(contraction), C.byref(ms)))
    return ms.value


def device_info():
    sm, ma, mi, hbm = C.c_int(), C.c_int(), C.c_int(), C.c_size_t()
    _check(lib().tnr_device_info(C.byref(sm), C.byref(ma), C.byref(mi), C.byref(hbm)))
    return {"sm_count": sm.value, "cc": (ma.value, mi.value), "hbm_bytes": hbm.value}


def kernel_launches():
    return int(lib().tnr_kernel_launches())


class Timer:
    """Device time on a scheme's stream (CUDA events)."""

    def __init__(self, scheme):
        self.s = scheme

    def __enter__(self):
        _check(lib().tnr_timer_start(self.s._h), self.s._h)
        return self

    def __exit__(self, *exc):
        ms = C.c_double()
        _check(lib().tnr_timer_stop(self.s._h, C.byref(ms)), self.s._h)
        self.ms = ms.value
        return False
