"""CPU-only checks: the C-ABI library loads and exports every declared symbol,
error paths return status codes without a GPU, and the host-side model
constructors match the oracle's."""
import ctypes
import os
import re
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def tnr():
    import __graft_entry__ as ge
    ge.build()
    return ge.package()


def header_symbols():
    syms = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            syms += re.findall(r"\b(tnr_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(syms))


def test_library_exports_header(tnr):
    lib = ctypes.CDLL(tnr.LIB_PATH)
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) <= set(tnr.EXPORTS)


def test_status_strings(tnr):
    L = tnr.lib()
    assert L.tnr_status_string(0) == b"ok"
    assert L.tnr_status_string(5) == b"admission refused"
    assert b"sm_103a" in L.tnr_version()


def test_free_energy_host(tnr, oracle):
    data = [1.5, 2.25, 3.0, 0.75]
    for sf, init in [(2.0, 1.0), (4.0, 1.0), (8.0, 2.0)]:
        assert tnr.free_energy(data, 0.4, sf, init) == pytest.approx(
            oracle.free_energy(data, 0.4, sf, init), rel=1e-15)


def test_create_rejects_bad_input(tnr):
    # invalid arguments are refused before any device work
    with pytest.raises(ValueError):
        tnr.TRG(np.ones((2, 2, 2)))
    bad = np.ones((2, 2, 2, 2))
    bad[0, 0, 0, 0] = np.nan
    with pytest.raises(tnr.TNRError):
        tnr.TRG(bad)


def test_no_device_is_an_error_not_a_crash(tnr):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(tnr.TNRError) as e:
        tnr.TRG(tnr.classical_ising())
    assert e.value.status in (8, 4)


@pytest.mark.parametrize("name", ["ising", "ising_triv", "ising_impurity", "potts3", "clock6", "clock3", "ising3d",
                                  "sixvertex", "phi4_triv", "phi4_z2", "phi4_imp1", "phi4_imp2", "phi4_complex"])
def test_models_match_oracle(tnr, oracle, name):
    o = oracle
    if name == "ising":
        a, b = tnr.classical_ising("Z2"), o.classical_ising(symmetry="Z2")
    elif name == "ising_impurity":
        a, b = tnr.classical_ising_impurity(0.41, 0.3), o.classical_ising_impurity(0.41, 0.3)
    elif name == "ising_triv":
        a, b = tnr.classical_ising("Trivial", 0.37), o.classical_ising(0.37, "Trivial")
    elif name == "potts3":
        a, b = tnr.classical_potts(3, 0.8), o.classical_potts(3, 0.8)
    elif name == "clock6":
        a, b = tnr.classical_clock(6, 0.9), o.classical_clock(6, 0.9)
    elif name == "clock3":
        a, b = tnr.classical_clock(3, 0.9, "Trivial"), o.classical_clock(3, 0.9, "Trivial")
    elif name == "sixvertex":
        a, b = tnr.sixvertex("Trivial", 1.0, 2.0, 3.0), o.sixvertex(1.0, 2.0, 3.0)
    elif name == "phi4_triv":
        a, b = tnr.phi4_real(8, -1.0, 1.0, 0.1, symmetry="Trivial"), o.phi4_real(8, -1.0, 1.0, 0.1, symmetry="Trivial")
    elif name == "phi4_z2":
        a, b = tnr.phi4_real(8, -1.0, 1.0), o.phi4_real(8, -1.0, 1.0)
    elif name == "phi4_imp1":
        a, b = tnr.phi4_real_imp1(8, -2.0, 1.0), o.phi4_real_imp1(8, -2.0, 1.0)
    elif name == "phi4_complex":
        a, b = tnr.phi4_complex("Trivial", 4, -1.0, 1.0), o.phi4_complex(4, -1.0, 1.0)
    elif name == "phi4_imp2":
        a, b = tnr.phi4_real_imp2(8, -2.0, 1.0), o.phi4_real_imp2(8, -2.0, 1.0)
    else:
        a, b = tnr.classical_ising_3D(), o.classical_ising_3D()
    np.testing.assert_allclose(a.array, b.a, rtol=1e-13, atol=1e-14 * max(1.0, np.abs(b.a).max()))
    if b.q is not None:
        for qa, qb, l in zip(a.charges, b.q, range(b.a.ndim)):
            # the package stores plain charges; the oracle stores signed ones (domain legs negated)
            sign = 1 if (l < 2 or b.a.ndim == 6) else -1
            np.testing.assert_array_equal(qa % b.N, (sign * qb) % b.N)


def test_random_hotrg_tensor(tnr, oracle):
    a = tnr.random_hotrg_tensor(6, 3)
    b = oracle.random_hotrg_tensor(6, 3)
    np.testing.assert_allclose(a.array, b.a, rtol=1e-14)
    assert np.linalg.norm(a.array) == pytest.approx(1.0)


def header_defines():
    txt = open(os.path.join(ROOT, "include", "tnr_gb300.h")).read()
    return {k: int(v) for k, v in re.findall(r"#define\s+(TNR_[A-Z0-9_]+)\s+(\d+)\b", txt)}


def test_python_constants_match_header(tnr):
    """The host layer's scheme kinds, precisions and profiler classes are the header's."""
    d = header_defines()
    assert (tnr.TNR_TRG, tnr.TNR_BTRG, tnr.TNR_HOTRG, tnr.TNR_HOTRG_3D) == (
        d["TNR_TRG"], d["TNR_BTRG"], d["TNR_HOTRG"], d["TNR_HOTRG_3D"])
    assert (tnr.TNR_IMPURITY_HOTRG, tnr.TNR_IMPURITY_TRG, tnr.TNR_CORRELATION_HOTRG, tnr.TNR_ATRG, tnr.TNR_ATRG_3D) == (
        d["TNR_IMPURITY_HOTRG"], d["TNR_IMPURITY_TRG"], d["TNR_CORRELATION_HOTRG"], d["TNR_ATRG"], d["TNR_ATRG_3D"])
    assert (tnr.default_Finalizer.code, tnr.two_by_two_Finalizer.code) == (
        d["TNR_FINALIZER_DEFAULT"], d["TNR_FINALIZER_TWO_BY_TWO"])
    assert (tnr.PREC_F64, tnr.PREC_SPLIT) == (d["TNR_PREC_F64"], d["TNR_PREC_SPLIT"])
    prof = {k[len("TNR_PROF_"):].lower(): v for k, v in d.items() if k.startswith("TNR_PROF_")}
    assert prof == tnr.PROFILE_CLASSES
    codes = sorted(v for k, v in d.items() if k.startswith("TNR_ERR_") or k == "TNR_OK")
    assert codes == list(range(len(codes)))          # 0..8, no gaps


def test_footprint_grows_and_saturates(tnr):
    """tnr_footprint_bytes (host): grows with chi, HOTRG above BTRG, 3D above 2D, and a
    chi far beyond any device saturates instead of wrapping around."""
    a = [tnr.footprint_bytes("BTRG", chi, [2, 2, 2, 2]) for chi in (8, 16, 32, 64)]
    assert a == sorted(a) and a[0] > 0
    assert tnr.footprint_bytes("HOTRG", 32, [2] * 4) > tnr.footprint_bytes("BTRG", 32, [2] * 4)
    assert tnr.footprint_bytes("HOTRG_3D", 16, [2] * 6) > tnr.footprint_bytes("HOTRG", 16, [2] * 4)
    assert tnr.footprint_bytes("HOTRG_3D", 10 ** 6, [2] * 6) >= 9 * 10 ** 18


def test_server_admission_and_errors_without_device(tnr):
    """The serving loop's host logic: a request that can never fit the HBM budget is refused
    at submission (TNR_ERR_ADMISSION); an admitted request on a machine without a GPU comes
    back with TNR_ERR_NO_DEVICE through poll, and the server shuts down cleanly."""
    srv = tnr.Server(hbm_budget_bytes=1 << 30, max_active=2)
    T = tnr.classical_ising("Trivial")
    try:
        with pytest.raises(tnr.TNRError) as e:
            srv.submit(T, "HOTRG", 256, 10)
        assert e.value.status == 5
        rid = srv.submit(T, "BTRG", 8, 4)
        with pytest.raises(tnr.TNRError) as e:
            srv.result(rid)
        assert e.value.status == 8
        assert srv.stats()["active"] == 0
    finally:
        srv.close()


def test_run_batch_rejects_a_handle_twice(tnr):
    """A handle is single-owner; tnr_run_batch refuses a batch that names one twice before it
    touches the handles (the two entries are the same opaque pointer value, never dereferenced)."""
    fake = ctypes.c_void_p(0x1000)
    hs = (ctypes.c_void_p * 2)(fake, fake)
    chi = (ctypes.c_int * 2)(8, 8)
    mi = (ctypes.c_int * 2)(4, 4)
    norms = (ctypes.c_double * 20)()
    counts = (ctypes.c_size_t * 2)()
    lib = tnr.lib()
    st = lib.tnr_run_batch(hs, 2, chi, mi, 1, norms, 10, counts, None, None)
    assert st == 1                       # TNR_ERR_INVALID_ARG


def test_run_batch_argument_checks(tnr):
    assert tnr.run_batch([], [], []) == []
    with pytest.raises(ValueError):
        tnr.run_batch([], [8], [])


def test_correlation_hotrg_argument_checks(tnr):
    """CorrelationHOTRG refuses a negative distance in the host layer and in the C ABI, before
    any device work (src/schemes/correlationhotrg.jl:57)."""
    T = tnr.classical_ising("Trivial")
    with pytest.raises(ValueError):
        tnr.CorrelationHOTRG(T, T, T, -1)
    a = np.asfortranarray(T.array)
    p = a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    dims = (ctypes.c_int64 * 4)(*a.shape)
    h = ctypes.c_void_p()
    L = tnr.lib()
    assert L.tnr_create_correlation_hotrg(ctypes.byref(h), dims, p, p, p, -1, None) == header_defines()["TNR_ERR_INVALID_ARG"]
    assert not h.value
    bad = np.ones((2, 2, 2, 2))
    with pytest.raises(ValueError):
        tnr.CorrelationHOTRG(np.ones((2, 2, 2)), bad, bad, 1)


HQR_SHIM = """
#include "hqr.cuh"
extern "C" int hqr_eigvals(double* a, int n, double* wr, double* wi, double* work) {
    return tnr::real_eigvals(a, n, wr, wi, work);
}
"""


def _match(x, y):
    """largest distance of a greedy one-to-one matching of two multisets of complex numbers"""
    y, err = list(y), 0.0
    for v in x:
        i = int(np.argmin([abs(v - u) for u in y]))
        err = max(err, abs(v - y[i]))
        y.pop(i)
    return err


def test_transfer_eigvals_routine_on_the_host(tmp_path):
    """The eigenvalue routine the device runs for cft_data / ground_state_degeneracy
    (csrc/hqr.cuh: Hessenberg reduction and Francis double-shift QR) is one source for host and
    device; compiled here with g++ it matches LAPACK's eigenvalues on random matrices up to
    n = 160 and on structured ones (zero, identity, triangular, repeated, rotation blocks,
    nilpotent, rank-deficient), and on the oracle's fixed-point transfer matrices."""
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    src = tmp_path / "shim.cpp"
    src.write_text(HQR_SHIM)
    so = tmp_path / "libhqr.so"
    subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-I", os.path.join(ROOT, "tnrkit.jl_gb300", "csrc"),
                    "-o", str(so), str(src)], check=True)
    L = ctypes.CDLL(str(so))
    pd = ctypes.POINTER(ctypes.c_double)

    def eig(A):
        n = A.shape[0]
        a = np.array(A, dtype=np.float64, order="F")
        wr, wi, w = np.zeros(n), np.zeros(n), np.zeros(max(n, 1))
        st = L.hqr_eigvals(a.ctypes.data_as(pd), n, wr.ctypes.data_as(pd), wi.ctypes.data_as(pd), w.ctypes.data_as(pd))
        assert st == 0
        return wr + 1j * wi

    rng = np.random.default_rng(0)
    for n in (1, 2, 3, 5, 16, 24, 64, 160):
        for _ in range(3):
            A = rng.standard_normal((n, n))
            ref = np.linalg.eigvals(A)
            assert _match(eig(A), ref) <= 1e-12 * max(1.0, np.abs(ref).max())
    Q = np.linalg.qr(rng.standard_normal((5, 5)))[0]
    for A in (np.zeros((5, 5)), np.eye(6), np.triu(rng.standard_normal((7, 7))), np.diag([3.0, 3.0, 1.0, 1.0]),
              np.kron(np.eye(3), np.array([[0.0, -2.0], [2.0, 0.0]])), np.ones((6, 6)), np.diag(np.ones(6), 1),
              Q @ np.diag([1.0, 1e-8, 1e-16, 0.0, -0.5]) @ Q.T):
        assert _match(eig(A), np.linalg.eigvals(A)) <= 1e-13 * max(1.0, np.abs(A).max())
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import tnr_oracle as o
    s = o.TRG(o.classical_ising())
    o.run(s, o.truncrank(24), o.maxiter(10))
    M = o.transfer_matrix(s)
    ref = np.linalg.eigvals(M)
    assert _match(eig(M), ref) <= 1e-13 * np.abs(ref).max()


def test_cft_and_gsd_host_postprocessing(tnr, oracle, monkeypatch):
    """cft_data and ground_state_degeneracy sort and filter the device's transfer-matrix
    eigenvalues on the host (src/utility/cft.jl:17-36, 296-309); fed the oracle's eigenvalues,
    in a scrambled order, they return the oracle's values."""
    o = oracle
    s = o.TRG(o.classical_ising())
    o.run(s, o.truncrank(16), o.maxiter(8))
    lam = np.linalg.eigvals(o.transfer_matrix(s))
    rng = np.random.default_rng(1)
    monkeypatch.setattr(tnr, "transfer_eigvals", lambda scheme, unitcell=1: lam[rng.permutation(len(lam))])
    np.testing.assert_allclose(tnr.cft_data(None), o.cft_data(s), rtol=1e-12, atol=1e-14)
    assert tnr.ground_state_degeneracy(None) == pytest.approx(o.ground_state_degeneracy(s), rel=1e-12)


def test_stopping_criteria(tnr, oracle):
    """maxiter, convcrit, trivial_convcrit, ``&`` (MultipleCrit) and ATRG_3D_convcrit follow
    src/utility/stopping.jl and src/schemes/atrg3d.jl:98 (evaluated on host data, as run! does)."""
    data = [1.0, 0.5, 0.25]
    assert tnr.maxiter(3)(2, data) and not tnr.maxiter(3)(3, data)
    assert tnr.trivial_convcrit(0.1)(1, data) and not tnr.trivial_convcrit(0.3)(1, data)
    both = tnr.maxiter(10) & tnr.convcrit(0.2, lambda steps, d: d[-1])
    assert isinstance(both, tnr.MultipleCrit) and both(3, data) and not both(10, data)
    assert not (tnr.maxiter(10) & tnr.convcrit(0.3, lambda steps, d: d[-1]))(3, data)
    assert tnr.ATRG_3D_convcrit(3, [2.0]) == pytest.approx(abs(np.log(2.0)) / 64.0)
    with pytest.raises(TypeError):
        tnr.run(None, tnr.truncrank(4), 5)


def test_new_entry_points_refuse_null_handles(tnr):
    """Every entry point added for the schemes around the hot path returns TNR_ERR_INVALID_ARG
    on a NULL handle or NULL outputs instead of crashing (no device needed)."""
    L = tnr.lib()
    bad = header_defines()["TNR_ERR_INVALID_ARG"]
    d = ctypes.c_double()
    n = ctypes.c_size_t()
    buf = (ctypes.c_double * 8)()
    dims = (ctypes.c_int64 * 8)()
    nl = ctypes.c_int()
    assert L.tnr_set_finalizer(None, 1) == bad
    assert L.tnr_transfer_eigvals(None, 1, buf, buf, 8, ctypes.byref(n)) == bad
    assert L.tnr_gu_wen_ratio(None, ctypes.byref(d), ctypes.byref(d)) == bad
    assert L.tnr_central_charge(None, 1.0, ctypes.byref(d)) == bad
    assert L.tnr_run_correlation(None, 8, 4, buf, 8, ctypes.byref(n)) == bad
    assert L.tnr_correlation_ratio(None, ctypes.byref(d)) == bad
    assert L.tnr_get_impurity_tensor(None, 0, buf, 8, dims, ctypes.byref(nl)) == bad
    assert L.tnr_finalize_impurity(None, buf) == bad
    assert L.tnr_run_impurity(None, 8, 4, 1, buf, 8, ctypes.byref(n)) == bad
    u64 = ctypes.c_uint64()
    assert L.tnr_decomposition_stats(None, ctypes.byref(u64), ctypes.byref(u64), ctypes.byref(nl)) == bad
    h = ctypes.c_void_p()
    assert L.tnr_create(ctypes.byref(h), 10, 4, dims, buf, None) == bad       # unknown kind
    assert L.tnr_create(ctypes.byref(h), header_defines()["TNR_ATRG_3D"], 4, dims, buf, None) == bad   # 6 legs


def test_impurity_constructors_check_arguments(tnr):
    """The impurity constructors refuse mismatched tensors in the host layer and NULL tensors
    or non-square legs in the C ABI, before any device work."""
    T = tnr.classical_ising("Trivial")
    with pytest.raises(ValueError):
        tnr.ImpurityTRG(T, np.ones((2, 2, 2, 3)), T, T, T)
    with pytest.raises(ValueError):
        tnr.ImpurityHOTRG(T, T, np.ones((2, 2, 2)), T)
    L = tnr.lib()
    bad = header_defines()["TNR_ERR_INVALID_ARG"]
    a = np.asfortranarray(T.array)
    p = a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    dims = (ctypes.c_int64 * 4)(*a.shape)
    h = ctypes.c_void_p()
    assert L.tnr_create_impurity_trg(ctypes.byref(h), dims, p, p, p, None, p, None) == bad
    assert L.tnr_create_impurity_hotrg(ctypes.byref(h), dims, p, None, p, p, None) == bad
    ragged = (ctypes.c_int64 * 4)(2, 2, 3, 2)
    assert L.tnr_create_impurity_trg(ctypes.byref(h), ragged, p, p, p, p, p, None) == bad
    assert not h.value


def _split_top(args):
    out, depth, cur = [], 0, ""
    for ch in args:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return [a for a in out if a]


def _header_prototypes():
    protos = {}
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", f)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        for m in re.finditer(r"([A-Za-z_][\w \t\*]*?)\b(tnr_[a-z0-9_]+)\s*\(([^;{()]*)\)\s*;", txt):
            args = " ".join(m.group(3).split())
            n = 0 if args in ("", "void") else len(_split_top(args))
            protos[m.group(2)] = (" ".join(m.group(1).split()), n)
    return protos


def test_julia_ccalls_match_header():
    """Every ccall of the Julia binding names a declared entry point with the declared number of
    arguments and a matching return type (the binding cannot run here: no Julia)."""
    protos = _header_prototypes()
    jl = open(os.path.join(ROOT, "tnrkit.jl_gb300", "julia", "TNRKitGB300.jl")).read()
    calls = re.findall(r"ccall\(\(:(tnr_\w+),\s*libtnr\),\s*(\w+),\s*\((.*?)\)\s*,", jl, flags=re.S)
    assert len(calls) >= 20
    ret_map = {"Cint": "int", "Cvoid": "void", "Csize_t": "size_t", "UInt64": "uint64_t", "Cdouble": "double"}
    for name, ret, args in calls:
        assert name in protos, name
        c_ret, c_n = protos[name]
        assert len(_split_top(args)) == c_n, (name, args, c_n)
        assert ret_map.get(ret, ret) == c_ret.replace("const ", "").strip() or \
            (ret in ("Cstring", "Ptr{UInt8}") and "char" in c_ret), (name, ret, c_ret)
