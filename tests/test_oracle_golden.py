"""Pins the CPU oracle against the reference's own golden values and test tolerances.

Golden values: tests/golden/reference_golden.json, extracted from the reference's README.md
(BTRG, Z2 Ising, chi=16, 25 iterations) and the free-energy checks of test/schemes.jl by
tests/golden/make_golden.py (each entry records its file and line); the free-energy
tolerances of test/models.jl are cited inline below.
"""
import json
import math
import os

import numpy as np
import pytest

GOLDEN = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                     "reference_golden.json"), encoding="utf-8"))


def _f(o, scheme, chi, n, beta, sf):
    data = o.run(scheme, o.truncrank(chi), o.maxiter(n))
    return data, o.free_energy(data, beta, scalefactor=sf)


@pytest.mark.parametrize("symmetry", ["Z2", "Trivial"])
def test_readme_btrg_golden(oracle, symmetry):
    # README.md: 26 norms, the printed f to every digit FP64 holds, and its printed relative error
    g = GOLDEN["readme_btrg"]
    o = oracle
    data, f = _f(o, o.BTRG(o.classical_ising(o.ISING_BETA_C, symmetry)), g["chi"], g["maxiter"], o.ISING_BETA_C, 2.0)
    assert len(data) == g["maxiter"] + 1
    assert f == pytest.approx(float(g["f"]), rel=1e-14, abs=0)
    assert abs((f - o.F_ONSAGER) / o.F_ONSAGER) == pytest.approx(g["rel_err_onsager"], rel=0.01)


@pytest.mark.parametrize("case", GOLDEN["schemes"], ids=lambda c: c["scheme"])
def test_schemes_onsager(oracle, case):
    # test/schemes.jl: each scheme's free energy against Onsager's at the reference's rtol
    o = oracle
    _, f = _f(o, getattr(o, case["scheme"])(o.classical_ising()), case["chi"], case["maxiter"], o.ISING_BETA_C,
              case["scalefactor"])
    assert f == pytest.approx(o.F_ONSAGER, rel=case["rtol"])


def test_models_trg16(oracle):
    # test/models.jl:5-39 (the Trivial / Z_N models on the hot path), TRG chi=16, rtol 1e-3
    o = oracle
    b3 = 2.0 * math.log(math.sqrt(3) + 1) / 3
    b4 = math.log(math.sqrt(2) + 1)
    cases = [
        (o.classical_ising(symmetry="Trivial"), o.ISING_BETA_C, o.F_ONSAGER),
        (o.classical_ising(), o.ISING_BETA_C, o.F_ONSAGER),
        (o.classical_clock(3, b3, "Trivial"), b3, -4.17924244901635),
        (o.classical_clock(3, b3), b3, -4.17924244901635),
        (o.classical_clock(4, b4, "Trivial"), b4, 2 * o.F_ONSAGER),
        (o.classical_clock(4, b4), b4, 2 * o.F_ONSAGER),
        (o.classical_potts(3, symmetry="Trivial"), o.potts_beta_c(3), -4.119552029995684),
        (o.classical_potts(3), o.potts_beta_c(3), -4.119552029995684),
    ]
    for T, beta, ans in cases:
        _, f = _f(o, o.TRG(T), 16, 25, beta, 2.0)
        assert f == pytest.approx(ans, rel=1e-3)


@pytest.mark.slow
@pytest.mark.parametrize("symmetry,ans", [("Z2", -3.507), ("Trivial", -3.508)])
def test_hotrg3d_chi8(oracle, symmetry, ans):
    # test/schemes.jl:376-383 and test/models.jl:29-32,80-86: chi=8, 25 iterations, sf=8, rtol 1e-3
    o = oracle
    _, f = _f(o, o.HOTRG_3D(o.classical_ising_3D(symmetry=symmetry)), 8, 25, o.ISING_BETA_C_3D, 8.0)
    assert f == pytest.approx(ans, rel=1e-3)


def test_symmetric_equals_dense(oracle):
    """Z2 block-sparse and dense decompositions give the same norms (no ties at the cut here)."""
    o = oracle
    for cls in ("TRG", "HOTRG"):
        d1 = o.run(getattr(o, cls)(o.classical_ising(symmetry="Z2")), o.truncrank(12), o.maxiter(8))
        d2 = o.run(getattr(o, cls)(o.classical_ising(symmetry="Trivial")), o.truncrank(12), o.maxiter(8))
        np.testing.assert_allclose(d1, d2, rtol=1e-11)


def test_free_energy_formula(oracle):
    # src/utility/free_energy.jl:13-20
    o = oracle
    data = [2.0, 3.0, 5.0]
    f = o.free_energy(data, 0.5, scalefactor=4.0, initial_size=2.0)
    x = 1 - math.log(2.0) / math.log(4.0)
    ref = -sum(math.log(z) * 4.0 ** (x - i) for i, z in enumerate(data, 1)) / 0.5
    assert f == pytest.approx(ref, rel=1e-15)


def test_pseudopow(oracle):
    # src/schemes/btrg.jl:50-58: values below eps^(3/4) are left unchanged
    o = oracle
    s = np.array([4.0, 1e-13, 0.25])
    np.testing.assert_allclose(o.pseudopow(s, -0.5), [0.5, 1e-13, 2.0])


def test_maxiter(oracle):
    # src/utility/stopping.jl:18
    c = oracle.maxiter(3)
    assert c(2, None) and not c(3, None)


def test_hotrg3d_gram_positive_semidefinite(oracle):
    """test/schemes.jl:385-397 checks that the HOTRG_3D Gram matrices are positive
    (semi)definite; here on seeded random bosonic 6-leg tensors (fermionic twists are out of
    scope): MM^dag and M^dag M are symmetric with no eigenvalue below -1e-12 of the largest."""
    o = oracle
    rng = np.random.default_rng(4)
    for d in (2, 3):
        A1 = o.Tensor(rng.standard_normal((d,) * 6), 2)
        A2 = o.Tensor(rng.standard_normal((d,) * 6), 2)
        for G in (o._mmdag_3d(A1, A2), o._mdagm_3d(A1, A2)):
            M = G.a.reshape(d * d, d * d)
            assert np.allclose(M, M.T, atol=1e-12 * np.abs(M).max())
            w = np.linalg.eigvalsh(M)
            assert w.min() >= -1e-12 * w.max()


@pytest.mark.parametrize("cls", ["TRG", "BTRG", "HOTRG"])
@pytest.mark.parametrize("symmetry", ["Trivial", "Z2"])
def test_space_consistency_chi7(oracle, cls, symmetry):
    """test/spaces.jl:6-24: each scheme runs 25 iterations at chi = 7 on Trivial and Z2
    inputs; here the norms are finite and positive and the free energy is within 1e-3 of
    Onsager's (test/models.jl tolerance)."""
    o = oracle
    data = o.run(getattr(o, cls)(o.classical_ising(o.ISING_BETA_C, symmetry)), o.truncrank(7), o.maxiter(25))
    assert len(data) == 26 and all(np.isfinite(data)) and min(data) > 0
    sf = 4.0 if cls == "HOTRG" else 2.0
    f = o.free_energy(data, o.ISING_BETA_C, sf)
    assert f == pytest.approx(o.F_ONSAGER, rel=1e-3)


def test_impurity_hotrg_onsager(oracle):
    """test/schemes.jl:400-410: ImpurityHOTRG(T, T_imp1, T_imp1, T) on the Ising model at
    beta_c, truncrank(16), maxiter(25): the pure norms give Onsager's f to 6e-7 (sf 4)."""
    o = oracle
    T = o.classical_ising(o.ISING_BETA_C, "Trivial")
    imp = o.classical_ising_impurity()
    data = o.run(o.ImpurityHOTRG(T, imp, imp, T), o.truncrank(16), o.maxiter(25))
    assert len(data) == 26 and all(len(d) == 4 for d in data)
    f = o.free_energy([d[0] for d in data], o.ISING_BETA_C, 4.0)
    assert f == pytest.approx(o.F_ONSAGER, rel=6e-7)


@pytest.mark.parametrize("beta,m2,tol", [(0.2, 0.0, 1e-14), (1.0, 1.0, 1e-2)])
def test_impurity_hotrg_magnetisation_limits(oracle, beta, m2, tol):
    """test/schemes.jl:412-440: <m^2> = n_2 / n of the last step tends to 0 at high
    temperature (atol 1e-14) and to 1 at low temperature (rtol 1e-2), truncrank(8)."""
    o = oracle
    T = o.classical_ising(beta, "Trivial")
    imp = o.classical_ising_impurity(beta)
    data = o.run(o.ImpurityHOTRG(T, imp, imp, o.classical_ising(beta, "Trivial")), o.truncrank(8), o.maxiter(25))
    got = data[-1][3] / data[-1][0]
    if m2 == 0.0:
        assert abs(got) <= tol
    else:
        assert got == pytest.approx(m2, rel=tol)


def test_impurity_trg_onsager(oracle):
    """test/schemes.jl:443-452: ImpurityTRG(T, T_imp, T, T, T) on the Ising model at beta_c,
    truncrank(24), maxiter(25): the pure norms give Onsager's f to 2e-6 (sf 2)."""
    o = oracle
    T = o.classical_ising(o.ISING_BETA_C, "Trivial")
    data = o.run(o.ImpurityTRG(T, o.classical_ising_impurity(), T, T, T), o.truncrank(24), o.maxiter(25))
    assert len(data) == 26 and all(len(d) == 2 for d in data)
    f = o.free_energy([d[0] for d in data], o.ISING_BETA_C)
    assert f == pytest.approx(o.F_ONSAGER, rel=2e-6)


@pytest.mark.parametrize("beta,h,m,tol", [(0.1, 0.0, 0.0, 1e-4), (2.0, 1e-6, 1.0, 1e-4)])
def test_impurity_trg_magnetisation_limits(oracle, beta, h, m, tol):
    """test/schemes.jl:454-480: <sigma> = n_imp / n_pure of the last step tends to 0 at high
    temperature (atol 1e-4) and to 1 at low temperature in a tiny field (rtol 1e-4), chi 16."""
    o = oracle
    T = o.classical_ising(beta, "Trivial", h=h)
    data = o.run(o.ImpurityTRG(T, o.classical_ising_impurity(beta, h=h), T, T, T), o.truncrank(16), o.maxiter(25))
    got = data[-1][1] / data[-1][0]
    if m == 0.0:
        assert abs(got) <= tol
    else:
        assert got == pytest.approx(m, rel=tol)


def test_impurity_trg_plaquette_depends_on_svd_signs(oracle, monkeypatch):
    """The reference's ImpurityTRG contracts factors of an impurity's SVD12 with factors of
    the pure tensor's (src/schemes/impuritytrg.jl:84-88), so its plaquette norm after a step
    moves when an SVD flips the sign of a kept vector, while the pure norms and the
    converged <sigma> = n_imp/n_pure do not.  Random sign flips in the oracle's SVD12 show
    both: the GPU parity test holds the engine to the sign-free quantities only."""
    o = oracle
    beta, h = 0.5, 0.05
    T, imp = o.classical_ising(beta, "Trivial", h=h), o.classical_ising_impurity(beta, h=h)
    a = np.array(o.run(o.ImpurityTRG(T, imp, T, T, T), o.truncrank(16), o.maxiter(3)))
    svd12, rng = o.SVD12, np.random.default_rng(0)

    def flipped(t, chi):
        A, B, s = svd12(t, chi)
        f = rng.choice([-1.0, 1.0], size=s.shape)
        A.a = A.a * f
        B.a = B.a * f[:, None, None]
        return A, B, s

    monkeypatch.setattr(o, "SVD12", flipped)
    b = np.array(o.run(o.ImpurityTRG(T, imp, T, T, T), o.truncrank(16), o.maxiter(3)))
    np.testing.assert_allclose(b[:, 0], a[:, 0], rtol=1e-13)
    assert b[0, 1] == pytest.approx(a[0, 1], rel=1e-13)
    assert np.abs(b[1:, 1] / a[1:, 1] - 1).max() > 1e-3
    T, imp = o.classical_ising(2.0, "Trivial", h=1e-6), o.classical_ising_impurity(2.0, h=1e-6)
    b = o.run(o.ImpurityTRG(T, imp, T, T, T), o.truncrank(16), o.maxiter(25))
    monkeypatch.setattr(o, "SVD12", svd12)
    a = o.run(o.ImpurityTRG(T, imp, T, T, T), o.truncrank(16), o.maxiter(25))
    assert b[-1][1] / b[-1][0] == pytest.approx(a[-1][1] / a[-1][0], rel=1e-10)


def _sector_svd12(o):
    """SVD12 over the sectors of the matrix's exact zeros (the engine's tsvd_sectors): connected
    components of the bipartite graph row r -- column c iff M[r, c] != 0, one SVD per block,
    the chi largest values over all blocks kept (descending, ties in sector order), each
    vector zero outside its sector."""
    def svd12(t, chi):
        d = t.a.shape
        m, n = d[0] * d[1], d[2] * d[3]
        M = t.a.reshape(m, n, order='F')
        parent = list(range(m + n))

        def find(x):
            while parent[x] != x:
                parent[x] = parent[parent[x]]
                x = parent[x]
            return x
        for r, cc in zip(*np.nonzero(M)):
            a_, b_ = find(int(r)), find(m + int(cc))
            if a_ != b_:
                parent[max(a_, b_)] = min(a_, b_)
        comps = {}
        for x in range(m + n):
            comps.setdefault(find(x), []).append(x)
        picks = []
        for nodes in comps.values():
            rows = [x for x in nodes if x < m]
            cols = [x - m for x in nodes if x >= m]
            if rows and cols:
                u, sv, vh = np.linalg.svd(M[np.ix_(rows, cols)], full_matrices=False)
                picks += [(sv[i], rows, cols, u[:, i], vh[i]) for i in range(len(sv))]
        picks.sort(key=lambda p: -p[0])
        k = min(chi, m, n)
        U, S, V = np.zeros((m, k)), np.zeros(k), np.zeros((k, n))
        for t_, (sv_, rows, cols, u, v) in enumerate(picks[:k]):
            S[t_] = sv_
            U[rows, t_] = u
            V[t_, cols] = v
        r = np.sqrt(S)
        A = o.Tensor((U * r).reshape(d[0], d[1], k, order='F'), 2, None, t.N)
        B = o.Tensor((r[:, None] * V).reshape(k, d[2], d[3], order='F'), 1, None, t.N)
        return A, B, S
    return svd12


def test_impurity_trg_high_temperature_needs_parity_pure_vectors(oracle, monkeypatch):
    """The reference's high-temperature check (test/schemes.jl:454-467, |<sigma>| <= 1e-4 at
    beta = 0.1) holds because LAPACK returns parity-pure singular vectors inside the
    degenerate pairs of the Z2-odd impurity's SVD.  Any other orthonormal basis of those
    pairs is an equally valid SVD, yet it mixes parities across sites of the plaquette and
    leaves <sigma> at O(1e-2): random rotations inside every degenerate group show it.  The
    engine's SVD over the sectors of the exact zeros, restated here, keeps every vector in one
    sector: every step's ratio stays within the reference's bar, as LAPACK's own do (both
    reach ~1e-5 at single steps, where degenerate groups inside one sector still leave a basis
    choice), and the pure norms are the plain ones."""
    o = oracle
    svd12, rng = o.SVD12, np.random.default_rng(0)

    def rotated(t, chi):
        A, B, s = svd12(t, chi)
        Q, i = np.eye(len(s)), 0
        while i < len(s):
            j = i + 1
            while j < len(s) and abs(s[j] - s[i]) <= 1e-10 * s[0]:
                j += 1
            if j - i > 1:
                Q[i:j, i:j] = np.linalg.qr(rng.standard_normal((j - i, j - i)))[0]
            i = j
        A.a = np.einsum('abk,kl->abl', A.a, Q)
        B.a = np.einsum('lk,kcd->lcd', Q.T, B.a)
        return A, B, s

    T, imp = o.classical_ising(0.1, "Trivial"), o.classical_ising_impurity(0.1)
    a = o.run(o.ImpurityTRG(T, imp, T, T, T), o.truncrank(16), o.maxiter(25))
    monkeypatch.setattr(o, "SVD12", rotated)
    b = o.run(o.ImpurityTRG(T, imp, T, T, T), o.truncrank(16), o.maxiter(25))
    monkeypatch.setattr(o, "SVD12", _sector_svd12(o))
    c = o.run(o.ImpurityTRG(T, imp, T, T, T), o.truncrank(16), o.maxiter(25))
    np.testing.assert_allclose([x[0] for x in b], [x[0] for x in a], rtol=1e-10)
    np.testing.assert_allclose([x[0] for x in c], [x[0] for x in a], rtol=1e-10)
    assert abs(a[-1][1] / a[-1][0]) <= 1e-4
    assert max(abs(x[1] / x[0]) for x in a) <= 1e-4
    assert max(abs(x[1] / x[0]) for x in b) > 1e-3
    # the sector basis: every step's ratio back under the bar
    assert max(abs(x[1] / x[0]) for x in c) <= 1e-4


def test_impurity_trg_sector_svd_without_zeros_is_the_plain_svd(oracle, monkeypatch):
    """With a field (beta = 2, h = 1e-6) the tensors have no exact zeros: one sector, so the
    sector SVD is the plain SVD and <sigma> is the oracle's to 1e-12.  (A basis rule keyed on
    nearly equal values instead rotated resolved vectors of different parity there: an error
    of 1e-13 s_0 in the odd sector is a 1e-7 relative error in h = 1e-6, and <sigma> moved by
    1.7e-8.)"""
    o = oracle
    T, imp = o.classical_ising(2.0, "Trivial", h=1e-6), o.classical_ising_impurity(2.0, h=1e-6)
    assert np.count_nonzero(T.a) == T.a.size and np.count_nonzero(imp.a) == imp.a.size
    a = o.run(o.ImpurityTRG(T, imp, T, T, T), o.truncrank(16), o.maxiter(25))
    monkeypatch.setattr(o, "SVD12", _sector_svd12(o))
    b = o.run(o.ImpurityTRG(T, imp, T, T, T), o.truncrank(16), o.maxiter(25))
    assert b[-1][1] / b[-1][0] == pytest.approx(a[-1][1] / a[-1][0], rel=1e-12)


def test_correlation_hotrg_onsager(oracle):
    """test/schemes.jl:483-493: CorrelationHOTRG(T, T_imp, T_imp, 5) at beta_c, truncrank(16),
    maxiter(25); the pure norms give Onsager's f to 1e-4 with scalefactor 4, initial_size 4."""
    o = oracle
    T, imp = o.classical_ising(o.ISING_BETA_C, "Trivial"), o.classical_ising_impurity()
    data = o.run(o.CorrelationHOTRG(T, imp, imp, 5), o.truncrank(16), o.maxiter(25))
    assert len(data) == 25 and all(len(d) == 3 for d in data)
    f = o.free_energy([d[0] for d in data], o.ISING_BETA_C, scalefactor=4.0, initial_size=4.0)
    assert f == pytest.approx(o.F_ONSAGER, rel=1e-4)


@pytest.mark.parametrize("beta,want,rtol", [(0.2, 7.396177e-6, 1e-5), (None, 0.2981409, 1e-5), (3.0, 1.0, 1e-4)])
def test_correlation_hotrg_magnetisation_correlation(oracle, beta, want, rtol):
    """test/schemes.jl:495-531: |tr Timp_final| / |tr Tpure| after 25 steps of
    CorrelationHOTRG(T, T_imp, T_imp, 5), truncrank(16): 7.396177e-6 at beta = 0.2, 0.2981409 at
    beta_c (both rtol 1e-5) and 1 at beta = 3 (rtol 1e-4).  The merge happens at step 5: the
    norms switch from (n, n_1, n_2) to (n, n_imp, n_imp) there."""
    o = oracle
    beta = o.ISING_BETA_C if beta is None else beta
    T, imp = o.classical_ising(beta, "Trivial"), o.classical_ising_impurity(beta)
    s = o.CorrelationHOTRG(T, imp, imp, 5)
    data = o.run(s, o.truncrank(16), o.maxiter(25))
    assert s.Timp1 is None and s.Timp2 is None and s.iter == 25
    assert all(d[1] == d[2] for d in data[5:])
    assert o.correlation_ratio(s) == pytest.approx(want, rel=rtol)


def test_correlation_hotrg_rejects_short_runs(oracle):
    """run!(::CorrelationHOTRG) asserts niter > dist; the constructor asserts dist >= 0."""
    o = oracle
    T, imp = o.classical_ising(o.ISING_BETA_C, "Trivial"), o.classical_ising_impurity()
    with pytest.raises(AssertionError):
        o.run(o.CorrelationHOTRG(T, imp, imp, 3), o.truncrank(8), o.maxiter(3))
    with pytest.raises(AssertionError):
        o.CorrelationHOTRG(T, imp, imp, -1)


ISING_CFT_EXACT = (1 / 8, 1.0)        # the first two scaling dimensions above the identity (src/models/ising.jl:3-4)


@pytest.mark.parametrize("cls,chi,n,tol1,tol2", [("TRG", 24, 10, 2e-4, 1e-2), ("BTRG", 24, 10, 3e-4, 2e-2),
                                                 ("HOTRG", 16, 4, 6e-4, 1e-2)])
def test_cft_data_ising(oracle, cls, chi, n, tol1, tol2):
    """test/schemes.jl:25-33, 64-70, 101-107: cft_data of the Z2 Ising tensor at beta_c after
    run!(truncrank(chi), maxiter(n)); the first two scaling dimensions after the identity."""
    o = oracle
    s = getattr(o, cls)(o.classical_ising())
    o.run(s, o.truncrank(chi), o.maxiter(n))
    cft = o.cft_data(s)
    assert cft[0] == 0.0
    assert cft[1] == pytest.approx(ISING_CFT_EXACT[0], rel=tol1)
    assert cft[2] == pytest.approx(ISING_CFT_EXACT[1], rel=tol2)


@pytest.mark.parametrize("cls,chi", [("TRG", 16), ("BTRG", 16), ("HOTRG", 12)])
def test_ground_state_degeneracy_and_gu_wen(oracle, cls, chi):
    """test/schemes.jl:35-54, 72-90, 109-127: 20 steps at beta_c -+ 0.01: the disordered fixed
    point has GSD = X1 = X2 = 1, the ordered one 2 (rtol 1e-2 each)."""
    o = oracle
    for db, want in [(-0.01, 1.0), (0.01, 2.0)]:
        s = getattr(o, cls)(o.classical_ising(o.ISING_BETA_C + db))
        o.run(s, o.truncrank(chi), o.maxiter(20))
        x1, x2 = o.gu_wen_ratio(s)
        assert o.ground_state_degeneracy(s) == pytest.approx(want, rel=1e-2)
        assert x1 == pytest.approx(want, rel=1e-2)
        assert x2 == pytest.approx(want, rel=1e-2)


def test_transfer_matrix_ring(oracle):
    """The unitcell-u transfer matrix is the ring of u tensors of cft.jl:7-15: for u = 1 its
    entries are sum_a T[a, b, c, a], for u = 2 sum_{a1, a2} T[a1, b1, c1, a2] T[a2, b2, c2, a1]
    with rows (b1, b2) and columns (c1, c2)."""
    o = oracle
    rng = np.random.default_rng(3)
    s = o.TRG(o.Tensor(rng.standard_normal((3, 2, 2, 3)), 2, None, 1))
    T = s.T.a
    M1 = o.transfer_matrix(s, 1)
    np.testing.assert_allclose(M1, np.einsum('abca->bc', T), rtol=1e-14)
    M2 = o.transfer_matrix(s, 2).reshape(2, 2, 2, 2)          # [b1, b2, c1, c2]
    np.testing.assert_allclose(M2, np.einsum('xbcy,yefx->becf', T, T), rtol=1e-13)


def test_two_by_two_finalizer(oracle):
    """src/utility/finalize.jl:17-41: the 2 x 2 plaquette norm (BTRG with its bond weights,
    against the network written with explicit diagonal bond matrices); after the division a
    second call returns 1."""
    o = oracle
    for cls in ("TRG", "BTRG"):
        s = getattr(o, cls)(o.classical_ising(o.ISING_BETA_C, "Trivial"))
        o.run(s, o.truncrank(12), o.maxiter(6))
        T = s.T.a
        if cls == "BTRG":
            S1, S2 = np.diag(s.S1), np.diag(s.S2)
            n = abs(np.einsum('kaih,hb,bfjk,cf,gjcl,dg,lied,ea->', T, S2, T, S1, T, S2, T, S1, optimize=True))
        else:
            n = abs(np.einsum('gaed,dbfg,cfbh,heac->', T, T, T, T, optimize=True))
        assert o.finalize_two_by_two(s) == pytest.approx(n ** 0.25, rel=1e-13)
        assert o.finalize_two_by_two(s) == pytest.approx(1.0, rel=1e-13)


def test_central_charge_ising_trg(oracle):
    """finalize_central_charge! (src/utility/finalize.jl:145-148, cft.jl:256-260) on TRG's Ising
    flow at beta_c, truncrank(24): c = 1/2 of the Ising CFT, to 1e-2 between steps 13 and 15."""
    o = oracle
    s = o.TRG(o.classical_ising())
    o.run(s, o.truncrank(24), o.maxiter(12))
    for _ in range(3):
        o.step(s, 24)
        n = o.finalize(s)
        assert o.central_charge(s, n) == pytest.approx(0.5, abs=1e-2)


def test_atrg_ising(oracle):
    """test/schemes.jl:130-165: ATRG on the Z2 Ising tensor.  truncrank(24), maxiter(25): f to
    3e-6 (scalefactor 4); maxiter(3): the first two scaling dimensions to 1e-2; truncrank(16),
    maxiter(20) at beta_c -+ 0.01: GSD, X1, X2 = 1 and 2 to 1e-2."""
    o = oracle
    s = o.ATRG(o.classical_ising())
    data = o.run(s, o.truncrank(24), o.maxiter(25))
    assert o.free_energy(data, o.ISING_BETA_C, scalefactor=4.0) == pytest.approx(o.F_ONSAGER, rel=3e-6)
    s = o.ATRG(o.classical_ising())
    o.run(s, o.truncrank(24), o.maxiter(3))
    cft = o.cft_data(s)
    assert cft[1] == pytest.approx(ISING_CFT_EXACT[0], rel=1e-2)
    assert cft[2] == pytest.approx(ISING_CFT_EXACT[1], rel=1e-2)
    for db, want in [(-0.01, 1.0), (0.01, 2.0)]:
        s = o.ATRG(o.classical_ising(o.ISING_BETA_C + db))
        o.run(s, o.truncrank(16), o.maxiter(20))
        x1, x2 = o.gu_wen_ratio(s)
        for v in (o.ground_state_degeneracy(s), x1, x2):
            assert v == pytest.approx(want, rel=1e-2)


@pytest.mark.slow
def test_atrg3d_ising(oracle):
    """test/schemes.jl:365-373: ATRG_3D on the 3D Ising tensor, truncrank(12), scalefactor 8:
    f = -3.507 (Phys. Rev. B 102, 054432, Fig. 5) to 5e-3.  Ten steps instead of 25: step i
    enters f with weight 8^(1-i), so steps 11..25 move it by < 1e-8."""
    o = oracle
    data = o.run(o.ATRG_3D(o.classical_ising_3D()), o.truncrank(12), o.maxiter(10))
    assert o.free_energy(data, o.ISING_BETA_C_3D, scalefactor=8.0) == pytest.approx(-3.507, rel=5e-3)


def test_atrg3d_projectors_ignore_the_orthogonal_factor(oracle, monkeypatch):
    """ATRG_3D's oblique projectors (src/schemes/atrg3d.jl:54-69) use the R / L factors of
    left_orth / right_orth only through R1 R2 and its SVD, so R -> O R and L -> L O' with any
    orthogonal O, O' leave every norm unchanged: the engine's R = Q^T M from CholeskyQR3 is as
    good as LAPACK's."""
    o = oracle
    rng = np.random.default_rng(4)
    ref = np.array(o.run(o.ATRG_3D(o.classical_ising_3D()), o.truncrank(6), o.maxiter(4)))
    left, right = o._left_orth_r, o._right_orth_l

    def orth(n):
        return np.linalg.qr(rng.standard_normal((n, n)))[0]

    monkeypatch.setattr(o, "_left_orth_r", lambda M: (lambda R: orth(R.shape[0]) @ R)(left(M)))
    monkeypatch.setattr(o, "_right_orth_l", lambda M: (lambda L: L @ orth(L.shape[1]))(right(M)))
    got = np.array(o.run(o.ATRG_3D(o.classical_ising_3D()), o.truncrank(6), o.maxiter(4)))
    np.testing.assert_allclose(got, ref, rtol=1e-11)


@pytest.mark.parametrize("model,temp,answer,rtol", [
    ("sixvertex", 1.0, 1.5 * math.log(0.75), 1e-3),
    ("phi4_trivial", -1.0, 0.4241912271276211, 1e-12),
    ("phi4_z2", -1.0, 0.4232381701937374, 1e-10),
    ("phi4_complex", -1.0, 0.7583605364656325, 1e-9),
])
def test_models_trg16_sixvertex_phi4(oracle, model, temp, answer, rtol):
    """test/models.jl:17-23,37-41: TRG, truncrank(16), maxiter(25) on the six-vertex model (Trivial;
    the reference's bar is rtol 1e-3 against 3/2 log(3/4)) and the real phi^4 model K = 10, mu0 = -1,
    lam = 1 (Trivial and Z2), and the complex phi^4 model (Trivial, K = 6, bond dimension 36).  The
    phi^4 answers are the reference's printed results to 16 digits; the oracle reproduces them to
    6e-16 (real, Trivial), 4e-13 (real, Z2) and 4e-10 (complex), so they are held far tighter than the
    reference's 1e-3."""
    o = oracle
    T = {"sixvertex": lambda: o.sixvertex(), "phi4_trivial": lambda: o.phi4_real(10, -1.0, 1.0, symmetry="Trivial"),
         "phi4_z2": lambda: o.phi4_real(10, -1.0, 1.0),
         "phi4_complex": lambda: o.phi4_complex(6, -1.0, 1.0)}[model]()
    data = o.run(o.TRG(T), o.truncrank(16), o.maxiter(25))
    assert o.free_energy(data, temp) == pytest.approx(answer, rel=rtol)


def test_impurity_hotrg_phi4_order_parameter(oracle):
    """test/models.jl:89-121: ImpurityHOTRG(Tpure, T_imp1, T_imp1, T_imp2) of the real phi^4
    model (Trivial, K = 10, lam = 1), truncrank(16), maxiter(25): <phi^2>-like ratio
    data[end][4] / data[end][1] is 0 in the disordered phase (mu0 = 0, atol 1e-3) and
    1.5317112652447245 in the ordered one (mu0 = -2); the oracle reproduces the latter to 7e-15,
    held here at 1e-12."""
    o = oracle
    for mu0, want in [(0.0, 0.0), (-2.0, 1.5317112652447245)]:
        args = (10, mu0, 1.0)
        Tp, i1, i2 = o.phi4_real(*args, symmetry="Trivial"), o.phi4_real_imp1(*args), o.phi4_real_imp2(*args)
        data = o.run(o.ImpurityHOTRG(Tp, i1, i1, i2), o.truncrank(16), o.maxiter(25))
        got = data[-1][3] / data[-1][0]
        if want == 0.0:
            assert abs(got) <= 1e-3
        else:
            assert got == pytest.approx(want, rel=1e-12)
