"""Pins the CPU oracle against the reference's own golden values and test tolerances.

Golden values: README.md:78-93 (BTRG, Z2 Ising, chi=16, 25 iterations) and the
free-energy tolerances of test/schemes.jl and test/models.jl.
"""
import math

import numpy as np
import pytest


def _f(o, scheme, chi, n, beta, sf):
    data = o.run(scheme, o.truncrank(chi), o.maxiter(n))
    return data, o.free_energy(data, beta, scalefactor=sf)


@pytest.mark.parametrize("symmetry", ["Z2", "Trivial"])
def test_readme_btrg_golden(oracle, symmetry):
    # README.md:78-93: 26 norms, f = -2.1096504926141826902647832, rel. err 3.1e-7
    o = oracle
    data, f = _f(o, o.BTRG(o.classical_ising(o.ISING_BETA_C, symmetry)), 16, 25, o.ISING_BETA_C, 2.0)
    assert len(data) == 26
    assert f == pytest.approx(-2.1096504926141826902647832, rel=1e-14, abs=0)
    assert abs((f - o.F_ONSAGER) / o.F_ONSAGER) == pytest.approx(3.1e-7, rel=0.01)


@pytest.mark.parametrize("cls,chi,sf,rtol", [
    ("TRG", 24, 2.0, 2e-6),     # test/schemes.jl:18-23
    ("BTRG", 24, 2.0, 6e-8),    # test/schemes.jl:57-62
    ("HOTRG", 16, 4.0, 6e-7),   # test/schemes.jl:94-99
])
def test_schemes_onsager(oracle, cls, chi, sf, rtol):
    o = oracle
    _, f = _f(o, getattr(o, cls)(o.classical_ising()), chi, 25, o.ISING_BETA_C, sf)
    assert f == pytest.approx(o.F_ONSAGER, rel=rtol)


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
    # src/schemes/btrg.jl:156-164: values below eps^(3/4) are left unchanged
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
