"""GPU parity of ImpurityTRG and CorrelationHOTRG against the oracle, through the C ABI.

ImpurityTRG's plaquette norm after a step depends on the basis each SVD picks (signs and
rotations inside degenerate groups); the engine fixes a canonical basis inside degenerate
groups (degenerate_basis), which keeps the Z2-odd impurity's degenerate pairs parity-pure.
CorrelationHOTRG uses one isometry for every tensor of a step, so all its outputs are
basis-free.  This file runs after the other GPU tests.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tnr():
    import __graft_entry__ as ge
    ge.build()
    return ge.package()


def test_impurity_trg(tnr, oracle):
    """ImpurityTRG (src/schemes/impuritytrg.jl:63-91, finalize.jl:75-88) with the
    magnetisation impurity on site 1, truncrank(16).  The plaquette norm after a step
    depends on the sign each SVD gives its kept vectors (the factors of one SVD land on
    different sites), which the reference leaves to LAPACK and the engine to its own SVD;
    so the bar is the gauge-free part: the pure norms of every step and the plaquette norm
    before the first step to 1e-10, and the reference's low-temperature magnetisation check
    (test/schemes.jl:470-480) with <sigma> against the oracle's (sign-independent) value."""
    o = oracle
    beta, h = 0.5, 0.05
    T, imp = tnr.classical_ising("Trivial", beta, h=h), tnr.classical_ising_impurity(beta, h)
    To, impo = o.classical_ising(beta, "Trivial", h=h), o.classical_ising_impurity(beta, h)
    d = np.array(tnr.run(tnr.ImpurityTRG(T, imp, T, T, T), tnr.truncrank(16), tnr.maxiter(6)))
    do = np.array(o.run(o.ImpurityTRG(To, impo, To, To, To), o.truncrank(16), o.maxiter(6)))
    assert d.shape == do.shape == (7, 2)
    np.testing.assert_allclose(d[:, 0], do[:, 0], rtol=1e-10)
    np.testing.assert_allclose(d[0, 1], do[0, 1], rtol=1e-10)
    assert np.all(np.isfinite(d)) and np.all(d[:, 1] >= 0)
    beta, h = 2.0, 1e-6
    T, imp = tnr.classical_ising("Trivial", beta, h=h), tnr.classical_ising_impurity(beta, h)
    d = tnr.run(tnr.ImpurityTRG(T, imp, T, T, T), tnr.truncrank(16), tnr.maxiter(25))
    To, impo = o.classical_ising(beta, "Trivial", h=h), o.classical_ising_impurity(beta, h)
    do = o.run(o.ImpurityTRG(To, impo, To, To, To), o.truncrank(16), o.maxiter(25))
    got = d[-1][1] / d[-1][0]
    assert got == pytest.approx(1.0, rel=1e-4)
    assert got == pytest.approx(do[-1][1] / do[-1][0], rel=1e-8)


def test_impurity_trg_high_temperature(tnr):
    """The reference's high-temperature check (test/schemes.jl:454-467): beta = 0.1, no field,
    truncrank(16), maxiter(25): |<sigma>| = n_imp / n_pure of the last step <= 1e-4.  It needs
    parity-pure vectors inside the degenerate pairs of every SVD, which the canonical basis
    gives; every step's ratio is held, not only the last."""
    T, imp = tnr.classical_ising("Trivial", 0.1), tnr.classical_ising_impurity(0.1)
    d = tnr.run(tnr.ImpurityTRG(T, imp, T, T, T), tnr.truncrank(16), tnr.maxiter(25))
    assert len(d) == 26
    assert max(abs(x[1] / x[0]) for x in d) <= 1e-4


def test_correlation_hotrg(tnr, oracle):
    """CorrelationHOTRG (src/schemes/correlationhotrg.jl:92-250, finalize.jl:104-124) with the
    magnetisation impurity at both ends.  At beta_c, dist 2, truncrank(16), 6 steps, every
    step's three norms against the oracle to 1e-10 (the phase-1 traces of the Z2-odd
    impurities vanish up to rounding: an absolute floor of 1e-12 of the largest norm); then
    the reference's own checks at dist 5, 25 steps (test/schemes.jl:483-531): Onsager's f to
    1e-4 and the correlation |tr Timp_final| / |tr Tpure| at beta = 0.2, beta_c and 3, each
    against the reference's value and (beta = 0.2, beta_c) the oracle's to 1e-8."""
    o = oracle
    T, imp = tnr.classical_ising("Trivial"), tnr.classical_ising_impurity()
    To, impo = o.classical_ising(o.ISING_BETA_C, "Trivial"), o.classical_ising_impurity()
    d = np.array(tnr.run(tnr.CorrelationHOTRG(T, imp, imp, 2), tnr.truncrank(16), tnr.maxiter(6)))
    do = np.array(o.run(o.CorrelationHOTRG(To, impo, impo, 2), o.truncrank(16), o.maxiter(6)))
    assert d.shape == do.shape == (6, 3)
    np.testing.assert_allclose(d, do, rtol=1e-10, atol=1e-12 * np.abs(do).max())
    for beta, want, rtol in [(0.2, 7.396177e-6, 1e-5), (tnr.ising_βc, 0.2981409, 1e-5), (3.0, 1.0, 1e-4)]:
        T, imp = tnr.classical_ising("Trivial", beta), tnr.classical_ising_impurity(beta)
        s = tnr.CorrelationHOTRG(T, imp, imp, 5)
        d = tnr.run(s, tnr.truncrank(16), tnr.maxiter(25))
        assert len(d) == 25
        got = s.correlation()
        assert got == pytest.approx(want, rel=rtol)
        if beta == tnr.ising_βc:
            f = tnr.free_energy([x[0] for x in d], beta, scalefactor=4.0, initial_size=4.0)
            assert f == pytest.approx(tnr.f_onsager, rel=1e-4)
        if beta < 1.0:
            To, impo = o.classical_ising(beta, "Trivial"), o.classical_ising_impurity(beta)
            so = o.CorrelationHOTRG(To, impo, impo, 5)
            o.run(so, o.truncrank(16), o.maxiter(25))
            assert got == pytest.approx(o.correlation_ratio(so), rel=1e-8)
