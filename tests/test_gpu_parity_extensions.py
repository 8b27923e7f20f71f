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
    """CorrelationHOTRG (src/schemes/correlationhotrg.jl:94-250, finalize.jl:104-124) with the
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
        # the reference's own expression over the scheme's fields (test/schemes.jl:506)
        tr = lambda t: abs(np.einsum('abba->', t))        # noqa: E731
        assert tr(s.Timp_final) / tr(s.Tpure) == pytest.approx(got, rel=1e-12)
        if beta == tnr.ising_βc:
            f = tnr.free_energy([x[0] for x in d], beta, scalefactor=4.0, initial_size=4.0)
            assert f == pytest.approx(tnr.f_onsager, rel=1e-4)
        if beta < 1.0:
            To, impo = o.classical_ising(beta, "Trivial"), o.classical_ising_impurity(beta)
            so = o.CorrelationHOTRG(To, impo, impo, 5)
            o.run(so, o.truncrank(16), o.maxiter(25))
            assert got == pytest.approx(o.correlation_ratio(so), rel=1e-8)


ISING_CFT_EXACT = (1 / 8, 1.0)        # src/models/ising.jl:3-4


@pytest.mark.parametrize("cls,chi,n,tol1,tol2", [("TRG", 24, 10, 2e-4, 1e-2), ("BTRG", 24, 10, 3e-4, 2e-2),
                                                 ("HOTRG", 16, 4, 6e-4, 1e-2)])
def test_cft_data(tnr, oracle, cls, chi, n, tol1, tol2):
    """cft_data (src/utility/cft.jl:5-73) from the device's transfer-matrix eigenvalues: the
    reference's Ising checks (test/schemes.jl:25-33, 64-70, 101-107) and the first eight
    values against the oracle to 1e-9."""
    o = oracle
    s = getattr(tnr, cls)(tnr.classical_ising())
    tnr.run(s, tnr.truncrank(chi), tnr.maxiter(n))
    so = getattr(o, cls)(o.classical_ising())
    o.run(so, o.truncrank(chi), o.maxiter(n))
    cft, ref = tnr.cft_data(s), o.cft_data(so)
    assert cft[1] == pytest.approx(ISING_CFT_EXACT[0], rel=tol1)
    assert cft[2] == pytest.approx(ISING_CFT_EXACT[1], rel=tol2)
    np.testing.assert_allclose(cft[:8], ref[:8], rtol=0, atol=1e-9)


@pytest.mark.parametrize("cls,chi", [("TRG", 16), ("BTRG", 16), ("HOTRG", 12)])
def test_ground_state_degeneracy_and_gu_wen(tnr, oracle, cls, chi):
    """ground_state_degeneracy and gu_wen_ratio (src/utility/cft.jl:278-396) at beta_c -+ 0.01
    after 20 steps: the reference's checks (1 and 2, rtol 1e-2; test/schemes.jl:35-54) and the
    oracle's values to 1e-8 where the run has no tie at the cut (BTRG at beta_c - 0.01 has one)."""
    o = oracle
    for db, want in [(-0.01, 1.0), (0.01, 2.0)]:
        s = getattr(tnr, cls)(tnr.classical_ising("Z2", tnr.ising_βc + db))
        tnr.run(s, tnr.truncrank(chi), tnr.maxiter(20))
        gsd, (x1, x2) = tnr.ground_state_degeneracy(s), tnr.gu_wen_ratio(s)
        for v in (gsd, x1, x2):
            assert v == pytest.approx(want, rel=1e-2)
        if cls == "BTRG" and db < 0:
            continue
        so = getattr(o, cls)(o.classical_ising(o.ISING_BETA_C + db))
        o.run(so, o.truncrank(chi), o.maxiter(20))
        assert gsd == pytest.approx(o.ground_state_degeneracy(so), rel=1e-8)
        np.testing.assert_allclose((x1, x2), o.gu_wen_ratio(so), rtol=1e-8)


def test_central_charge_trg(tnr, oracle):
    """finalize_central_charge! (src/utility/finalize.jl:145-148, cft.jl:256-260) on TRG at
    beta_c, truncrank(24): c = 1/2 to 1e-2 and the oracle's value to 1e-9 at steps 13, 14."""
    o = oracle
    s, so = tnr.TRG(tnr.classical_ising()), o.TRG(o.classical_ising())
    tnr.run(s, tnr.truncrank(24), tnr.maxiter(12))
    o.run(so, o.truncrank(24), o.maxiter(12))
    for _ in range(2):
        tnr.step(s, tnr.truncrank(24))
        o.step(so, 24)
        c, co = tnr.central_charge(s, tnr.finalize(s)), o.central_charge(so, o.finalize(so))
        assert c == pytest.approx(0.5, abs=1e-2)
        assert c == pytest.approx(co, abs=1e-9)


@pytest.mark.parametrize("cls,chi,n", [("TRG", 16, 6), ("BTRG", 16, 6), ("HOTRG", 12, 4)])
def test_two_by_two_finalizer(tnr, oracle, cls, chi, n):
    """run! with two_by_two_Finalizer (src/utility/finalize.jl:17-41,151): every entry
    n^(1/4) against the oracle to 1e-10; the scheme keeps the finalizer for a later finalize."""
    o = oracle
    s = getattr(tnr, cls)(tnr.classical_ising())
    d = tnr.run(s, tnr.truncrank(chi), tnr.maxiter(n), tnr.two_by_two_Finalizer)
    do = o.run(getattr(o, cls)(o.classical_ising()), o.truncrank(chi), o.maxiter(n),
               finalizer=o.finalize_two_by_two)
    np.testing.assert_allclose(d, do, rtol=1e-10)
    assert tnr.finalize(s) == pytest.approx(1.0, rel=1e-12)


def test_atrg(tnr, oracle):
    """ATRG (src/schemes/atrg.jl:38-81) on the Z2 Ising tensor at beta_c: every norm of
    truncrank(16), maxiter(6) against the oracle to 1e-10 (ATRG's network pairs the factors of
    each SVD, so it is basis-free); then the reference's checks (test/schemes.jl:130-165):
    truncrank(24), maxiter(25): f to 3e-6 with scalefactor 4; maxiter(3): the first two scaling
    dimensions to 1e-2; and GSD / X1 / X2 at beta_c -+ 0.01 (truncrank(16), 20 steps)."""
    o = oracle
    d = np.array(tnr.run(tnr.ATRG(tnr.classical_ising()), tnr.truncrank(16), tnr.maxiter(6)))
    do = np.array(o.run(o.ATRG(o.classical_ising()), o.truncrank(16), o.maxiter(6)))
    np.testing.assert_allclose(d, do, rtol=1e-10)
    d = tnr.run(tnr.ATRG(tnr.classical_ising()), tnr.truncrank(24), tnr.maxiter(25))
    assert tnr.free_energy(d, tnr.ising_βc, scalefactor=4.0) == pytest.approx(tnr.f_onsager, rel=3e-6)
    s = tnr.ATRG(tnr.classical_ising())
    tnr.run(s, tnr.truncrank(24), tnr.maxiter(3))
    cft = tnr.cft_data(s)
    assert cft[1] == pytest.approx(ISING_CFT_EXACT[0], rel=1e-2)
    assert cft[2] == pytest.approx(ISING_CFT_EXACT[1], rel=1e-2)
    for db, want in [(-0.01, 1.0), (0.01, 2.0)]:
        s = tnr.ATRG(tnr.classical_ising("Z2", tnr.ising_βc + db))
        tnr.run(s, tnr.truncrank(16), tnr.maxiter(20))
        x1, x2 = tnr.gu_wen_ratio(s)
        for v in (tnr.ground_state_degeneracy(s), x1, x2):
            assert v == pytest.approx(want, rel=1e-2)


def test_atrg3d(tnr, oracle):
    """ATRG_3D (src/schemes/atrg3d.jl:35-90) on the 3D Ising tensor: every norm of
    truncrank(6), maxiter(5) against the oracle to 1e-10 (the engine's QR factors differ from
    LAPACK's by an orthogonal factor, which the oblique projectors do not see); and the
    reference's check (test/schemes.jl:365-373): truncrank(12), maxiter(25), f = -3.507 to 5e-3."""
    o = oracle
    d = np.array(tnr.run(tnr.ATRG_3D(tnr.classical_ising_3D()), tnr.truncrank(6), tnr.maxiter(5)))
    do = np.array(o.run(o.ATRG_3D(o.classical_ising_3D()), o.truncrank(6), o.maxiter(5)))
    np.testing.assert_allclose(d, do, rtol=1e-10)
    d = tnr.run(tnr.ATRG_3D(tnr.classical_ising_3D()), tnr.truncrank(12), tnr.maxiter(25))
    assert tnr.free_energy(d, tnr.ising_βc_3D, scalefactor=8.0) == pytest.approx(-3.507, rel=5e-3)


def test_convcrit_run(tnr, oracle):
    """run! with maxiter(30) & convcrit (src/utility/stopping.jl:7-22, evaluated on the host
    after every device step): TRG on the Ising model at beta = 0.50, truncrank(16), stopping
    once successive norms agree to 1e-8 (step 13 in the oracle, well before maxiter); the norms
    equal the oracle's maxiter run of as many steps.  beta = 0.50 is well conditioned: the
    oracle's own norms move by < 1e-14 under a 1e-14 input perturbation there, while at
    beta = 0.40 steps 14-16 sit at a near-tie of the cut and move by 1e-6
    (test_oracle_conditioning.py)."""
    o = oracle
    crit = tnr.maxiter(30) & tnr.convcrit(1e-8, lambda steps, d: abs(d[-1] / d[-2] - 1))
    d = tnr.run(tnr.TRG(tnr.classical_ising("Trivial", 0.50)), tnr.truncrank(16), crit)
    assert 2 < len(d) < 31
    do = o.run(o.TRG(o.classical_ising(0.50, "Trivial")), o.truncrank(16), o.maxiter(len(d) - 1))
    np.testing.assert_allclose(d, do, rtol=1e-10)


def test_cft_data_unitcell2(tnr, oracle):
    """cft_data and ground_state_degeneracy with unitcell = 2 (src/utility/cft.jl:7-15: two
    tensors on the ring, a 144 x 144 transfer matrix at truncrank(12)) against the oracle."""
    o = oracle
    s, so = tnr.TRG(tnr.classical_ising()), o.TRG(o.classical_ising())
    tnr.run(s, tnr.truncrank(12), tnr.maxiter(8))
    o.run(so, o.truncrank(12), o.maxiter(8))
    np.testing.assert_allclose(tnr.cft_data(s, unitcell=2)[:8], o.cft_data(so, unitcell=2)[:8], rtol=0, atol=1e-9)
    assert tnr.ground_state_degeneracy(s, 2) == pytest.approx(o.ground_state_degeneracy(so, 2), rel=1e-9)


def test_phi4_and_sixvertex_models(tnr, oracle):
    """Models of test/models.jl:17-23,89-121 through the tested TRG and ImpurityHOTRG paths.
    Their late-step norms sit near ties at the cut (the oracle's own move by 3e-7 to 2e-2 under a
    1e-14 perturbation), while f and the order parameter move by < 1e-13: those are held.  TRG,
    truncrank(16), maxiter(25): the real phi^4 f (Trivial, K = 10, mu0 = -1) against the reference's
    printed 0.4241912271276211 to 1e-10, the six-vertex f against the oracle's to 1e-10; the phi^4
    ImpurityHOTRG order parameter at mu0 = -2 against the reference's 1.5317112652447245 to 1e-10."""
    o = oracle
    d = tnr.run(tnr.TRG(tnr.phi4_real(10, -1.0, 1.0, symmetry="Trivial")), tnr.truncrank(16), tnr.maxiter(25))
    assert tnr.free_energy(d, -1.0) == pytest.approx(0.4241912271276211, rel=1e-10)
    # complex phi^4 (bond dimension 36): the oracle's own f moves by up to 1.1e-9 under a 1e-14
    # input perturbation (test_oracle_conditioning.py), so f is held to 5e-9 against the oracle
    # and to the same bar against the reference's printed 0.7583605364656325
    d = tnr.run(tnr.TRG(tnr.phi4_complex("Trivial", 6, -1.0, 1.0)), tnr.truncrank(16), tnr.maxiter(25))
    do = o.run(o.TRG(o.phi4_complex(6, -1.0, 1.0)), o.truncrank(16), o.maxiter(25))
    assert tnr.free_energy(d, -1.0) == pytest.approx(o.free_energy(do, -1.0), rel=5e-9)
    assert tnr.free_energy(d, -1.0) == pytest.approx(0.7583605364656325, rel=5e-9)
    d = tnr.run(tnr.TRG(tnr.sixvertex()), tnr.truncrank(16), tnr.maxiter(25))
    do = o.run(o.TRG(o.sixvertex()), o.truncrank(16), o.maxiter(25))
    assert tnr.free_energy(d, 1.0) == pytest.approx(o.free_energy(do, 1.0), rel=1e-10)
    args = (10, -2.0, 1.0)
    s = tnr.ImpurityHOTRG(tnr.phi4_real(*args, symmetry="Trivial"), tnr.phi4_real_imp1(*args), tnr.phi4_real_imp1(*args),
                          tnr.phi4_real_imp2(*args))
    d = tnr.run(s, tnr.truncrank(16), tnr.maxiter(25))
    assert d[-1][3] / d[-1][0] == pytest.approx(1.5317112652447245, rel=1e-10)
