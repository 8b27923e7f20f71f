"""GPU parity of the plain FP64 path against the CPU oracle (through the C ABI).

Bar (plain path): every returned norm within 1e-10 relative, every kept singular
value / Gram eigenvalue within 1e-10 of the largest one of its decomposition
(normwise relative: the reference's LAPACK has the same absolute error scale),
and the README golden free energy of BTRG chi=16.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NORM_RTOL = 1e-10
SVAL_TOL = 1e-10


@pytest.fixture(scope="module")
def tnr():
    import __graft_entry__ as ge
    ge.build()
    return ge.package()


def _pair(tnr, o, cls, T, To, chi, n, **kw):
    s = getattr(tnr, cls)(T, **kw)
    so = getattr(o, cls)(To, **({"k": kw["k"]} if "k" in kw else {}))
    d = tnr.run(s, tnr.truncrank(chi), tnr.maxiter(n))
    do = o.run(so, o.truncrank(chi), o.maxiter(n))
    return s, so, np.array(d), np.array(do)


def _check_svals(s, so, nlast):
    got = s.singular_values()
    ref = so.svals[-nlast:]
    assert len(got) == len(ref)
    for g, r in zip(got, ref):
        r = np.asarray(r)[:len(g)]
        assert len(g) == len(r)
        np.testing.assert_allclose(g, r, rtol=0, atol=SVAL_TOL * max(abs(r[0]), 1e-300))


def test_trg_ising_chi16(tnr, oracle):
    o = oracle
    s, so, d, do = _pair(tnr, o, "TRG", tnr.classical_ising("Trivial"), o.classical_ising(symmetry="Trivial"), 16, 25)
    assert len(d) == 26
    np.testing.assert_allclose(d, do, rtol=NORM_RTOL)
    _check_svals(s, so, 2)
    f, fo = tnr.free_energy(d, tnr.ising_βc), o.free_energy(do, o.ISING_BETA_C)
    assert f == pytest.approx(fo, rel=1e-12)
    assert f == pytest.approx(o.F_ONSAGER, rel=1e-3)       # test/models.jl:5-39


def test_btrg_readme_golden(tnr, oracle):
    # README.md:78-93: BTRG, Z2 Ising at beta_c, truncrank(16), maxiter(25)
    o = oracle
    s, so, d, do = _pair(tnr, o, "BTRG", tnr.classical_ising("Z2"), o.classical_ising(symmetry="Z2"), 16, 25)
    np.testing.assert_allclose(d, do, rtol=NORM_RTOL)
    f = tnr.free_energy(d, tnr.ising_βc)
    assert f == pytest.approx(-2.1096504926141826902647832, rel=1e-12)
    _check_svals(s, so, 2)
    s1, s2 = s.S1, s.S2
    np.testing.assert_allclose(np.sort(s1), np.sort(so.S1), rtol=1e-8)
    np.testing.assert_allclose(np.sort(s2), np.sort(so.S2), rtol=1e-8)


def test_hotrg_ising_chi16(tnr, oracle):
    o = oracle
    s, so, d, do = _pair(tnr, o, "HOTRG", tnr.classical_ising("Z2"), o.classical_ising(symmetry="Trivial"), 16, 12)
    np.testing.assert_allclose(d, do, rtol=NORM_RTOL)
    _check_svals(s, so, 2)


def test_hotrg3d_ising(tnr, oracle):
    o = oracle
    s, so, d, do = _pair(tnr, o, "HOTRG_3D", tnr.classical_ising_3D(), o.classical_ising_3D(symmetry="Trivial")
                         if False else o.classical_ising_3D(), 4, 5)
    np.testing.assert_allclose(d, do, rtol=NORM_RTOL)
    _check_svals(s, so, 6)


# chi chosen so that no exactly degenerate pair (charge sectors c and -c) is cut in these
# 10 steps: potts3 cuts one at chi = 13, clock6 at chi = 12
@pytest.mark.parametrize("model,chi", [("potts3", 12), ("clock6", 13)])
def test_zn_models_trg(tnr, oracle, model, chi):
    o = oracle
    if model == "potts3":
        T, To, beta = tnr.classical_potts(3), o.classical_potts(3), tnr.potts_βc(3)
    else:
        T, To, beta = tnr.classical_clock(6, 0.7), o.classical_clock(6, 0.7), 0.7
    s, so, d, do = _pair(tnr, o, "TRG", T, To, chi, 10)
    np.testing.assert_allclose(d, do, rtol=NORM_RTOL)


# tie-free cuts over these 6 steps (the smallest relative gap at the cut is 0.3 for potts3 at
# chi = 16 and 0.08 for clock6 at chi = 13)
@pytest.mark.parametrize("model,chi", [("potts3", 16), ("clock6", 13)])
def test_zn_models_hotrg_blocks(tnr, oracle, model, chi):
    """HOTRG on Z_N tensors runs block by block over the charge sectors (blocked contractions,
    per-sector eigh with the global truncrank cut) and matches the oracle's block-sparse path:
    every norm to 1e-10 and every kept Gram eigenvalue to 1e-10 of the largest."""
    o = oracle
    if model == "potts3":
        T, To = tnr.classical_potts(3), o.classical_potts(3)
    else:
        T, To = tnr.classical_clock(6, 0.7), o.classical_clock(6, 0.7)
    s, so, d, do = _pair(tnr, o, "HOTRG", T, To, chi, 6)
    np.testing.assert_allclose(d, do, rtol=NORM_RTOL)
    _check_svals(s, so, 2)
    assert s.T.shape == so.T.a.shape      # the bond dimensions the sectors hold, as in the oracle


def test_cut_through_degenerate_pair(tnr, oracle):
    """Clock Z6 spectra come in exactly degenerate pairs (charge sectors c and -c); truncrank(12)
    cuts one, so the kept subspace depends on tie-breaking (the reference's order is not
    visible): parity is unpinned there and only the free energy is held, to 1e-4."""
    o = oracle
    s, so, d, do = _pair(tnr, o, "TRG", tnr.classical_clock(6, 0.7), o.classical_clock(6, 0.7), 12, 10)
    f, fo = tnr.free_energy(d, 0.7), o.free_energy(do, 0.7)
    assert f == pytest.approx(fo, rel=1e-4)


def test_btrg_clock6(tnr, oracle):
    o = oracle
    s, so, d, do = _pair(tnr, o, "BTRG", tnr.classical_clock(6, 1.1), o.classical_clock(6, 1.1), 12, 10)
    np.testing.assert_allclose(d, do, rtol=NORM_RTOL)


@pytest.mark.parametrize("chi,seed", [(16, 1), (32, 1)])
def test_hotrg_random_single_step(tnr, oracle, chi, seed):
    """One HOTRG step on the seeded random chi^4 tensor (the single-step workload, small chi)."""
    o = oracle
    T, To = tnr.random_hotrg_tensor(chi, seed), o.random_hotrg_tensor(chi, seed)
    s = tnr.HOTRG(T)
    so = o.HOTRG(To)
    tnr.step(s, tnr.truncrank(chi))
    o.step(so, chi)
    n, no = tnr.finalize(s), o.finalize(so)
    assert n == pytest.approx(no, rel=NORM_RTOL)
    _check_svals(s, so, 2)
    eps = s.truncation_errors()
    ref = np.array([x for pair in so.eps for x in pair])
    np.testing.assert_allclose(eps, ref, rtol=1e-6)


def test_impurity_hotrg(tnr, oracle):
    """ImpurityHOTRG (src/schemes/impurityhotrg.jl:48-84, finalize.jl:91-101) on the Ising
    model at beta_c with the magnetisation impurity, truncrank(16), 4 steps: the four norms
    of every step (pure, +1, -1, second order) against the oracle to 1e-10.  The first-order
    impurity is Z2-odd, so its trace vanishes up to rounding: an absolute floor of 1e-12 of
    the largest norm covers those entries."""
    o = oracle
    T, imp = tnr.classical_ising("Trivial"), tnr.classical_ising_impurity()
    s = tnr.ImpurityHOTRG(T, imp, imp, T)
    d = np.array(tnr.run(s, tnr.truncrank(16), tnr.maxiter(4)))
    To, impo = o.classical_ising(o.ISING_BETA_C, "Trivial"), o.classical_ising_impurity()
    do = np.array(o.run(o.ImpurityHOTRG(To, impo, impo, To), o.truncrank(16), o.maxiter(4)))
    assert d.shape == do.shape == (5, 4)
    np.testing.assert_allclose(d, do, rtol=1e-10, atol=1e-12 * np.abs(do).max())
    # the handle keeps HOTRG's API: one more step and finalize (the four norms) work on it
    tnr.step(s, tnr.truncrank(16))
    assert len(tnr.finalize(s)) == 4


def test_edge_cases(tnr, oracle):
    o = oracle
    T, To = tnr.classical_ising("Trivial"), o.classical_ising(symmetry="Trivial")
    # chi = 1, maxiter(0) runs the body once, finalize_beginning=False
    s = tnr.TRG(T)
    d = tnr.run(s, tnr.truncrank(1), tnr.maxiter(0), finalize_beginning=False)
    do = o.run(o.TRG(To), o.truncrank(1), o.maxiter(0), finalize_beginning=False)
    assert len(d) == len(do) == 1
    np.testing.assert_allclose(d, do, rtol=NORM_RTOL)
    # chi above every bond dimension reached: no truncation in the first steps
    s = tnr.HOTRG(T)
    d = tnr.run(s, tnr.truncrank(200), tnr.maxiter(2))
    do = o.run(o.HOTRG(To), o.truncrank(200), o.maxiter(2))
    np.testing.assert_allclose(d, do, rtol=NORM_RTOL)
    # step / finalize one at a time equals run
    s = tnr.BTRG(T)
    so = o.BTRG(To)
    a = [tnr.finalize(s)] + [(tnr.step(s, tnr.truncrank(8)), tnr.finalize(s))[1] for _ in range(5)]
    b = o.run(so, o.truncrank(8), o.maxiter(5))
    np.testing.assert_allclose(a, b, rtol=NORM_RTOL)
    # invalid chi is refused with a status, the handle stays usable
    with pytest.raises(tnr.TNRError):
        tnr.step(s, tnr.truncrank(0))
    tnr.step(s, tnr.truncrank(8))


def test_batch_equals_single(tnr):
    betas = [0.35, 0.44, 0.52]
    chis = [8, 12, 16]
    schemes = [tnr.BTRG(tnr.classical_ising("Trivial", b)) for b in betas]
    out = tnr.run_batch(schemes, chis, [10, 10, 10])
    for b, chi, d in zip(betas, chis, out):
        s = tnr.BTRG(tnr.classical_ising("Trivial", b))
        ref = tnr.run(s, tnr.truncrank(chi), tnr.maxiter(10))
        np.testing.assert_allclose(d, ref, rtol=1e-12)


@pytest.mark.parametrize("k", [256, 2304, 16384])
def test_split_gemm_same_sign_bias(tnr, k):
    """Same-sign operands (every Ising contraction starts so): the tensor cores truncate
    when adding into the FP32 accumulator, a bias that grows with K (-6e-6 relative at
    K = 2304 in one accumulation).  The contraction path accumulates K in chunks of 64
    summed with round-to-nearest, which bounds the mean relative error by 4e-7 at any K."""
    rng = np.random.default_rng(11)
    A = rng.uniform(0, 1, (256, k))
    B = rng.uniform(0, 1, (k, 192))
    got = tnr.debug_gemm(A, B, False, False, tnr.PREC_SPLIT)
    ref = A @ B
    rel = (got - ref) / ref
    assert abs(rel.mean()) < 4e-7, rel.mean()
    assert np.abs(rel).max() < 1e-6, np.abs(rel).max()


@pytest.mark.parametrize("m,n,k,ta,tb,batch", [
    (256, 256, 256, False, False, 1),
    (300, 200, 77, False, True, 1),
    (129, 135, 520, True, False, 1),
    (2304, 96, 2304, True, True, 1),
    (64, 4096, 256, False, False, 3),
])
def test_split_gemm_tc(tnr, m, n, k, ta, tb, batch):
    """tcgen05 3xBF16 GEMM (six plane products, FP32 accumulation) against FP64.
    Tolerance: the FP32 accumulator's random-walk error, 6e-8 * sqrt(k) normwise (a
    three-term split would sit near 1e-5, a broken kernel at O(1))."""
    rng = np.random.default_rng(7)
    sa = (batch, k, m) if ta else (batch, m, k)
    sb = (batch, n, k) if tb else (batch, k, n)
    A = rng.standard_normal(sa)
    B = rng.standard_normal(sb)
    if batch == 1:
        A, B = A[0], B[0]
    got = tnr.debug_gemm(A, B, ta, tb, tnr.PREC_SPLIT)
    opA = np.swapaxes(A, -1, -2) if ta else A
    opB = np.swapaxes(B, -1, -2) if tb else B
    ref = opA @ opB
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err < 6e-8 * np.sqrt(k), err
    f64 = tnr.debug_gemm(A, B, ta, tb, tnr.PREC_F64)
    assert np.linalg.norm(f64 - ref) / np.linalg.norm(ref) < 1e-14


@pytest.mark.parametrize("cls,chi", [("BTRG", 24), ("TRG", 24)])
@pytest.mark.parametrize("precision", ["f64", "split"])
def test_lockstep_group_equals_single(tnr, cls, chi, precision):
    """Equal-chi instances in one run_batch step in lockstep (one batched launch per kernel);
    each must match its own single run.  FP64: every norm to 1e-11 (the group iterates as
    long as its slowest member needs).  Split precision: the free energy to 1e-7, its
    accuracy contract; its norms only to FP32 level, since the products of the truncated
    SVD carry errors of ~1e-7 sigma_1 and the late, small singular directions move with
    the random start.  The betas are well conditioned: the oracle's norms move by at most
    2e-13 under a 1e-14 relative perturbation of the input tensor (at beta = 0.33 they move
    by 3e-7: a near-tie sits at the cut, where two runs with different random starts may
    keep different vectors)."""
    prec = tnr.PREC_F64 if precision == "f64" else tnr.PREC_SPLIT
    betas = [0.40, 0.42, 0.44, 0.46, 0.47]
    group = [getattr(tnr, cls)(tnr.classical_ising("Trivial", b), precision=prec) for b in betas]
    out = tnr.run_batch(group, [chi] * len(betas), [12] * len(betas))
    for b, d, g in zip(betas, out, group):
        s = getattr(tnr, cls)(tnr.classical_ising("Trivial", b), precision=prec)
        ref = tnr.run(s, tnr.truncrank(chi), tnr.maxiter(12))
        if precision == "f64":
            np.testing.assert_allclose(d, ref, rtol=1e-11)
        else:
            assert tnr.free_energy(d, b) == pytest.approx(tnr.free_energy(ref, b), rel=1e-7)
            np.testing.assert_allclose(d, ref, rtol=1e-3)
        # the member is left in its final state, like after run!
        assert g.T.shape == s.T.shape


@pytest.mark.parametrize("cls,chi,beta", [("BTRG", 24, 0.53), ("BTRG", 24, 0.57), ("TRG", 16, 0.53),
                                          ("TRG", 24, 0.6)])
def test_ordered_phase_f64(tnr, oracle, cls, chi, beta):
    """Ordered phase (beta > beta_c): the kept spectrum falls to ~1e-12 sigma_1, so the
    subspace iteration must stay backward stable in FP64 for the small directions
    (shifted CholeskyQR3); 12 steps against the oracle at 1e-10."""
    s = getattr(tnr, cls)(tnr.classical_ising("Trivial", beta))
    got = tnr.run(s, tnr.truncrank(chi), tnr.maxiter(12))
    ref = oracle.run(getattr(oracle, cls)(oracle.classical_ising(beta, "Trivial")), oracle.truncrank(chi),
                     oracle.maxiter(12))
    np.testing.assert_allclose(got, ref, rtol=1e-10)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_split_group_fixed_point_flows(tnr, seed):
    """A lockstep group of ten chi = 32 BTRG instances over 30 steps, in which beta = 0.584
    flows to the ordered and beta = 0.378 to the disordered fixed point: their matrices
    become numerically rank 1-2 while the group keeps iterating for the others, so most
    basis columns are noise.  The split path must orthonormalise those columns stably
    (shifted CholeskyQR3): every member's free energy within the 1e-7 contract of the FP64
    group's (an unstable orthonormalisation diverged here, |df/f| = 0.3)."""
    betas = [0.548, 0.402, 0.458, 0.404, 0.584, 0.378, 0.465, 0.441, 0.503, 0.398]

    def run(prec, sd):
        out = tnr.run_batch([tnr.BTRG(tnr.classical_ising("Trivial", b), precision=prec, seed=sd) for b in betas],
                            [32] * len(betas), [30] * len(betas))
        return [tnr.free_energy(o, b) for o, b in zip(out, betas)]

    ref = run(tnr.PREC_F64, 0)
    got = run(tnr.PREC_SPLIT, seed)
    for b, g, r in zip(betas, got, ref):
        assert abs(g / r - 1) <= 1e-7, (b, g, r)


@pytest.mark.parametrize("chi", [24, 32])
def test_split_high_temperature_band(tnr, oracle, chi):
    """The headline sweep draws beta ~ U[0.30, 0.60]; at beta = 0.30-0.36 late-step norms sit
    near ties at the cut (they move by 1e-7 under a 1e-14 input perturbation), while f does
    not (4e-15, test_oracle_conditioning.py).  BTRG, 30 steps, as one lockstep group: every
    split-precision f within 1e-7 of the FP64 path's, and the FP64 path's f at beta = 0.33
    within 1e-12 of the oracle's."""
    betas = [0.30, 0.31, 0.32, 0.33, 0.34, 0.35, 0.36]

    def run(prec):
        out = tnr.run_batch([tnr.BTRG(tnr.classical_ising("Trivial", b), precision=prec) for b in betas],
                            [chi] * len(betas), [30] * len(betas))
        return [tnr.free_energy(o, b) for o, b in zip(out, betas)]

    ref, got = run(tnr.PREC_F64), run(tnr.PREC_SPLIT)
    for b, g, r in zip(betas, got, ref):
        assert abs(g / r - 1) <= 1e-7, (b, g, r)
    o = oracle
    fo = o.free_energy(o.run(o.BTRG(o.classical_ising(0.33, "Trivial")), o.truncrank(chi), o.maxiter(30)), 0.33)
    assert ref[3] == pytest.approx(fo, rel=1e-12)


def test_split_small_chi_runs_plain(tnr, oracle):
    """A 2D split-precision solve at chi <= 16 runs every step on the plain FP64 path (the
    split products moved f by 2.2e-7 at chi = 16, beta = 0.304): at beta = 0.45 its norms equal
    the oracle's to 1e-10, and at beta = 0.304 (whose late norms sit at a near-tie of the cut)
    its f equals the oracle's to 1e-12, like the plain path's."""
    o = oracle
    d = tnr.run(tnr.BTRG(tnr.classical_ising("Trivial", 0.45), precision=tnr.PREC_SPLIT), tnr.truncrank(16),
                tnr.maxiter(30))
    do = o.run(o.BTRG(o.classical_ising(0.45, "Trivial")), o.truncrank(16), o.maxiter(30))
    np.testing.assert_allclose(d, do, rtol=1e-10)
    d = tnr.run(tnr.BTRG(tnr.classical_ising("Trivial", 0.304), precision=tnr.PREC_SPLIT), tnr.truncrank(16),
                tnr.maxiter(30))
    do = o.run(o.BTRG(o.classical_ising(0.304, "Trivial")), o.truncrank(16), o.maxiter(30))
    assert tnr.free_energy(d, 0.304) == pytest.approx(o.free_energy(do, 0.304), rel=1e-12)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_chol_inv_kernel(tnr, precision):
    """The one-CTA Cholesky + triangular-inverse kernel of CholeskyQR3 (blocked by 32 columns)
    against NumPy on batches of SPD matrices of every block shape up to the 160 limit, and its
    breakdown flag on an indefinite matrix."""
    prec = tnr.PREC_F64 if precision == "f64" else tnr.PREC_SPLIT
    rng = np.random.default_rng(5)
    for r in (1, 7, 31, 32, 33, 64, 100, 128, 160):
        A = rng.standard_normal((3, 2 * r + 4, r))
        G = np.einsum('bkr,bks->brs', A, A)
        got, bad = tnr.debug_chol(G, 0.0, prec)
        assert not bad
        for b in range(3):
            ref = np.linalg.inv(np.linalg.cholesky(G[b]))
            err = np.abs(got[b] - ref).max() / np.abs(ref).max()
            assert err < (1e-12 if precision == "f64" else 1e-4), (r, b, err)
            assert np.all(np.triu(got[b], 1) == 0)
    G = np.eye(40)
    G[17, 17] = -1.0
    _, bad = tnr.debug_chol(G, 0.0, prec)
    assert bad



@pytest.mark.parametrize("precision", ["f64", "split"])
def test_gap_fallback_flat_spectrum(tnr, oracle, flat_spectrum_tensor, precision):
    """Spectral-gap fallback: a TRG tensor (d = 12) whose first decomposition is near-flat at
    chi = 24 (sigma_24 / sigma_25 - 1 = 1e-5) is decomposed in full FP64 (the exact one-CTA
    Jacobi path for the 144 x 144 matrix) in both precisions, and the handle reports it.
    One step: the first decomposition's kept singular values equal the oracle's (LAPACK SVD)
    to 1e-10 of the largest in both precisions, the second's in FP64 (in split precision it
    may iterate on split products).  Norms over two steps: 2e-9 in FP64, where a
    1e-14 perturbation of the input moves the oracle's own norms by up to 5e-10
    (test_oracle_conditioning.py); 1e-6 in split precision, the bound of its contractions'
    products (6e-8 sqrt(K) at K = 576)."""
    o = oracle
    a = flat_spectrum_tensor(12, 1e-5, 3)
    prec = tnr.PREC_F64 if precision == "f64" else tnr.PREC_SPLIT
    s = tnr.TRG(a, precision=prec)
    tnr.run(s, tnr.truncrank(24), tnr.maxiter(1))
    so = o.TRG(o.Tensor(a, 2, None, 1))
    o.run(so, o.truncrank(24), o.maxiter(1))
    ndec, nfall, _ = s.decomposition_stats()
    assert ndec == 2 and nfall >= 1, (ndec, nfall)
    got, ref = s.singular_values(), so.svals[-2:]
    for g, r in list(zip(got, ref))[:2 if precision == "f64" else 1]:
        r = np.asarray(r)
        assert len(g) == len(r) == 24
        np.testing.assert_allclose(g, r, rtol=0, atol=SVAL_TOL * abs(r[0]))
    s2 = tnr.TRG(a, precision=prec)
    d = np.array(tnr.run(s2, tnr.truncrank(24), tnr.maxiter(2)))
    do = np.array(o.run(o.TRG(o.Tensor(a, 2, None, 1)), o.truncrank(24), o.maxiter(2)))
    np.testing.assert_allclose(d, do, rtol=2e-9 if precision == "f64" else 1e-6)


def test_gap_fallback_in_lockstep_group(tnr, oracle, flat_spectrum_tensor):
    """A lockstep group whose members include a flat-spectrum tensor: that member alone is
    decomposed again by the FP64 gap fallback and its norms equal the oracle's to 2e-9 (the
    problem's conditioning, as above); the other member's norms equal its single run's."""
    o = oracle
    ts = [flat_spectrum_tensor(12, 1e-5, 3), np.random.default_rng(11).standard_normal((12,) * 4)]
    out = tnr.run_batch([tnr.TRG(t) for t in ts], [24, 24], [2, 2])
    do = o.run(o.TRG(o.Tensor(ts[0], 2, None, 1)), o.truncrank(24), o.maxiter(2))
    np.testing.assert_allclose(out[0], do, rtol=2e-9)
    single = tnr.run(tnr.TRG(ts[1]), tnr.truncrank(24), tnr.maxiter(2))
    np.testing.assert_allclose(out[1], single, rtol=NORM_RTOL)
