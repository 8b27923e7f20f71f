"""CPU FP64 oracle for TNRKit's coarse-graining hot path (TEST INFRASTRUCTURE ONLY).

This module is the oracle: a NumPy/SciPy restatement of the reference algorithm,
operation for operation.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import it, and only as the result to compare
against or as the timed CPU restatement.  The product path (``tnrkit.jl_gb300``) never calls it.

Reference: TNRKit.jl v0.5.1 (pure Julia).  The arithmetic the reference delegates
to third-party packages that are not vendored with it is restated here from
their published behaviour:

* TensorKit 0.16.2 (``Project.toml:33``): dense ``Trivial`` tensors are
  column-major arrays ``T[i1,i2,i3,i4]``; ``permute``/``transpose`` of bosonic
  legs only reorder axes; abelian (Z_N) tensors are block diagonal in the total
  charge of the row legs.
* MatrixAlgebraKit 0.6.1 (``Project.toml:29``): ``svd_trunc``/``eigh_trunc!``
  with ``truncrank(chi)`` keep the ``min(chi, n)`` values largest in absolute
  value, globally across charge blocks; the returned truncation error is the
  2-norm of the discarded values; ``project_hermitian!`` replaces ``M`` by
  ``(M + M')/2``.

Parity pins (the reference cannot run in this container: no Julia):
* ``README.md:78-93``: BTRG, Z2 Ising at beta_c, truncrank(16), maxiter(25),
  26 norms -> f = -2.1096504926141826902647832, |f - f_Onsager|/|f| = 3.1e-7.
* ``test/schemes.jl:18-23,57-62,94-99,376-383`` and ``test/models.jl:5-39``:
  free energies against Onsager / published values at the stated rtol.
Ties between equal singular values at the truncation cut are resolved by a
stable sort here; the reference's tie order is not visible (parity unpinned at
exact ties only).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# ---------------------------------------------------------------------------
# constants  (src/models/ising.jl:1-2,8)
# ---------------------------------------------------------------------------
ISING_BETA_C = math.log(1.0 + math.sqrt(2.0)) / 2.0
F_ONSAGER = -2.10965114460820745966777928351108478082549327543540531781696107967700291143188081390114126499095041781
ISING_BETA_C_3D = 1.0 / 4.51152469
F_BENCHMARK_3D = -3.507           # test/schemes.jl:10
EPS = np.finfo(np.float64).eps


def potts_beta_c(q):
    """src/models/potts.jl:39"""
    return math.log(1.0 + math.sqrt(q))


# ---------------------------------------------------------------------------
# Tensors with optional abelian charges
# ---------------------------------------------------------------------------
@dataclass
class Tensor:
    """Dense FP64 array plus, for Z_N-symmetric tensors, one signed-charge vector per leg.

    ``q[l][i]`` is the charge that basis index ``i`` of leg ``l`` contributes to
    the conservation law ``sum_l q[l][i_l] == 0 (mod N)``.  Codomain legs carry
    ``+charge``, domain legs ``-charge``; a permute keeps the signed charges and
    a conjugate negates them.  ``N == 1`` means no symmetry (``Trivial``).
    """

    a: np.ndarray
    nout: int                      # number of codomain legs
    q: list = field(default=None)  # list of int arrays or None
    N: int = 1

    @property
    def ndim(self):
        return self.a.ndim

    def copy(self):
        return Tensor(self.a.copy(), self.nout,
                      None if self.q is None else [x.copy() for x in self.q], self.N)


def _charges(spec, *ts):
    """Output-leg charges of a contraction; checks that contracted legs carry
    opposite signed charges (the flow rule of a symmetric contraction).
    A tensor passed as ``('c', t)`` enters conjugated: its charges are negated."""
    ins, out = spec.split('->')
    seen, N = {}, 1
    for lab, t in zip(ins.split(','), ts):
        neg = isinstance(t, tuple)
        t = t[1] if neg else t
        N = max(N, t.N)
        if t.q is None:
            continue
        for c, qq in zip(lab, t.q):
            qq = (-qq) % t.N if neg else qq % t.N
            if c in seen and c not in out:
                assert np.array_equal((seen[c] + qq) % t.N, np.zeros_like(qq)), f"charge flow mismatch on leg {c}"
            seen.setdefault(c, qq)
    if N == 1:
        return None, 1
    return [seen[c] for c in out], N


def _ein(spec, *ts, path=None):
    """Contract Tensors with an einsum spec; output charges follow the leg labels.

    ``path`` is an explicit pairwise order (numpy ``einsum_path`` form) so every
    contraction runs at the cost the reference's network has (chi^6 / chi^7)."""
    arrs = [(t[1] if isinstance(t, tuple) else t).a for t in ts]
    q, N = _charges(spec, *ts)
    opt = ['einsum_path'] + list(path) if path is not None else True
    return np.einsum(spec, *arrs, optimize=opt), q, N


def permute(t: Tensor, perm, nout):
    """TensorKit ``permute``/``transpose`` of bosonic legs: an axis reorder."""
    q = None if t.q is None else [t.q[p] for p in perm]
    return Tensor(np.ascontiguousarray(np.transpose(t.a, perm)), nout, q, t.N)


# ---------------------------------------------------------------------------
# truncated decompositions (MatrixAlgebraKit 0.6.1, called at
# src/utility/projectors.jl:215, src/schemes/btrg.jl:61,72,
# src/schemes/hotrg.jl:103,110,139,146, src/schemes/hotrg3d.jl:93,96)
# ---------------------------------------------------------------------------
def _row_col_keys(t: Tensor, nrow):
    """Charge of each matrix row / column of the (rows <- cols) reshape."""
    if t.q is None:
        return None, None
    N = t.N
    rk = np.zeros(1, dtype=np.int64)
    for qq in t.q[:nrow]:
        rk = (rk[:, None] + qq[None, :]).reshape(-1) % N
    ck = np.zeros(1, dtype=np.int64)
    for qq in t.q[nrow:]:
        ck = (ck[:, None] + qq[None, :]).reshape(-1) % N
    return rk, (-ck) % N


def _select_global(vals_per_block, chi):
    """Keep the ``chi`` largest |values| over all blocks (truncrank(chi), by=abs, rev=true)."""
    allv = []
    for b, v in enumerate(vals_per_block):
        for i, x in enumerate(v):
            allv.append((abs(x), b, i))
    # stable: ties keep block order then index order
    order = sorted(range(len(allv)), key=lambda j: -allv[j][0])
    keep = order[:min(chi, len(allv))]
    kept = [[] for _ in vals_per_block]
    for j in keep:
        _, b, i = allv[j]
        kept[b].append(i)
    # truncation error = 2-norm of the discarded values
    disc = [allv[j][0] for j in order[min(chi, len(allv)):]]
    err = float(np.sqrt(np.sum(np.square(disc)))) if disc else 0.0
    return [sorted(k) for k in kept], err


def svd_trunc(t: Tensor, nrow, chi):
    """``U, S, V, eps = svd_trunc(t; trunc=truncrank(chi))`` on the rows<-cols reshape.

    Returns U (row legs + bond), s (descending per kept value), Vh (bond + col
    legs), the truncation error, and the bond charges (U side, V side)."""
    dims = t.a.shape
    rdim = int(np.prod(dims[:nrow]))
    M = t.a.reshape(rdim, -1)
    cdim = M.shape[1]
    rk, ck = _row_col_keys(t, nrow)
    if rk is None:
        sectors = [(np.arange(rdim), np.arange(cdim), 0)]
    else:
        sectors = []
        for c in range(t.N):
            r = np.nonzero(rk == c)[0]
            cc = np.nonzero(ck == c)[0]
            if len(r) and len(cc):
                sectors.append((r, cc, c))
    decs, vals = [], []
    for r, cc, c in sectors:
        u, s, vh = np.linalg.svd(M[np.ix_(r, cc)], full_matrices=False)
        decs.append((u, s, vh))
        vals.append(s)
    kept, err = _select_global(vals, chi)
    # assemble in descending order of value
    cols = []
    for b, idx in enumerate(kept):
        for i in idx:
            cols.append((vals[b][i], b, i))
    cols.sort(key=lambda x: -x[0])
    k = len(cols)
    U = np.zeros((rdim, k))
    Vh = np.zeros((k, cdim))
    s = np.zeros(k)
    bond = np.zeros(k, dtype=np.int64)
    for j, (_, b, i) in enumerate(cols):
        r, cc, c = sectors[b]
        u, sv, vh = decs[b]
        U[r, j] = u[:, i]
        Vh[j, cc] = vh[i, :]
        s[j] = sv[i]
        bond[j] = c
    U = U.reshape(dims[:nrow] + (k,))
    Vh = Vh.reshape((k,) + dims[nrow:])
    if t.q is None:
        return U, s, Vh, err, None
    return U, s, Vh, err, ((-bond) % t.N, bond % t.N)


def eigh_trunc(t: Tensor, nrow, chi):
    """``_, U, eps = eigh_trunc!(project_hermitian!(MM); trunc=truncrank(chi))``."""
    dims = t.a.shape
    rdim = int(np.prod(dims[:nrow]))
    M = t.a.reshape(rdim, rdim)
    M = 0.5 * (M + M.T)                        # project_hermitian! (real data)
    rk, _ = _row_col_keys(t, nrow)
    if rk is None:
        sectors = [(np.arange(rdim), 0)]
    else:
        sectors = [(np.nonzero(rk == c)[0], c) for c in range(t.N)]
        sectors = [x for x in sectors if len(x[0])]
    decs, vals = [], []
    for r, c in sectors:
        w, v = np.linalg.eigh(M[np.ix_(r, r)])
        decs.append(v)
        vals.append(w)
    kept, err = _select_global(vals, chi)
    cols = []
    for b, idx in enumerate(kept):
        for i in idx:
            cols.append((vals[b][i], b, i))
    cols.sort(key=lambda x: -abs(x[0]))
    k = len(cols)
    U = np.zeros((rdim, k))
    lam = np.zeros(k)
    bond = np.zeros(k, dtype=np.int64)
    for j, (_, b, i) in enumerate(cols):
        r, c = sectors[b]
        U[r, j] = decs[b][:, i]
        lam[j] = vals[b][i]
        bond[j] = c
    U = U.reshape(dims[:nrow] + (k,))
    q = None if t.q is None else list(t.q[:nrow]) + [(-bond) % t.N]
    return Tensor(U, nrow, q, t.N), lam, err


# ---------------------------------------------------------------------------
# models  (src/models/ising.jl, potts.jl, clock.jl)
# ---------------------------------------------------------------------------
def _leg_charges(d, nout, nleg, N):
    if N == 1:
        return None
    base = np.arange(d, dtype=np.int64) % N
    return [base.copy() if l < nout else (-base) % N for l in range(nleg)]


def classical_ising(beta=ISING_BETA_C, symmetry="Z2", h=0.0):
    """src/models/ising.jl:10-15,44-67.  Trivial and Z2 give the same dense array at h=0."""
    x, y = math.cosh(beta), math.sinh(beta)
    if symmetry == "Z2":
        assert h == 0.0, "External magnetic field is not compatible with Z2 symmetry"
    b = np.array([[math.sqrt(x), 0.0], [0.0, math.sqrt(y)]])
    init = np.zeros((2, 2, 2, 2))
    for i, j, k, l in np.ndindex(2, 2, 2, 2):
        init[i, j, k, l] = math.cosh(h * beta) if (i + j + k + l) % 2 == 0 else math.sinh(h * beta)
    # T[-1 -2; -3 -4] := 2 init[1 2; 3 4] b[-1;1] b[-2;2] b[3;-3] b[4;-4]
    a = 2.0 * np.einsum('abcd,ia,jb,ck,dl->ijkl', init, b, b, b, b)
    N = 2 if symmetry == "Z2" else 1
    return Tensor(a, 2, _leg_charges(2, 2, 4, N), N)


def classical_ising_impurity(beta=ISING_BETA_C, h=0.0):
    """src/models/ising.jl:87-102 (Trivial): the magnetisation impurity, whose even-parity
    entries carry sinh(h beta) and odd-parity ones cosh(h beta) (the pure tensor swaps them)."""
    x, y = math.cosh(beta), math.sinh(beta)
    b = np.array([[math.sqrt(x), 0.0], [0.0, math.sqrt(y)]])
    init = np.zeros((2, 2, 2, 2))
    for i, j, k, l in np.ndindex(2, 2, 2, 2):
        init[i, j, k, l] = math.sinh(h * beta) if (i + j + k + l) % 2 == 0 else math.cosh(h * beta)
    a = 2.0 * np.einsum('abcd,ia,jb,ck,dl->ijkl', init, b, b, b, b)
    return Tensor(a, 2, None, 1)


def classical_ising_3D(beta=ISING_BETA_C_3D, symmetry="Z2", J=1.0):
    """src/models/ising.jl:130-165 (Z2 branch; the Trivial branch is the same model in a
    different basis).  Legs: D (x) U' <- N (x) E (x) S' (x) W'."""
    if symmetry == "Z2":
        x, y = math.cosh(beta * J), math.sinh(beta * J)
        W = np.array([[math.sqrt(x), math.sqrt(y)], [math.sqrt(x), -math.sqrt(y)]])
        t = np.einsum('ai,aj,ak,al,am,an->ijklmn', W, W, W, W, W, W)
        # permute(t, ((1, 4), (5, 6, 2, 3)))
        a = np.ascontiguousarray(np.transpose(t, (0, 3, 4, 5, 1, 2)))
        base = np.arange(2, dtype=np.int64)
        return Tensor(a, 2, [base.copy() for _ in range(6)], 2)
    K = beta * J
    tm = np.array([[math.exp(K), math.exp(-K)], [math.exp(-K), math.exp(K)]])
    w, v = np.linalg.eigh(tm)
    qm = v @ np.diag(np.sqrt(w)) @ v.T
    O = np.zeros((2,) * 6)
    O[(0,) * 6] = 1.0
    O[(1,) * 6] = 1.0
    a = np.einsum('abcdef,ia,jb,kc,ld,me,nf->ijklmn', O, qm, qm, qm, qm, qm, qm)
    return Tensor(a, 2, None, 1)


def _fourier_real_zn(A, q, conj_first_two=True):
    """(P'(x)P') A (P(x)P) with P[k,c] = w^{kc}/sqrt(q); real part (potts.jl:71-81, clock.jl:32-49)."""
    w = np.exp(2j * np.pi / q)
    P = np.array([[w ** (k * c) for c in range(q)] for k in range(q)]) / math.sqrt(q)
    U = np.einsum('ijkl,ia,jb,kc,ld->abcd', A.astype(complex), P.conj(), P.conj(), P, P)
    return np.real(U)


def classical_potts(q=3, beta=None, symmetry="ZN"):
    """src/models/potts.jl:22-30,68-81."""
    if beta is None:
        beta = potts_beta_c(q)
    A = np.zeros((q, q, q, q))
    for i, j, k, l in np.ndindex(q, q, q, q):
        E = -(int(i == j) + int(j == l) + int(k == l) + int(k == i))
        A[i, j, k, l] = math.exp(-beta * E)
    if symmetry == "Trivial":
        return Tensor(A, 2, None, 1)
    a = _fourier_real_zn(A, q)
    t = Tensor(a, 2, _leg_charges(q, 2, 4, q), q)
    return _project_symmetric(t)


def classical_clock(q=6, beta=1.0, symmetry="ZN"):
    """src/models/clock.jl:1-12,29-49 (Trivial and Z_q branches)."""
    A = np.zeros((q, q, q, q))

    def clock(i, j):
        return -math.cos(2 * math.pi / q * (i - j))
    for i, j, k, l in np.ndindex(q, q, q, q):
        E = clock(i, j) + clock(j, l) + clock(l, k) + clock(k, i)
        A[i, j, k, l] = math.exp(-beta * E)
    if symmetry == "Trivial":
        return Tensor(A, 2, None, 1)
    a = _fourier_real_zn(A, q)
    t = Tensor(a, 2, _leg_charges(q, 2, 4, q), q)
    return _project_symmetric(t)


def sixvertex(a=1.0, b=1.0, c=1.0):
    """src/models/sixvertex.jl:29-37 (Trivial): the 4 x 4 vertex weights (a on the two
    all-equal configurations, c and b on the two mixed ones) as T[i1, i2; i3, i4]."""
    W = np.array([[a, 0, 0, 0], [0, c, b, 0], [0, b, c, 0], [0, 0, 0, a]], dtype=np.float64)
    return Tensor(W.reshape(2, 2, 2, 2, order='F'), 2, None, 1)


def _phi4_real_site(K, mu0, lam, h, power):
    """src/models/phi4_real.jl:5-23,88-111,186-209,241-264 (Trivial): Gauss-Hermite nodes y_p and
    weights w_p, the link matrix F[i, j] = exp(-(y_i - y_j)^2/2 - mu0 (y_i^2 + y_j^2)/8
    - lam (y_i^4 + y_j^4)/16 + h (y_i + y_j)/4) = U S V, and
    T[i,j,k,l] = sum_p sqrt(S_i S_j S_k S_l) y_p^power w_p exp(y_p^2) U[p,i] U[p,j] V[k,p] V[l,p]."""
    y, w = np.polynomial.hermite.hermgauss(K)
    Y1, Y2 = np.meshgrid(y, y, indexing='ij')
    F = np.exp(-0.5 * (Y1 - Y2) ** 2 - mu0 / 8 * (Y1 ** 2 + Y2 ** 2) - lam / 16 * (Y1 ** 4 + Y2 ** 4) + h / 4 * (Y1 + Y2))
    U, S, Vh = np.linalg.svd(F)
    r = np.sqrt(S)
    site = w * np.exp(y ** 2) * y ** power
    Uw, Vw = U * r, (r[:, None] * Vh)
    return np.einsum('p,pi,pj,kp,lp->ijkl', site, Uw, Uw, Vw, Vw)


def phi4_real(K, mu0, lam, h=0.0, symmetry="Z2"):
    """src/models/phi4_real.jl:85-154: the real phi^4 site tensor, Trivial (Gauss-Hermite, bond
    dimension K) or Z2 (Taylor expansion of the link term to order K-1: t[s1..s4] =
    M_{s1+s2+s3+s4} / sqrt(s1! s2! s3! s4!) for an even order sum, M_n = int exp(-a phi^2 - b phi^4)
    phi^n, a = (4 + mu0)/2, b = lam/4; even orders first, then odd, as the two charge sectors)."""
    if symmetry == "Trivial":
        return Tensor(_phi4_real_site(K, mu0, lam, h, 0), 2, None, 1)
    assert h == 0.0 and K % 2 == 0
    from scipy.integrate import quad
    a, b = (4 + mu0) / 2, lam / 4
    M = np.zeros(4 * (K - 1) + 1)
    for n in range(0, 4 * (K - 1) + 1, 2):
        M[n] = quad(lambda x, n=n: math.exp(-a * x * x - b * x ** 4) * x ** n, -np.inf, np.inf)[0]
    lf = np.array([math.lgamma(s + 1) for s in range(K)])
    t = np.zeros((K, K, K, K))
    for s1, s2, s3, s4 in np.ndindex(K, K, K, K):
        n = s1 + s2 + s3 + s4
        if n % 2 == 0:
            t[s1, s2, s3, s4] = M[n] / math.exp((lf[s1] + lf[s2] + lf[s3] + lf[s4]) / 2)
    perm = list(range(0, K, 2)) + list(range(1, K, 2))
    t = t[np.ix_(perm, perm, perm, perm)]
    qv = np.array([0] * (K // 2) + [1] * (K // 2), dtype=np.int64)
    return Tensor(t, 2, [qv.copy(), qv.copy(), (-qv) % 2, (-qv) % 2], 2)


def phi4_complex(K, mu0, lam):
    """src/models/phi4_complex.jl:6-36,108-138,194-206 (Trivial, real entries): Gauss-Hermite
    nodes for the real and imaginary parts, link matrix F[(a,b),(c,d)] = exp(-((y_a - y_c)^2
    + (y_b - y_d)^2)/2 - mu0 (|phi_1|^2 + |phi_2|^2)/8 - lam (|phi_1|^4 + |phi_2|^4)/16) = U S V on the
    K^2 pairs (pair index a K + b), site weights w_a w_b exp(y_a^2 + y_b^2), and
    T[i,j,k,l] = sum_p sqrt(S_i S_j S_k S_l) W_p U[p,i] U[p,j] V[k,p] V[l,p] (bond dimension K^2).
    F is symmetric positive definite, so U = V^T and T is fully symmetric, as the reference's
    sorted-index fill assumes."""
    y, w = np.polynomial.hermite.hermgauss(K)
    R1, I1, R2, I2 = np.meshgrid(y, y, y, y, indexing='ij')
    F = np.exp(-0.5 * ((R1 - R2) ** 2 + (I1 - I2) ** 2) - mu0 / 8 * (R1 ** 2 + I1 ** 2 + R2 ** 2 + I2 ** 2)
               - lam / 16 * ((R1 ** 2 + I1 ** 2) ** 2 + (R2 ** 2 + I2 ** 2) ** 2)).reshape(K * K, K * K)
    U, S, Vh = np.linalg.svd(F)
    Wt = (w[:, None] * w[None, :] * np.exp(y[:, None] ** 2 + y[None, :] ** 2)).reshape(-1)
    r = np.sqrt(S)
    Ul, Vr = U * r, r[:, None] * Vh
    return Tensor(np.einsum('p,pi,pj,kp,lp->ijkl', Wt, Ul, Ul, Vr, Vr, optimize=True), 2, None, 1)


def phi4_real_imp1(K, mu0, lam, h=0.0):
    """src/models/phi4_real.jl:186-209: the site tensor with a phi insertion (Trivial)."""
    return Tensor(_phi4_real_site(K, mu0, lam, h, 1), 2, None, 1)


def phi4_real_imp2(K, mu0, lam, h=0.0):
    """src/models/phi4_real.jl:241-264: the site tensor with a phi^2 insertion (Trivial)."""
    return Tensor(_phi4_real_site(K, mu0, lam, h, 2), 2, None, 1)


def _project_symmetric(t: Tensor):
    """Zero the entries that break charge conservation (TensorKit keeps only symmetric blocks)."""
    if t.q is None:
        return t
    tot = np.zeros((1,) * t.ndim, dtype=np.int64)
    for l, qq in enumerate(t.q):
        shape = [1] * t.ndim
        shape[l] = len(qq)
        tot = tot + qq.reshape(shape)
    mask = (tot % t.N) == 0
    assert np.max(np.abs(t.a[~mask]), initial=0.0) < 1e-10 * np.max(np.abs(t.a))
    return Tensor(np.where(mask, t.a, 0.0), t.nout, t.q, t.N)


def random_hotrg_tensor(chi, seed, decay=6.0):
    """Seeded dense 4-leg test tensor: N(0,1) entries weighted per leg by exp(-k/decay),
    Frobenius-normalised (the single-step HOTRG workload)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = rng.standard_normal((chi,) * 4)
    s = np.exp(-np.arange(chi) / decay)
    a = a * s[:, None, None, None] * s[None, :, None, None] * s[None, None, :, None] * s[None, None, None, :]
    a /= np.linalg.norm(a)
    return Tensor(a, 2, None, 1)


# ---------------------------------------------------------------------------
# schemes
# ---------------------------------------------------------------------------
class TRG:
    """src/schemes/trg.jl:26-33"""
    scalefactor = 2.0

    def __init__(self, T: Tensor):
        assert T.ndim == 4
        self.T = T.copy()
        self.svals = []          # kept singular values of every decomposition, in order


class BTRG:
    """src/schemes/btrg.jl:26-48: S1 = id(space(T,2)), S2 = id(space(T,1)), k = -1/2."""
    scalefactor = 2.0

    def __init__(self, T: Tensor, k=-0.5):
        assert T.ndim == 4
        self.T = T.copy()
        self.S1 = np.ones(T.a.shape[1])      # diagonal bond tensors
        self.S2 = np.ones(T.a.shape[0])
        self.k = float(k)
        self.svals = []


class HOTRG:
    """src/schemes/hotrg.jl:27-34"""
    scalefactor = 4.0

    def __init__(self, T: Tensor):
        assert T.ndim == 4
        self.T = T.copy()
        self.svals = []
        self.eps = []


class HOTRG_3D:
    """src/schemes/hotrg3d.jl:27-34"""
    scalefactor = 8.0

    def __init__(self, T: Tensor):
        assert T.ndim == 6
        self.T = T.copy()
        self.svals = []
        self.eps = []


class ImpurityHOTRG:
    """src/schemes/impurityhotrg.jl:26-46: the pure tensor, the two first-order impurity
    tensors and the second-order one, all of the same spaces."""

    def __init__(self, T: Tensor, T_imp_order1_1: Tensor, T_imp_order1_2: Tensor, T_imp_order2: Tensor):
        for t in (T_imp_order1_1, T_imp_order1_2):
            assert t.a.shape == T.a.shape, "the first-order impurities need the spaces of T"
        self.T = T.copy()
        self.T_imp_order1_1 = T_imp_order1_1.copy()
        self.T_imp_order1_2 = T_imp_order1_2.copy()
        self.T_imp_order2 = T_imp_order2.copy()


class ATRG:
    """src/schemes/atrg.jl:26-33: the central tensor; one step is two anisotropic half steps
    (linear rescaling sqrt(2) each)."""
    scalefactor = 2.0

    def __init__(self, T: Tensor):
        assert T.ndim == 4
        self.T = T.copy()
        self.svals = []


class ATRG_3D:
    """src/schemes/atrg3d.jl:26-33: the central 6-leg tensor T[1 2; 3 4 5 6]; one step is three
    half steps, one along each axis (volume factor 8).  Dense (Trivial) arrays only."""
    scalefactor = 8.0

    def __init__(self, T: Tensor):
        assert T.ndim == 6
        self.T = Tensor(np.array(T.a), 2, None, 1)
        self.svals = []


class CorrelationHOTRG:
    """src/schemes/correlationhotrg.jl:29-71: the pure tensor and two first-order impurities
    2^dist sites apart; after dist steps they merge into one impurity (Timp_final)."""

    def __init__(self, Tpure: Tensor, Timp1: Tensor, Timp2: Tensor, dist: int):
        assert dist >= 0, "Distance must be non-negative"
        for t in (Timp1, Timp2):
            assert t.a.shape == Tpure.a.shape, "the impurities need the spaces of Tpure"
        self.Tpure = Tpure.copy()
        self.Timp1 = Timp1.copy()
        self.Timp2 = Timp2.copy()
        self.Timp_final = None
        self.dist = dist
        self.iter = 0


class ImpurityTRG:
    """src/schemes/impuritytrg.jl:38-61: the pure tensor and impurity tensors on the four
    sites of a plaquette, all of the same spaces."""

    def __init__(self, T: Tensor, T_imp1: Tensor, T_imp2: Tensor, T_imp3: Tensor, T_imp4: Tensor):
        for t in (T_imp1, T_imp2, T_imp3, T_imp4):
            assert t.a.shape == T.a.shape, "the impurities need the spaces of T"
        self.T = T.copy()
        self.T_imp = [t.copy() for t in (T_imp1, T_imp2, T_imp3, T_imp4)]


def SVD12(T: Tensor, chi):
    """src/utility/projectors.jl:211-217: U*sqrt(s), sqrt(s)*V."""
    U, s, Vh, _, bq = svd_trunc(T, 2, chi)
    r = np.sqrt(s)
    A = Tensor(U * r, 2, None if bq is None else [T.q[0], T.q[1], bq[0]], T.N)
    B = Tensor(r[:, None, None] * Vh, 1, None if bq is None else [bq[1], T.q[2], T.q[3]], T.N)
    return A, B, s


def step_trg(scheme: TRG, chi):
    """src/schemes/trg.jl:35-41"""
    T = scheme.T
    A, B, s1 = SVD12(T, chi)
    Tp = permute(T, (1, 3, 0, 2), 2)                       # transpose(T, ((2,4),(1,3)))
    C, D, s2 = SVD12(Tp, chi)
    # T[-1 -2; -3 -4] := D[-2; 1 2] B[-1; 4 1] C[4 3; -3] A[3 2; -4]
    a, q, N = _ein('bpq,arp,rsc,sqd->abcd', D, B, C, A, path=[(0, 1), (0, 1), (0, 1)])
    scheme.T = Tensor(a, 2, q, N)
    scheme.svals += [s1, s2]


def _trg_contract(D, B, C, A):
    """T[-1 -2; -3 -4] := D[-2; 1 2] B[-1; 4 1] C[4 3; -3] A[3 2; -4] (src/schemes/trg.jl:39)"""
    a, q, N = _ein('bpq,arp,rsc,sqd->abcd', D, B, C, A, path=[(0, 1), (0, 1), (0, 1)])
    return Tensor(a, 2, q, N)


def step_impurity_trg(scheme: ImpurityTRG, chi):
    """src/schemes/impuritytrg.jl:63-91: SVD12 of sites 1 and 3 and the pure tensor, of
    sites 2 and 4 and the pure tensor transposed ((2,4),(1,3)); five TRG contractions."""
    tp = lambda t: permute(t, (1, 3, 0, 2), 2)       # noqa: E731
    I1, I2, I3, I4 = scheme.T_imp
    A1, B1, _ = SVD12(I1, chi)
    C2, D2, _ = SVD12(tp(I2), chi)
    A3, B3, _ = SVD12(I3, chi)
    C4, D4, _ = SVD12(tp(I4), chi)
    Ap, Bp, _ = SVD12(scheme.T, chi)
    Cp, Dp, _ = SVD12(tp(scheme.T), chi)
    scheme.T = _trg_contract(Dp, Bp, Cp, Ap)
    scheme.T_imp = [_trg_contract(Dp, B1, C2, Ap), _trg_contract(D2, B3, Cp, Ap),
                    _trg_contract(D4, Bp, Cp, A3), _trg_contract(Dp, Bp, C4, A1)]


def finalize_impurity_trg(scheme: ImpurityTRG):
    """src/utility/finalize.jl:75-88: every tensor /= the pure trace norm, then the norm of
    the four impurities contracted around the plaquette
    T_imp1[5 4; 6 1] T_imp2[1 2; 7 5] T_imp3[3 7; 2 8] T_imp4[8 6; 4 3]."""
    npure = abs(np.einsum('abba->', scheme.T.a))
    scheme.T.a = scheme.T.a / npure
    for t in scheme.T_imp:
        t.a = t.a / npure
    t1, t2, t3, t4 = (t.a for t in scheme.T_imp)
    x = np.einsum('edfa,abge->dfbg', t1, t2)
    y = np.einsum('cgbh,hfdc->gbfd', t3, t4)
    nimp = abs(np.einsum('dfbg,gbfd->', x, y))
    return float(npure), float(nimp)


def pseudopow(s, a, tol=EPS ** 0.75):
    """src/schemes/btrg.jl:50-58"""
    out = s.copy()
    m = s >= tol
    out[m] = s[m] ** a
    return out


def step_btrg(scheme: BTRG, chi):
    """src/schemes/btrg.jl:60-94"""
    T = scheme.T
    k = scheme.k
    U, s, Vh, _, bq = svd_trunc(T, 2, chi)
    sa, sb = pseudopow(s, (1 - k) / 2), pseudopow(s, k)
    A = Tensor(U * sa, 2, None if bq is None else [T.q[0], T.q[1], bq[0]], T.N)
    B = Tensor(sa[:, None, None] * Vh, 1, None if bq is None else [bq[1], T.q[2], T.q[3]], T.N)
    S1n = sb
    P = permute(T, (2, 0, 3, 1), 2)                         # permute(T, ((3,1),(4,2)))
    U2, s2, Vh2, _, bq2 = svd_trunc(P, 2, chi)
    sa2, sb2 = pseudopow(s2, (1 - k) / 2), pseudopow(s2, k)
    C = Tensor(U2 * sa2, 2, None if bq2 is None else [P.q[0], P.q[1], bq2[0]], T.N)
    D = Tensor(sa2[:, None, None] * Vh2, 1, None if bq2 is None else [bq2[1], P.q[2], P.q[3]], T.N)
    S2n = sb2
    S1, S2 = scheme.S1, scheme.S2
    # T[-1 -2; -3 -4] := D[-1;4 7] S1[1;7] B[-2;1 3] S2[3;2] C[8 2;-4] S1[8;5] A[6 5;-3] S2[4;6]
    # diagonal S1/S2: fold them into D's leg 7 and C's leg 8 / B's leg 3 and D's leg 4 equivalents
    Dd = Tensor(D.a * S1[None, None, :], D.nout, D.q, D.N)            # D[-1;4 7] S1[7]
    Dd = Tensor(Dd.a * S2[None, :, None], Dd.nout, Dd.q, Dd.N)        # S2[4;6] (diag: 4 == 6)
    Bd = Tensor(B.a * S2[None, None, :], B.nout, B.q, B.N)            # S2[3;2]  (3 == 2)
    Cd = Tensor(C.a * S1[:, None, None], C.nout, C.q, C.N)            # S1[8;5]  (8 == 5)
    # now D[-1;4 1] B[-2;1 2] C[5 2;-4] A[4 5;-3]
    a, q, N = _ein('axp,bpy,zyd,xzc->abcd', Dd, Bd, Cd, A, path=[(0, 1), (0, 1), (0, 1)])
    scheme.T = Tensor(a, 2, q, N)
    scheme.S1, scheme.S2 = S1n, S2n
    scheme.svals += [s, s2]


def _hotrg_xproj(A1: Tensor, A2: Tensor, chi):
    """src/schemes/hotrg.jl:82-116"""
    a, q, N = _ein('aeij,bkel,cfij,dkfl->abcd', A2, A1, ('c', A2), ('c', A1), path=[(0, 2), (0, 1), (0, 1)])
    U, lam, eps = eigh_trunc(Tensor(a, 2, q, N), 2, chi)
    a, q, N = _ein('jeia,lkeb,jfic,lkfd->abcd', ('c', A2), ('c', A1), A2, A1, path=[(0, 2), (0, 1), (0, 1)])
    U2, lam2, eps2 = eigh_trunc(Tensor(a, 2, q, N), 2, chi)
    if eps > eps2:
        return U2, lam2, eps2, (eps, eps2)
    return U, lam, eps, (eps, eps2)


def _hotrg_yproj(A1: Tensor, A2: Tensor, chi):
    """src/schemes/hotrg.jl:118-152"""
    a, q, N = _ein('iajp,pblk,icjr,rdlk->abcd', A1, A2, ('c', A1), ('c', A2), path=[(0, 2), (0, 1), (0, 1)])
    U, lam, eps = eigh_trunc(Tensor(a, 2, q, N), 2, chi)
    a, q, N = _ein('ijap,plbk,ijcr,rldk->abcd', ('c', A1), ('c', A2), A1, A2, path=[(0, 2), (0, 1), (0, 1)])
    U2, lam2, eps2 = eigh_trunc(Tensor(a, 2, q, N), 2, chi)
    if eps > eps2:
        return U2, lam2, eps2, (eps, eps2)
    return U, lam, eps, (eps, eps2)


def _hotrg_step_y(A1, A2, Ux):
    """src/schemes/hotrg.jl:42-60: conj(Ux[1 2;-1]) Ux[3 4;-4] A2[1 5;-3 3] A1[2 -2;5 4]"""
    a, q, N = _ein('ija,kld,iegk,jbel->abgd', ('c', Ux), Ux, A2, A1, path=[(0, 2), (1, 2), (0, 1)])
    return Tensor(a, 2, q, N)


def _hotrg_step_x(A1, A2, Uy):
    """src/schemes/hotrg.jl:62-80: A1[-1 1;3 5] A2[5 2;4 -4] conj(Uy[1 2;-2]) Uy[3 4;-3]"""
    a, q, N = _ein('aike,ejld,ijb,klc->abcd', A1, A2, ('c', Uy), Uy, path=[(0, 2), (0, 2), (0, 1)])
    return Tensor(a, 2, q, N)


def step_hotrg(scheme: HOTRG, chi):
    """src/schemes/hotrg.jl:154-160"""
    T = scheme.T
    Ux, lx, ex, pair = _hotrg_xproj(T, T, chi)
    T = _hotrg_step_y(T, T, Ux)
    Uy, ly, ey, pair2 = _hotrg_yproj(T, T, chi)
    T = _hotrg_step_x(T, T, Uy)
    scheme.T = T
    scheme.svals += [lx, ly]
    scheme.eps += [pair, pair2]


def _mmdag_3d(A1, A2):
    """src/schemes/hotrg3d.jl:48-65 (bosonic: the twists are identities)."""
    a, q, N = _ein('zwYXyx,vwYXyu->xzvu', A2, ('c', A2))
    M1 = Tensor(a, 4, q, N)
    a, q, N = _ein('xzvu,pzYXyr,pvYXys->rxsu', M1, A1, ('c', A1))
    return Tensor(0.5 * (a + np.transpose(a, (2, 3, 0, 1))), 2, q, N)


def _mdagm_3d(A1, A2):
    """src/schemes/hotrg3d.jl:67-84"""
    a, q, N = _ein('zwYxyX,vwYuyX->xzvu', ('c', A2), A2)
    M1 = Tensor(a, 4, q, N)
    a, q, N = _ein('xzvu,pzYryX,pvYsyX->rxsu', M1, ('c', A1), A1)
    return Tensor(0.5 * (a + np.transpose(a, (2, 3, 0, 1))), 2, q, N)


def _hotrg3d_xproj(A1, A2, chi):
    """src/schemes/hotrg3d.jl:86-98"""
    U, lam, eps = eigh_trunc(_mmdag_3d(A1, A2), 2, chi)
    U2, lam2, eps2 = eigh_trunc(_mdagm_3d(A1, A2), 2, chi)
    if eps > eps2:
        return U2, lam2, eps2, (eps, eps2)
    return U, lam, eps, (eps, eps2)


def _hotrg3d_yproj(A1, A2, chi):
    """src/schemes/hotrg3d.jl:100-106"""
    perm = (0, 1, 3, 2, 5, 4)
    return _hotrg3d_xproj(permute(A1, perm, 2), permute(A2, perm, 2), chi)


def _step_hotrg3d(A1, A2, Ux, Uy, max_entries=1 << 28):
    """src/schemes/hotrg3d.jl:108-117:
    T[-1 -2;-3 -4 -5 -6] = conj(Ux[x1 x2;-6]) Ux[x1' x2';-4] conj(Uy[y1 y2;-5]) Uy[y1' y2';-3]
                           A1[-1 z; y1' x1' y1 x1] A2[z -2; y2' x2' y2 x2]
    Contracted in an order whose largest intermediate has chi^8 entries (leading
    cost chi^11), sliced over the open leg -1 so no intermediate exceeds
    ``max_entries`` entries."""
    specs = ('azPQyx,QRd->azPyxRd', 'azPyxRd,PSc->azyxRdSc', 'azyxRdSc,zbSRuv->ayxdcbuv',
             'ayxdcbuv,xvf->aydcbuf', 'aydcbuf,yue->abcdef')
    # output charges: follow the labels through the whole network
    q, N = _charges('azPQyx,QRd,PSc,zbSRuv,xvf,yue->abcdef', A1, Ux, Uy, A2, ('c', Ux), ('c', Uy))
    da = A1.a.shape[0]
    per_a = int(np.prod(A1.a.shape[1:])) * max(Ux.a.shape[1], 1) * Uy.a.shape[1] * Uy.a.shape[2] * Ux.a.shape[2]
    chunk = max(1, min(da, max_entries // max(per_a, 1)))
    out = None
    for a0 in range(0, da, chunk):
        X = np.einsum(specs[0], A1.a[a0:a0 + chunk], Ux.a, optimize=True)
        Y = np.einsum(specs[1], X, Uy.a, optimize=True)
        del X
        Z = np.einsum(specs[2], Y, A2.a, optimize=True)
        del Y
        W = np.einsum(specs[3], Z, Ux.a, optimize=True)
        del Z
        part = np.einsum(specs[4], W, Uy.a, optimize=True)
        if out is None:
            out = np.empty((da,) + part.shape[1:])
        out[a0:a0 + chunk] = part
    return Tensor(out, 2, q, N)


def step_hotrg3d(scheme: HOTRG_3D, chi):
    """src/schemes/hotrg3d.jl:120-135"""
    for _ in range(3):
        T = scheme.T
        Ux, lx, ex, p1 = _hotrg3d_xproj(T, T, chi)
        Uy, ly, ey, p2 = _hotrg3d_yproj(T, T, chi)
        T = _step_hotrg3d(T, T, Ux, Uy)
        scheme.T = permute(T, (5, 3, 1, 2, 0, 4), 2)      # permute(T, ((6,4),(2,3,1,5)))
        scheme.svals += [lx, ly]
        scheme.eps += [p1, p2]


def _combine(terms):
    """sum of c * t for (c, t) pairs of equal-space tensors"""
    t0 = terms[0][1]
    return Tensor(sum(c * t.a for c, t in terms), t0.nout, t0.q, t0.N)


def step_impurity_hotrg(scheme: ImpurityHOTRG, chi):
    """src/schemes/impurityhotrg.jl:48-84: the y projector of the pure tensor, x-steps of the
    pure / impurity pairs; then the x projector and y-steps, with the symmetrised averages."""
    for proj, stepf in ((_hotrg_yproj, _hotrg_step_x), (_hotrg_xproj, _hotrg_step_y)):
        T, T11, T12, T2 = scheme.T, scheme.T_imp_order1_1, scheme.T_imp_order1_2, scheme.T_imp_order2
        U = proj(T, T, chi)[0]
        st = lambda a, b: stepf(a, b, U)          # noqa: E731
        scheme.T = st(T, T)
        scheme.T_imp_order1_1 = _combine([(0.5, st(T11, T)), (0.5, st(T, T11))])
        scheme.T_imp_order1_2 = _combine([(0.5, st(T12, T)), (0.5, st(T, T12))])
        scheme.T_imp_order2 = _combine([(0.25, st(T2, T)), (0.25, st(T, T2)), (0.25, st(T11, T12)),
                                        (0.25, st(T12, T11))])


def _svd_parts(t: Tensor, chi):
    """svd_trunc of a (2, 2) tensor: U[i1, i2; k], s, V[k; i3, i4] as tensors with charges."""
    U, s, Vh, _, bq = svd_trunc(t, 2, chi)
    qu = None if bq is None else [t.q[0], t.q[1], bq[0]]
    qv = None if bq is None else [bq[1], t.q[2], t.q[3]]
    return (lambda a: Tensor(a, 2, qu, t.N)), s, (lambda a: Tensor(a, 1, qv, t.N)), U, Vh


def _atrg_half(T: Tensor, chi):
    """_step!(::ATRG) (src/schemes/atrg.jl:47-81): SVD of T as (1,3) x (2,4) into A S D; the
    swapped pair M = (S D)(A S) is SVD'd into X Y (sqrt(S) on both); Q = A D X Y is SVD'd
    into H G (sqrt(S) on both) and T[-1 -2; -3 -4] = G[-1; -3 1] H[1 -2; -4]."""
    Tp = permute(T, (0, 2, 1, 3), 2)
    mkU, s1, mkV, U, Vh = _svd_parts(Tp, chi)
    A, D = mkU(U), mkV(Vh)
    C, B = mkU(U * s1), mkV(s1[:, None, None] * Vh)
    # M[-1 -2; -3 -4] := B[-3; 1 -4] C[-1 1; -2]
    a, q, N = _ein('cxd,axb->abcd', B, C)
    Mp = permute(Tensor(a, 2, q, N), (0, 2, 1, 3), 2)
    mkU, s2, mkV, U, Vh = _svd_parts(Mp, chi)
    r = np.sqrt(s2)
    X, Y = mkU(U * r), mkV(r[:, None, None] * Vh)
    # Q[-1 -2; -3 -4] := A[3 -3; 2] D[1; -2 4] X[4 2; -4] Y[-1 1; 3]
    a, q, N = _ein('czb,ayd,dbw,xac->xyzw', A, D, X, Y, path=[(0, 2), (0, 2), (0, 1)])
    Q = Tensor(a, 2, q, N)
    mkU, s3, mkV, U, Vh = _svd_parts(Q, chi)
    r = np.sqrt(s3)
    H, G = mkU(U * r), mkV(r[:, None, None] * Vh)
    # T[-1 -2; -3 -4] := G[-1; -3 1] H[1 -2; -4]
    a, q, N = _ein('acx,xbd->abcd', G, H)
    return Tensor(a, 2, q, N), [s1, s2, s3]


def step_atrg(scheme: ATRG, chi):
    """step!(::ATRG) (src/schemes/atrg.jl:38-45): a half step, permute ((2,4),(1,3)), a half
    step, permute ((3,1),(4,2))."""
    T, sv1 = _atrg_half(scheme.T, chi)
    T, sv2 = _atrg_half(permute(T, (1, 3, 0, 2), 2), chi)
    scheme.T = permute(T, (2, 0, 3, 1), 2)
    scheme.svals += sv1 + sv2


def _svd_dense(M, chi):
    """truncated SVD of a dense matrix (rank chi): U, s, Vh"""
    U, s, Vh = np.linalg.svd(M, full_matrices=False)
    k = min(chi, len(s))
    return U[:, :k], s[:k], Vh[:k]


def _left_orth_r(Mat):
    """left_orth (MatrixAlgebraKit QR): Mat = Q R, the R factor"""
    return np.linalg.qr(Mat, mode='r')


def _right_orth_l(Mat):
    """right_orth (MatrixAlgebraKit LQ): Mat = L Q, the L factor"""
    return np.linalg.qr(Mat.T, mode='r').T


def _atrg3d_half(T, chi):
    """_step!(::ATRG_3D) (src/schemes/atrg3d.jl:35-78) on a dense T[t1..t6]: SVD of (2,5,6) x
    (3,4,1) into A S D; M = (S D)(A S) SVD'd into X Y (sqrt(S) on both); AX and YD; the R factors
    of left_orth / right_orth of YD and AX on two leg pairs give the oblique projectors
    (R2 V1^T s1^-1/2, s1^-1/2 U1^T R1 with pseudopow), and T = G H."""
    d = T.shape
    U, s, Vh = _svd_dense(T.transpose(1, 4, 5, 2, 3, 0).reshape(d[1] * d[4] * d[5], -1), chi)
    k = len(s)
    U4 = U.reshape(d[1], d[4], d[5], k)                 # U[t2, t5, t6; k]
    V4 = Vh.reshape(k, d[2], d[3], d[0])                # V[k; t3, t4, t1]
    A = U4.transpose(3, 0, 1, 2)                        # A[k, t2; t5, t6]
    D = V4.transpose(3, 0, 1, 2)                        # D[t1, k; t3, t4]
    C = (U4 * s).transpose(3, 0, 1, 2)
    B = (s[:, None, None, None] * V4).transpose(3, 0, 1, 2)
    # M[-1 -2; -3 -4 -5 -6] := B[1 -2; -3 -4] C[-1 1; -5 -6]
    M = np.einsum('xbcd,axef->abcdef', B, C, optimize=True)
    m = M.shape
    U, s2, Vh = _svd_dense(M.transpose(1, 4, 5, 2, 3, 0).reshape(m[1] * m[4] * m[5], -1), chi)
    k2, r = len(s2), np.sqrt(s2)
    X = (U * r).reshape(m[1], m[4], m[5], k2).transpose(3, 0, 1, 2)                  # X[k2, m2; m5, m6]
    Y = (r[:, None] * Vh).reshape(k2, m[2], m[3], m[0]).transpose(3, 0, 1, 2)      # Y[m1, k2; m3, m4]
    # AX[-1 -2; -3 -4 -5 -6] := A[1 -2; -3 -5] X[-1 1; -4 -6];  YD likewise with Y, D
    AX = np.einsum('xbce,axdf->abcdef', A, X, optimize=True)
    YD = np.einsum('xbce,axdf->abcdef', Y, D, optimize=True)
    ax, yd = AX.shape, YD.shape

    r_left, r_right = _left_orth_r, _right_orth_l
    R1 = r_left(YD.reshape(-1, yd[4] * yd[5]))                                          # [r; y5 y6]
    R2 = r_right(AX.transpose(4, 5, 0, 1, 2, 3).reshape(ax[4] * ax[5], -1))            # [a5 a6; r]
    R3 = r_left(YD.transpose(0, 1, 4, 5, 2, 3).reshape(-1, yd[2] * yd[3]))              # [r; y3 y4]
    R4 = r_right(AX.transpose(2, 3, 0, 1, 4, 5).reshape(ax[2] * ax[3], -1))            # [a3 a4; r]

    def projectors(Rl, Rr):
        U1, s1, V1h = _svd_dense(Rl @ Rr, chi)
        inv = pseudopow(s1, -0.5)
        return Rr @ V1h.T * inv, (inv[:, None] * U1.T) @ Rl      # Proj_a [pq; k], Proj_b [k; pq]

    P1, P2 = projectors(R1, R2)
    P3, P4 = projectors(R3, R4)
    # H[-1 -2; -3 -4] := YD[-1 -2; 1 2 3 4] Proj_3[1 2; -3] Proj_1[3 4; -4]
    YDm = YD.reshape(yd[0] * yd[1], yd[2] * yd[3], yd[4] * yd[5])
    H = np.einsum('xpq,pc,qd->xcd', YDm, P3, P1, optimize=True).reshape(yd[0], yd[1], P3.shape[1], P1.shape[1])
    # G[-1 -2; -3 -4] := AX[-1 -2; 1 2 3 4] Proj_4[-3; 1 2] Proj_2[-4; 3 4]
    AXm = AX.reshape(ax[0] * ax[1], ax[2] * ax[3], ax[4] * ax[5])
    G = np.einsum('xpq,cp,dq->xcd', AXm, P4, P2, optimize=True).reshape(ax[0], ax[1], P4.shape[0], P2.shape[0])
    # T[-1 -2; -3 -4 -5 -6] := G[1 -2; -5 -6] H[-1 1; -3 -4]
    Tn = np.einsum('xbef,axcd->abcdef', G, H, optimize=True)
    return Tn, [s, s2]


def step_atrg3d(scheme: ATRG_3D, chi):
    """step!(::ATRG_3D) (src/schemes/atrg3d.jl:80-90): three half steps, each followed by
    permute(T, ((4, 6), (2, 5, 1, 3)))."""
    T = scheme.T.a
    for _ in range(3):
        T, sv = _atrg3d_half(T, chi)
        T = T.transpose(3, 5, 1, 4, 0, 2)
        scheme.svals += sv
    scheme.T = Tensor(np.ascontiguousarray(T), 2, None, 1)


def _correlation_phase(scheme: CorrelationHOTRG):
    """src/schemes/correlationhotrg.jl:177-185: 1 for the first dist steps, 2 for the merge, then 3."""
    if scheme.iter < scheme.dist:
        return 1
    return 2 if scheme.iter == scheme.dist else 3


def step_correlation_hotrg(scheme: CorrelationHOTRG, chi):
    """src/schemes/correlationhotrg.jl:94-135,177-250: the y projector of the pure tensor and
    x-steps, then the x projector and y-steps (the order of ImpurityHOTRG); an impurity step is
    the average of the (impurity, pure) and (pure, impurity) steps.  Phase 2's x-step merges the
    two impurities (their average, both orders); finalize! follows (src/utility/finalize.jl:104-124):
    phase 1 returns (n, n_1, n_2), phases 2 and 3 (n, n_imp, n_imp), every tensor /= n."""
    phase = _correlation_phase(scheme)
    for half, (proj, stepf) in enumerate(((_hotrg_yproj, _hotrg_step_x), (_hotrg_xproj, _hotrg_step_y))):
        T = scheme.Tpure
        U = proj(T, T, chi)[0]
        st = lambda a, b: stepf(a, b, U)                                   # noqa: E731
        sym = lambda a, b: _combine([(0.5, st(a, b)), (0.5, st(b, a))])   # noqa: E731
        if phase == 1:
            scheme.Timp1 = sym(scheme.Timp1, T)
            scheme.Timp2 = sym(scheme.Timp2, T)
        elif phase == 2 and half == 0:
            scheme.Timp_final = sym(scheme.Timp1, scheme.Timp2)
        else:
            scheme.Timp_final = sym(scheme.Timp_final, T)
        scheme.Tpure = st(T, T)
    tr = lambda t: abs(np.einsum('abba->', t.a))                           # noqa: E731
    n = tr(scheme.Tpure)
    if phase == 1:
        out = (float(n), float(tr(scheme.Timp1)), float(tr(scheme.Timp2)))
        live = (scheme.Tpure, scheme.Timp1, scheme.Timp2)
    else:
        ni = float(tr(scheme.Timp_final))
        out = (float(n), ni, ni)
        live = (scheme.Tpure, scheme.Timp_final)
        if phase == 2:
            scheme.Timp1 = scheme.Timp2 = None
    for t in live:
        t.a = t.a / n
    scheme.iter += 1
    return out


def run_correlation(scheme: CorrelationHOTRG, trunc, crit):
    """run!(::CorrelationHOTRG) (src/schemes/correlationhotrg.jl:138-162): no finalize at the
    beginning; each step returns its own 3-tuple; maxiter must exceed dist."""
    assert crit.n > scheme.dist, "niter must be larger than dist"
    data, steps, go = [], 0, True
    while go:
        data.append(step_correlation_hotrg(scheme, trunc.howmany))
        steps += 1
        go = crit(steps, data)
    return data


def correlation_ratio(scheme: CorrelationHOTRG):
    """|tr Timp_final| / |tr Tpure| (test/schemes.jl:506,517,530)."""
    return float(abs(np.einsum('abba->', scheme.Timp_final.a)) / abs(np.einsum('abba->', scheme.Tpure.a)))


def finalize_impurity_hotrg(scheme: ImpurityHOTRG):
    """src/utility/finalize.jl:91-101: the four trace norms; every tensor /= the pure one's."""
    tr = [abs(np.einsum('abba->', t.a)) for t in (scheme.T, scheme.T_imp_order1_1, scheme.T_imp_order1_2,
                                                  scheme.T_imp_order2)]
    for t in (scheme.T, scheme.T_imp_order1_1, scheme.T_imp_order1_2, scheme.T_imp_order2):
        t.a = t.a / tr[0]
    return tuple(float(x) for x in tr)


def step(scheme, chi):
    """``step!(scheme, truncrank(chi))`` dispatch (src/schemes/tnrscheme.jl:2)."""
    if isinstance(scheme, TRG):
        step_trg(scheme, chi)
    elif isinstance(scheme, BTRG):
        step_btrg(scheme, chi)
    elif isinstance(scheme, HOTRG):
        step_hotrg(scheme, chi)
    elif isinstance(scheme, HOTRG_3D):
        step_hotrg3d(scheme, chi)
    elif isinstance(scheme, ATRG):
        step_atrg(scheme, chi)
    elif isinstance(scheme, ATRG_3D):
        step_atrg3d(scheme, chi)
    elif isinstance(scheme, ImpurityHOTRG):
        step_impurity_hotrg(scheme, chi)
    elif isinstance(scheme, ImpurityTRG):
        step_impurity_trg(scheme, chi)
    else:
        raise TypeError(type(scheme))
    return scheme


def finalize(scheme):
    """src/utility/finalize.jl:4-14,62-66: trace norm, then T /= n (ImpurityHOTRG: the
    tuple of four norms, src/utility/finalize.jl:91-101)."""
    if isinstance(scheme, ImpurityHOTRG):
        return finalize_impurity_hotrg(scheme)
    if isinstance(scheme, ImpurityTRG):
        return finalize_impurity_trg(scheme)
    T = scheme.T.a
    if isinstance(scheme, (TRG, HOTRG, ATRG)):
        n = abs(np.einsum('abba->', T))                 # T[1 2; 2 1]
    elif isinstance(scheme, BTRG):
        # T[1 2; 4 3] S1[4; 2] S2[3; 1] with diagonal S1, S2
        n = abs(_btrg_trace(T, scheme.S1, scheme.S2))
    elif isinstance(scheme, (HOTRG_3D, ATRG_3D)):
        n = abs(np.einsum('aabcbc->', T))               # T[1 1; 2 3 2 3] (finalize.jl:56-66)
    else:
        raise TypeError(type(scheme))
    scheme.T.a = T / n
    return float(n)


# ---------------------------------------------------------------------------
# finalizers on the fixed-point tensor (src/utility/cft.jl, src/utility/finalize.jl:17-41)
# ---------------------------------------------------------------------------

def unit_tensor(scheme):
    """The tensor the fixed-point finalizers read: T itself, or for BTRG
    T_unit[-1 -2; -3 -4] = T[1 2; -3 -4] S1[-2; 2] S2[-1; 1] (src/utility/cft.jl:42-43), i.e.
    T[a, b, c, d] S1[b] S2[a] with the diagonal bond tensors."""
    T = scheme.T.a
    if isinstance(scheme, BTRG):
        return T * scheme.S1[None, :, None, None] * scheme.S2[:, None, None, None]
    return T


def transfer_matrix(scheme, unitcell=1):
    """The column transfer matrix of cft_data / ground_state_degeneracy (src/utility/cft.jl:7-15,
    278-296): unitcell copies of T_unit joined along the horizontal legs into a ring,
    indices [i, -i, -(i + u), i + 1] with the last leg closing on the first; rows are the
    upper legs (-1..-u), columns the lower ones.  unitcell 1: M[b, c] = sum_a T[a, b, c, a]."""
    T = unit_tensor(scheme)
    d = T.shape
    X = np.einsum('abcd->adbc', T)                      # X[a, a', b, c]: T as a map on the horizontal leg
    cur = X
    for _ in range(unitcell - 1):
        cur = np.einsum('xy...,yzbc->xz...bc', cur, X)
    M = np.einsum('xx...->...', cur)                     # close the ring: [b1, c1, b2, c2, ...]
    u = unitcell
    perm = [2 * i for i in range(u)] + [2 * i + 1 for i in range(u)]
    M = M.transpose(perm)
    return M.reshape(d[1] ** u, d[2] ** u)


def cft_data(scheme, v=1.0, unitcell=1, is_real=True):
    """src/utility/cft.jl:5-37 (BTRG :39-73): the transfer matrix's eigenvalues, sorted by
    magnitude (descending), those with real part <= 0 or magnitude <= 1e-12 dropped, as
    unitcell / (2 pi v) log(lambda_1 / lambda)."""
    lam = np.linalg.eigvals(transfer_matrix(scheme, unitcell))
    lam = lam[np.argsort(-np.abs(lam), kind='stable')]
    lam = lam[lam.real > 0]
    lam = lam[np.abs(lam) > 1e-12]
    if is_real:
        lam = lam.real
    return unitcell * (1.0 / (2.0 * math.pi * v)) * np.log(lam[0] / lam)


def ground_state_degeneracy(scheme, unitcell=1):
    """src/utility/cft.jl:278-340: exp of the Shannon entropy of |lambda / tr(D)| over the
    transfer matrix's nonzero eigenvalues."""
    lam = np.linalg.eigvals(transfer_matrix(scheme, unitcell))
    p = np.abs(lam / lam.sum())
    p = p[p != 0]
    return float(np.exp(-np.sum(p * np.log(p))))


def gu_wen_ratio(scheme):
    """src/utility/cft.jl:374-396: X1 = |T[1 2; 2 1]|^2 / |T[1 2; 2 3] T[3 4; 4 1]| and
    X2 = |T[1 2; 2 1]|^2 / |T[1 2; 3 4] T[4 3; 2 1]| of T_unit."""
    T = unit_tensor(scheme)
    one = abs(np.einsum('abba->', T))
    M = np.einsum('abbc->ac', T)
    x1 = abs(np.einsum('ac,ca->', M, M))
    x2 = abs(np.einsum('abcd,dcba->', T, T))
    return one ** 2 / x1, one ** 2 / x2


def central_charge(scheme, n):
    """src/utility/cft.jl:256-269: log(sigma_1) 6 / pi of M[-1; -2] = T[1 -1; -2 1] / n (BTRG:
    T[1 -1; 3 2] S1[3; -2] S2[2; 1] / n, i.e. sum_a T[a, b, c, a] S1[c] S2[a] / n)."""
    T = scheme.T.a
    if isinstance(scheme, BTRG):
        M = np.einsum('abca,c,a->bc', T, scheme.S1, scheme.S2) / n
    else:
        M = np.einsum('abca->bc', T) / n
    return float(math.log(np.linalg.svd(M, compute_uv=False)[0]) * 6.0 / math.pi)


def finalize_two_by_two(scheme):
    """src/utility/finalize.jl:17-41: n = |T[7 1; 5 4] T[4 2; 6 7] T[3 6; 2 8] T[8 5; 1 3]| over a
    2 x 2 plaquette (BTRG: with S1 on the bonds 1 and 6 and S2 on 8 and 4), T /= n^(1/4);
    returns n^(1/4)."""
    T = scheme.T.a
    T1 = T2 = T4 = T
    if isinstance(scheme, BTRG):
        T1 = T * scheme.S1[None, :, None, None] * scheme.S2[None, None, None, :]
        T2 = T * scheme.S1[None, :, None, None]
        T4 = T * scheme.S2[None, None, None, :]
    n = abs(np.einsum('gaed,dbfg,cfbh,heac->', T1, T2, T, T4, optimize=True))
    r = n ** 0.25
    scheme.T.a = T / r
    return float(r)


def _btrg_trace(T, S1, S2):
    """sum_{a,b} T[a,b,b,a] S1[b] S2[a] for diagonal S1 (leg 2) and S2 (leg 1)."""
    d1, d2 = T.shape[0], T.shape[1]
    ia = np.arange(d1)[:, None]
    ib = np.arange(d2)[None, :]
    return float(np.sum(T[ia, ib, ib, ia] * S1[None, :] * S2[:, None]))


@dataclass
class truncrank:
    """MatrixAlgebraKit ``truncrank(howmany)``"""
    howmany: int


@dataclass
class maxiter:
    """src/utility/stopping.jl:3-5,18: continue while steps < n."""
    n: int

    def __call__(self, steps, data):
        return steps < self.n


def run(scheme, trunc: truncrank, crit: maxiter, finalize_beginning=True, verbosity=0, finalizer=None):
    """src/schemes/tnrscheme.jl:33-57 with the default Finalizer (finalize!, Float64), or the
    given finalizer function (e.g. finalize_two_by_two); CorrelationHOTRG has its own run!
    (run_correlation)."""
    if isinstance(scheme, CorrelationHOTRG):
        return run_correlation(scheme, trunc, crit)
    fin = finalize if finalizer is None else finalizer
    data = []
    if finalize_beginning:
        data.append(fin(scheme))
    steps = 0
    go = True
    while go:
        step(scheme, trunc.howmany)
        data.append(fin(scheme))
        steps += 1
        go = crit(steps, data)
    return data


def free_energy(data, beta, scalefactor=2.0, initial_size=1.0):
    """src/utility/free_energy.jl:13-20"""
    lnz = 0.0
    x = 1.0 - math.log(initial_size) / math.log(scalefactor)
    for i, z in enumerate(data, start=1):
        lnz += math.log(z) * scalefactor ** (x - i)
    return -lnz / beta
