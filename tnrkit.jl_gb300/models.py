"""Initial partition-function tensors of the models the coarse-graining path runs on.

Host-side constructors (NumPy, FP64) that build the dense arrays TensorKit stores
for the reference's models; the arrays are indexed ``T[i1, i2, i3, i4]`` (leg order
left, down, up, right) and, for 3D, ``T[D, U, N, E, S, W]``.  Z_N-symmetric models
also carry the charge of every basis index so the engine can check conservation.

Reference: src/models/ising.jl, src/models/potts.jl, src/models/clock.jl.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

ising_βc = ising_beta_c = math.log(1.0 + math.sqrt(2.0)) / 2.0                      # ising.jl:1
f_onsager = -2.1096511446082074596677792835110847808254932754354                # ising.jl:2
ising_βc_3D = ising_beta_c_3D = 1.0 / 4.51152469                                # ising.jl:8


def potts_βc(q):
    """potts.jl:39"""
    return math.log(1.0 + math.sqrt(q))


potts_beta_c = potts_βc


@dataclass
class SymTensor:
    """Dense array plus the Z_N charge of each basis index of each leg (N = 1: Trivial)."""

    array: np.ndarray
    charges: list | None = None
    N: int = 1

    @property
    def shape(self):
        return self.array.shape


def _charges(d, nlegs, N):
    return None if N == 1 else [np.arange(d, dtype=np.int32) % N for _ in range(nlegs)]


def classical_ising(symmetry="Z2", beta=ising_βc, h=0.0):
    """``classical_ising(S, β; h)`` (ising.jl:10-15,39-67).  Trivial and Z2 share the array at h = 0."""
    if symmetry not in ("Z2", "Trivial"):
        raise ValueError("symmetry must be 'Trivial' or 'Z2'")
    if symmetry == "Z2" and h != 0.0:
        raise ValueError("External magnetic field is not compatible with Z2 symmetry")
    x, y = math.cosh(beta), math.sinh(beta)
    w = np.array([math.sqrt(x), math.sqrt(y)])
    par = np.add.outer(np.add.outer(np.arange(2), np.arange(2)), np.add.outer(np.arange(2), np.arange(2))) % 2
    init = np.where(par == 0, math.cosh(h * beta), math.sinh(h * beta))
    a = 2.0 * init * w[:, None, None, None] * w[None, :, None, None] * w[None, None, :, None] * w[None, None, None, :]
    N = 2 if symmetry == "Z2" else 1
    return SymTensor(np.ascontiguousarray(a), _charges(2, 4, N), N)


def classical_ising_impurity(beta=ising_βc, h=0.0):
    """``classical_ising_impurity(Trivial, β; h)`` (ising.jl:87-102): the magnetisation impurity,
    whose even-parity entries carry sinh(hβ) and odd-parity ones cosh(hβ)."""
    x, y = math.cosh(beta), math.sinh(beta)
    w = np.array([math.sqrt(x), math.sqrt(y)])
    par = np.add.outer(np.add.outer(np.arange(2), np.arange(2)), np.add.outer(np.arange(2), np.arange(2))) % 2
    init = np.where(par == 0, math.sinh(h * beta), math.cosh(h * beta))
    a = 2.0 * init * w[:, None, None, None] * w[None, :, None, None] * w[None, None, :, None] * w[None, None, None, :]
    return SymTensor(np.ascontiguousarray(a), None, 1)


def classical_ising_3D(symmetry="Z2", beta=ising_βc_3D, J=1.0):
    """``classical_ising_3D(Z2Irrep, β; J)`` (ising.jl:149-165): legs D, U', N, E, S', W'."""
    x, y = math.cosh(beta * J), math.sinh(beta * J)
    W = np.array([[math.sqrt(x), math.sqrt(y)], [math.sqrt(x), -math.sqrt(y)]])
    t = np.einsum('ai,aj,ak,al,am,an->ijklmn', W, W, W, W, W, W)
    a = np.ascontiguousarray(np.transpose(t, (0, 3, 4, 5, 1, 2)))   # permute(t, ((1,4),(5,6,2,3)))
    if symmetry == "Z2":
        return SymTensor(a, _charges(2, 6, 2), 2)
    if symmetry == "Trivial":
        # ising.jl:130-148: same model in the spin basis
        K = beta * J
        tm = np.array([[math.exp(K), math.exp(-K)], [math.exp(-K), math.exp(K)]])
        ev, v = np.linalg.eigh(tm)
        q = v @ np.diag(np.sqrt(ev)) @ v.T
        O = np.zeros((2,) * 6)
        O[(0,) * 6] = O[(1,) * 6] = 1.0
        b = np.einsum('abcdef,ia,jb,kc,ld,me,nf->ijklmn', O, q, q, q, q, q, q)
        return SymTensor(np.ascontiguousarray(b), None, 1)
    raise ValueError("symmetry must be 'Trivial' or 'Z2'")


def _zn_fourier(A, q):
    w = np.exp(2j * np.pi / q)
    P = np.array([[w ** (k * c) for c in range(q)] for k in range(q)]) / math.sqrt(q)
    U = np.einsum('ijkl,ia,jb,kc,ld->abcd', A.astype(complex), P.conj(), P.conj(), P, P)
    a = np.real(U)
    ch = np.arange(q)
    tot = (ch[:, None, None, None] + ch[None, :, None, None] - ch[None, None, :, None] - ch[None, None, None, :]) % q
    return np.ascontiguousarray(np.where(tot == 0, a, 0.0))


def classical_potts(q=3, beta=None, symmetry="ZN"):
    """``classical_potts(S, q, β)`` (potts.jl:22-30,68-81)."""
    beta = potts_βc(q) if beta is None else beta
    i = np.arange(q)
    d = (i[:, None] == i[None, :]).astype(float)
    E = -(d[:, :, None, None] + d[None, :, None, :] + d[None, None, :, :] + d.T[:, None, :, None])
    A = np.exp(-beta * E)
    if symmetry == "Trivial":
        return SymTensor(np.ascontiguousarray(A), None, 1)
    return SymTensor(_zn_fourier(A, q), _charges(q, 4, q), q)


def classical_clock(q=6, beta=1.0, symmetry="ZN"):
    """``classical_clock(S, q, β)`` (clock.jl:1-12,29-49), Trivial and Z_q."""
    i = np.arange(q)
    cl = -np.cos(2 * np.pi / q * (i[:, None] - i[None, :]))
    E = cl[:, :, None, None] + cl[None, :, None, :] + cl.T[None, None, :, :] + cl.T[:, None, :, None]
    A = np.exp(-beta * E)
    if symmetry == "Trivial":
        return SymTensor(np.ascontiguousarray(A), None, 1)
    return SymTensor(_zn_fourier(A, q), _charges(q, 4, q), q)


def sixvertex(symmetry="Trivial", a=1.0, b=1.0, c=1.0):
    """``sixvertex(Trivial; a, b, c)`` (sixvertex.jl:29-37): the vertex weights as T[i1, i2; i3, i4],
    a on the two all-equal configurations, c and b on the mixed ones.  The U(1)/CU(1) forms
    carry non-abelian or continuous sectors and are not built here."""
    if symmetry != "Trivial":
        raise ValueError("sixvertex: only the Trivial form runs on this engine")
    W = np.array([[a, 0, 0, 0], [0, c, b, 0], [0, b, c, 0], [0, 0, 0, a]], dtype=np.float64)
    return SymTensor(np.ascontiguousarray(W.reshape(2, 2, 2, 2, order="F")), None, 1)


def _phi4_gauss_hermite(K, mu0, lam, h, power):
    """Gauss-Hermite form of the real phi^4 site (phi4_real.jl:5-23,88-111): link matrix F = U S V
    on the quadrature nodes, T = sum_p sqrt(S)^4 y_p^power w_p e^{y_p^2} U U V V."""
    y, w = np.polynomial.hermite.hermgauss(K)
    yi, yj = y[:, None], y[None, :]
    F = np.exp(-0.5 * (yi - yj) ** 2 - mu0 / 8.0 * (yi ** 2 + yj ** 2) - lam / 16.0 * (yi ** 4 + yj ** 4) + h / 4.0 * (yi + yj))
    U, S, V = np.linalg.svd(F)
    left = U * np.sqrt(S)                      # [p, i]
    right = np.sqrt(S)[:, None] * V            # [k, p]
    weight = w * np.exp(y ** 2) * y ** power
    return np.ascontiguousarray(np.einsum("p,pi,pj,kp,lp->ijkl", weight, left, left, right, right))


def phi4_real(K, mu0, lam, h=0.0, symmetry="Z2"):
    """``phi4_real([S,] K, μ0, λ[, h])`` (phi4_real.jl:85-154).  Trivial: Gauss-Hermite quadrature
    with K nodes (bond dimension K).  Z2: the link term Taylor-expanded to order K-1, entries
    M_n / sqrt(s1! s2! s3! s4!) for even n = s1+s2+s3+s4 with M_n = ∫ exp(-(4+μ0)/2 φ² - λ/4 φ⁴) φⁿ dφ,
    even orders then odd orders as the two sectors (no field)."""
    if symmetry == "Trivial":
        return SymTensor(_phi4_gauss_hermite(K, mu0, lam, h, 0), None, 1)
    if symmetry != "Z2":
        raise ValueError("symmetry must be 'Trivial' or 'Z2'")
    if h != 0.0 or K % 2:
        raise ValueError("the Z2 form needs h = 0 and an even K")
    from scipy.integrate import quad
    a, b = (4.0 + mu0) / 2.0, lam / 4.0
    moments = {n: quad(lambda x, n=n: math.exp(-a * x * x - b * x ** 4) * x ** n, -math.inf, math.inf)[0]
               for n in range(0, 4 * (K - 1) + 1, 2)}
    half_log_fact = np.array([math.lgamma(k + 1) / 2.0 for k in range(K)])
    order = np.arange(K)
    n_tot = order[:, None, None, None] + order[None, :, None, None] + order[None, None, :, None] + order[None, None, None, :]
    scale = np.exp(-(half_log_fact[:, None, None, None] + half_log_fact[None, :, None, None]
                     + half_log_fact[None, None, :, None] + half_log_fact[None, None, None, :]))
    t = np.where(n_tot % 2 == 0, np.vectorize(lambda n: moments.get(int(n), 0.0))(n_tot), 0.0) * scale
    perm = np.r_[0:K:2, 1:K:2]                 # even orders (charge 0), then odd (charge 1)
    t = t[np.ix_(perm, perm, perm, perm)]
    q = np.r_[np.zeros(K // 2, dtype=np.int32), np.ones(K // 2, dtype=np.int32)]
    return SymTensor(np.ascontiguousarray(t), [q.copy() for _ in range(4)], 2)


def phi4_complex(symmetry, K, mu0, lam):
    """``phi4_complex(Trivial, K, μ0, λ)`` (phi4_complex.jl:6-36,108-138,194-206): Gauss-Hermite
    quadrature over the real and imaginary parts (K nodes each), bond dimension K²; the entries
    are real.  The U(1) and Z2×Z2 forms are not built here."""
    if symmetry != "Trivial":
        raise ValueError("phi4_complex: only the Trivial form runs on this engine")
    y, w = np.polynomial.hermite.hermgauss(K)
    re1, im1, re2, im2 = np.meshgrid(y, y, y, y, indexing="ij")
    F = np.exp(-0.5 * ((re1 - re2) ** 2 + (im1 - im2) ** 2) - mu0 / 8.0 * (re1 ** 2 + im1 ** 2 + re2 ** 2 + im2 ** 2)
               - lam / 16.0 * ((re1 ** 2 + im1 ** 2) ** 2 + (re2 ** 2 + im2 ** 2) ** 2)).reshape(K * K, K * K)
    U, S, V = np.linalg.svd(F)
    left = U * np.sqrt(S)
    right = np.sqrt(S)[:, None] * V
    weight = (w[:, None] * w[None, :] * np.exp(y[:, None] ** 2 + y[None, :] ** 2)).reshape(-1)
    return SymTensor(np.ascontiguousarray(np.einsum("p,pi,pj,kp,lp->ijkl", weight, left, left, right, right,
                                                    optimize=True)), None, 1)


def phi4_real_imp1(K, mu0, lam, h=0.0):
    """``phi4_real_imp1(Trivial, K, μ0, λ[, h])`` (phi4_real.jl:186-209): a φ insertion on the site."""
    return SymTensor(_phi4_gauss_hermite(K, mu0, lam, h, 1), None, 1)


def phi4_real_imp2(K, mu0, lam, h=0.0):
    """``phi4_real_imp2(Trivial, K, μ0, λ[, h])`` (phi4_real.jl:241-264): a φ² insertion on the site."""
    return SymTensor(_phi4_gauss_hermite(K, mu0, lam, h, 2), None, 1)


def random_hotrg_tensor(chi, seed, decay=6.0):
    """Seeded dense 4-leg tensor for the single-step HOTRG workload: N(0,1) entries times
    exp(-k/decay) per leg index k, normalised to Frobenius norm 1 (numpy PCG64)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = rng.standard_normal((chi,) * 4)
    s = np.exp(-np.arange(chi) / decay)
    a = a * s[:, None, None, None] * s[None, :, None, None] * s[None, None, :, None] * s[None, None, None, :]
    return SymTensor(a / np.linalg.norm(a), None, 1)
