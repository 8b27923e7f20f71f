"""A NumPy replay of the engine's index bookkeeping for the device paths that are new around
the hot path, checked against the oracle on the CPU.

The replay follows the C++ line by line: column-major tensors (first leg fastest, so every
matrix view is an order='F' reshape), the label-based pairwise `contract`, `permuted`, the
SVD views of `svd22`, and the leg scalings. It covers `atrg_half` / `step_atrg`
(csrc/schemes.cu), `atrg3d_half` / `step_atrg3d` with R factors taken in a rotated basis as
CholeskyQR3 produces them, `ring_transfer`, the 2 x 2 plaquette labels, the Gu-Wen sums
(csrc/fixedpoint.cu), `trg_contract`, and the ImpurityTRG plaquette. A wrong label or leg order
in the C++ shows up here as a mismatch with the oracle before the path runs on a GPU.
"""
import numpy as np


def permuted(T, perm):
    return np.transpose(T, perm)


def contract(A, la, B, lb, lout):
    L = 'abcdefghijklmnopqrstuvwxyz'
    return np.einsum(''.join(L[i] for i in la) + ',' + ''.join(L[i] for i in lb) + '->' + ''.join(L[i] for i in lout), A, B)


La, Lb, Lc, Ld, Le, Lf, Lg, Lh, Li, Lj, Lk, Ll, Lm, Ln, Lo, Lp, Lq, Lr, Ls, Lt, Lu, Lv, Lw, Lx, Ly, Lz = range(26)


def tsvd(Mat, k):
    U, s, Vh = np.linalg.svd(Mat, full_matrices=False)
    return U[:, :k], s[:k], Vh[:k]


def svd22(M4, chi):
    m = M4.shape[0] * M4.shape[1]; n = M4.shape[2] * M4.shape[3]
    k = min(chi, m, n)
    U, s, Vt = tsvd(M4.reshape(m, n, order='F'), k)
    return U.reshape(M4.shape[0], M4.shape[1], k, order='F'), s, Vt.reshape(k, M4.shape[2], M4.shape[3], order='F')


def scale_leg(T, leg, v):
    sh = [1] * T.ndim; sh[leg] = -1
    return T * v.reshape(sh)


def atrg_half(T, chi):
    Tp = permuted(T, (0, 2, 1, 3))
    A, s1, D = svd22(Tp, chi)
    C = scale_leg(A, 2, s1); B = scale_leg(D, 0, s1)
    M = contract(B, [Lc, Lx, Ld], C, [La, Lx, Lb], [La, Lb, Lc, Ld])
    Mp = permuted(M, (0, 2, 1, 3))
    X, s2, Y = svd22(Mp, chi)
    X = scale_leg(X, 2, np.sqrt(s2)); Y = scale_leg(Y, 0, np.sqrt(s2))
    AX = contract(A, [Lc, Lz, Lb], X, [Ld, Lb, Lw], [Lc, Lz, Ld, Lw])
    YD = contract(Y, [Lx, La, Lc], D, [La, Ly, Ld], [Lx, Lc, Ly, Ld])
    Q = contract(YD, [Lx, Lc, Ly, Ld], AX, [Lc, Lz, Ld, Lw], [Lx, Ly, Lz, Lw])
    H, s3, G = svd22(Q, chi)
    H = scale_leg(H, 2, np.sqrt(s3)); G = scale_leg(G, 0, np.sqrt(s3))
    return contract(G, [La, Lc, Lx], H, [Lx, Lb, Ld], [La, Lb, Lc, Ld])


def step_atrg(T, chi):
    T = atrg_half(T, chi)
    T = atrg_half(permuted(T, (1, 3, 0, 2)), chi)
    return permuted(T, (2, 0, 3, 1))


_rng = np.random.default_rng(0)


def qr_r(Mat):
    # CholeskyQR-style: Q with orthonormal columns spanning Mat, in a basis unlike LAPACK's, then R = Q^T Mat
    Q, _ = np.linalg.qr(Mat)
    Q = Q @ np.linalg.qr(_rng.standard_normal((Q.shape[1], Q.shape[1])))[0]
    return Q.T @ Mat


def pseudopow(s, a, tol=np.finfo(float).eps ** 0.75):
    out = s.copy(); m = s >= tol; out[m] = s[m] ** a; return out


def oblique(Rl, Rrt, chi):
    n = Rl.shape[1]
    tmp = Rl @ Rrt.T
    k = min(chi, n)
    U, s, Vt = tsvd(tmp, k)
    inv = pseudopow(s, -0.5)
    Pa = (Rrt.T @ Vt.T) * inv
    Pb = (inv[:, None] * U.T) @ Rl
    return Pa, Pb, k


def atrg3d_half(T, chi):
    Tp = permuted(T, (1, 4, 5, 2, 3, 0))
    m = np.prod(Tp.shape[:3]); n = np.prod(Tp.shape[3:])
    k = min(chi, m, n)
    U, sv, V = tsvd(Tp.reshape(m, n, order='F'), k)
    U = U.reshape(*Tp.shape[:3], k, order='F'); V = V.reshape(k, *Tp.shape[3:], order='F')
    A = permuted(U, (3, 0, 1, 2)); D = permuted(V, (3, 0, 1, 2))
    C = scale_leg(A, 0, sv); B = scale_leg(D, 1, sv)
    M = contract(B, [Lx, Lb, Lc, Ld], C, [La, Lx, Le, Lf], [La, Lb, Lc, Ld, Le, Lf])
    Mp = permuted(M, (1, 4, 5, 2, 3, 0))
    m = np.prod(Mp.shape[:3]); n = np.prod(Mp.shape[3:])
    k = min(chi, m, n)
    U, sv, V = tsvd(Mp.reshape(m, n, order='F'), k)
    U = U * np.sqrt(sv); V = np.sqrt(sv)[:, None] * V
    U = U.reshape(*Mp.shape[:3], k, order='F'); V = V.reshape(k, *Mp.shape[3:], order='F')
    X = permuted(U, (3, 0, 1, 2)); Y = permuted(V, (3, 0, 1, 2))
    AX = contract(A, [Lx, Lb, Lc, Le], X, [La, Lx, Ld, Lf], [La, Lb, Lc, Ld, Le, Lf])
    YD = contract(Y, [Lx, Lb, Lc, Le], D, [La, Lx, Ld, Lf], [La, Lb, Lc, Ld, Le, Lf])
    y0, y1, x0, x1 = YD.shape[0], YD.shape[1], AX.shape[0], AX.shape[1]
    ab_y, ab_x = y0 * y1, x0 * x1
    n1 = YD.shape[4] * YD.shape[5]; n3 = YD.shape[2] * YD.shape[3]
    assert n1 == AX.shape[4] * AX.shape[5] and n3 == AX.shape[2] * AX.shape[3]
    R1 = qr_r(YD.reshape(ab_y * n3, n1, order='F'))
    R2t = qr_r(AX.reshape(ab_x * n3, n1, order='F'))
    P1, P2, k1 = oblique(R1, R2t, chi)
    YDp = permuted(YD, (0, 1, 4, 5, 2, 3)); AXp = permuted(AX, (0, 1, 4, 5, 2, 3))
    R3 = qr_r(YDp.reshape(ab_y * n1, n3, order='F'))
    R4t = qr_r(AXp.reshape(ab_x * n1, n3, order='F'))
    P3, P4, k3 = oblique(R3, R4t, chi)
    YD3 = YD.reshape(ab_y, n3, n1, order='F'); AX3 = AX.reshape(ab_x, n3, n1, order='F')
    Z = contract(YD3, [La, Lp, Lq], P1, [Lq, Lb], [La, Lp, Lb])
    H = contract(Z, [La, Lp, Lb], P3, [Lp, Lc], [La, Lc, Lb])
    Z = contract(AX3, [La, Lp, Lq], P2, [Lb, Lq], [La, Lp, Lb])
    G = contract(Z, [La, Lp, Lb], P4, [Lc, Lp], [La, Lc, Lb])
    H = H.reshape(y0, y1, k3, k1, order='F'); G = G.reshape(x0, x1, k3, k1, order='F')
    return contract(G, [Lx, Lb, Le, Lf], H, [La, Lx, Lc, Ld], [La, Lb, Lc, Ld, Le, Lf])


def _run(T, step, trace, chi, n):
    out = []
    t = trace(T)
    T = T / t
    out.append(t)
    for _ in range(n):
        T = step(T, chi)
        t = trace(T)
        T = T / t
        out.append(t)
    return np.array(out)


def _tr2(T):
    return abs(np.einsum('abba->', T))


def _tr3(T):
    return abs(np.einsum('aabcbc->', T))


def test_atrg_replay(oracle):
    o = oracle
    e = _run(o.classical_ising(o.ISING_BETA_C, "Trivial").a, step_atrg, _tr2, 16, 6)
    r = np.array(o.run(o.ATRG(o.classical_ising(o.ISING_BETA_C, "Trivial")), o.truncrank(16), o.maxiter(6)))
    np.testing.assert_allclose(e, r, rtol=1e-11)


def test_atrg3d_replay(oracle):
    o = oracle

    def step3(T, chi):
        for _ in range(3):
            T = permuted(atrg3d_half(T, chi), (3, 5, 1, 4, 0, 2))
        return T

    e = _run(o.classical_ising_3D(symmetry="Trivial").a, step3, _tr3, 6, 5)
    r = np.array(o.run(o.ATRG_3D(o.classical_ising_3D()), o.truncrank(6), o.maxiter(5)))
    np.testing.assert_allclose(e, r, rtol=1e-10)


def test_fixed_point_and_impurity_labels(oracle):
    o = oracle
    s = o.TRG(o.classical_ising(o.ISING_BETA_C, "Trivial"))
    o.run(s, o.truncrank(12), o.maxiter(5))
    T = s.T.a
    # ring_transfer with unitcell 2: chain, close the ring, order rows (b1, b2) and columns (c1, c2)
    da, db, dc = T.shape[0], T.shape[1], T.shape[2]
    nxt = contract(T.reshape(da, -1, da, order='F'), [La, Lb, Lx], T, [Lx, Lc, Ld, Le], [La, Lb, Lc, Ld, Le])
    P = nxt.reshape(da, -1, da, order='F')
    ring = np.einsum('aia->i', P).reshape(db, dc, db, dc, order='F')
    M = permuted(ring, (0, 2, 1, 3)).reshape(db * db, dc * dc, order='F')
    np.testing.assert_allclose(np.sort_complex(np.linalg.eigvals(M)),
                               np.sort_complex(np.linalg.eigvals(o.transfer_matrix(s, 2))), atol=1e-13)
    # the 2 x 2 plaquette of finalize_two_by_two_async
    X = contract(T, [Lg, La, Le, Ld], T, [Ld, Lb, Lf, Lg], [La, Le, Lb, Lf])
    Y = contract(T, [Lc, Lf, Lb, Lh], T, [Lh, Le, La, Lc], [Lf, Lb, Le, La])
    assert np.isclose(np.einsum('aebf,fbea->', X, Y), np.einsum('gaed,dbfg,cfbh,heac->', T, T, T, T), rtol=1e-13)
    # the Gu-Wen sums of k_gu_wen_partial / k_gu_wen_sums
    one = np.einsum('abba->', T)
    Pm = np.einsum('abbc->ac', T)
    x1 = one ** 2 / abs(np.einsum('ac,ca->', Pm, Pm))
    x2 = one ** 2 / abs(np.einsum('abcd,dcba->', T, T))
    np.testing.assert_allclose((x1, x2), o.gu_wen_ratio(s), rtol=1e-13)
    # trg_contract and the ImpurityTRG plaquette labels
    rng = np.random.default_rng(1)
    D, B = rng.standard_normal((3, 4, 4)), rng.standard_normal((3, 4, 4))
    C, A = rng.standard_normal((4, 4, 3)), rng.standard_normal((4, 4, 3))
    Xx = contract(D, [Lb, Lp, Lq], B, [La, Lr, Lp], [La, Lb, Lq, Lr])
    Yy = contract(C, [Lr, Ls, Lc], A, [Ls, Lq, Ld], [Lq, Lr, Lc, Ld])
    np.testing.assert_allclose(contract(Xx, [La, Lb, Lq, Lr], Yy, [Lq, Lr, Lc, Ld], [La, Lb, Lc, Ld]),
                               np.einsum('bpq,arp,rsc,sqd->abcd', D, B, C, A), atol=1e-12)
    t = [rng.standard_normal((3, 4, 4, 3)) for _ in range(4)]
    Xp = contract(t[0], [Le, Ld, Lf, La], t[1], [La, Lb, Lg, Le], [Ld, Lf, Lb, Lg])
    Yp = contract(t[2], [Lc, Lg, Lb, Lh], t[3], [Lh, Lf, Ld, Lc], [Lg, Lb, Lf, Ld])
    assert np.isclose(np.einsum('dfbg,gbfd->', Xp, Yp), np.einsum('edfa,abge,cgbh,hfdc->', *t), rtol=1e-12)
