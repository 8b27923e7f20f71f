"""Serving loop: requests admitted by HBM footprint, solved concurrently.  Each result in
the mix equals the same request solved alone: to 1e-12 for a request solved on its own
stream (the kernels are deterministic and every request owns its sketch seed), and to 1e-10
for TRG/BTRG requests that the server batches with equal ones (one lockstep group: a shared
random start and the group's iteration count change the rounding, on well-conditioned
instances)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tnr():
    import __graft_entry__ as ge
    ge.build()
    return ge.package()


def _requests(tnr):
    return [
        (tnr.classical_ising("Z2", 0.44), "BTRG", 12, 12),
        (tnr.classical_potts(3, 1.1), "HOTRG", 10, 8),
        (tnr.classical_clock(6, 0.8), "BTRG", 9, 10),
        (tnr.classical_ising("Trivial", 0.44), "TRG", 24, 14),
        (tnr.classical_ising_3D(), "HOTRG_3D", 4, 3),
        (tnr.classical_ising("Z2", 0.52), "HOTRG", 12, 10),
    ]


@pytest.mark.parametrize("precision", ["f64", "split"])
def test_mix_equals_alone(tnr, precision):
    prec = tnr.PREC_F64 if precision == "f64" else tnr.PREC_SPLIT
    reqs = _requests(tnr)
    alone = []
    for T, sch, chi, n in reqs:
        s = getattr(tnr, sch)(T, precision=prec)
        alone.append(tnr.run(s, tnr.truncrank(chi), tnr.maxiter(n)))
        s.close()
    srv = tnr.Server(hbm_budget_bytes=40 << 30, max_active=8, precision=prec)
    ids = [srv.submit(T, sch, chi, n) for T, sch, chi, n in reqs for _ in range(2)]
    for i, rid in enumerate(ids):
        norms, lat, q = srv.result(rid)
        T, sch = reqs[i // 2][:2]
        batchable = sch in ("TRG", "BTRG") and getattr(T, "N", 1) == 1
        np.testing.assert_allclose(norms, alone[i // 2], rtol=1e-10 if batchable else 1e-12)
        assert lat >= q >= 0.0
    srv.close()


def test_server_batches_equal_requests(tnr):
    """Continuous batching: three equal BTRG requests that queue behind a running one are
    admitted together and stepped as one lockstep group, so their results equal a lockstep
    batch of the same three (run_batch) to rounding, and the plain solve to 1e-10."""
    srv = tnr.Server(hbm_budget_bytes=40 << 30, max_active=1)
    first = srv.submit(tnr.classical_ising("Trivial", 0.44), "HOTRG", 24, 8)      # occupies the one slot
    T = tnr.classical_ising("Trivial", 0.44)
    ids = [srv.submit(T, "BTRG", 24, 8) for _ in range(3)]
    got = [srv.result(r)[0] for r in ids]
    srv.result(first)
    srv.close()
    ref = tnr.run_batch([tnr.BTRG(T) for _ in range(3)], [24] * 3, [8] * 3)
    alone = tnr.run(tnr.BTRG(T), tnr.truncrank(24), tnr.maxiter(8))
    for g, r in zip(got, ref):
        np.testing.assert_allclose(g, r, rtol=1e-13)
        np.testing.assert_allclose(g, alone, rtol=1e-10)


def test_admission_and_queueing(tnr):
    T = tnr.classical_ising("Trivial", 0.44)
    need = tnr.footprint_bytes("BTRG", 16, T.shape)
    # a budget for one request at a time: the others queue and are admitted as memory frees
    srv = tnr.Server(hbm_budget_bytes=int(need * 1.5), max_active=4)
    ids = [srv.submit(T, "BTRG", 16, 6) for _ in range(4)]
    qs = [srv.result(r)[2] for r in ids]
    assert max(qs) > 0.0
    ref = srv.result(ids[0])[0]
    for r in ids[1:]:
        np.testing.assert_allclose(srv.result(r)[0], ref, rtol=1e-12)
    # a request that can never fit is refused at submission
    with pytest.raises(tnr.TNRError) as e:
        srv.submit(T, "HOTRG", 4096, 3)
    assert e.value.status == 5
    srv.close()
