"""Serving loop: requests admitted by HBM footprint, solved concurrently.  Each result in
the mix equals the same request solved alone (tolerance 1e-12: the kernels are
deterministic and every request owns its sketch seed)."""
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
        (tnr.classical_ising("Trivial", 0.35), "TRG", 16, 14),
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
        np.testing.assert_allclose(norms, alone[i // 2], rtol=1e-12)
        assert lat >= q >= 0.0
    srv.close()


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
