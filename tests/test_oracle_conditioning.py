"""Conditioning of the oracle's norms under a tiny perturbation of the input tensor.

The GPU parity tests hold the engine to 1e-10 / 1e-11 only where the problem allows it:
at beta in [0.40, 0.47] the oracle's norms move by at most ~2e-13 under a 1e-14 relative
perturbation of the initial tensor, while at beta = 0.33 a near-tie sits at the truncation
cut and they move by ~1e-7 (two runs with different rounding may keep different vectors
there).  These checks pin that statement for the lockstep tests' betas.
"""
import numpy as np
import pytest


def _sensitivity(o, cls, chi, beta, steps=12, seed=5):
    rng = np.random.default_rng(seed)
    n0 = np.array(o.run(getattr(o, cls)(o.classical_ising(beta, "Trivial")), o.truncrank(chi), o.maxiter(steps)))
    T = o.classical_ising(beta, "Trivial")
    T.a = T.a * (1 + 1e-14 * rng.standard_normal(T.a.shape))
    n1 = np.array(o.run(getattr(o, cls)(T), o.truncrank(chi), o.maxiter(steps)))
    return float(np.abs(n1 / n0 - 1).max())


@pytest.mark.parametrize("cls,chi", [("TRG", 16), ("BTRG", 24)])
@pytest.mark.parametrize("beta", [0.40, 0.44, 0.47])
def test_lockstep_betas_are_well_conditioned(oracle, cls, chi, beta):
    assert _sensitivity(oracle, cls, chi, beta) < 1e-12


def test_high_temperature_near_tie_is_ill_conditioned(oracle):
    assert _sensitivity(oracle, "TRG", 16, 0.33) > 1e-9
