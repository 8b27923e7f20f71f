"""GEMM probes through the C ABI.

``python tnrkit.jl_gb300/gemm_probe.py 4096`` runs the split-precision tcgen05 GEMM on
seeded n x n x n operands (``tnr_debug_gemm``, the contraction path), twice, and prints its
relative error against FP64.

``python tnrkit.jl_gb300/gemm_probe.py contract 2304 2304 4`` runs one batched product on the
contraction path (chunked accumulation), the target of ncu captures of
``k_gemm_split_tc_chunked``; ``single`` instead of ``contract`` runs the single-accumulation
kernel ``k_gemm_split_tc`` of the truncated SVD's products.

``python tnrkit.jl_gb300/gemm_probe.py shapes`` times (``tnr_gemm_time``, CUDA events,
device-resident operands) the batched products of one BTRG step of a lockstep group
of 51 instances at chi = 48 and chi = 32 -- the contractions of the coarse-graining step
(chunked accumulation; the large-K one also with a single accumulation) and the products
of the truncated SVD -- in both precisions, with the per-class split of the time (plane
pass / GEMM) from the engine's launch profiler.
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import __graft_entry__ as ge  # noqa: E402


def error_probe(tnr, n):
    rng = np.random.default_rng(1)
    A = rng.standard_normal((n, n))
    B = rng.standard_normal((n, n))
    C = None
    for _ in range(2):
        C = tnr.debug_gemm(A, B, False, False, tnr.PREC_SPLIT)
    ref = A @ B
    print("n=%d rel err %.3e" % (n, np.linalg.norm(C - ref) / np.linalg.norm(ref)))


def step_shapes(chi, batch):
    m = chi * chi
    r = min(128, (3 * chi + 7) // 8 * 8)
    return [
        ("contract X=D.B (k=chi)", m, m, chi, batch, False, False, True),
        ("contract T=X.Y (k=chi^2)", m, m, m, batch, False, False, True),
        ("  same, one accumulation", m, m, m, batch, False, False, False),
        ("tsvd Y=M.Q", m, r, m, batch, False, False, False),
        ("tsvd Z=M^T.U", m, r, m, batch, True, False, False),
        ("tsvd gram Z^T Z", r, r, m, batch, True, False, False),
        ("tsvd rotate Z.W", m, r, r, batch, False, False, False),
    ]


def shapes_probe(tnr, reps):
    print("%-26s %6s %6s %6s %5s %6s %10s %10s %10s %10s" % ("product", "m", "n", "k", "batch", "prec", "ms",
                                                           "TF/s(2mnk)", "plane ms", "gemm ms"))
    for chi in (48, 32):
        for name, m, n, k, b, ta, tb, con in step_shapes(chi, 51):
            for prec, tag in ((tnr.PREC_SPLIT, "split"), (tnr.PREC_F64, "f64")):
                if prec == tnr.PREC_SPLIT and (m < 64 or n < 16 or k < 16):
                    continue
                if prec == tnr.PREC_F64 and not con and name.startswith("  "):
                    continue
                tnr.profile_reset()
                tnr.profile_enable(True)
                ms = tnr.gemm_time(m, n, k, b, ta, tb, prec, reps, con)
                tnr.profile_enable(False)
                prof = tnr.profile_read()
                calls = reps + 1
                plane = prof["split"][1] / calls
                gemm = (prof["tc"][1] + prof["gemm_bulk"][1] + prof["gemm_f64"][1]) / calls
                tf = 2.0 * m * n * k * b / (ms * 1e-3) / 1e12
                print("%-26s %6d %6d %6d %5d %6s %10.3f %10.1f %10.3f %10.3f" % (name, m, n, k, b, tag, ms, tf, plane,
                                                                              gemm), flush=True)


def contract_probe(tnr, m, k, batch, contraction=True):
    """One warm-up and one timed batched m x m x k product on the contraction path (the
    chunked kernel when k > 64), or with contraction=False on the single-accumulation
    kernel of the truncated SVD's products: the targets of ncu captures."""
    ms = tnr.gemm_time(m, m, k, batch, False, False, tnr.PREC_SPLIT, 1, contraction)
    print("%s m=n=%d k=%d batch=%d: %.3f ms, %.1f TFLOP/s (2mnk)" % (
        "contract" if contraction else "single", m, k, batch, ms, 2.0 * m * m * k * batch / ms / 1e9))


def main():
    arg = sys.argv[1] if len(sys.argv) > 1 else "4096"
    ge.build()
    tnr = ge.package()
    if arg == "shapes":
        shapes_probe(tnr, int(sys.argv[2]) if len(sys.argv) > 2 else 3)
    elif arg in ("contract", "single"):
        contract_probe(tnr, int(sys.argv[2]), int(sys.argv[3]), int(sys.argv[4]), arg == "contract")
    else:
        error_probe(tnr, int(arg))


if __name__ == "__main__":
    main()
