"""Runs the split-precision tcgen05 GEMM on seeded n x n x n operands through the C ABI
(``tnr_debug_gemm``), twice, and prints its relative error against FP64.

Used as the target of ncu captures of ``k_gemm_split_tc``:
    python tnrkit.jl_gb300/gemm_probe.py 4096
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import __graft_entry__ as ge  # noqa: E402


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 4096
    ge.build()
    tnr = ge.package()
    rng = np.random.default_rng(1)
    A = rng.standard_normal((n, n))
    B = rng.standard_normal((n, n))
    C = None
    for _ in range(2):
        C = tnr.debug_gemm(A, B, False, False, tnr.PREC_SPLIT)
    ref = A @ B
    print("n=%d rel err %.3e" % (n, np.linalg.norm(C - ref) / np.linalg.norm(ref)))


if __name__ == "__main__":
    main()
