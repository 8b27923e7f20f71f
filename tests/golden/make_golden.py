"""Extracts the reference's own golden values for the hot path from its sources, read as text,
into reference_golden.json (committed; the tests never read the reference tree).

    python tests/golden/make_golden.py /path/to/TNRKit.jl

Entries:
  * readme_btrg: README.md's BTRG example (classical_ising at ising_betac, truncrank(16),
    maxiter(25)): the printed free energy and its printed relative error to Onsager's value;
  * schemes: the @testset "<scheme> - Ising Model" free-energy checks of test/schemes.jl for
    TRG, BTRG and HOTRG: truncrank, maxiter, scalefactor and rtol against f_onsager.
Every entry records the file and line it came from.
"""
import json
import os
import re
import sys


def readme_btrg(root):
    path = os.path.join(root, "README.md")
    lines = open(path, encoding="utf-8").read().splitlines()
    out = {}
    for i, l in enumerate(lines, 1):
        m = re.search(r"f = free_energy\(data, ising_βc\) # (-?[0-9.]+)", l)
        if m:
            out["f"] = m.group(1)
            out["f_source"] = "README.md:%d" % i
        m = re.fullmatch(r"\s*([0-9.]+e-[0-9]+)\s*", l)
        if m and "f" in out and "rel_err_onsager" not in out:
            out["rel_err_onsager"] = float(m.group(1))
            out["rel_err_source"] = "README.md:%d" % i
        m = re.search(r"run!\(scheme, truncrank\((\d+)\), maxiter\((\d+)\)\)", l)
        if m and "chi" not in out:
            out["chi"], out["maxiter"] = int(m.group(1)), int(m.group(2))
            out["run_source"] = "README.md:%d" % i
    out["scheme"] = "BTRG"
    return out


def schemes(root):
    path = os.path.join(root, "test", "schemes.jl")
    lines = open(path, encoding="utf-8").read().splitlines()
    out, current = [], None
    for i, l in enumerate(lines, 1):
        m = re.search(r'@testset "(\w+) - Ising Model"', l)
        if m:
            current = {"scheme": m.group(1), "testset_source": "test/schemes.jl:%d" % i}
            continue
        if current is None:
            continue
        m = re.search(r"data = run!\(scheme, truncrank\((\d+)\), maxiter\((\d+)\)\)", l)
        if m and "chi" not in current:
            current["chi"], current["maxiter"] = int(m.group(1)), int(m.group(2))
            continue
        m = re.search(r"@test free_energy\(data, ising_βc(?:; scalefactor = ([0-9.]+))?\) ≈ f_onsager rtol = ([0-9.e-]+)", l)
        if m and "chi" in current:
            current["scalefactor"] = float(m.group(1)) if m.group(1) else 2.0
            current["rtol"] = float(m.group(2))
            current["check_source"] = "test/schemes.jl:%d" % i
            if current["scheme"] in ("TRG", "BTRG", "HOTRG"):
                out.append(current)
            current = None
    return out


def main():
    root = sys.argv[1]
    data = {"reference": "TNRKit.jl (read as text)", "readme_btrg": readme_btrg(root), "schemes": schemes(root)}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.json")
    with open(dst, "w") as f:
        json.dump(data, f, indent=1, ensure_ascii=False)
        f.write("\n")
    print(dst)


if __name__ == "__main__":
    main()
