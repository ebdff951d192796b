"""Regenerate the golden fixtures under tests/golden/ from the reference checkout.

The fixtures are the reference's own known answers for this path:
  * class_Pk.txt   <- test/class_Pk.dat  (k [H0/c], P(k) [(c/H0)^3]; CLASS, ΛCDM(lmax=5)+Planck18)
  * class_Cl.txt   <- test/class_Cl.dat  (l, D_l^TT, D_l^EE, D_l^φφ; same model)
  * quadrature.txt <- paper/aa57450-25.tex:1370-1395 (momentum bins x_i and weights W_i, N=1..8)
Usage: python tests/golden/make_golden.py REFERENCE_ROOT   (the SymBoltz.jl checkout)
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    for src, dst in (("test/class_Pk.dat", "class_Pk.txt"), ("test/class_Cl.dat", "class_Cl.txt")):
        d = np.loadtxt(os.path.join(ref, src))
        np.savetxt(os.path.join(HERE, dst), d, fmt="%.16e",
                   header=f"copied from the reference's {src} (CLASS output used by test/runtests.jl)")
    tex = open(os.path.join(ref, "paper/aa57450-25.tex"), encoding="utf-8").read()
    start = tex.index("$N$ & $x_1$")
    block = tex[start:tex.index("\\bottomrule", start)]
    rows = [ln for ln in block.splitlines() if re.match(r"^\s*\d+ &", ln)]
    xs, ws = rows[:8], rows[8:16]
    out = []
    for rx, rw in zip(xs, ws):
        fx = [float(v) for v in rx.replace("\\\\", "").split("&")[1:] if v.strip()]
        fw = [float(v) for v in rw.replace("\\\\", "").split("&")[1:] if v.strip()]
        n = int(rx.split("&")[0])
        out.append([n] + fx + [0.0] * (8 - len(fx)) + fw + [0.0] * (8 - len(fw)))
    np.savetxt(os.path.join(HERE, "quadrature.txt"), np.array(out), fmt="%.5f",
               header="N x_1..x_8 W_1..W_8 (paper/aa57450-25.tex:1370-1395, 5 decimals)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_ROOT")
    main(sys.argv[1])
