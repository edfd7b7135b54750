"""Regenerates tests/golden/reference_overlaps.json: Slater-orbital overlaps
computed with the reference's own formula and table.

MolDS evaluates the diatomic-frame overlap of two valence Slater orbitals
(Cndo2::CalcDiatomicOverlapAOsInDiatomicFrame, src/cndo/Cndo2.cpp:5801-5869)
as
    S = pre * D(la, lb, m) * sum_ij Y[na][nb][la][lb][m][i][j] A_i(p) B_j(q),
    p = (alpha + beta) / 2, q = (alpha - beta) / 2, alpha = zeta_A R, beta = zeta_B R,
    pre = (2 zeta_A)^(na+1/2) (2 zeta_B)^(nb+1/2) / sqrt((2 na)! (2 nb)!) (R/2)^(na+nb+1),
with Pople's reduced-overlap coefficients Y (the generated table
src/cndo/ReducedOverlapAOsParameters.h, integers) and the auxiliary
integrals A_k (Cndo2.cpp:6385-6400), B_k (:6413-6447) and D (:6459-6477).
This script restates those steps in Python, reads the Y table from the
reference's header as text, and writes the overlaps of s / p-sigma / p-pi
pairs for the exponents and valence shells of H, C, N, O, S and Cl at a range
of distances: "S" evaluated in 60-digit arithmetic (the value the formula
defines) and "S_double" as the reference's double-precision code evaluates it
(its closed-form B_k loses digits to cancellation when |q| is small and k
large).  The oracle computes the same overlaps by its own prolate-spheroidal
expansion; tests/test_overlap_cpu.py compares the two.

Usage:  python tests/golden/make_overlaps.py <path to the MolDS src directory>
"""
import json
import math
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_y(src):
    t = open(os.path.join(src, "cndo", "ReducedOverlapAOsParameters.h")).read()
    iy = t.index("ReducedOverlapAOsParameters::Y[")
    body = t[t.index("{", iy) + 1:t.index("}", iy)]
    vals = [float(x) for x in re.findall(r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?", body)]
    return np.array(vals).reshape(5, 5, 4, 4, 4, 9, 9)   # ShellType_end = 4


def aux_a(k, rho):                      # Cndo2::GetAuxiliaryA
    s = 0.0
    for mu in range(1, k + 2):
        s += 1.0 / (rho ** mu * math.factorial(k - mu + 1))
    return math.exp(-rho) * math.factorial(k) * s


def aux_b(k, rho):                      # Cndo2::GetAuxiliaryB
    if rho == 0.0:
        return 2.0 / (1.0 + k) if k % 2 == 0 else 0.0
    t1 = t2 = 0.0
    for mu in range(1, k + 2):
        f = math.factorial(k) // math.factorial(k - mu + 1)
        t1 += f / rho ** mu
        t2 += f * (1.0 if (k - mu) % 2 == 0 else -1.0) / rho ** mu
    return -math.exp(-rho) * t1 - math.exp(rho) * t2


def aux_d(la, lb, m):                   # Cndo2::GetAuxiliaryD
    pre = (math.factorial(m + 1) / 8.0) ** 2
    ta = (2.0 * la + 1.0) * math.factorial(la - m) / (2.0 * math.factorial(la + m))
    tb = (2.0 * lb + 1.0) * math.factorial(lb - m) / (2.0 * math.factorial(lb + m))
    return pre * math.sqrt(ta) * math.sqrt(tb)


def overlap(Y, na, la, za, nb, lb, zb, m, R):
    alpha, beta = za * R, zb * R
    red = 0.0
    for i in range(9):
        for j in range(9):
            y = Y[na][nb][la][lb][m][i][j]
            if y != 0.0:
                red += y * aux_a(i, 0.5 * (alpha + beta)) * aux_b(j, 0.5 * (alpha - beta))
    red *= aux_d(la, lb, m)
    pre = (2.0 * za) ** (na + 0.5) * (2.0 * zb) ** (nb + 0.5)
    pre /= math.sqrt(math.factorial(2 * na) * math.factorial(2 * nb))
    pre *= (R / 2.0) ** (na + nb + 1.0)
    return pre * red


def overlap_exact(Y, na, la, za, nb, lb, zb, m, R):
    """The same formula in 60-digit arithmetic (mpmath): the value MolDS's
    formula defines, free of the cancellation its double-precision B_k has
    for small |q| (k up to 8 for M-shell pairs)."""
    import mpmath as mp
    mp.mp.dps = 60
    za, zb, R = mp.mpf(za), mp.mpf(zb), mp.mpf(R)
    p, q = (za + zb) * R / 2, (za - zb) * R / 2

    def a_(k, rho):
        return mp.exp(-rho) * mp.factorial(k) * mp.fsum(1 / (rho ** mu * mp.factorial(k - mu + 1))
                                                       for mu in range(1, k + 2))

    def b_(k, rho):
        if rho == 0:
            return mp.mpf(2) / (1 + k) if k % 2 == 0 else mp.mpf(0)
        t1 = mp.fsum(mp.factorial(k) / mp.factorial(k - mu + 1) / rho ** mu for mu in range(1, k + 2))
        t2 = mp.fsum(mp.factorial(k) / mp.factorial(k - mu + 1) * (1 if (k - mu) % 2 == 0 else -1) / rho ** mu
                     for mu in range(1, k + 2))
        return -mp.exp(-rho) * t1 - mp.exp(rho) * t2

    red = mp.fsum(int(Y[na][nb][la][lb][m][i][j]) * a_(i, p) * b_(j, q)
                  for i in range(9) for j in range(9) if Y[na][nb][la][lb][m][i][j] != 0.0)
    red *= aux_d(la, lb, m)
    pre = (2 * za) ** (na + mp.mpf(1) / 2) * (2 * zb) ** (nb + mp.mpf(1) / 2)
    pre /= mp.sqrt(mp.factorial(2 * na) * mp.factorial(2 * nb))
    pre *= (R / 2) ** (na + nb + 1)
    return float(pre * red)


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_overlaps.py <MolDS src directory>")
    Y = read_y(sys.argv[1])
    params = json.load(open(os.path.join(HERE, "reference_parameters.json")))["elements"]
    shells = {"k": 1, "l": 2, "m": 3}
    cases = []
    # orbital pairs of the diatomic frame: (l_A, l_B, m) = ss, s-p_sigma, p_sigma-s, p_sigma-p_sigma, p_pi-p_pi
    kinds = [(0, 0, 0), (0, 1, 0), (1, 0, 0), (1, 1, 0), (1, 1, 1)]
    pairs = [("H", "H"), ("C", "H"), ("C", "C"), ("O", "H"), ("N", "O"), ("O", "O"), ("S", "C"), ("Cl", "H"),
             ("S", "Cl")]
    for theory in ("mndo", "am1", "pm3"):
        for a, b in pairs:
            ea, eb = params[a], params[b]
            na, nb = shells[ea["valenceShell"]], shells[eb["valenceShell"]]
            for la, lb, m in kinds:
                if (la and ea["valenceOrbitals"] == 1) or (lb and eb["valenceOrbitals"] == 1):
                    continue
                za = ea[theory + ("OrbitalExponentP" if la else "OrbitalExponentS")]
                zb = eb[theory + ("OrbitalExponentP" if lb else "OrbitalExponentS")]
                for R in (0.9, 1.5, 2.1, 2.9, 4.0, 6.5, 10.0):
                    cases.append({"theory": theory, "A": a, "B": b, "na": na, "la": la, "zeta_a": za, "nb": nb,
                                  "lb": lb, "zeta_b": zb, "m": m, "R": R,
                                  "S": overlap_exact(Y, na, la, za, nb, lb, zb, m, R),
                                  "S_double": overlap(Y, na, la, za, nb, lb, zb, m, R)})
    out = {"source": "MolDS src/cndo/Cndo2.cpp:5801-5869, 6185-6204, 6385-6477 with the Y table of "
                     "src/cndo/ReducedOverlapAOsParameters.h", "cases": cases}
    with open(os.path.join(HERE, "reference_overlaps.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", len(cases), "overlaps")


if __name__ == "__main__":
    main()
