"""ORACLE -- test infrastructure, not product code.

Per-atom NDDO parameters of the oracle, built from the reference's own
definitions: tests/golden/reference_parameters.json holds, for H, C, N, O, F,
S and Cl, every numeric field MolDS's SetAtomicParameters assigns (already in
atomic units, evaluated from src/base/atoms/<El>atom.cpp by
tests/golden/make_parameters.py), MolDS's unit constants
(src/base/Parameters.cpp:45-57) and the STO-6G tables
(src/base/GTOExpansionSTO.cpp:314-347).  Nothing here reads the product's
parameter tables.

The theory -> field mapping restates MolDS's Atom getters:
  U_ss / U_pp ........ GetCoreIntegral, src/base/atoms/Atom.cpp:1072-1109
                       (GetMndo/Am1/Am1D/Pm3/Pm3D/Pm3PddgCoreIntegral)
  beta ............... GetBondingParameter, Atom.cpp:263-341
  zeta ............... GetOrbitalExponent, Atom.cpp:366-480 (AM1-D uses AM1's,
                       PM3-D PM3's)
  alpha .............. GetNddoAlpha, Atom.cpp:709-727
  D, rho ............. GetNddoDerivedParameterD / Rho, Atom.cpp:730-826
                       (AM1-D: AM1's, PM3-D: PM3's)
  K, L, M ............ GetNddoParameterK / L / M, Atom.cpp:830-900 (none for MNDO)
  Gss .. Hsp ......... GetNddoGss .. GetNddoHsp, Atom.cpp:940-1049 (PDDG: PM3's)
  Hpp ................ GetNddoHpp = (Gpp - Gpp2) / 2, Atom.cpp:1051-1070
  core mass .......... Atom::GetCoreMass, src/base/atoms/Atom.h:34
  PDDG Pa, Da ........ GetPm3PddgParameterPa / Da
"""
from __future__ import annotations

import json
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "..", "tests", "golden", "reference_parameters.json")

# theory slots of the oracle (the same numbering the product's C ABI uses)
MNDO, AM1, PM3, AM1D, PM3D, PM3PDDG = 0, 1, 2, 3, 4, 5
Z_TO_SYMBOL = {1: "H", 6: "C", 7: "N", 8: "O", 9: "F", 16: "S", 17: "Cl"}

# field order of one record (must match struct oracle_atom in nddo_oracle.c)
RECORD = ["core_charge", "u_s", "u_p", "zeta_s", "zeta_p", "beta_s", "beta_p", "alpha",
          "gss", "gsp", "gpp", "gp2", "hsp", "hpp", "d0", "d1", "d2", "rho0", "rho1", "rho2",
          "gk0", "gk1", "gk2", "gk3", "gl0", "gl1", "gl2", "gl3", "gm0", "gm1", "gm2", "gm3",
          "e_atom", "dhf_atom", "core_mass", "vdw_c6", "vdw_r0", "pddg_pa0", "pddg_pa1", "pddg_da0", "pddg_da1",
          "n_ao", "principal_n", "atomic_number"]

_data = None


def data():
    global _data
    if _data is None:
        with open(FIXTURE) as f:
            _data = json.load(f)
    return _data


def constants():
    return data()["constants"]


def _prefix(theory, kind):
    """MolDS field prefix of a parameter kind for a theory."""
    own = {MNDO: "mndo", AM1: "am1", AM1D: "am1D", PM3: "pm3", PM3D: "pm3D", PM3PDDG: "pm3Pddg"}
    base = {MNDO: "mndo", AM1: "am1", AM1D: "am1", PM3: "pm3", PM3D: "pm3", PM3PDDG: "pm3Pddg"}
    gset = {MNDO: "mndo", AM1: "am1", AM1D: "am1", PM3: "pm3", PM3D: "pm3", PM3PDDG: "pm3"}
    return {"own": own, "base": base, "g": gset}[kind][theory]


def atom_record(theory: int, Z: int) -> dict | None:
    """The oracle's parameters of element Z under a theory slot (atomic units),
    or None when MolDS has no such parameter set for it."""
    sym = Z_TO_SYMBOL.get(int(Z))
    if sym is None:
        return None
    e = data()["elements"][sym]
    own, base, g = _prefix(theory, "own"), _prefix(theory, "base"), _prefix(theory, "g")
    # a set the element file does not define completely is absent: e.g. the
    # AM1-D alpha of F and Cl is never assigned (Fatom.cpp:153 and
    # Clatom.cpp:171 assign am1DAlpha to itself)
    if any(own + k not in e for k in ("CoreintegralS", "CoreintegralP", "BondingParameterS", "BondingParameterP",
                                      "Alpha")):
        return None
    r = {}
    r["core_charge"] = e["coreCharge"]
    r["u_s"], r["u_p"] = e[own + "CoreintegralS"], e[own + "CoreintegralP"]
    r["beta_s"], r["beta_p"] = e[own + "BondingParameterS"], e[own + "BondingParameterP"]
    r["alpha"] = e[own + "Alpha"]
    r["zeta_s"], r["zeta_p"] = e[base + "OrbitalExponentS"], e[base + "OrbitalExponentP"]
    d = e[base + "DerivedParameterD"]
    rho = e[base + "DerivedParameterRho"]
    r["d0"], r["d1"], r["d2"] = d[0], d[1], d[2]
    r["rho0"], r["rho1"], r["rho2"] = rho[0], rho[1], rho[2]
    for key, name in (("gk", "ParameterK"), ("gl", "ParameterL"), ("gm", "ParameterM")):
        vals = e.get(base + name, [0.0] * 4) if theory != MNDO else [0.0] * 4
        vals = list(vals) + [0.0] * (4 - len(vals))
        for i in range(4):
            r[f"{key}{i}"] = vals[i]
    r["gss"], r["gsp"], r["gpp"] = e[g + "Gss"], e[g + "Gsp"], e[g + "Gpp"]
    r["gp2"], r["hsp"] = e[g + "Gpp2"], e[g + "Hsp"]
    r["hpp"] = 0.5 * (r["gpp"] - r["gp2"])
    r["e_atom"] = e.get("mndoElecEnergyAtom", 0.0) if theory == MNDO else 0.0
    r["dhf_atom"] = e.get("mndoHeatsFormAtom", 0.0) if theory == MNDO else 0.0
    r["core_mass"] = e["atomicMass"] - float(e["numberValenceElectrons"])
    r["vdw_c6"] = e.get("vdWCoefficient", 0.0)
    r["vdw_r0"] = e.get("vdWRadii", 0.0)
    pa = e.get("pm3PddgParameterPa", [0.0, 0.0]) if theory == PM3PDDG else [0.0, 0.0]
    da = e.get("pm3PddgParameterDa", [0.0, 0.0]) if theory == PM3PDDG else [0.0, 0.0]
    r["pddg_pa0"], r["pddg_pa1"], r["pddg_da0"], r["pddg_da1"] = pa[0], pa[1], da[0], da[1]
    r["n_ao"] = e["valenceOrbitals"]
    r["principal_n"] = {"k": 1, "l": 2, "m": 3}[e["valenceShell"]]
    r["atomic_number"] = int(Z)
    return r


def record_array(theory: int, Z: int):
    r = atom_record(theory, Z)
    if r is None:
        return None
    return [float(r[k]) for k in RECORD]


def sto6g_tables():
    """(exponents, coefficients) as [shell K, L, M][s, p][6] nested lists."""
    s = data()["sto6g"]
    ex, co = [], []
    for shell in ("k", "l", "m"):
        ex.append([s["exponents"].get(shell + "s", [0.0] * 6), s["exponents"].get(shell + "p", [0.0] * 6)])
        co.append([s["coefficients"].get(shell + "s", [0.0] * 6), s["coefficients"].get(shell + "p", [0.0] * 6)])
    return ex, co


def sto_normalisation(zeta: float, n: int) -> float:
    """(2 zeta)^(n + 1/2) / sqrt((2n)!): the radial normalisation of a Slater orbital."""
    return (2.0 * zeta) ** (n + 0.5) / math.sqrt(math.factorial(2 * n))
