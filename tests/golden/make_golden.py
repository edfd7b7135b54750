"""Regenerates tests/golden/reference_fixtures.json (SCF fixtures) and
tests/golden/reference_md_fixtures.json (ground-state MD force runs) from the
MolDS test suite.

Reads the reference's own golden input/output pairs (test/<case>.in and
test/<case>.dat of the MolDS tree, registered in test/Test_Of_MolDS.rb) and
keeps, per case, the input text and the printed values that pin the NDDO SCF
path: the per-iteration RMS density and DIIS error, MO energies, electronic
energy (incl. core repulsion), core repulsion, Mulliken charges, the total,
electronic and core dipole moments (x, y, z in a.u.), the empirical van der
Waals energy where the run has one and, for MNDO, the heat of formation.  MolDS prints these with %e (7 significant digits,
src/cndo/Cndo2.cpp:1087-1089, 1193-1198), so they pin results to ~5e-7 relative.

Usage:  python tests/golden/make_golden.py <path to the MolDS test directory>
"""
import json
import os
import re
import sys

CASES = [f"{m}_{t}" for m in ("ch4", "c2h6", "ch3f", "ch3cl") for t in ("mndo", "am1", "pm3")]
# the dispersion-corrected theories and the vdW option
CASES += ["c2h6_am1d", "c2h6_pm3d", "c2h6_pm3_vdw", "c2h6_pm3pddg"]
# SCF blocks printed before a frequency run: the first SCF of each pins PM3 for
# O (with the H-O core-core rule) and for C=C.
EXTRA = ["h2o_pm3_freq_num_proj_s1", "c2h4_pm3_freq_num_proj", "c2h6-nh3-cluster_pm3d_freq",
         "c2h6-h2o-cluster_pm3pddg_freq"]
# water dimers: the first SCF of an Ehrenfest run (AM1-D, which keeps AM1's O
# zeta, D / rho, G / H and Gaussians) and of a geometry optimisation (PM3-D)
EXTRA += ["h2o-dimer_am1d_ehrenfest", "h2o-dimer_pm3d_opt_bfgs_space_fixed"]


def scf_text(text):
    """The first SCF section as printed: from its start banner to its done
    banner (inclusive)."""
    m = re.search(r"\*{10}  START: [^\n]*-SCF  \*{10}\n", text)
    b = text.find("**********  DONE: ", m.start())
    b = text.find("\n", b)
    return text[m.start():b + 1]


def parse_dat(text, natoms):
    """Values of the first SCF block (frequency runs print several)."""
    start = text.find("-SCF  **********")
    body = text[start:]
    end = body.find("**********  DONE:")
    body = body[:end] if end >= 0 else body
    trace = []
    for a, b, c, rest in re.findall(r"SCF iter (\d+)\t(\S+)\t(\S+)([^\n]*)", body):
        trace.append({"iter": int(a), "rms": float(b), "diis_error": float(c),
                      "diis_on": rest.strip().startswith("on")})
    mo = [float(x) for x in re.findall(r"Energy of MO:\t\d+\t\S+\t(\S+)", body)]
    e = float(re.search(r"Electronic energy\(SCF\):\t(\S+)", body).group(1))
    ec = float(re.search(r"Core repulsion energy:\t(\S+)", body).group(1))
    q = [float(x) for x in re.findall(r"Mulliken charge\(SCF\):\t0\t\d+\t\S+\t\S+\t(\S+)", body)][:natoms]
    hof = re.search(r"Heats of formation:\t(\S+)", body)
    dip = []
    for label in (r"Total Dipole moment\(SCF\):", r"Electronic Dipole moment\(SCF\):",
                  r"Core Dipole moment:"):
        m = re.search(label + r"\t+(\S+)\t(\S+)\t(\S+)", body)
        dip.append([float(m.group(i)) for i in (1, 2, 3)])
    out = {"trace": trace, "mo_energies": mo, "energy": e, "core_repulsion": ec,
           "mulliken": q, "dipole": dip, "scf_text": scf_text(text)}
    vdw = re.search(r"Empirical van der Waals correction:\t(\S+)", body)
    if vdw:
        out["vdw_energy"] = float(vdw.group(1))
    if hof:
        out["heat_of_formation"] = float(hof.group(1))
    return out


# ground-state MD runs from rest: the momenta printed after each step follow
# from the analytic forces (MD::UpdateMomenta / UpdateCoordinates,
# src/md/MD.cpp:97-149)
MD_CASES = ["c2h6_mndo_force", "c2h6_am1_force", "c2h6_pm3_force", "c2h6_pm3pddg_force", "c2h6_pm3_vdw_force"]


def parse_md(inp, dat, natoms):
    md = re.search(r"(?is)^\s*md\s*$(.*?)^\s*md_end", inp, re.M).group(1)
    dt = float(re.search(r"(?i)\bdt\s+(\S+)", md).group(1))
    steps = int(re.search(r"(?i)total_steps\s+(\d+)", md).group(1))
    momenta = []
    for s in range(1, steps + 1):
        a = dat.find(f"START: MD step {s}\n")
        b = dat.find(f"DONE: MD step {s}\n", a)
        block = dat[a:b]
        # Molecule::OutputMomenta (src/base/Molecule.cpp:555-575) prints
        # p / momentumUnit2AU under the "[a.u.]" heading and the stored
        # momentum, in atomic units, under "[u]": keep the second triple
        rows = re.findall(r"Atom momenta:\t\d+\t\S+\t\S+\t\S+\t\S+\t\t(\S+)\t(\S+)\t(\S+)", block)
        momenta.append([[float(x) for x in r] for r in rows[:natoms]])
    return {"dt_fs": dt, "steps": steps, "momenta": momenta}


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <MolDS test directory>")
    src = sys.argv[1]
    fixtures = []
    for name in CASES + EXTRA:
        inp = open(os.path.join(src, name + ".in")).read()
        dat = open(os.path.join(src, name + ".dat")).read()
        natoms = int(re.search(r"Total number of atoms: (\d+)", dat).group(1))
        nao = int(re.search(r"Total number of valence AOs: (\d+)", dat).group(1))
        rec = {"name": name, "input": inp, "natoms": natoms, "n_ao": nao}
        rec.update(parse_dat(dat, natoms))
        fixtures.append(rec)
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "reference_fixtures.json"), "w") as f:
        json.dump({"source": "MolDS test/*.in, test/*.dat", "cases": fixtures}, f, indent=1)
    print(f"wrote {len(fixtures)} cases")
    md = []
    for name in MD_CASES:
        inp = open(os.path.join(src, name + ".in")).read()
        dat = open(os.path.join(src, name + ".dat")).read()
        natoms = int(re.search(r"Total number of atoms: (\d+)", dat).group(1))
        rec = {"name": name, "input": inp, "natoms": natoms}
        rec.update(parse_md(inp, dat, natoms))
        md.append(rec)
    with open(os.path.join(here, "reference_md_fixtures.json"), "w") as f:
        json.dump({"source": "MolDS test/*_force.in, test/*_force.dat (momenta after each MD step)", "cases": md},
                  f, indent=1)
    print(f"wrote {len(md)} MD cases")


if __name__ == "__main__":
    main()
