"""MolDS's SCF output text (row f1: Cndo2::OutputSCFResults and the iteration
log, src/cndo/Cndo2.cpp:585-729,1063-1221,1299-1303; Mndo.cpp:412-420)
against the reference's own output files.

The product's formatter (nddo_format_scf_text, no GPU needed) is fed the
oracle's results for each of the reference fixtures and must reproduce the
SCF section of the fixture's .dat file line by line
(tests/golden/reference_fixtures.json, "scf_text"; the comparison rule is in
tests/scf_text_compare.py).  The GPU path's own text is checked in
tests/test_gpu_parity.py.
"""
import json
import os
import re

import numpy as np
import pytest

import molds_gb300 as M
from oracle import oracle as O
from scf_text_compare import compare_scf_text

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = json.load(open(os.path.join(HERE, "golden", "reference_fixtures.json")))["cases"]


@pytest.fixture(scope="module", autouse=True)
def built():
    from molds_gb300 import build
    build.build()


@pytest.mark.parametrize("case", FIX, ids=[c["name"] for c in FIX])
def test_scf_text_matches_reference_output(case):
    mol, p = O.parse_input(case["input"])
    ref = O.scf(mol, p)
    # the fixtures' SCF blocks may sit beside blocks outside this path (CIS,
    # frequencies), which the product's parser rejects: read the option alone
    scf_block = re.search(r"(?is)^\s*scf\s*$(.*?)^\s*scf_end", case["input"], re.M).group(1)
    sums = [(int(a), int(b)) for a, b in re.findall(r"(?i)sum_charges\s+(\d+)\s+(\d+)", scf_block)]
    nocc = int(round(O.atom_info(mol)[:, 0].sum())) // 2
    vdw = bool(p.vdw) or mol.theory in (3, 4)
    text = M.format_scf_text(mol.theory, mol.Z, ref.eps, nocc, ref.trace, ref.energy, ref.core_repulsion,
                             ref.charges, dipole=ref.dipole, vdw=vdw, vdw_energy=ref.vdw_energy,
                             heat_of_formation=ref.heat_of_formation or 0.0, sum_charges=sums)
    bad = compare_scf_text(text, case["scf_text"], skip_iterations=p.rms_density < 1e-12)
    assert not bad, "\n".join(bad[:10])


def test_not_converged_text_ends_after_the_iteration_log():
    """A non-converged SCF prints only the banner, the title and the iteration
    lines (MolDS throws there, Cndo2.cpp:700-704)."""
    trace = [(0, 0.5, 0.0, False, False), (1, 0.25, 0.0, False, True)]
    text = M.format_scf_text("pm3", [1, 1], [-0.5, 0.3], 1, trace, 0.0, 0.0, [0.0, 0.0], converged=False)
    lines = text.rstrip("\n").split("\n")
    assert lines[0] == "**********  START: PM3-SCF  **********"
    assert lines[-1] == "\tSCF iter 1\t2.500000e-01\t0.000000e+00\t\t\ton"
    assert "DONE" not in text
