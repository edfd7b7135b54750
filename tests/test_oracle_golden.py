"""The oracle against the golden values of MolDS's own test suite.

tests/golden/reference_fixtures.json holds the reference's printed results
(7 significant digits: energies, MO energies, Mulliken charges, dipole
moments, iteration trace) for its 12 SCF-only NDDO cases
(test/{ch4,c2h6,ch3f,ch3cl}_{mndo,am1,pm3}) plus the first SCF of two PM3
frequency cases (water: O and the H-O core-core rule; ethylene).  Passing here
is what pins the oracle before it is used to check the CUDA path.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = json.load(open(os.path.join(HERE, "golden", "reference_fixtures.json")))["cases"]
PRINT_REL = 1e-6     # %e prints 7 significant digits: half-ulp is 5e-7 relative


def close(a, b, rel=PRINT_REL, abs_=5e-7):
    return abs(a - b) <= max(rel * abs(b), abs_)


@pytest.fixture(scope="module", params=FIX, ids=[c["name"] for c in FIX])
def case(request):
    c = request.param
    mol, params = O.parse_input(c["input"])
    return c, mol, O.scf(mol, params)


def test_energy_and_core_repulsion(case):
    c, mol, r = case
    assert close(r.energy, c["energy"]), (r.energy, c["energy"])
    assert close(r.core_repulsion, c["core_repulsion"]), (r.core_repulsion, c["core_repulsion"])


def test_mo_energies(case):
    c, mol, r = case
    ref = np.array(c["mo_energies"])
    assert r.eps.shape == ref.shape
    assert np.all(np.abs(r.eps - ref) <= np.maximum(PRINT_REL * np.abs(ref), 5e-7))


def test_mulliken_charges(case):
    c, mol, r = case
    ref = np.array(c["mulliken"])
    # charges are printed to 7 digits; the worst case is a value near 0.1-1
    assert np.max(np.abs(r.charges - ref)) < 1e-7 + 1e-6 * np.max(np.abs(ref))


def test_iteration_trace(case):
    """Same iteration count and the same printed RMS-density / DIIS-error trace."""
    c, mol, r = case
    ref = c["trace"]
    ours = r.trace
    if min(x["rms"] for x in ref) > 1e-13:          # fixtures converged well above round-off
        assert len(ours) == len(ref)
    for mine, theirs in zip(ours, ref):
        if theirs["rms"] < 1e-12:                    # below this the trace is round-off noise
            break
        it, rms, derr, on, _ = mine
        assert it == theirs["iter"]
        assert close(rms, theirs["rms"], rel=2e-6), (it, rms, theirs["rms"])
        if theirs["diis_error"] > 1e-10:
            assert close(derr, theirs["diis_error"], rel=2e-6), (it, derr, theirs["diis_error"])
        assert on == theirs["diis_on"]


def test_heat_of_formation(case):
    c, mol, r = case
    if "heat_of_formation" in c:
        assert close(r.heat_of_formation, c["heat_of_formation"])
    else:
        assert r.heat_of_formation is None


def test_dipole_moments(case):
    """Total, electronic and core dipole (Cndo2.cpp:1126-1185 prints x, y, z in
    a.u.): every component to the printed 7 digits; components that are
    round-off noise in the reference (|mu_k| ~ 1e-11 or below) to 1e-9 a.u."""
    c, mol, r = case
    ref = np.array(c["dipole"])
    assert r.dipole.shape == (3, 3)
    for mine, theirs in zip(r.dipole.ravel(), ref.ravel()):
        assert close(mine, theirs, rel=PRINT_REL, abs_=1e-9), (mine, theirs)


def test_vdw_energy(case):
    """Empirical dispersion energy (Cndo2.cpp:464-513, printed at :1118-1122)
    of the AM1-D / PM3-D cases and of PM3 with vdW yes; 0 elsewhere."""
    c, mol, r = case
    if "vdw_energy" in c:
        assert close(r.vdw_energy, c["vdw_energy"], abs_=1e-12), (r.vdw_energy, c["vdw_energy"])
    else:
        assert r.vdw_energy == 0.0


def test_aos_match(case):
    c, mol, r = case
    assert O.num_aos(mol) == c["n_ao"]


def test_warm_start_from_previous_density():
    """DoSCF(false) after the molecule moved (src/md/MD.cpp:108): the oracle
    started from the previous density converges to the cold-start energy in
    no more iterations."""
    c = [c for c in FIX if c["name"] == "ch3f_pm3"][0]
    mol, params = O.parse_input(c["input"])
    r0 = O.scf(mol, params)
    moved = O.make_molecule(mol.theory, mol.Z, mol.xyz + np.random.default_rng(3).normal(scale=0.01, size=mol.xyz.shape))
    warm = O.scf(moved, params, requires_guess=False, P0=r0.P)
    cold = O.scf(moved, params)
    assert abs(warm.energy - cold.energy) < 1e-9
    assert warm.iterations <= cold.iterations

