"""Analytic forces (row f2: Mndo::CalcForce, src/mndo/Mndo.cpp:2711-2986,
ground state) against the oracle and against the reference's own output.

1. Finite differences of the oracle: the energy with the converged density P
   held fixed, E(R; P) = 1/2 tr P (H + F(P)) + E_core (+ E_vdW), built from
   the oracle's own integrals at displaced geometries (central differences,
   h = 1e-4 bohr: truncation ~1e-9), must equal -F from the GPU.  Cases cover
   MNDO, AM1, PM3, PDDG/PM3, AM1-D and the vdW option, Cl, and bonds along a
   coordinate axis (the local frame's degenerate case).
2. The reference's ground-state MD runs from rest (test/c2h6_*_force.dat):
   MolDS's velocity Verlet (MD::UpdateMomenta / UpdateCoordinates,
   src/md/MD.cpp:97-149: p += dt/2 F, x += dt p / m_core, SCF from the previous
   density, p += dt/2 F) driven by these forces must reproduce the momenta the
   reference printed after each of its five steps (7 significant digits).
"""
import json
import os

import numpy as np
import pytest

import molds_gb300 as M
from molds_gb300 import workloads as W
from oracle import oracle as O
from oracle import parameters as OP

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = {c["name"]: c for c in json.load(open(os.path.join(HERE, "golden", "reference_fixtures.json")))["cases"]}
MD = json.load(open(os.path.join(HERE, "golden", "reference_md_fixtures.json")))["cases"]
FS2AU = 1.0 / 2.418884326505e-2   # src/base/Parameters.cpp:52


@pytest.fixture(scope="module")
def ctx():
    from molds_gb300 import build
    build.build()
    return M.Context(0)


def _params(p):
    return M.SCFParams(max_iter=p.max_iter, rms_density=p.rms_density, damping_thresh=p.damping_thresh,
                       damping_weight=p.damping_weight, diis_num_error_vect=p.diis_num_error_vect,
                       diis_start_error=p.diis_start_error, diis_end_error=p.diis_end_error, vdw=p.vdw,
                       vdw_s6=p.vdw_s6, vdw_d=p.vdw_d)


def frozen_energy(theory, Z, xyz, P, p):
    om = O.make_molecule(theory, Z, xyz)
    S, eri, ecore = O.integrals(om)
    F = O.fock(om, S, eri, P)
    H = O.fock(om, S, eri, np.zeros_like(P))
    e = 0.5 * float(np.sum(P * (F + H))) + ecore
    dtheory = theory in (3, 4)
    if p.vdw or dtheory:
        e += O.vdw_energy(om, 1.40 if dtheory else p.vdw_s6, 23.0 if dtheory else p.vdw_d)
    return e


def fd_forces(theory, Z, xyz, P, p, h=1e-4):
    xyz = np.array(xyz, dtype=np.float64)
    f = np.zeros_like(xyz)
    for a in range(len(Z)):
        for k in range(3):
            xp, xm = xyz.copy(), xyz.copy()
            xp[a, k] += h
            xm[a, k] -= h
            f[a, k] = -(frozen_energy(theory, Z, xp, P, p) - frozen_energy(theory, Z, xm, P, p)) / (2 * h)
    return f


def _axis_molecules():
    ang = M.ANG2AU
    # N2 along z, and methane with one C-H bond along each coordinate axis
    n2 = M.Molecule(np.array([7, 7], dtype=np.int32), np.array([[0, 0, 0], [0, 0, 1.10]]) * ang)
    ch = 1.09 / np.sqrt(3.0)
    ch4 = M.Molecule(np.array([6, 1, 1, 1, 1], dtype=np.int32),
                     np.array([[0, 0, 0], [1.09, 0, 0], [0, 1.09, 0], [0, 0, 1.09], [-ch, -ch, -ch]]) * ang)
    return [("mndo", n2), ("am1", ch4)]


CASES = ["c2h6_mndo", "c2h6_am1", "c2h6_pm3", "c2h6_pm3pddg", "c2h6_pm3_vdw", "c2h6_am1d", "ch3cl_pm3",
         "h2o-dimer_am1d_ehrenfest"]


@pytest.mark.parametrize("name", CASES + ["axis_n2", "axis_ch4", "water8_am1"])
def test_forces_match_oracle_finite_differences(ctx, name):
    if name in FIX:
        mol, p = O.parse_input(FIX[name]["input"])
        theory, Z, xyz = mol.theory, np.array(mol.Z), np.array(mol.xyz).reshape(-1, 3)
        params = _params(p)
    else:
        if name == "water8_am1":
            theory, m = "am1", W.water_cluster(shape=(2, 2, 2), seed=2)
        else:
            theory, m = _axis_molecules()[0 if name == "axis_n2" else 1]
        Z, xyz = np.array(m.Z), np.array(m.xyz).reshape(-1, 3)
        params = M.SCFParams(max_iter=500, rms_density=1e-10, damping_thresh=1.0, damping_weight=0.0,
                             diis_num_error_vect=5, diis_start_error=0.1, diis_end_error=0.0)
        theory = M.THEORIES[theory]
        p = O.SCFParams(max_iter=500, rms_density=1e-10, damping_thresh=1.0, damping_weight=0.0,
                        diis_num_error_vect=5, diis_start_error=0.1, diis_end_error=0.0)
    es = M.ElectronicStructure(theory, params, context=ctx)
    es.SetMolecule(M.Molecule(np.asarray(Z, dtype=np.int32), xyz))
    es.DoSCF(True)
    F = es.GetForce()
    P = es.GetOrbitalElectronPopulation()
    ref = fd_forces(theory, Z, xyz, P, p)
    assert np.max(np.abs(F - ref)) < 2e-7, (np.max(np.abs(F - ref)), np.max(np.abs(ref)))
    # Newton's third law: the forces of an isolated molecule sum to zero
    assert np.max(np.abs(F.sum(axis=0))) < 1e-10


@pytest.mark.parametrize("case", MD, ids=[c["name"] for c in MD])
def test_md_momenta_match_reference(ctx, case):
    mol, p = O.parse_input(case["input"])
    Z = np.array(mol.Z)
    x = np.array(mol.xyz, dtype=np.float64).reshape(-1, 3)
    mass = np.array([OP.atom_record(mol.theory, int(z))["core_mass"] for z in Z])
    dt = case["dt_fs"] * FS2AU
    es = M.ElectronicStructure(mol.theory, _params(p), context=ctx)
    es.SetMolecule(M.Molecule(Z.astype(np.int32), x))
    es.DoSCF(True)
    F = es.GetForce()
    mom = np.zeros_like(x)
    for step, ref in enumerate(case["momenta"]):
        mom += 0.5 * dt * F
        x = x + dt * mom / mass[:, None]
        es.SetCoordinates(x)
        es.DoSCF(False)
        F = es.GetForce()
        mom += 0.5 * dt * F
        ref = np.array(ref)
        err = np.abs(mom - ref)
        assert np.all(err <= 2e-6 * np.abs(ref) + 1e-11), (step + 1, float(np.max(err / (np.abs(ref) + 1e-30))))


def test_resident_batch_forces_match_plain_path(ctx):
    """Forces of each molecule of a resident batch (nddo_batch_get_forces)
    equal those of the plain path for the same molecule."""
    mols = [W.water_cluster(shape=(2, 2, 1), seed=s) for s in (2, 3)] + [W.octane()]
    theories = ["am1", "am1", "am1"]
    params = M.SCFParams(max_iter=500, rms_density=1e-10, damping_thresh=1.0, damping_weight=0.0,
                         diis_num_error_vect=5, diis_start_error=0.1, diis_end_error=0.0)
    rb = M.ResidentBatch("am1", mols, context=ctx)
    rb.run(params)
    for m, mol in enumerate(mols):
        es = M.ElectronicStructure(theories[m], params, context=ctx)
        es.SetMolecule(mol)
        es.DoSCF(True)
        assert np.max(np.abs(rb.forces(m) - es.GetForce())) < 1e-8

