"""Environmental point charges (MolDS EPC, row f4) on the GPU against the
oracle, through the public API.

Each charge q adds -q (mu nu|s s) to the one-centre blocks of every
non-guess Fock matrix and of H, and sum Z_A q / R to the energy
(src/mndo/Mndo.cpp:329-331, 474-484, 546-556, 6602-6613;
src/cndo/Cndo2.cpp:418-426, 1324-1416).  Cases: the reference fixtures'
molecules in all six theories and the vdW option, each with seeded point
charges 2-4 Angstrom outside the molecule (a TIP3P-like -0.834 / +0.417
pattern), one with more charges than atoms; the molecule's pool growing and
shrinking with the charge count; charges that stay in place when the atoms
move; and the forces, which, as Mndo::CalcForce, carry no explicit atom-EPC
term.
"""
import json
import os

import numpy as np
import pytest

import molds_gb300 as M
from oracle import oracle as O
from scf_text_compare import compare_scf_text

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = {c["name"]: c for c in json.load(open(os.path.join(HERE, "golden", "reference_fixtures.json")))["cases"]}


@pytest.fixture(scope="module")
def ctx():
    from molds_gb300 import build
    build.build()
    return M.Context(0)


def point_charges(xyz, n, seed):
    """n charges 2-4 Angstrom outside the molecule's atoms, in triples
    -0.834, +0.417, +0.417 (the last triple cut short when n % 3 != 0)."""
    rng = np.random.default_rng(seed)
    c = xyz.mean(axis=0)
    rad = np.max(np.linalg.norm(xyz - c, axis=1))
    out = []
    while len(out) < n:
        d = rng.normal(size=3)
        p = c + d / np.linalg.norm(d) * (rad + rng.uniform(2.0, 4.0) * M.ANG2AU)
        if np.min(np.linalg.norm(xyz - p, axis=1)) < 2.0 * M.ANG2AU:
            continue
        out.append(list(p) + [-0.834 if len(out) % 3 == 0 else 0.417])
    return np.array(out)


def _params(p):
    return M.SCFParams(max_iter=p.max_iter, rms_density=p.rms_density, damping_thresh=p.damping_thresh,
                       damping_weight=p.damping_weight, diis_num_error_vect=p.diis_num_error_vect,
                       diis_start_error=p.diis_start_error, diis_end_error=p.diis_end_error, vdw=p.vdw,
                       vdw_s6=p.vdw_s6, vdw_d=p.vdw_d)


CASES = [("ch4_mndo", 3), ("ch3f_am1", 6), ("ch3cl_pm3", 4), ("c2h6_am1d", 9), ("c2h6_pm3d", 3),
         ("c2h6_pm3_vdw", 6), ("c2h6_pm3pddg", 5), ("c2h6_mndo", 30)]


def _run(ctx, name, n_epc, seed=11):
    mol, p = O.parse_input(FIX[name]["input"])
    pc = point_charges(mol.xyz, n_epc, seed)
    om = O.make_molecule(mol.theory, mol.Z, mol.xyz, pc)
    es = M.ElectronicStructure(mol.theory, _params(p), context=ctx)
    es.SetMolecule(M.Molecule(mol.Z, mol.xyz, pc))
    return om, p, es


@pytest.mark.parametrize("name,n_epc", CASES, ids=[c[0] for c in CASES])
def test_scf_with_point_charges(ctx, name, n_epc):
    om, p, es = _run(ctx, name, n_epc)
    ref = O.scf(om, p)
    # H = F(P = 0) carries the point charges' one-centre terms
    S, eri, _ = O.integrals(om)
    H_ref = O.fock(om, S, eri, np.zeros((S.shape[0], S.shape[0])))
    assert np.max(np.abs(es.GetCoreHamiltonian() - H_ref)) < 1e-11
    es.DoSCF(True)
    assert es.GetIterations() == ref.iterations
    assert abs(es.GetElectronicEnergy(0) - ref.energy) < 1e-8
    assert abs(es.GetCoreEpcCoulombEnergy() - ref.core_epc) < 1e-11
    assert abs(es.GetCoreRepulsionEnergy() - ref.core_repulsion) < 1e-10
    assert abs(es.GetVdWCorrectionEnergy() - ref.vdw_energy) < 1e-12
    assert np.max(np.abs(es.GetMullikenCharges() - ref.charges)) < 1e-6
    assert np.max(np.abs(es.GetEnergiesMO() - ref.eps)) < 1e-7
    assert np.max(np.abs(es.GetDipoleMoments() - ref.dipole)) < 1e-6
    if om.theory == 0:
        assert abs(es.GetHeatsFormation() - ref.heat_of_formation) < 1e-8
    # the charges matter: without them the answer differs
    bare = O.scf(O.make_molecule(om.theory, om.Z, om.xyz), p)
    assert abs(bare.energy - ref.energy) > 1e-4


def test_output_text_with_point_charges(ctx):
    om, p, es = _run(ctx, "c2h6_pm3_vdw", 6)
    ref = O.scf(om, p)
    es.DoSCF(True)
    mine = es.OutputSCFResults()
    nocc = int(round(O.atom_info(om)[:, 0].sum())) // 2
    expect = M.format_scf_text(om.theory, om.Z, ref.eps, nocc, ref.trace, ref.energy, ref.core_repulsion,
                               ref.charges, dipole=ref.dipole, vdw=True, vdw_energy=ref.vdw_energy,
                               core_epc=ref.core_epc)
    bad = compare_scf_text(mine, expect)
    assert not bad, "\n".join(bad[:10])
    assert "Coulomb interaction between cores and EPCs energy:" in mine


def test_pool_regrows_and_reuses(ctx):
    """The molecule's one-slot pool grows for more point charges and keeps
    serving fewer; a molecule without charges after one with charges gives
    the bare result."""
    mol, p = O.parse_input(FIX["c2h6_am1"]["input"])
    es = M.ElectronicStructure(mol.theory, _params(p), context=ctx)
    results = {}
    for n in (2, 12, 0, 5):
        pc = point_charges(mol.xyz, n, 3) if n else None
        es.SetMolecule(M.Molecule(mol.Z, mol.xyz, pc))
        es.DoSCF(True)
        ref = O.scf(O.make_molecule(mol.theory, mol.Z, mol.xyz, pc), p)
        assert abs(es.GetElectronicEnergy(0) - ref.energy) < 1e-8, n
        assert abs(es.GetCoreEpcCoulombEnergy() - ref.core_epc) < 1e-11, n
        results[n] = es.GetElectronicEnergy(0)
    assert len(set(results.values())) == 4


def test_charges_stay_when_atoms_move(ctx):
    """SetCoordinates moves the atoms; the point charges keep their places
    (MolDS's MD moves real atoms only, src/md/MD.cpp:128-149)."""
    om, p, es = _run(ctx, "ch3f_am1", 6)
    es.DoSCF(True)
    xyz2 = om.xyz + np.random.default_rng(5).normal(scale=0.05, size=om.xyz.shape)
    es.SetCoordinates(xyz2)
    es.DoSCF(False)
    ref = O.scf(O.make_molecule(om.theory, om.Z, xyz2, om.epc), p)
    assert abs(es.GetElectronicEnergy(0) - ref.energy) < 1e-8
    assert abs(es.GetCoreEpcCoulombEnergy() - ref.core_epc) < 1e-11
    assert np.max(np.abs(es.GetMullikenCharges() - ref.charges)) < 1e-6


def test_forces_carry_no_explicit_epc_term(ctx):
    """Mndo::CalcForce (src/mndo/Mndo.cpp:2711-2986) differentiates the atom
    pairs' terms only; the point charges act through the converged density.
    So the GPU forces equal central differences of the frozen-density pair
    energy without the charges, at the density of the SCF with them."""
    om, p, es = _run(ctx, "ch3cl_pm3", 4)
    es.DoSCF(True)
    P = es.GetOrbitalElectronPopulation()
    F = es.GetForce()

    def frozen(xyz):
        m = O.make_molecule(om.theory, om.Z, xyz)
        S, eri, ecore = O.integrals(m)
        return 0.5 * float(np.sum(P * (O.fock(m, S, eri, P) + O.fock(m, S, eri, np.zeros_like(P))))) + ecore

    h = 1e-4
    fd = np.zeros_like(om.xyz)
    for a in range(om.natoms):
        for k in range(3):
            xp, xm = om.xyz.copy(), om.xyz.copy()
            xp[a, k] += h
            xm[a, k] -= h
            fd[a, k] = -(frozen(xp) - frozen(xm)) / (2 * h)
    assert np.max(np.abs(F - fd)) < 2e-7, np.max(np.abs(F - fd))


def test_batch_with_point_charges(ctx):
    """nddo_batch_create_epc: molecules with and without charges in one
    resident batch, each against the oracle; new coordinates move the atoms
    and keep the charges."""
    names = ["ch4_mndo", "c2h6_mndo", "ch3f_mndo", "ch3cl_mndo"]
    mols, oms = [], []
    for i, nm in enumerate(names):
        mol, p = O.parse_input(FIX[nm]["input"])
        pc = point_charges(mol.xyz, 2 + 3 * i, 20 + i) if i != 1 else None
        mols.append(M.Molecule(mol.Z, mol.xyz, pc))
        oms.append(O.make_molecule(mol.theory, mol.Z, mol.xyz, pc))
    b = M.ResidentBatch("mndo", mols, context=ctx)
    b.run(_params(p))
    res, charges = b.results()
    for om, r, q in zip(oms, res, charges):
        ref = O.scf(om, p)
        assert r["status"] == M.STATUS_CONVERGED and r["iterations"] == ref.iterations
        assert abs(r["energy"] - ref.energy) < 1e-8
        assert abs(r["core_epc_coulomb"] - ref.core_epc) < 1e-11
        assert np.max(np.abs(q - ref.charges)) < 1e-6
    shift = np.random.default_rng(9).normal(scale=0.03, size=(sum(m.natoms for m in mols), 3))
    b.set_coordinates(np.concatenate([m.xyz for m in mols]) + shift)
    b.run(_params(p), requires_guess=False)
    res, _ = b.results()
    o = 0
    for om, r in zip(oms, res):
        moved = O.make_molecule(om.theory, om.Z, om.xyz + shift[o:o + om.natoms], om.epc)
        o += om.natoms
        ref = O.scf(moved, p)
        assert abs(r["energy"] - ref.energy) < 1e-8
        assert abs(r["core_epc_coulomb"] - ref.core_epc) < 1e-11
    b.close()
    # the one-call wrapper takes the same molecules
    res2, _ = M.batch_scf("mndo", mols, _params(p), context=ctx)
    for om, r in zip(oms, res2):
        assert abs(r["energy"] - O.scf(om, p).energy) < 1e-8


def test_serving_with_point_charges(ctx):
    """nddo_server_submit_epc: requests with charges in a stream with plain
    ones, against the oracle; a request with a charge on an atom fails alone
    without stopping the server."""
    names = ["ch3f_pm3", "c2h6_pm3", "ch3cl_pm3"]
    p = O.parse_input(FIX[names[0]]["input"])[1]   # one SCF block for the whole stream
    srv = M.Server(_params(p), context=ctx, hbm_budget_bytes=2 << 30, max_basis=256)
    want = {}
    for i, nm in enumerate(names):
        mol = O.parse_input(FIX[nm]["input"])[0]
        pc = point_charges(mol.xyz, 3 + 4 * i, 40 + i) if i != 1 else None
        t = srv.submit("pm3", M.Molecule(mol.Z, mol.xyz, pc))
        want[t] = O.scf(O.make_molecule(mol.theory, mol.Z, mol.xyz, pc), p)
    mol, _ = O.parse_input(FIX["ch4_pm3"]["input"])
    bad = srv.submit("pm3", M.Molecule(mol.Z, mol.xyz, np.c_[mol.xyz[:1], [0.5]]))
    res = {r["ticket"]: r for r in srv.drain()}
    srv.close()
    assert res[bad]["status"] == M.STATUS_FAILED
    for t, ref in want.items():
        r = res[t]
        assert r["status"] == M.STATUS_CONVERGED and r["iterations"] == ref.iterations
        assert abs(r["energy"] - ref.energy) < 1e-8
        assert abs(r["core_epc_coulomb"] - ref.core_epc) < 1e-11
        assert np.max(np.abs(r["charges"] - ref.charges)) < 1e-6


def test_edge_cases(ctx):
    """Charges of zero change nothing, bit for bit; a charge on an atom's
    position, a non-finite charge and a row count that is not a multiple of
    four are rejected and leave no molecule set."""
    mol, p = O.parse_input(FIX["c2h6_am1"]["input"])
    es = M.ElectronicStructure(mol.theory, _params(p), context=ctx)
    es.SetMolecule(M.Molecule(mol.Z, mol.xyz))
    es.DoSCF(True)
    e0, q0 = es.GetElectronicEnergy(0), es.GetMullikenCharges()
    zero = np.c_[point_charges(mol.xyz, 5, 3)[:, :3], np.zeros(5)]
    es.SetMolecule(M.Molecule(mol.Z, mol.xyz, zero))
    es.DoSCF(True)
    assert es.GetElectronicEnergy(0) == e0 and es.GetCoreEpcCoulombEnergy() == 0.0
    assert np.array_equal(es.GetMullikenCharges(), q0)
    for bad in (np.c_[mol.xyz[1:2], [0.3]], np.array([[5.0, 5.0, 5.0, np.nan]])):
        with pytest.raises(M.NddoError):
            es.SetMolecule(M.Molecule(mol.Z, mol.xyz, bad))
        with pytest.raises(M.NddoError):
            es.DoSCF(True)   # no molecule is set after a rejected one
    Z = np.ascontiguousarray(mol.Z, dtype=np.int32)
    xyz = np.ascontiguousarray(mol.xyz, dtype=np.float64)
    rc = ctx.lib.nddo_set_molecule_epc(ctx.h, mol.theory, int(Z.size), Z.ctypes.data_as(M._IP),
                                       xyz.ctypes.data_as(M._DP), -1, None)
    assert rc == M.ERR_ARGUMENT
