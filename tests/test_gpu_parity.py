"""Parity of the CUDA path with the oracle, through the C ABI.

Bars (from the reference's own correctness targets):
  * plain FP64 path: total energy within 1e-8 Eh, Mulliken charges within 1e-6
  * mixed precision: total energy within 1e-6 Eh
  * one-time integrals (pair blocks, core Hamiltonian): 1e-11 absolute
  * dipole moments (total, electronic, core): 1e-6 a.u., the Mulliken bar
    times a bohr; the STO-6G Cartesian matrix: 1e-11 relative to its largest
    element
"""
import ctypes
import json
import re
import os

import numpy as np
import pytest

import molds_gb300 as M
from molds_gb300 import workloads as W
from oracle import oracle as O
from scf_text_compare import compare_scf_text

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = json.load(open(os.path.join(HERE, "golden", "reference_fixtures.json")))["cases"]
E_TOL_FP64 = 1e-8
Q_TOL = 1e-6
E_TOL_MIXED = 1e-6
DIP_TOL = 1e-6


@pytest.fixture(scope="module")
def ctx():
    from molds_gb300 import build
    build.build()
    return M.Context(0)


def oracle_params(p: M.SCFParams):
    return O.SCFParams(max_iter=p.max_iter, rms_density=p.rms_density, damping_thresh=p.damping_thresh,
                       damping_weight=p.damping_weight, diis_num_error_vect=p.diis_num_error_vect,
                       diis_start_error=p.diis_start_error, diis_end_error=p.diis_end_error)


BENCH_SCF = M.SCFParams(max_iter=500, rms_density=1e-8, damping_thresh=1.0, damping_weight=0.0,
                        diis_num_error_vect=5, diis_start_error=0.1, diis_end_error=0.0)


def packed_from_oracle(mol, eri):
    """Oracle 4-index pair blocks -> the library's packed layout."""
    info = O.atom_info(mol)
    nao = info[:, 1].astype(int)
    out = []
    pidx = 0
    idx = [(0, 0), (0, 1), (0, 2), (0, 3), (1, 1), (1, 2), (1, 3), (2, 2), (2, 3), (3, 3)]
    A = mol.natoms
    for a in range(A):
        for b in range(a + 1, A):
            da = 10 if nao[a] == 4 else 1
            db = 10 if nao[b] == 4 else 1
            W4 = eri[pidx]
            blk = np.zeros((da, db))
            for P in range(da):
                for Q in range(db):
                    m, n = idx[P]
                    l, s = idx[Q]
                    blk[P, Q] = W4[m, n, l, s]
            out.append(blk.ravel())
            pidx += 1
    return np.concatenate(out) if out else np.zeros(0)


MOLS = {
    "ch3cl_pm3": lambda: O.parse_input([c for c in FIX if c["name"] == "ch3cl_pm3"][0]["input"])[0],
    "ch3f_mndo": lambda: O.parse_input([c for c in FIX if c["name"] == "ch3f_mndo"][0]["input"])[0],
    "water2_am1": lambda: O.make_molecule("am1", *_w2()),
    "nh3_h2s_mndo": lambda: O.make_molecule("mndo", np.array([7, 1, 1, 1, 16, 1, 1], dtype=np.int32),
                                            np.array([[0, 0, 0], [1.9, 0, 0], [-0.6, 1.8, 0], [-0.6, -0.9, 1.6],
                                                      [5.0, 1.0, 0.5], [6.0, 2.2, 0.5], [5.5, -0.3, 1.7]])),
}


def _w2():
    m = W.water_cluster(shape=(2, 1, 1), seed=7)
    return m.Z, m.xyz


@pytest.mark.parametrize("name", sorted(MOLS))
def test_pair_blocks_and_core_hamiltonian(ctx, name):
    mol = MOLS[name]()
    S, eri, ecore = O.integrals(mol)
    es = M.ElectronicStructure(mol.theory, context=ctx)
    es.SetMolecule(M.Molecule(mol.Z, mol.xyz))
    blocks = es.GetPairBlocks()
    ref = packed_from_oracle(mol, eri)
    assert blocks.shape == ref.shape
    assert np.max(np.abs(blocks - ref)) < 1e-11
    H = es.GetCoreHamiltonian()
    H_ref = O.fock(mol, S, eri, np.zeros_like(S), guess=False)
    assert np.max(np.abs(H - H_ref)) < 1e-11


@pytest.mark.parametrize("name", sorted(MOLS) + ["octane_pm3"])
def test_cartesian_matrix(ctx, name):
    """<mu| r_k |nu> of the STO-6G expansion (Cndo2.cpp:1946-2130) against the
    oracle's case-by-case restatement, every AO pair including same-atom ones."""
    mol = O.make_molecule("pm3", W.octane().Z, W.octane().xyz) if name == "octane_pm3" else MOLS[name]()
    es = M.ElectronicStructure(mol.theory, context=ctx)
    es.SetMolecule(M.Molecule(mol.Z, mol.xyz))
    X = es.GetCartesianMatrix()
    X_ref = O.cartesian_matrix(mol)
    assert X.shape == X_ref.shape
    assert np.max(np.abs(X - X_ref)) <= 1e-11 * max(1.0, np.max(np.abs(X_ref)))


@pytest.mark.parametrize("case", FIX, ids=[c["name"] for c in FIX])
def test_reference_fixtures_fp64(ctx, case):
    mol, p = O.parse_input(case["input"])
    ref = O.scf(mol, p)
    params = M.SCFParams(max_iter=p.max_iter, rms_density=p.rms_density, damping_thresh=p.damping_thresh,
                         damping_weight=p.damping_weight, diis_num_error_vect=p.diis_num_error_vect,
                         diis_start_error=p.diis_start_error, diis_end_error=p.diis_end_error,
                         vdw=p.vdw, vdw_s6=p.vdw_s6, vdw_d=p.vdw_d)
    es = M.ElectronicStructure(mol.theory, params, context=ctx)
    es.SetMolecule(M.Molecule(mol.Z, mol.xyz))
    es.DoSCF(True)
    assert abs(es.GetElectronicEnergy(0) - ref.energy) < E_TOL_FP64
    assert abs(es.GetCoreRepulsionEnergy() - ref.core_repulsion) < 1e-10
    assert np.max(np.abs(es.GetMullikenCharges() - ref.charges)) < Q_TOL
    assert np.max(np.abs(es.GetEnergiesMO() - ref.eps)) < 1e-7
    D = es.GetDipoleMoments()
    assert np.max(np.abs(D - ref.dipole)) < DIP_TOL
    assert abs(es.GetVdWCorrectionEnergy() - ref.vdw_energy) < 1e-12
    # the printed values of the reference itself (7 significant digits)
    assert abs(es.GetElectronicEnergy(0) - case["energy"]) <= 1e-6 * abs(case["energy"])
    for mine, theirs in zip(D.ravel(), np.array(case["dipole"]).ravel()):
        assert abs(mine - theirs) <= max(1e-6 * abs(theirs), 1e-9), (mine, theirs)
    if p.rms_density >= 1e-12:
        assert es.GetIterations() == ref.iterations
        tr = es.GetTrace()
        for (i, rms, derr, on, _), (_, rrms, rderr, ron, _) in zip(tr, ref.trace):
            assert abs(rms - rrms) <= 1e-6 * rrms + 1e-12, (i, rms, rrms)
            assert on == ron
    if mol.theory == 0:
        assert abs(es.GetHeatsFormation() - ref.heat_of_formation) < E_TOL_FP64
    # MolDS's SCF output text from the GPU results, against the reference's own
    # output file (the SCF section of the .dat, line by line)
    scf_block = re.search(r"(?is)^\s*scf\s*$(.*?)^\s*scf_end", case["input"], re.M).group(1)
    sums = [(int(a), int(b)) for a, b in re.findall(r"(?i)sum_charges\s+(\d+)\s+(\d+)", scf_block)]
    if sums:
        es.ctx.check(es.ctx.lib.nddo_set_sum_charges(es.ctx.h, len(sums), np.ascontiguousarray(
            np.array(sums, dtype=np.int32).ravel()).ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
    bad = compare_scf_text(es.OutputSCFResults(), case["scf_text"], skip_iterations=p.rms_density < 1e-12)
    assert not bad, "\n".join(bad[:10])


def test_density_and_eigenvectors_fp64(ctx):
    case = [c for c in FIX if c["name"] == "c2h6_am1"][0]
    mol, p = O.parse_input(case["input"])
    ref = O.scf(mol, p)
    es = M.ElectronicStructure(mol.theory, M.SCFParams(**{k: getattr(p, k) for k in vars(p)}), context=ctx)
    es.SetMolecule(M.Molecule(mol.Z, mol.xyz))
    es.DoSCF(True)
    P = es.GetOrbitalElectronPopulation()
    assert np.max(np.abs(P - ref.P)) < 1e-8
    C = es.GetFockMatrix()
    eps = es.GetEnergiesMO()
    # rows are orthonormal eigenvectors with component sum >= 0 (Lapack.cpp:141-150;
    # a row whose sum vanishes by symmetry may carry either sign at round-off level)
    assert np.max(np.abs(C @ C.T - np.eye(len(eps)))) < 1e-10
    assert np.all(C.sum(axis=1) >= -1e-12)


def test_octane_pm3_fp64(ctx):
    """The plain one-molecule FP64 path at N = 50 (the cluster Jacobi: one
    8-CTA cluster per molecule) against the oracle's LAPACK dsyevd run."""
    mol = W.octane()
    ref = O.scf(O.make_molecule("pm3", mol.Z, mol.xyz), oracle_params(BENCH_SCF))
    es = M.ElectronicStructure("pm3", BENCH_SCF, context=ctx)
    es.SetMolecule(mol)
    es.DoSCF(True)
    assert abs(es.GetElectronicEnergy(0) - ref.energy) < E_TOL_FP64
    assert np.max(np.abs(es.GetMullikenCharges() - ref.charges)) < Q_TOL
    assert es.GetIterations() == ref.iterations
    assert np.max(np.abs(es.GetEnergiesMO() - ref.eps)) < 1e-9
    assert np.max(np.abs(es.GetOrbitalElectronPopulation() - ref.P)) < 1e-8
    C = es.GetFockMatrix()
    assert np.max(np.abs(C @ C.T - np.eye(C.shape[0]))) < 1e-10
    assert np.all(C.sum(axis=1) >= -1e-12)
    assert np.max(np.abs(es.GetDipoleMoments() - ref.dipole)) < DIP_TOL


def test_plain_water32_fp64(ctx):
    """(H2O)32 AM1 (N = 192) on the plain path: the largest basis the cluster
    Jacobi serves."""
    mol = W.water_replicas(W.water_cluster(shape=(4, 4, 2), seed=2), 1)[0]
    ref = O.scf(O.make_molecule("am1", mol.Z, mol.xyz), oracle_params(BENCH_SCF))
    es = M.ElectronicStructure("am1", BENCH_SCF, context=ctx)
    es.SetMolecule(mol)
    es.DoSCF(True)
    assert abs(es.GetElectronicEnergy(0) - ref.energy) < E_TOL_FP64
    assert np.max(np.abs(es.GetMullikenCharges() - ref.charges)) < Q_TOL
    assert es.GetIterations() == ref.iterations
    assert np.max(np.abs(es.GetEnergiesMO() - ref.eps)) < 1e-9


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_water_cluster_am1(ctx, precision):
    mol = W.water_cluster(shape=(2, 2, 2), seed=2)          # (H2O)8, 48 basis functions
    ref = O.scf(O.make_molecule("am1", mol.Z, mol.xyz), oracle_params(BENCH_SCF))
    p = M.SCFParams(**{**vars(BENCH_SCF), "precision": precision})
    es = M.ElectronicStructure("am1", p, context=ctx)
    es.SetMolecule(mol)
    es.DoSCF(True)
    tol = E_TOL_FP64 if precision == "fp64" else E_TOL_MIXED
    assert abs(es.GetElectronicEnergy(0) - ref.energy) < tol
    assert np.max(np.abs(es.GetMullikenCharges() - ref.charges)) < Q_TOL
    assert np.max(np.abs(es.GetDipoleMoments() - ref.dipole)) < DIP_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_oracle_and_is_invariant(ctx, precision):
    base = W.water_cluster(shape=(2, 2, 1), seed=2)          # (H2O)4
    mols = W.water_replicas(base, 6)
    p = M.SCFParams(**{**vars(BENCH_SCF), "precision": precision})
    res, charges = M.batch_scf("am1", mols, p, context=ctx)
    tol = E_TOL_FP64 if precision == "fp64" else E_TOL_MIXED
    for m, r, q in zip(mols, res, charges):
        ref = O.scf(O.make_molecule("am1", m.Z, m.xyz), oracle_params(BENCH_SCF))
        assert r["status"] == M.STATUS_CONVERGED
        assert abs(r["energy"] - ref.energy) < tol
        assert np.max(np.abs(q - ref.charges)) < Q_TOL
        assert np.max(np.abs(r["dipole"] - ref.dipole)) < DIP_TOL
    # each molecule's result is the same alone and in the batch (bitwise)
    alone, qa = M.batch_scf("am1", [mols[3]], p, context=ctx)
    assert alone[0]["energy"] == res[3]["energy"]
    assert np.array_equal(qa[0], charges[3])
    assert np.array_equal(alone[0]["dipole"], res[3]["dipole"])
    # dipole = 0 skips the property and reports zeros
    skip, _ = M.batch_scf("am1", [mols[3]], M.SCFParams(**{**vars(p), "dipole": False}), context=ctx)
    assert skip[0]["energy"] == res[3]["energy"]
    assert not np.any(skip[0]["dipole"])


def test_uneven_batch(ctx):
    # seeds whose SCF converges (random trees with 1 A contacts can make density DIIS stall)
    mols = [W.random_alkane(3100000 + j, n_range=(3, 20)) for j in range(4)]
    mols.append(W.octane())
    res, charges = M.batch_scf("pm3", mols, BENCH_SCF, context=ctx)
    for m, r, q in zip(mols, res, charges):
        ref = O.scf(O.make_molecule("pm3", m.Z, m.xyz), oracle_params(BENCH_SCF))
        assert abs(r["energy"] - ref.energy) < E_TOL_FP64
        assert np.max(np.abs(q - ref.charges)) < Q_TOL
        assert np.max(np.abs(r["dipole"] - ref.dipole)) < DIP_TOL
        assert r["iterations"] == ref.iterations
    # a molecule's dipole does not depend on the sizes of its batch partners
    alone, _ = M.batch_scf("pm3", [mols[0]], BENCH_SCF, context=ctx)
    assert np.array_equal(alone[0]["dipole"], res[0]["dipole"])


def test_errors(ctx):
    es = M.ElectronicStructure("pm3", context=ctx)
    with pytest.raises(M.NddoError):          # odd electron count (Cndo2.cpp:351-357)
        es.SetMolecule(M.Molecule(np.array([1], dtype=np.int32), np.zeros((1, 3))))
    with pytest.raises(M.NddoError):          # no parameters for the element
        es.SetMolecule(M.Molecule(np.array([54, 54], dtype=np.int32), np.array([[0, 0, 0], [3.0, 0, 0]])))
    with pytest.raises(M.NddoError):          # coincident atoms (EularAngle.cpp:42-46)
        es.SetMolecule(M.Molecule(np.array([1, 1], dtype=np.int32), np.zeros((2, 3))))
    with pytest.raises(M.NddoError):          # non-finite coordinate
        es.SetMolecule(M.Molecule(np.array([1, 1], dtype=np.int32), np.array([[0, 0, 0], [np.nan, 0, 0]])))
    es.SetMolecule(W.octane())
    with pytest.raises(M.SCFNotConverged):    # Cndo2.cpp:700-704
        es.DoSCF(True, M.SCFParams(max_iter=3))
    tiny = M.Context(0, hbm_budget_bytes=1024)
    with pytest.raises(M.BudgetExceeded):
        M.ElectronicStructure("pm3", context=tiny).SetMolecule(W.octane())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_large_basis_block_jacobi(ctx, precision):
    """Bases above the one-CTA Jacobi's limit (N > 194) go through the block
    Jacobi; (H2O)40 (N = 240) and a C40 alkane (N = 242) against the oracle."""
    mols = [W.water_cluster_k(40, 7), W.random_alkane(3100000, n=40)]
    ref = []
    for m in mols:
        try:
            ref.append(O.scf(O.make_molecule("am1", m.Z, m.xyz), oracle_params(BENCH_SCF)))
        except O.NotConverged:
            ref.append(None)
    res, charges = M.batch_scf("am1", mols, M.SCFParams(**{**BENCH_SCF.__dict__, "precision": precision}),
                               context=ctx)
    checked = 0
    for r, q, rf in zip(res, charges, ref):
        if rf is None:          # density DIIS does not converge for this geometry (oracle and GPU alike)
            continue
        checked += 1
        assert r["status"] == M.STATUS_CONVERGED
        tol = E_TOL_FP64 if precision == "fp64" else E_TOL_MIXED
        assert abs(r["energy"] - rf.energy) < tol
        assert np.max(np.abs(q - rf.charges)) < Q_TOL
        if precision == "fp64":
            assert r["iterations"] == rf.iterations
    assert checked >= 1


def test_batch_scf_reuses_arrays_for_new_coordinates(ctx):
    """A second nddo_batch_scf call with the same molecules and new coordinates
    reuses the context's batch and gives what a fresh context gives."""
    base = W.water_cluster(shape=(2, 2, 1), seed=3)
    a = W.water_replicas(base, 4, seed0=10)
    b = W.water_replicas(base, 4, seed0=20)
    p = M.SCFParams(**{**BENCH_SCF.__dict__, "precision": "fp64"})
    M.batch_scf("am1", a, p, context=ctx)
    r1, q1 = M.batch_scf("am1", b, p, context=ctx)
    fresh = M.Context(0)
    r2, q2 = M.batch_scf("am1", b, p, context=fresh)
    fresh.close()
    for x, y, qa, qb in zip(r1, r2, q1, q2):
        assert x["status"] == M.STATUS_CONVERGED
        assert x["energy"] == y["energy"] and x["iterations"] == y["iterations"]
        assert np.array_equal(qa, qb)


def test_grouped_batch_new_coordinates_match_plain_path(ctx):
    """A resident batch of 100 molecules runs as concurrent groups; after
    nddo_batch_set_coordinates its results equal the plain one-molecule path."""
    base = W.water_cluster(shape=(2, 1, 1), seed=5)
    first = W.water_replicas(base, 100, seed0=500)
    moved = W.water_replicas(base, 100, seed0=900)
    p = M.SCFParams(**{**BENCH_SCF.__dict__, "precision": "fp64"})
    rb = M.ResidentBatch("am1", first, context=ctx)
    rb.run(p)
    rb.set_coordinates(np.concatenate([m.xyz for m in moved]))
    rb.run(p)
    res, q = rb.results()
    rb.close()
    es = M.ElectronicStructure("am1", p, context=ctx)
    for i in (0, 37, 63, 99):
        es.SetMolecule(moved[i])
        es.DoSCF()
        assert res[i]["status"] == M.STATUS_CONVERGED
        assert abs(res[i]["energy"] - es.GetElectronicEnergy()) <= 1e-10
        assert np.max(np.abs(q[i] - es.GetMullikenCharges())) <= 1e-10


def test_warm_start_after_coordinate_change(ctx):
    """The MD / MC step: the molecule moves and DoSCF(false) starts from the
    previous density (Cndo2::DoSCF with requiresGuess = false,
    src/cndo/Cndo2.cpp:585-729; src/md/MD.cpp:108), on the plain path and on a
    resident batch, against the oracle started from its own previous density."""
    base = W.water_cluster(shape=(2, 2, 2), seed=2)          # (H2O)8, 48 basis functions
    rng = np.random.default_rng(11)
    new_xyz = base.xyz + rng.normal(scale=0.02, size=base.xyz.shape)
    r0 = O.scf(O.make_molecule("am1", base.Z, base.xyz), oracle_params(BENCH_SCF))
    om1 = O.make_molecule("am1", base.Z, new_xyz)
    ref = O.scf(om1, oracle_params(BENCH_SCF), requires_guess=False, P0=r0.P)
    cold = O.scf(om1, oracle_params(BENCH_SCF))
    assert ref.iterations < cold.iterations
    es = M.ElectronicStructure("am1", BENCH_SCF, context=ctx)
    es.SetMolecule(base)
    es.DoSCF(True)
    es.SetCoordinates(new_xyz)
    es.DoSCF(False)
    assert abs(es.GetElectronicEnergy(0) - ref.energy) < E_TOL_FP64
    assert np.max(np.abs(es.GetMullikenCharges() - ref.charges)) < Q_TOL
    assert es.GetIterations() == ref.iterations
    # the same step for three replicas resident on the device
    mols = W.water_replicas(base, 3)
    b = M.ResidentBatch("am1", mols, context=ctx)
    b.run(BENCH_SCF)
    moved = [m.xyz + rng.normal(scale=0.02, size=m.xyz.shape) for m in mols]
    b.set_coordinates(np.concatenate(moved))
    b.run(BENCH_SCF, requires_guess=False)
    res, charges = b.results()
    for m, x, r, q in zip(mols, moved, res, charges):
        p0 = O.scf(O.make_molecule("am1", m.Z, m.xyz), oracle_params(BENCH_SCF)).P
        rr = O.scf(O.make_molecule("am1", m.Z, x), oracle_params(BENCH_SCF), requires_guess=False, P0=p0)
        assert abs(r["energy"] - rr.energy) < E_TOL_FP64
        assert np.max(np.abs(q - rr.charges)) < Q_TOL
        assert r["iterations"] == rr.iterations
    b.close()

