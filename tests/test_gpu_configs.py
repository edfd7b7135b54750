"""Parity with the oracle on the benchmark's own workloads and on the SCF
options the reference fixtures leave unexercised (through the C ABI).

Bars: plain FP64 path 1e-8 Eh in the total energy and 1e-6 in the Mulliken
charges, the same iteration count and per-iteration RMS trace; mixed
precision 1e-6 Eh.
"""
import numpy as np
import pytest

import molds_gb300 as M
from molds_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

E_TOL_FP64 = 1e-8
Q_TOL = 1e-6
E_TOL_MIXED = 1e-6
SCF = dict(max_iter=500, rms_density=1e-8, damping_thresh=1.0, damping_weight=0.0, diis_num_error_vect=5,
           diis_start_error=0.1, diis_end_error=0.0)


@pytest.fixture(scope="module")
def ctx():
    from molds_gb300 import build
    build.build()
    return M.Context(0)


def oracle_scf(theory, mol, **kw):
    return O.scf(O.make_molecule(theory, mol.Z, mol.xyz), O.SCFParams(**{**SCF, **kw}))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_active_damping(ctx, precision):
    """Damping switched on (Cndo2::DoDamp, src/cndo/Cndo2.cpp:1030-1061): while
    the RMS density change is above damping_thresh the new density is mixed
    with the old one by damping_weight.  Octane PM3 and an (H2O)8 AM1 cluster,
    batched, against the oracle run with the same settings; the per-iteration
    damping flags must agree too."""
    damp = dict(damping_thresh=1e-3, damping_weight=0.5)
    cases = [("pm3", W.octane()), ("am1", W.water_cluster(shape=(2, 2, 2), seed=2))]
    for theory, mol in cases:
        ref = oracle_scf(theory, mol, **damp)
        assert any(t[4] for t in ref.trace), "the damping threshold never triggers"
        es = M.ElectronicStructure(theory, M.SCFParams(**{**SCF, **damp, "precision": precision}), context=ctx)
        es.SetMolecule(mol)
        es.DoSCF(True)
        tol = E_TOL_FP64 if precision == "fp64" else E_TOL_MIXED
        assert abs(es.GetElectronicEnergy(0) - ref.energy) < tol
        assert np.max(np.abs(es.GetMullikenCharges() - ref.charges)) < Q_TOL
        if precision == "fp64":
            assert es.GetIterations() == ref.iterations
            for (i, rms, derr, on, dmp), (_, rrms, rderr, ron, rdmp) in zip(es.GetTrace(), ref.trace):
                assert abs(rms - rrms) <= 1e-6 * rrms + 1e-12, (i, rms, rrms)
                assert on == ron and dmp == rdmp, i


def test_water32_replicas_fp64(ctx):
    """32 of the benchmark's 256 (H2O)32 AM1 replicas (the same generator and
    seeds), solved as one batch on the FP64 path: every energy, every
    Mulliken charge and every iteration count against the oracle."""
    base = W.water_cluster(shape=(4, 4, 2), spacing=2.9, jitter=0.2, seed=2)
    mols = W.water_replicas(base, 256, sigma=0.05, seed0=1000)[::8]
    res, charges = M.batch_scf("am1", mols, M.SCFParams(**SCF), context=ctx)
    for m, r, q in zip(mols, res, charges):
        ref = oracle_scf("am1", m)
        assert r["status"] == M.STATUS_CONVERGED
        assert abs(r["energy"] - ref.energy) < E_TOL_FP64
        assert np.max(np.abs(q - ref.charges)) < Q_TOL
        assert r["iterations"] == ref.iterations


def test_water32_replicas_mixed(ctx):
    """The same replicas on the mixed-precision path: within 1e-6 Eh of the
    oracle's FP64 energies."""
    base = W.water_cluster(shape=(4, 4, 2), spacing=2.9, jitter=0.2, seed=2)
    mols = W.water_replicas(base, 256, sigma=0.05, seed0=1000)[4::16]
    res, charges = M.batch_scf("am1", mols, M.SCFParams(**SCF, precision="mixed"), context=ctx)
    for m, r, q in zip(mols, res, charges):
        ref = oracle_scf("am1", m)
        assert abs(r["energy"] - ref.energy) < E_TOL_MIXED
        assert np.max(np.abs(q - ref.charges)) < 1e-5


def test_alkanes_up_to_sixty_carbons(ctx):
    """Random alkanes of the uneven workload's generator up to C60H122 (N =
    362: the tridiagonalisation runs on its global-memory workspace), solved
    in one uneven batch.  Molecules whose density DIIS also fails to converge
    in the oracle (the reference's own algorithm) are skipped; the rest must
    match."""
    # (seed, n): converging cases up to C60 and one whose density DIIS cycles
    picks = [(3100000, 30), (3100004, 40), (3100000, 50), (3100002, 50), (3100017, 60), (3100002, 30)]
    mols = [W.random_alkane(seed, n=n) for seed, n in picks]
    res, charges = M.batch_scf("pm3", mols, M.SCFParams(**SCF), context=ctx)
    checked = 0
    for m, r, q in zip(mols, res, charges):
        try:
            ref = oracle_scf("pm3", m)
        except O.NotConverged:
            assert r["status"] != M.STATUS_CONVERGED
            continue
        checked += 1
        assert r["status"] == M.STATUS_CONVERGED
        assert abs(r["energy"] - ref.energy) < E_TOL_FP64
        assert np.max(np.abs(q - ref.charges)) < Q_TOL
        assert r["iterations"] == ref.iterations
    assert checked == 5
