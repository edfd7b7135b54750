"""The allocation-free pair-integral entry point against the regular one.

nddo_pair_integrals_noalloc exists for callers that cannot call cudaMalloc
(their device memory comes from their own arena, or allocation is not allowed
where they call us): it writes the pair blocks and core Hamiltonian into device
buffers the caller owns and takes its scratch from a fixed static device array.
Here the caller's buffers are torch tensors; the results must equal what
nddo_set_molecule computes (read back through nddo_get_pair_blocks /
nddo_get_core_hamiltonian, and the core-core energy of nddo_scf), on two
different molecules called back to back.  This file is named to be collected
last, so a failure here stops a -x run only after every other test ran.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import molds_gb300 as M
from molds_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-12


def _regular(ctx, mol, theory):
    es = M.ElectronicStructure(theory, M.SCFParams(max_iter=500, rms_density=1e-8, damping_weight=0.0,
                                                   diis_start_error=0.1, diis_end_error=0.0), context=ctx)
    es.SetMolecule(mol)
    blocks = es.GetPairBlocks()
    H = es.GetCoreHamiltonian()
    es.DoSCF(True)
    return blocks, H, es.GetCoreRepulsionEnergy()


def _noalloc(lib, theory, mol, capacity, n_ao, torch):
    blocks = torch.full((max(capacity, 1),), float("nan"), dtype=torch.float64, device="cuda")
    H = torch.full((n_ao, n_ao), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    Z = np.ascontiguousarray(mol.Z, dtype=np.int32)
    xyz = np.ascontiguousarray(mol.xyz, dtype=np.float64)
    ecore = ctypes.c_double(float("nan"))
    err = ctypes.create_string_buffer(256)
    rc = lib.nddo_pair_integrals_noalloc(0, M.THEORIES[theory], int(Z.shape[0]), Z.ctypes.data_as(M._IP),
                                         xyz.ctypes.data_as(M._DP), ctypes.c_void_p(blocks.data_ptr()), capacity,
                                         ctypes.c_void_p(H.data_ptr()), ctypes.byref(ecore), None, err, 256)
    assert rc == 0, err.value.decode()
    return blocks.cpu().numpy()[:capacity], H.cpu().numpy(), ecore.value


def test_noalloc_matches_regular_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    ctx = M.Context(0)
    lib = ctx.lib
    fix = json.load(open(os.path.join(HERE, "golden", "reference_fixtures.json")))["cases"]
    m1, _ = O.parse_input([c for c in fix if c["name"] == "ch3cl_pm3"][0]["input"])
    first = (M.Molecule(m1.Z, m1.xyz), "pm3")
    w = W.water_cluster(shape=(2, 2, 1), seed=3)
    second = (w, "am1")
    regular = [_regular(ctx, mol, th) for mol, th in (first, second)]
    for (mol, th), (b_ref, h_ref, e_ref) in zip((first, second), regular):
        b, h, e = _noalloc(lib, th, mol, b_ref.size, h_ref.shape[0], torch)
        assert np.max(np.abs(b - b_ref)) < TOL
        assert np.max(np.abs(h - h_ref)) < TOL
        assert abs(e - e_ref) < TOL


def test_noalloc_rejects_oversized_input():
    ctx = M.Context(0)
    n = 513
    Z = np.ones(n, dtype=np.int32)
    xyz = np.arange(3 * n, dtype=np.float64)
    err = ctypes.create_string_buffer(256)
    rc = ctx.lib.nddo_pair_integrals_noalloc(0, 2, n, Z.ctypes.data_as(M._IP), xyz.ctypes.data_as(M._DP),
                                             ctypes.c_void_p(1), 10**9, ctypes.c_void_p(1), None, None, err, 256)
    assert rc == M.ERR_BUDGET
    assert b"512" in err.value
