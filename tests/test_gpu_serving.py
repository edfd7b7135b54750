"""Serving loop (continuous batching) on the GPU: results of requests that
share the device with others equal the results of the same requests solved
alone, and equal the plain FP64 path."""
import numpy as np
import pytest

import molds_gb300 as M
from molds_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SCF = dict(max_iter=500, rms_density=1e-8, damping_thresh=1.0, damping_weight=0.0, diis_num_error_vect=5,
           diis_start_error=0.1, diis_end_error=0.0)


@pytest.fixture(scope="module")
def ctx():
    from molds_gb300 import build
    build.build()
    return M.Context(0)


def _mix():
    # molecules whose SCF converges robustly (some random alkanes make density
    # DIIS oscillate; whether they converge can differ between FP64 and mixed)
    mols = [W.water_cluster_k(3, 11), W.random_alkane(21, n=5), W.water_cluster_k(9, 12), W.random_alkane(22, n=14),
            W.water_cluster_k(20, 13), W.water_cluster_k(28, 15), W.water_cluster_k(40, 14)]   # N up to 240
    return mols


def _solve_alone(ctx, mols, params, **kw):
    out = []
    for m in mols:
        srv = M.Server(params, context=ctx, **kw)
        srv.submit("pm3", m)
        res = srv.drain()
        srv.close()
        assert len(res) == 1
        out.append(res[0])
    return out


def test_alone_equals_mix(ctx):
    params = M.SCFParams(**SCF, precision="mixed")
    mols = _mix()
    alone = _solve_alone(ctx, mols, params, hbm_budget_bytes=4 << 30, max_basis=256)
    srv = M.Server(params, context=ctx, hbm_budget_bytes=4 << 30, max_basis=256)
    filler = [W.water_cluster_k(k, 100 + k) for k in (2, 5, 7, 12, 16, 25)] + \
             [W.random_alkane(s, n=n) for s, n in ((200, 3), (201, 8), (202, 17))] + [W.water_cluster_k(30, 16)]
    tickets = {}
    results = []
    # staggered arrivals: some requests join while others are mid-SCF
    for i, m in enumerate(mols):
        tickets[srv.submit("pm3", m)] = i
        srv.submit("pm3", filler[i % len(filler)])
        results += srv.poll(3000)
    for f in filler:
        srv.submit("pm3", f)
        results += srv.poll(500)
    results += srv.drain()
    srv.close()
    by_ticket = {r["ticket"]: r for r in results}
    assert len(by_ticket) == len(mols) + len(mols) + len(filler)
    for t, i in tickets.items():
        r, a = by_ticket[t], alone[i]
        assert r["status"] == M.STATUS_CONVERGED
        assert r["iterations"] == a["iterations"]
        assert abs(r["energy"] - a["energy"]) <= 1e-12, (i, r["energy"], a["energy"])
        assert np.max(np.abs(r["charges"] - a["charges"])) <= 1e-12
    lanes = {by_ticket[t]["lane"] for t in tickets}
    assert lanes == {0, 1}          # the (H2O)40 request (N = 240) runs in the large lane


def test_serving_matches_plain_fp64(ctx):
    params = M.SCFParams(**SCF, precision="fp64")
    mols = _mix()[:6]
    srv = M.Server(params, context=ctx, hbm_budget_bytes=2 << 30, max_basis=194)
    tickets = [srv.submit("pm3", m) for m in mols]
    res = {r["ticket"]: r for r in srv.drain()}
    srv.close()
    es = M.ElectronicStructure("pm3", params, context=ctx)
    for t, m in zip(tickets, mols):
        es.SetMolecule(m)
        es.DoSCF()
        assert res[t]["iterations"] == es.GetIterations()
        assert abs(res[t]["energy"] - es.GetElectronicEnergy()) <= 1e-9
        assert np.max(np.abs(res[t]["charges"] - es.GetMullikenCharges())) <= 1e-9


def test_admission_waits_for_memory_and_reuses_slots(ctx):
    """A budget that holds only a couple of molecules: later requests wait in
    the queue, are admitted into freed space, and still give the alone result."""
    params = M.SCFParams(**SCF, precision="mixed")
    mols = [W.water_cluster_k(8 + (i % 3), 300 + i) for i in range(8)]     # N = 48..60
    alone = _solve_alone(ctx, mols[:3], params, hbm_budget_bytes=3 << 20, max_basis=64)
    srv = M.Server(params, context=ctx, hbm_budget_bytes=3 << 20, max_basis=64)
    tickets = [srv.submit("pm3", m) for m in mols]
    peak = 0
    res = []
    while True:
        res += srv.poll(2000)
        q, f = srv.pending()
        peak = max(peak, f)
        if q == 0 and f == 0:
            res += srv.poll(0)
            break
    srv.close()
    assert peak < len(mols)                 # never all resident at once
    by = {r["ticket"]: r for r in res}
    assert sorted(by) == sorted(tickets)
    for i in range(3):
        assert abs(by[tickets[i]]["energy"] - alone[i]["energy"]) <= 1e-12
    for k in range(3, 8):
        assert by[tickets[k]]["status"] == M.STATUS_CONVERGED


def test_slot_reuse_by_molecules_of_other_sizes(ctx):
    """A budget for one molecule at a time: each request reuses the same slot
    with a different basis size, and still gives its alone result."""
    params = M.SCFParams(**SCF, precision="mixed")
    mols = [W.water_cluster_k(10, 400), W.water_cluster_k(4, 401), W.water_cluster_k(8, 402), W.water_cluster_k(2, 403)]
    budget = 1200 * 1024            # about 5000 elements of the N x N arena: one N = 60 molecule at a time
    alone = _solve_alone(ctx, mols, params, hbm_budget_bytes=budget, max_basis=64)
    srv = M.Server(params, context=ctx, hbm_budget_bytes=budget, max_basis=64)
    tickets = [srv.submit("pm3", m) for m in mols]
    by = {r["ticket"]: r for r in srv.drain()}
    srv.close()
    for t, a in zip(tickets, alone):
        assert by[t]["status"] == M.STATUS_CONVERGED
        assert abs(by[t]["energy"] - a["energy"]) <= 1e-12
        assert np.max(np.abs(by[t]["charges"] - a["charges"])) <= 1e-12


def test_server_rejects_bad_requests(ctx):
    srv = M.Server(M.SCFParams(**SCF), context=ctx, hbm_budget_bytes=64 << 20, max_basis=64)
    with pytest.raises(M.NddoError):
        srv.submit("pm3", M.Molecule(np.array([1], dtype=np.int32), np.zeros((1, 3))))     # odd electron count
    with pytest.raises(M.NddoError):
        srv.submit("pm3", W.water_cluster_k(20, 1))                                         # N = 120 > 64
    srv.close()
