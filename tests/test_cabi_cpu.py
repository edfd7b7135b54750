"""CPU-side checks of the boundary: the CUDA library builds and loads, exports
every entry point that include/nddo_gpu.h declares, and the host-side input
handling mirrors MolDS's parser.  No kernel is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest

import molds_gb300 as M
from molds_gb300 import inputfile, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "nddo_gpu.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(nddo_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from molds_gb300 import build
    build.build()
    return M.load_library()


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s


def test_python_binding_covers_the_header():
    assert set(declared_symbols()) == set(M.SIGNATURES)


def test_default_params_match_molds_defaults(lib):
    p = M.ScfParamsC()
    lib.nddo_default_params(ctypes.byref(p))
    # src/base/Parameters.cpp:133-139
    assert p.max_iter == 100 and p.rms_density == 1e-8 and p.damping_thresh == 1.0
    assert p.damping_weight == 0.8 and p.diis_num_error_vect == 5
    assert p.diis_start_error == 1e-2 and p.diis_end_error == 1e-8


def test_parse_reference_style_input():
    text = """THEORY
   pm3
THEORY_END
// a comment
SCF
   max_iter 500
   rms_density 1e-8
   damping_thresh 1.0
   damping_weight 0.0
   diis_num_error_vect 5
   diis_start_error 0.1
   diis_end_error 0.0
SCF_END
MEMORY
   limit_heap 1024
MEMORY_END
GEOMETRY
  C   0.0 0.0 0.0
  Cl  1.0 0.0 0.0   // trailing comment
GEOMETRY_END
"""
    f = inputfile.parse(text)
    assert f.theory == 2
    assert f.scf.max_iter == 500 and f.scf.damping_weight == 0.0 and f.scf.diis_end_error == 0.0
    assert f.limit_heap_mb == 1024
    assert list(f.molecule.Z) == [6, 17]
    assert abs(f.molecule.xyz[1, 0] - 1.0 / 0.5291772) < 1e-15


@pytest.mark.parametrize("name,theory", [("am1-d", 3), ("pm3-d", 4), ("pm3/pddg", 5)])
def test_parser_variants_and_vdw_keys(name, theory):
    """THEORY am1-d / pm3-d / pm3/pddg and the SCF keys vdW, vdW_s6, vdW_d
    (src/base/InputParser.cpp:286-293, 684-712) reach the C parameter block."""
    text = f"THEORY\n {name}\nTHEORY_END\nSCF\n vdW yes\n vdW_s6 0.88\n vdW_d 20\nSCF_END\n" \
           "GEOMETRY\n C 0 0 0\n O 1.2 0 0\nGEOMETRY_END"
    f = inputfile.parse(text)
    assert f.theory == theory
    assert f.scf.vdw and f.scf.vdw_s6 == 0.88 and f.scf.vdw_d == 20.0
    import molds_gb300 as M
    c = M.to_c_params(f.scf)
    assert c.vdw == 1 and c.vdw_s6 == 0.88 and c.vdw_d == 20.0 and c.dipole == 1


@pytest.mark.parametrize("bad", ["THEORY\n zindos\nTHEORY_END\nGEOMETRY\n H 0 0 0\n H 1 0 0\nGEOMETRY_END",
                                 "THEORY\n pm3\nTHEORY_END\nGEOMETRY\n Xe 0 0 0\nGEOMETRY_END",
                                 "THEORY\n pm3\nTHEORY_END\nCIS\nCIS_END\nGEOMETRY\n H 0 0 0\nGEOMETRY_END",
                                 "THEORY\n pm3\nTHEORY_END"])
def test_parser_rejects_out_of_scope_or_broken_input(bad):
    with pytest.raises(inputfile.InputError):
        inputfile.parse(bad)


def test_workloads_shapes():
    o = workloads.octane()
    assert o.natoms == 26 and (o.Z == 6).sum() == 8
    w = workloads.water_cluster()
    assert w.natoms == 96 and (w.Z == 8).sum() == 32
    reps = workloads.water_replicas(w, 3)
    assert len(reps) == 3 and np.all(reps[0].Z == w.Z)
    assert not np.allclose(reps[0].xyz, reps[1].xyz)
    a = workloads.random_alkane(3000000, n=9)
    assert (a.Z == 6).sum() == 9 and (a.Z == 1).sum() == 20


def test_octane_geometry_is_ideal():
    o = workloads.octane()
    x = o.xyz / inputfile.ANG2AU
    d = np.sqrt(((x[:, None] - x[None]) ** 2).sum(-1))
    c = np.nonzero(o.Z == 6)[0]
    for i in range(7):
        assert abs(d[c[i], c[i + 1]] - 1.54) < 1e-12
    # all-trans: C1...C4 of an anti dihedral are 3.9 A apart (gauche: 2.5-3.2 A)
    assert d[c[0], c[3]] > 3.8


def _bond_graph_distances(Z, d):
    """Graph distances of an alkane from its ideal bond lengths."""
    n = len(Z)
    bonded = (np.abs(d - 1.54) < 1e-9) & (Z[:, None] == 6) & (Z[None] == 6)
    bonded |= (np.abs(d - 1.09) < 1e-9) & (((Z[:, None] == 6) & (Z[None] == 1)) | ((Z[:, None] == 1) & (Z[None] == 6)))
    G = np.full((n, n), 99)
    np.fill_diagonal(G, 0)
    G[bonded] = 1
    for k in range(n):
        G = np.minimum(G, G[:, k:k + 1] + G[k:k + 1, :])
    return G


@pytest.mark.parametrize("seed", [3000000, 3000001, 3000002, 3000003])
def test_random_alkane_rules(seed):
    """Tree of CnH2n+2 with ideal bonds and angles; non-bonded pairs >= 3 bonds
    apart respect the C-C 1.8 A and 1.0 A floors; deterministic per seed."""
    a = workloads.random_alkane(seed)
    b = workloads.random_alkane(seed)
    assert np.array_equal(a.Z, b.Z) and np.array_equal(a.xyz, b.xyz)
    nc = int((a.Z == 6).sum())
    assert 3 <= nc <= 60 and (a.Z == 1).sum() == 2 * nc + 2
    x = a.xyz / inputfile.ANG2AU
    d = np.sqrt(((x[:, None] - x[None]) ** 2).sum(-1))
    G = _bond_graph_distances(a.Z, d)
    assert G.max() < 99                                   # connected
    assert (G == 1).sum() // 2 == a.natoms - 1            # a tree
    for i in np.nonzero(a.Z == 6)[0]:                     # every carbon has four bonds
        assert (G[i] == 1).sum() == 4
    ang13 = d[G == 2]                                     # tetrahedral 1-3 distances
    assert np.all(np.isin(np.round(ang13, 6), np.round([2 * 1.54 * np.sin(np.arccos(-1 / 3) / 2),
                                                        np.sqrt(1.54 ** 2 + 1.09 ** 2 + 2 * 1.54 * 1.09 / 3),
                                                        2 * 1.09 * np.sin(np.arccos(-1 / 3) / 2)], 6)))
    far = G >= 3
    cc = far & (a.Z[:, None] == 6) & (a.Z[None] == 6)
    assert np.all(d[cc] >= 1.8) and np.all(d[far] >= 1.0)
