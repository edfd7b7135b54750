"""Environmental point charges (MolDS EPC, row f4) on the CPU: the oracle's
restatement, the input block and the output lines.

The reference ships no input or output file with an EPC block, so these pin
the oracle's EPC terms to properties that follow from the reference's
definition (src/mndo/Mndo.cpp:329-331, 474-484, 546-556, 6602-6613): the
atom-EPC integrals of a hydrogen reduce to 1/R (no rho, s only), every
one-centre integral tends to the point-charge limit 1/R far away, the terms
are linear in the charges, a zero charge changes nothing, and energies are
invariant under a common rotation and translation of atoms and charges.  The
integral code underneath is the one the reference fixtures pin.
"""
import numpy as np
import pytest

import molds_gb300 as M
from molds_gb300 import inputfile
from oracle import oracle as O


def _water():
    ang = M.ANG2AU
    return np.array([8, 1, 1], dtype=np.int32), np.array([[0.0, 0.0, 0.0], [0.9572, 0.0, 0.0],
                                                          [-0.2400, 0.9266, 0.0]]) * ang


def test_hydrogen_term_is_coulomb():
    Z = np.array([1, 1], dtype=np.int32)
    xyz = np.array([[0.0, 0.0, 0.0], [1.4, 0.0, 0.0]])
    pc = np.array([[0.3, 2.0, -1.0, 0.7]])
    V, e = O.epc_terms(O.make_molecule("pm3", Z, xyz, pc))
    R = np.linalg.norm(xyz - pc[0, :3], axis=1)
    assert np.allclose(np.diag(V), -0.7 / R, rtol=0, atol=1e-15)
    assert np.count_nonzero(V - np.diag(np.diag(V))) == 0
    assert abs(e - 0.7 * np.sum(1.0 / R)) < 1e-15


@pytest.mark.parametrize("theory", ["mndo", "am1", "pm3"])
def test_far_charge_is_point_charge_limit(theory):
    Z, xyz = _water()
    for R in (200.0, 2000.0):
        pc = np.array([[R, 0.0, 0.0, -1.0]])
        V, _ = O.epc_terms(O.make_molecule(theory, Z, xyz, pc))
        d = np.linalg.norm(xyz - pc[0, :3], axis=1)
        # oxygen's four diagonal entries and each hydrogen's s: 1/R to O(D^2/R^3)
        assert np.allclose(np.diag(V)[:4], 1.0 / d[0], rtol=1e-4 * (200.0 / R) ** 2, atol=0)
        assert np.allclose(np.diag(V)[4:], 1.0 / d[1:], rtol=1e-12, atol=0)
        # s-p terms fall off as the dipole D1 / R^2
        assert np.max(np.abs(V[0, 1:4])) < 5.0 / R ** 2


def test_terms_are_linear_in_the_charges():
    Z, xyz = _water()
    pts = np.array([[4.0, 3.0, -2.0], [-5.0, 1.0, 3.5]])
    Va, ea = O.epc_terms(O.make_molecule("am1", Z, xyz, np.c_[pts, [0.4, 0.0]]))
    Vb, eb = O.epc_terms(O.make_molecule("am1", Z, xyz, np.c_[pts, [0.0, -1.1]]))
    Vc, ec = O.epc_terms(O.make_molecule("am1", Z, xyz, np.c_[pts, [0.4, -1.1]]))
    assert np.allclose(Va + Vb, Vc, rtol=0, atol=1e-15)
    assert abs(ea + eb - ec) < 1e-15


def test_zero_charge_changes_nothing():
    Z, xyz = _water()
    p = O.SCFParams(rms_density=1e-10)
    plain = O.scf(O.make_molecule("pm3", Z, xyz), p)
    zero = O.scf(O.make_molecule("pm3", Z, xyz, [[3.0, 3.0, 3.0, 0.0]]), p)
    assert zero.energy == plain.energy and zero.iterations == plain.iterations and zero.core_epc == 0.0


def test_rotation_and_translation_invariance():
    Z, xyz = _water()
    pc = np.array([[4.5, 1.0, 0.5, -0.8], [-3.0, 4.0, 1.5, 0.45]])
    p = O.SCFParams(rms_density=1e-10, max_iter=200)
    ref = O.scf(O.make_molecule("mndo", Z, xyz, pc), p)
    rng = np.random.default_rng(7)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    shift = np.array([1.5, -2.0, 0.25])
    moved = O.scf(O.make_molecule("mndo", Z, xyz @ q.T + shift, np.c_[pc[:, :3] @ q.T + shift, pc[:, 3]]), p)
    assert abs(moved.energy - ref.energy) < 1e-9
    assert abs(moved.core_epc - ref.core_epc) < 1e-12
    assert np.max(np.abs(moved.charges - ref.charges)) < 1e-7
    # the charges polarise the molecule: the result differs from the bare one
    bare = O.scf(O.make_molecule("mndo", Z, xyz), p)
    assert abs(bare.energy - ref.energy) > 1e-3 and np.max(np.abs(bare.charges - ref.charges)) > 1e-3


EPC_INPUT = """
THEORY
   am1
THEORY_END
GEOMETRY
   O  0.0000  0.0000  0.0000
   H  0.9572  0.0000  0.0000
   H -0.2400  0.9266  0.0000
GEOMETRY_END
EPC
   3.0  0.5 -1.0 charge -0.834
   -2.5 2.0  1.5 charge 0.417
   0.0  0.0  4.0
EPC_END
"""


def test_input_epc_block():
    f = inputfile.parse(EPC_INPUT)
    om, _ = O.parse_input(EPC_INPUT)
    assert f.molecule.epc.shape == (3, 4)
    assert np.array_equal(f.molecule.epc, om.epc)
    assert f.molecule.epc[2, 3] == 0.0      # no "charge" term: 0
    assert np.allclose(f.molecule.epc[0], [3.0 * M.ANG2AU, 0.5 * M.ANG2AU, -1.0 * M.ANG2AU, -0.834])
    assert inputfile.parse(EPC_INPUT.split("EPC\n")[0]).molecule.epc is None


@pytest.fixture(scope="module")
def built():
    from molds_gb300 import build
    build.build()


@pytest.mark.parametrize("vdw", [False, True])
def test_output_lines(built, vdw):
    """OutputSCFEnergies with point charges (src/cndo/Cndo2.cpp:1080-1124):
    the note names the core-EPC term and a block of its own follows the core
    repulsion."""
    Z, xyz = _water()
    om = O.make_molecule("pm3", Z, xyz, [[4.0, 0.0, 0.0, -0.5]])
    ref = O.scf(om, O.SCFParams(vdw=vdw))
    text = M.format_scf_text("pm3", Z, ref.eps, 4, ref.trace, ref.energy, ref.core_repulsion, ref.charges,
                             dipole=ref.dipole, vdw=vdw, vdw_energy=ref.vdw_energy, core_epc=ref.core_epc)
    lines = text.split("\n")
    note = ("\tNote that this electronic energy includes core-repulsions, core-EPC coulomb, and vdW correction."
            if vdw else "\tNote that this electronic energy includes core-repulsions and core-EPC coulomb.")
    assert note in lines
    k = lines.index("\tCoulomb interaction between cores and EPCs energy:\t%e\t%e" % (
        ref.core_epc, ref.core_epc / 0.03674903))   # eV2AU, src/base/Parameters.cpp:45
    assert lines[k - 1] == "\t\t\t\t\t\t\t\t|   [a.u.]   |   [eV]   |"
    assert lines[k - 3].startswith("\tCore repulsion energy:\t")
    plain = M.format_scf_text("pm3", Z, ref.eps, 4, ref.trace, ref.energy, ref.core_repulsion, ref.charges,
                              dipole=ref.dipole, vdw=vdw, vdw_energy=ref.vdw_energy)
    assert "EPC" not in plain


@pytest.mark.parametrize("theory", ["mndo", "am1", "pm3", "pm3/pddg"])
@pytest.mark.parametrize("Z", [6, 7, 8, 9, 16, 17])
def test_blocks_are_the_point_charge_model(theory, Z):
    """An independent restatement of the atom-charge block: MNDO's point-charge
    model of each orbital product (Dewar & Thiel 1977) with rho = 0 seen from
    a bare charge q on the local z axis at distance R -- ss a unit charge;
    s p_sigma +-1/2 at +-D_1 along the axis; p p (the monopole and the linear
    quadrupole) +1/2 at the centre and +1/4 at +-2 D_2 along the p axis --
    rotated into the space frame: (s s|ss) = s0, (s p_i|ss) = s10 u_i,
    (p_i p_j|ss) = s3 delta_ij + (s4 - s3) u_i u_j.  The oracle gets the same
    block through its general multipole case tree and 4-index rotation."""
    try:
        d = O.multipole_params(theory, Z)
    except ValueError:
        pytest.skip(f"no {theory} parameters for Z = {Z}")
    D1, D2 = d[1], d[2]
    rng = np.random.default_rng(Z * 31 + len(theory))
    for _ in range(5):
        at = rng.normal(size=3)
        v = rng.normal(size=3)
        pc = at + v / np.linalg.norm(v) * rng.uniform(3.0, 12.0)
        q = rng.uniform(-1.0, 1.0)
        V, e = O.epc_terms(O.make_molecule(theory, [Z], at[None, :], [[*pc, q]]))
        R = float(np.linalg.norm(pc - at))
        u = (pc - at) / R
        s0 = 1.0 / R
        s10 = 0.5 / (R - D1) - 0.5 / (R + D1)
        s3 = 0.5 / R + 0.5 / np.sqrt(R * R + 4.0 * D2 * D2)          # p_pi p_pi
        s4 = 0.5 / R + 0.25 / (R - 2.0 * D2) + 0.25 / (R + 2.0 * D2)  # p_sigma p_sigma
        uo = np.array([0.0, u[1], u[2], u[0]])                        # orbital order s, py, pz, px
        ref = np.zeros((4, 4))
        ref[0, 0] = s0
        for i in range(1, 4):
            ref[0, i] = ref[i, 0] = s10 * uo[i]
            for j in range(1, 4):
                ref[i, j] = (s3 if i == j else 0.0) + (s4 - s3) * uo[i] * uo[j]
        assert np.max(np.abs(V - (-q) * ref)) < 1e-14 * max(1.0, abs(q) / R)
        assert abs(e - O.atom_info(O.make_molecule(theory, [Z], at[None, :]))[0, 0] * q / R) < 1e-15
