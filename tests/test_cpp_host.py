"""The C++ host layer (include/nddo_electronic_structure.hpp): MolDS's
ElectronicStructure call surface over the C ABI, built with g++ against the
library as a MolDS translation unit would be.

CPU: it compiles, links and reports a missing GPU as a thrown MolDSException
(exit 3, status NDDO_ERR_CUDA), not a crash.  GPU: SetMolecule + DoSCF through
it give the oracle's energy, charges and iteration count."""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from scf_text_compare import compare_scf_text

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
FIX = json.load(open(os.path.join(HERE, "golden", "reference_fixtures.json")))["cases"]


def _program(tmp_path):
    from molds_gb300 import build
    build.build()
    libdir = os.path.join(ROOT, "molds_gb300", "_build")
    exe = str(tmp_path / "es_main")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "cpp", "electronic_structure_main.cpp"), "-o", exe,
                    "-L", libdir, "-lnddo_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    return exe


def _write_molecule(tmp_path, mol):
    p = tmp_path / "mol.txt"
    lines = [str(int(mol.theory))] + [f"{int(z)} {float(x):.17g} {float(y):.17g} {float(w):.17g}"
                                       for z, (x, y, w) in zip(mol.Z, mol.xyz)]
    if getattr(mol, "epc", None) is not None:
        lines += [f"epc {x:.17g} {y:.17g} {w:.17g} {q:.17g}" for x, y, w, q in np.asarray(mol.epc, dtype=float)]
    p.write_text("\n".join(lines) + "\n")
    return str(p)


def _args(p):
    return [str(int(p.max_iter)), f"{float(p.rms_density):.17g}", f"{float(p.damping_thresh):.17g}",
            f"{float(p.damping_weight):.17g}", str(int(p.diis_num_error_vect)), f"{float(p.diis_start_error):.17g}",
            f"{float(p.diis_end_error):.17g}"]


def _parse(out):
    vals = {}
    out, _, text = out.partition("scf_text\n")
    vals["scf_text"] = [text]
    for line in out.splitlines():
        k, v = line.split(" ", 1)
        vals.setdefault(k, []).append(v)
    return vals


def test_cpp_host_builds_and_reports_errors_as_exceptions(tmp_path):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present: the GPU test covers this program")
    except ImportError:
        pass
    exe = _program(tmp_path)
    mol, p = O.parse_input([c for c in FIX if c["name"] == "ch3f_pm3"][0]["input"])
    r = subprocess.run([exe, _write_molecule(tmp_path, mol)] + _args(p), capture_output=True, text=True)
    assert r.returncode == 3, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.startswith("error -2 ")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ch3f_pm3", "c2h6_pm3pddg", "ch3cl_mndo"])
def test_cpp_host_matches_oracle(tmp_path, name):
    exe = _program(tmp_path)
    case = [c for c in FIX if c["name"] == name][0]
    mol, p = O.parse_input(case["input"])
    ref = O.scf(mol, p)
    r = subprocess.run([exe, _write_molecule(tmp_path, mol)] + _args(p), capture_output=True, text=True)
    assert r.returncode == 0, (r.stdout, r.stderr)
    v = _parse(r.stdout)
    assert abs(float(v["energy"][0]) - ref.energy) < 1e-8
    assert abs(float(v["core_repulsion"][0]) - ref.core_repulsion) < 1e-10
    assert int(v["iterations"][0]) == ref.iterations
    q = np.array([float(x) for x in v["charge"]])
    assert np.max(np.abs(q - ref.charges)) < 1e-6
    assert abs(float(v["homo"][0]) - ref.eps[0]) < 1e-7
    assert np.max(np.abs(np.array([float(x) for x in v["dipole"]]) - ref.dipole[0])) < 1e-6
    assert int(v["excited_state_error"][0]) == -1
    # MolDS's SCF output text, against the reference's own output file
    assert not compare_scf_text(v["scf_text"][0], case["scf_text"], skip_iterations=p.rms_density < 1e-12)


@pytest.mark.gpu
def test_cpp_host_point_charges(tmp_path):
    """Environmental point charges through Molecule::epcs and
    GetCoreEpcCoulombEnergy, against the oracle; the SCF text carries the
    core-EPC lines."""
    import molds_gb300 as M
    exe = _program(tmp_path)
    mol, p = O.parse_input([c for c in FIX if c["name"] == "ch3f_am1"][0]["input"])
    pc = np.array([[6.0, 1.0, -2.0, -0.834], [-5.5, 3.0, 1.0, 0.417], [0.5, -6.5, 2.5, 0.417]])
    om = O.make_molecule(mol.theory, mol.Z, mol.xyz, pc)
    ref = O.scf(om, p)
    r = subprocess.run([exe, _write_molecule(tmp_path, om)] + _args(p), capture_output=True, text=True)
    assert r.returncode == 0, (r.stdout, r.stderr)
    v = _parse(r.stdout)
    assert abs(float(v["energy"][0]) - ref.energy) < 1e-8
    assert abs(float(v["core_epc"][0]) - ref.core_epc) < 1e-11
    assert int(v["iterations"][0]) == ref.iterations
    q = np.array([float(x) for x in v["charge"]])
    assert np.max(np.abs(q - ref.charges)) < 1e-6
    nocc = int(round(O.atom_info(om)[:, 0].sum())) // 2
    expect = M.format_scf_text(om.theory, om.Z, ref.eps, nocc, ref.trace, ref.energy, ref.core_repulsion,
                               ref.charges, dipole=ref.dipole, core_epc=ref.core_epc)
    assert not compare_scf_text(v["scf_text"][0], expect)
