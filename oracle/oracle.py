"""ORACLE -- test infrastructure, not product code.

CPU restatement of the MolDS closed-shell NDDO SCF (MNDO / AM1 / PM3):
integrals, Fock build and core-core terms come from the plain-C restatement in
``oracle/nddo_oracle.c`` (compiled to ``oracle/_build/liboracle.so``); the SCF
state machine below follows ``Cndo2::DoSCF`` (src/cndo/Cndo2.cpp:585-729) with
the reference's own LAPACK routines (``dsyevd`` for the Fock matrix,
``dsysv`` for the DIIS system) reached through scipy.

Only ``tests/``, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
use this module, as the checker or as the timed CPU reference.  The product
(``molds_gb300``) never imports it.

Reference semantics restated here (file:line in the MolDS tree):
  * guess Fock on iteration 0, DIIS/damping skipped there ...... Cndo2.cpp:631-640, 678
  * convergence test before DIIS: rms(P_old - P) < threshold ... Cndo2.cpp:663-670, 1472-1517
  * eigenvectors as rows with component-sum >= 0 ............... wrappers/Lapack.cpp:102-160
  * P = 2 C_occ^T C_occ ......................................... Cndo2.cpp:1702-1719
  * density DIIS (history shift, e = P - P_old, B row, solve) ... Cndo2.cpp:920-1028
  * damping ..................................................... Cndo2.cpp:1030-1061
  * E = 1/2 sum P (F + H) + E_core, F and H rebuilt ............. Cndo2.cpp:1324-1416
  * Mulliken q_A = Z_A - sum_mu P_mu,mu ......................... Cndo2.cpp:1187-1199, 1733-1747
  * MNDO heat of formation ...................................... mndo/Mndo.cpp:395-404
  * environmental point charges: -q (mu nu|s s) in every non-guess Fock,
    sum Z_A q / R in the energy .................................. mndo/Mndo.cpp:329-331,
                                                                    474-484, 546-556, 6602-6613
  * dipole: STO-6G Cartesian matrix (C restatement), origin at the
    centre of core mass, -sum P X + origin * sum P S, core part ... Cndo2.cpp:1871-1944,
                                                                    base/Molecule.cpp:396-419
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
import warnings
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg

try:
    from . import parameters as P
except ImportError:          # loaded as a top-level module
    import parameters as P

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "nddo_oracle.c")]

THEORIES = {"mndo": 0, "am1": 1, "pm3": 2, "am1-d": 3, "pm3-d": 4, "pm3/pddg": 5}
SYMBOL_TO_Z = {"h": 1, "c": 6, "n": 7, "o": 8, "f": 9, "s": 16, "cl": 17}
ANG2AU = P.constants()["angstrom2AU"]        # src/base/Parameters.cpp:48
KCAL2AU = P.constants()["kcalMolin2AU"]      # src/base/Parameters.cpp:47


def build(force: bool = False) -> str:
    """Compile the C restatement into oracle/_build/liboracle.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SOURCES)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c99", "-o", tmp] + SOURCES + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None
_lib_lock = threading.Lock()


def lib():
    global _lib
    with _lib_lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            dp = ctypes.POINTER(ctypes.c_double)
            ip = ctypes.POINTER(ctypes.c_int)
            L.oracle_num_aos.argtypes = [ctypes.c_int, ctypes.c_int, ip]
            L.oracle_integrals.argtypes = [ctypes.c_int, ctypes.c_int, ip, dp, dp, dp, dp]
            L.oracle_epc.argtypes = [ctypes.c_int, ctypes.c_int, ip, dp, ctypes.c_int, dp, dp, dp]
            L.oracle_multipole_params.argtypes = [ctypes.c_int, ctypes.c_int, dp]
            L.oracle_fock.argtypes = [ctypes.c_int, ctypes.c_int, ip, dp, dp, dp, ctypes.c_int, dp]
            L.oracle_atom_info.argtypes = [ctypes.c_int, ctypes.c_int, ip, dp]
            L.oracle_cartesian.argtypes = [ctypes.c_int, ctypes.c_int, ip, dp, dp]
            L.oracle_core_masses.argtypes = [ctypes.c_int, ctypes.c_int, ip, dp]
            L.oracle_vdw_params.argtypes = [ctypes.c_int, ctypes.c_int, ip, dp]
            L.oracle_sto_overlap_local.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                   ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                   ctypes.c_double]
            L.oracle_sto_overlap_local.restype = ctypes.c_double
            L.oracle_set_atom.argtypes = [ctypes.c_int, ctypes.c_int, dp]
            L.oracle_set_atom.restype = ctypes.c_int
            L.oracle_set_constants.argtypes = [ctypes.c_double, dp, dp]
            # every parameter set of the reference's element files (tests/golden/reference_parameters.json)
            ex, co = P.sto6g_tables()
            L.oracle_set_constants(ANG2AU, _dp(np.ascontiguousarray(ex, dtype=np.float64)),
                                   _dp(np.ascontiguousarray(co, dtype=np.float64)))
            for theory in range(6):
                for z in P.Z_TO_SYMBOL:
                    rec = P.record_array(theory, z)
                    if rec is not None and L.oracle_set_atom(theory, z, _dp(np.asarray(rec, dtype=np.float64))) != 0:
                        raise RuntimeError(f"oracle parameter record of Z={z} theory={theory} rejected")
            _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


@dataclass
class SCFParams:
    """SCF block defaults of src/base/Parameters.cpp:133-139."""
    max_iter: int = 100
    rms_density: float = 1e-8
    damping_thresh: float = 1.0
    damping_weight: float = 0.8
    diis_num_error_vect: int = 5
    diis_start_error: float = 1e-2
    diis_end_error: float = 1e-8
    vdw: bool = False                 # Parameters.cpp:140-142
    vdw_s6: float = 1.40
    vdw_d: float = 23.0


@dataclass
class Molecule:
    theory: int
    Z: np.ndarray            # int32 atomic numbers
    xyz: np.ndarray          # (A, 3) bohr
    epc: np.ndarray | None = None   # (n, 4): point charges x, y, z (bohr), charge

    @property
    def natoms(self):
        return int(self.Z.shape[0])


@dataclass
class SCFResult:
    converged: bool
    iterations: int
    energy: float            # electronic energy incl. core repulsion
    core_repulsion: float
    eps: np.ndarray
    C: np.ndarray            # eigenvectors as rows
    P: np.ndarray
    charges: np.ndarray
    heat_of_formation: float | None
    trace: list = field(default_factory=list)   # (iter, rms, diis_error, diis_on, damp_on)
    dipole: np.ndarray | None = None   # (3, 3): total, electronic, core; x y z [a.u.]
    vdw_energy: float = 0.0            # empirical dispersion energy, included in energy
    core_epc: float = 0.0              # sum Z_A q / R over cores and point charges, included in energy


class NotConverged(RuntimeError):
    pass


def make_molecule(theory, Z, xyz_bohr, epc=None) -> Molecule:
    if isinstance(theory, str):
        theory = THEORIES[theory.lower()]
    if epc is not None:
        epc = np.ascontiguousarray(epc, dtype=np.float64).reshape(-1, 4)
        epc = epc if epc.shape[0] else None
    return Molecule(int(theory), np.ascontiguousarray(Z, dtype=np.int32),
                    np.ascontiguousarray(xyz_bohr, dtype=np.float64).reshape(-1, 3), epc)


def multipole_params(theory, Z):
    """(D_0, D_1, D_2, rho_0, rho_1, rho_2) of one element [bohr]."""
    if isinstance(theory, str):
        theory = THEORIES[theory.lower()]
    out = np.zeros(6)
    if lib().oracle_multipole_params(int(theory), int(Z), _dp(out)) != 0:
        raise ValueError("element without NDDO parameters")
    return out


def epc_terms(mol: Molecule):
    """Point-charge terms: V (N x N, the -q (mu nu|s s) one-centre blocks of
    every non-guess Fock matrix) and sum Z_A q / R."""
    N = num_aos(mol)
    V = np.zeros((N, N))
    e = np.zeros(1)
    if mol.epc is None:
        return V, 0.0
    pc = np.ascontiguousarray(mol.epc, dtype=np.float64)
    if lib().oracle_epc(mol.theory, mol.natoms, _ip(mol.Z), _dp(mol.xyz), int(pc.shape[0]), _dp(pc),
                        _dp(V), _dp(e)) < 0:
        raise ValueError("element without NDDO parameters")
    return V, float(e[0])


def num_aos(mol: Molecule) -> int:
    n = lib().oracle_num_aos(mol.theory, mol.natoms, _ip(mol.Z))
    if n < 0:
        raise ValueError("element without NDDO parameters")
    return n


def atom_info(mol: Molecule) -> np.ndarray:
    out = np.zeros((mol.natoms, 4))
    if lib().oracle_atom_info(mol.theory, mol.natoms, _ip(mol.Z), _dp(out)) != 0:
        raise ValueError("element without NDDO parameters")
    return out


def integrals(mol: Molecule):
    """Overlap S (N x N), pair integrals eri[pair, 4,4,4,4] (a < b), E_core."""
    N = num_aos(mol)
    A = mol.natoms
    npairs = A * (A - 1) // 2
    S = np.zeros((N, N))
    eri = np.zeros((max(npairs, 1), 4, 4, 4, 4))
    ecore = np.zeros(1)
    r = lib().oracle_integrals(mol.theory, A, _ip(mol.Z), _dp(mol.xyz), _dp(S), _dp(eri), _dp(ecore))
    if r < 0:
        raise ValueError("oracle_integrals failed")
    return S, eri[:npairs], float(ecore[0])


def cartesian_matrix(mol: Molecule) -> np.ndarray:
    """<mu| r_k |nu> over all AO pairs, (3, N, N) [bohr] (Cndo2.cpp:1946-2130)."""
    N = num_aos(mol)
    X = np.zeros((3, N, N))
    if lib().oracle_cartesian(mol.theory, mol.natoms, _ip(mol.Z), _dp(mol.xyz), _dp(X)) < 0:
        raise ValueError("element without NDDO parameters")
    return X


def dipole(mol: Molecule, S, P, X=None) -> np.ndarray:
    """Total, electronic and core dipole moments (rows), x y z [a.u.]:
    origin c = centre of core mass (base/Molecule.cpp:396-419), core part
    sum_A Z_A (R_A - c) (Cndo2.cpp:1871-1882), electronic part
    -sum P X + c sum P S (Cndo2.cpp:1906-1936)."""
    X = cartesian_matrix(mol) if X is None else X
    info = atom_info(mol)
    mass = np.zeros(mol.natoms)
    lib().oracle_core_masses(mol.theory, mol.natoms, _ip(mol.Z), _dp(mass))
    center = np.zeros(3)
    for k in range(3):
        for a in range(mol.natoms):
            center[k] += mol.xyz[a, k] * mass[a]
    center /= mass.sum()
    core = np.array([sum(info[a, 0] * (mol.xyz[a, k] - center[k]) for a in range(mol.natoms))
                     for k in range(3)])
    pop = float(np.dot(P.ravel(), S.ravel()))
    elec = np.array([-float(np.dot(P.ravel(), X[k].ravel())) + center[k] * pop for k in range(3)])
    return np.stack([elec + core, elec, core])


def vdw_energy(mol: Molecule, s6: float, d: float) -> float:
    """Cndo2::CalcVdWCorrectionEnergy / GetDiatomVdWCorrectionEnergy
    (src/cndo/Cndo2.cpp:464-513): -s6 C6_AB f(R) / R^6 over atom pairs."""
    prm = np.zeros(2 * mol.natoms)
    if lib().oracle_vdw_params(mol.theory, mol.natoms, _ip(mol.Z), _dp(prm)) != 0:
        raise ValueError("element without dispersion parameters")
    c6, r0 = prm[0::2], prm[1::2]
    value = 0.0
    for i in range(mol.natoms):
        for j in range(i + 1, mol.natoms):
            dist = float(np.sqrt(np.sum((mol.xyz[i] - mol.xyz[j]) ** 2)))
            tmp = c6[i] + c6[j]
            if tmp <= 0.0:
                continue
            c = 2.0 * c6[i] * c6[j] / tmp
            damping = 1.0 / (1.0 + np.exp(-1.0 * d * (dist / (r0[i] + r0[j]) - 1.0)))
            value += -1.0 * s6 * c * damping / dist ** 6
    return value


def fock(mol: Molecule, S, eri, P, guess=False):
    N = S.shape[0]
    F = np.zeros((N, N))
    Pc = np.ascontiguousarray(P, dtype=np.float64)
    eri_c = np.ascontiguousarray(eri) if eri.size else np.zeros((1, 4, 4, 4, 4))
    lib().oracle_fock(mol.theory, mol.natoms, _ip(mol.Z), _dp(S), _dp(eri_c), _dp(Pc),
                      1 if guess else 0, _dp(F))
    if mol.epc is not None and not guess:
        F += epc_terms(mol)[0]
    return F


def diagonalize(F):
    """dsyevd on the upper triangle; eigenvectors returned as rows with
    component sum >= 0 (src/wrappers/Lapack.cpp:102-160)."""
    w, v = scipy.linalg.eigh(F, lower=False, driver="evd", check_finite=False)
    C = np.ascontiguousarray(v.T)
    flip = C.sum(axis=1) < 0
    C[flip] *= -1.0
    return w, C


def density(C, nocc):
    Co = C[:nocc]
    return 2.0 * (Co.T @ Co)


class _DIIS:
    """Density DIIS of Cndo2::DoDIIS (src/cndo/Cndo2.cpp:920-1028)."""

    def __init__(self, m, N):
        self.m = m
        self.dens = np.zeros((m, N, N))
        self.err = np.zeros((m, N, N))
        self.B = np.zeros((m + 1, m + 1))

    def step(self, P, P_old, step, start, end):
        m = self.m
        self.dens[:-1] = self.dens[1:].copy()
        self.err[:-1] = self.err[1:].copy()
        self.dens[-1] = P
        self.err[-1] = P - P_old
        self.B[:m - 1, :m - 1] = self.B[1:m, 1:m].copy()
        e_new = self.err[-1].ravel()
        row = self.err.reshape(m, -1) @ e_new
        self.B[m - 1, :m] = row
        self.B[:m, m - 1] = row
        self.B[:m, m] = -1.0
        self.B[m, :m] = -1.0
        self.B[m, m] = 0.0
        rhs = np.zeros(m + 1)
        rhs[m] = -1.0
        err = float(np.max(np.abs(e_new)))
        applied = False
        if m <= step and end < err < start:
            try:
                with warnings.catch_warnings():
                    # near convergence B is nearly singular; MolDS only skips the
                    # step when dsysv reports an exactly singular pivot
                    warnings.simplefilter("ignore", scipy.linalg.LinAlgWarning)
                    c = scipy.linalg.solve(self.B.copy(), rhs, assume_a="sym", check_finite=False)
            except (scipy.linalg.LinAlgError, np.linalg.LinAlgError):
                return P, err, False      # singular: skip (Cndo2.cpp:1003-1008)
            P = np.tensordot(c[:m], self.dens, axes=(0, 0))
            applied = True
        return P, err, applied


def scf(mol: Molecule, params: SCFParams | None = None, requires_guess=True, P0=None,
        log=None) -> SCFResult:
    params = params or SCFParams()
    info = atom_info(mol)
    nelec = int(round(info[:, 0].sum()))
    if nelec % 2:
        raise ValueError(f"odd number of valence electrons: {nelec}")
    nocc = nelec // 2
    S, eri, ecore = integrals(mol)
    N = S.shape[0]
    P = np.zeros((N, N)) if P0 is None else np.array(P0, dtype=np.float64)
    m = params.diis_num_error_vect
    diis = _DIIS(m, N) if m > 0 else None
    diis_err, diis_on, damp_on = 0.0, False, False
    trace = []
    for it in range(params.max_iter):
        P_old = P.copy()
        is_guess = (it == 0 and requires_guess)
        F = fock(mol, S, eri, P, guess=is_guess)
        eps, C = diagonalize(F)
        P = density(C, nocc)
        rms = float(np.sqrt(np.sum((P_old - P) ** 2) / (N * N)))
        trace.append((it, rms, diis_err, diis_on, damp_on))
        if log is not None:
            log(it, rms, diis_err, diis_on, damp_on)
        if rms < params.rms_density:
            return _properties(mol, S, eri, ecore, P, eps, C, info, it + 1, trace, params)
        if not is_guess:
            if diis is not None:
                P, diis_err, diis_on = diis.step(P, P_old, it, params.diis_start_error,
                                                 params.diis_end_error)
            damp_on = False
            if params.damping_weight > 0.0 and params.damping_thresh < rms:
                P = (1.0 - params.damping_weight) * P + params.damping_weight * P_old
                damp_on = True
    raise NotConverged(f"SCF did not met convergence criterion. maxIterationsSCF={params.max_iter}")


def _properties(mol, S, eri, ecore, P, eps, C, info, iters, trace, params) -> SCFResult:
    F = fock(mol, S, eri, P, guess=False)
    H = fock(mol, S, eri, np.zeros_like(P), guess=False)
    e_elec = 0.5 * float(np.sum(P * (F + H)))
    # AM1-D / PM3-D switch the dispersion term on with s6 = 1.40, d = 23
    # (InputParser::ValidateVdWConditions, src/base/InputParser.cpp:1657-1664)
    dtheory = mol.theory in (THEORIES["am1-d"], THEORIES["pm3-d"])
    evdw = 0.0
    if params.vdw or dtheory:
        evdw = vdw_energy(mol, 1.40 if dtheory else params.vdw_s6, 23.0 if dtheory else params.vdw_d)
    eepc = epc_terms(mol)[1] if mol.epc is not None else 0.0
    energy = e_elec + ecore + eepc + evdw
    firsts = np.concatenate([[0], np.cumsum(info[:, 1].astype(int))[:-1]])
    diag = np.diag(P)
    pop = np.array([diag[f:f + int(n)].sum() for f, n in zip(firsts, info[:, 1])])
    charges = info[:, 0] - pop
    hof = None
    if mol.theory == THEORIES["mndo"]:
        hof = energy - float(info[:, 2].sum()) + float(info[:, 3].sum())
    return SCFResult(True, iters, energy, ecore, eps, C, P, charges, hof, trace,
                     dipole(mol, S, P), evdw, eepc)


# --------------------------------------------------------------------------
# MolDS input format (THEORY / SCF / GEOMETRY / MEMORY blocks), restated from
# src/base/InputParser.cpp:516-582, 646-734, 1397-1453 for the oracle's tests.
# --------------------------------------------------------------------------
def parse_input(text: str):
    tokens = []
    for line in text.splitlines():
        line = line.split("//")[0]
        tokens += line.lower().split()
    theory, params, atoms, epcs = None, SCFParams(), [], []
    i = 0
    while i < len(tokens):
        t = tokens[i]
        if t == "theory":
            theory = tokens[i + 1]
            i += 2
            while tokens[i] != "theory_end":
                i += 1
        elif t == "scf":
            i += 1
            while tokens[i] != "scf_end":
                k, v = tokens[i], tokens[i + 1]
                if k == "max_iter":
                    params.max_iter = int(v)
                elif k == "rms_density":
                    params.rms_density = float(v)
                elif k == "damping_thresh":
                    params.damping_thresh = float(v)
                elif k == "damping_weight":
                    params.damping_weight = float(v)
                elif k == "diis_num_error_vect":
                    params.diis_num_error_vect = int(v)
                elif k == "diis_start_error":
                    params.diis_start_error = float(v)
                elif k == "diis_end_error":
                    params.diis_end_error = float(v)
                elif k == "vdw":                     # InputParser.cpp:684-693
                    params.vdw = v == "yes"
                elif k == "vdw_s6":
                    params.vdw_s6 = float(v)
                elif k == "vdw_d":
                    params.vdw_d = float(v)
                else:
                    i -= 1
                i += 2
        elif t == "geometry":
            i += 1
            while tokens[i] != "geometry_end":
                sym = tokens[i]
                xyz = [float(tokens[i + 1]) * ANG2AU, float(tokens[i + 2]) * ANG2AU,
                       float(tokens[i + 3]) * ANG2AU]
                atoms.append((SYMBOL_TO_Z[sym], xyz))
                i += 4
        elif t == "epc":                      # InputParser.cpp:626-644
            i += 1
            while tokens[i] != "epc_end":
                xyz = [float(tokens[i + k]) * ANG2AU for k in range(3)]
                i += 3
                q = 0.0
                if tokens[i] == "charge":
                    q = float(tokens[i + 1])
                    i += 2
                epcs.append(xyz + [q])
            continue
        i += 1
    Z = np.array([a[0] for a in atoms], dtype=np.int32)
    xyz = np.array([a[1] for a in atoms], dtype=np.float64)
    return make_molecule(theory, Z, xyz, epcs if epcs else None), params
