"""GB300-native closed-shell NDDO (MNDO / AM1 / PM3) SCF.

The compute path is the CUDA library ``molds_gb300/_build/libnddo_gb300.so``
(sm_103a), reached through its C ABI (``include/nddo_gpu.h``).  This module is
the Python mirror of MolDS's ``ElectronicStructure`` interface
(src/base/ElectronicStructure.h:23-53) on top of that ABI.  There is no CPU
fallback: when the library is missing the import of the engine fails with an
error telling how to build it.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .inputfile import (ANG2AU, THEORIES, THEORY_NAMES, InputError, InputFile, Molecule, SCFParams,  # noqa: F401
                        parse)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnddo_gb300.so")

NDDO_OK, NDDO_NOT_CONVERGED = 0, 1
ERR_ARGUMENT, ERR_CUDA, ERR_BUDGET, ERR_STATE = -1, -2, -3, -4
STATUS_CONVERGED, STATUS_NOT_CONVERGED, STATUS_FAILED = 1, 2, 3


class NddoError(RuntimeError):
    """Error raised across the C ABI (MolDS raises MolDSException)."""

    def __init__(self, code, message):
        super().__init__(message)
        self.code = code


class SCFNotConverged(NddoError):
    pass


class BudgetExceeded(NddoError):
    pass


class ScfParamsC(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_int), ("rms_density", ctypes.c_double),
                ("damping_thresh", ctypes.c_double), ("damping_weight", ctypes.c_double),
                ("diis_num_error_vect", ctypes.c_int), ("diis_start_error", ctypes.c_double),
                ("diis_end_error", ctypes.c_double), ("precision", ctypes.c_int),
                ("fp64_switch_error", ctypes.c_double), ("tensor_cores", ctypes.c_int),
                ("dipole", ctypes.c_int), ("vdw", ctypes.c_int), ("vdw_s6", ctypes.c_double),
                ("vdw_d", ctypes.c_double), ("eigensolver", ctypes.c_int)]


class ScfResultC(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int), ("energy", ctypes.c_double),
                ("core_repulsion", ctypes.c_double), ("heat_of_formation", ctypes.c_double),
                ("final_rms", ctypes.c_double), ("final_diis_error", ctypes.c_double),
                ("dipole", ctypes.c_double * 9), ("vdw_energy", ctypes.c_double),
                ("core_epc_coulomb", ctypes.c_double)]


class ServeResultC(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_longlong), ("status", ctypes.c_int), ("iterations", ctypes.c_int),
                ("n_atoms", ctypes.c_int), ("lane", ctypes.c_int), ("energy", ctypes.c_double),
                ("core_repulsion", ctypes.c_double), ("heat_of_formation", ctypes.c_double),
                ("final_rms", ctypes.c_double), ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double),
                ("t_done", ctypes.c_double), ("core_epc_coulomb", ctypes.c_double)]


# every entry point of include/nddo_gpu.h with its argument types
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_CTX = ctypes.c_void_p
SIGNATURES = {
    "nddo_default_params": (None, [ctypes.POINTER(ScfParamsC)]),
    "nddo_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]),
    "nddo_destroy": (None, [_CTX]),
    "nddo_last_error": (ctypes.c_char_p, [_CTX]),
    "nddo_set_molecule": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.c_int, _IP, _DP]),
    "nddo_set_molecule_epc": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.c_int, _IP, _DP, ctypes.c_int, _DP]),
    "nddo_set_coordinates": (ctypes.c_int, [_CTX, _DP]),
    "nddo_num_aos": (ctypes.c_int, [_CTX]),
    "nddo_num_atoms": (ctypes.c_int, [_CTX]),
    "nddo_scf": (ctypes.c_int, [_CTX, ctypes.POINTER(ScfParamsC), ctypes.c_int, ctypes.POINTER(ScfResultC)]),
    "nddo_get_energies_mo": (ctypes.c_int, [_CTX, _DP]),
    "nddo_get_fock_matrix": (ctypes.c_int, [_CTX, _DP]),
    "nddo_get_density": (ctypes.c_int, [_CTX, _DP]),
    "nddo_get_mulliken": (ctypes.c_int, [_CTX, _DP]),
    "nddo_get_core_hamiltonian": (ctypes.c_int, [_CTX, _DP]),
    "nddo_get_dipole": (ctypes.c_int, [_CTX, _DP]),
    "nddo_get_cartesian_matrix": (ctypes.c_int, [_CTX, _DP]),
    "nddo_get_trace": (ctypes.c_int, [_CTX, ctypes.c_int, _DP, _DP, _IP, _IP]),
    "nddo_scf_output_text": (ctypes.c_int, [_CTX, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "nddo_format_scf_text": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _IP, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            _DP, _DP, _IP, _IP, ctypes.c_int, _DP, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double, _DP, _DP,
                                            ctypes.c_double, ctypes.c_int,
                                            _IP, ctypes.c_double, ctypes.c_char_p, ctypes.c_size_t,
                                            ctypes.POINTER(ctypes.c_size_t)]),
    "nddo_set_sum_charges": (ctypes.c_int, [_CTX, ctypes.c_int, _IP]),
    "nddo_get_forces": (ctypes.c_int, [_CTX, _DP]),
    "nddo_batch_get_forces": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _DP]),
    "nddo_get_pair_blocks": (ctypes.c_int, [_CTX, _DP, ctypes.POINTER(ctypes.c_size_t)]),
    "nddo_batch_scf": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.c_int, _IP, _IP, _DP, ctypes.POINTER(ScfParamsC),
                                      ctypes.POINTER(ScfResultC), _DP]),
    "nddo_batch_create": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.c_int, _IP, _IP, _DP, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "nddo_batch_create_epc": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.c_int, _IP, _IP, _DP, _IP, _DP, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_void_p)]),
    "nddo_batch_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ScfParamsC)]),
    "nddo_batch_run_ex": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ScfParamsC), ctypes.c_int]),
    "nddo_batch_set_coordinates": (ctypes.c_int, [ctypes.c_void_p, _DP]),
    "nddo_batch_results": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ScfResultC), _DP]),
    "nddo_batch_device_bytes": (ctypes.c_size_t, [ctypes.c_void_p]),
    "nddo_batch_get_matrix": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _DP]),
    "nddo_batch_destroy": (None, [ctypes.c_void_p]),
    "nddo_batch_profile": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "nddo_batch_kernel_times": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _DP,
                                               ctypes.POINTER(ctypes.c_longlong), _DP]),
    "nddo_kernel_class_name": (ctypes.c_char_p, [ctypes.c_int]),
    "nddo_batch_timer": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _DP]),
    "nddo_measure_fma_peak": (ctypes.c_int, [_CTX, ctypes.c_int, _DP]),
    "nddo_batch_launch_count": (ctypes.c_longlong, [ctypes.c_void_p]),
    "nddo_batch_graph_launch_count": (ctypes.c_longlong, [ctypes.c_void_p]),
    "nddo_batch_jacobi_sweeps": (ctypes.c_longlong, [ctypes.c_void_p]),
    "nddo_server_create": (ctypes.c_int, [_CTX, ctypes.POINTER(ScfParamsC), ctypes.c_size_t, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_void_p)]),
    "nddo_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _IP, _DP,
                                          ctypes.POINTER(ctypes.c_longlong)]),
    "nddo_server_submit_epc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _IP, _DP, ctypes.c_int, _DP,
                                              ctypes.POINTER(ctypes.c_longlong)]),
    "nddo_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ServeResultC), _DP,
                                        ctypes.c_size_t, _IP]),
    "nddo_server_pending": (ctypes.c_int, [ctypes.c_void_p, _IP, _IP]),
    "nddo_server_clock": (ctypes.c_double, [ctypes.c_void_p]),
    "nddo_server_device_bytes": (ctypes.c_size_t, [ctypes.c_void_p]),
    "nddo_server_destroy": (None, [ctypes.c_void_p]),
    "nddo_pair_integrals_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _IP, _DP, ctypes.c_void_p,
                                                   ctypes.c_size_t, ctypes.c_void_p, _DP, ctypes.c_void_p,
                                                   ctypes.c_char_p, ctypes.c_size_t]),
}

_lib = None


def load_library(path: str = LIB_PATH):
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m molds_gb300.build` "
                          "(or __graft_entry__.build()); there is no CPU fallback")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(_DP)


def _ip(a):
    return a.ctypes.data_as(_IP)


def to_c_params(p: SCFParams) -> ScfParamsC:
    c = ScfParamsC()
    c.max_iter = int(p.max_iter)
    c.rms_density = float(p.rms_density)
    c.damping_thresh = float(p.damping_thresh)
    c.damping_weight = float(p.damping_weight)
    c.diis_num_error_vect = int(p.diis_num_error_vect)
    c.diis_start_error = float(p.diis_start_error)
    c.diis_end_error = float(p.diis_end_error)
    c.precision = 1 if str(p.precision).lower() == "mixed" else 0
    c.fp64_switch_error = float(p.fp64_switch_error)
    c.tensor_cores = 1 if getattr(p, "tensor_cores", True) else 0
    c.dipole = 1 if getattr(p, "dipole", True) else 0
    c.vdw = 1 if getattr(p, "vdw", False) else 0
    c.vdw_s6 = float(getattr(p, "vdw_s6", 1.40))
    c.vdw_d = float(getattr(p, "vdw_d", 23.0))
    c.eigensolver = {"auto": 0, "jacobi": 1, "householder": 2}[str(getattr(p, "eigensolver", "auto")).lower()]
    return c


def _dipole3(r) -> np.ndarray:
    """(3, 3): total, electronic, core dipole rows, x y z [a.u.]."""
    return np.array(r.dipole[:], dtype=np.float64).reshape(3, 3)


class Context:
    """An engine on one GPU (nddo_create / nddo_destroy)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.nddo_create(device, hbm_budget_bytes, ctypes.byref(h))
        self.h = h
        if rc != NDDO_OK:
            msg = self.lib.nddo_last_error(h).decode() if h.value else "nddo_create failed"
            if h.value:
                self.lib.nddo_destroy(h)
            self.h = None
            raise NddoError(rc, msg)

    def check(self, rc):
        if rc >= 0 and rc != NDDO_NOT_CONVERGED:
            return rc
        msg = self.lib.nddo_last_error(self.h).decode()
        if rc == NDDO_NOT_CONVERGED:
            raise SCFNotConverged(rc, msg)
        if rc == ERR_BUDGET:
            raise BudgetExceeded(rc, msg)
        raise NddoError(rc, msg)

    def close(self):
        if getattr(self, "h", None):
            self.lib.nddo_destroy(self.h)
            self.h = None

    def fma_peak_tflops(self, precision="fp32") -> float:
        v = ctypes.c_double()
        self.check(self.lib.nddo_measure_fma_peak(self.h, 0 if precision == "fp32" else 1, ctypes.byref(v)))
        return v.value

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ElectronicStructure:
    """MolDS ElectronicStructure for MNDO / AM1 / PM3 on one GB300.

    Same call sequence as the reference (src/base/MolDS.cpp:165-178):
    SetMolecule(molecule) once, DoSCF(requiresGuess) any number of times, then
    the getters.  Errors are raised as NddoError (SCFNotConverged when
    max_iter is reached, as Cndo2::DoSCF throws at src/cndo/Cndo2.cpp:700-704).
    """

    def __init__(self, theory, params: SCFParams | None = None, device: int = 0, hbm_budget_bytes: int = 0,
                 context: Context | None = None):
        self.theory = THEORIES[theory.lower()] if isinstance(theory, str) else int(theory)
        self.params = params or SCFParams()
        self.ctx = context or Context(device, hbm_budget_bytes)
        self.molecule = None
        self.result = None

    def GetTheoryType(self):
        return THEORY_NAMES[self.theory]

    def SetMolecule(self, molecule: Molecule):
        Z = np.ascontiguousarray(molecule.Z, dtype=np.int32)
        xyz = np.ascontiguousarray(molecule.xyz, dtype=np.float64).reshape(-1, 3)
        epc = getattr(molecule, "epc", None)
        epc = np.zeros((0, 4)) if epc is None else np.ascontiguousarray(epc, dtype=np.float64).reshape(-1, 4)
        self.ctx.check(self.ctx.lib.nddo_set_molecule_epc(self.ctx.h, self.theory, int(Z.shape[0]), _ip(Z), _dp(xyz),
                                                          int(epc.shape[0]), _dp(epc) if epc.size else None))
        self.molecule = molecule
        self.n = self.ctx.lib.nddo_num_aos(self.ctx.h)
        self.result = None

    def SetCoordinates(self, xyz_bohr):
        """Moves the molecule (same atoms): integrals are recomputed and the
        last density is kept, so DoSCF(False) starts from it (the MD / MC /
        optimiser pattern, src/md/MD.cpp:108)."""
        x = np.ascontiguousarray(xyz_bohr, dtype=np.float64).reshape(-1, 3)
        self.ctx.check(self.ctx.lib.nddo_set_coordinates(self.ctx.h, _dp(x)))
        self.molecule = Molecule(self.molecule.Z, x, getattr(self.molecule, "epc", None))

    def DoSCF(self, requiresGuess: bool = True, params: SCFParams | None = None):
        sp = params or self.params
        pairs = np.ascontiguousarray(np.array(sp.sum_charges, dtype=np.int32).reshape(-1, 2))
        self.ctx.check(self.ctx.lib.nddo_set_sum_charges(self.ctx.h, len(pairs), _ip(pairs) if len(pairs) else None))
        p = to_c_params(sp)
        r = ScfResultC()
        rc = self.ctx.lib.nddo_scf(self.ctx.h, ctypes.byref(p), 1 if requiresGuess else 0, ctypes.byref(r))
        self.result = r
        self.ctx.check(rc)
        return r

    def _vec(self, fn, n):
        out = np.zeros(n)
        self.ctx.check(fn(self.ctx.h, _dp(out)))
        return out

    def GetElectronicEnergy(self, elecState: int = 0) -> float:
        if elecState != 0:
            raise NddoError(ERR_ARGUMENT, "only the ground state is computed on this path")
        return self.result.energy

    def GetCoreRepulsionEnergy(self) -> float:
        return self.result.core_repulsion

    def GetVdWCorrectionEnergy(self) -> float:
        """Empirical dispersion energy, included in GetElectronicEnergy (Cndo2.cpp:825)."""
        return self.result.vdw_energy

    def GetCoreEpcCoulombEnergy(self) -> float:
        """Coulomb energy of the cores and the environmental point charges,
        sum Z_A q / R, included in GetElectronicEnergy (Cndo2.cpp:418-426, 1414)."""
        return self.result.core_epc_coulomb

    def GetHeatsFormation(self) -> float:
        return self.result.heat_of_formation

    def GetIterations(self) -> int:
        return self.result.iterations

    def GetEnergiesMO(self) -> np.ndarray:
        return self._vec(self.ctx.lib.nddo_get_energies_mo, self.n)

    def GetFockMatrix(self) -> np.ndarray:
        """After DoSCF: eigenvectors as rows (as MolDS returns them)."""
        return self._vec(self.ctx.lib.nddo_get_fock_matrix, self.n * self.n).reshape(self.n, self.n)

    def GetOrbitalElectronPopulation(self) -> np.ndarray:
        return self._vec(self.ctx.lib.nddo_get_density, self.n * self.n).reshape(self.n, self.n)

    def GetMullikenCharges(self) -> np.ndarray:
        return self._vec(self.ctx.lib.nddo_get_mulliken, self.molecule.natoms)

    def GetDipoleMoments(self) -> np.ndarray:
        """(3, 3): total, electronic and core dipole (rows), x y z [a.u.]
        (the three lines of Cndo2::OutputSCFDipole, src/cndo/Cndo2.cpp:1126-1185)."""
        return self._vec(self.ctx.lib.nddo_get_dipole, 9).reshape(3, 3)

    def GetCartesianMatrix(self) -> np.ndarray:
        """STO-6G <mu| r_k |nu>, (3, N, N) [bohr] (Cndo2.cpp:1946-2130)."""
        return self._vec(self.ctx.lib.nddo_get_cartesian_matrix, 3 * self.n * self.n).reshape(3, self.n, self.n)

    def GetCoreHamiltonian(self) -> np.ndarray:
        return self._vec(self.ctx.lib.nddo_get_core_hamiltonian, self.n * self.n).reshape(self.n, self.n)

    def GetPairBlocks(self) -> np.ndarray:
        cnt = ctypes.c_size_t()
        self.ctx.check(self.ctx.lib.nddo_get_pair_blocks(self.ctx.h, None, ctypes.byref(cnt)))
        out = np.zeros(cnt.value)
        self.ctx.check(self.ctx.lib.nddo_get_pair_blocks(self.ctx.h, _dp(out), ctypes.byref(cnt)))
        return out

    def GetForce(self) -> np.ndarray:
        """Forces -dE/dR on the atoms (n_atoms, 3) [Hartree/bohr] of the last
        converged SCF (Mndo::CalcForce, src/mndo/Mndo.cpp:2711-2986; ground
        state), analytic."""
        return self._vec(self.ctx.lib.nddo_get_forces, 3 * self.molecule.natoms).reshape(-1, 3)

    def OutputSCFResults(self) -> str:
        """The SCF section of MolDS's output for the last DoSCF (the text
        Cndo2::DoSCF prints between its banners, src/cndo/Cndo2.cpp:585-729,
        with OutputSCFResults :1299-1303)."""
        need = ctypes.c_size_t()
        self.ctx.check(self.ctx.lib.nddo_scf_output_text(self.ctx.h, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value)
        self.ctx.check(self.ctx.lib.nddo_scf_output_text(self.ctx.h, buf, need.value, ctypes.byref(need)))
        return buf.value.decode()

    def GetTrace(self):
        n = self.result.iterations
        rms, de = np.zeros(n), np.zeros(n)
        on, dm = np.zeros(n, dtype=np.int32), np.zeros(n, dtype=np.int32)
        # the return value is the entry count (>= 0), or a negative error code
        k = self.ctx.lib.nddo_get_trace(self.ctx.h, n, _dp(rms), _dp(de), _ip(on), _ip(dm))
        if k < 0:
            self.ctx.check(k)
        return [(i, float(rms[i]), float(de[i]), bool(on[i]), bool(dm[i])) for i in range(k)]


def format_scf_text(theory, Z, eps, nocc, trace, energy, core_repulsion, charges, dipole=None, vdw=False,
                    vdw_energy=0.0, heat_of_formation=0.0, converged=True, seconds=0.0, sum_charges=(),
                    core_epc=None) -> str:
    """MolDS's SCF output section from explicit values (nddo_format_scf_text;
    no GPU needed).  trace: [(iteration, rms, diis_error, diis_on, damping_on)];
    core_epc: the cores' Coulomb energy with environmental point charges (None:
    the molecule has none, no point-charge lines)."""
    L = load_library()
    th = THEORIES[theory.lower()] if isinstance(theory, str) else int(theory)
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    eps = np.ascontiguousarray(eps, dtype=np.float64)
    q = np.ascontiguousarray(charges, dtype=np.float64)
    rms = np.ascontiguousarray([t[1] for t in trace], dtype=np.float64)
    de = np.ascontiguousarray([t[2] for t in trace], dtype=np.float64)
    on = np.ascontiguousarray([int(t[3]) for t in trace], dtype=np.int32)
    dm = np.ascontiguousarray([int(t[4]) for t in trace], dtype=np.int32)
    dip = None if dipole is None else np.ascontiguousarray(np.ravel(dipole), dtype=np.float64)
    sp = np.ascontiguousarray(np.ravel(np.array(sum_charges, dtype=np.int32).reshape(-1, 2)), dtype=np.int32)
    args = (th, int(Z.size), _ip(Z), int(eps.size), int(nocc), len(trace), _dp(rms), _dp(de), _ip(on), _ip(dm),
            int(bool(converged)), _dp(eps), float(energy), float(core_repulsion), int(bool(vdw)), float(vdw_energy),
            int(core_epc is not None), float(core_epc or 0.0), None if dip is None else _dp(dip), _dp(q), float(heat_of_formation), int(sp.size // 2),
            _ip(sp) if sp.size else None, float(seconds))
    need = ctypes.c_size_t()
    rc = L.nddo_format_scf_text(*args, None, 0, ctypes.byref(need))
    if rc != 0:
        raise NddoError(rc, "nddo_format_scf_text: invalid arguments")
    buf = ctypes.create_string_buffer(need.value)
    L.nddo_format_scf_text(*args, buf, need.value, ctypes.byref(need))
    return buf.value.decode()


class ElectronicStructureFactory:
    """ElectronicStructureFactory::Create (src/base/factories/ElectronicStructureFactory.cpp:58-98)
    for the theories this package implements."""

    @staticmethod
    def Create(theory, **kw) -> ElectronicStructure:
        name = theory.lower() if isinstance(theory, str) else THEORY_NAMES[int(theory)].lower()
        if name not in THEORIES:
            raise NddoError(ERR_ARGUMENT, f"theory {theory} is not implemented on the GB300 path")
        return ElectronicStructure(name, **kw)


def batch_scf(theory, molecules, params: SCFParams | None = None, context: Context | None = None):
    """Batched SCF of many molecules in one device-resident launch sequence.

    Returns (results, charges): a list of dicts and a list of per-molecule
    Mulliken charge arrays."""
    ctx = context or Context()
    if any(getattr(m, "epc", None) is not None for m in molecules):
        # molecules with point charges: a resident batch (the context's cached
        # batch keys on atoms only)
        b = ResidentBatch(theory, molecules, (params or SCFParams()).diis_num_error_vect, context=ctx)
        try:
            b.run(params or SCFParams())
            return b.results()
        finally:
            b.close()
    th = THEORIES[theory.lower()] if isinstance(theory, str) else int(theory)
    nat = np.array([m.natoms for m in molecules], dtype=np.int32)
    Z = np.ascontiguousarray(np.concatenate([m.Z for m in molecules]), dtype=np.int32)
    xyz = np.ascontiguousarray(np.concatenate([np.asarray(m.xyz).reshape(-1, 3) for m in molecules]))
    res = (ScfResultC * len(molecules))()
    ch = np.zeros(int(nat.sum()))
    p = to_c_params(params or SCFParams())
    rc = ctx.lib.nddo_batch_scf(ctx.h, th, len(molecules), _ip(nat), _ip(Z), _dp(xyz), ctypes.byref(p), res, _dp(ch))
    if rc < 0:
        ctx.check(rc)
    out = [dict(status=r.status, iterations=r.iterations, energy=r.energy, core_repulsion=r.core_repulsion,
                heat_of_formation=r.heat_of_formation, final_rms=r.final_rms,
                final_diis_error=r.final_diis_error, dipole=_dipole3(r), vdw_energy=r.vdw_energy) for r in res]
    offs = np.concatenate([[0], np.cumsum(nat)])
    return out, [ch[offs[i]:offs[i + 1]] for i in range(len(molecules))]


class ResidentBatch:
    """A batch of molecules kept on the device (nddo_batch_*): run() repeats
    integrals + SCF + energies with no host traffic besides the per-iteration
    convergence count."""

    def __init__(self, theory, molecules, diis_num_error_vect=5, context: Context | None = None):
        self.ctx = context or Context()
        th = THEORIES[theory.lower()] if isinstance(theory, str) else int(theory)
        self.nat = np.array([m.natoms for m in molecules], dtype=np.int32)
        Z = np.ascontiguousarray(np.concatenate([m.Z for m in molecules]), dtype=np.int32)
        xyz = np.ascontiguousarray(np.concatenate([np.asarray(m.xyz).reshape(-1, 3) for m in molecules]))
        h = ctypes.c_void_p()
        # environmental point charges per molecule (Molecule.epc rows x, y, z, q)
        epcs = [np.zeros((0, 4)) if getattr(m, "epc", None) is None else np.asarray(m.epc, dtype=np.float64).reshape(-1, 4)
                for m in molecules]
        n_epc = np.array([e.shape[0] for e in epcs], dtype=np.int32)
        if n_epc.any():
            ep = np.ascontiguousarray(np.concatenate(epcs))
            self.ctx.check(self.ctx.lib.nddo_batch_create_epc(self.ctx.h, th, len(molecules), _ip(self.nat), _ip(Z),
                                                              _dp(xyz), _ip(n_epc), _dp(ep), diis_num_error_vect,
                                                              ctypes.byref(h)))
        else:
            self.ctx.check(self.ctx.lib.nddo_batch_create(self.ctx.h, th, len(molecules), _ip(self.nat), _ip(Z),
                                                          _dp(xyz), diis_num_error_vect, ctypes.byref(h)))
        self.h = h
        self.n = len(molecules)

    def run(self, params: SCFParams, requires_guess: bool = True):
        """Integrals + SCF + properties of every molecule; requires_guess=False
        starts each molecule from its density of the previous run (DoSCF(false))."""
        p = to_c_params(params)
        self.ctx.check(self.ctx.lib.nddo_batch_run_ex(self.h, ctypes.byref(p), 1 if requires_guess else 0))

    def set_coordinates(self, xyz):
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        self.ctx.check(self.ctx.lib.nddo_batch_set_coordinates(self.h, _dp(x)))

    def results(self):
        res = (ScfResultC * self.n)()
        ch = np.zeros(int(self.nat.sum()))
        rc = self.ctx.lib.nddo_batch_results(self.h, res, _dp(ch))
        if rc < 0:
            self.ctx.check(rc)
        offs = np.concatenate([[0], np.cumsum(self.nat)])
        out = [dict(status=r.status, iterations=r.iterations, energy=r.energy, core_repulsion=r.core_repulsion,
                    heat_of_formation=r.heat_of_formation, final_rms=r.final_rms,
                    final_diis_error=r.final_diis_error, dipole=_dipole3(r), vdw_energy=r.vdw_energy,
                    core_epc_coulomb=r.core_epc_coulomb) for r in res]
        return out, [ch[offs[i]:offs[i + 1]] for i in range(self.n)]

    def device_bytes(self) -> int:
        return int(self.ctx.lib.nddo_batch_device_bytes(self.h))

    def forces(self, m: int) -> np.ndarray:
        """Analytic forces (n_atoms, 3) [Hartree/bohr] of molecule m after run()."""
        out = np.zeros((int(self.nat[m]), 3))
        self.ctx.check(self.ctx.lib.nddo_batch_get_forces(self.h, m, _dp(out)))
        return out

    def density(self, m: int, nao: int) -> np.ndarray:
        out = np.zeros((nao, nao))
        self.ctx.check(self.ctx.lib.nddo_batch_get_matrix(self.h, 0, int(m), _dp(out)))
        return out

    def jacobi_sweeps(self) -> int:
        return int(self.ctx.lib.nddo_batch_jacobi_sweeps(self.h))

    def launch_count(self) -> int:
        return int(self.ctx.lib.nddo_batch_launch_count(self.h))

    def graph_launch_count(self) -> int:
        """CUDA-graph replays (one per SCF iteration of a molecule group)."""
        return int(self.ctx.lib.nddo_batch_graph_launch_count(self.h))

    def timer(self, op):
        ms = ctypes.c_double()
        self.ctx.check(self.ctx.lib.nddo_batch_timer(self.h, op, ctypes.byref(ms)))
        return ms.value

    def profile(self, enable=True):
        self.ctx.check(self.ctx.lib.nddo_batch_profile(self.h, 1 if enable else 0))

    def kernel_times(self):
        k = 16
        ms, w = np.zeros(k), np.zeros(k)
        ln = (ctypes.c_longlong * k)()
        n = self.ctx.check(self.ctx.lib.nddo_batch_kernel_times(self.h, k, _dp(ms), ln, _dp(w)))
        return {self.ctx.lib.nddo_kernel_class_name(i).decode(): dict(ms=float(ms[i]), launches=int(ln[i]),
                                                                      work=float(w[i])) for i in range(n)}

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.nddo_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request loop over single-point SCFs (nddo_server_*).

    submit() queues a molecule and returns a ticket at once; poll() drives the
    device lanes for up to max_wait_us and returns the finished requests as
    dicts (ticket, status, iterations, energy, core_repulsion,
    heat_of_formation, charges, lane, t_submit, t_admit, t_done -- seconds on
    the server clock, see clock()).
    """

    def __init__(self, params: SCFParams | None = None, hbm_budget_bytes: int = 0, max_basis: int = 1024,
                 context: Context | None = None, device: int = 0):
        self.ctx = context or Context(device)
        self.lib = self.ctx.lib
        h = ctypes.c_void_p()
        p = to_c_params(params or SCFParams())
        self.ctx.check(self.lib.nddo_server_create(self.ctx.h, ctypes.byref(p), int(hbm_budget_bytes), int(max_basis),
                                                   ctypes.byref(h)))
        self.h = h
        self._cap = 1 << 16
        self._out = (ServeResultC * 512)()
        self._charges = np.zeros(self._cap)

    def submit(self, theory, molecule: Molecule) -> int:
        t = THEORIES[theory.lower()] if isinstance(theory, str) else int(theory)
        Z = np.ascontiguousarray(molecule.Z, dtype=np.int32)
        xyz = np.ascontiguousarray(molecule.xyz, dtype=np.float64).reshape(-1, 3)
        ticket = ctypes.c_longlong()
        epc = getattr(molecule, "epc", None)
        if epc is not None and np.size(epc):
            ep = np.ascontiguousarray(epc, dtype=np.float64).reshape(-1, 4)
            self.ctx.check(self.lib.nddo_server_submit_epc(self.h, t, int(Z.shape[0]), _ip(Z), _dp(xyz),
                                                           int(ep.shape[0]), _dp(ep), ctypes.byref(ticket)))
        else:
            self.ctx.check(self.lib.nddo_server_submit(self.h, t, int(Z.shape[0]), _ip(Z), _dp(xyz),
                                                       ctypes.byref(ticket)))
        return ticket.value

    def poll(self, max_wait_us: int = 1000, max_results: int = 512):
        n = ctypes.c_int()
        max_results = min(max_results, len(self._out))
        self.ctx.check(self.lib.nddo_server_poll(self.h, int(max_wait_us), max_results, self._out, _dp(self._charges),
                                                 self._cap, ctypes.byref(n)))
        res, off = [], 0
        for k in range(n.value):
            o = self._out[k]
            q = self._charges[off:off + o.n_atoms].copy()
            off += o.n_atoms
            res.append({"ticket": o.ticket, "status": o.status, "iterations": o.iterations, "energy": o.energy,
                        "core_repulsion": o.core_repulsion, "heat_of_formation": o.heat_of_formation,
                        "final_rms": o.final_rms, "lane": o.lane, "t_submit": o.t_submit, "t_admit": o.t_admit,
                        "t_done": o.t_done, "core_epc_coulomb": o.core_epc_coulomb, "charges": q})
        return res

    def pending(self):
        q, f = ctypes.c_int(), ctypes.c_int()
        self.ctx.check(self.lib.nddo_server_pending(self.h, ctypes.byref(q), ctypes.byref(f)))
        return q.value, f.value

    def clock(self) -> float:
        return self.lib.nddo_server_clock(self.h)

    def device_bytes(self) -> int:
        return self.lib.nddo_server_device_bytes(self.h)

    def drain(self, max_wait_us: int = 2000):
        """Polls until nothing is queued or in flight; returns every result."""
        out = []
        while True:
            out.extend(self.poll(max_wait_us))
            q, f = self.pending()
            if q == 0 and f == 0:
                while True:
                    rest = self.poll(0)
                    if not rest:
                        return out
                    out.extend(rest)

    def close(self):
        if getattr(self, "h", None):
            self.lib.nddo_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
