"""MolDS input format, restricted to the blocks of the NDDO SCF path.

Follows src/base/InputParser.cpp: the file is read as whitespace tokens,
lower-cased, with ``//`` comments removed (:516-540); the THEORY block selects
the Hamiltonian (:284-295, 1397-1439), the SCF block sets the SCF parameters
(:311-325, 646-734), GEOMETRY lists ``El x y z`` in Angstrom converted to bohr
at parse time (:542-582), EPC lists environmental point charges
``x y z [charge q]`` in Angstrom (:626-644, charge 0 when omitted) and MEMORY
sets ``limit_heap`` in MB (:394-396, 1441-1453).  Other MolDS blocks are rejected: this package implements the
closed-shell NDDO SCF only.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

ANG2AU = 1.0 / 0.5291772             # src/base/Parameters.cpp:48
THEORIES = {"mndo": 0, "am1": 1, "pm3": 2, "am1-d": 3, "pm3-d": 4, "pm3/pddg": 5}   # src/base/InputParser.cpp:286-293
THEORY_NAMES = {0: "MNDO", 1: "AM1", 2: "PM3", 3: "AM1-D", 4: "PM3-D", 5: "PM3/PDDG"}
SYMBOL_TO_Z = {"h": 1, "c": 6, "n": 7, "o": 8, "f": 9, "s": 16, "cl": 17}
Z_TO_SYMBOL = {1: "H", 6: "C", 7: "N", 8: "O", 9: "F", 16: "S", 17: "Cl"}


class InputError(ValueError):
    pass


@dataclass
class SCFParams:
    """The SCF block; defaults of src/base/Parameters.cpp:133-139."""
    max_iter: int = 100
    rms_density: float = 1e-8
    damping_thresh: float = 1.0
    damping_weight: float = 0.8
    diis_num_error_vect: int = 5
    diis_start_error: float = 1e-2
    diis_end_error: float = 1e-8
    precision: str = "fp64"          # "fp64" or "mixed" (not a MolDS key)
    fp64_switch_error: float = 1e-4
    tensor_cores: bool = True        # mixed: FP32-phase GEMMs on tcgen05 (not a MolDS key)
    vdw: bool = False                # vdW yes/no (always on for AM1-D / PM3-D)
    vdw_s6: float = 1.40             # vdW_s6 (src/base/Parameters.cpp:141)
    vdw_d: float = 23.0              # vdW_d (src/base/Parameters.cpp:142)
    dipole: bool = True              # dipole moment after convergence, as DoSCF (not a MolDS key)
    eigensolver: str = "auto"        # FP64 eigensolves: "auto" / "householder" or "jacobi" (not a MolDS key)
    sum_charges: tuple = ()          # sum_charges first last (src/base/InputParser.cpp:694-700): ((first, last), ...)


@dataclass
class Molecule:
    """Atoms in input order; coordinates in bohr.  epc: environmental point
    charges, one row of x, y, z (bohr) and charge each, or None."""
    Z: np.ndarray
    xyz: np.ndarray
    epc: np.ndarray | None = None

    @property
    def natoms(self) -> int:
        return int(self.Z.shape[0])

    def symbols(self):
        return [Z_TO_SYMBOL[int(z)] for z in self.Z]


@dataclass
class InputFile:
    theory: int
    scf: SCFParams
    molecule: Molecule
    limit_heap_mb: float = 256.0     # src/base/Parameters.cpp:199
    tokens: list = field(default_factory=list)


_SCF_KEYS = {
    "max_iter": ("max_iter", int),
    "rms_density": ("rms_density", float),
    "damping_thresh": ("damping_thresh", float),
    "damping_weight": ("damping_weight", float),
    "diis_num_error_vect": ("diis_num_error_vect", int),
    "diis_start_error": ("diis_start_error", float),
    "diis_end_error": ("diis_end_error", float),
    "vdw_s6": ("vdw_s6", float),
    "vdw_d": ("vdw_d", float),
}


def tokenize(text: str):
    toks = []
    for line in text.splitlines():
        line = line.split("//")[0]
        toks += line.lower().split()
    return toks


def parse(text: str) -> InputFile:
    toks = tokenize(text)
    theory = None
    scf = SCFParams()
    atoms = []
    epcs = []
    limit = 256.0
    i = 0

    def need(k):
        if k >= len(toks):
            raise InputError("unexpected end of input")
        return toks[k]

    while i < len(toks):
        t = toks[i]
        if t == "theory":
            name = need(i + 1)
            if name not in THEORIES:
                raise InputError(f"theory '{name}' is not an NDDO theory (mndo, am1, pm3, am1-d, pm3-d, pm3/pddg)")
            theory = THEORIES[name]
            i += 2
            if need(i) != "theory_end":
                raise InputError("THEORY block must hold exactly one theory")
        elif t == "scf":
            i += 1
            while need(i) != "scf_end":
                key = toks[i]
                if key in _SCF_KEYS:
                    attr, conv = _SCF_KEYS[key]
                    setattr(scf, attr, conv(need(i + 1)))
                    i += 2
                elif key == "vdw":                 # src/base/InputParser.cpp:684-693
                    scf.vdw = need(i + 1) == "yes"
                    i += 2
                elif key == "sum_charges":         # src/base/InputParser.cpp:694-700
                    try:
                        pair = (int(need(i + 1)), int(need(i + 2)))
                    except ValueError as e:
                        raise InputError("sum_charges needs two atom indices") from e
                    scf.sum_charges = tuple(scf.sum_charges) + (pair,)
                    i += 3
                elif key in ("mpi", "scalapack"):
                    i += 2
                else:
                    raise InputError(f"unknown SCF keyword '{key}'")
        elif t == "geometry":
            i += 1
            while need(i) != "geometry_end":
                sym = toks[i]
                if sym not in SYMBOL_TO_Z:
                    raise InputError(f"element '{sym}' has no NDDO parameters here")
                try:
                    xyz = [float(need(i + k)) * ANG2AU for k in (1, 2, 3)]
                except ValueError as e:
                    raise InputError(f"bad coordinate for atom {len(atoms)}") from e
                atoms.append((SYMBOL_TO_Z[sym], xyz))
                i += 4
        elif t == "epc":                         # src/base/InputParser.cpp:626-644
            i += 1
            while need(i) != "epc_end":
                try:
                    xyz = [float(need(i + k)) * ANG2AU for k in (0, 1, 2)]
                except ValueError as e:
                    raise InputError(f"bad coordinate for point charge {len(epcs)}") from e
                i += 3
                q = 0.0
                if need(i) == "charge":
                    try:
                        q = float(need(i + 1))
                    except ValueError as e:
                        raise InputError(f"bad charge for point charge {len(epcs)}") from e
                    i += 2
                epcs.append(xyz + [q])
        elif t == "memory":
            i += 1
            while need(i) != "memory_end":
                if toks[i] == "limit_heap":
                    limit = float(need(i + 1))
                    i += 2
                else:
                    raise InputError(f"unknown MEMORY keyword '{toks[i]}'")
        else:
            raise InputError(f"block '{t}' is outside the NDDO SCF path")
        i += 1
    if theory is None:
        raise InputError("no THEORY block")
    if not atoms:
        raise InputError("no GEOMETRY block")
    Z = np.array([a[0] for a in atoms], dtype=np.int32)
    xyz = np.array([a[1] for a in atoms], dtype=np.float64)
    epc = np.array(epcs, dtype=np.float64).reshape(-1, 4) if epcs else None
    return InputFile(theory, scf, Molecule(Z, xyz, epc), limit, toks)
