"""The product's element-parameter tables against the reference's own values.

tests/golden/reference_parameters.json holds every numeric parameter that
MolDS's SetAtomicParameters assigns (src/base/atoms/<El>atom.cpp, evaluated
from the source text by tests/golden/make_parameters.py).  The oracle maps
them onto each theory the way MolDS's Atom getters do (oracle/parameters.py).
This test compiles the product's header-only parameter code
(molds_gb300/csrc/nddo_units.h: the published tables and their conversion to
atomic units) into a small host program and compares every field of every
(theory, element) record with the oracle's, so a wrong digit in the product's
tables cannot hide behind a shared table.  No GPU is needed.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import parameters as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
THEORIES = {0: "MNDO", 1: "AM1", 2: "PM3", 3: "AM1-D", 4: "PM3-D", 5: "PDDG/PM3"}

DUMP = r"""
#include <stdio.h>
#include "nddo_units.h"
int main(void) {
  static const int zs[] = {1, 6, 7, 8, 9, 16, 17};
  printf("[");
  int first = 1;
  for (int t = 0; t < NDDO_NUM_THEORY_SLOTS; ++t)
    for (int k = 0; k < 7; ++k) {
      nddo_atom_params p;
      if (nddo_fill_atom_params(t, zs[k], &p) != 0) continue;
      printf("%s{\"theory\": %d, \"Z\": %d, \"core_charge\": %.17g, \"u_s\": %.17g, \"u_p\": %.17g, "
             "\"zeta_s\": %.17g, \"zeta_p\": %.17g, \"beta_s\": %.17g, \"beta_p\": %.17g, \"alpha\": %.17g, "
             "\"gss\": %.17g, \"gsp\": %.17g, \"gpp\": %.17g, \"gp2\": %.17g, \"hsp\": %.17g, \"hpp\": %.17g, "
             "\"d0\": %.17g, \"d1\": %.17g, \"d2\": %.17g, \"rho0\": %.17g, \"rho1\": %.17g, \"rho2\": %.17g, "
             "\"gk\": [%.17g, %.17g, %.17g, %.17g], \"gl\": [%.17g, %.17g, %.17g, %.17g], "
             "\"gm\": [%.17g, %.17g, %.17g, %.17g], \"e_atom\": %.17g, \"dhf_atom\": %.17g, "
             "\"core_mass\": %.17g, \"vdw_c6\": %.17g, \"vdw_r0\": %.17g, \"pddg_pa\": [%.17g, %.17g], "
             "\"pddg_da\": [%.17g, %.17g], \"n_ao\": %d, \"principal_n\": %d}",
             first ? "" : ",", t, zs[k], p.core_charge, p.u[0], p.u[1], p.zeta[0], p.zeta[1], p.beta[0],
             p.beta[1], p.alpha, p.gss, p.gsp, p.gpp, p.gp2, p.hsp, p.hpp, p.d[0], p.d[1], p.d[2], p.rho[0],
             p.rho[1], p.rho[2], p.gk[0], p.gk[1], p.gk[2], p.gk[3], p.gl[0], p.gl[1], p.gl[2], p.gl[3],
             p.gm[0], p.gm[1], p.gm[2], p.gm[3], p.e_atom, p.dhf_atom, p.core_mass, p.vdw_c6, p.vdw_r0,
             p.pddg_pa[0], p.pddg_pa[1], p.pddg_da[0], p.pddg_da[1], p.n_ao, p.principal_n);
      first = 0;
    }
  printf("]\n");
  return 0;
}
"""


@pytest.fixture(scope="module")
def product_records(tmp_path_factory):
    d = tmp_path_factory.mktemp("params")
    src = d / "dump.c"
    src.write_text(DUMP)
    exe = d / "dump"
    subprocess.run(["gcc", "-O0", "-std=c99", "-I", os.path.join(ROOT, "molds_gb300", "csrc"), "-o", str(exe),
                    str(src), "-lm"], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {(r["theory"], r["Z"]): r for r in json.loads(out)}


def _flat(r):
    """The product record as the oracle's field names."""
    f = {k: r[k] for k in ("core_charge", "u_s", "u_p", "zeta_s", "zeta_p", "beta_s", "beta_p", "alpha", "gss",
                           "gsp", "gpp", "gp2", "hsp", "hpp", "d0", "d1", "d2", "rho0", "rho1", "rho2", "e_atom",
                           "dhf_atom", "core_mass", "vdw_c6", "vdw_r0", "n_ao", "principal_n")}
    for i in range(4):
        f[f"gk{i}"], f[f"gl{i}"], f[f"gm{i}"] = r["gk"][i], r["gl"][i], r["gm"][i]
    for i in range(2):
        f[f"pddg_pa{i}"], f[f"pddg_da{i}"] = r["pddg_pa"][i], r["pddg_da"][i]
    return f


def test_every_product_record_matches_the_reference(product_records):
    """Every field of every (theory, element) the product serves equals the
    value the reference's element files define (atomic units, 1e-15 relative:
    the same decimal constants through the same operations)."""
    assert len(product_records) >= 36
    for (t, z), rec in product_records.items():
        ref = P.atom_record(t, z)
        assert ref is not None, f"{THEORIES[t]} Z={z}: the product serves a set the reference does not define"
        mine = _flat(rec)
        for k, v in mine.items():
            want = ref[k]
            assert abs(v - want) <= 1e-15 * max(1.0, abs(want)), (THEORIES[t], z, k, v, want)


def test_product_serves_every_reference_set_of_its_elements(product_records):
    """MNDO, AM1 and PM3 cover all seven elements in both; AM1-D, PM3-D and
    PDDG/PM3 are served for H, C, N, O and S (the elements MolDS's dispersion
    and PDDG sets are complete for; the AM1-D alpha of F and Cl is never
    assigned in the reference)."""
    for t in range(6):
        for z in P.Z_TO_SYMBOL:
            ref = P.atom_record(t, z)
            if t < 3:
                assert ref is not None and (t, z) in product_records, (THEORIES[t], z)
            elif z in (1, 6, 7, 8, 16):
                assert ref is not None and (t, z) in product_records, (THEORIES[t], z)


def test_am1_oxygen_pinned_by_the_reference_values():
    """The headline workload's theory/element pair, spelled out: AM1 O U_ss,
    zeta_s, beta, alpha, G_ss, D1, rho1 and the Gaussian K/L/M as MolDS
    assigns them (src/base/atoms/Oatom.cpp, AM1 block) in atomic units."""
    c = P.constants()
    r = P.atom_record(1, 8)
    assert r["u_s"] == -97.830000 * c["eV2AU"]
    assert r["zeta_s"] == 3.108032 and r["zeta_p"] == 2.524039
    assert r["beta_s"] == -29.272773 * c["eV2AU"]
    assert r["alpha"] == 4.455371 / c["angstrom2AU"]
    assert r["gss"] == 15.42 * c["eV2AU"]
    assert r["d1"] == 0.4988896404 and r["rho1"] == 0.5 / 0.9960801167
    assert r["gk0"] == 0.280962 * c["eV2AU"] and r["gl1"] == 7.00 / c["angstrom2AU"] ** 2.0
    assert r["gm0"] == 0.847918 * c["angstrom2AU"]
