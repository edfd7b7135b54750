"""Regenerates tests/golden/reference_parameters.json from the MolDS sources.

Reads, as text, the reference's own definitions of the NDDO parameters and
evaluates them the way MolDS's constructors do:

  * src/base/Parameters.cpp -- the unit constants (eV2AU, angstrom2AU, ...),
    `const double Parameters::<name> = <expression>;`;
  * src/base/atoms/<El>atom.cpp, SetAtomicParameters -- every numeric
    `this-><field>[<i>] = <expression>;` of H, C, N, O, F, S and Cl (atomic
    mass, core charge, MNDO / AM1 / AM1-D / PM3 / PM3-D / PDDG parameters,
    van der Waals C6 and radius), with the Parameters getters replaced by the
    constants and `this-><field>` by the values assigned before it;
  * src/base/GTOExpansionSTO.cpp -- the STO-6G exponents and coefficients of
    the K, L and M shells.

Each expression is evaluated with IEEE double arithmetic in the source's
operator order, so the fixture holds the values MolDS's Atom objects hold.
The oracle builds its per-atom parameters from this file (oracle/parameters.py)
and a CPU test compares the product's tables against it field by field.

Usage:  python tests/golden/make_parameters.py <path to the MolDS src directory>
"""
import json
import math
import os
import re
import sys

ELEMENTS = [("H", 1), ("C", 6), ("N", 7), ("O", 8), ("F", 9), ("S", 16), ("Cl", 17)]
GETTERS = {"GetEV2AU": "eV2AU", "GetJ2AU": "j2AU", "GetKcalMolin2AU": "kcalMolin2AU",
           "GetAngstrom2AU": "angstrom2AU", "GetNm2AU": "nm2AU", "GetGMolin2AU": "gMolin2AU",
           "GetAvogadro": "avogadro", "GetDebye2AU": "debye2AU"}


def strip_comments(text):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def evaluate(expr, names):
    """Evaluates a C++ arithmetic expression of numbers, pow() and known names."""
    py = " ".join(expr.split())
    bare = re.sub(r"(?<![A-Za-z_0-9])(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?", " ", py)   # literals out of the name scan
    for tok in re.findall(r"[A-Za-z_][A-Za-z_0-9]*", bare):
        if tok not in names and tok not in ("pow", "M_PI"):
            raise KeyError(tok)
    return float(eval(py, {"__builtins__": {}}, dict(names, pow=math.pow, M_PI=math.pi)))


def constants(src):
    text = strip_comments(open(os.path.join(src, "base", "Parameters.cpp")).read())
    env = {}
    for name, expr in re.findall(r"const\s+double\s+Parameters::(\w+)\s*=\s*([^;]+);", text):
        expr = re.sub(r"Parameters::(\w+)", r"\1", expr)
        try:
            env[name] = evaluate(expr, env)
        except (KeyError, SyntaxError, NameError):
            continue
    return env


def element(src, symbol, const):
    text = strip_comments(open(os.path.join(src, "base", "atoms", f"{symbol}atom.cpp")).read())
    m = re.search(r"void\s+\w+::SetAtomicParameters\s*\(\s*\)\s*\{", text)
    depth, i = 1, m.end()
    while depth:
        depth += {"{": 1, "}": -1}.get(text[i], 0)
        i += 1
    body = text[m.end():i - 1]
    fields = {}
    shell = re.search(r"this->valenceShellType\s*=\s*(\w)Shell", body)
    fields["valenceShell"] = shell.group(1)                                  # k, l, m
    # s and p orbitals (the d set is pushed only under CNDO/2, e.g. Satom.cpp:57-63)
    fields["valenceOrbitals"] = len(re.findall(r"this->valence\.push_back\((?:s|px|py|pz)\)", body))
    scalars = dict(const)
    for stmt in body.split(";"):
        a = re.match(r"[\s{}]*this->(\w+)\s*(?:\[\s*(\d+)\s*\])?\s*=\s*(.+)$", stmt, flags=re.S)
        if not a:
            continue
        name, idx, expr = a.group(1), a.group(2), a.group(3)
        expr = re.sub(r"Parameters::GetInstance\(\)->(\w+)\(\)", lambda g: GETTERS.get(g.group(1), g.group(1)),
                      expr)
        expr = re.sub(r"this->(\w+)\s*\[\s*(\d+)\s*\]", lambda g: f"{g.group(1)}__{g.group(2)}", expr)
        expr = re.sub(r"this->(\w+)", r"\1", expr)
        try:
            v = evaluate(expr, scalars)
        except (KeyError, SyntaxError, NameError, TypeError):
            continue   # enum and container assignments (atomType, valence, ...)
        if idx is None:
            fields[name] = v
            scalars[name] = v
        else:
            k = int(idx)
            arr = fields.setdefault(name, [])
            while len(arr) <= k:
                arr.append(0.0)
            arr[k] = v
            scalars[f"{name}__{k}"] = v
    return fields


def sto6g(src):
    text = strip_comments(open(os.path.join(src, "base", "GTOExpansionSTO.cpp")).read())
    out = {"exponents": {}, "coefficients": {}}
    for kind in ("exponents", "coefficients"):
        for shell, az, i, val in re.findall(
                kind + r"\[STO6G\]\[(\w+)Shell\]\[(\w)Azimuthal\]\[(\d)\]\s*=\s*([-+0-9.eE]+)", text):
            out[kind].setdefault(f"{shell}{az}", [0.0] * 6)[int(i)] = float(val)
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_parameters.py <MolDS src directory>")
    src = sys.argv[1]
    const = constants(src)
    data = {"source": "MolDS src/base/Parameters.cpp, src/base/atoms/<El>atom.cpp SetAtomicParameters, "
                      "src/base/GTOExpansionSTO.cpp (STO-6G)",
            "constants": const,
            "elements": {sym: dict(element(src, sym, const), atomic_number=z) for sym, z in ELEMENTS},
            "sto6g": sto6g(src)}
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "reference_parameters.json"), "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    print("wrote", sum(len(v) for v in data["elements"].values()), "fields of", len(ELEMENTS), "elements")


if __name__ == "__main__":
    main()
