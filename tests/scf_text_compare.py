"""Line-by-line comparison of MolDS's SCF output text (shared by the CPU and
GPU output tests).

The reference's own harness diffs its output files after dropping timing
lines (test/Test_Of_MolDS.rb:48); here the elapsed-time line is dropped and
every other line must have the same tab-separated fields: equal text, or two
numbers that differ by at most one unit in the sixth decimal of the mantissa
(the printed precision; the two programs round independently computed
values), or two numbers both below 1e-9 in magnitude (dipole components that
are round-off noise in the reference, printed as e.g. -2.3e-12).
"""


def _num(s):
    try:
        return float(s)
    except ValueError:
        return None


def _lines(text):
    out = [l for l in text.rstrip("\n").split("\n") if "Elapsed time(omp) for the SCF" not in l]
    while out and not out[-1].strip():
        out.pop()
    return out


def compare_scf_text(mine, ref, skip_iterations=False):
    """Returns a list of mismatch descriptions (empty when the texts agree)."""
    a, b = _lines(mine), _lines(ref)
    if skip_iterations:
        a = [l for l in a if not l.startswith("\tSCF iter ")]
        b = [l for l in b if not l.startswith("\tSCF iter ")]
    bad = []
    if len(a) != len(b):
        bad.append(f"{len(a)} lines vs {len(b)}")
    for i, (x, y) in enumerate(zip(a, b)):
        fx, fy = x.split("\t"), y.split("\t")
        if len(fx) != len(fy):
            bad.append(f"line {i}: {x!r} vs {y!r}")
            continue
        for u, v in zip(fx, fy):
            if u == v:
                continue
            nu, nv = _num(u), _num(v)
            if nu is None or nv is None:
                bad.append(f"line {i}: {u!r} vs {v!r}")
                continue
            if abs(nu) < 1e-9 and abs(nv) < 1e-9:
                continue
            if abs(nu - nv) <= 1.001e-6 * max(abs(nu), abs(nv)):
                continue
            bad.append(f"line {i}: {u} vs {v}")
    return bad
