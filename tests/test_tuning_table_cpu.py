"""The committed launch-shape table (molds_gb300/tuning.txt, written by
molds_gb300/autotune.py and read by csrc/tuning.cpp) holds only keys and
values the loader accepts, so no entry is silently dropped."""
import os

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(os.path.dirname(HERE), "molds_gb300", "tuning.txt")


def _entries():
    for line in open(TABLE):
        line = line.strip()
        if line and not line.startswith("#"):
            yield line.split()


def test_every_entry_is_accepted():
    seen = set()
    for parts in _entries():
        key, vals = parts[0], [int(v) for v in parts[1:]]
        seen.add(key)
        if key == "check_block":
            assert len(vals) == 1 and 1 <= vals[0] <= 16
            continue
        assert len(vals) == 2, parts
        a, b = vals
        assert a >= 1, parts
        if key == "groups":
            assert 1 <= b <= 16
        elif key == "tridiag_threads":
            assert 32 <= b <= 1024 and b & (b - 1) == 0
        elif key == "vec_pairs":
            assert 1 <= b <= 16
        elif key == "vec_smem":
            assert b in (0, 1)
        else:
            raise AssertionError(f"unknown key {key}")
    assert {"groups", "tridiag_threads", "check_block", "vec_smem"} <= seen


def test_size_thresholds_ascend_to_a_catch_all():
    rows = {}
    for parts in _entries():
        if parts[0] in ("tridiag_threads", "vec_smem"):
            rows.setdefault(parts[0], []).append(int(parts[1]))
    for key, th in rows.items():
        assert th == sorted(th), key
        assert th[-1] >= 1 << 30, key   # every basis size has an entry
