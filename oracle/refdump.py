"""Reader for the binary state dumps written by oracle/ref_harness.cpp.

Test infrastructure only: used by tests/golden/make_golden.py (in the container that holds the
reference sources) to turn reference runs into committed fixtures.
"""
import numpy as np

_DT = {b"f": np.float32, b"d": np.float64, b"i": np.int32, b"I": np.uint32,
       b"Q": np.uint64, b"B": np.uint8}


def read_dump(path):
    """Return {name: [(step, array), ...]} in file order."""
    out = {}
    with open(path, "rb") as f:
        buf = f.read()
    assert buf[:4] == b"BGR1", "not a harness dump"
    off = 4
    while off < len(buf):
        name = buf[off:off + 24].split(b"\0", 1)[0].decode()
        dt = _DT[buf[off + 24:off + 25]]
        n, step = np.frombuffer(buf, dtype=np.uint64, count=2, offset=off + 32)
        off += 48
        nbytes = int(n) * np.dtype(dt).itemsize
        arr = np.frombuffer(buf, dtype=dt, count=int(n), offset=off).copy()
        off += nbytes
        if name == "end":
            break
        out.setdefault(name, []).append((int(step), arr))
    return out


def first(d, name):
    return d[name][0][1]


def series(d, name):
    """Stack all records of one name into a 2-D array [records, n] plus their steps."""
    recs = d.get(name, [])
    if not recs:
        return np.zeros(0, dtype=np.int64), None
    steps = np.array([s for s, _ in recs], dtype=np.int64)
    return steps, np.stack([a for _, a in recs])
