"""Snapshot files (flecsph_gb300/snapshot.py) on the host: the time record
of FSPHSOA2 and the older FSPHSOA1 layout."""
import numpy as np

from flecsph_gb300 import setups, snapshot
from flecsph_gb300.abi import DOUBLE_FIELDS


def test_roundtrip_with_time(tmp_path):
    s, p, m = setups.sod3d(8, 4, 4)
    s["Ye"][:] = 0.5
    f = tmp_path / "a.bin"
    snapshot.write(f, s, 3, time=(17, 2.5e-4, 0.125))
    out, dim, tm = snapshot.read(f, with_time=True)
    assert dim == 3 and tm == (17, 2.5e-4, 0.125)
    for k in DOUBLE_FIELDS:
        assert np.array_equal(out[k], s[k]), k
    assert np.array_equal(out["id"], s["id"])
    out2, dim2 = snapshot.read(f)
    assert np.array_equal(out2["x"], s["x"])


def test_reads_v1_without_time(tmp_path):
    s, p, m = setups.sod3d(8, 4, 4)
    n = len(s["x"])
    f = tmp_path / "v1.bin"
    with open(f, "wb") as fp:
        fp.write(b"FSPHSOA1")
        fp.write(np.int64(n).tobytes())
        fp.write(np.int32(3).tobytes())
        fp.write(np.int32(29).tobytes())
        for k in DOUBLE_FIELDS[:29]:
            fp.write(np.ascontiguousarray(s[k], np.float64).tobytes())
        fp.write(np.ascontiguousarray(s["id"], np.int64).tobytes())
    out, dim, tm = snapshot.read(f, with_time=True)
    assert tm is None and dim == 3
    assert np.array_equal(out["m"], s["m"])
    for k in DOUBLE_FIELDS[29:]:
        assert not out[k].any()
