"""Raw particle snapshots read and written by the C++ hydro driver.

Layout (little endian): b"FSPHSOA2", int64 n, int32 dim, int32 nfields (32),
int64 iteration, float64 dt, float64 time, then the 32 FP64 arrays of
fsph_soa_view in header order, then int64 id[n].  The time record is the
state's place in the run: the iteration it starts, the timestep and the
total time, which a restart restores (mpisph/io.h:523-586,818-836 read
"timestep" and "time" from the step whose "iteration" matches).
b"FSPHSOA1" files have no time record; files with fewer arrays (29 to 31,
written before the divergence and electron-fraction fields existed) read
with the missing arrays zero.
The reference writes H5part files (mpisph/io.h:874-1088); HDF5 is not part
of this build, so snapshots are raw SoA.
"""
import numpy as np

from .abi import DOUBLE_FIELDS

MAGIC = b"FSPHSOA2"
MAGIC_V1 = b"FSPHSOA1"


def write(path, state, dim, time=None):
    """Write `state`; `time` = (iteration, dt, total time) or None (0, 0, 0:
    a run that starts at iteration 0)."""
    n = len(state["x"])
    it, dt, t = time if time is not None else (0, 0.0, 0.0)
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(np.int64(n).tobytes())
        f.write(np.int32(dim).tobytes())
        f.write(np.int32(len(DOUBLE_FIELDS)).tobytes())
        f.write(np.int64(it).tobytes())
        f.write(np.float64(dt).tobytes())
        f.write(np.float64(t).tobytes())
        for k in DOUBLE_FIELDS:
            f.write(np.ascontiguousarray(state[k], np.float64).tobytes())
        f.write(np.ascontiguousarray(state["id"], np.int64).tobytes())


def read(path, with_time=False):
    """(state, dim), or (state, dim, (iteration, dt, time)) with with_time;
    the time record is None for an FSPHSOA1 file."""
    with open(path, "rb") as f:
        magic = f.read(8)
        if magic not in (MAGIC, MAGIC_V1):
            raise ValueError("not an FSPHSOA snapshot")
        n = int(np.frombuffer(f.read(8), np.int64)[0])
        dim = int(np.frombuffer(f.read(4), np.int32)[0])
        nf = int(np.frombuffer(f.read(4), np.int32)[0])
        if not 0 < nf <= len(DOUBLE_FIELDS):
            raise ValueError(f"snapshot holds {nf} fields")
        tm = None
        if magic == MAGIC:
            it = int(np.frombuffer(f.read(8), np.int64)[0])
            dt = float(np.frombuffer(f.read(8), np.float64)[0])
            t = float(np.frombuffer(f.read(8), np.float64)[0])
            tm = (it, dt, t)
        out = {k: np.frombuffer(f.read(8 * n), np.float64).copy()
               for k in DOUBLE_FIELDS[:nf]}
        for k in DOUBLE_FIELDS[nf:]:
            out[k] = np.zeros(n)
        out["id"] = np.frombuffer(f.read(8 * n), np.int64).copy()
    if with_time:
        return out, dim, tm
    return out, dim
