"""Raw particle snapshots read and written by the C++ hydro driver.

Layout (little endian): b"FSPHSOA1", int64 n, int32 dim, int32 nfields (32),
then the 32 FP64 arrays of fsph_soa_view in header order, then int64 id[n].
Files with fewer arrays (29 to 31, written before the divergence and
electron-fraction fields existed) read with the missing arrays zero.
The reference writes H5part files (mpisph/io.h:874-1088); HDF5 is not part
of this build, so snapshots are raw SoA.
"""
import numpy as np

from .abi import DOUBLE_FIELDS

MAGIC = b"FSPHSOA1"


def write(path, state, dim):
    n = len(state["x"])
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(np.int64(n).tobytes())
        f.write(np.int32(dim).tobytes())
        f.write(np.int32(len(DOUBLE_FIELDS)).tobytes())
        for k in DOUBLE_FIELDS:
            f.write(np.ascontiguousarray(state[k], np.float64).tobytes())
        f.write(np.ascontiguousarray(state["id"], np.int64).tobytes())


def read(path):
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError("not an FSPHSOA1 snapshot")
        n = int(np.frombuffer(f.read(8), np.int64)[0])
        dim = int(np.frombuffer(f.read(4), np.int32)[0])
        nf = int(np.frombuffer(f.read(4), np.int32)[0])
        if not 0 < nf <= len(DOUBLE_FIELDS):
            raise ValueError(f"snapshot holds {nf} fields")
        out = {k: np.frombuffer(f.read(8 * n), np.float64).copy()
               for k in DOUBLE_FIELDS[:nf]}
        for k in DOUBLE_FIELDS[nf:]:
            out[k] = np.zeros(n)
        out["id"] = np.frombuffer(f.read(8 * n), np.int64).copy()
    return out, dim
