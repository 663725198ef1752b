"""fsph_sort_keys_noalloc: the key sort for callers that may not allocate
device memory (an application whose device memory belongs to its own pool
allocator, or a time-critical loop where cudaMalloc/cudaFree could stall on
a device synchronisation).  Its scratch is a fixed static device array in
the library, so it must reproduce exactly what the allocating path
(fsph_update_iteration) computes, call after call, with nothing allocated.

Collected last (file name) so that a failure here cannot hide other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NOALLOC_MAX = 1 << 20


def _lib():
    from flecsph_gb300 import build
    from flecsph_gb300.sph import library
    build.build()
    lib = library()
    f = lib.fsph_sort_keys_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                  C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return lib


@pytest.mark.parametrize("n1d", [32, 64])
def test_noalloc_sort_matches_update_iteration(n1d):
    torch = pytest.importorskip("torch")
    from flecsph_gb300 import setups
    from flecsph_gb300.sph import BodySystem
    lib = _lib()
    s, p, meta = setups.sedov3d(n1d)
    s = setups.shuffled(s, 17)
    n = meta["n"]
    # the allocating path: fsph_update_iteration, then the sorted keys/ids
    bs = BodySystem(p, n)
    bs.read_bodies(s)
    bs.update_iteration()
    ref = bs.download(fields=["key", "id"])
    bs.close()
    dev = torch.device("cuda:0")
    d = {k: torch.from_numpy(np.ascontiguousarray(s[k])).to(dev) for k in ("x", "y", "z", "h")}
    keys = torch.empty(n, dtype=torch.int64, device=dev)
    perm = torch.empty(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):
        keys.fill_(0)
        perm.fill_(-1)
        st = lib.fsph_sort_keys_noalloc(d["x"].data_ptr(), d["y"].data_ptr(),
                                        d["z"].data_ptr(), d["h"].data_ptr(), n, 3,
                                        keys.data_ptr(), perm.data_ptr(), stream)
        assert st == 0, st
        torch.cuda.synchronize(dev)
        k = keys.cpu().numpy().view(np.uint64)
        pm = perm.cpu().numpy().astype(np.int64)
        assert np.array_equal(k, ref["key"]), call
        assert np.array_equal(s["id"][pm], ref["id"]), call


def test_noalloc_sort_2d_and_allocates_nothing():
    """2D (z = NULL, y stands in for it) against update_iteration, twice;
    after the first call on the device, a call leaves the device's free
    memory unchanged."""
    torch = pytest.importorskip("torch")
    from flecsph_gb300 import setups
    from flecsph_gb300.sph import BodySystem
    lib = _lib()
    s, p, meta = setups.sod2d(200, 40)
    s = setups.shuffled(s, 23)
    n = meta["n"]
    bs = BodySystem(p, n)
    bs.read_bodies(s)
    bs.update_iteration()
    ref = bs.download(fields=["key", "id"])
    bs.close()
    dev = torch.device("cuda:0")
    d = {k: torch.from_numpy(np.ascontiguousarray(s[k])).to(dev) for k in ("x", "y", "h")}
    keys = torch.empty(n, dtype=torch.int64, device=dev)
    perm = torch.empty(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream

    def call():
        st = lib.fsph_sort_keys_noalloc(d["x"].data_ptr(), d["y"].data_ptr(), None,
                                        d["h"].data_ptr(), n, 2, keys.data_ptr(),
                                        perm.data_ptr(), stream)
        assert st == 0, st
        torch.cuda.synchronize(dev)

    for rep in range(2):
        keys.fill_(0)
        perm.fill_(-1)
        call()
        k = keys.cpu().numpy().view(np.uint64)
        pm = perm.cpu().numpy().astype(np.int64)
        assert np.array_equal(k, ref["key"]), rep
        assert np.array_equal(s["id"][pm], ref["id"]), rep
    free0, _ = torch.cuda.mem_get_info(dev)
    call()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0, (free0, free1)


def test_noalloc_sort_rejects_too_many_particles():
    torch = pytest.importorskip("torch")
    lib = _lib()
    dev = torch.device("cuda:0")
    a = torch.zeros(4, dtype=torch.float64, device=dev)
    k = torch.zeros(4, dtype=torch.int64, device=dev)
    p = torch.zeros(4, dtype=torch.int32, device=dev)
    # the size check happens on the host before anything is enqueued
    st = lib.fsph_sort_keys_noalloc(a.data_ptr(), a.data_ptr(), a.data_ptr(),
                                    a.data_ptr(), NOALLOC_MAX + 1, 3, k.data_ptr(),
                                    p.data_ptr(), None)
    assert st == 1
