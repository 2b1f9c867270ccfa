"""rdsim_get_pairs_static: the neighbour-pair entry point that allocates nothing.

Callers that cannot allocate device memory (processes whose device memory is
already committed, e.g. to a preallocated pool, where cudaMalloc fails; loops
that must not pay cudaFree's device-wide synchronisation) use
rdsim_get_pairs_static instead of rdsim_get_pairs.  It keeps its scratch
in a static device array, so its result must equal rdsim_get_pairs' result --
also on a second call in a row, which reuses the array left by the first.

Called through the C ABI with ctypes.  This file is collected last so that a
run stopping at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pairs(lib, h, fn, sys=0):
    n = C.c_int64()
    rc = getattr(lib, fn)(h, sys, None, 0, C.byref(n))
    assert rc in (0, 20), rc  # 20 = RDSIM_ERR_CAPACITY: buffer of size 0
    out = np.empty((max(1, n.value), 2), dtype=np.int32)
    rc = getattr(lib, fn)(h, sys, out.ctypes.data_as(C.POINTER(C.c_int32)), n.value, C.byref(n))
    assert rc == 0, lib.rdsim_last_error().decode()
    return out[: n.value].copy()


def _systems():
    from helpers import deck_dict, load_fixture, system_from_deck
    from pyrdsim_gb300 import workloads
    fx = load_fixture("patchy")
    yield system_from_deck(deck_dict(fx), int(fx["seed"]))
    fx = load_fixture("two_species_wall_rx")
    yield system_from_deck(deck_dict(fx), int(fx["seed"]))
    yield workloads.active_wall_fluid(n=8192, seed=9)


def test_static_pairs_match_allocating_pairs_twice():
    from pyrdsim_gb300.engine import Engine
    for sd in _systems():
        eng = Engine([sd])
        lib, h = eng.lib, eng.h
        ref = _pairs(lib, h, "rdsim_get_pairs")
        assert len(ref) > 0
        first = _pairs(lib, h, "rdsim_get_pairs_static")
        second = _pairs(lib, h, "rdsim_get_pairs_static")
        np.testing.assert_array_equal(first, ref)
        np.testing.assert_array_equal(second, ref)
        # the static array keeps the previous call's contents: after the
        # state moves, the static call must follow the allocating one again
        eng.step(10)
        x, t = eng.state()
        eng.set_state(x, t)
        ref2 = _pairs(lib, h, "rdsim_get_pairs")
        np.testing.assert_array_equal(_pairs(lib, h, "rdsim_get_pairs_static"), ref2)
        eng.close()


def test_static_pairs_capacity_errors():
    from pyrdsim_gb300.engine import Engine
    sd = next(_systems())
    eng = Engine([sd])
    n = C.c_int64()
    buf = np.empty((1, 2), dtype=np.int32)
    rc = eng.lib.rdsim_get_pairs_static(eng.h, 0, buf.ctypes.data_as(C.POINTER(C.c_int32)),
                                        1, C.byref(n))
    assert rc == 20 and n.value > 1
    assert eng.lib.rdsim_get_pairs_static(eng.h, 5, None, 0, C.byref(n)) == 1
    eng.close()


def test_static_pairs_with_device_memory_full():
    """The motivating caller: a process whose device memory is already
    committed (here: one tensor holding all but 2-4 MiB of the free
    memory).  The allocating entry point then fails with RDSIM_ERR_NOMEM,
    while the static one still returns its pairs: it allocated nothing."""
    import torch
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.engine import Engine
    sd = workloads.active_wall_fluid(n=40000, seed=9)
    eng = Engine([sd])
    lib, h = eng.lib, eng.h
    ref = _pairs(lib, h, "rdsim_get_pairs")
    need = 8 * len(ref)                     # bytes rdsim_get_pairs allocates
    assert need > (4 << 20), need
    _pairs(lib, h, "rdsim_get_pairs_static")  # set-up call
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free, _ = torch.cuda.mem_get_info()
    block = 2 << 20
    # leaves between 2 and 4 MiB free: less than rdsim_get_pairs needs
    hog = torch.empty(max(0, (free - (2 << 20)) // block * block), dtype=torch.uint8,
                      device="cuda")
    try:
        left, _ = torch.cuda.mem_get_info()
        assert left < need, (left, need)
        got = _pairs(lib, h, "rdsim_get_pairs_static")
        n = C.c_int64()
        buf = np.empty((len(ref), 2), dtype=np.int32)
        rc = lib.rdsim_get_pairs(h, 0, buf.ctypes.data_as(C.POINTER(C.c_int32)), len(ref),
                                 C.byref(n))
        assert rc == 3, rc  # RDSIM_ERR_NOMEM: the allocating call cannot run
        again = _pairs(lib, h, "rdsim_get_pairs_static")
    finally:
        del hog
        torch.cuda.empty_cache()
    np.testing.assert_array_equal(got, ref)
    np.testing.assert_array_equal(again, ref)
    eng.close()
