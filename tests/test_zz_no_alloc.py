"""The no-allocation variant of the one-particle energy call.

sc_one_to_all_noalloc serves callers that must not allocate device memory (another
allocator holds the free memory, or a cudaMalloc would stall a latency-critical
loop); it stages its data in a fixed array inside the library.  Here it is called
through the C ABI twice in a row and must give the same energies as sc_one_to_all
within the parity tolerance.  The file name keeps it last in the collection order.
"""
import ctypes as C

import numpy as np
import pytest

import goldens

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_call_twice():
    from sc_gb300 import ScError, System
    from sc_gb300 import _lib as L

    g = goldens.load("syn_cpsc_spa_npt_small")
    inp = g["inputs"]
    s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
    lib = L.load()
    targets = np.arange(s.n, dtype=np.int32)
    # before any allocating call the state is not on the device: refused, nothing allocated
    out = np.zeros(s.n)
    rc = lib.sc_one_to_all_noalloc(s._h, s.n, targets.ctypes.data_as(C.POINTER(C.c_int)),
                                   out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == -6
    want = s.one_to_all(targets)          # allocating entry point, puts the state on the GPU
    scale = max(1.0, float(np.abs(want).max()))
    for call in range(2):
        out = np.full(s.n, np.nan)
        L.check(lib.sc_one_to_all_noalloc(s._h, s.n, targets.ctypes.data_as(C.POINTER(C.c_int)),
                                          out.ctypes.data_as(C.POINTER(C.c_double))))
        assert np.all(np.abs(out - want) <= 1e-12 * scale), call
    # a different subset in a second round reuses the same array
    sub = targets[::3].copy()
    out = np.zeros(len(sub))
    L.check(lib.sc_one_to_all_noalloc(s._h, len(sub), sub.ctypes.data_as(C.POINTER(C.c_int)),
                                      out.ctypes.data_as(C.POINTER(C.c_double))))
    assert np.all(np.abs(out - want[::3]) <= 1e-12 * scale)
    # sizes beyond the array are refused
    big = np.zeros(16385, dtype=np.int32)
    out = np.zeros(16385)
    with pytest.raises(ScError) as ei:
        L.check(lib.sc_one_to_all_noalloc(s._h, 16385, big.ctypes.data_as(C.POINTER(C.c_int)),
                                          out.ctypes.data_as(C.POINTER(C.c_double))))
    assert "RANGE" in str(ei.value)
    s.close()


def _noalloc(lib, s, targets):
    out = np.full(len(targets), np.nan)
    rc = lib.sc_one_to_all_noalloc(s._h, len(targets), targets.ctypes.data_as(C.POINTER(C.c_int)),
                                   out.ctypes.data_as(C.POINTER(C.c_double)))
    return rc, out


def test_noalloc_refuses_a_host_edit_until_an_allocating_call():
    """A particle changed through the API lives only on the host until an allocating call
    uploads it: the no-alloc call refuses (it would read the old device copy), and after
    sc_one_to_all it gives that call's energies of the edited state."""
    from sc_gb300 import System
    from sc_gb300 import _lib as L

    g = goldens.load("syn_cpsc_spa_npt_small")
    inp = g["inputs"]
    s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
    lib = L.load()
    targets = np.arange(s.n, dtype=np.int32)
    s.one_to_all(targets)
    p = s.particles(5, 1)
    p[0].pos[0] += 0.01
    s.set_particles(5, p)
    rc, _ = _noalloc(lib, s, targets)
    assert rc == -6
    want = s.one_to_all(targets)
    scale = max(1.0, float(np.abs(want).max()))
    rc, out = _noalloc(lib, s, targets)
    assert rc == 0
    assert np.all(np.abs(out - want) <= 1e-12 * scale)
    s.close()


def test_noalloc_after_sweeps_reads_the_moved_state():
    """After device sweeps the device copy is the newer one: the no-alloc energies are those
    of the moved configuration, equal to sc_one_to_all's on the same state, twice in a row."""
    from sc_gb300 import System
    from sc_gb300 import _lib as L

    g = goldens.load("syn_cpsc_spa_npt_small")
    inp = g["inputs"]
    s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
    lib = L.load()
    targets = np.arange(s.n, dtype=np.int32)
    before = s.one_to_all(targets)
    st = s.simulate(nsweeps=5, seed=3, check_every=0)
    assert st.acc_trans + st.acc_rot > 0
    first = _noalloc(lib, s, targets)
    second = _noalloc(lib, s, targets)
    want = s.one_to_all(targets)
    scale = max(1.0, float(np.abs(want).max()))
    for rc, out in (first, second):
        assert rc == 0
        assert np.all(np.abs(out - want) <= 1e-12 * scale)
    assert np.any(np.abs(want - before) > 1e-9)
    s.close()
