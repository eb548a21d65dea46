"""Host-side particle passes split across threads (sc_gb300/csrc/host_parallel.h).

sc_set_particles, sc_get_particles and the state's packing into (and unpacking from) the
pinned staging block run their per-particle loops in contiguous chunks on several host
threads.  These CPU tests check that the split visits every record exactly once, for sizes
on both sides of the threshold where a range starts being split, and that the library's
record copies through it give back exactly what was set, on the 65,536-particle benchmark
system (no GPU is needed for these two calls while the device has not been used).
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from sc_gb300 import System, workloads
from sc_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = r"""
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <utility>
#include <vector>
#include "host_parallel.h"

int main(int argc, char** argv) {
    for (int a = 1; a < argc; ++a) {
        const int n = std::atoi(argv[a]);
        std::vector<int> hits(n > 0 ? n : 1, 0);
        std::mutex m;
        std::vector<std::pair<int, int>> chunks;
        scg::parallelRange(n, [&](int lo, int hi) {
            for (int i = lo; i < hi; ++i) hits[i] += 1;
            std::lock_guard<std::mutex> g(m);
            chunks.push_back({lo, hi});
        });
        long bad = 0;
        for (int i = 0; i < n; ++i) bad += hits[i] != 1;
        std::printf("%d %ld %zu %d\n", n, bad, chunks.size(), scg::hostThreads(n));
    }
    return 0;
}
"""


def test_parallel_range_visits_every_index_once(tmp_path):
    src = tmp_path / "harness.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "harness"
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", os.path.join(ROOT, "sc_gb300", "csrc"), str(src),
                    "-o", str(exe)], check=True)
    sizes = [0, 1, 8191, 8192, 8193, 16383, 16384, 16385, 24577, 65536, 100003, 1 << 20]
    out = subprocess.run([str(exe)] + [str(n) for n in sizes], check=True, capture_output=True, text=True).stdout
    rows = [list(map(int, l.split())) for l in out.splitlines()]
    assert [r[0] for r in rows] == sizes
    for n, bad, nchunks, nthreads in rows:
        assert bad == 0, (n, bad)
        # one chunk per thread; ranges below the threshold are not split
        assert nchunks == (0 if n == 0 else nthreads), (n, nchunks, nthreads)
        if n <= 8192:
            assert nthreads == 1


def _records(arr):
    return np.frombuffer((C.c_char * (C.sizeof(arr))).from_buffer(arr), dtype=np.uint8).copy()


@pytest.fixture(scope="module")
def big():
    s = System.from_text(*workloads.psc_cpsc(65536, phi=0.2, seed=1))
    yield s
    s.close()


def test_set_then_get_gives_back_every_record(big):
    s = big
    start = s.particles()
    assert len(start) == 65536
    rng = np.random.default_rng(3)
    mod = (L.Particle * s.n)()
    C.memmove(mod, start, C.sizeof(start))
    shift = rng.uniform(-0.01, 0.01, (s.n, 3))
    for k in range(0, s.n, 97):           # a scattered subset, in every chunk
        for d in range(3):
            mod[k].pos[d] += shift[k, d]
            mod[k].patchsides[k % 4][d] += 1e-3
    s.set_particles(0, mod)
    back = s.particles()
    assert np.array_equal(_records(back), _records(mod))
    # a sub-range starting inside a chunk
    sub = (L.Particle * 30000)()
    C.memmove(sub, C.byref(mod, C.sizeof(L.Particle) * 20001), C.sizeof(sub))
    for k in range(len(sub)):
        sub[k].dir[0] = -sub[k].dir[0]
    s.set_particles(20001, sub)
    got = s.particles(20001, 30000)
    assert np.array_equal(_records(got), _records(sub))
    whole = s.particles()
    assert np.array_equal(_records(whole)[: 20001 * C.sizeof(L.Particle)], _records(mod)[: 20001 * C.sizeof(L.Particle)])
    # the caller's buffer is filled in place
    out = (L.Particle * s.n)()
    assert s.particles(out=out) is out
    assert np.array_equal(_records(out), _records(whole))
    s.set_particles(0, start)


def test_a_refused_set_changes_nothing(big):
    s = big
    before = s.particles()
    bad = (L.Particle * s.n)()
    C.memmove(bad, before, C.sizeof(before))
    for k in range(s.n):
        bad[k].pos[0] += 0.5
    bad[40000].type = bad[40000].type + 1            # a type change is refused
    with pytest.raises(L.ScError):
        s.set_particles(0, bad)
    assert np.array_equal(_records(s.particles()), _records(before))
