"""Replicas moved together: batching must not change any trajectory, and the
parallel-tempering exchange keeps every ladder a permutation of its temperatures."""
import numpy as np
import pytest

from test_gpu_sweep import ens, opts_text

pytestmark = pytest.mark.gpu
GOLDEN = 0x9E3779B97F4A7C15


def open_systems(name, k):
    from sc_gb300 import System

    e = ens(name)
    return [System.from_text(opts_text(e["options"]), e["inputs"]["top.init"], e["inputs"]["config.init"])
            for _ in range(k)]


def test_batched_replicas_reproduce_single_runs():
    from sc_gb300 import ReplicaSet

    sysA = open_systems("psc_nvt", 3)
    sysB = open_systems("psc_nvt", 3)
    temps = [0.6, 0.8, 1.1]
    R = ReplicaSet(sysA, temps, ladder=[0, 1, 2])
    st, T, E, _, _ = R.run(40, exchange_every=0, seed=77, stencil=2)
    assert list(T) == temps
    for k, s in enumerate(sysB):
        single = s.simulate(nsweeps=40, seed=(77 + GOLDEN * (k + 1)) % (1 << 64), temper=temps[k], stencil=2,
                            check_every=0)
        assert single.energy == E[k]
        pa, pb = sysA[k].particles(), s.particles()
        assert all(list(x.pos) == list(y.pos) and list(x.dir) == list(y.dir) for x, y in zip(pa, pb))
    assert st.moves == 3 * 40 * sysA[0].n
    R.close()


def test_exchanges_keep_ladders_and_energies():
    from sc_gb300 import ReplicaSet

    sys8 = open_systems("psc_nvt", 8)
    # neighbouring temperatures close enough that swaps of 250-particle replicas get accepted
    temps = list(np.geomspace(0.9, 1.0, 4)) * 2
    ladder = [0] * 4 + [1] * 4
    R = ReplicaSet(sys8, temps, ladder=ladder)
    st, T, E, tried, acc = R.run(400, exchange_every=20, seed=5)
    for g in (0, 1):
        assert sorted(T[4 * g: 4 * g + 4]) == pytest.approx(sorted(temps[4 * g: 4 * g + 4]))
    assert tried.sum() > 0 and acc.sum() > 0
    for k, s in enumerate(sys8):
        exact = s.all_to_all()
        assert abs(E[k] - exact) <= 1e-9 * max(1.0, abs(exact))
    R.close()


def test_uneven_sizes_in_one_batch():
    from sc_gb300 import ReplicaSet, System, workloads

    systems = [System.from_text(*workloads.nvt_psc(n, phi=0.15, seed=3 + n)) for n in (120, 400, 260)]
    R = ReplicaSet(systems, [1.0, 1.0, 1.0], ladder=[0, 1, 2])
    st, T, E, _, _ = R.run(30, exchange_every=0, seed=9)
    assert st.moves == 30 * sum(s.n for s in systems)
    for k, s in enumerate(systems):
        exact = s.all_to_all()
        assert abs(E[k] - exact) <= 1e-9 * max(1.0, abs(exact))
    R.close()


def test_dataflow_sweep_in_a_batch_of_uneven_systems():
    """The dataflow launch over a batch: each system takes its cells from its own ticket
    counter; trajectories equal those of the colour-phase launches."""
    from sc_gb300 import ReplicaSet, System, workloads

    def batch(variant):
        systems = [System.from_text(*workloads.nvt_psc(n, phi=0.15, seed=3 + n)) for n in (120, 400, 260)]
        R = ReplicaSet(systems, [1.0, 0.9, 1.1], ladder=[0, 1, 2])
        st, T, E, _, _ = R.run(30, exchange_every=10, seed=19, variant=variant)
        R.close()
        return systems, st, T, E

    sa, a, Ta, Ea = batch(0)
    sb, b, Tb, Eb = batch(4)
    assert list(Ea) == list(Eb) and list(Ta) == list(Tb)
    assert a.acc_trans == b.acc_trans and a.acc_rot == b.acc_rot
    for x, y in zip(sa, sb):
        assert all(list(p.pos) == list(q.pos) for p, q in zip(x.particles(), y.particles()))
        exact = y.all_to_all()
        assert abs(Eb[sb.index(y)] - exact) <= 1e-9 * max(1.0, abs(exact))
    for s in sa + sb:
        s.close()


# --- the exchange decision against a restatement of the reference's rule -------------------
_M = 0xFFFFFFFF


def _philox(c, k0, k1):
    """Philox4x32-10 (Salmon et al., SC'11), as the kernels' counter-based stream uses it."""
    x, y, z, w = c
    for _ in range(10):
        p0, p1 = 0xD2511F53 * x, 0xCD9E8D57 * z
        x, y, z, w = ((p1 >> 32) ^ y ^ k0) & _M, p1 & _M, ((p0 >> 32) ^ w ^ k1) & _M, p0 & _M
        k0, k1 = (k0 + 0x9E3779B9) & _M, (k1 + 0xBB67AE85) & _M
    return x, y, z, w


def _uniforms(seed, a, b, c):
    """The uniforms of one (stream id, event) Philox stream, two per block."""
    k0, k1 = seed & _M, (seed >> 32) & _M
    w = 0
    while True:
        r = _philox((a, b, c, w), k0, k1)
        w += 1
        for hi, lo in ((r[0], r[1]), (r[2], r[3])):
            yield (((hi << 21) ^ (lo >> 11)) & ((1 << 53) - 1)) / 9007199254740992.0


def test_philox_known_answers():
    """The restatement reproduces Random123's published Philox4x32-10 vectors."""
    assert _philox((0, 0, 0, 0), 0, 0) == (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)
    assert _philox((_M, _M, _M, _M), _M, _M) == (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)


def test_exchange_decisions_follow_the_reference_rule():
    """Every exchange decision of the device step equals the one the reference's rule takes
    (MoveCreator::replicaExchangeMove, movecreator.cpp:713-745: accept when
    change = (1/T_i - 1/T_j)(E_i - E_j) + (P_i/T_i - P_j/T_j)(V_i - V_j) > 0 or a uniform is
    below exp(change)), restated here on the energies, temperatures and the uniforms of the
    exchange's own random stream: even and odd neighbour pairs alternate, each ladder ordered
    by temperature."""
    import math

    from sc_gb300 import ReplicaSet

    reps = open_systems("psc_nvt", 4)
    temps = list(np.geomspace(0.9, 1.0, 4))
    R = ReplicaSet(reps, temps, ladder=[0] * 4)
    seed = 31
    ex_seed = seed ^ 0xA5A5A5A5
    T = np.array(temps)
    decided = accepted = 0
    for ev in range(40):
        st, T_after, E, tried, acc = R.run(2, exchange_every=2, seed=seed)
        ladder = list(np.argsort(T, kind="stable"))
        want = T.copy()
        u = _uniforms(ex_seed, 0xFFFFFFE0, ev & _M, ev >> 32)
        for k in range(ev & 1, len(ladder) - 1, 2):
            ri, rj = ladder[k], ladder[k + 1]
            change = (1.0 / T[ri] - 1.0 / T[rj]) * (E[ri] - E[rj])     # NVT: equal volumes, no pressure term
            x = next(u)
            if change >= 0.0 or math.exp(change) > x:
                want[ri], want[rj] = T[rj], T[ri]
                accepted += 1
            decided += 1
        assert np.array_equal(T_after, want), (ev, T, T_after, want, E)
        assert int(tried.sum()) == decided and int(acc.sum()) == accepted
        T = T_after
    assert 0 < accepted < decided
    R.close()
