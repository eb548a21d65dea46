"""The learned surrogate on the GPU against its CPU restatement (oracle/surrogate_ref.py),
its training, and delayed-acceptance moves: exact running energies, the same ensemble
as plain moves, and what the trained network saves over the method without it."""
import math
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import surrogate_ref as S  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def melted():
    from sc_gb300 import System, workloads

    s = System.from_text(*workloads.psc_cpsc(2000, phi=0.2, seed=7))
    s.simulate(nsweeps=300, seed=1, check_every=0)
    yield s
    s.close()


def near_pairs(s, cut=4.5, limit=40000):
    parts = s.particles()
    pos = np.array([p.pos for p in parts])
    box = s.box
    d = pos[:, None, :] - pos[None, :, :]
    d = (d - np.rint(d)) * box
    r2 = (d * d).sum(-1)
    I, J = np.nonzero((r2 < cut * cut) & ~np.eye(len(parts), dtype=bool))
    return I[:limit].astype(np.int32), J[:limit].astype(np.int32)


def oracle_features(s, I, J):
    parts = s.particles()
    box32 = s.box.astype(np.float32)
    pos = np.array([p.pos for p in parts])
    dirs = np.array([p.dir for p in parts]).astype(np.float32)
    pd0 = np.array([p.patchdir[0] for p in parts]).astype(np.float32)
    types = np.array([p.type for p in parts])
    used = sorted(set(types.tolist()))
    compact = np.array([used.index(t) for t in types])
    nt = len(used)
    tc = (compact.astype(np.float32) / np.float32(max(1, nt - 1))).astype(np.float32) if nt > 1 else np.zeros(len(parts), np.float32)
    pp = {(a, b): s.pair_param(used[a], used[b]) for a in range(nt) for b in range(nt)}
    h1 = np.array([pp[(compact[i], compact[j])].half_len[0] for i, j in zip(I, J)], np.float32)
    h2 = np.array([pp[(compact[i], compact[j])].half_len[1] for i, j in zip(I, J)], np.float32)
    c = S.frac32(pos)
    r = S.pair_vec(c[I], c[J], box32)
    f, d2 = S.pair_features(r, dirs[I], pd0[I], h1, tc[I], dirs[J], pd0[J], h2, tc[J])
    rcut_s = max(p.rcut for p in pp.values())
    elig = d2 < np.float32(rcut_s) ** 2
    w = np.array([S.wca32(d2[k], pp[(compact[i], compact[j])].sigma, pp[(compact[i], compact[j])].epsilon,
                          pp[(compact[i], compact[j])].rcutwcaSq) for k, (i, j) in enumerate(zip(I, J))], np.float32)
    return f, elig, np.where(elig, w, np.float32(0.0))


def test_features_bit_exact_against_cpu_restatement(melted):
    I, J = near_pairs(melted)
    X, W, E = melted.pair_features(I, J)
    F, elig, w = oracle_features(melted, I, J)
    assert len(I) > 5000 and elig.sum() > 1000
    np.testing.assert_array_equal(X, F)
    np.testing.assert_array_equal(E, elig)
    np.testing.assert_array_equal(W, w)


def test_predict_matches_cpu_forward(melted):
    from sc_gb300 import Surrogate

    sur = Surrogate(melted, seed=3)
    I, J = near_pairs(melted, limit=3000)
    X, _, _ = melted.pair_features(I, J)
    y = sur.predict(X)
    yo, _ = S.forward(sur.weights, X, emulate=True)
    err = np.abs(y - yo)
    assert err.max() <= 2e-2 * (1.0 + np.abs(yo).max()), err.max()
    assert err.mean() <= 2e-3 * (1.0 + np.abs(yo).mean())
    sur.close()


@pytest.mark.parametrize("n", [64, 500])
def test_gradient_matches_cpu_backward(melted, n):
    from sc_gb300 import Surrogate

    sur = Surrogate(melted, seed=5)
    rng = np.random.default_rng(n)
    I, J = near_pairs(melted, limit=20000)
    pick = rng.choice(len(I), n, replace=False)
    X, _, _ = melted.pair_features(I[pick], J[pick])
    t = rng.normal(scale=0.4, size=n).astype(np.float32)
    g, loss = sur.gradient(X, t)
    go, lo = S.backward(sur.weights, X, t, emulate=True)
    assert abs(loss - lo) <= 1e-3 * lo
    blocks = [(S.OFF_W1, S.OFF_W2), (S.OFF_W2, S.OFF_B2), (S.OFF_B2, S.OFF_W3), (S.OFF_W3, S.OFF_B3),
              (S.OFF_B3, S.OFF_W4), (S.OFF_W4, S.OFF_B4), (S.OFF_B4, S.N_PARAMS)]
    for a, b in blocks:
        ga, gb = g[a:b].astype(np.float64), go[a:b]
        rel = np.linalg.norm(ga - gb) / max(np.linalg.norm(gb), 1e-30)
        assert rel <= 2e-2, (a, b, rel)
    assert np.linalg.norm(g - go) / np.linalg.norm(go) <= 1e-2
    sur.close()


@pytest.fixture(scope="module")
def trained(melted):
    from sc_gb300 import Surrogate

    sur = Surrogate(melted, seed=11, capacity=3_000_000)
    for k in range(20):
        melted.simulate(nsweeps=10, seed=100 + k, check_every=0)
        sur.collect(melted)
    st, losses = sur.train(epochs=30, batch=4096, lr=3e-3, warmup_steps=50, seed=2)
    yield sur, st, losses
    sur.close()


def test_training_reduces_the_error(melted, trained):
    sur, st, losses = trained
    assert st.samples > 100000
    assert st.loss_last < 0.3 * st.loss_first, (st.loss_first, st.loss_last)
    ev = sur.evaluate(melted)
    # error against the exact energies of a configuration it was not trained on
    melted.simulate(nsweeps=20, seed=999, check_every=0)
    ev2 = sur.evaluate(melted)
    assert ev2["pairs"] > 5000
    # the attraction the network learns spans [-1, 0]; predicting 0 leaves an rms error of
    # about 0.45 on these pairs
    assert ev2["rmse"] < 0.2 and ev2["rmse"] < 1.5 * ev["rmse"] + 0.02, (ev, ev2)


def test_delayed_acceptance_keeps_the_running_energy_exact(melted, trained):
    from sc_gb300 import ScError

    sur = trained[0]
    melted.set_surrogate(sur)
    st = melted.simulate(nsweeps=40, seed=9, check_every=20, delayed=1)
    assert st.da_stage1_rejected > 0 and st.da_stage2_tried > 0
    assert st.da_stage1_rejected + st.da_stage2_tried <= st.moves
    e1 = melted.all_to_all()
    assert abs(st.energy - e1) <= 1e-9 * max(1.0, abs(e1))
    assert abs(st.energy_check - e1) <= 1e-9 * max(1.0, abs(e1))
    melted.set_surrogate(None)
    with pytest.raises(ScError):
        melted.simulate(nsweeps=1, seed=9, delayed=1)


def exact_per_accepted(st):
    acc = st.acc_trans + st.acc_rot
    exact = st.da_stage2_tried if st.da_stage2_tried or st.da_stage1_rejected else st.moves
    return exact / max(1, acc)


def test_trained_network_saves_exact_evaluations(melted, trained):
    """Exact pair-energy passes per accepted move: plain moves evaluate every move exactly;
    delayed acceptance with the trained network only the moves its stage lets through,
    and more of those are then accepted than with the network zeroed (WCA32 alone)."""
    from sc_gb300 import Surrogate

    sur = trained[0]
    plain = melted.simulate(nsweeps=30, seed=21, check_every=0)
    melted.set_surrogate(sur)
    da = melted.simulate(nsweeps=30, seed=21, check_every=0, delayed=1)
    zero = Surrogate(melted, seed=1)
    w = np.zeros(Surrogate.N_PARAMS, np.float32)
    zero.weights = w
    melted.set_surrogate(zero)
    wca_only = melted.simulate(nsweeps=30, seed=21, check_every=0, delayed=1)
    melted.set_surrogate(None)
    zero.close()
    p, d, z = exact_per_accepted(plain), exact_per_accepted(da), exact_per_accepted(wca_only)
    acc2_d = 1 - da.da_stage2_rejected / da.da_stage2_tried
    acc2_z = 1 - wca_only.da_stage2_rejected / wca_only.da_stage2_tried
    report = dict(plain=p, trained=d, wca_only=z, stage2_acc_trained=acc2_d, stage2_acc_wca=acc2_z,
                  err_rms=da.da_err_rms)
    assert d < 0.8 * p, report
    assert d < z and acc2_d > acc2_z, report
    assert acc2_d > 0.8, report


def _series(systems, sur, delayed, nsweeps, burn, every, seed):
    from sc_gb300 import ReplicaSet

    for s in systems:
        s.set_surrogate(sur if delayed else None)
    R = ReplicaSet(systems, [1.0] * len(systems), ladder=list(range(len(systems))))
    p = systems[0].default_run()
    p.check_every = 0
    p.delayed = 1 if delayed else 0
    E = [[] for _ in systems]
    done = 0
    while done < nsweeps:
        _, _, en, _, _ = R.run(every, exchange_every=0, seed=seed, params=p)
        done += every
        if done > burn:
            for k, s in enumerate(systems):
                E[k].append(en[k] / s.n)
    R.close()
    return np.array([np.mean(x) for x in E])


def test_delayed_acceptance_samples_the_plain_ensemble(trained):
    """Six independent trajectories each way from the same start; mean energy per
    particle within 2 standard errors."""
    from sc_gb300 import System, workloads

    sur = trained[0]
    texts = workloads.psc_cpsc(500, phi=0.2, seed=17)
    A = [System.from_text(*texts) for _ in range(6)]
    B = [System.from_text(*texts) for _ in range(6)]
    ma = _series(A, sur, False, 3000, 1000, 20, seed=31)
    mb = _series(B, sur, True, 3000, 1000, 20, seed=37)
    se = math.sqrt(ma.var(ddof=1) / len(ma) + mb.var(ddof=1) / len(mb))
    assert abs(ma.mean() - mb.mean()) <= 2.0 * se + 1e-4, (ma.mean(), mb.mean(), se)
    for s in A + B:
        s.set_surrogate(None)
        s.close()
