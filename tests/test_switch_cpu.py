"""Type-switch input handling on the host (no GPU): "particles: TYPE SWITCHTYPE DELTA_MU"
(inicializer.cpp:955-985), switched particles in config.init taking their switch type
(inicializer.cpp:226-236), and the run's switchprob (initSwitchList, inicializer.cpp:60-87)."""
import json
import os

import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def lib():
    from sc_gb300 import _lib

    try:
        return _lib.load()
    except Exception as e:  # the library is built by __graft_entry__.build()
        pytest.skip(f"library not built: {e}")


def _case():
    with open(os.path.join(GOLDEN, "ens_switch_psc.json")) as f:
        g = json.load(f)
    from golden.make_golden import OPTION_KEYS

    o = dict(OPTION_KEYS)
    o.update(g["options"])
    o["paraltemper"] = o["temper"]
    return "".join(f"{k} = {v}\n" for k, v in o.items()), g["inputs"]["top.init"], g["inputs"]["config.init"]


def test_switch_types_parse(lib):
    from sc_gb300 import System

    opts, top, cfg = _case()
    s = System.from_text(opts, top, cfg)
    assert s.default_run().switchprob == 0.1
    parts = s.particles()
    assert all(p.type == 1 for p in parts[:150]) and all(p.type == 3 for p in parts[150:])
    s.close()
    # no switchable particle: no switch moves, as initSwitchList sets switchprob to 0
    s = System.from_text(opts, top.replace("particles: 1 2 1.6", "particles: 1"), cfg)
    assert s.default_run().switchprob == 0.0
    s.close()


def test_switched_particles_take_their_switch_type(lib, tmp_path):
    from sc_gb300 import ScError, System

    opts, top, cfg = _case()
    lines = cfg.splitlines()
    lines[1] = lines[1].rsplit(" ", 1)[0] + " 1"          # particle 1 (a P) switched
    s = System.from_text(opts, top, "\n".join(lines) + "\n")
    parts = s.particles()
    assert parts[0].type == 2 and parts[1].type == 1
    s.write_config(str(tmp_path / "c"))
    row = (tmp_path / "c").read_text().splitlines()[1].split()
    assert row[9] == "1" and row[10] == "0"
    s.close()
    lines = cfg.splitlines()
    lines[-1] = lines[-1].rsplit(" ", 1)[0] + " 1"        # a sphere (no switch type) switched
    with pytest.raises(ScError) as ei:
        System.from_text(opts, top, "\n".join(lines) + "\n")
    assert "no switchtype" in str(ei.value)


def test_particle_line_needs_one_or_three_fields(lib):
    from sc_gb300 import ScError, System

    opts, top, cfg = _case()
    with pytest.raises(ScError) as ei:
        System.from_text(opts, top.replace("particles: 1 2 1.6", "particles: 1 2"), cfg)
    assert "could not read a particle" in str(ei.value)
    with pytest.raises(ScError):
        System.from_text(opts, top.replace("particles: 1 2 1.6", "particles: 1 7 1.6"), cfg)


def test_oracle_switch_of_a_lone_particle_follows_delta_mu():
    """The oracle's restatement of switchTypeMove on one PSC alone in a box: with no partner
    the switched fraction is exp(-dmu/T) / (1 + exp(-dmu/T)), dmu read as the reference's int
    (1.7 acts as 1)."""
    import math

    import numpy as np

    import oracle_ffi as O
    from golden.make_golden import options_text, top_text

    top = top_text([("P", 1, "PSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, 3.0, 0.0]),
                    ("C", 2, "CPSC", [1.0, 1.0, 1.12, 0.2, 120.0, 10.0, 3.0, 0.0])],
                   [("M", ["1 2 1.7"], [])], [("M", 1)])
    ts = O.TextSystem(options_text(switchprob=0.5, transmx=0.2, rotmx=10.0), top, "20 20 20\n1 1 1 0 0 1 1 0 0 0\n")
    run = O.McRun(ts, seed=5)
    frac = []
    for _ in range(400):
        st = run.advance(500)
        frac.append(ts.switched[0])
    run.close()
    want = math.exp(-1.0) / (1.0 + math.exp(-1.0))
    assert st.acc_switch > 1000 and st.rej_switch > 1000
    assert abs(np.mean(frac) - want) < 0.06, (np.mean(frac), want)
    # every accepted switch flipped the type and the flag together
    assert (ts.parts[0].type == 2) == (ts.switched[0] == 1)


def test_oracle_switching_samples_the_reference_ensemble():
    """The oracle's switch moves on the switching golden's system (150 PSC <-> CPSC with
    delta_mu 1.6, 50 spheres): the switched fraction and the energy per particle of four
    short oracle runs agree with the reference's own twelve long runs within 3 combined
    standard errors."""
    import math

    import numpy as np

    import oracle_ffi as O

    opts, top, cfg = _case()
    with open(os.path.join(GOLDEN, "ens_switch_psc.json")) as f:
        g = json.load(f)
    F, E = [], []
    for seed in (11, 12, 13, 14):
        ts = O.TextSystem(opts, top, cfg)
        run = O.McRun(ts, seed=seed, fast=True)
        f_ser, e_ser = [], []
        for k in range(150):                  # 3000 sweeps, samples every 20 after 600
            st = run.advance(20 * ts.sys.n)
            if k >= 30:
                f_ser.append(sum(ts.switched[i] for i in range(150)) / 150.0)
                e_ser.append(st.energy / ts.sys.n)
        run.close()
        F.append(np.mean(f_ser))
        E.append(np.mean(e_ser))
    for key, got in (("switched_fraction", F), ("energy_per_particle", E)):
        ref = g["stats"][key]
        se = math.sqrt(np.var(got, ddof=1) / len(got) + ref["se"] ** 2)
        assert abs(np.mean(got) - ref["mean"]) <= 3.0 * se, (key, np.mean(got), ref)
