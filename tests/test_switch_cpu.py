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
