"""Grand-canonical input handling on the host (no GPU): ACTIVITY and nGrandCanon as the
reference reads them (inicializer.cpp:36-47, 1087-1096; main.cpp:104-108, 128-139), the
species records, the inputs the GPU path refuses, and top.last (main.cpp:313-331)."""
import json
import math
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


def _case(name):
    with open(os.path.join(GOLDEN, f"ens_{name}.json")) as f:
        g = json.load(f)
    from golden.make_golden import OPTION_KEYS

    o = dict(OPTION_KEYS)
    o.update(g["options"])
    o["paraltemper"] = o["temper"]
    return "".join(f"{k} = {v}\n" for k, v in o.items()), g["inputs"]["top.init"], g["inputs"]["config.init"]


def test_species_records(lib):
    from sc_gb300 import System

    opts, top, cfg = _case("gc_psc")
    s = System.from_text(opts, top, cfg)
    (g,) = s.grand_stats()
    assert g.mol_type == 1 and g.type == 1 and g.count == 15
    assert g.activity == 0.02
    assert g.chem_pot == pytest.approx(math.log(0.02 * 6.022137e23 * 1e-24), rel=1e-15)
    assert g.steps == 0 and g.average_particles == 0.0
    assert s.default_run().grand_every == 1
    s.close()


def test_activity_needs_ngrandcanon_and_back(lib):
    from sc_gb300 import ScError, System

    opts, top, cfg = _case("gc_spa")
    with pytest.raises(ScError) as ei:
        System.from_text(opts.replace("nGrandCanon = 1", "nGrandCanon = 0"), top, cfg)
    assert "Activity stated in top.init, But nGrandCanon=0 in options" in str(ei.value)
    with pytest.raises(ScError) as ei:
        System.from_text(opts, top.replace("ACTIVITY: 0.1\n", ""), cfg)
    assert "no activity set for any species" in str(ei.value)


def test_refused_species_layouts(lib):
    """Chains come from a [Pool] (outside the GPU path); single particles only from the first
    grand-canonical species on (an insertion or removal moves the particles behind it)."""
    from golden.make_golden import options_text, top_text
    from sc_gb300 import ScError, System

    types = [("A", 1, "SPA", [1.0, 1.0, 1.1225, 0.5])]
    cfg = "10 10 10\n" + "".join(f"{1.0 + 2 * k} 1 1 0 0 1 1 0 0 0\n" for k in range(4))
    opts = options_text(nGrandCanon=1)
    chain = top_text(types, [("C", [1, 1], ["bond1: 10 1.0", "ACTIVITY: 0.1"])], [("C", 2)])
    with pytest.raises(ScError) as ei:
        System.from_text(opts, chain, cfg)
    assert ei.value.code == -7 and "Pool" in str(ei.value)
    behind = top_text(types, [("G", [1], ["ACTIVITY: 0.1"]), ("C", [1, 1], ["bond1: 10 1.0"])], [("G", 2), ("C", 1)])
    with pytest.raises(ScError) as ei:
        System.from_text(opts, behind, cfg)
    assert ei.value.code == -7 and "last" in str(ei.value)
    ok = top_text(types, [("C", [1, 1], ["bond1: 10 1.0"]), ("G", [1], ["ACTIVITY: 0.1"])], [("C", 1), ("G", 2)])
    s = System.from_text(opts, ok, cfg)
    assert [g.mol_type for g in s.grand_stats()] == [1]
    s.close()


def test_empty_box_opens(lib):
    from golden.make_golden import options_text, top_text
    from sc_gb300 import System

    top = top_text([("A", 1, "SPA", [1.0, 1.0, 1.1225, 0.5])], [("A", [1], ["ACTIVITY: 0.1"])], [("A", 0)])
    s = System.from_text(options_text(nGrandCanon=2), top, "8 8 8\n")
    assert s.n == 0 and s.grand_stats()[0].count == 0
    s.close()


def test_top_last(lib, tmp_path):
    from sc_gb300 import System

    opts, top, cfg = _case("gc_psc")
    s = System.from_text(opts, top, cfg)
    path = tmp_path / "top.last"
    s.write_top_last(path)
    text = path.read_text()
    head, tail = top.split("[System]\n")
    assert text == head + "[System]\nA 20\nP 15\n"
    s.close()
