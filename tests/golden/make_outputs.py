#!/usr/bin/env python3
"""Output-file goldens: the reference's own energy.dat, stat.dat, movie and config.last.

Runs the reference binary built from its own sources (oracle/_ref/sc_ref, see
oracle/Makefile) for two sweeps on systems whose moves change nothing (zero displacement
and rotation steps: every proposal is the identity), reporting and writing a movie frame
every sweep, and stores the inputs and the files it wrote as tests/golden/ref_outputs.json.
The GPU output loop (sc_gb300/updater.py) must write the same files for the same state.

Run here (needs the reference tree): python tests/golden/make_outputs.py
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))
import goldens  # noqa: E402
import oracle_ffi as O  # noqa: E402

SC_REF = os.path.join(REPO, "oracle", "_ref", "sc_ref")
CASES = ["ref_test_01_normal_PSC", "ref_test_12_normal_SPA_CPSC", "ref_test_20_chain_bond12"]
OVERRIDE = dict(nsweeps="2", report="1", movie="1", transmx="0.0", rotmx="0.0", chainmmx="0.0", chainrmx="0.0",
                nequil="0", adjust="0", shave="0", edge_mx="0.0", pairlist_update="0", paramfrq="0",
                write_cluster="0", nrepchange="0")


def run(case):
    inp = goldens.load(case)["inputs"]
    opts = O.parse_options(inp["options"])
    opts.update(OVERRIDE)
    otext = "".join(f"{k} = {v}\n" for k, v in opts.items())
    with tempfile.TemporaryDirectory() as tmp:
        for name, text in (("options", otext), ("top.init", inp["top.init"]), ("config.init", inp["config.init"])):
            with open(os.path.join(tmp, name), "w") as f:
                f.write(text)
        subprocess.run([SC_REF], cwd=tmp, check=True, capture_output=True)
        files = {k: open(os.path.join(tmp, k)).read() for k in ("energy.dat", "stat.dat", "movie", "config.last")}
    return {"inputs": {"options": otext, "top.init": inp["top.init"], "config.init": inp["config.init"]},
            "files": files}


def main():
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "ref", "-j8"], check=True, capture_output=True)
    out = {c: run(c) for c in CASES}
    with open(os.path.join(HERE, "ref_outputs.json"), "w") as f:
        json.dump(out, f, indent=0)
    for c, v in out.items():
        print(c, {k: len(t) for k, t in v["files"].items()})


if __name__ == "__main__":
    main()
