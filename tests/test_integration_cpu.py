"""The reference-side binding shown in INTEGRATION.md compiles against the reference's
own headers.

The C++ block under "C++ binding a maintainer would add to scOOP" is a TotalE subclass
(scOOP/mc/totalenergycalculator.h:136-297) that forwards to include/sc_gb300.h; it is
extracted from the document, instantiated for the reference's PairE and compiled with
g++ -fsyntax-only against the reference tree (SC_REFERENCE, else the location the oracle
recipe resolves).  Skipped when the reference tree is absent.
"""
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _scoop():
    env = os.environ.get("SC_REFERENCE")
    if env:
        return os.path.join(env, "scOOP")
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "print-ref"], capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


def _binding():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = text.split("## C++ binding a maintainer would add to scOOP", 1)[1]
    m = re.search(r"```cpp\n(.*?)```", sec, re.S)
    return m.group(1)


def test_binding_covers_every_particle_vector():
    code = _binding()
    for field in ("pos", "dir", "patchdir[k]", "chdir[k]", "patchsides[k]", "type", "molType"):
        assert f"q.{field}" in code, field
    assert "/*" not in code.split("void push()")[1].split("}\n")[0]


@pytest.mark.skipif(not os.path.isdir(_scoop()), reason="the reference tree is absent")
def test_binding_compiles_against_reference_headers():
    scoop = _scoop()
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "binding.cpp")
        with open(src, "w") as f:
            f.write(_binding())
            f.write("\ntemplate class TotalEGpu<PairE>;\n")
        r = subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-w", "-I", os.path.join(scoop, "mc"), "-I",
                            scoop, "-I", os.path.join(ROOT, "include"), src], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
