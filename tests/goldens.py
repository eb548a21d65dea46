"""Loader for the golden vectors under tests/golden (made by tests/golden/make_golden.py)."""
import glob
import gzip
import json
import os

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[: -len(".json.gz")] for p in glob.glob(os.path.join(GOLDEN, "*.json.gz")))


_cache = {}


def load(name):
    if name not in _cache:
        with gzip.open(os.path.join(GOLDEN, name + ".json.gz"), "rt") as f:
            _cache[name] = json.load(f)
    return _cache[name]


def write_inputs(g, directory):
    """Write the golden's options / top.init / config.init into a directory."""
    for fn, txt in g["inputs"].items():
        with open(os.path.join(directory, fn), "w", encoding="latin-1") as f:
            f.write(txt)
