"""The product never reaches into the oracle: no module of the package imports it and no
library source includes or loads it (the oracle is test infrastructure only)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _files(top, exts):
    for d, _, fs in os.walk(os.path.join(ROOT, top)):
        if "__pycache__" in d or "_build" in d:
            continue
        for f in fs:
            if f.endswith(exts):
                yield os.path.join(d, f)


def test_package_does_not_import_the_oracle():
    bad = []
    for f in _files("votca_gb300", (".py",)):
        src = open(f).read()
        if re.search(r"^\s*(import\s+oracle|from\s+oracle\b)", src, flags=re.M):
            bad.append(f)
    assert not bad, bad


def test_library_sources_do_not_reference_the_oracle():
    bad = []
    for f in list(_files("votca_gb300/csrc", (".cu", ".cuh", ".cpp", ".hpp", ".h"))) + \
            list(_files("include", (".h",))):
        if re.search(r"oracle|bse_oracle", open(f).read()):
            bad.append(f)
    assert not bad, bad


def test_no_batched_memcpy_calls():
    """The batched memcpy entry points are closed on the GPU pool this library is tested on: no
    source names them (the names are assembled here so that this file does not)."""
    names = [p + "Memcpy" + d + "BatchAsync" for p in ("cuda", "cu") for d in ("", "3D")]
    bad = []
    for top in ("votca_gb300", "include", "oracle", "tests"):
        for f in _files(top, (".py", ".cu", ".cuh", ".cpp", ".hpp", ".h", ".c")):
            src = open(f, errors="ignore").read()
            if any(n in src for n in names):
                bad.append(f)
    for f in ("bench.py", "__graft_entry__.py"):
        if any(n in open(os.path.join(ROOT, f)).read() for n in names):
            bad.append(f)
    assert not bad, bad
