"""The C-ABI library builds, loads without a GPU and exports every entry point declared in
include/oxgb.h; the ctypes table covers the same set."""
import ctypes
import os
import re

from conftest import REPO

HEADER = os.path.join(REPO, "include", "oxgb.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(oxgb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from oxdna_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    names = declared()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_table_matches_header():
    from oxdna_gb300 import _abi
    assert sorted(_abi.SIGNATURES) == declared()


def test_version_and_defaults_need_no_gpu():
    import oxdna_gb300 as ox
    L = ox.lib()
    assert L.oxgb_version().startswith(b"oxgb")
    s = ox.dna2_settings(0.1, 0.5)
    assert s.average == 1 and s.dh_half_charged_ends == 1 and abs(s.dh_lambda - 0.3616455) < 1e-12
    m = ox.md_settings(thermostat="bussi")
    assert m.thermostat == 2 and m.steps_per_graph == 16


def test_noalloc_limits_match_header():
    import re

    from oxdna_gb300 import _abi
    text = open(HEADER).read()
    assert int(re.search(r"#define OXGB_NOALLOC_MAX_N (\d+)", text).group(1)) == _abi.NOALLOC_MAX_N
    assert int(re.search(r"#define OXGB_NOALLOC_MAX_CELLS (\d+)", text).group(1)) == _abi.NOALLOC_MAX_CELLS
