"""The reference-side plugin (oxdna_gb300/shim) compiles against the reference's own headers and
exports the entry points the reference's plugin manager looks up.

Needs the oxDNA sources (the src/ folder of the checkout OXDNA_REFERENCE names, or of the copy
oracle/ref/Makefile's `stage` target leaves in baseline/_ref/oxDNA) and nvcc; skipped where either
is missing.  No GPU is used: the object is
compiled, not run.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "oxdna_gb300", "shim", "CUDAGB300DNA2Interaction.cu")
_REF = os.environ.get("OXDNA_REFERENCE") or os.path.join(ROOT, "baseline", "_ref", "oxDNA")
OXDNA_SRC = os.path.join(_REF, "src")


@pytest.fixture(scope="module")
def shim_object(tmp_path_factory):
    if not os.path.isfile(os.path.join(OXDNA_SRC, "CUDA", "Interactions", "CUDABaseInteraction.h")):
        pytest.skip("oxDNA sources not present")
    if shutil.which("nvcc") is None or shutil.which("nm") is None:
        pytest.skip("nvcc / nm not available")
    out = str(tmp_path_factory.mktemp("shim") / "shim.o")
    cmd = ["nvcc", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC",
           "-I" + OXDNA_SRC, "-I" + os.path.join(OXDNA_SRC, "extern"), "-DJSON_ENABLED",
           "-I" + os.path.join(ROOT, "include"), "-c", SHIM, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _symbols(obj, flag):
    r = subprocess.run(["nm", flag, obj], capture_output=True, text=True, check=True)
    return {ln.split()[-1] for ln in r.stdout.splitlines() if ln.strip()}


def test_shim_exports_plugin_entry_points(shim_object):
    defined = _symbols(shim_object, "--defined-only")
    # PluginManager looks up make_<name> for CUDA<interaction_type> and <interaction_type>
    for name in ("make_CUDAGB300DNA2", "make_GB300DNA2", "make_GB300VerletList"):
        assert name in defined


def test_shim_calls_only_declared_abi(shim_object):
    undefined = _symbols(shim_object, "--undefined-only")
    used = {s for s in undefined if s.startswith("oxgb_")}
    header = open(os.path.join(ROOT, "include", "oxgb.h")).read()
    assert used, "the shim must call the library"
    for s in used:
        assert s + "(" in header, s
    assert {"oxgb_dna2_create", "oxgb_dna2_compute_forces", "oxgb_verlet_update"} <= used
