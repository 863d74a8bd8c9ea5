"""GPU force/torque/energy parity against the reference fixtures (through the C ABI).

double precision: the same physics in FP64 must reproduce the reference's DNA2_nomesh output
to 1e-10 relative.  Mixed precision (FP32 pair math with compensated site vectors and sums, FP64
state): the force error of a system, ||F - F_ref|| / ||F_ref|| over all nucleotides, is at most
1e-5 (torques likewise); every nucleotide's error is at most 5e-5 of max(|F_ref,i|, 0.1 RMS|F_ref|)
(the FP32 conditioning floor of the stiff Morse and FENE terms); energies agree to 1e-5.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from gpu_util import force_errors, system_from_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_double_precision_matches_reference(case):
    g = load_golden(case)
    sysm, _ = system_from_golden(g, precision="double")
    F, T, E, Es = sysm.compute_forces()
    fs = max(1.0, np.abs(g["F"]).max())
    ts = max(1.0, np.abs(g["Tq"]).max())
    assert np.abs(F - g["F"]).max() <= 1e-10 * fs
    assert np.abs(T - g["Tq"]).max() <= 1e-10 * ts
    assert np.abs(Es - g["split"]).max() <= 1e-10 * max(1.0, np.abs(g["split"]).max())
    assert abs(E.sum() / 2 - float(g["energy"])) <= 1e-9 * max(1.0, abs(float(g["energy"])))
    sysm.close()


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_mixed_precision_within_tolerance(case):
    g = load_golden(case)
    sysm, _ = system_from_golden(g, precision="mixed")
    F, T, E, Es = sysm.compute_forces()
    fmax, fnorm = force_errors(F, g["F"])
    tmax, tnorm = force_errors(T, g["Tq"])
    print(f"{case}: force max-rel {fmax:.2e} norm {fnorm:.2e}; torque max-rel {tmax:.2e} norm {tnorm:.2e}; "
          f"split {np.abs(Es - g['split']).max():.2e}")
    assert fnorm <= 1e-5 and tnorm <= 1e-5
    assert fmax <= 5e-5 and tmax <= 5e-5
    assert np.abs(Es - g["split"]).max() <= 1e-5 * max(1.0, np.abs(g["split"]).max())
    sysm.close()
