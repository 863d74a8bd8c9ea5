"""External forces through the C ABI against the oracle's restatement (every force type the
engine implements, with rates, dir_as_centre and a periodic mutual trap), and a mutual trap that
pulls two nucleotides together over an MD run.

The record set is the one of fixture ext_forces, for which test_oracle_pin.py holds the oracle
to the reference's own CPU force classes (1e-12), so the chain GPU -> oracle -> reference is
closed on the same records."""
import json

import numpy as np
import pytest

import oracle
from conftest import load_golden
from gpu_util import system_from_golden

pytestmark = pytest.mark.gpu


def _forces(N, box):
    recs = json.loads(str(load_golden("ext_forces")["forces"]))
    assert max(max(d.get("particle", 0), d.get("ref_particle", 0), *d.get("com_list", []), *d.get("ref_list", []))
               for d in recs) < N
    return recs


@pytest.mark.parametrize("run_before", [0, 12])
def test_external_forces_match_oracle(run_before):
    g = load_golden("duplex24")
    N = g["pos"].shape[0]
    box = float(g["box"])
    sysm, _ = system_from_golden(g, precision="mixed", dt=0.003)
    if run_before:
        sysm.run(run_before)
    F0, T0, _ = sysm.get_forces()
    forces = _forces(N, box)
    sysm.set_external_forces(forces)
    F1, T1, _ = sysm.get_forces()
    st = sysm.get_state()
    ext = oracle.external_forces(st["pos"], sysm.info()["step"], forces, box)
    assert np.abs(ext).max() > 0.1
    scale = max(1.0, np.abs(F1).max())
    assert np.abs((F1 - F0) - ext).max() <= 2e-6 * scale
    assert np.array_equal(T1, T0)  # no torques
    sysm.set_external_forces([])
    F2, _, _ = sysm.get_forces()
    assert np.array_equal(F2, F0)
    sysm.close()


def test_mutual_trap_pulls_nucleotides_together():
    g = load_golden("duplex24")
    N = g["pos"].shape[0]
    sysm, _ = system_from_golden(g, precision="mixed", dt=0.003, thermostat="john", newtonian_steps=53, pt=0.1)
    p, q = 0, N // 2 - 1  # the two ends of one strand
    d0 = np.linalg.norm(sysm.get_state()["pos"][q] - sysm.get_state()["pos"][p])
    sysm.set_external_forces([dict(type="mutual_trap", particle=p, ref_particle=q, stiff=2.0, r0=0.0),
                              dict(type="mutual_trap", particle=q, ref_particle=p, stiff=2.0, r0=0.0)])
    sysm.run(1500)
    st = sysm.get_state()
    d1 = np.linalg.norm(st["pos"][q] - st["pos"][p])
    assert np.all(np.isfinite(st["pos"]))
    assert d1 < d0 - 0.3
    sysm.close()
