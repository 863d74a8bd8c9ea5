"""Pins the CPU oracle to the reference implementation (no GPU needed).

* every golden fixture: forces, torques and the 8-term energy split printed by the reference
  CPU code (DNA2_nomesh) must be reproduced to ~1e-12 relative;
* the reference's own regression values (test/DNA/FORCE_FIELD/*/reference.dat, mesh DNA2
  printed to 6 decimals) must be met within the rounding of the file (the exact f4 differs
  from the mesh by up to 1e-6 in the hydrogen-bonding column);
* a 200-step NVE run of the reference MD backend must be reproduced by the oracle integrator.
"""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN_CASES, load_golden, oracle_settings


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_matches_reference_forces(case):
    g = load_golden(case)
    p = oracle.make_params(oracle_settings(g))
    assert abs(p.rcut - float(g["rcut"])) < 1e-12
    rc, F, T, Es, Ep = oracle.forces(p, g["pos"], g["a1"], g["a2"], g["a3"], g["n3"], g["n5"], g["type"], g["btype"],
                                     float(g["box"]))
    assert rc == 0
    fscale = max(1.0, np.abs(g["F"]).max())
    tscale = max(1.0, np.abs(g["Tq"]).max())
    assert np.abs(F - g["F"]).max() <= 1e-12 * fscale
    assert np.abs(T - g["Tq"]).max() <= 1e-12 * tscale
    assert np.abs(Es - g["split"]).max() <= 1e-12 * max(1.0, np.abs(g["split"]).max())
    # per-particle energies count each pair on both particles
    assert abs(Ep.sum() / 2 - g["energy"]) <= 1e-10 * max(1.0, abs(float(g["energy"])))


def test_oracle_meets_reference_regression_values():
    gold = load_golden("ff16_reference_dat")
    for case, key in (("ff16_avg", "avg_seq"), ("ff16_seqdep", "seq_dep")):
        g = load_golden(case)
        # both reference decks set use_average_seq = true
        g = dict(g, average=np.int64(1))
        p = oracle.make_params(oracle_settings(g))
        rc, F, T, Es, Ep = oracle.forces(p, g["pos"], g["a1"], g["a2"], g["a3"], g["n3"], g["n5"], g["type"],
                                         g["btype"], float(g["box"]))
        per_nuc = Es / g["pos"].shape[0]
        tol = np.full(8, 6e-7)
        tol[4] = 2e-6  # exact f4 vs the reference's interpolation meshes, HB column
        assert np.all(np.abs(per_nuc - gold[key]) <= tol), (per_nuc, gold[key])


def test_oracle_integrator_matches_reference_md():
    g = load_golden("md_nve")
    from oxdna_gb300 import io as oxio
    p = oracle.make_params(oracle_settings(g))
    N = g["pos"].shape[0]
    md = oracle.MD()
    md.dt = float(g["dt"])
    md.thermostat = 0
    st = dict(pos=g["pos"].copy(), quat=oxio.frame_to_quat(g["a1"], g["a2"], g["a3"]), vel=g["vel"].copy(),
              Lmom=g["Lmom"].copy(), F=np.zeros((N, 3)), T=np.zeros((N, 3)))
    rc, F, T, Es, Ep = oracle.forces(p, g["pos"], g["a1"], g["a2"], g["a3"], g["n3"], g["n5"], g["type"], g["btype"],
                                     float(g["box"]))
    st["F"][:], st["T"][:] = F, T
    rc, Es = oracle.md_run(p, md, st, g["n3"], g["n5"], g["type"], g["btype"], float(g["box"]), 0, int(g["steps"]))
    assert rc == 0
    L = float(g["box"])
    d = st["pos"] - g["final_pos"]
    d -= L * np.round(d / L)  # the reference may shift whole strands by box vectors
    assert np.abs(d).max() < 1e-9
    a1, a2, a3 = oxio.quat_to_frame(st["quat"])
    assert np.abs(a1 - g["final_a1"]).max() < 1e-9
    assert np.abs(a3 - g["final_a3"]).max() < 1e-9
    assert np.abs(st["vel"] - g["final_vel"]).max() < 1e-9
    assert np.abs(st["Lmom"] - g["final_Lmom"]).max() < 1e-9


def test_oracle_external_forces_match_reference():
    """The six external-force types the engine implements (constant / string with a rate and
    with dir_as_centre, mutual traps with rates and periodic images, moving trap, low-dimensional
    moving trap, moving repulsion plane with an end position, attraction plane), as the
    reference's CPU force classes compute them at MD step 1000 (fixture ext_forces: the
    reference's forces with the records minus its forces without); the records add no torques."""
    import json
    g = load_golden("ext_forces")
    forces = json.loads(str(g["forces"]))
    F = oracle.external_forces(g["pos"], int(g["step"]), forces, float(g["box"]))
    assert np.abs(g["F_ext"]).max() > 1.0
    assert np.abs(F - g["F_ext"]).max() <= 1e-12 * np.abs(g["F_ext"]).max()
    assert np.abs(g["T_ext"]).max() == 0.0
