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


@pytest.mark.parametrize("case", ["contact", "mixed", "duplex24", "ff16_seqdep"])
def test_order_parameter_hb_energies_sum_to_the_reference_hb_term(case):
    """The oracle's FFS order-parameter energies (CUDA_DNA.cuh:910-961: f1 times the six f4
    factors of a pair) summed over every pair equal the hydrogen-bonding term the reference
    printed for the fixture; the nearly-bonded flag is set on every pair with a non-zero energy."""
    g = load_golden(case)
    p = oracle.make_params(oracle_settings(g))
    N = g["pos"].shape[0]
    i, j = np.triu_indices(N, 1)
    bonded = (g["n3"][i] == j) | (g["n5"][i] == j)
    i, j = i[~bonded], j[~bonded]
    args = (p, g["pos"], g["a1"], g["a3"], g["type"], g["btype"], float(g["box"]), i, j)
    e = oracle.order_params(*args, 0)
    near = oracle.order_params(*args, 1)
    dist = oracle.order_params(*args, 2)
    hb = float(g["split"][4])
    assert abs(e.sum() - hb) <= 1e-12 * max(1.0, abs(hb)), (e.sum(), hb)
    assert np.all(near[e != 0] == 1)
    r = g["pos"][j] - g["pos"][i]
    r -= np.rint(r / float(g["box"])) * float(g["box"])
    rb = r + float(np.float32(0.4)) * g["a1"][j] - float(np.float32(0.4)) * g["a1"][i]
    assert np.allclose(dist, np.linalg.norm(rb, axis=1), rtol=1e-12, atol=1e-12)
