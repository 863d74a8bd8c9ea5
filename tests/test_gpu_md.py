"""Integrator and thermostat parity.

* NVE: 200 steps of the reference MD backend (fixture md_nve) reproduced by the GPU in double
  precision to 1e-8, and in mixed precision to 1e-4 in positions;
* Brownian and Bussi: the GPU and the oracle draw from the same counter-based Philox stream,
  so in double precision their trajectories must agree step for step;
* graph replay (several steps per launch, conditional list rebuild) and one-step launches give
  identical states.
"""
import numpy as np
import pytest

import oracle
from conftest import load_golden
from gpu_util import settings_from_golden, system_from_golden
from oxdna_gb300 import io as oxio

pytestmark = pytest.mark.gpu


def wrapped_diff(a, b, L):
    d = a - b
    return d - L * np.round(d / L)


@pytest.mark.parametrize("precision,tol", [("double", 1e-8), ("mixed", 1e-4)])
def test_nve_matches_reference_md(precision, tol):
    g = load_golden("md_nve")
    sysm, _ = system_from_golden(g, precision=precision, dt=float(g["dt"]))
    sysm.run(int(g["steps"]))
    st = sysm.get_state()
    L = float(g["box"])
    assert np.abs(wrapped_diff(st["pos"], g["final_pos"], L)).max() < tol
    a1, a2, a3 = oxio.quat_to_frame(st["quat"])
    assert np.abs(a1 - g["final_a1"]).max() < tol
    assert np.abs(a3 - g["final_a3"]).max() < tol
    assert np.abs(st["vel"] - g["final_vel"]).max() < 10 * tol
    assert np.abs(st["Lmom"] - g["final_Lmom"]).max() < 10 * tol
    sysm.close()


def test_float_precision_integrates_in_fp32():
    """backend_precision = float: the state stays FP32-representable, and the 200-step NVE run
    of the reference follows it to FP32 accuracy"""
    g = load_golden("md_nve")
    sysm, _ = system_from_golden(g, precision="float", dt=float(g["dt"]))
    st0 = sysm.get_state()
    for key in ("pos", "quat", "vel", "Lmom"):
        assert np.array_equal(st0[key], st0[key].astype(np.float32).astype(np.float64)), key
    sysm.run(int(g["steps"]))
    st = sysm.get_state()
    for key in ("pos", "quat", "vel", "Lmom"):
        assert np.array_equal(st[key], st[key].astype(np.float32).astype(np.float64)), key
    L = float(g["box"])
    err = np.abs(wrapped_diff(st["pos"], g["final_pos"], L)).max()
    assert 1e-7 < err < 1e-3
    a1, a2, a3 = oxio.quat_to_frame(st["quat"])
    assert np.abs(a1 - g["final_a1"]).max() < 1e-3
    assert np.abs(np.linalg.norm(st["quat"], axis=1) - 1).max() < 1e-6
    sysm.close()


def oracle_run(g, thermostat, nsteps, n, seed, pt=0.0, tau=10.0, dt=0.003):
    p = oracle.make_params(oracle.make_settings(float(g["T"]), float(g["salt"])))
    md = oracle.MD()
    md.dt = dt
    md.thermostat = thermostat
    md.newtonian_steps = n
    md.seed = seed
    md.bussi_tau = tau
    N = g["pos"].shape[0]
    T = float(g["T"])
    dtf = float(np.float32(dt))
    md.pt = float(np.float32(pt))
    Dp = T * n * dtf * (1.0 / md.pt - 0.5)
    md.pr = (2 * T * n * dtf) / (T * n * dtf + 2 * 3 * Dp)
    md.bussi_K_t = 0.5 * 3 * (N - 1) * T
    md.bussi_K_r = 0.5 * 3 * N * T
    st = dict(pos=g["pos"].copy(), quat=oxio.frame_to_quat(g["a1"], g["a2"], g["a3"]), vel=g["vel"].copy(),
              Lmom=g["Lmom"].copy(), F=np.zeros((N, 3)), T=np.zeros((N, 3)))
    rc, F, Tq, Es, Ep = oracle.forces(p, g["pos"], g["a1"], g["a2"], g["a3"], g["n3"], g["n5"], g["type"], g["btype"],
                                      float(g["box"]))
    st["F"][:], st["T"][:] = F, Tq
    rc, Es = oracle.md_run(p, md, st, g["n3"], g["n5"], g["type"], g["btype"], float(g["box"]), 0, nsteps)
    assert rc == 0
    return st


@pytest.mark.parametrize("thermostat,name", [(1, "john"), (2, "bussi")])
def test_thermostat_trajectory_matches_oracle(thermostat, name):
    g = load_golden("md_nve")
    nsteps, n, seed = 60, 5, 1234
    kw = dict(dt=0.003, thermostat=name, newtonian_steps=n, seed=seed)
    if name == "john":
        kw["pt"] = 0.3
    else:
        kw["bussi_tau"] = 10.0
    sysm, _ = system_from_golden(g, precision="double", **kw)
    sysm.run(nsteps)
    st = sysm.get_state()
    ref = oracle_run(g, thermostat, nsteps, n, seed, pt=0.3, tau=10.0)
    L = float(g["box"])
    assert np.abs(wrapped_diff(st["pos"], ref["pos"], L)).max() < 1e-8
    assert np.abs(st["vel"] - ref["vel"]).max() < 1e-7
    assert np.abs(st["Lmom"] - ref["Lmom"]).max() < 1e-7
    sysm.close()


def test_graph_replay_equals_single_steps():
    g = load_golden("mixed")
    a, _ = system_from_golden(g, precision="mixed", dt=0.002, steps_per_graph=8)
    b, _ = system_from_golden(g, precision="mixed", dt=0.002, steps_per_graph=1)
    a.run(64)
    for _ in range(8):
        b.run(8)
    sa, sb = a.get_state(), b.get_state()
    assert np.array_equal(sa["pos"], sb["pos"])
    assert np.array_equal(sa["quat"], sb["quat"])
    assert a.info()["step"] == 64 and b.info()["step"] == 64
    assert a.info()["rebuilds"] == b.info()["rebuilds"]
    a.close()
    b.close()


def test_rebuild_node_kinds_agree():
    """The conditional rebuild node and the always-launched rebuild kernels give the same run."""
    g = load_golden("mixed")
    a, _ = system_from_golden(g, precision="mixed", dt=0.003, steps_per_graph=10)
    b, _ = system_from_golden(g, precision="mixed", dt=0.003, steps_per_graph=10, list_rebuild_node="kernel")
    a.run(300)
    b.run(300)
    sa, sb = a.get_state(), b.get_state()
    assert np.array_equal(sa["pos"], sb["pos"])
    assert np.array_equal(sa["vel"], sb["vel"])
    assert np.array_equal(sa["quat"], sb["quat"])
    assert a.info()["rebuilds"] == b.info()["rebuilds"] >= 2
    a.close()
    b.close()


@pytest.mark.parametrize("precision", ["mixed", "double"])
def test_lists_stay_complete_between_rebuilds(precision):
    """Forces from term lists carried over many steps equal forces from freshly built lists."""
    g = load_golden("mixed")
    sysm, _ = system_from_golden(g, precision=precision, dt=0.003, steps_per_graph=10)
    for _ in range(6):
        sysm.run(50)
        F1, T1, E1 = sysm.get_forces()
        F2, T2, E2, _ = sysm.compute_forces()  # rebuilds every list first
        scale = max(1.0, np.abs(F2).max())
        tol = 1e-12 if precision == "double" else 1e-5
        assert np.abs(F1 - F2).max() <= tol * scale
        assert np.abs(T1 - T2).max() <= tol * max(1.0, np.abs(T2).max())
    assert sysm.info()["rebuilds"] >= 2
    sysm.close()


def test_state_round_trip_and_rejected_state():
    """set_state then get_state returns the state (quaternions normalised); a state with a
    quaternion that cannot be normalised is rejected and leaves the current one in place."""
    from oxdna_gb300._abi import OxgbError
    g = load_golden("mixed")
    sysm, _ = system_from_golden(g, precision="mixed", dt=0.002)
    st = sysm.get_state()
    q = st["quat"] * 3.0  # scaled: normalised on upload
    sysm.set_state(st["pos"], q, st["vel"], st["Lmom"])
    back = sysm.get_state()
    assert np.array_equal(back["pos"], st["pos"]) and np.array_equal(back["vel"], st["vel"])
    assert np.array_equal(back["Lmom"], st["Lmom"])
    assert np.abs(back["quat"] - st["quat"]).max() < 1e-15
    bad = st["quat"].copy()
    bad[5] = 0.0
    with pytest.raises(OxgbError, match="nucleotide 5"):
        sysm.set_state(st["pos"] + 1.0, bad, st["vel"], st["Lmom"])
    after = sysm.get_state()
    assert np.array_equal(after["pos"], back["pos"])
    sysm.run(10)
    assert np.all(np.isfinite(sysm.get_state()["pos"]))
    sysm.close()


def test_output_files_follow_the_engine(tmp_path):
    """Energy file and trajectory written from the engine (oxdna_gb300.output) agree with the
    engine's own state and FP64 energies at the printing steps."""
    from oxdna_gb300 import output
    g = load_golden("duplex24")
    sysm, _ = system_from_golden(g, precision="mixed", dt=0.003)
    from gpu_util import topology_from_golden
    top = topology_from_golden(g)
    e, t = str(tmp_path / "energy.dat"), str(tmp_path / "traj.dat")
    out = output.Output(sysm, top, float(g["box"]), 0.003, energy_file=e, trajectory_file=t, back_in_box=False)
    output.run_with_output(sysm, 300, out, print_energy_every=100, print_conf_interval=300)
    rows = np.loadtxt(e)
    assert rows.shape == (4, 4)
    U, Kt, Kr = sysm.energies()
    N = g["pos"].shape[0]
    assert abs(rows[-1, 1] - U / N) < 1e-6 and abs(rows[-1, 2] - (Kt + Kr) / N) < 1e-6
    frames = open(t).read().split("t = ")[1:]
    assert len(frames) == 2
    last = tmp_path / "last.dat"
    last.write_text("t = " + frames[-1])
    conf = oxio.read_conf(str(last))
    st = sysm.get_state()
    assert conf.t == 300 and np.abs(conf.pos - st["pos"]).max() < 1e-12
    sysm.close()
