"""Verlet-list parity: the GPU build must give exactly the cell of every nucleotide and exactly
the neighbour set of the FP32 restatement in the oracle (oxo_verlet_f32), and must contain every
pair within the interaction cutoff found by an FP64 search."""
import numpy as np
import pytest

import oracle
from conftest import load_golden
from gpu_util import system_from_golden, settings_from_golden
from oxdna_gb300 import MDSystem, md_settings
from oxdna_gb300 import generate as G
from oxdna_gb300 import io as oxio

pytestmark = pytest.mark.gpu


def check_list(sysm, pos, box, n3, n5, rcut, skin=0.05):
    nnb, nb, cell, ns = sysm.neighbours()
    rv = np.float32(np.float32(rcut) + np.float32(2.0) * np.float32(skin))
    pos4 = np.zeros((pos.shape[0], 4), np.float32)
    pos4[:, :3] = pos.astype(np.float32)
    rc, ns_o, cell_o, nnb_o, nb_o = oracle.verlet_f32(pos4, box, float(rv), n3, n5, True, max_nb=nb.shape[1] + 64)
    assert rc == 0
    assert ns == ns_o
    assert np.array_equal(cell, cell_o)
    assert np.array_equal(nnb, nnb_o)
    for i in range(pos.shape[0]):
        assert np.array_equal(np.sort(nb[i, :nnb[i]]), nb_o[i, :nnb_o[i]]), i
    # every non-bonded pair within rcut (FP64) is listed
    pairs = oracle.pairs_within(pos, box, rcut)
    rows = [set(nb[i, :nnb[i]].tolist()) for i in range(pos.shape[0])]
    for i, j in pairs:
        if n3[i] == j or n5[i] == j:
            continue
        assert j in rows[i] and i in rows[j]


@pytest.mark.parametrize("case", ["mixed", "contact", "duplex24"])
def test_list_matches_oracle_on_fixtures(case):
    g = load_golden(case)
    sysm, _ = system_from_golden(g)
    p = oracle.make_params(oracle.make_settings(float(g["T"]), float(g["salt"])))
    check_list(sysm, g["pos"], float(g["box"]), g["n3"], g["n5"], p.rcut)
    sysm.close()


@pytest.mark.parametrize("kernel", ["warp", "thread", "group4", "group8", "group16"])
@pytest.mark.parametrize("cfg,scale", [(1, 0.1), (2, 0.02)])
def test_list_matches_oracle_on_generated(cfg, scale, kernel):
    s = G.system_for_config(cfg, seed=11, scale=scale)
    a1, a2, a3 = s.frames()
    q = oxio.frame_to_quat(a1, a2, a3)
    from oxdna_gb300 import dna2_settings
    sysm = MDSystem(s.box, s.top, dna2_settings(s.T, 0.5), md_settings(list_kernel=kernel))
    sysm.set_state(s.pos, q, s.vel, s.L)
    p = oracle.make_params(oracle.make_settings(s.T, 0.5))
    check_list(sysm, s.pos, s.box, s.top.n3, s.top.n5, p.rcut)
    sysm.close()


@pytest.mark.parametrize("cfg,scale", [(1, 0.1), (2, 0.02)])
def test_list_kernels_give_identical_rows_and_trajectories(cfg, scale):
    """the warp, thread and 4/8/16-lane neighbour kernels write the same rows, entry for entry (the
    order of every row, not only its set), so Brownian trajectories are bit-identical"""
    from oxdna_gb300 import dna2_settings
    s = G.system_for_config(cfg, seed=12, scale=scale)
    a1, a2, a3 = s.frames()
    q = oxio.frame_to_quat(a1, a2, a3)
    out = []
    for kernel in ("warp", "thread", "group4", "group8", "group16"):
        m = MDSystem(s.box, s.top, dna2_settings(s.T, 0.5),
                     md_settings(dt=0.003, thermostat="john", newtonian_steps=3, pt=0.2, seed=9, list_kernel=kernel))
        m.set_state(s.pos, q, s.vel, s.L)
        assert m.force_shape()["list_kernel"] == kernel
        rows0 = m.neighbours()
        m.run(300)
        rows1 = m.neighbours()
        st = m.get_state()
        out.append((rows0, rows1, st, m.info()["rebuilds"]))
        m.close()
    (w0, w1, ws, wr) = out[0]
    assert wr >= 3
    for (t0, t1, ts, tr) in out[1:]:
        assert wr == tr
        for a_, b_ in ((w0, t0), (w1, t1)):
            assert np.array_equal(a_[0], b_[0])
            for i in range(s.N):
                assert np.array_equal(a_[1][i, :a_[0][i]], b_[1][i, :b_[0][i]]), i
        for key in ("pos", "quat", "vel", "Lmom"):
            assert np.array_equal(ws[key], ts[key]), key


def test_autotuner_picks_a_list_kernel():
    from oxdna_gb300 import dna2_settings
    s = G.system_for_config(2, seed=13, scale=0.02)
    a1, a2, a3 = s.frames()
    m = MDSystem(s.box, s.top, dna2_settings(s.T, 0.5), md_settings(autotune=True))
    m.set_state(s.pos, oxio.frame_to_quat(a1, a2, a3), s.vel, s.L)
    sh = m.force_shape()
    print(f"autotuned: {sh}")
    assert sh["list_kernel"] in ("warp", "thread", "group4", "group8", "group16")
    m.close()
