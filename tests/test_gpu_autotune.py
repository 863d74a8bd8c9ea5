"""The autotuner of the MD step's force kernels (md_settings(autotune=True)).

Shapes differ in how the work is dealt out (nucleotides per pair-block warp queue, lanes per
nucleotide in the non-bonded kernel, register cap), not in the arithmetic of a pair, so every
shape must give the default shape's forces and torques up to the order of the compensated sums
(1e-6 of the largest force), and a tuned engine must run the dynamics like an untuned one.
"""
import numpy as np
import pytest

from oxdna_gb300 import MDSystem, dna2_settings, md_settings
from oxdna_gb300 import generate as G

pytestmark = pytest.mark.gpu


def _engine(s, **kw):
    m = MDSystem(s.box, s.top, dna2_settings(s.T, 0.5),
                 md_settings(dt=0.003, thermostat="john", newtonian_steps=103, diff_coeff=2.5, seed=9, **kw))
    m.set_state(s.pos, s.quats(), s.vel, s.L)
    return m


def test_every_shape_gives_the_default_forces():
    s = G.system_for_config(1, seed=21, scale=0.1)
    m = _engine(s)
    F0, T0, _ = m.get_forces()
    scale = max(1.0, np.abs(F0).max())
    shapes = set()
    for k in range(6):
        m.set_force_shape(k)
        sh = m.force_shape()
        shapes.add((sh["pair_npw"], sh["nb_lanes"], sh["nb_min_blocks"]))
        F, T, _ = m.get_forces()
        assert np.abs(F - F0).max() <= 1e-6 * scale, k
        assert np.abs(T - T0).max() <= 1e-6 * max(1.0, np.abs(T0).max()), k
    assert len(shapes) == 6
    # every shape also runs inside the step graph (captured again after each change)
    for k in range(6):
        m.set_force_shape(k)
        m.run(50)
        assert np.all(np.isfinite(m.get_state()["pos"])), k
    m.close()


def test_autotuned_engine_runs_like_the_default():
    s = G.system_for_config(1, seed=22, scale=0.1)
    a = _engine(s, autotune=True)
    b = _engine(s)
    sh = a.force_shape()
    assert sh["launch_us"] > 0 and sh["nb_lanes"] in (2, 4, 8) and sh["pair_npw"] in (16, 32)
    assert b.force_shape()["launch_us"] == 0
    a.run(200)
    b.run(200)
    sa, sb = a.get_state(), b.get_state()
    # the same dynamics to the rounding of the force sums, amplified over 200 steps
    assert np.abs(sa["pos"] - sb["pos"]).max() < 1e-3
    Ua, _, _ = a.energies()
    Ub, _, _ = b.energies()
    assert abs(Ua - Ub) < 1e-3 * abs(Ub)
    # a second engine of the same size class takes the cached choice
    c = _engine(s, autotune=True)
    assert c.force_shape() == sh
    for m in (a, b, c):
        m.close()
