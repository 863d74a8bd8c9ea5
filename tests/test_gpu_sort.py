"""Spatially ordered storage (md_settings(sort_every=k), the reference's CUDA_sort_every): every
k-th list rebuild moves the nucleotides on the device into the order of their cells -- along a
Hilbert curve (sort_order "hilbert", the default, the reference's key) or row-major ("cells").  Cells are
ordered and base/stack pairs owned by the caller's index, so the neighbour rows list the same
partners in the same order as without sorting, and the Philox draws are keyed by the caller's
index: forces, Brownian and NVE trajectories are bit-identical to an unsorted run, and the state,
forces and external forces cross the interface in the caller's order.  Bussi sums the kinetic
energy over storage slots, so its trajectories agree to rounding."""
import numpy as np
import pytest

from oxdna_gb300 import MDSystem, dna2_settings, md_settings
from oxdna_gb300 import generate as G
from oxdna_gb300 import io as oxio

pytestmark = pytest.mark.gpu


def _state(s):
    a1, a2, a3 = s.frames()
    return s.pos, oxio.frame_to_quat(a1, a2, a3), s.vel, s.L


@pytest.fixture(scope="module")
def duplexes():
    return G.system_for_config(1, seed=4, scale=0.05)  # 50 random 20-bp duplexes, 2000 nt


def _engine(s, **kw):
    m = MDSystem(s.box, s.top, dna2_settings(s.T, 0.5), md_settings(**kw))
    m.set_state(*_state(s))
    return m


def _same(a, b):
    sa, sb = a.get_state(), b.get_state()
    for key in ("pos", "quat", "vel", "Lmom"):
        assert np.array_equal(sa[key], sb[key]), key
    Fa, Ta, Ea = a.get_forces()
    Fb, Tb, Eb = b.get_forces()
    assert np.array_equal(Fa, Fb) and np.array_equal(Ta, Tb)


@pytest.mark.parametrize("order", ["hilbert", "cells"])
@pytest.mark.parametrize("thermostat,every", [("john", 1), ("no", 1), ("john", 3)])
def test_sorted_run_is_bit_identical(duplexes, thermostat, every, order):
    kw = dict(dt=0.003, thermostat=thermostat, newtonian_steps=3, pt=0.2, seed=5, steps_per_graph=10)
    a = _engine(duplexes, **kw)
    b = _engine(duplexes, sort_every=every, sort_order=order, **kw)
    N = duplexes.N
    for n in (100, 105, 95):  # graph launches and eager remainders
        a.run(n)
        b.run(n)
        _same(a, b)
    order = b.storage_order()
    assert np.array_equal(np.sort(order), np.arange(N))
    assert not np.array_equal(order, np.arange(N))  # nucleotides did move
    assert np.array_equal(a.storage_order(), np.arange(N))
    assert b.info()["rebuilds"] >= 4
    Ua, Kta, Kra = a.energies()
    Ub, Ktb, Krb = b.energies()
    assert abs(Ua - Ub) <= 1e-12 * abs(Ua) and abs(Kta - Ktb) <= 1e-12 * Kta
    F, T, E, Es = a.compute_forces()
    Fs, Ts, Esp, Ess = b.compute_forces()
    assert np.array_equal(F, Fs) and np.array_equal(T, Ts)
    assert np.abs(Es - Ess).max() <= 1e-12 * np.abs(Es).max()
    a.close()
    b.close()


def test_sorted_batch_and_external_forces():
    systems = G.batched_systems(n_systems=4, seed=6, n_min=16, n_max=400, t_low=280.0, t_high=360.0)
    a1s = [_state(s) for s in systems]
    cat = [np.concatenate(x) for x in zip(*a1s)]
    kw = dict(dt=0.003, thermostat="john", newtonian_steps=3, pt=0.2, seed=7, steps_per_graph=8)
    runs = []
    for every in (0, 1):
        m = MDSystem([s.box for s in systems], [s.top for s in systems], [dna2_settings(s.T, 0.5) for s in systems],
                     md_settings(sort_every=every, **kw))
        m.set_state(*cat)
        lo = int(m.offsets[2])
        m.set_external_forces([dict(type="mutual_trap", particle=lo, ref_particle=lo + 9, stiff=1.0, r0=1.0),
                               dict(type="constant", particle=3, F0=0.5, dir=(0.0, 0.0, 1.0))])
        m.run(120)
        m.set_temperature(0.11, 1)  # one system rebuilt alone
        m.run(80)
        runs.append(m)
    _same(*runs)
    assert not np.array_equal(runs[1].storage_order(), np.arange(runs[1].N))
    for m in runs:
        m.close()


def test_bussi_sorted_agrees_to_rounding(duplexes):
    """Bussi's kinetic sums run over storage slots, so a sorted run rounds them differently from
    an unsorted one (forces, rows and draws are identical): after 10 steps the states agree to
    rounding; the dynamics then amplifies that difference (to ~1e-9 in the velocities after 200
    steps), with no systematic drift between the two."""
    kw = dict(dt=0.003, thermostat="bussi", bussi_tau=30.0, newtonian_steps=1, seed=9, steps_per_graph=10)
    a = _engine(duplexes, **kw)
    b = _engine(duplexes, sort_every=1, **kw)
    a.run(10)
    b.run(10)
    sa, sb = a.get_state(), b.get_state()
    d10 = np.abs(sa["vel"] - sb["vel"]).max()
    assert np.abs(sa["pos"] - sb["pos"]).max() < 1e-13
    assert d10 < 1e-12
    a.run(190)
    b.run(190)
    sa, sb = a.get_state(), b.get_state()
    d200 = np.abs(sa["vel"] - sb["vel"]).max()
    print(f"max |dv|: {d10:.2e} after 10 steps, {d200:.2e} after 200")
    assert np.abs(sa["pos"] - sb["pos"]).max() < 1e-9
    assert d200 < 1e-8
    ka, kb = a.energies(potential=False), b.energies(potential=False)
    assert abs(ka[1] - kb[1]) <= 1e-9 * abs(ka[1]) and abs(ka[2] - kb[2]) <= 1e-9 * abs(ka[2])
    a.close()
    b.close()


def test_state_and_topology_round_trip_while_sorted(duplexes):
    m = _engine(duplexes, dt=0.003, thermostat="john", seed=3, sort_every=1)
    m.run(150)
    st = m.get_state()
    m.set_state(st["pos"], st["quat"], st["vel"], st["Lmom"])
    st2 = m.get_state()
    for key in ("pos", "vel", "Lmom"):
        assert np.array_equal(st[key], st2[key]), key
    assert np.abs(st["quat"] - st2["quat"]).max() <= 1e-15  # renormalised on upload
    from oxdna_gb300 import _abi
    t = duplexes.top
    c = lambda x: np.ascontiguousarray(x, np.int32)
    _abi.check(_abi.lib().oxgb_md_set_topology(m.handle, c(t.n3), c(t.n5), c(t.btype), c(t.type)))
    st3 = m.get_state()
    assert np.array_equal(st2["pos"], st3["pos"])
    m.run(50)
    assert np.all(np.isfinite(m.get_state()["pos"]))
    m.close()


def test_hilbert_and_cell_orders_differ(duplexes):
    kw = dict(dt=0.003, thermostat="john", newtonian_steps=3, pt=0.2, seed=5, steps_per_graph=10, sort_every=1)
    h = _engine(duplexes, sort_order="hilbert", **kw)
    c = _engine(duplexes, sort_order="cells", **kw)
    h.run(50)
    c.run(50)
    _same(h, c)
    assert not np.array_equal(h.storage_order(), c.storage_order())
    h.close()
    c.close()
