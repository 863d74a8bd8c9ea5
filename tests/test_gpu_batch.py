"""A batch of independent systems in one engine evolves each system exactly as it would alone.

Every system has its own box, temperature (hence tables and Debye-Hueckel cutoff), cell grid,
Verlet lists and thermostat; system k uses the seed md.seed + k and draws keyed by the index
within the system.  The kernels do the same arithmetic in the same order for a nucleotide in a
batch as alone, so states, forces and energies must be bit-identical, for Brownian and Bussi
thermostats alike, across list rebuilds of some systems and not others, and after a temperature
change of one system (the replica-exchange hook).
"""
import numpy as np
import pytest

from oxdna_gb300 import MDSystem, dna2_settings, md_settings
from oxdna_gb300 import generate as G
from oxdna_gb300 import io as oxio

pytestmark = pytest.mark.gpu


def _systems(n=6, seed=3):
    return G.batched_systems(n_systems=n, seed=seed, n_min=16, n_max=400, t_low=280.0, t_high=360.0)


def _state(s):
    a1, a2, a3 = s.frames()
    return s.pos, oxio.frame_to_quat(a1, a2, a3), s.vel, s.L


def _batch(systems, **mdkw):
    b = MDSystem([s.box for s in systems], [s.top for s in systems], [dna2_settings(s.T, 0.5) for s in systems],
                 md_settings(**mdkw))
    cat = [np.concatenate(x) for x in zip(*[_state(s) for s in systems])]
    b.set_state(*cat)
    return b


def _alone(s, k, **mdkw):
    kw = dict(mdkw)
    kw["seed"] = kw.get("seed", 1) + k
    m = MDSystem(s.box, s.top, dna2_settings(s.T, 0.5), md_settings(**kw))
    m.set_state(*_state(s))
    return m


@pytest.mark.parametrize("thermostat", ["john", "bussi"])
def test_batch_equals_systems_alone(thermostat):
    systems = _systems()
    kw = dict(dt=0.003, thermostat=thermostat, newtonian_steps=3, pt=0.2, bussi_tau=30.0, seed=11, steps_per_graph=10)
    b = _batch(systems, **kw)
    b.run(150)
    sb = b.get_state()
    Fb, Tb, Eb = b.get_forces()
    Ub, Ktb, Krb = b.energies()
    for k, s in enumerate(systems):
        lo, hi = b.offsets[k], b.offsets[k + 1]
        m = _alone(s, k, **kw)
        m.run(150)
        sm = m.get_state()
        for key in ("pos", "quat", "vel", "Lmom"):
            assert np.array_equal(sb[key][lo:hi], sm[key]), (k, key)
        F, T, E = m.get_forces()
        assert np.array_equal(Fb[lo:hi], F) and np.array_equal(Tb[lo:hi], T) and np.array_equal(Eb[lo:hi], E)
        U, Kt, Kr = m.energies()
        assert Ub[k] == U and Ktb[k] == Kt and Krb[k] == Kr
        m.close()
    assert b.info()["step"] == 150
    b.close()


def test_batch_energy_split_and_temperature_change():
    systems = _systems(n=4, seed=5)
    kw = dict(dt=0.003, thermostat="john", newtonian_steps=5, pt=0.1, seed=2, steps_per_graph=8)
    b = _batch(systems, **kw)
    _, _, _, split = b.compute_forces()
    assert split.shape == (4, 8)
    # the hottest system cools to the coldest temperature (its cutoff shrinks: only its own
    # lists are rebuilt), then everything runs on
    T_cold = systems[0].T
    b.set_temperature(T_cold, 3)
    b.run(64)
    sb = b.get_state()
    for k, s in enumerate(systems):
        m = _alone(s, k, **kw)
        _, _, _, sp = m.compute_forces()
        assert np.array_equal(split[k], sp)
        if k == 3:
            m.set_temperature(T_cold)
        m.run(64)
        sm = m.get_state()
        lo, hi = b.offsets[k], b.offsets[k + 1]
        assert np.array_equal(sb["pos"][lo:hi], sm["pos"]), k
        assert np.array_equal(sb["vel"][lo:hi], sm["vel"]), k
        m.close()
    b.close()


def test_batch_replica_swap_keeps_lists_complete():
    """A temperature swap that raises a cutoff (possibly a new cell layout): the lists carried
    over the following steps still give the forces of freshly built ones."""
    systems = _systems(n=4, seed=7)
    b = _batch(systems, dt=0.003, thermostat="bussi", newtonian_steps=1, bussi_tau=100.0, seed=4, steps_per_graph=10)
    T0, T3 = systems[0].T, systems[3].T
    b.set_temperature(T3, 0)
    b.set_temperature(T0, 3)
    for _ in range(3):
        b.run(40)
        F1, T1, _ = b.get_forces()
        F2, T2, _, _ = b.compute_forces()
        assert np.abs(F1 - F2).max() <= 1e-5 * max(1.0, np.abs(F2).max())
        assert np.abs(T1 - T2).max() <= 1e-5 * max(1.0, np.abs(T2).max())
    U, Kt, Kr = b.energies()
    assert np.all(np.isfinite(U)) and np.all(Kt > 0) and np.all(Kr > 0)
    b.close()
