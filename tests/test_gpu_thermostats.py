"""The thermostats pinned statistically, the way the reference pins its own.

The reference's regression tests test/THERMOSTATS/{JOHN,BUSSI} run an LJ fluid at T = 2 and
require the average kinetic energy per particle (3/2 T = 3) within 0.1, i.e. 3.3 %.  Our
Brownian and Bussi trajectories cannot be compared with the reference's step for step (the
random streams differ: counter-based Philox here, drand48 / curand there), so these tests ask the
same statistical questions of the engine, on DNA:

* equipartition: the time average of the translational and of the rotational kinetic energy per
  nucleotide is 3/2 T (unit mass and moment of inertia), within 2 %, for every system of a batch
  at two temperatures (Brownian: newtonian_steps 103, diff_coeff 2.5; Bussi);
* Bussi samples the canonical ensemble, in which the kinetic energy of the 3 (N - 1) internal
  translational degrees of freedom has the Gamma distribution of shape 3 (N - 1) / 2 and scale T:
  mean 3 (N - 1) T / 2 and variance 3 (N - 1) T^2 / 2.  The sample variance of K_t (pooled over
  the systems, ~10^3 samples of a correlation time ~tau each) must match within 25 %, and so
  must that of K_r (3 N degrees of freedom); an NVE run or a plain velocity rescaling would give
  a far smaller (or a zero) variance.

The systems are groups of 40 random 20-bp duplexes (1,600 nucleotides) at the 40k workload's
density, run as one batch.
"""
import numpy as np
import pytest

from oxdna_gb300 import MDSystem, dna2_settings, md_settings
from oxdna_gb300 import generate as G

pytestmark = pytest.mark.gpu

TEMPS = [G.kelvin(300.0), G.kelvin(300.0), G.kelvin(350.0), G.kelvin(350.0)]


def _batch(thermostat, **md):
    systems = []
    for k, T in enumerate(TEMPS):
        s = G.system_for_config(1, seed=200 + k, scale=0.04)
        s.T = T
        systems.append(s)
    m = MDSystem([s.box for s in systems], [s.top for s in systems], [dna2_settings(s.T, 0.5) for s in systems],
                 md_settings(dt=0.003, thermostat=thermostat, seed=17, precision="mixed", steps_per_graph=25, **md))
    m.set_state(np.concatenate([s.pos for s in systems]), np.concatenate([s.quats() for s in systems]),
                np.concatenate([s.vel * np.sqrt(s.T / 0.1) for s in systems]), np.concatenate([s.L * np.sqrt(s.T / 0.1) for s in systems]))
    return m, systems


def _sample(m, equil, n_samples, every):
    m.run(equil)
    kt, kr = [], []
    for _ in range(n_samples):
        m.run(every)
        _, a, b = m.energies(potential=False)
        kt.append(a)
        kr.append(b)
    return np.array(kt), np.array(kr)


def test_brownian_equipartition():
    m, systems = _batch("john", newtonian_steps=103, diff_coeff=2.5)
    kt, kr = _sample(m, equil=50000, n_samples=200, every=500)
    m.close()
    for k, s in enumerate(systems):
        et, er = kt[:, k].mean() / (1.5 * s.N * s.T), kr[:, k].mean() / (1.5 * s.N * s.T)
        print(f"Brownian system {k} (T = {s.T:.4f}): <K_t> / (3/2 N T) = {et:.4f}, <K_r> / (3/2 N T) = {er:.4f}")
        assert abs(et - 1) < 0.02 and abs(er - 1) < 0.02


def test_bussi_canonical_kinetic_energy():
    tau = 100
    m, systems = _batch("bussi", newtonian_steps=1, bussi_tau=float(tau))
    kt, kr = _sample(m, equil=10 * tau, n_samples=1000, every=tau)
    m.close()
    zt, zr = [], []
    for k, s in enumerate(systems):
        dof_t, dof_r = 3 * (s.N - 1), 3 * s.N
        mt, mr = kt[:, k].mean() / (0.5 * dof_t * s.T), kr[:, k].mean() / (0.5 * dof_r * s.T)
        vt, vr = kt[:, k].var(ddof=1) / (0.5 * dof_t * s.T ** 2), kr[:, k].var(ddof=1) / (0.5 * dof_r * s.T ** 2)
        print(f"Bussi system {k} (T = {s.T:.4f}): mean K_t {mt:.4f}, K_r {mr:.4f} of canonical; "
              f"variance K_t {vt:.3f}, K_r {vr:.3f} of canonical")
        assert abs(mt - 1) < 0.02 and abs(mr - 1) < 0.02
        zt.append(vt)
        zr.append(vr)
    # pooled over the systems: ~4000 samples, a few hundred correlation times
    assert abs(np.mean(zt) - 1) < 0.25, zt
    assert abs(np.mean(zr) - 1) < 0.25, zr
