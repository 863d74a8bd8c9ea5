"""Mixed-precision forces against the FP64 oracle at the bench's full sizes, after MD.

The fixtures of test_gpu_forces.py hold at most a few hundred nucleotides.  Here the engine's
own workloads are run for a while (so that thermal contacts -- the stiff excluded-volume
contacts above all -- are present) and the forces and torques of the mixed path (FP32 pair
arithmetic, FP64 state) on the resulting state are compared with the FP64 CPU oracle (oracle/,
pinned to the reference's DNA2_nomesh) on the same state:

  * the 40,000-nucleotide system of 1,000 duplexes after 2,000 Bussi steps;
  * a 10,000-nucleotide subsample of the single-strand melt (10 strands of 1,000 at the melt's
    density) after the melt's force-capped relaxation and 1,000 Brownian steps.

Tolerance.  Normwise, ||F - F_ref|| / ||F_ref|| <= 1e-5 (torques likewise).  Per nucleotide i
the bound is conditioning-weighted:

    |F_i - F_i,ref| <= 1e-5 max(|F_i,ref|, 0.1 RMS_j |F_j,ref|) + 2 s_i,

where s_i = |F_i,ref(axes rounded to FP32) - F_i,ref| is the FP64 oracle's own response to the
one input the mixed path rounds: the body axes, rounded to FP32 once per step.  The stiff radial
factors and excluded-volume contacts are evaluated with the axes' remainders (exact to ~1e-10),
but the angular factors take the FP32 axes; where an angle sits at its optimum (a hydrogen bond
at its well bottom) the oracle itself moves by ~1e-5 of such a nucleotide's force under that
rounding.  The plain measure (s_i = 0) is printed beside it: over 1e-5 for at most a few
nucleotides in 10^4.  The floor (0.1 of the RMS force) keeps the relative measure defined for
nucleotides whose net force nearly cancels.
"""
import os

import numpy as np
import pytest

from oxdna_gb300 import MDSystem, dna2_settings, md_settings
from oxdna_gb300 import generate as G
from oxdna_gb300 import io as oxio

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _oracle_forces(s, st, fp32_axes=False):
    import oracle
    a1, a2, a3 = oxio.quat_to_frame(st["quat"])
    if fp32_axes:
        a1 = a1.astype(np.float32).astype(np.float64)
        a3 = a3.astype(np.float32).astype(np.float64)
        a2 = np.cross(a3, a1)
    p = oracle.make_params(oracle.make_settings(s.T, 0.5))
    threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else 4
    _, F, T, Es, _ = oracle.forces(p, st["pos"], a1, a2, a3, s.top.n3, s.top.n5, s.top.type, s.top.btype, s.box,
                                   nthreads=threads)
    return F, T, Es


def _measure(X, Xref, Xrnd):
    n = np.linalg.norm(Xref, axis=1)
    den = np.maximum(n, 0.1 * np.sqrt(np.mean(n ** 2)))
    err = np.linalg.norm(X - Xref, axis=1)
    sens = np.linalg.norm(Xrnd - Xref, axis=1)
    return err / den, err / (TOL * den + 2 * sens), float(np.linalg.norm(X - Xref) / np.linalg.norm(Xref))


def _check(name, s, st, sysm):
    F, T, E, Es = sysm.compute_forces()
    Fo, To, Eso = _oracle_forces(s, st)
    Fr, Tr, _ = _oracle_forces(s, st, fp32_axes=True)
    fr, fb, fn = _measure(F, Fo, Fr)
    tr, tb, tn = _measure(T, To, Tr)
    print(f"{name}: N={s.N} force normwise {fn:.2e}, per nucleotide max {fr.max():.2e} (99.99th "
          f"{np.percentile(fr, 99.99):.2e}, {int((fr > TOL).sum())} over 1e-5), of the bound {fb.max():.2f}; "
          f"torque normwise {tn:.2e}, max {tr.max():.2e} ({int((tr > TOL).sum())} over 1e-5), of the bound {tb.max():.2f}; "
          f"energy {abs(Es.sum() - Eso.sum()) / abs(Eso.sum()):.1e}")
    assert fn <= TOL and tn <= TOL
    assert fb.max() <= 1.0, f"worst nucleotide {int(np.argmax(fb))}: {fb.max():.3f} of the bound"
    assert tb.max() <= 1.0, f"worst nucleotide {int(np.argmax(tb))}: {tb.max():.3f} of the bound"
    # the plain measure: at most a few nucleotides in 10^4 over 1e-5, none over 3e-5
    assert (fr > TOL).sum() <= max(3, s.N // 5000) and fr.max() <= 3 * TOL
    assert abs(Es.sum() - Eso.sum()) <= 1e-5 * abs(Eso.sum())


def test_plain40k_after_bussi_md():
    s = G.system_for_config(1, seed=11)
    m = MDSystem(s.box, s.top, dna2_settings(s.T, 0.5),
                 md_settings(dt=0.003, thermostat="bussi", newtonian_steps=1, bussi_tau=1000.0, seed=3,
                             precision="mixed", steps_per_graph=25))
    m.set_state(s.pos, s.quats(), s.vel, s.L)
    m.run(2000)
    st = m.get_state()
    _check("plain40k", s, st, m)
    m.close()


def test_melt_subsample_after_relaxation_and_brownian_md():
    s = G.system_for_config(2, seed=12, scale=0.04)
    pos, quat, vel, L = s.pos, s.quats(), s.vel, s.L
    # the melt's relaxation: backbone force capped at 5, then at 50, Brownian refresh
    for fmax, steps in ((5.0, 1000), (50.0, 200)):
        m = MDSystem(s.box, s.top, dna2_settings(s.T, 0.5, mbf_fmax=fmax),
                     md_settings(dt=0.003, thermostat="john", newtonian_steps=1, pt=0.1, seed=5, precision="mixed"))
        m.set_state(pos, quat, vel, L)
        m.run(steps)
        st = m.get_state()
        m.close()
        pos, quat, vel, L = st["pos"], st["quat"], st["vel"], st["Lmom"]
    m = MDSystem(s.box, s.top, dna2_settings(s.T, 0.5),
                 md_settings(dt=0.003, thermostat="john", newtonian_steps=103, diff_coeff=2.5, seed=6, precision="mixed",
                             steps_per_graph=25))
    m.set_state(pos, quat, vel, L)
    m.run(1000)
    st = m.get_state()
    _check("melt10k", s, st, m)
    m.close()
