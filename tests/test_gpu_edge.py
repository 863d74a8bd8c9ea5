"""use_edge: the pair-parallel evaluation of Debye-Hueckel and the excluded volume.

With md_settings(use_edge=True) the engine evaluates those two terms once per unordered pair in
the edge blocks of the bonded/pair kernel and adds both nucleotides' shares with atomic adds --
the scheme of the reference's use_edge kernels (src/CUDA/Interactions/CUDA_DNA.cuh:727-830) --
instead of from both ends of the full rows.  The physics is the same, only the summation order
differs, so forces, torques and energies must agree with the default evaluation to rounding:
  * FP64 engine: 1e-12 of max(|F_i|, 0.1 RMS) per nucleotide, energies 1e-12;
  * mixed engine: normwise 1e-6, per nucleotide 1e-5 of max(|F_i|, 0.1 RMS), energy split 1e-6;
on 4,000 nucleotides of duplexes and on a melt subsample, and an MD run with it stays sound.
"""
import numpy as np
import pytest

from oxdna_gb300 import MDSystem, dna2_settings, md_settings
from oxdna_gb300 import generate as G

pytestmark = pytest.mark.gpu


def _forces(s, precision, edge):
    m = MDSystem(s.box, s.top, dna2_settings(s.T, 0.5), md_settings(dt=0.003, precision=precision, use_edge=edge))
    m.set_state(s.pos, s.quats(), s.vel, s.L)
    F, T, E, Es = m.compute_forces()
    m.close()
    return F, T, np.asarray(Es)


def _rel(X, Xref):
    n = np.linalg.norm(Xref, axis=1)
    den = np.maximum(n, 0.1 * np.sqrt(np.mean(n ** 2)))
    return np.linalg.norm(X - Xref, axis=1) / den, np.linalg.norm(X - Xref) / np.linalg.norm(Xref)


@pytest.mark.parametrize("cfg,scale", [(1, 0.1), (2, 0.02)])
@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_edge_evaluation_matches_the_row_evaluation(cfg, scale, precision):
    s = G.system_for_config(cfg, seed=41, scale=scale)
    F0, T0, Es0 = _forces(s, precision, False)
    F1, T1, Es1 = _forces(s, precision, True)
    fr, fn = _rel(F1, F0)
    tr, tn = _rel(T1, T0)
    es = np.abs(Es1 - Es0).max() / np.abs(Es0).sum()
    print(f"{precision} N={s.N}: force per nucleotide max {fr.max():.2e} (normwise {fn:.2e}), torque {tr.max():.2e}, "
          f"energy split {es:.2e}")
    if precision == "double":
        assert fr.max() <= 1e-12 and tr.max() <= 1e-12 and es <= 1e-12
    else:
        assert fn <= 1e-6 and tn <= 1e-6
        assert fr.max() <= 1e-5 and tr.max() <= 1e-5
        assert es <= 1e-6


def test_edge_md_runs():
    s = G.system_for_config(1, seed=42, scale=0.1)
    out = []
    for edge in (False, True):
        m = MDSystem(s.box, s.top, dna2_settings(s.T, 0.5),
                     md_settings(dt=0.003, thermostat="bussi", newtonian_steps=1, bussi_tau=1000.0, seed=7,
                                 precision="mixed", use_edge=edge, steps_per_graph=25))
        m.set_state(s.pos, s.quats(), s.vel, s.L)
        m.run(2000)
        U, Kt, Kr = m.energies()
        st = m.get_state()
        m.close()
        assert np.all(np.isfinite(st["pos"]))
        out.append(float(np.atleast_1d(U)[0]) / s.N)
    print(f"potential energy per nucleotide after 2000 Bussi steps: rows {out[0]:.5f}, edges {out[1]:.5f}")
    assert abs(out[0] - out[1]) < 0.02
