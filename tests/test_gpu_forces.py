"""GPU force/torque/energy parity against the reference fixtures (through the C ABI).

double precision: the same physics in FP64 must reproduce the reference's DNA2_nomesh output
to 1e-10 relative.  Mixed precision (FP32 pair math with compensated site vectors and sums, FP64
state): the force error of a system, ||F - F_ref|| / ||F_ref|| over all nucleotides, is at most
1e-5 (torques likewise); every nucleotide's error is at most 5e-5 of max(|F_ref,i|, 0.1 RMS|F_ref|)
(the FP32 conditioning floor of the stiff Morse and FENE terms); energies agree to 1e-5.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from gpu_util import force_errors, system_from_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_double_precision_matches_reference(case):
    g = load_golden(case)
    sysm, _ = system_from_golden(g, precision="double")
    F, T, E, Es = sysm.compute_forces()
    fs = max(1.0, np.abs(g["F"]).max())
    ts = max(1.0, np.abs(g["Tq"]).max())
    assert np.abs(F - g["F"]).max() <= 1e-10 * fs
    assert np.abs(T - g["Tq"]).max() <= 1e-10 * ts
    assert np.abs(Es - g["split"]).max() <= 1e-10 * max(1.0, np.abs(g["split"]).max())
    assert abs(E.sum() / 2 - float(g["energy"])) <= 1e-9 * max(1.0, abs(float(g["energy"])))
    sysm.close()


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_mixed_precision_within_tolerance(case):
    g = load_golden(case)
    sysm, _ = system_from_golden(g, precision="mixed")
    F, T, E, Es = sysm.compute_forces()
    fmax, fnorm = force_errors(F, g["F"])
    tmax, tnorm = force_errors(T, g["Tq"])
    print(f"{case}: force max-rel {fmax:.2e} norm {fnorm:.2e}; torque max-rel {tmax:.2e} norm {tnorm:.2e}; "
          f"split {np.abs(Es - g['split']).max():.2e}")
    assert fnorm <= 1e-5 and tnorm <= 1e-5
    assert fmax <= 5e-5 and tmax <= 5e-5
    assert np.abs(Es - g["split"]).max() <= 1e-5 * max(1.0, np.abs(g["split"]).max())
    sysm.close()


def _sites(p, q):
    from oxdna_gb300 import generate as G
    from oxdna_gb300 import io as oxio
    a1, a2, a3 = oxio.quat_to_frame(q[None, :])
    return p + G.BACK1 * a1[0] + G.BACK2 * a2[0], p + 0.4 * a1[0]


def _contact_pairs(rng, box, shift_rng=None):
    """196 two-nucleotide contacts on a 14 x 14 grid of slots 10 apart in y and z (no cross
    talk), each at a random orientation and centre distance 0.7-1.1, so that excluded volume,
    and at times hydrogen bonding or stacking, is on; no two sites of a pair closer than 0.85
    of their exclusion diameter (deep overlaps would make the RMS force floor meaningless).
    With shift_rng every nucleotide is then moved by a random whole number of box sides
    (-2..2 per axis, the two of a pair to different images; drawn from shift_rng, so that the
    contacts are those without it): the unwrapped coordinates of the partners are up to five
    box sides apart."""
    sig = {("back", "back"): 0.70, ("back", "base"): 0.515, ("base", "back"): 0.515, ("base", "base"): 0.33}
    n = 14
    pos, quat = [], []
    for a in range(n):
        for b in range(n):
            while True:
                A = np.array([rng.uniform(10.0, box - 10.0), 5.0 + 10.0 * a, 5.0 + 10.0 * b])
                u = rng.standard_normal(3)
                B = A + u / np.linalg.norm(u) * rng.uniform(0.7, 1.1)
                qa, qb = rng.standard_normal(4), rng.standard_normal(4)
                qa, qb = qa / np.linalg.norm(qa), qb / np.linalg.norm(qb)
                sa, sb = dict(zip(("back", "base"), _sites(A, qa))), dict(zip(("back", "base"), _sites(B, qb)))
                if all(np.linalg.norm(sa[x] - sb[y]) >= 0.85 * sig[(x, y)] for (x, y) in sig):
                    break
            if shift_rng is not None:
                while True:
                    ka, kb = shift_rng.integers(-2, 3, 3), shift_rng.integers(-2, 3, 3)
                    if np.any(ka != kb):
                        break
                A, B = A + box * ka, B + box * kb
            pos += [A, B]
            quat += [qa, qb]
    return np.array(pos), np.array(quat)


def test_mixed_precision_across_periodic_images():
    """Pairs whose unwrapped coordinates lie in different periodic images (a strand that has
    crossed the box face, or drifted by whole box sides) keep the mixed-precision accuracy of
    pairs in one image: the high parts of such coordinates differ by box sides and their FP32
    difference rounds at the ulp of the box side, which the kernel recovers exactly."""
    from oxdna_gb300 import MDSystem, dna2_settings, md_settings
    from oxdna_gb300 import io as oxio
    box = 150.0
    errs = {}
    for shift in (False, True):
        pos, quat = _contact_pairs(np.random.default_rng(11), box, np.random.default_rng(13) if shift else None)
        N = pos.shape[0]
        typ = np.random.default_rng(12).integers(0, 4, N).astype(np.int32)
        minus = -np.ones(N, np.int32)
        top = oxio.Topology(minus, minus, typ, typ, np.arange(N, dtype=np.int32), N)
        out = []
        for precision in ("mixed", "double"):
            m = MDSystem(box, top, dna2_settings(0.1, 0.5), md_settings(precision=precision))
            m.set_state(pos, quat, np.zeros((N, 3)), np.zeros((N, 3)))
            out.append(m.compute_forces())
            m.close()
        (Fm, Tm, _, Esm), (Fd, Td, _, Esd) = out
        errs[shift] = force_errors(Fm, Fd) + force_errors(Tm, Td)
        print(f"images {'shifted' if shift else 'local'}: force max-rel {errs[shift][0]:.2e} norm {errs[shift][1]:.2e}; "
              f"torque max-rel {errs[shift][2]:.2e} norm {errs[shift][3]:.2e}; |F| max {np.abs(Fd).max():.3g}")
        assert errs[shift][1] <= 1e-5 and errs[shift][3] <= 1e-5
        assert errs[shift][0] <= 5e-5 and errs[shift][2] <= 5e-5
        assert np.abs(Esm - Esd).max() <= 1e-5 * max(1.0, np.abs(Esd).max())
    # the same contacts, so the shifted errors stay at the level of the local ones
    assert errs[True][0] <= 4 * errs[False][0] + 1e-6


@pytest.mark.parametrize("box", [7.5, 9.5])
def test_mixed_precision_small_boxes(box):
    """A 12-bp duplex in cubes of side 7.5 and 9.5, just above the list's limit of 2 r_verlet
    (6.73 at salt 0.5, skin 0.05): three cells per side, the 27 cells of a scan are the whole
    grid, and Debye-Hueckel acts across the faces; the mixed path against the FP64 path."""
    from oxdna_gb300 import MDSystem, dna2_settings, md_settings
    from oxdna_gb300 import generate as G
    from oxdna_gb300 import io as oxio
    s = G.system_for_config(0, seed=3)
    a1, a2, a3 = s.frames()
    quat = oxio.frame_to_quat(a1, a2, a3)
    out = []
    for precision in ("mixed", "double"):
        m = MDSystem(box, s.top, dna2_settings(s.T, 0.5), md_settings(precision=precision))
        m.set_state(s.pos, quat, s.vel, s.L)
        out.append(m.compute_forces())
        m.close()
    (Fm, Tm, _, Esm), (Fd, Td, _, Esd) = out
    fmax, fnorm = force_errors(Fm, Fd)
    tmax, tnorm = force_errors(Tm, Td)
    print(f"box {box}: force max-rel {fmax:.2e} norm {fnorm:.2e}; torque max-rel {tmax:.2e} norm {tnorm:.2e}; "
          f"E_DH {Esd[:, 7].sum() if Esd.ndim == 2 else Esd[7]:.4g}")
    assert fnorm <= 1e-5 and tnorm <= 1e-5
    assert fmax <= 5e-5 and tmax <= 5e-5
    assert np.abs(Esm - Esd).max() <= 1e-5 * max(1.0, np.abs(Esd).max())
