"""The seeded workload generator: a crowded self-avoiding melt keeps every interaction site of a
nucleotide at least the exclusion distance from every site of every other nucleotide but its
bonded neighbour (dead ends are taken back and regrown, never accepted), and every backbone bond
starts unstretched."""
import numpy as np

from oxdna_gb300 import generate as G


def _sites(mols):
    out = []
    for m in mols:
        a1 = m.a1 / np.linalg.norm(m.a1, axis=1, keepdims=True)
        a3 = m.a3 / np.linalg.norm(m.a3, axis=1, keepdims=True)
        a2 = np.cross(a3, a1)
        back = m.pos + G.BACK1 * a1 + G.BACK2 * a2
        base = m.pos + 0.4 * a1
        out.append((back, base))
    return out


def test_crowded_melt_has_no_overlaps():
    rng = np.random.default_rng(5)
    n_str, n = 12, 150
    box = (n_str * n / 0.05) ** (1.0 / 3.0)  # 2.5 times the large workload's density
    mols = G.random_walk_melt(n_str, n, box, rng)
    sites = _sites(mols)
    back = np.concatenate([s[0] for s in sites])
    base = np.concatenate([s[1] for s in sites])
    nuc = np.arange(back.shape[0])
    strand = np.repeat(np.arange(n_str), n)
    pts = np.concatenate([back, base])
    owner = np.concatenate([nuc, nuc])
    for k in range(pts.shape[0]):
        d = pts - pts[k]
        d -= box * np.round(d / box)
        r = np.sqrt((d * d).sum(axis=1))
        # every other nucleotide except the bonded neighbours along the strand
        far = np.abs(owner - owner[k]) > 1
        far |= strand[owner] != strand[owner[k]]
        assert r[far].min() >= 0.8 - 1e-9, k
    # backbone bonds at the FENE rest length
    for s in sites:
        bond = np.linalg.norm(np.diff(s[0], axis=0), axis=1)
        assert np.allclose(bond, G.FENE_R0, atol=1e-9)


def test_walk_backs_out_of_a_dead_end():
    """A strand started inside a closed cage of occupied sites cannot grow: the walk takes its
    nucleotides back down to the start, moves the start and grows outside."""
    box = 20.0
    occ = G._Occupancy(0.8, box)
    c = np.array([10.0, 10.0, 10.0])
    k = np.arange(600) + 0.5
    th, ph = np.arccos(1 - 2 * k / 600), np.pi * (1 + 5 ** 0.5) * k
    cage = c + 1.6 * np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], axis=1)
    for q in cage:
        occ.add(q, ("cage", 0))
    m = G.random_walk_strand(40, np.random.default_rng(3), occ=occ, start=c.copy(), strand_tag=1)
    back = _sites([m])[0][0]
    d = back[:, None, :] - cage[None, :, :]
    d -= box * np.round(d / box)
    assert np.sqrt((d * d).sum(axis=2)).min() >= 0.8 - 1e-9
    assert np.linalg.norm(back[0] - c) > 1.0  # the start moved out of the cage
    assert np.allclose(np.linalg.norm(np.diff(back, axis=0), axis=1), G.FENE_R0, atol=1e-9)
