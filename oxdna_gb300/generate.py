"""Seeded synthetic oxDNA systems (host side, numpy only).

Building blocks:
* `duplex(seq)`: an ideal right-handed B helix (rise 0.3897, twist 34.8 deg per base pair),
  nucleotide centres at radius 0.6 from the axis with a1 pointing at the axis, so paired base
  sites sit 0.4 apart (the hydrogen-bond r0) and a3 points towards the 5' neighbour, as in
  the reference's configurations;
* `hairpin(stem_seq, loop_len)`: a stem duplex whose two halves are joined by a loop laid on a
  circular arc with backbone sites one FENE r0 apart;
* `random_walk_strand(n)`: a self-avoiding random walk of backbone sites one FENE r0 apart,
  frames carried along the chain with a small random twist (centres end up ~0.7 apart).

`place(...)` drops copies at random positions and orientations in a periodic cube, rejecting
overlaps, and `system_for_config(...)` builds the five benchmark/parity workloads.  All the
geometry is in double precision; the result is a `System` that converts to and from the
oxDNA topology/configuration files in oxdna_gb300.io.
"""

from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import io as oxio

RISE = 0.3897
TWIST = math.radians(34.8)
CENTRE_RADIUS = 0.6
FENE_R0 = 0.7564
BACK1, BACK2 = -0.34, 0.3408  # grooved backbone offsets along a1 and a2

COMPLEMENT = {"A": "T", "T": "A", "G": "C", "C": "G"}


@dataclasses.dataclass
class Molecule:
    pos: np.ndarray  # [n, 3]
    a1: np.ndarray
    a3: np.ndarray
    seq: str  # one letter per nucleotide, in index order
    strands: List[Tuple[int, int, bool]]  # (first index, length, circular); 5'->3' = increasing index


@dataclasses.dataclass
class System:
    box: float
    pos: np.ndarray
    a1: np.ndarray
    a3: np.ndarray
    vel: np.ndarray
    L: np.ndarray
    top: oxio.Topology
    T: float = 0.1

    @property
    def N(self) -> int:
        return int(self.pos.shape[0])

    def frames(self):
        return oxio.orthonormal_frame(self.a1, self.a3)

    def quats(self) -> np.ndarray:
        a1, a2, a3 = self.frames()
        return oxio.frame_to_quat(a1, a2, a3)

    def write(self, top_path: str, conf_path: str) -> None:
        oxio.write_topology(top_path, self.top)
        oxio.write_conf(conf_path, oxio.Configuration(0, np.array([self.box] * 3), self.pos, self.a1, self.a3,
                                                      self.vel, self.L))


def random_sequence(rng: np.random.Generator, n: int) -> str:
    return "".join(rng.choice(list("ACGT"), size=n))


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _helix_strand(n: int, phase0: float, z0: float, up: bool):
    """Centres and frames of one strand of the ideal helix, nucleotide k at height z0 +- k*rise."""
    pos = np.zeros((n, 3))
    a1 = np.zeros((n, 3))
    a3 = np.zeros((n, 3))
    for k in range(n):
        level = k if up else -k
        phi = phase0 + level * TWIST
        u = np.array([math.cos(phi), math.sin(phi), 0.0])
        z = z0 + level * RISE
        pos[k] = CENTRE_RADIUS * u + np.array([0.0, 0.0, z])
        a1[k] = -u
        a3[k] = np.array([0.0, 0.0, -1.0 if up else 1.0])
    return pos, a1, a3


def duplex(seq: str) -> Molecule:
    """Strand 1 (indices 0..n-1) runs 5'->3' up the axis; strand 2 (n..2n-1) runs down, its
    first nucleotide paired with strand 1's last."""
    n = len(seq)
    p1, a11, a31 = _helix_strand(n, 0.0, 0.0, True)
    top_phase = (n - 1) * TWIST + math.pi
    p2, a12, a32 = _helix_strand(n, top_phase, (n - 1) * RISE, False)
    comp = "".join(COMPLEMENT[c] for c in reversed(seq))
    pos = np.concatenate([p1, p2])
    pos -= pos.mean(axis=0)
    return Molecule(pos, np.concatenate([a11, a12]), np.concatenate([a31, a32]), seq + comp,
                    [(0, n, False), (n, n, False)])


def _frame_from(a1: np.ndarray, a3: np.ndarray) -> np.ndarray:
    return np.cross(a3, a1)


def _back_site(c, a1, a3):
    return c + BACK1 * a1 + BACK2 * _frame_from(a1, a3)


def hairpin(stem_seq: str, loop_len: int, rng: np.random.Generator) -> Molecule:
    """One strand: stem_seq up the helix, loop_len loop nucleotides, then the complement down."""
    s = len(stem_seq)
    p1, a11, a31 = _helix_strand(s, 0.0, 0.0, True)
    top_phase = (s - 1) * TWIST + math.pi
    p2, a12, a32 = _helix_strand(s, top_phase, (s - 1) * RISE, False)
    b_start = _back_site(p1[-1], a11[-1], a31[-1])
    b_end = _back_site(p2[0], a12[0], a32[0])
    chord_vec = b_end - b_start
    chord = np.linalg.norm(chord_vec)
    arc = (loop_len + 1) * FENE_R0
    # circle through both ends with arc length `arc`: solve 2 R sin(theta/2) = chord, R theta = arc
    lo, hi = 1e-6, 2 * math.pi - 1e-6
    for _ in range(200):
        th = 0.5 * (lo + hi)
        if arc * math.sin(th / 2) / (th / 2) > chord:
            lo = th
        else:
            hi = th
    th = 0.5 * (lo + hi)
    R = arc / th
    mid = 0.5 * (b_start + b_end)
    ex = chord_vec / chord
    ez = np.array([0.0, 0.0, 1.0])
    ez = ez - ex * np.dot(ez, ex)
    ez /= np.linalg.norm(ez)
    h = R * math.cos(th / 2)  # distance of the circle centre from the chord (centre below the arc)
    centre = mid - h * ez
    start_ang = math.atan2(np.dot(b_start - centre, ez), np.dot(b_start - centre, ex))
    end_ang = math.atan2(np.dot(b_end - centre, ez), np.dot(b_end - centre, ex))
    if end_ang > start_ang:
        end_ang -= 2 * math.pi
    lp = np.zeros((loop_len, 3))
    la1 = np.zeros((loop_len, 3))
    la3 = np.zeros((loop_len, 3))
    for k in range(loop_len):
        ang = start_ang + (end_ang - start_ang) * (k + 1) / (loop_len + 1)
        radial = math.cos(ang) * ex + math.sin(ang) * ez
        back = centre + R * radial
        tangent = -math.sin(ang) * ex + math.cos(ang) * ez  # direction of increasing angle (towards 5')
        a3 = tangent / np.linalg.norm(tangent)
        # bases point out of the loop plane, so that they never converge on the inner side
        a1 = np.cross(ex, ez)
        a1 = a1 - a3 * np.dot(a1, a3)
        a1 /= np.linalg.norm(a1)
        a2 = np.cross(a3, a1)
        lp[k] = back - BACK1 * a1 - BACK2 * a2
        la1[k] = a1
        la3[k] = a3
    comp = "".join(COMPLEMENT[c] for c in reversed(stem_seq))
    loop_seq = "".join(rng.choice(list("ACGT"), size=loop_len))
    pos = np.concatenate([p1, lp, p2])
    pos -= pos.mean(axis=0)
    n = 2 * s + loop_len
    return Molecule(pos, np.concatenate([a11, la1, a12]), np.concatenate([a31, la3, a32]), stem_seq + loop_seq + comp,
                    [(0, n, False)])


class _Occupancy:
    """Backbone sites placed so far, hashed on a grid of cells no smaller than the exclusion
    distance; periodic with minimum-image distances when a box side is given."""

    def __init__(self, cut: float, box: Optional[float] = None):
        self.cut = cut
        self.box = box
        self.n = max(1, int(box // cut)) if box else 0
        self.cs = box / self.n if box else cut
        self.cells = {}

    def _key(self, p):
        if self.box:
            return tuple(int(np.floor((c % self.box) / self.cs)) % self.n for c in p)
        return tuple(int(np.floor(c / self.cs)) for c in p)

    def free(self, p, skip_tag) -> bool:
        k = self._key(p)
        c2 = self.cut * self.cut
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    kk = (k[0] + dx, k[1] + dy, k[2] + dz)
                    if self.box:
                        kk = (kk[0] % self.n, kk[1] % self.n, kk[2] % self.n)
                    for (x, y, z, tag) in self.cells.get(kk, ()):
                        if tag == skip_tag:
                            continue
                        d0, d1, d2 = x - p[0], y - p[1], z - p[2]
                        if self.box:
                            d0 -= self.box * round(d0 / self.box)
                            d1 -= self.box * round(d1 / self.box)
                            d2 -= self.box * round(d2 / self.box)
                        if d0 * d0 + d1 * d1 + d2 * d2 < c2:
                            return False
        return True

    def add(self, p, tag):
        self.cells.setdefault(self._key(p), []).append((float(p[0]), float(p[1]), float(p[2]), tag))

    def remove(self, p, tag):
        cell = self.cells.get(self._key(p), [])
        for k, e in enumerate(cell):
            if e[3] == tag:
                del cell[k]
                return


def random_walk_strand(n: int, rng: np.random.Generator, step: float = FENE_R0, min_sep: float = 0.8,
                       occ: Optional[_Occupancy] = None, start: Optional[np.ndarray] = None,
                       strand_tag: int = 0) -> Molecule:
    """Self-avoiding random walk of the backbone sites with steps of one FENE r0 (so every
    backbone bond starts unstretched; nucleotide centres end up ~0.7 apart).  a3 points back
    along the walk (towards the 5' neighbour); a1 is carried along by parallel transport with
    a small random twist, and each centre sits at back - (BACK1 a1 + BACK2 a2).  A step is
    redrawn unless its backbone and base sites keep min_sep from every site placed before
    (bonded predecessor excepted) and clear the bonded excluded-volume ranges of the
    predecessor.  With a shared occupancy `occ` (periodic for a melt of many strands) the walk
    avoids every strand grown before; positions are then absolute and not recentred."""
    own = occ is None
    if own:
        occ = _Occupancy(min_sep)
    back = np.zeros((n, 3))
    a1 = np.zeros((n, 3))
    a3 = np.zeros((n, 3))

    def frame(t, v_prev):
        v = v_prev - t * np.dot(v_prev, t)
        v /= np.linalg.norm(v)
        w = np.cross(t, v)
        ang = rng.uniform(-0.3, 0.3)
        return math.cos(ang) * v + math.sin(ang) * w

    def base_of(i_back, i_a1, i_a3):
        return i_back + (0.4 - BACK1) * i_a1 - BACK2 * np.cross(i_a3, i_a1)

    if start is not None:
        back[0] = start
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    a3[0] = -d
    a1[0] = frame(a3[0], np.cross(a3[0], rng.normal(size=3)))
    occ.add(back[0], (strand_tag, 0))
    occ.add(base_of(back[0], a1[0], a3[0]), (strand_tag, 0))
    i, backtracks = 1, 0
    while i < n:
        ok = False
        for attempt in range(1000):
            trial = d + (0.25 + 0.002 * attempt) * rng.normal(size=3)
            trial /= np.linalg.norm(trial)
            p = back[i - 1] + step * trial
            t3 = -trial
            t1 = frame(t3, a1[i - 1])
            bi = base_of(p, t1, t3)
            bprev = base_of(back[i - 1], a1[i - 1], a3[i - 1])
            if np.linalg.norm(bi - bprev) > 0.45 and np.linalg.norm(bi - back[i - 1]) > 0.6 and \
                    np.linalg.norm(p - bprev) > 0.6 and occ.free(p, (strand_tag, i - 1)) and occ.free(bi, (strand_tag, i - 1)):
                ok = True
                break
        if not ok:
            # a dead end (every trial overlaps a site placed before): take back the last few
            # nucleotides, or move the start if the walk is stuck at it, and grow again
            backtracks += 1
            if backtracks > 100000:
                raise RuntimeError("self-avoiding walk: no room left in the box")
            b = min(i, int(rng.integers(5, 25)))
            for j in range(i - b, i):
                occ.remove(back[j], (strand_tag, j))
                occ.remove(base_of(back[j], a1[j], a3[j]), (strand_tag, j))
            i -= b
            if i == 0:
                for _ in range(100000):
                    back[0] = rng.uniform(0, occ.box, size=3) if occ.box else back[0] + rng.normal(size=3)
                    d = rng.normal(size=3)
                    d /= np.linalg.norm(d)
                    a3[0] = -d
                    a1[0] = frame(a3[0], np.cross(a3[0], rng.normal(size=3)))
                    if occ.free(back[0], None) and occ.free(base_of(back[0], a1[0], a3[0]), None):
                        break
                else:
                    raise RuntimeError("self-avoiding walk: no room left in the box")
                occ.add(back[0], (strand_tag, 0))
                occ.add(base_of(back[0], a1[0], a3[0]), (strand_tag, 0))
                i = 1
                continue
            d = -a3[i - 1]
            continue
        back[i], a3[i], a1[i] = p, t3, t1
        d = trial
        occ.add(p, (strand_tag, i))
        occ.add(base_of(p, t1, t3), (strand_tag, i))
        i += 1
    a2 = np.cross(a3, a1)
    pos = back - (BACK1 * a1 + BACK2 * a2)
    if own:
        pos -= pos.mean(axis=0)
    return Molecule(pos, a1, a3, random_sequence(rng, n), [(0, n, False)])


def random_walk_melt(n_strands: int, n: int, box: float, rng: np.random.Generator, min_sep: float = 0.8) -> List[Molecule]:
    """n_strands self-avoiding strands of n nucleotides grown one after the other in a periodic
    cube, each avoiding every backbone site already placed."""
    occ = _Occupancy(min_sep, box)
    mols = []
    for k in range(n_strands):
        for _ in range(10000):
            start = rng.uniform(0, box, size=3)
            if occ.free(start, None):
                break
        mols.append(random_walk_strand(n, rng, occ=occ, start=start, strand_tag=k + 1))
    return mols


def _rotate(m: Molecule, R: np.ndarray, shift: np.ndarray) -> Molecule:
    return Molecule(m.pos @ R.T + shift, m.a1 @ R.T, m.a3 @ R.T, m.seq, m.strands)


def _sites(m: Molecule) -> np.ndarray:
    """backbone and base sites of every nucleotide (grooved backbone), shape [2n, 3]"""
    a1 = m.a1 / np.linalg.norm(m.a1, axis=1, keepdims=True)
    a3 = m.a3 / np.linalg.norm(m.a3, axis=1, keepdims=True)
    a2 = np.cross(a3, a1)
    back = m.pos + BACK1 * a1 + BACK2 * a2
    base = m.pos + 0.4 * a1
    return np.concatenate([back, base])


def place(molecules: Sequence[Molecule], box: float, rng: np.random.Generator, min_dist: float = 0.9,
          max_tries: int = 2000) -> List[Molecule]:
    """Random centres and orientations in a periodic cube.  A copy is rejected if any of its
    backbone or base sites comes within min_dist (minimum image) of a site of a molecule placed
    before, so different molecules start outside every excluded-volume range (at most 0.71)."""
    placed: List[Molecule] = []
    occ = _Occupancy(min_dist, box)
    for k, m in enumerate(molecules):
        for _ in range(max_tries):
            R = random_rotation(rng)
            shift = rng.uniform(0, box, size=3)
            cand = _rotate(m, R, shift)
            sites = _sites(cand)
            if all(occ.free(p, None) for p in sites):
                for p in sites:
                    occ.add(p, k)
                placed.append(cand)
                break
        else:
            raise RuntimeError("could not place a molecule without overlaps; lower the density")
    return placed


def assemble(mols: Sequence[Molecule], box: float, T: float, rng: np.random.Generator,
             thermal: bool = True) -> System:
    pos, a1, a3, seq = [], [], [], []
    n3, n5, strand = [], [], []
    off = 0
    s_id = 0
    for m in mols:
        n = m.pos.shape[0]
        pos.append(m.pos)
        a1.append(m.a1)
        a3.append(m.a3)
        seq.append(m.seq)
        loc3 = np.full(n, -1)
        loc5 = np.full(n, -1)
        sid = np.zeros(n, int)
        for (f, ln, circ) in m.strands:
            for k in range(ln):
                i = f + k
                sid[i] = s_id
                if k > 0:
                    loc5[i] = off + i - 1
                if k < ln - 1:
                    loc3[i] = off + i + 1
            if circ:
                loc3[f + ln - 1] = off + f
                loc5[f] = off + f + ln - 1
            s_id += 1
        n3.append(loc3)
        n5.append(loc5)
        strand.append(sid)
        off += n
    seqs = "".join(seq)
    btype = np.array([oxio.BASE_CODE[c] for c in seqs], np.int32)
    top = oxio.Topology(np.concatenate(n3).astype(np.int32), np.concatenate(n5).astype(np.int32), btype,
                        btype.copy(), np.concatenate(strand).astype(np.int32), s_id)
    P = np.concatenate(pos)
    N = P.shape[0]
    if thermal:
        vel = rng.normal(size=(N, 3)) * math.sqrt(T)
        Lm = rng.normal(size=(N, 3)) * math.sqrt(T)
    else:
        vel = np.zeros((N, 3))
        Lm = np.full((N, 3), 1e-3)
    return System(box, P, np.concatenate(a1), np.concatenate(a3), vel, Lm, top, T)


def kelvin(T_K: float) -> float:
    return T_K * 0.1 / 300.0


def system_for_config(idx: int, seed: int = 1, scale: float = 1.0) -> System:
    """The five workloads: 0 = one 12-bp duplex in a cube of side 20; 1 = 1000 x 20-bp duplexes at
    0.01 nucleotides/unit^3; 2 = 250 x 1000-nt self-avoiding random-walk strands grown in the cube
    at 0.02 (scale shrinks the duplex or strand count); 3 = the 40,000-nt system of workload 1;
    4 is batched (see batched_systems)."""
    rng = np.random.default_rng(seed)
    T = kelvin(300.0)
    if idx == 0:
        m = duplex(random_sequence(rng, 12))
        return assemble(place([m], 20.0, rng), 20.0, T, rng)
    if idx in (1, 3):
        n_dup = max(1, int(round(1000 * scale)))
        N = 40 * n_dup
        box = (N / 0.01) ** (1.0 / 3.0)
        mols = [duplex(random_sequence(rng, 20)) for _ in range(n_dup)]
        return assemble(place(mols, box, rng), box, T, rng)
    if idx == 2:
        n_str = max(1, int(round(250 * scale)))
        N = 1000 * n_str
        box = (N / 0.02) ** (1.0 / 3.0)
        return assemble(random_walk_melt(n_str, 1000, box, rng), box, T, rng)
    raise ValueError("workload 4 is batched: use batched_systems()")


def batched_systems(n_systems: int = 256, seed: int = 1, n_min: int = 16, n_max: int = 4000,
                    t_low: float = 280.0, t_high: float = 360.0) -> List[System]:
    """Independent systems with log-uniform sizes, each a random duplex or a hairpin, each in its
    own cube at 0.005 nucleotides/unit^3, temperatures on a geometric ladder."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_systems):
        target = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        if target <= 44 and rng.uniform() < 0.5:
            # hairpin: stem 6-12 bp and loop 4-20 nt, sized to the drawn total where possible
            stem = int(np.clip((target - 4) // 2, 6, 12))
            loop = int(np.clip(target - 2 * stem, 4, 20))
            mols = [hairpin(random_sequence(rng, stem), loop, rng)]
        else:
            # duplex of target/2 bp (8-2000); one longer than the cube cannot be laid straight
            # in it, so long ones are built as fragments of at most 50 bp
            nbp = int(np.clip(target // 2, 8, 2000))
            frags = [50] * (nbp // 50) + ([nbp % 50] if nbp % 50 else [])
            if len(frags) > 1 and frags[-1] < 8:
                frags[-2] -= 8 - frags[-1]
                frags[-1] = 8
            mols = [duplex(random_sequence(rng, f)) for f in frags]
        n = sum(m.pos.shape[0] for m in mols)
        box = (n / 0.005) ** (1.0 / 3.0)
        box = max(box, float(max(np.ptp(m.pos, axis=0).max() for m in mols)) + 8.0)
        T_K = t_low * (t_high / t_low) ** (k / (n_systems - 1)) if n_systems > 1 else t_low
        T = kelvin(T_K)
        out.append(assemble(place(mols, box, rng), box, T, rng))
    return out
