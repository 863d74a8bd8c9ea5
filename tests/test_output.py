"""Output in the reference's formats (oxdna_gb300.output), with a stand-in engine (no GPU):
the print schedule of run_with_output, the energy-file columns, and trajectory frames that
io.read_conf reads back (strands brought into the box by whole box sides)."""
import numpy as np

from oxdna_gb300 import io as oxio
from oxdna_gb300 import output


class FakeEngine:
    def __init__(self, N, box):
        rng = np.random.default_rng(1)
        self.pos = rng.uniform(-box, 2 * box, (N, 3))
        q = rng.normal(size=(N, 4))
        self.quat = q / np.linalg.norm(q, axis=1)[:, None]
        self.vel = rng.normal(size=(N, 3))
        self.L = rng.normal(size=(N, 3))
        self.runs = []
        self.step = 0

    def run(self, n):
        self.runs.append(n)
        self.step += n
        self.pos = self.pos + 0.001 * n

    def energies(self):
        return -1.5 * len(self.pos) + self.step * 1e-3, 0.15 * len(self.pos), 0.15 * len(self.pos)

    def get_state(self):
        return dict(pos=self.pos.copy(), quat=self.quat.copy(), vel=self.vel.copy(), Lmom=self.L.copy())


def test_schedule_formats_and_read_back(tmp_path):
    N, box = 10, 7.0
    top = oxio.Topology(np.array([1, 2, 3, 4, -1, 6, 7, 8, 9, -1], np.int32), np.array([-1, 0, 1, 2, 3, -1, 5, 6, 7, 8], np.int32),
                        np.zeros(N, np.int32), np.zeros(N, np.int32), np.array([0] * 5 + [1] * 5, np.int32), 2)
    eng = FakeEngine(N, box)
    e, t, lc = str(tmp_path / "energy.dat"), str(tmp_path / "traj.dat"), str(tmp_path / "last.dat")
    out = output.Output(eng, top, box, 0.005, energy_file=e, trajectory_file=t, lastconf_file=lc)
    end = output.run_with_output(eng, 250, out, print_energy_every=40, print_conf_interval=100)
    assert end == 250 and sum(eng.runs) == 250
    assert eng.runs == [40, 40, 20, 20, 40, 40, 40, 10]
    rows = np.loadtxt(e)
    assert rows.shape == (7, 4)
    np.testing.assert_allclose(rows[:, 0], np.arange(0, 250, 40) * 0.005)
    np.testing.assert_allclose(rows[:, 3], rows[:, 1] + rows[:, 2], atol=2e-6)
    frames = open(t).read().count("t = ")
    assert frames == 3
    last = oxio.read_conf(lc)
    assert last.t == 250 and np.allclose(last.box, box)
    # strands shifted by whole box sides, their centres of mass inside the box
    shift = last.pos - eng.pos
    assert np.allclose(shift / box, np.round(shift / box))
    for s in (0, 1):
        com = last.pos[top.strand == s].mean(axis=0)
        assert np.all(com >= 0) and np.all(com < box)
    a1, _, a3 = oxio.quat_to_frame(eng.quat)
    assert np.allclose(last.a1, a1) and np.allclose(last.a3, a3) and np.allclose(last.vel, eng.vel)
