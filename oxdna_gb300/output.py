"""Simulation output in the reference's file formats, from an engine's FP64 energies and state.

The reference prints, every print_energy_every steps, the energy file of MDBackend's default
observables (src/Backends/MDBackend.cpp:71-76: the time in MD units, then the total_energy
observable's potential, kinetic and total energy per particle,
src/Observables/TotalEnergy.cpp:32-38), and every print_conf_interval steps a configuration
appended to the trajectory (src/Observables/Configurations/Configuration.cpp:85-140: "t = step",
"b = box", "E = Etot U K" per particle, then position, a1, a3, velocity and angular momentum
per nucleotide, 15 significant digits), plus the last configuration at the end.  With
back_in_box (the reference's default for trajectories) every strand is shifted by whole box
sides so that its centre of mass lies in the box.

`run_with_output` advances an MDSystem in chunks between printing steps: the dynamics inside a
chunk runs as CUDA graphs on the device, and each print reads the FP64 energies (device sums,
one small copy) and, for configurations, the state (one packed copy).
"""

from __future__ import annotations

from typing import Optional

import numpy as np

from . import io as oxio


def _energy_line(t_md: float, U: float, K: float) -> str:
    return f"{t_md:.6g} {U:.6f} {K:.6f} {U + K:.6f}\n"


def _strand_shift(pos: np.ndarray, strand: np.ndarray, box: float) -> np.ndarray:
    """per nucleotide, the whole box sides that bring its strand's centre of mass into the box"""
    n = int(strand.max()) + 1 if strand.size else 0
    com = np.zeros((n, 3))
    np.add.at(com, strand, pos)
    com /= np.maximum(np.bincount(strand, minlength=n), 1)[:, None]
    return -np.floor(com / box)[strand] * box


class Output:
    """Energy file, trajectory and last configuration of one system (system k of a batch with
    offsets; k = 0 for a plain engine)."""

    def __init__(self, sysm, top: oxio.Topology, box: float, dt: float, energy_file: Optional[str] = None,
                 trajectory_file: Optional[str] = None, lastconf_file: Optional[str] = None,
                 back_in_box: bool = True, system: int = 0):
        self.sysm, self.top, self.box, self.dt = sysm, top, float(box), float(dt)
        self.k = int(system)
        self.back_in_box = back_in_box
        self.energy_file, self.trajectory_file, self.lastconf_file = energy_file, trajectory_file, lastconf_file
        for f in (energy_file, trajectory_file):
            if f:
                open(f, "w").close()

    def _slice(self):
        off = getattr(self.sysm, "offsets", None)
        if off is None or len(off) <= 2:
            return slice(None)
        return slice(int(off[self.k]), int(off[self.k + 1]))

    def _energies(self):
        U, Kt, Kr = self.sysm.energies()
        U, Kt, Kr = (float(np.atleast_1d(x)[self.k]) for x in (U, Kt, Kr))
        n = self.top.N
        return U / n, (Kt + Kr) / n

    def print_energy(self, step: int):
        U, K = self._energies()
        if self.energy_file:
            with open(self.energy_file, "a") as fh:
                fh.write(_energy_line(step * self.dt, U, K))
        return U, K

    def _conf(self, step: int) -> str:
        st = self.sysm.get_state()
        sl = self._slice()
        pos, quat, vel, L = st["pos"][sl], st["quat"][sl], st["vel"][sl], st["Lmom"][sl]
        if self.back_in_box:
            pos = pos + _strand_shift(pos, np.asarray(self.top.strand), self.box)
        a1, _, a3 = oxio.quat_to_frame(quat)
        U, K = self._energies()
        lines = [f"t = {int(step)}\n", "b = %.15g %.15g %.15g\n" % (self.box, self.box, self.box),
                 "E = %.15g %.15g %.15g\n" % (U + K, U, K)]
        rows = np.concatenate([pos, a1, a3, vel, L], axis=1)
        lines += [" ".join("%.15g" % x for x in r) + "\n" for r in rows]
        return "".join(lines)

    def print_conf(self, step: int):
        if self.trajectory_file:
            with open(self.trajectory_file, "a") as fh:
                fh.write(self._conf(step))

    def print_last_conf(self, step: int):
        if self.lastconf_file:
            with open(self.lastconf_file, "w") as fh:
                fh.write(self._conf(step))


def run_with_output(sysm, steps: int, out: Output, print_energy_every: int = 0, print_conf_interval: int = 0,
                    start_step: int = 0) -> int:
    """Runs `steps` MD steps printing energies every print_energy_every steps and
    configurations every print_conf_interval steps (0: never), both at the first step as the
    reference does (SimManager prints before its step loop), and the last configuration at the
    end; returns the final step."""
    marks = [m for m in (print_energy_every, print_conf_interval) if m > 0]
    step = start_step
    end = start_step + steps

    def prints(s):
        if print_energy_every > 0 and s % print_energy_every == 0:
            out.print_energy(s)
        if print_conf_interval > 0 and s % print_conf_interval == 0:
            out.print_conf(s)

    prints(step)
    while step < end:
        nxt = end
        for m in marks:
            nxt = min(nxt, (step // m + 1) * m)
        sysm.run(nxt - step)
        step = nxt
        if step < end or any(step % m == 0 for m in marks):
            prints(step)
    out.print_last_conf(step)
    return step
