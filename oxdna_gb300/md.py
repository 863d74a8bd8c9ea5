"""Host-side front end of the MD backend (oxgb_md_* in include/oxgb.h).

`MDSystem` mirrors the reference's MD backend life cycle -- get_settings (keyword arguments
named after the input keys), init (topology + configuration upload), sim_step (run) and
apply_simulation_data_changes (state download) -- on top of the C ABI.
"""

from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _abi
from . import io as oxio


def dna2_settings(T: float, salt: float = 0.5, average: bool = True, seq: Optional[dict] = None,
                  hb_multiplier: float = 1.0, half_charged_ends: bool = True, dh_lambda: float = 0.3616455,
                  dh_strength: float = 0.0543, mbf_fmax: Optional[float] = None, mbf_finf: float = 0.04,
                  reference_cuda_eps: bool = False) -> _abi.DNA2Settings:
    s = _abi.DNA2Settings()
    _abi.lib().oxgb_dna2_default_settings(C.byref(s), float(T), float(salt))
    s.average = 1 if average else 0
    if seq is not None:
        order = "AGCT"
        for i in range(4):
            for j in range(4):
                s.seq_stck[i][j] = seq[f"STCK_{order[i]}_{order[j]}"]
        s.seq_stck_fact_eps = seq["STCK_FACT_EPS"]
        s.seq_hydr_at = seq.get("HYDR_A_T", seq.get("HYDR_T_A"))
        s.seq_hydr_gc = seq.get("HYDR_G_C", seq.get("HYDR_C_G"))
    s.hb_multiplier = hb_multiplier
    s.dh_half_charged_ends = 1 if half_charged_ends else 0
    s.dh_lambda = dh_lambda
    s.dh_strength = dh_strength
    if mbf_fmax is not None:
        s.use_mbf = 1
        s.mbf_fmax = mbf_fmax
        s.mbf_finf = mbf_finf
    s.reference_cuda_eps = 1 if reference_cuda_eps else 0
    return s


# the neighbour-row kernels of the list build (OXGB_LIST_*): identical rows, different speeds
LIST_KERNELS = {"auto": 0, "warp": 1, "thread": 2, "group4": 3, "group8": 4, "group16": 5}


def md_settings(dt: float = 0.003, verlet_skin: float = 0.05, thermostat: str = "no", newtonian_steps: int = 103,
                pt: float = 0.0, diff_coeff: float = 2.5, bussi_tau: float = 1000.0, seed: int = 1,
                precision: str = "mixed", cells_auto_optimisation: bool = True, max_neigh: int = 0,
                steps_per_graph: int = 16, list_rebuild_node: str = "conditional", sort_every: int = 0,
                autotune: bool = False, use_edge: bool = False, sort_order: str = "hilbert",
                list_kernel: str = "auto") -> _abi.MDSettings:
    m = _abi.MDSettings()
    _abi.lib().oxgb_md_default_settings(C.byref(m))
    m.dt = dt
    m.verlet_skin = verlet_skin
    m.thermostat = _abi.THERMOSTATS[thermostat]
    m.newtonian_steps = newtonian_steps
    m.pt = pt
    m.diff_coeff = diff_coeff
    m.bussi_tau = bussi_tau
    m.seed = seed
    m.precision = {"mixed": 0, "double": 1, "float": 2}[precision]
    m.cells_auto_optimisation = 1 if cells_auto_optimisation else 0
    m.max_neigh = max_neigh
    m.steps_per_graph = steps_per_graph
    m.list_rebuild_node = {"conditional": 0, "kernel": 1}[list_rebuild_node]
    m.sort_every = sort_every
    m.autotune = 1 if autotune else 0
    m.use_edge = 1 if use_edge else 0
    m.sort_order = {"hilbert": 0, "cells": 1}[sort_order]
    m.list_kernel = LIST_KERNELS[list_kernel]
    return m


def force_shapes():
    """the autotuner's shape table: (pair_npw, nb_lanes, nb_min_blocks) of shape 0, 1, ..."""
    out, k = [], 0
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    while _abi.lib().oxgb_force_shape_table(k, C.byref(a), C.byref(b), C.byref(c)) == 0:
        out.append((a.value, b.value, c.value))
        k += 1
    return out


class MDSystem:
    """One system -- or a batch of independent systems -- on the GPU: topology, FP64 state,
    Verlet lists, integrator and thermostat.

    A batch is given as lists: `box`, `top` and `dna` hold one entry per system.  Its systems are
    packed one after the other (per-nucleotide arrays of `set_state`/`get_state` are the
    concatenation, system k at rows `offsets[k]:offsets[k + 1]`); each keeps its own box,
    temperature, cutoff, cell grid, Verlet lists and thermostat, and its random stream uses the
    seed `md.seed + k`.  Per-system results (energies, energy split) come back per system.
    """

    def __init__(self, box, top, dna, md: _abi.MDSettings):
        L = _abi.lib()
        boxes = [float(b) for b in box] if isinstance(box, (list, tuple, np.ndarray)) else [float(box)]
        tops = list(top) if isinstance(top, (list, tuple)) else [top]
        dnas = list(dna) if isinstance(dna, (list, tuple)) else [dna]
        if not (len(boxes) == len(tops) == len(dnas)):
            raise ValueError("box, top and dna need one entry per system")
        self.n_systems = len(tops)
        self.offsets = np.zeros(self.n_systems + 1, np.int32)
        for k, t in enumerate(tops):
            self.offsets[k + 1] = self.offsets[k] + t.N
        self.N = int(self.offsets[-1])
        self.box = boxes[0] if self.n_systems == 1 else np.array(boxes)
        dna_arr = (_abi.DNA2Settings * self.n_systems)(*dnas)
        h = C.c_void_p()
        _abi.check(L.oxgb_md_create(self.n_systems, self.offsets, np.array(boxes, np.float64), dna_arr, C.byref(md),
                                    C.byref(h)))
        self._h = h

        def cat(name, shift):
            parts = []
            for k, t in enumerate(tops):
                a = np.asarray(getattr(t, name), np.int32)
                parts.append(np.where(a >= 0, a + self.offsets[k], a) if shift else a)
            return np.ascontiguousarray(np.concatenate(parts), np.int32)

        _abi.check(L.oxgb_md_set_topology(h, cat("n3", True), cat("n5", True), cat("btype", False), cat("type", False)))

    def close(self):
        if self._h:
            _abi.lib().oxgb_md_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, pos, quat, vel, Lmom):
        c = lambda a: np.ascontiguousarray(a, np.float64).reshape(-1)
        _abi.check(_abi.lib().oxgb_md_set_state(self._h, c(pos), c(quat), c(vel), c(Lmom)))

    def get_state(self, out=None):
        """the FP64 state in the caller's order; `out` (a dict from an earlier call) is filled in
        place instead of allocating new arrays"""
        N = self.N
        if out is None:
            out = dict(pos=np.zeros((N, 3)), quat=np.zeros((N, 4)), vel=np.zeros((N, 3)), Lmom=np.zeros((N, 3)))
        for key, w in (("pos", 3), ("quat", 4), ("vel", 3), ("Lmom", 3)):
            a = out[key]
            if a.dtype != np.float64 or a.shape != (N, w) or not a.flags["C_CONTIGUOUS"]:
                raise ValueError(f"out[{key!r}] must be a C-contiguous float64 array of shape ({N}, {w})")
        _abi.check(_abi.lib().oxgb_md_get_state(self._h, _abi.ptr(out["pos"]), _abi.ptr(out["quat"]),
                                                _abi.ptr(out["vel"]), _abi.ptr(out["Lmom"])))
        return out

    def run(self, nsteps: int, sync: bool = True):
        _abi.check(_abi.lib().oxgb_md_run(self._h, int(nsteps), 1 if sync else 0))

    def compute_forces(self):
        """forces, torques, per-nucleotide energies and the 8-term energy split (per system for a
        batch) of the current state, from freshly built lists"""
        N = self.N
        F, T, E, Es = np.zeros((N, 3)), np.zeros((N, 3)), np.zeros(N), np.zeros(8 * self.n_systems)
        _abi.check(_abi.lib().oxgb_md_compute_forces(self._h, _abi.ptr(F), _abi.ptr(T), _abi.ptr(E), _abi.ptr(Es)))
        return F, T, E, (Es if self.n_systems == 1 else Es.reshape(self.n_systems, 8))

    def storage_order(self):
        """the caller's index of the nucleotide in each storage slot (the identity unless the
        engine sorts into cell order, md_settings(sort_every=...))"""
        out = np.zeros(self.N, np.int32)
        _abi.check(_abi.lib().oxgb_md_storage_order(self._h, _abi.ptr(out)))
        return out

    def get_forces(self):
        """forces, torques and per-nucleotide energies of the last step, not recomputed"""
        N = self.N
        F, T, E = np.zeros((N, 3)), np.zeros((N, 3)), np.zeros(N)
        _abi.check(_abi.lib().oxgb_md_get_forces(self._h, _abi.ptr(F), _abi.ptr(T), _abi.ptr(E)))
        return F, T, E

    def energies(self, potential: bool = True):
        """potential, translational and rotational kinetic energy (FP64 sums; arrays per system
        for a batch).  potential=False skips the force evaluation the potential energy needs and
        returns 0 for it."""
        n = self.n_systems
        U, Kt, Kr = np.zeros(n), np.zeros(n), np.zeros(n)
        _abi.check(_abi.lib().oxgb_md_energies(self._h, _abi.ptr(U) if potential else None, _abi.ptr(Kt), _abi.ptr(Kr)))
        if n == 1:
            return float(U[0]), float(Kt[0]), float(Kr[0])
        return U, Kt, Kr

    def set_temperature(self, T: float, k: int = 0):
        _abi.check(_abi.lib().oxgb_md_set_temperature(self._h, int(k), float(T)))

    def set_external_forces(self, forces):
        """External forces (oxgb_md_set_external_forces): a list of dicts with 'type' (constant /
        string, mutual_trap, trap / moving_trap, lowdim_trap, repulsion_plane, attraction_plane,
        sphere, sphere_smooth, LJ_wall, generic_central_force, repulsion_plane_moving, LJ_cone,
        twist, ellipsoid, com, yukawa_sphere, repulsive_sphere_moving), 'particle' and the
        parameters under the reference's external_forces_file keys ('ref_particle', 'F0',
        'rate', 'stiff', 'stiff_rate', 'r0', 'position', 'dir', 'pos0', 'center', 'r_ext',
        'smooth', 'alpha', 'sigma', 'n', 'only_repulsive', 'inner_cut_off', 'outer_cut_off',
        'base', 'axis', 'mask', 'r_1', 'r_2', 'com_list', 'ref_list', 'radius', 'WCA_epsilon',
        'WCA_sigma', 'WCA_n', 'debye_length', 'debye_A', 'cutoff', 'origin', 'target', 'steps',
        and 'dir_as_centre' / 'PBC' / 'visibility' for the flags; the reference's defaults where
        a key is left out).  Particle indices are global (offsets[k] + index within system k);
        repulsion_plane_moving takes one reference particle per record; a com record (lists of
        indices in com_list and ref_list) acts on every particle of its com_list, as the
        reference's COMForce does."""
        recs, groups = [], {}

        def group(members):
            key = tuple(int(x) for x in members)
            if key not in groups:
                groups[key] = len(groups)
            return groups[key]

        for d in forces:
            if d["type"] == "com":
                g_com, g_ref = group(d["com_list"]), group(d["ref_list"])
                for i in d["com_list"]:
                    recs.append((dict(d, particle=int(i)), g_com, g_ref))
            else:
                recs.append((d, -1, -1))
        arr = (_abi.ExtForce * max(1, len(recs)))()
        for m, (d, g_com, g_ref) in enumerate(recs):
            e = arr[m]
            t = d["type"]
            e.type = _abi.FORCE_TYPES[t]
            e.particle = int(d["particle"])
            e.ref_particle = int(d.get("ref_particle", -1))
            flags = 0
            if d.get("dir_as_centre") or d.get("PBC"):
                flags |= 1
            vis = d.get("visibility", (True, True, True))
            for bit, on in zip((2, 4, 8), vis):
                if on:
                    flags |= bit
            e.flags = flags
            stiff_default = 1.0 if t in ("LJ_wall", "LJ_cone") else 0.0
            for key in ("F0", "rate", "stiff_rate", "r0", "position"):
                setattr(e, key, float(d.get(key, 0.0)))
            e.stiff = float(d.get("stiff", stiff_default))
            pos0 = d.get("center", d.get("pos0", (0.0, 0.0, 0.0)))
            for c in range(3):
                e.dir[c] = float(d.get("dir", (0.0, 0.0, 0.0))[c])
                e.pos0[c] = float(pos0[c])
            e.n = int(d.get("n", 6))
            if t in ("sphere", "sphere_smooth"):
                e.cutoff = float(d.get("r_ext", 1e10))
                e.sigma = float(d.get("smooth", -1.0))
                e.p1 = float(d.get("alpha", -1.0))
                if t == "sphere_smooth":
                    e.r0 = float(d.get("r0", -1.0))
                if t == "sphere":
                    e.r0 = float(d.get("r0", -1.0))
            elif t in ("LJ_wall", "LJ_cone"):
                e.sigma = float(d.get("sigma", 1.0))
                e.cutoff = 2.0 ** (1.0 / e.n) if d.get("only_repulsive") else 1e6
                e.p1 = float(d.get("alpha", 0.0))
                if t == "LJ_wall":
                    e.position = float(d.get("position", -1.0))
            elif t == "generic_central_force":
                e.p1 = float(d.get("inner_cut_off", 0.0))
                e.p2 = float(d.get("outer_cut_off", 0.0))
            elif t == "twist":
                # ConstantRateTorque reads the start angle as 'base' and normalises the axis
                e.F0 = float(d.get("base", 0.0))
                axis = np.asarray(d["axis"], np.float64)
                axis = axis / np.linalg.norm(axis)
                centre, mask = d.get("center", (0.0, 0.0, 0.0)), d.get("mask", (0.0, 0.0, 0.0))
                for c in range(3):
                    e.dir[c], e.pos0[c] = float(axis[c]), float(d["pos0"][c])
                    e.v1[c], e.v2[c] = float(centre[c]), float(mask[c])
            elif t == "ellipsoid":
                r1, r2 = d.get("r_1", (1e-6, 1e-6, 1e-6)), d["r_2"]
                for c in range(3):
                    e.v1[c], e.v2[c] = float(r1[c]), float(r2[c])
            elif t == "com":
                e.n, e.ref_particle = g_com, g_ref
            elif t == "yukawa_sphere":
                e.r0 = float(d["radius"])
                e.stiff = float(d.get("WCA_epsilon", 1.0))
                e.sigma = float(d.get("WCA_sigma", 1.0))
                e.n = int(d.get("WCA_n", 6))
                e.p1 = e.sigma * 2.0 ** (1.0 / e.n)
                e.p2 = float(d["debye_length"])
                e.F0 = float(d["debye_A"])
                e.cutoff = float(d.get("cutoff", 4.0 * e.p2))
            elif t == "repulsive_sphere_moving":
                e.r0 = float(d["r0"])
                e.cutoff = float(d.get("r_ext", 1e10))
                centre = d.get("center", (0.0, 0.0, 0.0))
                origin, target = d.get("origin", centre), d.get("target", (0.0, 0.0, 0.0))
                e.p1 = float(int(d.get("steps", d.get("move_steps", 0))))
                for c in range(3):
                    e.v1[c], e.v2[c] = float(origin[c]), float(target[c])
        lib = _abi.lib()
        if groups:
            # the groups are replaced with no records pointing at them
            _abi.check(lib.oxgb_md_set_external_forces(self._h, 0, arr))
            members = [list(k) for k in sorted(groups, key=groups.get)]
            off = np.zeros(len(members) + 1, np.int32)
            off[1:] = np.cumsum([len(x) for x in members])
            flat = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int32) for x in members]), np.int32)
            _abi.check(lib.oxgb_md_set_force_groups(self._h, len(members), off.ctypes.data_as(C.c_void_p),
                                                    flat.ctypes.data_as(C.c_void_p)))
        _abi.check(lib.oxgb_md_set_external_forces(self._h, len(recs), arr))

    def scale_momenta(self, f: float, k: int = 0):
        _abi.check(_abi.lib().oxgb_md_scale_momenta(self._h, int(k), float(f)))

    def replica_exchange(self, temps, rng, parity: int = 0):
        """One round of parallel-tempering swaps between neighbouring rungs of a temperature
        ladder (oxdna_gb300.pt.swap_round).  temps[k] is the current temperature of system k;
        rungs (r, r + 1) with r of the given parity are tried with the Metropolis rule on the
        FP64 potential energies, min(1, exp((1/T_r - 1/T_r+1) (U_r - U_r+1))), one uniform
        draw from rng per tried pair; an accepted pair exchanges temperatures (tables,
        thermostat) and rescales its momenta by sqrt(T_new / T_old).  Returns the new
        temperatures and the number of accepted swaps."""
        from . import pt
        temps = np.asarray(temps, np.float64)
        U, _, _ = self.energies()
        draws = rng.uniform(size=pt.pairs_in_round(len(temps), parity))
        new, swaps = pt.swap_round(temps, np.atleast_1d(U), parity, draws)
        pt.apply_swaps(self, temps, swaps)
        return new, len(swaps)

    def neighbours(self):
        N = self.N
        nnb = np.zeros(N, np.int32)
        cell = np.zeros(N, np.int32)
        ns = C.c_int(0)
        mx = C.c_int(0)
        _abi.check(_abi.lib().oxgb_md_info(self._h, None, None, C.byref(mx)))
        nb = np.zeros(N * mx.value, np.int32)
        _abi.check(_abi.lib().oxgb_md_neighbours(self._h, _abi.ptr(nnb), _abi.ptr(nb), mx.value, _abi.ptr(cell),
                                                 C.byref(ns)))
        return nnb, nb.reshape(N, mx.value), cell, ns.value

    def force_shape(self):
        """the shape of the MD step's force kernels (autotuned with md_settings(autotune=True)):
        pair_npw, nb_lanes, nb_min_blocks and the measured launch time in microseconds"""
        a, b, c, t = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        _abi.check(_abi.lib().oxgb_md_force_shape(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(t)))
        out = dict(pair_npw=a.value, nb_lanes=b.value, nb_min_blocks=c.value, launch_us=t.value)
        out["index"] = next((k for k, sh in enumerate(force_shapes()) if sh == (a.value, b.value, c.value)), None)
        lk = C.c_int()
        _abi.check(_abi.lib().oxgb_md_list_kernel(self._h, C.byref(lk)))
        out["list_kernel"] = {v: k for k, v in LIST_KERNELS.items()}[lk.value]
        return out

    def set_force_shape(self, k: int):
        """pins shape k of the MD step's force kernels (0 the default)"""
        _abi.check(_abi.lib().oxgb_md_set_force_shape(self._h, int(k)))

    def info(self):
        r, s, m = C.c_longlong(0), C.c_longlong(0), C.c_int(0)
        _abi.check(_abi.lib().oxgb_md_info(self._h, C.byref(r), C.byref(s), C.byref(m)))
        return dict(rebuilds=r.value, step=s.value, max_neigh=m.value)

    @property
    def handle(self):
        return self._h

    @property
    def stream(self):
        return _abi.lib().oxgb_md_stream(self._h)
