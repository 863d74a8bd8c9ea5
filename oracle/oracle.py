"""ORACLE (test infrastructure only): ctypes front end of the CPU FP64 restatement in
dna2_oracle.c.  Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
as the checker; the product package never imports it.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboxgb_oracle.so")
_lib = None

NTERMS = 8
TERM_NAMES = ("fene", "bonded_excl", "stacking", "nonbonded_excl", "hb", "cross_stacking", "coaxial_stacking",
              "debye_huckel")


class Settings(C.Structure):
    _fields_ = [
        ("T", C.c_double), ("salt", C.c_double), ("average", C.c_int),
        ("seq_stck", (C.c_double * 4) * 4), ("seq_stck_fact_eps", C.c_double),
        ("seq_hydr_at", C.c_double), ("seq_hydr_gc", C.c_double), ("hb_multiplier", C.c_double),
        ("dh_half_charged_ends", C.c_int), ("dh_lambda", C.c_double), ("dh_strength", C.c_double),
        ("use_mbf", C.c_int), ("mbf_fmax", C.c_double), ("mbf_finf", C.c_double),
    ]


_D2 = C.c_double * 2
_D255 = ((C.c_double * 5) * 5) * 2


class Params(C.Structure):
    _fields_ = [
        ("T", C.c_double), ("f1_eps", _D255), ("f1_shift", _D255),
        ("f1_a", _D2), ("f1_rc", _D2), ("f1_r0", _D2), ("f1_blow", _D2), ("f1_bhigh", _D2), ("f1_rlow", _D2),
        ("f1_rhigh", _D2), ("f1_rclow", _D2), ("f1_rchigh", _D2),
        ("f2_k", _D2), ("f2_rc", _D2), ("f2_r0", _D2), ("f2_blow", _D2), ("f2_rlow", _D2), ("f2_rclow", _D2),
        ("f2_bhigh", _D2), ("f2_rhigh", _D2), ("f2_rchigh", _D2),
        ("f4_a", C.c_double * 13), ("f4_b", C.c_double * 13), ("f4_t0", C.c_double * 13),
        ("f4_ts", C.c_double * 13), ("f4_tc", C.c_double * 13), ("f4_sa", C.c_double), ("f4_sb", C.c_double),
        ("f5_a", C.c_double * 4), ("f5_b", C.c_double * 4), ("f5_xc", C.c_double * 4), ("f5_xs", C.c_double * 4),
        ("hb_multiplier", C.c_double), ("dh_half_charged_ends", C.c_int),
        ("dh_prefactor", C.c_double), ("dh_rhigh", C.c_double), ("dh_rc", C.c_double), ("dh_b", C.c_double),
        ("dh_minus_kappa", C.c_double), ("dh_lambda", C.c_double),
        ("use_mbf", C.c_int), ("mbf_fmax", C.c_double), ("mbf_finf", C.c_double), ("mbf_xmax", C.c_double),
        ("fene_r0", C.c_double), ("rcut", C.c_double),
    ]


class MD(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("thermostat", C.c_int), ("newtonian_steps", C.c_int), ("pt", C.c_double),
        ("pr", C.c_double), ("bussi_tau", C.c_double), ("bussi_K_t", C.c_double), ("bussi_K_r", C.c_double),
        ("seed", C.c_ulonglong), ("verlet_skin", C.c_double),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle library (gcc, a few seconds)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        fp = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        L.oxo_params_init.argtypes = [C.POINTER(Settings), C.POINTER(Params)]
        L.oxo_params_init.restype = C.c_int
        L.oxo_forces.argtypes = [C.POINTER(Params), C.c_int, dp, dp, dp, dp, ip, ip, ip, ip, C.c_double,
                                 C.c_void_p, C.c_int, dp, dp, dp, dp, C.c_int]
        L.oxo_forces.restype = C.c_int
        L.oxo_pairs_within.argtypes = [C.c_int, dp, C.c_double, C.c_double, ip, C.c_long]
        L.oxo_pairs_within.restype = C.c_long
        L.oxo_order_params.argtypes = [C.POINTER(Params), dp, dp, dp, ip, ip, C.c_double, ip, ip, C.c_int, C.c_int, dp]
        L.oxo_order_params.restype = None
        L.oxo_verlet_f32.argtypes = [C.c_int, fp, C.c_float, C.c_float, ip, ip, C.c_int, C.POINTER(C.c_int), ip, ip,
                                     ip, C.c_int]
        L.oxo_verlet_f32.restype = C.c_int
        L.oxo_philox.argtypes = [C.c_uint] * 6 + [np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")]
        L.oxo_md_run.argtypes = [C.POINTER(Params), C.POINTER(MD), C.c_int, dp, dp, dp, dp, ip, ip, ip, ip, C.c_double,
                                 dp, dp, C.c_longlong, C.c_int, dp, C.c_int]
        L.oxo_md_run.restype = C.c_int
        _lib = L
    return _lib


def make_settings(T: float, salt: float = 0.5, average: bool = True, seq: Optional[dict] = None,
                  hb_multiplier: float = 1.0, half_charged_ends: bool = True, dh_lambda: float = 0.3616455,
                  dh_strength: float = 0.0543, mbf_fmax: Optional[float] = None, mbf_finf: float = 0.04) -> Settings:
    s = Settings()
    s.T = T
    s.salt = salt
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
    return s


def make_params(settings: Settings) -> Params:
    p = Params()
    rc = lib().oxo_params_init(C.byref(settings), C.byref(p))
    if rc != 0:
        raise ValueError(f"oracle parameter error {rc}")
    return p


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def forces(params: Params, pos, a1, a2, a3, n3, n5, typ, btype, L: float, pairs=None, nthreads: int = 1):
    """Forces (lab), torques (body), energy split [8] and per-particle energies."""
    N = int(np.asarray(pos).shape[0])
    F = np.zeros(3 * N)
    T = np.zeros(3 * N)
    Es = np.zeros(NTERMS)
    Ep = np.zeros(max(N, 1))
    if pairs is None:
        pp, npairs = None, -1
    else:
        parr = _c(pairs, np.int32).reshape(-1)
        pp, npairs = parr.ctypes.data_as(C.c_void_p), parr.size // 2
    rc = lib().oxo_forces(C.byref(params), N, _c(pos, np.float64).reshape(-1), _c(a1, np.float64).reshape(-1),
                          _c(a2, np.float64).reshape(-1), _c(a3, np.float64).reshape(-1), _c(n3, np.int32),
                          _c(n5, np.int32), _c(typ, np.int32), _c(btype, np.int32), float(L), pp, npairs, F, T, Es,
                          Ep, nthreads)
    return rc, F.reshape(N, 3), T.reshape(N, 3), Es, Ep[:N]


def order_params(params: Params, pos, a1, a3, typ, btype, L: float, op1, op2, mode: int) -> np.ndarray:
    """FFS order-parameter quantities of the pairs (op1[k], op2[k]) (oxo_order_params): mode 0
    hydrogen-bonding energy, 1 nearly-bonded flag (0/1), 2 base-base distance."""
    op1, op2 = _c(op1, np.int32), _c(op2, np.int32)
    out = np.zeros(op1.size)
    lib().oxo_order_params(C.byref(params), _c(pos, np.float64).reshape(-1), _c(a1, np.float64).reshape(-1),
                           _c(a3, np.float64).reshape(-1), _c(typ, np.int32), _c(btype, np.int32), float(L), op1, op2,
                           int(op1.size), int(mode), out)
    return out


def pairs_within(pos, L: float, rc: float) -> np.ndarray:
    pos = _c(pos, np.float64).reshape(-1)
    N = pos.size // 3
    cap = 64 * N + 1024
    while True:
        buf = np.zeros(2 * cap, np.int32)
        n = lib().oxo_pairs_within(N, pos, float(L), float(rc), buf, cap)
        if n <= cap:
            return buf[:2 * n].reshape(-1, 2)
        cap = n


def verlet_f32(pos4: np.ndarray, L: float, rverlet: float, n3, n5, auto_opt: bool = True, max_nb: int = 256):
    pos4 = _c(pos4, np.float32).reshape(-1)
    N = pos4.size // 4
    ncs = C.c_int(0)
    cell = np.zeros(N, np.int32)
    nnb = np.zeros(N, np.int32)
    nb = np.zeros(N * max_nb, np.int32)
    rc = lib().oxo_verlet_f32(N, pos4, float(L), float(rverlet), _c(n3, np.int32), _c(n5, np.int32),
                              1 if auto_opt else 0, C.byref(ncs), cell, nnb, nb, max_nb)
    return rc, ncs.value, cell, nnb, nb.reshape(N, max_nb)


def philox(key0, key1, c0, c1, c2, c3) -> np.ndarray:
    out = np.zeros(4, np.uint32)
    lib().oxo_philox(key0, key1, c0, c1, c2, c3, out)
    return out


def md_run(params: Params, md: MD, state: dict, n3, n5, typ, btype, L: float, step0: int, nsteps: int,
           nthreads: int = 1):
    """Advance `state` (dict of float64 arrays pos[N,3], quat[N,4], vel, Lmom, F, T) in place."""
    N = state["pos"].shape[0]
    Es = np.zeros(NTERMS)
    rc = lib().oxo_md_run(C.byref(params), C.byref(md), N, state["pos"].reshape(-1), state["quat"].reshape(-1),
                          state["vel"].reshape(-1), state["Lmom"].reshape(-1), _c(n3, np.int32), _c(n5, np.int32),
                          _c(typ, np.int32), _c(btype, np.int32), float(L), state["F"].reshape(-1),
                          state["T"].reshape(-1), int(step0), int(nsteps), Es, nthreads)
    return rc, Es


def external_forces(pos, step, forces, box):
    """Forces of the external-force records on every nucleotide, as the reference computes them
    (src/CUDA/Backends/CUDA_MD.cuh:97-555 and the CPU force classes src/Forces/*.cpp cited per
    type), in FP64.  `forces` are the dicts MDSystem.set_external_forces takes (the reference's
    external_forces_file keys)."""
    pos = np.asarray(pos, np.float64)
    F = np.zeros_like(pos)
    st = float(step)
    for d in forces:
        t = d["type"]
        if t == "com":
            # COMForce::force (src/Forces/COMForce.cpp): on every particle of com_list
            com = pos[np.asarray(d["com_list"], np.int64)].mean(axis=0)
            ref = pos[np.asarray(d["ref_list"], np.int64)].mean(axis=0)
            dv = ref - com
            dm = np.linalg.norm(dv)
            f = dv * ((dm - (d.get("r0", 0.0) + d.get("rate", 0.0) * st)) * d.get("stiff", 0.0) / len(d["com_list"]) / dm)
            for i in d["com_list"]:
                F[int(i)] += f
            continue
        i = int(d["particle"])
        r = pos[i]
        direction = np.asarray(d.get("dir", (0.0, 0.0, 0.0)), np.float64)
        if t in ("constant", "string"):
            inten = d.get("F0", 0.0) + st * d.get("rate", 0.0)
            dv = direction.copy()
            if d.get("dir_as_centre"):
                dv = dv - r
                dv = dv / np.linalg.norm(dv)
            F[i] += dv * inten
        elif t == "mutual_trap":
            dr = pos[int(d["ref_particle"])] - r
            if d.get("PBC"):
                dr = dr - np.rint(dr / box) * box
            dm = np.linalg.norm(dr)
            F[i] += dr * ((dm - (d.get("r0", 0.0) + d.get("rate", 0.0) * st)) *
                          (d.get("stiff", 0.0) + st * d.get("stiff_rate", 0.0)) / dm)
        elif t in ("trap", "moving_trap", "lowdim_trap"):
            tgt = np.asarray(d.get("pos0", (0.0, 0.0, 0.0)), np.float64) + d.get("rate", 0.0) * st * direction
            f = -d.get("stiff", 0.0) * (r - tgt)
            if t == "lowdim_trap":
                f = f * np.asarray(d.get("visibility", (True, True, True)), np.float64)
            F[i] += f
        elif t == "repulsion_plane":
            p0, end = d.get("position", 0.0), d.get("r0", 0.0)
            p = p0 + d.get("rate", 0.0) * st
            if end > p0 and p > end:
                p = end
            if end < p0 and p < end:
                p = end
            dist = direction @ r + p
            if dist < 0:
                F[i] += -dist * d.get("stiff", 0.0) * direction
        elif t == "attraction_plane":
            dist = direction @ r + d.get("position", 0.0)
            F[i] += (-dist if dist < 0 else -1.0) * d.get("stiff", 0.0) * direction
        elif t in ("sphere", "sphere_smooth"):
            # RepulsiveSphere::force, RepulsiveSphereSmooth::force (src/Forces/RepulsiveSphere*.cpp)
            c0 = np.asarray(d.get("center", (0.0, 0.0, 0.0)), np.float64)
            dv = r - c0
            dv = dv - np.rint(dv / box) * box
            m = np.linalg.norm(dv)
            r_ext = d.get("r_ext", 1e10)
            if t == "sphere":
                R = d.get("r0", -1.0) + d.get("rate", 0.0) * st
                if R < m < r_ext:
                    F[i] += dv * (-d.get("stiff", 0.0) * (1.0 - R / m))
            elif not (m < d.get("r0", -1.0) or m > r_ext):
                k, alpha, smooth = d.get("stiff", 0.0), d.get("alpha", -1.0), d.get("smooth", -1.0)
                if m >= alpha:
                    F[i] += dv * (-(k * 0.5 * np.exp((m - alpha) / smooth)) / m)
                else:
                    F[i] += dv * (-(k * m - k * 0.5 * np.exp(-(m - alpha) / smooth)) / m)
        elif t in ("LJ_wall", "LJ_cone"):
            # LJWall::force, LJCone::force (src/Forces/LJWall.cpp, src/Forces/LJCone.cpp)
            n = int(d.get("n", 6))
            k, sigma = d.get("stiff", 1.0), d.get("sigma", 1.0)
            cutoff = 2.0 ** (1.0 / n) if d.get("only_repulsive") else 1e6
            if t == "LJ_wall":
                x = direction @ r + d.get("position", -1.0)
                nrm = direction
            else:
                alpha = d.get("alpha", 0.0)
                v = r - np.asarray(d.get("pos0", (0.0, 0.0, 0.0)), np.float64)
                along = v @ direction
                from_axis = np.linalg.norm(direction * along - v)
                x = along * np.sin(alpha) - from_axis * np.cos(alpha)
                nrm = (along + from_axis * np.tan(alpha)) * direction - v
                nrm = nrm / np.linalg.norm(nrm)
            if x / sigma <= cutoff:
                lj = (x / sigma) ** (-n)
                F[i] += nrm * (4 * n * k * (2 * lj * lj - lj) / x)
        elif t == "generic_central_force":
            # GenericCentralForce::force, force_type = gravity (src/Forces/GenericCentralForce.cpp)
            dv = np.asarray(d.get("center", (0.0, 0.0, 0.0)), np.float64) - r
            d2 = dv @ dv
            inner, outer = d.get("inner_cut_off", 0.0), d.get("outer_cut_off", 0.0)
            if not (d2 < inner * inner) and not (outer > 0 and d2 > outer * outer):
                F[i] += d.get("F0", 0.0) * dv / np.sqrt(d2)
        elif t == "repulsion_plane_moving":
            # RepulsionPlaneMoving::force (src/Forces/RepulsionPlaneMoving.cpp), one reference particle
            x = (r - pos[int(d["ref_particle"])]) @ direction
            F[i] += -d.get("stiff", 0.0) * direction * min(x, 0.0)
        elif t == "twist":
            # ConstantRateTorque::force (src/Forces/ConstantRateTorque.cpp): the trap pos0 rotated by
            # base + rate step radians about the (normalised) axis through the centre, masked
            ax = np.asarray(d["axis"], np.float64)
            ax = ax / np.linalg.norm(ax)
            th = d.get("base", 0.0) + d.get("rate", 0.0) * st
            K = np.array([[0.0, -ax[2], ax[1]], [ax[2], 0.0, -ax[0]], [-ax[1], ax[0], 0.0]])
            R = np.cos(th) * np.eye(3) + np.sin(th) * K + (1.0 - np.cos(th)) * np.outer(ax, ax)
            centre = np.asarray(d.get("center", (0.0, 0.0, 0.0)), np.float64)
            trap = R @ (np.asarray(d["pos0"], np.float64) - centre) + centre
            F[i] += -d.get("stiff", 0.0) * (r - trap) * np.asarray(d.get("mask", (0.0, 0.0, 0.0)), np.float64)
        elif t == "ellipsoid":
            # RepulsiveEllipsoid::force (src/Forces/RepulsiveEllipsoid.cpp)
            dv = r - np.asarray(d.get("center", (0.0, 0.0, 0.0)), np.float64)
            dv = dv - np.rint(dv / box) * box
            inner = np.sum(dv ** 2 / np.asarray(d["r_2"], np.float64) ** 2)
            outer = np.sum(dv ** 2 / np.asarray(d.get("r_1", (1e-6, 1e-6, 1e-6)), np.float64) ** 2)
            if not (inner < 1.0 and outer > 1.0):
                F[i] += -d.get("stiff", 0.0) * dv / np.linalg.norm(dv)
        elif t == "yukawa_sphere":
            # YukawaSphere::force (src/Forces/YukawaSphere.cpp)
            dv = r - np.asarray(d.get("center", (0.0, 0.0, 0.0)), np.float64)
            dv = dv - np.rint(dv / box) * box
            m = np.linalg.norm(dv)
            lam, A = d["debye_length"], d["debye_A"]
            eps, sig, n = d.get("WCA_epsilon", 1.0), d.get("WCA_sigma", 1.0), int(d.get("WCA_n", 6))
            s_ = d["radius"] - m
            if s_ < d.get("cutoff", 4.0 * lam):
                c = A * np.exp(-s_ / lam) * (1.0 / (s_ * lam) + 1.0 / s_ ** 2)
                if s_ < sig * 2.0 ** (1.0 / n):
                    w = (sig / s_) ** 6
                    c += 4 * eps * n * (2 * w * w - w) / s_
                F[i] += -dv / m * c
        elif t == "repulsive_sphere_moving":
            # RepulsiveSphereMoving::force (src/Forces/RepulsiveSphereMoving.cpp)
            centre = np.asarray(d.get("center", (0.0, 0.0, 0.0)), np.float64)
            origin = np.asarray(d.get("origin", centre), np.float64)
            target = np.asarray(d.get("target", (0.0, 0.0, 0.0)), np.float64)
            nsteps = int(d.get("steps", d.get("move_steps", 0)))
            f = min(max(st / nsteps, 0.0), 1.0) if nsteps > 0 else 0.0
            dv = r - (origin + (target - origin) * f)
            dv = dv - np.rint(dv / box) * box
            m = np.linalg.norm(dv)
            g = m - (d["r0"] + d.get("rate", 0.0) * st)
            if g < d.get("r_ext", 1e10) and m > 0 and g < np.sqrt(2.0):
                gs = max(g, 1e-9)
                A = 1.0 / gs ** 2
                F[i] += dv * (8.0 * d.get("stiff", 0.0) * (2 * A - 1) * A / gs / m)
    return F
