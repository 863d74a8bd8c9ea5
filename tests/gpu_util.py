"""Helpers shared by the GPU parity tests."""
import numpy as np

from oxdna_gb300 import MDSystem, dna2_settings, md_settings
from oxdna_gb300 import io as oxio


def settings_from_golden(g, **kw):
    seq = None
    if int(g["average"]) == 0:
        order = "AGCT"
        seq = {f"STCK_{order[i]}_{order[j]}": float(g["seq_stck"][i][j]) for i in range(4) for j in range(4)}
        seq["STCK_FACT_EPS"] = float(g["seq_fact"])
        seq["HYDR_A_T"] = float(g["seq_hydr_at"])
        seq["HYDR_G_C"] = float(g["seq_hydr_gc"])
    mbf = float(g["mbf_fmax"])
    return dna2_settings(float(g["T"]), float(g["salt"]), average=bool(int(g["average"])), seq=seq,
                         hb_multiplier=float(g["hb_multiplier"]), half_charged_ends=bool(int(g["half_charged_ends"])),
                         dh_lambda=float(g["dh_lambda"]), dh_strength=float(g["dh_strength"]),
                         mbf_fmax=(mbf if mbf >= 0 else None), mbf_finf=float(g["mbf_finf"]), **kw)


def topology_from_golden(g):
    N = g["pos"].shape[0]
    return oxio.Topology(g["n3"].astype(np.int32), g["n5"].astype(np.int32), g["btype"].astype(np.int32),
                         g["type"].astype(np.int32), np.zeros(N, np.int32), 1)


def system_from_golden(g, precision="mixed", **mdkw):
    sysm = MDSystem(float(g["box"]), topology_from_golden(g), settings_from_golden(g),
                    md_settings(precision=precision, **mdkw))
    q = oxio.frame_to_quat(g["a1"], g["a2"], g["a3"])
    sysm.set_state(g["pos"], q, g["vel"], g["Lmom"])
    return sysm, q


def force_errors(F, Fref):
    """max_i |dF_i| / max(|F_i|, floor) with floor = 0.1 * RMS |F|, and the normwise error"""
    n = np.linalg.norm(Fref, axis=1)
    floor = 0.1 * np.sqrt(np.mean(n ** 2))
    d = np.linalg.norm(F - Fref, axis=1)
    return float(np.max(d / np.maximum(n, floor))), float(np.linalg.norm(F - Fref) / np.linalg.norm(Fref))
