import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
for p in (REPO, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


GOLDEN_CASES = ["ff16_avg", "ff16_seqdep", "duplex24", "mixed", "contact", "dh_variants", "mbf", "hbmult"]


def oracle_settings(g):
    import oracle
    seq = None
    if int(g["average"]) == 0:
        order = "AGCT"
        seq = {f"STCK_{order[i]}_{order[j]}": float(g["seq_stck"][i][j]) for i in range(4) for j in range(4)}
        seq["STCK_FACT_EPS"] = float(g["seq_fact"])
        seq["HYDR_A_T"] = float(g["seq_hydr_at"])
        seq["HYDR_G_C"] = float(g["seq_hydr_gc"])
    mbf = float(g["mbf_fmax"])
    return oracle.make_settings(float(g["T"]), float(g["salt"]), average=bool(int(g["average"])), seq=seq,
                                hb_multiplier=float(g["hb_multiplier"]),
                                half_charged_ends=bool(int(g["half_charged_ends"])), dh_lambda=float(g["dh_lambda"]),
                                dh_strength=float(g["dh_strength"]), mbf_fmax=(mbf if mbf >= 0 else None),
                                mbf_finf=float(g["mbf_finf"]))


@pytest.fixture(scope="session")
def golden():
    return load_golden
