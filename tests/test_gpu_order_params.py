"""The FFS order-parameter kernels on the reference's device layout, through the C ABI.

oxgb_dna2_hb_op_precalc, oxgb_dna2_near_hb_op_precalc and oxgb_dna2_dist_op_precalc stand in
for CUDADNAInteraction's _hb_op_precalc, _near_hb_op_precalc and _dist_op_precalc
(src/CUDA/Interactions/CUDADNAInteraction.cu:205-218; kernels CUDA_DNA.cuh:910-1067).  On 2,000
nucleotides of duplexes, for every pair of nucleotides whose centres are within 2.0 of each other
(hydrogen-bonded, stacked and cross-stacked neighbours, and pairs in no interaction) plus the
complementary partners across a duplex, they are compared with the oracle's FP64 restatement
(oracle.order_params, whose energies are pinned to the reference's hydrogen-bonding term) on the
same FP32 inputs:
  * energies within 2e-5 of max(|E|, 0.01) (FP32 arithmetic of a product of seven factors);
  * the nearly-bonded flag equal on every pair but those where a factor sits within FP32
    rounding of its support's edge (at most 1 in 10^3);
  * base-base distances within 1e-6.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from oxdna_gb300 import _abi, dna2_settings
from oxdna_gb300 import generate as G
from oxdna_gb300 import io as oxio

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_order_parameters_match_the_oracle():
    s = G.system_for_config(1, seed=23, scale=0.05)
    N, box = s.N, float(s.box)
    pos = np.zeros((N, 4), np.float32)
    pos[:, :3] = s.pos.astype(np.float32)
    bt = np.asarray(s.top.btype, np.int32)
    pos[:, 3] = ((bt << 22) | np.arange(N, dtype=np.int32)).view(np.float32)
    q32 = s.quats().astype(np.float32)
    # the oracle sees the same FP32 inputs
    a1, a2, a3 = oxio.quat_to_frame(q32.astype(np.float64))
    p64 = pos[:, :3].astype(np.float64)

    pairs = oracle.pairs_within(p64, box, 2.0)
    i, j = pairs[:, 0].astype(np.int32), pairs[:, 1].astype(np.int32)
    bonded = (np.asarray(s.top.n3)[i] == j) | (np.asarray(s.top.n5)[i] == j)
    i, j = i[~bonded], j[~bonded]
    n = i.size
    assert n > 10000

    L = _abi.lib()
    h = C.c_void_p()
    st = dna2_settings(s.T, 0.5)
    _abi.check(L.oxgb_dna2_create(C.byref(st), C.byref(h)))
    d_pos, d_q = torch.from_numpy(pos).cuda(), torch.from_numpy(q32).cuda()
    d_i, d_j = torch.from_numpy(i).cuda(), torch.from_numpy(j).cuda()
    e = torch.zeros(n, dtype=torch.float32, device="cuda")
    near = torch.zeros(n, dtype=torch.bool, device="cuda")
    dist = torch.zeros(n, dtype=torch.float32, device="cuda")
    args = (h, box, d_pos.data_ptr(), d_q.data_ptr(), d_i.data_ptr(), d_j.data_ptr(), n)
    _abi.check(L.oxgb_dna2_hb_op_precalc(*args, e.data_ptr(), None))
    _abi.check(L.oxgb_dna2_near_hb_op_precalc(*args, near.data_ptr(), None))
    _abi.check(L.oxgb_dna2_dist_op_precalc(*args, dist.data_ptr(), None))
    torch.cuda.synchronize()
    _abi.check(L.oxgb_dna2_destroy(h))
    e, near, dist = e.cpu().numpy().astype(np.float64), near.cpu().numpy(), dist.cpu().numpy().astype(np.float64)

    P = oracle.make_params(oracle.make_settings(s.T, 0.5))
    oargs = (P, p64, a1, a3, s.top.type, s.top.btype, box, i, j)
    e_ref, near_ref, dist_ref = (oracle.order_params(*oargs, m) for m in (0, 1, 2))

    n_hb = int((e_ref < -0.1).sum())
    assert n_hb > 500, n_hb  # the duplexes' base pairs are there
    err = np.abs(e - e_ref) / np.maximum(np.abs(e_ref), 0.01)
    mism = int((near != (near_ref > 0.5)).sum())
    print(f"{n} pairs, {n_hb} hydrogen-bonded: energy error max {err.max():.2e}, near-bonded flags differing {mism}, "
          f"distance error max {np.abs(dist - dist_ref).max():.2e}")
    assert err.max() <= 2e-5
    assert mism <= n // 1000
    assert np.abs(dist - dist_ref).max() <= 1e-6
