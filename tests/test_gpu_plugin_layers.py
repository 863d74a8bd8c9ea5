"""The plugin-surface layers of the C ABI on the reference's own device layout.

* oxgb_verlet_* (CUDABaseList): the column-major neighbour matrix (element k of nucleotide i at
  k * N + i) holds exactly the pair set of the oracle's FP32 restatement of the list build, and
  every pair within the interaction cutoff;
* oxgb_dna2_* (CUDABaseInteraction): forces, torques and energies from float4 positions with the
  packed btype/index word, float4 quaternions and that neighbour matrix, accumulated into
  caller-initialised buffers.  These inputs are plain FP32 (no high/low split of the positions),
  as the reference's own CUDA backend stores them, so the tolerance is the FP32-input one:
  normwise 1e-4 and per nucleotide 1e-3 of max(|F_ref,i|, 0.1 RMS |F_ref|).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from conftest import load_golden
from gpu_util import force_errors, settings_from_golden
from oxdna_gb300 import _abi
from oxdna_gb300 import io as oxio

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


class _DeviceArray:
    """A raw device pointer seen as a torch tensor (no copy)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def view(ptr, shape, typestr):
    return torch.as_tensor(_DeviceArray(ptr, shape, typestr), device="cuda")


def reference_layout(g):
    N = g["pos"].shape[0]
    pos = np.zeros((N, 4), np.float32)
    pos[:, :3] = g["pos"].astype(np.float32)
    bt = g["btype"].astype(np.int32)
    pos[:, 3] = ((bt << 22) | np.arange(N, dtype=np.int32)).view(np.float32)
    q = oxio.frame_to_quat(g["a1"], g["a2"], g["a3"]).astype(np.float32)
    bonds = np.stack([g["n3"], g["n5"]], axis=1).astype(np.int32)
    return pos, q, bonds


@pytest.mark.parametrize("case", ["mixed", "duplex24"])
def test_verlet_and_interaction_layers(case):
    g = load_golden(case)
    N = g["pos"].shape[0]
    box = float(g["box"])
    L = _abi.lib()
    pos, q, bonds = reference_layout(g)
    d_pos = torch.from_numpy(pos).cuda()
    d_q = torch.from_numpy(q).cuda()
    d_bonds = torch.from_numpy(bonds).cuda()
    d_list_pos = torch.zeros_like(d_pos)

    s = settings_from_golden(g)
    h = C.c_void_p()
    _abi.check(L.oxgb_dna2_create(C.byref(s), C.byref(h)))
    rcut = C.c_double()
    _abi.check(L.oxgb_dna2_get_rcut(h, C.byref(rcut)))
    p = oracle.make_params(oracle.make_settings(float(g["T"]), float(g["salt"])))
    assert abs(rcut.value - p.rcut) < 1e-12

    skin = 0.05
    v = C.c_void_p()
    _abi.check(L.oxgb_verlet_create(N, box, rcut.value, skin, 1, 0, C.byref(v)))
    _abi.check(L.oxgb_verlet_update(v, d_pos.data_ptr(), d_list_pos.data_ptr(), d_bonds.data_ptr(), None))
    torch.cuda.synchronize()
    _abi.check(L.oxgb_verlet_status(v))
    nb_ptr, nnb_ptr = C.c_void_p(), C.c_void_p()
    max_nb, ns = C.c_int(), C.c_int()
    _abi.check(L.oxgb_verlet_buffers(v, C.byref(nb_ptr), C.byref(nnb_ptr), C.byref(max_nb), C.byref(ns)))
    nb = view(nb_ptr.value, (max_nb.value, N), "<i4").cpu().numpy()
    nnb = view(nnb_ptr.value, (N,), "<i4").cpu().numpy()
    assert np.array_equal(d_list_pos.cpu().numpy(), pos)

    rv = np.float32(np.float32(rcut.value) + np.float32(2.0) * np.float32(skin))
    rc, ns_o, cell_o, nnb_o, nb_o = oracle.verlet_f32(pos, box, float(rv), g["n3"], g["n5"], True,
                                                      max_nb=max_nb.value + 64)
    assert rc == 0 and ns.value == ns_o
    assert np.array_equal(nnb, nnb_o)
    for i in range(N):
        assert np.array_equal(np.sort(nb[:nnb[i], i]), nb_o[i, :nnb_o[i]]), i
    rows = [set(nb[:nnb[i], i].tolist()) for i in range(N)]
    for i, j in oracle.pairs_within(g["pos"], box, rcut.value):
        if g["n3"][i] != j and g["n5"][i] != j:
            assert j in rows[i] and i in rows[j]

    # forces accumulate into caller-initialised buffers: start from a known external force
    ext = np.zeros((N, 4), np.float32)
    ext[:, 0] = 0.25
    d_F = torch.from_numpy(ext).cuda()
    d_T = torch.zeros((N, 4), dtype=torch.float32, device="cuda")
    _abi.check(L.oxgb_dna2_compute_forces(h, N, box, d_pos.data_ptr(), d_q.data_ptr(), d_F.data_ptr(), d_T.data_ptr(),
                                          d_bonds.data_ptr(), nb_ptr.value, nnb_ptr.value, max_nb.value, 1, N, None))
    torch.cuda.synchronize()
    F4 = d_F.cpu().numpy().astype(np.float64)
    T4 = d_T.cpu().numpy().astype(np.float64)
    F = F4[:, :3] - ext[:, :3]
    fmax, fnorm = force_errors(F, g["F"])
    tmax, tnorm = force_errors(T4[:, :3], g["Tq"])
    print(f"{case}: force max-rel {fmax:.2e} norm {fnorm:.2e}; torque max-rel {tmax:.2e} norm {tnorm:.2e}")
    assert fnorm <= 1e-4 and tnorm <= 1e-4
    assert fmax <= 1e-3 and tmax <= 1e-3
    # w: every pair's energy on both nucleotides (total = sum / 2); torque w: hydrogen bonding
    E = F4[:, 3].sum() / 2
    assert abs(E - float(g["energy"])) <= 1e-4 * max(1.0, abs(float(g["energy"])))
    hb = T4[:, 3].sum() / 2
    assert abs(hb - float(g["split"][4])) <= 1e-4 * max(1.0, abs(float(g["split"][4])))
    _abi.check(L.oxgb_verlet_destroy(v))
    _abi.check(L.oxgb_dna2_destroy(h))
