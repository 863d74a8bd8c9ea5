"""oxgb_verlet_build_noalloc: the list build with static scratch and caller-owned outputs.

Through the C ABI it must give exactly what the handle-based oxgb_verlet_update gives: the same
counts, the same rows in the same order and the same list positions.  This is checked on two
different systems called back to back, and on the first one again after the second, so leftover
scratch would show.  Requests beyond its fixed limits must be refused before anything runs.
Neighbour lists are integer data, so the test tolerance is exact equality.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
from oxdna_gb300 import _abi
from oxdna_gb300 import generate as G

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SKIN = 0.05
RCUT = 3.2638  # the DNA2 cutoff at 300 K and 0.5 M, rounded: any cutoff works for this comparison


class _DeviceArray:
    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def _view(ptr, shape, typestr):
    return torch.as_tensor(_DeviceArray(ptr, shape, typestr), device="cuda")


def _inputs(pos, n3, n5, btype):
    N = pos.shape[0]
    p4 = np.zeros((N, 4), np.float32)
    p4[:, :3] = pos.astype(np.float32)
    p4[:, 3] = ((btype.astype(np.int32) << 22) | np.arange(N, dtype=np.int32)).view(np.float32)
    bonds = np.stack([n3, n5], axis=1).astype(np.int32)
    return torch.from_numpy(p4).cuda(), torch.from_numpy(bonds).cuda()


def _with_handle(d_pos, d_bonds, box):
    L = _abi.lib()
    N = d_pos.shape[0]
    v = C.c_void_p()
    _abi.check(L.oxgb_verlet_create(N, box, RCUT, SKIN, 1, 0, C.byref(v)))
    d_lp = torch.zeros_like(d_pos)
    _abi.check(L.oxgb_verlet_update(v, d_pos.data_ptr(), d_lp.data_ptr(), d_bonds.data_ptr(), None))
    torch.cuda.synchronize()
    _abi.check(L.oxgb_verlet_status(v))
    nb_ptr, nnb_ptr = C.c_void_p(), C.c_void_p()
    max_nb, ns = C.c_int(), C.c_int()
    _abi.check(L.oxgb_verlet_buffers(v, C.byref(nb_ptr), C.byref(nnb_ptr), C.byref(max_nb), C.byref(ns)))
    nb = _view(nb_ptr.value, (max_nb.value, N), "<i4").cpu().numpy()
    nnb = _view(nnb_ptr.value, (N,), "<i4").cpu().numpy()
    lp = d_lp.cpu().numpy()
    _abi.check(L.oxgb_verlet_destroy(v))
    return nb, nnb, lp, max_nb.value


def _without_alloc(d_pos, d_bonds, box, max_nb):
    L = _abi.lib()
    N = d_pos.shape[0]
    d_nb = torch.full((max_nb, N), -7, dtype=torch.int32, device="cuda")
    d_nnb = torch.full((N,), -7, dtype=torch.int32, device="cuda")
    d_lp = torch.zeros_like(d_pos)
    _abi.check(L.oxgb_verlet_build_noalloc(N, box, RCUT, SKIN, 1, d_pos.data_ptr(), d_lp.data_ptr(), d_bonds.data_ptr(),
                                           d_nb.data_ptr(), d_nnb.data_ptr(), max_nb, None))
    return d_nb.cpu().numpy(), d_nnb.cpu().numpy(), d_lp.cpu().numpy()


def _same(a, b):
    nb_a, nnb_a, lp_a = a[:3]
    nb_b, nnb_b, lp_b = b[:3]
    assert np.array_equal(nnb_a, nnb_b)
    assert np.array_equal(lp_a, lp_b)
    for i in range(nnb_a.shape[0]):
        assert np.array_equal(nb_a[:nnb_a[i], i], nb_b[:nnb_b[i], i]), i


def _systems():
    g = load_golden("mixed")
    a = (g["pos"], g["n3"], g["n5"], g["btype"], float(g["box"]))
    s = G.system_for_config(1, seed=5, scale=0.1)
    b = (s.pos, s.top.n3, s.top.n5, s.top.btype, float(s.box))
    return a, b


def test_noalloc_matches_handle_on_consecutive_calls():
    results = []
    a, b = _systems()
    for pos, n3, n5, bt, box in (a, b, a):
        d_pos, d_bonds = _inputs(pos, n3, n5, bt)
        ref = _with_handle(d_pos, d_bonds, box)
        got = _without_alloc(d_pos, d_bonds, box, ref[3])
        _same(ref, got)
        results.append(got)
    # the first system again, after the second: identical to its first build
    _same(results[0], results[2])


def test_noalloc_refuses_requests_beyond_its_limits():
    L = _abi.lib()
    d_pos = torch.zeros((8, 4), dtype=torch.float32, device="cuda")
    d_bonds = torch.full((8, 2), -1, dtype=torch.int32, device="cuda")
    d_nb = torch.zeros((8, 8), dtype=torch.int32, device="cuda")
    d_nnb = torch.zeros((8,), dtype=torch.int32, device="cuda")
    d_lp = torch.zeros_like(d_pos)
    args = (d_pos.data_ptr(), d_lp.data_ptr(), d_bonds.data_ptr(), d_nb.data_ptr(), d_nnb.data_ptr(), 8, None)
    # more nucleotides than the scratch holds: refused on the host, nothing launched
    rc = L.oxgb_verlet_build_noalloc(_abi.NOALLOC_MAX_N + 1, 100.0, RCUT, SKIN, 1, *args)
    assert rc == 1 and b"exceeds" in L.oxgb_last_error()
    # more cells than the scratch holds (a large box without the automatic cell sizing)
    rc = L.oxgb_verlet_build_noalloc(8, 400.0, RCUT, SKIN, 0, *args)
    assert rc == 1 and b"cells" in L.oxgb_last_error()
    torch.cuda.synchronize()


def test_noalloc_reports_overflow_and_the_next_call_starts_clean():
    """A max_neigh below the longest row returns OXGB_E_NEIGH_OVERFLOW; the status word lives in
    the shared scratch, so the next call with enough room must return OXGB_OK again, with the
    rows of the handle path."""
    L = _abi.lib()
    a, _ = _systems()
    pos, n3, n5, bt, box = a
    d_pos, d_bonds = _inputs(pos, n3, n5, bt)
    ref = _with_handle(d_pos, d_bonds, box)
    assert int(ref[1].max()) > 2
    N = d_pos.shape[0]
    small = 2
    d_nb = torch.zeros((small, N), dtype=torch.int32, device="cuda")
    d_nnb = torch.zeros((N,), dtype=torch.int32, device="cuda")
    d_lp = torch.zeros_like(d_pos)
    rc = L.oxgb_verlet_build_noalloc(N, box, RCUT, SKIN, 1, d_pos.data_ptr(), d_lp.data_ptr(), d_bonds.data_ptr(),
                                     d_nb.data_ptr(), d_nnb.data_ptr(), small, None)
    assert rc == 4  # OXGB_E_NEIGH_OVERFLOW
    got = _without_alloc(d_pos, d_bonds, box, ref[3])
    _same(ref, got)
