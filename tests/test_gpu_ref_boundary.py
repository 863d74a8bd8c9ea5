"""The drop-in boundary run inside the reference's own program, on the GPU, and the reference's
own Verlet list against ours.

Both routes are built from the reference's sources by oracle/ref/Makefile (no CMake) and run:

* link substitution (oxDNA_cuda_gb300): the reference's CUDA program with its CUDADNAInteraction
  and CUDASimpleVerletList translation units replaced by oxdna_gb300/shim/subst (the same class
  names over liboxgb), so that its own input keys -- backend = CUDA, interaction_type = DNA2,
  CUDA_list = verlet -- run our interaction and list kernels;
* plugin (CUDAGB300DNA2.so): the unmodified reference program with interaction_type = GB300DNA2
  and plugin_search_path, loaded by its PluginManager.

On a 4,000-nucleotide configuration the potential energy per nucleotide that the reference's
CUDA backend sums on the device (CUDA_print_energy: the w of the forces) must equal our
engine's (oxDNA2 well depths) to FP32 rounding and the printed 6 decimals; the stock reference
CUDA program must equal our engine run with reference_cuda_eps (the oxDNA1 average-sequence well
depths its CUDA class keeps).  Then 2,000 Brownian MD steps of the substituted program end in a
finite state.  Skipped where the reference sources are absent (OXDNA_REFERENCE unset and nothing
staged in baseline/_ref/oxDNA).
"""
import os
import tempfile

import numpy as np
import pytest

from oxdna_gb300 import MDSystem, dna2_settings, md_settings
from oxdna_gb300 import generate as G

pytestmark = pytest.mark.gpu

refrun = pytest.importorskip("refrun")


@pytest.fixture(scope="module")
def programs():
    if refrun.reference_checkout() is None and not os.path.exists(refrun.PROGRAMS["cuda-gb300"]):
        pytest.skip("reference sources not present")
    from oxdna_gb300 import build
    build.build()
    return {k: refrun.build(k) for k in ("cuda", "cuda-gb300", "plugin")}


@pytest.fixture(scope="module")
def system():
    return G.system_for_config(1, seed=31, scale=0.1)


def _ours(s, reference_cuda_eps):
    m = MDSystem(s.box, s.top, dna2_settings(s.T, 0.5, reference_cuda_eps=reference_cuda_eps), md_settings(dt=0.003))
    m.set_state(s.pos, s.quats(), s.vel, s.L)
    _, _, E, _ = m.compute_forces()
    m.close()
    return float(np.sum(E) / (2 * s.N))


def _close(a, b):
    return abs(a - b) <= 1e-5 * abs(b) + 2e-6


def test_link_substitution_runs_our_kernels_under_the_reference_keys(programs, system):
    e = refrun.cuda_energy_per_nucleotide(programs["cuda-gb300"], system)
    ours = _ours(system, False)
    print(f"substituted reference program: {e:.6f}, our engine {ours:.7f}")
    assert _close(e, ours)


def test_plugin_route(programs, system):
    d = os.path.dirname(programs["plugin"])
    e = refrun.cuda_energy_per_nucleotide(programs["cuda"], system, interaction="GB300DNA2",
                                          extra=f"plugin_search_path = {d}\n")
    ours = _ours(system, False)
    print(f"reference program + GB300DNA2 plugin: {e:.6f}, our engine {ours:.7f}")
    assert _close(e, ours)


def test_stock_reference_cuda_uses_oxdna1_average_well_depths(programs, system):
    e = refrun.cuda_energy_per_nucleotide(programs["cuda"], system)
    ours_ref, ours = _ours(system, True), _ours(system, False)
    print(f"stock reference CUDA: {e:.6f}; our engine with its well depths {ours_ref:.7f}, with oxDNA2's {ours:.7f}")
    assert _close(e, ours_ref)
    assert not _close(e, ours)


def test_substituted_program_runs_md(programs, system):
    with tempfile.TemporaryDirectory() as tmp:
        refrun.write_system(tmp, system)
        text = refrun.deck(system, backend="CUDA", steps=2000, dt=0.003, thermostat="john", newtonian_steps=103,
                           diff_coeff=2.5)
        r = refrun.run(programs["cuda-gb300"], tmp, text)
        conf = refrun.read_last_conf(tmp)
        assert np.all(np.isfinite(conf.pos)) and conf.pos.shape == system.pos.shape
        assert r["own_ms_per_step"] is not None
        print(f"substituted program: {r['own_ms_per_step']:.4f} ms per step (its own timer), 2000 steps")


def test_reference_verlet_list_has_our_pair_sets(programs, system):
    """The reference's own CUDASimpleVerletList (CUDA_list = verlet) on the GPU, dumped by the
    plugin with the FP32 positions it was built from, against the library's list built from the
    same positions (oxgb_verlet_*): the same partners for every nucleotide.  The reference fills
    its cells with atomic increments, so only the sets are compared, not the order in a row."""
    import ctypes as C
    import torch
    from oxdna_gb300 import _abi
    d = os.path.dirname(programs["plugin"])
    ref = refrun.reference_verlet_list(programs["cuda"], d, system)
    N = system.N
    L = _abi.lib()
    h = C.c_void_p()
    st = dna2_settings(system.T, 0.5)
    _abi.check(L.oxgb_dna2_create(C.byref(st), C.byref(h)))
    rcut = C.c_double()
    _abi.check(L.oxgb_dna2_get_rcut(h, C.byref(rcut)))
    _abi.check(L.oxgb_dna2_destroy(h))
    v = C.c_void_p()
    _abi.check(L.oxgb_verlet_create(N, float(system.box), rcut.value, 0.05, 1, 0, C.byref(v)))
    d_pos = torch.from_numpy(ref["pos"]).cuda()
    d_list_pos = torch.zeros_like(d_pos)
    bonds = np.stack([system.top.n3, system.top.n5], axis=1).astype(np.int32)
    d_bonds = torch.from_numpy(bonds).cuda()
    _abi.check(L.oxgb_verlet_update(v, d_pos.data_ptr(), d_list_pos.data_ptr(), d_bonds.data_ptr(), None))
    torch.cuda.synchronize()
    _abi.check(L.oxgb_verlet_status(v))
    nb_ptr, nnb_ptr = C.c_void_p(), C.c_void_p()
    max_nb, ns = C.c_int(), C.c_int()
    _abi.check(L.oxgb_verlet_buffers(v, C.byref(nb_ptr), C.byref(nnb_ptr), C.byref(max_nb), C.byref(ns)))
    from test_gpu_plugin_layers import view
    nnb = view(nnb_ptr.value, (N,), "<i4").cpu().numpy()
    nb = view(nb_ptr.value, (max_nb.value, N), "<i4").cpu().numpy()
    _abi.check(L.oxgb_verlet_destroy(v))
    assert np.array_equal(nnb, ref["counts"])
    total = 0
    for i in range(N):
        ours = np.sort(nb[:nnb[i], i])
        theirs = np.sort(ref["rows"][i, :ref["counts"][i]])
        assert np.array_equal(ours, theirs), i
        total += nnb[i]
    print(f"reference CUDASimpleVerletList vs ours on {N} nucleotides: {total} entries, identical sets")
