"""flygpu_eam_energy_gradient_noalloc: the EAM energy and gradient for callers that cannot allocate.

Callers running inside a framework that owns every device allocation, or in a loop that must not
touch the allocator after start-up, pass their own device inputs and outputs to this entry point; it
keeps its scratch in a fixed array inside the library. This test calls it through the C ABI on two
calls in a row (the scratch array is shared between calls and keeps the previous call's contents) and
checks each against the allocating entry point flygpu_eam_energy_gradient in binary64: gradients
within 1e-10 relative (norm-wise) and energies within 1e-10 relative, the reference's known-answer
tolerance (tests/potential/EAM/eam.cpp:125).
"""
import ctypes as C

import numpy as np
import pytest

from openfly_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def noalloc(gpu):
    fn = gpu.lib().flygpu_eam_energy_gradient_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_void_p, C.c_void_p]
    return fn


def call(gpu, noalloc, geam, s):
    import torch

    dev = torch.device("cuda", 0)
    pos = torch.tensor(s.pos.reshape(-1), dtype=torch.float64, device=dev)
    types = torch.tensor(s.types.astype(np.int32), device=dev)
    frozen = torch.tensor(s.frozen, device=dev)
    grad = torch.full((3 * s.n,), float("nan"), dtype=torch.float64, device=dev)
    energy = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    ext = np.ascontiguousarray(s.extents, dtype=np.float64)
    per = np.ascontiguousarray(s.periodic, dtype=np.int32)
    stream = torch.cuda.current_stream(dev).cuda_stream
    st = noalloc(geam.h, pos.data_ptr(), types.data_ptr(), frozen.data_ptr(), s.n, ext.ctypes.data, per.ctypes.data,
                 energy.data_ptr(), grad.data_ptr(), stream)
    gpu.check(st, "flygpu_eam_energy_gradient_noalloc")
    return float(energy.cpu()[0]), grad.cpu().numpy().reshape(-1, 3)


def allocating(gpu, geam, s):
    nl = gpu.List(s.extents, s.periodic, geam.r_cut())
    nl.rebuild(s.pos)
    return geam.energy_gradient(s.types, s.frozen, nl, gpu.FP64)


def test_noalloc_matches_allocating_entry_point(gpu, geam, noalloc):
    cl = W.cluster(np.random.default_rng(2), 9.5, n_vac=1, n_h=2)
    systems = [W.fe_vacancy_cell(), W.kat_lattice(), cl.sys]
    for s in systems + systems[:1]:  # consecutive calls reuse the shared scratch
        e, g = call(gpu, noalloc, geam, s)
        e_ref, g_ref = allocating(gpu, geam, s)
        assert abs(e - e_ref) <= TOL * abs(e_ref)
        assert np.linalg.norm(g - g_ref) <= TOL * max(np.linalg.norm(g_ref), 1.0)
        assert np.all(g[s.frozen == 1] == 0)


def test_noalloc_allocates_nothing_and_clears_its_error_word(gpu, geam, noalloc):
    # After a first call (which may load the library's device code), a call leaves the device's free
    # memory unchanged. A call with a type index beyond the potential's types is rejected; the next valid
    # call starts from a cleared error word and succeeds with the allocating entry point's results.
    import torch

    s = W.fe_vacancy_cell()
    call(gpu, noalloc, geam, s)
    dev = torch.device("cuda", 0)
    pos = torch.tensor(s.pos.reshape(-1), dtype=torch.float64, device=dev)
    bad_types = torch.full((s.n,), 7, dtype=torch.int32, device=dev)
    frozen = torch.tensor(s.frozen, device=dev)
    grad = torch.empty(3 * s.n, dtype=torch.float64, device=dev)
    energy = torch.empty(1, dtype=torch.float64, device=dev)
    ext = np.ascontiguousarray(s.extents, dtype=np.float64)
    per = np.ascontiguousarray(s.periodic, dtype=np.int32)
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(dev)
    st = noalloc(geam.h, pos.data_ptr(), bad_types.data_ptr(), frozen.data_ptr(), s.n, ext.ctypes.data,
                 per.ctypes.data, energy.data_ptr(), grad.data_ptr(), stream)
    free1, _ = torch.cuda.mem_get_info(dev)
    assert st == gpu.INVALID_ARG
    assert free1 == free0
    e, g = call(gpu, noalloc, geam, s)
    e_ref, g_ref = allocating(gpu, geam, s)
    assert abs(e - e_ref) <= TOL * abs(e_ref)
    assert np.linalg.norm(g - g_ref) <= TOL * np.linalg.norm(g_ref)


def test_noalloc_rejects_oversized_systems(gpu, geam, noalloc):
    ext = np.full(3, 100.0)
    per = np.zeros(3, np.int32)
    dummy = C.c_double()
    st = noalloc(geam.h, C.addressof(dummy), C.addressof(dummy), C.addressof(dummy), 4097, ext.ctypes.data,
                 per.ctypes.data, C.addressof(dummy), C.addressof(dummy), None)
    assert st == gpu.INVALID_ARG
    assert "4096" in gpu.lib().flygpu_last_error().decode()
