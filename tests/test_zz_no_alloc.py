"""GPU test of fedd_element_matrices_noalloc, the variant of
fedd_element_matrices that stages its output in a file-scope device array
instead of allocating.  Called through the C ABI, twice in a row, and
compared with the allocating entry point; the file name keeps it last in
collection so it also runs after every other test of the session."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCRATCH_DOUBLES = 1 << 19


@pytest.fixture(scope="module")
def env():
    import torch
    import feddlib_gb300 as F
    from feddlib_gb300 import _capi as A
    return F, A, torch


def _noalloc(A, torch, a, d_u, d_p, first, count, nd):
    K = np.full((count, nd, nd), np.nan)
    r = np.full((count, nd), np.nan)
    s = torch.cuda.current_stream()
    st = A.lib().fedd_element_matrices_noalloc(
        a.h, None if d_u is None else d_u.data_ptr(), None if d_p is None else d_p.data_ptr(), first, count,
        K.ctypes.data, r.ctypes.data, s.cuda_stream)
    return st, K, r


def _check_pair(A, torch, a, u, p, ranges, nd):
    dev = torch.device("cuda:0")
    d_u = None if u is None else torch.from_numpy(u).to(dev)
    d_p = None if p is None else torch.from_numpy(p).to(dev)
    torch.cuda.synchronize()
    for first, count in ranges:  # two calls in a row
        st, K, r = _noalloc(A, torch, a, d_u, d_p, first, count, nd)
        A.check(st, a.h)
        Ko, ro = a.element_matrices(u=u, p=p, first=first, count=count)
        assert np.array_equal(K, Ko)
        assert np.array_equal(r, ro)


def test_noalloc_navier_stokes(env):
    F, A, torch = env
    xyz2, el2 = F.structured_mesh(2, 2, seed=3)
    xyz1, el1 = F.structured_mesh(2, 1, seed=3)
    u = F.fourier_field(xyz2, seed=3)
    p = F.uniform_field(3, xyz1.shape[0])
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                    density=1.0, newton=True)
    _check_pair(A, torch, a, u, p, [(0, 40), (7, 41)], 34)


def test_noalloc_hyperelastic_and_laplace(env):
    F, A, torch = env
    xyz, el = F.structured_mesh(2, 2, seed=4)
    u = F.fourier_field(xyz, seed=4, kmin=1, kmax=2, scale=0.004)
    a = F.Assembler(F.NONLINEAR_ELASTICITY, xyz, el, E=32.0 / 11.0, poisson_ratio=5.0 / 11.0)
    _check_pair(A, torch, a, u, None, [(0, 48), (48, 0)], 30)
    xyz1, el1 = F.structured_mesh(3, 1, seed=1)
    lap = F.Assembler(F.LAPLACE, xyz1, el1, fe_order=1, source=1.0)
    _check_pair(A, torch, lap, None, None, [(0, el1.shape[0]), (11, 5)], 4)


def test_noalloc_rejects_oversize(env):
    F, A, torch = env
    xyz2, el2 = F.structured_mesh(5, 2, seed=3)
    xyz1, el1 = F.structured_mesh(5, 1, seed=3)
    u = F.fourier_field(xyz2, seed=3)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                    density=1.0, newton=True)
    cap = SCRATCH_DOUBLES // (34 * 35)
    assert cap == 440 and el2.shape[0] > cap
    d_u = torch.from_numpy(u).cuda()
    st, _, _ = _noalloc(A, torch, a, d_u, None, 0, cap + 1, 34)
    assert st == A.ERR_ARG
    buf = C.create_string_buffer(512)
    A.lib().fedd_last_error(a.h, buf, 512)
    assert b"exceeds the static scratch" in buf.value and b"at most 440" in buf.value
    # the handle stays usable, and the largest allowed call works
    st, K, r = _noalloc(A, torch, a, d_u, None, 0, cap, 34)
    A.check(st, a.h)
    Ko, ro = a.element_matrices(u=u, first=0, count=cap)
    assert np.array_equal(K, Ko) and np.array_equal(r, ro)


def test_noalloc_makes_no_allocation_after_setup(env):
    """After its first call the entry point leaves the device's free memory
    unchanged: nothing is allocated or freed per call."""
    F, A, torch = env
    xyz2, el2 = F.structured_mesh(3, 2, seed=3)
    xyz1, el1 = F.structured_mesh(3, 1, seed=3)
    u = F.fourier_field(xyz2, seed=3)
    p = F.uniform_field(3, xyz1.shape[0])
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                    density=1.0, newton=True)
    d_u = torch.from_numpy(u).cuda()
    d_p = torch.from_numpy(p).cuda()
    A.check(_noalloc(A, torch, a, d_u, d_p, 0, 100, 34)[0], a.h)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for first in (5, 40):
        A.check(_noalloc(A, torch, a, d_u, d_p, first, 120, 34)[0], a.h)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_generalized_newtonian(env):
    F, A, torch = env
    xyz2, el2 = F.structured_mesh(2, 2, seed=3)
    xyz1, el1 = F.structured_mesh(2, 1, seed=3)
    u = F.fourier_field(xyz2, seed=3)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                    density=1.0, newton=True)
    a.set_viscosity_law(0, [1.902, 0.22, 0.056, 0.00345, 1.25], gamma_min=1e-12)
    st, _, _ = _noalloc(A, torch, a, torch.from_numpy(u).cuda(), None, 0, 4, 34)
    assert st == A.ERR_UNSUPPORTED
    buf = C.create_string_buffer(512)
    A.lib().fedd_last_error(a.h, buf, 512)
    assert b"generalized-Newtonian" in buf.value
