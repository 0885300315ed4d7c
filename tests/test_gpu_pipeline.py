"""The host-buffer path (fedd_assemble) runs the element stage in chunks
interleaved with the row ranges whose copies to the host overlap the next
chunk.  Its values and residuals must equal the device path's (one element
launch, one row launch) bit for bit: on structured meshes, where the chunks
are proper slices of the elements, and on a shuffled numbering, where the
first chunk holds every element."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F():
    import feddlib_gb300 as F
    return F


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def device_path(torch, a, u, p, nb):
    dev = torch.device("cuda:0")
    du = None if u is None else torch.from_numpy(u).to(dev)
    dp = None if p is None else torch.from_numpy(p).to(dev)
    dv = [torch.full((max(a.block_info(b)[2], 1),), np.nan, dtype=torch.float64, device=dev) for b in range(nb)]
    dru = torch.full((a.n_u,), np.nan, dtype=torch.float64, device=dev)
    drp = torch.full((max(a.n_p, 1),), np.nan, dtype=torch.float64, device=dev) if a.n_p else None
    a.assemble_device(None if du is None else du.data_ptr(), None if dp is None else dp.data_ptr(),
                      [t.data_ptr() for t in dv], dru.data_ptr(), None if drp is None else drp.data_ptr(),
                      stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    out = [t.cpu().numpy() for t in dv] + [dru.cpu().numpy()]
    if drp is not None:
        out.append(drp.cpu().numpy())
    return out


def same_bits(x, y):
    x, y = np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64)
    return x.shape == y.shape and np.array_equal(x.view(np.uint64), y.view(np.uint64))


def shuffled(el, seed):
    return np.ascontiguousarray(el[np.random.default_rng(seed).permutation(el.shape[0])])


@pytest.mark.parametrize("shuffle", [False, True])
@pytest.mark.parametrize("problem", ["LINEAR_ELASTICITY", "NONLINEAR_ELASTICITY"])
def test_elasticity_host_path_is_bitwise_device_path(F, torch, problem, shuffle):
    xyz, el = F.structured_mesh(8, 2, seed=31)
    if shuffle:
        el = shuffled(el, 31)
    u = F.fourier_field(xyz, seed=31, kmin=1, kmax=2, scale=0.004)
    a = F.Assembler(getattr(F, problem), xyz, el, E=1000.0, poisson_ratio=0.3)
    (v,), r, _ = a.assemble(u=u)
    dv, dr = device_path(torch, a, u, None, 1)
    assert same_bits(v, dv) and same_bits(r, dr)


@pytest.mark.parametrize("gn", [False, True])
@pytest.mark.parametrize("shuffle,M", [(False, 8), (True, 8), (False, 24)])
def test_navier_stokes_host_path_is_bitwise_device_path(F, torch, gn, shuffle, M):
    """The device path takes the velocity rows' nodes from a global counter,
    the host path in fixed node ranges; M = 24 gives the counter a larger
    mesh."""
    xyz2, el2 = F.structured_mesh(M, 2, seed=32)
    xyz1, el1 = F.structured_mesh(M, 1, seed=32)
    if shuffle:
        perm = np.random.default_rng(32).permutation(el2.shape[0])
        el2, el1 = np.ascontiguousarray(el2[perm]), np.ascontiguousarray(el1[perm])
    u = F.fourier_field(xyz2, seed=32) * (0.5 if gn else 1.0)
    p = F.uniform_field(32, xyz1.shape[0])
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                    density=1.0, newton=True)
    if gn:
        a.set_viscosity_law(0, [1.902, 0.22, 0.056, 0.00345, 1.25], gamma_min=1e-12)
    vals, ru, rp = a.assemble(u=u, p=p)
    d = device_path(torch, a, u, p, 3)
    for b in range(3):
        assert same_bits(vals[b], d[b]), b
    assert same_bits(ru, d[3]) and same_bits(rp, d[4])


@pytest.mark.parametrize("shuffle", [False, True])
def test_surrogate_host_path_is_bitwise_device_path(F, torch, shuffle):
    """The surrogate's per-point stages run per element chunk on the host
    path; random weights and a narrow invariant box (so that some points take
    the plain-law fallback) suffice for a bit-exact comparison."""
    xyz, el = F.structured_mesh(8, 2, seed=33)
    if shuffle:
        el = shuffled(el, 33)
    u = F.fourier_field(xyz, seed=33, kmin=1, kmax=2, scale=0.004)
    rng = np.random.default_rng(33)
    H = 64
    model = {"W1": 0.5 * rng.standard_normal((H, 4)), "b1": 0.1 * rng.standard_normal(H),
             "W2": rng.standard_normal((H, H)) / 8.0, "b2": 0.1 * rng.standard_normal(H),
             "w3": 0.1 * rng.standard_normal(H), "b3": 0.0, "out_scale": 0.01,
             "in_shift": [0.0, 0.0, 1.0, 1.0], "in_scale": [0.0, 0.0, 20.0, 20.0]}
    a = F.Assembler(F.ANISO_FIBER, xyz, el, surrogate=True, E=32.0 / 11.0, poisson_ratio=5.0 / 11.0, k1=2.0,
                    k2=1.0, fiber_angle_deg=40.0)
    a.set_surrogate(model, inv_lo=(-1e30, -1e30, 0.99, 0.99), inv_hi=(1e30, 1e30, 1.01, 1.01))
    (v,), r, _ = a.assemble(u=u)
    fb_host = a.surrogate_fallbacks()
    dv, dr = device_path(torch, a, u, None, 1)
    fb_dev = a.surrogate_fallbacks()
    assert fb_host == fb_dev and 0 < fb_host[0] < fb_host[1]
    assert same_bits(v, dv) and same_bits(r, dr)
