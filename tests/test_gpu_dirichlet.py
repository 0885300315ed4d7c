"""GPU parity of the device Dirichlet rows (BCBuilder::setSystem / setRHS /
setBCMinusVector) against the oracle's restatement, applied to the same
assembled values: bit-exact."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    import feddlib_gb300 as F
    return F, torch


def _ns_masks(xyz2, n_p):
    """Velocity: all dofs on x = 0 ("Dirichlet"), dof 0 on x = 1
    ("Dirichlet_X"); pressure: dof 0."""
    mu = np.zeros(3 * xyz2.shape[0], dtype=np.uint8)
    lo = np.nonzero(np.abs(xyz2[:, 0]) < 1e-12)[0]
    hi = np.nonzero(np.abs(xyz2[:, 0] - 1.0) < 1e-12)[0]
    for d in range(3):
        mu[3 * lo + d] = 1
    mu[3 * hi] = 1
    mp = np.zeros(n_p, dtype=np.uint8)
    mp[0] = 1
    return mu, mp


def test_dirichlet_navier_stokes(env):
    F, torch = env
    dev = torch.device("cuda:0")
    xyz2, el2 = F.structured_mesh(2, 2, seed=3)
    xyz1, el1 = F.structured_mesh(2, 1, seed=3)
    u = F.fourier_field(xyz2, seed=3)
    p = F.uniform_field(3, xyz1.shape[0])
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                    density=1.0, newton=True)
    mu, mp = _ns_masks(xyz2, xyz1.shape[0])
    a.set_dirichlet(mu, mp)
    d_u, d_p = torch.from_numpy(u).to(dev), torch.from_numpy(p).to(dev)
    d_vals = [torch.empty(a.block_info(b)[2], dtype=torch.float64, device=dev) for b in range(3)]
    d_ru = torch.empty(a.n_u, dtype=torch.float64, device=dev)
    d_rp = torch.empty(a.n_p, dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream().cuda_stream
    a.assemble_device(d_u.data_ptr(), d_p.data_ptr(), [v.data_ptr() for v in d_vals], d_ru.data_ptr(),
                      d_rp.data_ptr(), stream=s)
    before = [v.cpu().numpy() for v in d_vals]
    ru0, rp0 = d_ru.cpu().numpy(), d_rp.cpu().numpy()
    a.dirichlet_system_device([v.data_ptr() for v in d_vals], stream=s)
    rng = np.random.default_rng(0)
    g_u, s_u = rng.standard_normal(a.n_u), rng.standard_normal(a.n_u)
    g_p = rng.standard_normal(a.n_p)
    dg_u, ds_u, dg_p = (torch.from_numpy(x).to(dev) for x in (g_u, s_u, g_p))
    a.dirichlet_rhs_device(d_ru.data_ptr(), d_rp.data_ptr(), d_g_u=dg_u.data_ptr(), d_g_p=dg_p.data_ptr(),
                           d_sub_u=ds_u.data_ptr(), stream=s)
    a.check(s)
    masks = (mu, mu, mp)
    for b in range(3):
        rp_, ci_, _ = a.pattern(b)
        want = O.dirichlet_rows(rp_, ci_, before[b], masks[b], b == 0)
        assert np.array_equal(d_vals[b].cpu().numpy(), want), b
    # identity rows in block (0,0): each Dirichlet row sums to one, at its diagonal
    rp0_, ci0_, _ = a.pattern(0)
    v00 = d_vals[0].cpu().numpy()
    for r in np.nonzero(mu)[0][:50]:
        seg = slice(rp0_[r], rp0_[r + 1])
        assert v00[seg].sum() == 1.0 and v00[seg][ci0_[seg] == r][0] == 1.0
    assert np.array_equal(d_ru.cpu().numpy(), O.dirichlet_rhs(ru0, mu, g_u, s_u))
    assert np.array_equal(d_rp.cpu().numpy(), O.dirichlet_rhs(rp0, mp, g_p))


def test_dirichlet_laplace_rows_and_load(env):
    F, torch = env
    dev = torch.device("cuda:0")
    xyz, el = F.structured_mesh(3, 1, seed=1)
    a = F.Assembler(F.LAPLACE, xyz, el, fe_order=1, source=1.0)
    on_boundary = (np.abs(xyz) < 1e-12).any(axis=1) | (np.abs(xyz - 1.0) < 1e-12).any(axis=1)
    a.set_dirichlet(on_boundary.astype(np.uint8))
    d_v = torch.empty(a.block_info(0)[2], dtype=torch.float64, device=dev)
    d_b = torch.empty(a.n_u, dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream().cuda_stream
    a.assemble_device(None, None, [d_v.data_ptr()], d_b.data_ptr(), None, stream=s)
    v0, b0 = d_v.cpu().numpy(), d_b.cpu().numpy()
    a.dirichlet_system_device([d_v.data_ptr()], stream=s)
    a.dirichlet_rhs_device(d_b.data_ptr(), stream=s)  # homogeneous values
    a.check(s)
    rp_, ci_, _ = a.pattern(0)
    assert np.array_equal(d_v.cpu().numpy(), O.dirichlet_rows(rp_, ci_, v0, on_boundary, True))
    assert np.array_equal(d_b.cpu().numpy(), O.dirichlet_rhs(b0, on_boundary))
    # the system with identity rows is non-singular: solve it on the host
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    K = sp.csr_matrix((d_v.cpu().numpy(), ci_, rp_), shape=(a.n_u, a.n_u))
    x = spla.spsolve(K.tocsc(), d_b.cpu().numpy())
    assert np.all(np.isfinite(x)) and np.allclose(x[on_boundary], 0.0) and x[~on_boundary].max() > 0
