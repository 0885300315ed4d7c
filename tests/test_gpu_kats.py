"""Known-answer properties of the assembled operators, checked on the
engine's own CSR output (the oracle's restatement passes the same checks in
test_oracle.py):
- rigid-body modes (three translations, three infinitesimal rotations) lie in
  the null space of every elasticity law's tangent at zero displacement;
- the hyperelastic tangents are symmetric at a nonzero displacement;
- Laplace stiffness rows sum to zero and the load vector sums to f |Omega|."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-6


@pytest.fixture(scope="module")
def F():
    import feddlib_gb300 as F
    return F


@pytest.fixture(scope="module")
def sp():
    sp = pytest.importorskip("scipy.sparse")
    pytest.importorskip("scipy.sparse.linalg")
    return sp


def csr(sp, a, vals):
    rp, ci, shape = a.pattern(0)
    return sp.csr_matrix((vals, ci, rp), shape=shape)


def assembler(F, problem, xyz, el):
    if problem == "ANISO_FIBER":
        return F.Assembler(F.ANISO_FIBER, xyz, el, E=32.0 / 11.0, poisson_ratio=5.0 / 11.0, k1=2.0, k2=1.0,
                           fiber_angle_deg=40.0)
    return F.Assembler(getattr(F, problem), xyz, el, E=1000.0, poisson_ratio=0.3)


def rigid_modes(xyz):
    n = xyz.shape[0]
    modes = []
    for d in range(3):
        m = np.zeros((n, 3))
        m[:, d] = 1.0
        modes.append(m.ravel())
    for w in np.eye(3):
        modes.append(np.cross(w, xyz).ravel())
    return modes


LAWS = ["LINEAR_ELASTICITY", "NONLINEAR_ELASTICITY", "NONLINEAR_ELASTICITY2", "ANISO_FIBER"]


@pytest.mark.parametrize("problem", LAWS)
def test_rigid_body_modes_in_null_space(F, sp, problem):
    xyz, el = F.structured_mesh(3, 2, seed=41)
    a = assembler(F, problem, xyz, el)
    (v,), _, _ = a.assemble(u=np.zeros(3 * xyz.shape[0]))
    K = csr(sp, a, v)
    knorm = sp.linalg.norm(K)
    for m in rigid_modes(xyz):
        assert np.linalg.norm(K @ m) <= TOL_FP32 * knorm * np.linalg.norm(m)


@pytest.mark.parametrize("problem", LAWS)
def test_tangent_is_symmetric(F, sp, problem):
    xyz, el = F.structured_mesh(3, 2, seed=42)
    u = F.fourier_field(xyz, seed=42, kmin=1, kmax=2, scale=0.004)
    a = assembler(F, problem, xyz, el)
    (v,), _, _ = a.assemble(u=u)
    K = csr(sp, a, v)
    assert sp.linalg.norm(K - K.T) <= TOL_FP32 * sp.linalg.norm(K)


@pytest.mark.parametrize("order", [1, 2])
def test_laplace_rows_sum_to_zero_and_load_to_volume(F, order):
    xyz, el = F.structured_mesh(4, order, seed=43)
    f = 3.0
    a = F.Assembler(F.LAPLACE, xyz, el, fe_order=order, source=f)
    (v,), load, _ = a.assemble()
    rp, _, _ = a.pattern(0)
    rows = np.add.reduceat(v, rp[:-1])
    assert np.abs(rows).max() <= 1e-12 * np.abs(v).max()
    # |Omega| from the vertex positions of the (straight-edged) tetrahedra
    p = xyz[el[:, :4]]
    vol = np.abs(np.einsum("ij,ij->i", np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), p[:, 3] - p[:, 0])).sum() / 6
    assert abs(load.sum() - f * vol) <= 1e-12 * f * vol
