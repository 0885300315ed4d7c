"""Unstructured meshes: the Delaunay tetrahedralisation of seeded random
points (scipy), oriented to det B > 0, refined to P2 on the device.  Such
meshes have vertices in more than 32 elements, which the structured meshes
never reach: the row kernels then take each node's incidences from the second
word of their per-lane incidence list.  Patterns bit-exact and values within
the usual bounds against the oracle."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-6
TOL_FP64 = 1e-12


@pytest.fixture(scope="module")
def F():
    import feddlib_gb300 as F
    return F


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def delaunay():
    spatial = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(7)
    pts = rng.random((400, 3))
    t = np.ascontiguousarray(spatial.Delaunay(pts).simplices, dtype=np.int32)
    p = pts[t]
    det = np.einsum("ij,ij->i", np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), p[:, 3] - p[:, 0])
    flip = det < 0
    t[flip, 1], t[flip, 2] = t[flip, 2].copy(), t[flip, 1].copy()
    valence = np.bincount(t.ravel(), minlength=pts.shape[0])
    assert valence.max() > 32, "the mesh must reach the second incidence word"
    return np.ascontiguousarray(pts), np.ascontiguousarray(t)


def test_laplace_p1_on_delaunay_mesh(F, delaunay):
    xyz, el = delaunay
    a = F.Assembler(F.LAPLACE, xyz, el, fe_order=1, source=1.0)
    (v,), b, _ = a.assemble()
    (orp, oci, ov) = O.assemble_laplace(1, 1, xyz, el)
    ob = O.assemble_rhs(1, 1, xyz, el, 1.0)
    rp, ci, _ = a.pattern(0)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert rel(v, ov) < TOL_FP64
    assert rel(b, ob) < TOL_FP64


@pytest.mark.parametrize("problem,law,npts", [("LINEAR_ELASTICITY", O.LAW_SKR1, 4),
                                               ("NONLINEAR_ELASTICITY", O.LAW_SKR2, 5),
                                               ("NONLINEAR_ELASTICITY2", O.LAW_SKR3, 5)])
def test_elasticity_on_delaunay_p2_mesh(F, delaunay, problem, law, npts):
    """The tangent at zero displacement: a displacement field interpolated on
    the Delaunay slivers inverts some of them (det F < 0, which the engine
    reports), so the sliver mesh checks the tangent's assembly alone."""
    x1, e1 = delaunay
    x2, e2 = F.p2_of_p1(x1, e1)
    u = np.zeros(3 * x2.shape[0])
    a = F.Assembler(getattr(F, problem), x2, e2, E=1000.0, poisson_ratio=0.3)
    (v,), r, _ = a.assemble(u=u)
    (orp, oci, ov), ores = O.assemble_vec(1, O.law_from_E_nu(law, 1000.0, 0.3), npts, x2, e2, u)
    rp, ci, _ = a.pattern(0)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert rel(v, ov) < TOL_FP32
    # zero displacement: zero stress (skr3's isochoric split cancels to rounding)
    assert np.abs(r).max() <= 1e-6 * np.abs(v).max() and np.abs(ores).max() <= 1e-12 * np.abs(ov).max()


def test_navier_stokes_on_delaunay_p2_p1_mesh(F, delaunay):
    x1, e1 = delaunay
    x2, e2 = F.p2_of_p1(x1, e1)
    u = F.fourier_field(x2, seed=7)
    p = F.uniform_field(7, x1.shape[0])
    a = F.Assembler(F.NAVIER_STOKES, x2, e2, elements_p=e1, num_nodes_p=x1.shape[0], viscosity=0.01,
                    density=1.0, newton=True)
    vals, ru, rp = a.assemble(u=u, p=p)
    blocks, (ou, op) = O.assemble_ns(x2, e2, e1, x1.shape[0], u, p, 0.01, 1.0, True, blocks=(0, 1, 2))
    for b in range(3):
        prp, pci, _ = a.pattern(b)
        np.testing.assert_array_equal(prp, blocks[b][0])
        np.testing.assert_array_equal(pci, blocks[b][1])
        assert rel(vals[b], blocks[b][2]) < TOL_FP32, b
    assert rel(ru, ou) < TOL_FP32
    assert rel(rp, op) < TOL_FP32


def test_laplace_p2_on_delaunay_p2_mesh(F, delaunay):
    x1, e1 = delaunay
    x2, e2 = F.p2_of_p1(x1, e1)
    a = F.Assembler(F.LAPLACE, x2, e2, fe_order=2, source=2.0)
    (v,), load, _ = a.assemble()
    orp, oci, ov = O.assemble_laplace(2, 5, x2, e2)
    rp, ci, _ = a.pattern(0)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert rel(v, ov) < TOL_FP64
    assert rel(load, O.assemble_rhs(2, 5, x2, e2, 2.0)) < TOL_FP64


def test_navier_stokes_fixed_point_on_delaunay_mesh(F, delaunay):
    x1, e1 = delaunay
    x2, e2 = F.p2_of_p1(x1, e1)
    u = F.fourier_field(x2, seed=8)
    p = F.uniform_field(8, x1.shape[0])
    a = F.Assembler(F.NAVIER_STOKES, x2, e2, elements_p=e1, num_nodes_p=x1.shape[0], viscosity=0.05,
                    density=2.0, newton=False)
    vals, ru, rp = a.assemble(u=u, p=p)
    blocks, (ou, op) = O.assemble_ns(x2, e2, e1, x1.shape[0], u, p, 0.05, 2.0, False, blocks=(0, 1, 2))
    for b in range(3):
        assert rel(vals[b], blocks[b][2]) < TOL_FP32, b
    assert rel(ru, ou) < TOL_FP32 and rel(rp, op) < TOL_FP32


def test_generalized_newtonian_on_delaunay_mesh(F, delaunay):
    """The viscous rows folded into the velocity rows, on nodes with more than
    32 elements; against the oracle's element restatement summed into sparse
    matrices."""
    sparse = pytest.importorskip("scipy.sparse")
    x1, e1 = delaunay
    x2, e2 = F.p2_of_p1(x1, e1)
    u = F.fourier_field(x2, seed=9) * 0.5
    p = F.uniform_field(9, x1.shape[0])
    prm = [1.902, 0.22, 0.056, 0.00345, 1.25]
    a = F.Assembler(F.NAVIER_STOKES, x2, e2, elements_p=e1, num_nodes_p=x1.shape[0], viscosity=0.01,
                    density=1.0, newton=True)
    a.set_viscosity_law(0, prm, gamma_min=1e-12)
    vals, ru, rp = a.assemble(u=u, p=p)
    L = O.visc_law(0, prm, 1e-12)
    n_u, n1 = 3 * x2.shape[0], x1.shape[0]
    coo = [([], [], []) for _ in range(3)]
    oru = np.zeros(n_u); orp = np.zeros(n1)
    U = u.reshape(-1, 3)
    for e in range(e2.shape[0]):
        Je, re = O.elem_gn(x2[e2[e]], U[e2[e]].ravel(), p[e1[e]], L, 1.0, True)
        vd = (3 * e2[e][:, None] + np.arange(3)).ravel()
        for k, (rows, cols, blk) in enumerate(((vd, vd, Je[:30, :30]), (vd, e1[e], Je[:30, 30:]),
                                               (e1[e], vd, Je[30:, :30]))):
            coo[k][0].append(np.repeat(rows, len(cols))); coo[k][1].append(np.tile(cols, len(rows)))
            coo[k][2].append(blk.ravel())
        np.add.at(oru, vd, re[:30]); np.add.at(orp, e1[e], re[30:])
    for b, shape in enumerate(((n_u, n_u), (n_u, n1), (n1, n_u))):
        ob = sparse.coo_matrix((np.concatenate(coo[b][2]), (np.concatenate(coo[b][0]), np.concatenate(coo[b][1]))),
                               shape=shape).tocsr()
        rpt, ci, _ = a.pattern(b)
        M = sparse.csr_matrix((vals[b], ci, rpt), shape=shape)
        assert sparse.linalg.norm(M - ob) / sparse.linalg.norm(ob) < TOL_FP32, b
    assert rel(ru, oru) < TOL_FP32 and rel(rp, orp) < TOL_FP32


def test_fibre_law_on_delaunay_p2_mesh(F, delaunay):
    """The two-fibre law's tangent at zero displacement on the sliver mesh
    (fibres at +-40 degrees in the xy-plane; at F = I they are at I4 = 1,
    the onset of the tension-only branch)."""
    x1, e1 = delaunay
    x2, e2 = F.p2_of_p1(x1, e1)
    u = np.zeros(3 * x2.shape[0])
    a = F.Assembler(F.ANISO_FIBER, x2, e2, E=32.0 / 11.0, poisson_ratio=5.0 / 11.0, k1=2.0, k2=1.0,
                    fiber_angle_deg=40.0)
    (v,), r, _ = a.assemble(u=u)
    Lw = O.LawSpec(O.LAW_ANISO, mu=1.0, lam=10.0, k1=2.0, k2=1.0, angle_deg=40.0)
    (orp, oci, ov), _ = O.assemble_vec(1, Lw, 4, x2, e2, u)
    rp, ci, _ = a.pattern(0)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert rel(v, ov) < TOL_FP32
