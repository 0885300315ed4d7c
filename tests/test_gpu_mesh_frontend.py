"""Mesh front end on the device against the host generator and the oracle:
the structured generator (buildMesh3D) made on the device bit for bit, the
P2 mesh of an unstructured P1 mesh (buildP2ofP1MeshEdge) against the oracle's
restatement, assembly on an unstructured medit mesh refined on the device,
and a device-resident mesh handed to the assembler without a host copy."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-6  # relative Frobenius error per block (FP32 element integrals)


@pytest.fixture(scope="module")
def F():
    import feddlib_gb300 as F
    return F


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def unstructured_p1(F, M, seed):
    """A structured P1 mesh with its nodes renumbered at random, its elements
    shuffled and each element's vertices 1, 2, 3 rotated (an even
    permutation: orientation kept), so nothing of the lattice order is left."""
    xyz, el = F.structured_mesh(M, 1, seed=seed)
    rng = np.random.default_rng(seed)
    perm = rng.permutation(xyz.shape[0])
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.size)
    xyz_u = xyz[perm]
    el_u = inv[el][rng.permutation(el.shape[0])]
    el_u = np.ascontiguousarray(el_u[:, [0, 2, 3, 1]], dtype=np.int32)
    return np.ascontiguousarray(xyz_u), el_u


@pytest.mark.parametrize("M,order,amp", [(1, 1, 0.1), (1, 2, 0.1), (3, 1, 0.1), (3, 2, 0.1), (8, 2, 0.1),
                                         (5, 2, 0.0), (7, 1, 0.25)])
def test_structured_device_is_bitwise_host(F, torch, M, order, amp):
    xh, ch = F.structured_mesh(M, order, seed=11, amp=amp)
    xd, cd = F.structured_mesh_device(M, order, seed=11, amp=amp)
    torch.cuda.synchronize()
    assert np.array_equal(bits(xd.cpu().numpy()), bits(xh))
    np.testing.assert_array_equal(cd.cpu().numpy(), ch)


@pytest.mark.parametrize("M,seed", [(2, 1), (5, 4)])
def test_p2_of_p1_matches_oracle(F, torch, M, seed):
    x1, e1 = unstructured_p1(F, M, seed)
    ox, oe = O.p2_of_p1(x1, e1)
    # host arrays in and out
    hx, he = F.p2_of_p1(x1, e1)
    np.testing.assert_array_equal(he, oe)
    assert np.array_equal(bits(hx), bits(ox))
    # device tensors in and out
    dx, de = F.p2_of_p1(torch.from_numpy(x1).cuda(), torch.from_numpy(e1).cuda())
    np.testing.assert_array_equal(de.cpu().numpy(), oe)
    assert np.array_equal(bits(dx.cpu().numpy()), bits(ox))


def test_p2_of_p1_of_structured_is_structured_p2(F):
    """P2-of-P1 of the structured P1 mesh is the structured P2 mesh up to node
    numbering: the same element node coordinates, bit for bit."""
    x1, e1 = F.structured_mesh(4, 1, seed=5)
    x2, e2 = F.structured_mesh(4, 2, seed=5)
    y2, d2 = F.p2_of_p1(x1, e1)
    assert y2.shape == x2.shape
    assert np.array_equal(bits(y2[d2]), bits(x2[e2]))


def test_p2_of_p1_rejects_bad_element(F):
    x1, e1 = F.structured_mesh(2, 1, seed=1)
    e1 = e1.copy()
    e1[3, 1] = x1.shape[0] + 7
    with pytest.raises(F.FeddError) as ei:
        F.p2_of_p1(x1, e1)
    assert ei.value.code == 3  # FEDD_ERR_MESH


def test_navier_stokes_on_unstructured_medit_mesh(F, tmp_path):
    """medit P1 mesh -> P2 on the device -> Taylor-Hood assembly, against the
    oracle assembling on its own P2-of-P1 mesh."""
    x1, e1 = unstructured_p1(F, 3, 8)
    path = tmp_path / "cube.mesh"
    F.medit_write(path, x1, e1)
    m = F.medit_read(path)
    x2, e2 = F.p2_of_p1(m["coords"], m["tets"])
    ox2, oe2 = O.p2_of_p1(x1, e1)
    np.testing.assert_array_equal(e2, oe2)
    u = F.fourier_field(x2, seed=8)
    p = F.uniform_field(8, x1.shape[0])
    a = F.Assembler(F.NAVIER_STOKES, x2, e2, elements_p=m["tets"], num_nodes_p=x1.shape[0],
                    viscosity=0.01, density=1.0, newton=True)
    vals, ru, rp = a.assemble(u=u, p=p)
    blocks, (ou, op) = O.assemble_ns(ox2, oe2, e1, x1.shape[0], u, p, 0.01, 1.0, True, blocks=(0, 1, 2))
    for b in range(3):
        prp, pci, _ = a.pattern(b)
        np.testing.assert_array_equal(prp, blocks[b][0])
        np.testing.assert_array_equal(pci, blocks[b][1])
        assert rel(vals[b], blocks[b][2]) < TOL_FP32, b
    assert rel(ru, ou) < TOL_FP32
    assert rel(rp, op) < TOL_FP32


def test_elasticity_on_unstructured_mesh(F):
    x1, e1 = unstructured_p1(F, 3, 12)
    x2, e2 = F.p2_of_p1(x1, e1)
    a = F.Assembler(F.LINEAR_ELASTICITY, x2, e2, E=1000.0, poisson_ratio=0.3)
    (v,), r, _ = a.assemble(u=np.zeros(3 * x2.shape[0]))
    Lw = O.law_from_E_nu(O.LAW_SKR1, 1000.0, 0.3)
    (orp, oci, ov), _ = O.assemble_vec(1, Lw, 4, x2, e2, np.zeros(3 * x2.shape[0]))
    prp, pci, _ = a.pattern(0)
    np.testing.assert_array_equal(prp, orp)
    np.testing.assert_array_equal(pci, oci)
    assert rel(v, ov) < TOL_FP32


def test_device_resident_mesh_assembles_bitwise(F, torch):
    """A mesh made on the device and handed over as device pointers gives the
    same pattern and values, bit for bit, as the same mesh from host arrays."""
    M, seed = 3, 6
    xd2, ed2 = F.structured_mesh_device(M, 2, seed=seed)
    xd1, ed1 = F.structured_mesh_device(M, 1, seed=seed)
    xh2, eh2 = F.structured_mesh(M, 2, seed=seed)
    xh1, eh1 = F.structured_mesh(M, 1, seed=seed)
    u = F.fourier_field(xh2, seed=seed)
    p = F.uniform_field(seed, xh1.shape[0])
    kw = dict(num_nodes_p=xh1.shape[0], viscosity=0.01, density=1.0, newton=True)
    ad = F.Assembler(F.NAVIER_STOKES, xd2, ed2, elements_p=ed1, **kw)
    ah = F.Assembler(F.NAVIER_STOKES, xh2, eh2, elements_p=eh1, **kw)
    vd, rud, rpd = ad.assemble(u=u, p=p)
    vh, ruh, rph = ah.assemble(u=u, p=p)
    for b in range(3):
        np.testing.assert_array_equal(ad.pattern(b)[1], ah.pattern(b)[1])
        assert np.array_equal(bits(vd[b]), bits(vh[b]))
    assert np.array_equal(bits(rud), bits(ruh)) and np.array_equal(bits(rpd), bits(rph))
