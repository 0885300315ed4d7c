"""GPU edge cases of the assembly path against the FP64 oracle: a mesh of a
single element, nodes that no element references (their rows are empty and
their residual entries zero, as a Tpetra matrix built by FE::addFeBlock
leaves them), and a mesh without elements (rejected).  Both the host-buffer
path and the device path are checked, the latter bit for bit against the
former."""
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


def one_element(xyz, el, e=0):
    """Element e of a mesh as a mesh of its own (nodes renumbered 0..npe-1)."""
    nodes = el[e]
    return np.ascontiguousarray(xyz[nodes]), np.arange(nodes.shape[0], dtype=np.int32)[None, :]


def with_isolated(xyz, el, at, far=10.0):
    """The mesh with an unreferenced node inserted before each old id in
    `at` (len(xyz) appends one at the end); their coordinates lie outside
    the mesh.  Returns the new coordinates, connectivity and the map old id
    -> new id."""
    n = xyz.shape[0]
    at = sorted(at)
    new_id = np.arange(n, dtype=np.int64) + np.searchsorted(np.asarray(at), np.arange(n), side="right")
    m = n + len(at)
    out = np.zeros((m, 3))
    out[new_id] = xyz
    iso = np.setdiff1d(np.arange(m), new_id)
    out[iso] = far + np.arange(len(iso))[:, None] * np.array([1.0, 2.0, 3.0])
    return out, new_id[el].astype(np.int32), new_id, iso


def _device_path_matches(F, a, u, p, hv, hru, hrp):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    du = torch.from_numpy(np.ascontiguousarray(u)).to(dev) if u is not None else None
    dp = torch.from_numpy(np.ascontiguousarray(p)).to(dev) if p is not None else None  # kept alive to the sync
    nb = a.nblocks
    dv = [torch.empty(max(a.block_info(b)[2], 1), dtype=torch.float64, device=dev) for b in range(nb)]
    dru = torch.empty(a.n_u, dtype=torch.float64, device=dev)
    drp = torch.empty(max(a.n_p, 1), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    a.assemble_device(du.data_ptr() if du is not None else None, dp.data_ptr() if dp is not None else None,
                      [t.data_ptr() for t in dv], dru.data_ptr(), drp.data_ptr() if a.n_p else None, stream=stream)
    torch.cuda.synchronize()
    for b in range(len(hv)):
        assert np.array_equal(dv[b].cpu().numpy()[:hv[b].shape[0]], hv[b]), b
    assert np.array_equal(dru.cpu().numpy(), hru)
    if hrp is not None:
        assert np.array_equal(drp.cpu().numpy()[:hrp.shape[0]], hrp)


# ----------------------------------------------------------- one element ----
def test_single_element_laplace_and_elasticity(F):
    xyz2, el2 = F.structured_mesh(1, 2, seed=11)
    for e in (0, 3):
        x, c = one_element(xyz2, el2, e)
        a = F.Assembler(F.LAPLACE, x, c, fe_order=2, source=1.5)
        (v,), load, _ = a.assemble()
        orp, oci, ov = O.assemble_laplace(2, 5, x, c)
        np.testing.assert_array_equal(a.pattern(0)[0], orp)
        np.testing.assert_array_equal(a.pattern(0)[1], oci)
        assert orp[-1] == 100
        assert rel(v, ov) < TOL_FP64
        assert rel(load, O.assemble_rhs(2, 5, x, c, 1.5)) < TOL_FP64
        a.close()

        u = F.fourier_field(x, seed=11, kmin=1, kmax=2, scale=0.02)
        a = F.Assembler(F.NONLINEAR_ELASTICITY, x, c, E=32.0 / 11.0, poisson_ratio=5.0 / 11.0)
        (v,), r, _ = a.assemble(u=u)
        (orp, oci, ov), ores = O.assemble_vec(1, O.law_from_E_nu(O.LAW_SKR2, 32.0 / 11.0, 5.0 / 11.0), 5, x, c, u)
        np.testing.assert_array_equal(a.pattern(0)[0], orp)
        np.testing.assert_array_equal(a.pattern(0)[1], oci)
        assert orp[-1] == 900
        assert rel(v, ov) < TOL_FP32
        assert rel(r, ores) < 1e-5
        _device_path_matches(F, a, u, None, [v], r, None)
        a.close()


def test_single_element_navier_stokes(F):
    xyz2, el2 = F.structured_mesh(1, 2, seed=12)
    for e in (1, 4):
        x2, c2 = one_element(xyz2, el2, e)
        x1, c1 = np.ascontiguousarray(x2[:4]), np.arange(4, dtype=np.int32)[None, :]
        u = F.fourier_field(x2, seed=12)
        p = F.uniform_field(12, 4)
        a = F.Assembler(F.NAVIER_STOKES, x2, c2, elements_p=c1, num_nodes_p=4, viscosity=0.01, density=1.0,
                        newton=True)
        vals, ru, rp = a.assemble(u=u, p=p)
        blocks, (ou, op) = O.assemble_ns(x2, c2, c1, 4, u, p, 0.01, 1.0, True, blocks=(0, 1, 2))
        for b in range(3):
            np.testing.assert_array_equal(a.pattern(b)[0], blocks[b][0])
            np.testing.assert_array_equal(a.pattern(b)[1], blocks[b][1])
            assert rel(vals[b], blocks[b][2]) < TOL_FP32, b
        assert blocks[0][0][-1] == 900 and blocks[1][0][-1] == 120 and blocks[2][0][-1] == 120
        assert rel(ru, ou) < TOL_FP32
        assert rel(rp, op) < TOL_FP32
        _device_path_matches(F, a, u, p, vals, ru, rp)
        a.close()


# ------------------------------------------------------- isolated nodes ----
def test_unreferenced_nodes_elasticity(F):
    xyz, el = F.structured_mesh(2, 2, seed=13)
    n = xyz.shape[0]
    x, c, new_id, iso = with_isolated(xyz, el, [0, n // 2, n])
    u = F.fourier_field(x, seed=13, kmin=1, kmax=2, scale=0.02)
    a = F.Assembler(F.NONLINEAR_ELASTICITY, x, c, E=32.0 / 11.0, poisson_ratio=5.0 / 11.0)
    (v,), r, _ = a.assemble(u=u)
    rp, ci, _ = a.pattern(0)
    (orp, oci, ov), ores = O.assemble_vec(1, O.law_from_E_nu(O.LAW_SKR2, 32.0 / 11.0, 5.0 / 11.0), 5, x, c, u)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert rel(v, ov) < TOL_FP32
    assert rel(r, ores) < 1e-5
    for k in iso:
        rows = 3 * k + np.arange(3)
        assert np.all(rp[rows + 1] == rp[rows])  # empty rows
        assert np.all(r[rows] == 0.0)
        assert not np.isin(ci // 3, [k]).any()  # and no column
    _device_path_matches(F, a, u, None, [v], r, None)
    a.close()


@pytest.mark.parametrize("iso_p1", [False, True])
def test_unreferenced_nodes_navier_stokes(F, iso_p1):
    """Unreferenced velocity nodes only (the vertices' velocity warps still
    assemble the pressure rows), and unreferenced pressure nodes as well (no
    P2 vertex maps onto them: the separate pressure-row pass runs)."""
    M = 2
    xyz2, el2 = F.structured_mesh(M, 2, seed=14)
    xyz1, el1 = F.structured_mesh(M, 1, seed=14)
    x2, c2, _, iso2 = with_isolated(xyz2, el2, [5, xyz2.shape[0]])
    x1, c1, _, iso1 = with_isolated(xyz1, el1, [0, 7] if iso_p1 else [])
    u = F.fourier_field(x2, seed=14)
    p = F.uniform_field(14, x1.shape[0])
    a = F.Assembler(F.NAVIER_STOKES, x2, c2, elements_p=c1, num_nodes_p=x1.shape[0], viscosity=0.01,
                    density=1.0, newton=True)
    vals, ru, rp = a.assemble(u=u, p=p)
    blocks, (ou, op) = O.assemble_ns(x2, c2, c1, x1.shape[0], u, p, 0.01, 1.0, True, blocks=(0, 1, 2))
    for b in range(3):
        np.testing.assert_array_equal(a.pattern(b)[0], blocks[b][0])
        np.testing.assert_array_equal(a.pattern(b)[1], blocks[b][1])
        assert rel(vals[b], blocks[b][2]) < TOL_FP32, b
    assert rel(ru, ou) < TOL_FP32
    assert rel(rp, op) < TOL_FP32
    r0 = a.pattern(0)[0]
    for k in iso2:
        rows = 3 * k + np.arange(3)
        assert np.all(r0[rows + 1] == r0[rows]) and np.all(ru[rows] == 0.0)
    r2 = a.pattern(2)[0]
    for k in iso1:
        assert r2[k + 1] == r2[k] and rp[k] == 0.0
    _device_path_matches(F, a, u, p, vals, ru, rp)
    a.close()


# ------------------------------------------------------------ no elements ----
def test_mesh_without_elements_is_rejected(F):
    xyz, _ = F.structured_mesh(1, 2, seed=1)
    with pytest.raises(F.FeddError) as ei:
        F.Assembler(F.LINEAR_ELASTICITY, xyz, np.zeros((0, 10), dtype=np.int32))
    assert ei.value.code == 1  # FEDD_ERR_ARG
