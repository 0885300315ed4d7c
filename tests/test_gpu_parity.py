"""GPU parity: the CUDA engine through the C ABI against the FP64 oracle.

Patterns must match bit-exactly.  Values: FP64 configuration (P1 Poisson)
within 1e-12 relative; FP32-bulk configurations within the stated bound
of 1e-6 relative Frobenius error per block, against the FP64 oracle."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-6   # relative Frobenius error per block (FP32 element integrals)
TOL_FP64 = 1e-12  # FP64 end to end (P1 Poisson)


@pytest.fixture(scope="module")
def F():
    import feddlib_gb300 as F
    return F


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def ns_case(F, M, seed):
    xyz2, el2 = F.structured_mesh(M, 2, seed=seed)
    xyz1, el1 = F.structured_mesh(M, 1, seed=seed)
    u = F.fourier_field(xyz2, seed=seed)
    p = F.uniform_field(seed, xyz1.shape[0])
    return xyz2, el2, xyz1, el1, u, p


# ---------------------------------------------------------------- Laplace ----
@pytest.mark.parametrize("M", [1, 4, 16])
def test_poisson_p1_fp64(F, M):
    xyz, el = F.structured_mesh(M, 1, seed=1)
    a = F.Assembler(F.LAPLACE, xyz, el, fe_order=1, source=1.0)
    (v,), load, _ = a.assemble()
    rp, ci, _ = a.pattern(0)
    orp, oci, ov = O.assemble_laplace(1, 1, xyz, el)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert rel(v, ov) < TOL_FP64
    ob = O.assemble_rhs(1, 1, xyz, el, 1.0)
    assert rel(load, ob) < TOL_FP64
    assert rp[-1] == 15 * M ** 3 + 21 * M ** 2 + 9 * M + 1


def test_laplace_p2(F):
    xyz, el = F.structured_mesh(3, 2, seed=2)
    a = F.Assembler(F.LAPLACE, xyz, el, fe_order=2, source=2.0)
    (v,), load, _ = a.assemble()
    rp, ci, _ = a.pattern(0)
    orp, oci, ov = O.assemble_laplace(2, 5, xyz, el)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert rel(v, ov) < TOL_FP64
    assert rel(load, O.assemble_rhs(2, 5, xyz, el, 2.0)) < TOL_FP64


def test_laplace_assfe_route(F):
    """FE::assemblyLaplaceAssFE through the Python facade: the oracle's
    AssembleFE_Laplace element (5-point rule for P1, determineDegree with
    UN Grad = 2) and the engine agree, and so do both FE routes
    (fe_test_laplace.cpp:104-161)."""
    xyz, el = F.structured_mesh(3, 1, seed=8)
    fe = F.FE((xyz, el))
    A1 = fe.assemblyLaplace(3, "P1", 1)
    A2 = fe.assemblyLaplaceAssFE(3, "P1", 1)
    orp, oci, ov = O.assemble_laplace(1, 5, xyz, el)
    np.testing.assert_array_equal(A2.rowptr, orp)
    np.testing.assert_array_equal(A2.colind, oci)
    assert rel(A2.values, ov) < TOL_FP64
    assert np.array_equal(A1.values, A2.values)


# --------------------------------------------------------------- elasticity --
@pytest.mark.parametrize("M", [1, 3])
def test_linear_elasticity_skr1_u0(F, M):
    xyz, el = F.structured_mesh(M, 2, seed=2)
    a = F.Assembler(F.LINEAR_ELASTICITY, xyz, el, E=1000.0, poisson_ratio=0.3)
    (v,), _, _ = a.assemble(u=None, residual=False)
    rp, ci, _ = a.pattern(0)
    L = O.law_from_E_nu(O.LAW_SKR1, 1000.0, 0.3)
    (orp, oci, ov), _ = O.assemble_vec(1, L, 4, xyz, el, None)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert rel(v, ov) < TOL_FP32
    assert rp[-1] == 9 * (230 * M ** 3 + 138 * M ** 2 + 24 * M + 1)


def _hyper_field(F, xyz, seed, scale):
    return F.fourier_field(xyz, seed=seed, kmin=1, kmax=2, scale=scale)


@pytest.mark.parametrize("problem,law,npts,E,nu", [
    ("LINEAR_ELASTICITY", O.LAW_SKR1, 4, 32.0 / 11.0, 5.0 / 11.0),
    ("NONLINEAR_ELASTICITY", O.LAW_SKR2, 5, 32.0 / 11.0, 5.0 / 11.0),
    ("NONLINEAR_ELASTICITY2", O.LAW_SKR3, 5, 32.0 / 11.0, 5.0 / 11.0),
    ("NONLINEAR_ELASTICITY2", O.LAW_SKR3, 5, 1000.0, 0.3),
])
def test_hyperelastic_tangent_and_residual(F, problem, law, npts, E, nu):
    xyz, el = F.structured_mesh(3, 2, seed=4)
    u = _hyper_field(F, xyz, 4, 0.02)
    a = F.Assembler(getattr(F, problem), xyz, el, E=E, poisson_ratio=nu)
    (v,), r, _ = a.assemble(u=u)
    Lw = O.law_from_E_nu(law, E, nu)
    (orp, oci, ov), ores = O.assemble_vec(1, Lw, npts, xyz, el, u)
    rp, ci, _ = a.pattern(0)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert rel(v, ov) < TOL_FP32
    assert rel(r, ores) < 1e-5  # residual: cancellation-prone sums of O(1) stresses


def test_fe_facade_neo_hooke_model_selects_skr3(F):
    """FE::assemblyNonLinearElasticity picks "NonLinearElasticity2" (skr3) for
    "Parameter/Neo-Hooke Modell" != 1 (FE_def.hpp:483-487), skr2 otherwise."""
    xyz, el = F.structured_mesh(2, 2, seed=9)
    u = _hyper_field(F, xyz, 9, 0.02)
    fe = F.FE((xyz, el))
    for model, law in ((1, O.LAW_SKR2), (2, O.LAW_SKR3)):
        params = {"Parameter": {"E": 32.0 / 11.0, "Poisson Ratio": 5.0 / 11.0, "Neo-Hooke Modell": model}}
        A, r = fe.assemblyNonLinearElasticity(3, "P2", 2, 3, u, params=params, assembleMode="Jacobian+Residual")
        (orp, oci, ov), ores = O.assemble_vec(1, O.law_from_E_nu(law, 32.0 / 11.0, 5.0 / 11.0), 5, xyz, el, u)
        assert rel(A.values, ov) < TOL_FP32, model
        assert rel(r, ores) < 1e-5, model


def test_aniso_plain_law(F):
    xyz, el = F.structured_mesh(2, 2, seed=5)
    u = _hyper_field(F, xyz, 5, 0.004)
    a = F.Assembler(F.ANISO_FIBER, xyz, el, E=32.0 / 11.0, poisson_ratio=5.0 / 11.0, k1=2.0, k2=1.0,
                    fiber_angle_deg=40.0)
    (v,), r, _ = a.assemble(u=u)
    Lw = O.LawSpec(O.LAW_ANISO, mu=1.0, lam=10.0, k1=2.0, k2=1.0, angle_deg=40.0)
    (orp, oci, ov), ores = O.assemble_vec(1, Lw, 4, xyz, el, u)
    assert rel(v, ov) < TOL_FP32
    assert rel(r, ores) < 1e-5


def test_element_matrices_hyper(F):
    xyz, el = F.structured_mesh(2, 2, seed=6)
    u = _hyper_field(F, xyz, 6, 0.02)
    a = F.Assembler(F.LINEAR_ELASTICITY, xyz, el, E=32.0 / 11.0, poisson_ratio=5.0 / 11.0)
    K, r = a.element_matrices(u=u, first=5, count=7)
    Lw = O.law_from_E_nu(O.LAW_SKR1, 32.0 / 11.0, 5.0 / 11.0)
    for k in range(7):
        e = 5 + k
        Ko, ro = O.elem_hyper(Lw, 4, xyz[el[e]], u.reshape(-1, 3)[el[e]].ravel())
        assert rel(K[k], Ko) < 2e-6
        assert rel(r[k], ro) < 1e-5


# ---------------------------------------------------------- Navier-Stokes ----
@pytest.mark.parametrize("M,newton", [(2, True), (4, True), (3, False)])
def test_navier_stokes_blocks(F, M, newton):
    xyz2, el2, xyz1, el1, u, p = ns_case(F, M, 3)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0],
                    viscosity=0.01, density=1.0, newton=newton)
    vals, ru, rp = a.assemble(u=u, p=p)
    blocks, (ou, op) = O.assemble_ns(xyz2, el2, el1, xyz1.shape[0], u, p, 0.01, 1.0, newton, blocks=(0, 1, 2, 3))
    for b in range(3):
        prp, pci, _ = a.pattern(b)
        np.testing.assert_array_equal(prp, blocks[b][0])
        np.testing.assert_array_equal(pci, blocks[b][1])
        assert rel(vals[b], blocks[b][2]) < TOL_FP32, b
    rp3, ci3, shape3 = a.pattern(3)
    assert rp3[-1] == 0 and blocks[3][0][-1] == 0
    assert rel(ru, ou) < TOL_FP32
    assert rel(rp, op) < TOL_FP32
    nnzB = 195 * M ** 3 + 171 * M ** 2 + 45 * M + 3
    assert a.block_info(1)[2] == nnzB and a.block_info(2)[2] == nnzB


@pytest.mark.parametrize("newton", [True, False])
def test_navier_stokes_constant_field(F, newton):
    """The reference's own NS cross-check field
    (core/AceFemAssembly/tests/fe_test_navierstokes.cpp:127-128: u = 100 in
    every component, p = 0): the Newton term vanishes for a constant field
    and advection dominates the diagonal blocks."""
    xyz2, el2, xyz1, el1, _, _ = ns_case(F, 3, 5)
    u = np.full(3 * xyz2.shape[0], 100.0)
    p = np.zeros(xyz1.shape[0])
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0],
                    viscosity=0.01, density=1.0, newton=newton)
    vals, ru, rp = a.assemble(u=u, p=p)
    blocks, (ou, op) = O.assemble_ns(xyz2, el2, el1, xyz1.shape[0], u, p, 0.01, 1.0, newton, blocks=(0, 1, 2))
    for b in range(3):
        assert rel(vals[b], blocks[b][2]) < TOL_FP32, b
    # the exact residual is zero: A and N annihilate a constant field (their
    # rows sum to zero), its divergence vanishes and p = 0; FP32 leaves
    # rounding at the operator's scale times the field
    scale = np.abs(vals[0]).max() * 100.0
    assert np.abs(ou).max() <= 1e-12 * scale and np.abs(op).max() <= 1e-12 * scale
    assert np.abs(ru).max() <= 1e-6 * scale and np.abs(rp).max() <= 1e-6 * scale
    if newton:  # W(u) = 0 for a constant u: Newton and FixedPoint Jacobians agree
        fp = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0],
                         viscosity=0.01, density=1.0, newton=False)
        vfp, _, _ = fp.assemble(u=u, p=p)
        assert rel(vals[0], vfp[0]) < TOL_FP32


def test_navier_stokes_element_matrices(F, golden):
    xyz2, el2, xyz1, el1, u, p = ns_case(F, 2, 3)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0],
                    viscosity=0.01, density=1.0, newton=True)
    K, r = a.element_matrices(u=u, p=p, first=0, count=10)
    for e in range(10):
        Jo, ro = O.elem_ns(xyz2[el2[e]], u.reshape(-1, 3)[el2[e]].ravel(), p[el1[e]], 0.01, 1.0, True)
        assert rel(K[e], Jo) < 2e-6
        assert rel(r[e], ro) < 2e-6


def test_determinism_bitwise(F):
    xyz2, el2, xyz1, el1, u, p = ns_case(F, 4, 8)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0],
                    viscosity=0.01, density=1.0, newton=True)
    v1, ru1, rp1 = a.assemble(u=u, p=p)
    v2, ru2, rp2 = a.assemble(u=u, p=p)
    for b in range(3):
        assert np.array_equal(v1[b].view(np.uint64), v2[b].view(np.uint64))
    assert np.array_equal(ru1.view(np.uint64), ru2.view(np.uint64))


def test_device_path_matches_host_path(F):
    torch = pytest.importorskip("torch")
    xyz2, el2, xyz1, el1, u, p = ns_case(F, 3, 9)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0],
                    viscosity=0.01, density=1.0, newton=True)
    hv, hru, hrp = a.assemble(u=u, p=p)
    dev = torch.device("cuda:0")
    du = torch.from_numpy(u).to(dev)
    dp = torch.from_numpy(p).to(dev)
    dv = [torch.empty(a.block_info(b)[2], dtype=torch.float64, device=dev) for b in range(3)]
    dru = torch.empty(a.n_u, dtype=torch.float64, device=dev)
    drp = torch.empty(a.n_p, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    a.assemble_device(du.data_ptr(), dp.data_ptr(), [t.data_ptr() for t in dv], dru.data_ptr(), drp.data_ptr(),
                      stream=stream)
    torch.cuda.synchronize()
    for b in range(3):
        assert np.array_equal(dv[b].cpu().numpy(), hv[b])
    assert np.array_equal(dru.cpu().numpy(), hru)
    assert np.array_equal(drp.cpu().numpy(), hrp)
    # element records with their NA part (one kernel), velocity rows (which
    # assemble the vertices' pressure rows as well: P1 nodes sit at the P2
    # vertices)
    assert a.launch_count() == 2


def test_navier_stokes_without_vertex_map(F):
    """P1 elements that list their vertices in another local order than the P2
    elements' first four nodes give no vertex map: a separate pressure-row pass
    assembles block (1,0) instead of the vertices' velocity-row warps.  Both
    follow the convention of the oracle (pressure basis k belongs to P1
    element node k)."""
    xyz2, el2, xyz1, el1, u, p = ns_case(F, 3, 4)
    fused = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0],
                        viscosity=0.01, density=1.0, newton=True)
    fused.set_profiling(True)
    fused.assemble(u=u, p=p)
    assert set(fused.stage_times()) == {"ns_record", "ns_vel_rows"}
    el1 = np.ascontiguousarray(el1[:, [1, 0, 2, 3]])
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0],
                    viscosity=0.01, density=1.0, newton=True)
    a.set_profiling(True)
    vals, ru, rp = a.assemble(u=u, p=p)
    assert set(a.stage_times()) == {"ns_record", "ns_vel_rows", "ns_pres_rows"}
    blocks, (ou, op) = O.assemble_ns(xyz2, el2, el1, xyz1.shape[0], u, p, 0.01, 1.0, True, blocks=(0, 1, 2))
    for b in range(3):
        prp, pci, _ = a.pattern(b)
        np.testing.assert_array_equal(prp, blocks[b][0])
        np.testing.assert_array_equal(pci, blocks[b][1])
        assert rel(vals[b], blocks[b][2]) < TOL_FP32, b
    assert rel(ru, ou) < TOL_FP32
    assert rel(rp, op) < TOL_FP32


# -------------------------------------------------------------- failures ----
def test_bad_connectivity_is_rejected(F):
    xyz, el = F.structured_mesh(2, 1, seed=1)
    el = el.copy()
    el[3, 2] = xyz.shape[0] + 5
    with pytest.raises(F.FeddError) as ei:
        F.Assembler(F.LAPLACE, xyz, el, fe_order=1)
    assert ei.value.code == 3  # FEDD_ERR_MESH


def test_degenerate_element_is_reported(F):
    xyz, el = F.structured_mesh(2, 2, seed=1)
    xyz = xyz.copy()
    xyz[el[0, 1]] = xyz[el[0, 0]]  # collapse an edge: det B = 0
    a = F.Assembler(F.LINEAR_ELASTICITY, xyz, el)
    with pytest.raises(F.FeddError) as ei:
        a.assemble(u=None, residual=False)
    assert ei.value.code == 4  # FEDD_ERR_NONFINITE


def test_geometry_fp64_inverse_rounded_once(F):
    """The element kernels' geometry: det B and B^-1 = adj(B) / det B in FP64
    as SmallMatrix::computeDet / computeInverse form them
    (feddlib/core/General/SmallMatrix.hpp:317-368), each entry of B^-1 then
    rounded once to FP32: every entry lies within half an FP32 ulp of the
    oracle's FP64 inverse (a separately rounded adjugate and determinant
    would miss that bound on a large share of the entries)."""
    xyz, el = F.structured_mesh(6, 2, seed=7)
    a = F.Assembler(F.LINEAR_ELASTICITY, xyz, el, E=1000.0, poisson_ratio=0.3)
    det, binv = a.element_geometry()
    a.close()
    ne = el.shape[0]
    dets = np.zeros(ne); inv = np.zeros((ne, 3, 3))
    for e in range(ne):
        dets[e], _, inv[e] = O.geometry(np.ascontiguousarray(xyz[el[e, :4]]))
    rel_det = np.abs(det - dets) / np.abs(dets)
    assert rel_det.max() <= 1e-13, rel_det.max()
    # half an FP32 ulp of the exact entry, plus the FP64 rounding of the
    # cofactors (relative to the matrix: a cofactor that cancels to zero in one
    # FP64 evaluation may keep a rounding residue in another)
    got = binv.astype(np.float64)
    half_ulp = 0.5 * np.spacing(np.abs(inv).astype(np.float32)).astype(np.float64)
    fp64 = 1e-13 * np.abs(inv).max(axis=(1, 2), keepdims=True)
    excess = np.abs(got - inv) - (half_ulp + fp64)
    assert excess.max() <= 0.0, (excess.max(), np.unravel_index(excess.argmax(), excess.shape))
    # rounding twice (FP32 adjugate and determinant, then their quotient) misses the bound
    adj32 = np.stack([np.linalg.inv(np.ascontiguousarray(xyz[el[e, 1:4]] - xyz[el[e, 0]]).T) * dets[e]
                      for e in range(ne)]).astype(np.float32)
    twice = (adj32 / dets.astype(np.float32)[:, None, None]).astype(np.float64)
    assert (np.abs(twice - inv) > half_ulp + fp64).mean() > 0.05


# ------------------------------------------------ residual coefficients ----
def _ns_residual_oracle(xyz2, el2, el1, n1, u, p, visc, dens, coeff):
    """The assembled residual with FE::assemblyNavierStokes' coeff: each
    element's (coeff .* ANB) x (AssembleFENavierStokes_def.hpp:199-224),
    scattered node-wise."""
    U = u.reshape(-1, 3)
    ru, rp = np.zeros(3 * xyz2.shape[0]), np.zeros(n1)
    for e in range(el2.shape[0]):
        _, r = O.elem_ns(xyz2[el2[e]], U[el2[e]].ravel(), p[el1[e]], visc, dens, True, coeff=coeff)
        for a in range(10):
            ru[3 * el2[e, a]:3 * el2[e, a] + 3] += r[3 * a:3 * a + 3]
        rp[el1[e]] += r[30:]
    return ru, rp


def test_navier_stokes_residual_coefficients(F):
    """setCoeff's block factors scale the residual's blocks, host and device
    paths and element residuals alike, and leave the matrices alone; all ones
    gives back the unscaled residual bit for bit."""
    torch = pytest.importorskip("torch")
    xyz2, el2, xyz1, el1, u, p = ns_case(F, 2, 5)
    co = (0.5, 2.0, -1.5, 3.0)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0],
                    viscosity=0.01, density=1.0, newton=True)
    v1, ru1, rp1 = a.assemble(u=u, p=p)
    a.set_coeff(np.reshape(co, (2, 2)))
    v2, ru2, rp2 = a.assemble(u=u, p=p)
    for b in range(3):
        assert np.array_equal(v1[b], v2[b])
    ou, op = _ns_residual_oracle(xyz2, el2, el1, xyz1.shape[0], u, p, 0.01, 1.0, co)
    assert rel(ru2, ou) < TOL_FP32 and rel(rp2, op) < TOL_FP32
    # the device path, bit for bit
    dev = torch.device("cuda:0")
    du, dp = torch.from_numpy(u).to(dev), torch.from_numpy(p).to(dev)
    dv = [torch.empty(a.block_info(b)[2], dtype=torch.float64, device=dev) for b in range(3)]
    dru = torch.empty(a.n_u, dtype=torch.float64, device=dev)
    drp = torch.empty(a.n_p, dtype=torch.float64, device=dev)
    a.assemble_device(du.data_ptr(), dp.data_ptr(), [t.data_ptr() for t in dv], dru.data_ptr(), drp.data_ptr(),
                      stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(dru.cpu().numpy(), ru2) and np.array_equal(drp.cpu().numpy(), rp2)
    # element residuals (the AssembleFE view)
    K, r = a.element_matrices(u=u, p=p, first=3, count=4)
    U = u.reshape(-1, 3)
    for k in range(4):
        e = 3 + k
        Jo, ro = O.elem_ns(xyz2[el2[e]], U[el2[e]].ravel(), p[el1[e]], 0.01, 1.0, True, coeff=co)
        assert rel(K[k], Jo) < 2e-6 and rel(r[k], ro) < 2e-6, e
    a.set_coeff(np.ones((2, 2)))
    _, ru3, rp3 = a.assemble(u=u, p=p)
    assert np.array_equal(ru3, ru1) and np.array_equal(rp3, rp1)
    with pytest.raises(F.FeddError) as ei:
        a.set_coeff([[1.0, float("nan")], [1.0, 1.0]])
    assert ei.value.code == 1  # FEDD_ERR_ARG
    a.close()
    xyz, el = F.structured_mesh(1, 2, seed=5)
    e = F.Assembler(F.LINEAR_ELASTICITY, xyz, el)
    with pytest.raises(F.FeddError) as ei:
        e.set_coeff(np.ones((2, 2)))
    assert ei.value.code == 7  # FEDD_ERR_STATE
    e.close()


def test_generalized_newtonian_residual_coefficients(F):
    """With a viscosity law the viscous residual (and the outflow term) is
    part of ANB_uu u (AssembleFEGeneralizedNewtonian_def.hpp:928-970): the
    scaled residual is c_uu R_uu + c_up R_up, the two parts taken from the
    unscaled residual at p and at p = 0."""
    xyz2, el2, xyz1, el1, u, p = ns_case(F, 2, 6)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0],
                    viscosity=0.0, density=1.0, newton=True)
    a.set_viscosity_law(F.Assembler.CARREAU_YASUDA, (1.902, 0.22, 0.056, 0.00345, 1.25), 1e-12)
    _, ru, rp = a.assemble(u=u, p=p)
    _, ru0, _ = a.assemble(u=u, p=np.zeros_like(p))
    co = (0.25, -2.0, 4.0, 1.0)
    a.set_coeff(np.reshape(co, (2, 2)))
    _, rus, rps = a.assemble(u=u, p=p)
    assert rel(rus, co[0] * ru0 + co[1] * (ru - ru0)) < TOL_FP32
    assert rel(rps, co[2] * rp) < 1e-12
    K, r = a.element_matrices(u=u, p=p, first=0, count=3)
    a.set_coeff(np.ones((2, 2)))
    K1, r1 = a.element_matrices(u=u, p=p, first=0, count=3)
    _, r0 = a.element_matrices(u=u, p=np.zeros_like(p), first=0, count=3)
    assert np.array_equal(K, K1)
    assert rel(r[:, :30], co[0] * r0[:, :30] + co[1] * (r1[:, :30] - r0[:, :30])) < 1e-6
    assert rel(r[:, 30:], co[2] * r1[:, 30:]) < 1e-12
    a.close()


# ------------------------------------------------------ E per element ----
@pytest.mark.parametrize("problem,law,npts", [
    ("LINEAR_ELASTICITY", O.LAW_SKR1, 4),
    ("NONLINEAR_ELASTICITY", O.LAW_SKR2, 5),
    ("NONLINEAR_ELASTICITY2", O.LAW_SKR3, 5),
])
def test_element_moduli_field(F, problem, law, npts):
    """The E-field variant of FE::assemblyNonLinearElasticity
    (FE_def.hpp:538-614): every element assembled with its own Young's
    modulus (updateParameter("E", eModVec[T])), against the oracle's
    elements at those moduli; clearing the field gives back the uniform
    assembly bit for bit."""
    xyz, el = F.structured_mesh(2, 2, seed=10)
    u = _hyper_field(F, xyz, 10, 0.02)
    Ev = np.random.default_rng(10).uniform(0.5, 4.0, el.shape[0])
    nu = 5.0 / 11.0
    a = F.Assembler(getattr(F, problem), xyz, el, E=32.0 / 11.0, poisson_ratio=nu)
    (v0,), r0, _ = a.assemble(u=u)
    a.set_element_moduli(Ev)
    (v,), r, _ = a.assemble(u=u)
    rp, ci, _ = a.pattern(0)
    n = 3 * xyz.shape[0]
    Kd, rd = np.zeros((n, n)), np.zeros(n)
    U = u.reshape(-1, 3)
    for e in range(el.shape[0]):
        Ko, ro = O.elem_hyper(O.law_from_E_nu(law, Ev[e], nu), npts, xyz[el[e]], U[el[e]].ravel())
        d = (3 * el[e][:, None] + np.arange(3)).ravel()
        Kd[np.ix_(d, d)] += Ko
        rd[d] += ro
    rows = np.repeat(np.arange(n), np.diff(rp))
    assert rel(v, Kd[rows, ci]) < TOL_FP32
    assert rel(r, rd) < 1e-5
    K, re = a.element_matrices(u=u, first=4, count=3)
    for k in range(3):
        Ko, ro = O.elem_hyper(O.law_from_E_nu(law, Ev[4 + k], nu), npts, xyz[el[4 + k]], U[el[4 + k]].ravel())
        assert rel(K[k], Ko) < 2e-6 and rel(re[k], ro) < 1e-5
    a.set_element_moduli(None)
    (v1,), r1, _ = a.assemble(u=u)
    assert np.array_equal(v1, v0) and np.array_equal(r1, r0)
    bad = Ev.copy()
    bad[3] = -1.0
    with pytest.raises(F.FeddError) as ei:
        a.set_element_moduli(bad)
    assert ei.value.code == 1  # FEDD_ERR_ARG
    a.close()


def test_element_moduli_rejected_for_other_problems(F):
    xyz2, el2, xyz1, el1, u, p = ns_case(F, 1, 3)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0])
    with pytest.raises(F.FeddError) as ei:
        a.set_element_moduli(np.ones(el2.shape[0]))
    assert ei.value.code == 7  # FEDD_ERR_STATE
    a.close()


# -------------------------------------------------- source functions ----
def test_rhs_with_source_functions(F):
    """FE::assemblyRHS (FE_def.hpp:7303-7400) with a source function, Scalar
    on P1 (1-point rule) and Vector on P2 (5-point rule), against the oracle's
    restatement; a constant function gives the constant-source load."""
    fs = lambda x: np.sin(3.0 * x[..., 0]) + x[..., 1] * x[..., 2]
    fv = lambda x: np.stack([x[..., 0] ** 2, x[..., 1] * x[..., 2], 1.0 + x[..., 0]], axis=-1)
    for order, npts, fieldType, f, nc in ((1, 1, "Scalar", fs, 1), (2, 5, "Vector", fv, 3)):
        xyz, el = F.structured_mesh(3 if order == 1 else 2, order, seed=12)
        fe = F.FE((xyz, el))
        b = fe.assemblyRHS(3, "P%d" % order, fieldType, f)
        ob = O.assemble_rhs_func(order, npts, xyz, el, f, nc)
        assert b.shape == ob.shape and rel(b, ob) < TOL_FP64, fieldType
        a = F.Assembler(F.LAPLACE, xyz, el, fe_order=order)
        assert np.abs(a.rhs_points() - O.rhs_points(npts, xyz, el)).max() < 1e-14
        a.close()
    xyz, el = F.structured_mesh(2, 2, seed=13)
    fe = F.FE((xyz, el))
    b1 = fe.assemblyRHS(3, "P2", "Scalar", lambda x: np.full(x.shape[0], 2.5))
    b0 = fe.assemblyRHS(3, "P2", "Scalar", 2.5)
    assert rel(b1, b0) < 1e-13
