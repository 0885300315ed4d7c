"""GPU parity of the generalized-Newtonian Navier-Stokes assembly
(AssembleFEGeneralizedNewtonian: stress-divergence viscous term with a
shear-rate dependent viscosity and its Newton derivative, on top of the
Navier-Stokes advection and divergence terms) against the FP64 oracle, which
is pinned to the reference's own element code.  Blocks are compared as dense
matrices on small meshes, relative Frobenius error per block <= 1e-6."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-6

# FEDDLib's own example values (steadyGeneralizedNewtonian_PowerLaw/parametersProblem.xml)
# for Carreau-Yasuda and Dimless-Carreau; a shear-thinning power law
LAWS = [(0, [1.902, 0.22, 0.056, 0.00345, 1.25]),
        (1, [0.035, 0.61, 0.35, 1e-10, 0.0]),
        (2, [0.8, 0.45, 230.633, 3.3707, 0.0012])]


@pytest.fixture(scope="module")
def F():
    import feddlib_gb300 as F
    return F


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_blocks(xyz2, el2, el1, n1, u, p, L, dens, newton):
    n_u = 3 * xyz2.shape[0]
    J00 = np.zeros((n_u, n_u)); J01 = np.zeros((n_u, n1)); J10 = np.zeros((n1, n_u))
    ru = np.zeros(n_u); rp = np.zeros(n1)
    U = u.reshape(-1, 3)
    for e in range(el2.shape[0]):
        Je, re = O.elem_gn(xyz2[el2[e]], U[el2[e]].ravel(), p[el1[e]], L, dens, newton)
        vd = (3 * el2[e][:, None] + np.arange(3)).ravel()
        pd = el1[e]
        J00[np.ix_(vd, vd)] += Je[:30, :30]
        J01[np.ix_(vd, pd)] += Je[:30, 30:]
        J10[np.ix_(pd, vd)] += Je[30:, :30]
        np.add.at(ru, vd, re[:30]); np.add.at(rp, pd, re[30:])
    return (J00, J01, J10), ru, rp


def dense(a, b, vals):
    rp, ci, shape = a.pattern(b)
    M = np.zeros(shape)
    rows = np.repeat(np.arange(shape[0]), np.diff(rp))
    M[rows, ci] = vals
    return M


@pytest.mark.parametrize("law", range(3))
@pytest.mark.parametrize("newton", [True, False])
def test_generalized_newtonian_blocks(F, law, newton):
    model, prm = LAWS[law]
    xyz2, el2 = F.structured_mesh(2, 2, seed=6)
    xyz1, el1 = F.structured_mesh(2, 1, seed=6)
    u = F.fourier_field(xyz2, seed=6) * 0.5
    p = F.uniform_field(6, xyz1.shape[0])
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                    density=1.0, newton=newton)
    a.set_viscosity_law(model, prm, gamma_min=1e-12)
    vals, ru, rp = a.assemble(u=u, p=p)
    (o00, o01, o10), oru, orp = oracle_blocks(xyz2, el2, el1, xyz1.shape[0], u, p,
                                             O.visc_law(model, prm, 1e-12), 1.0, newton)
    for b, ob in enumerate((o00, o01, o10)):
        assert rel(dense(a, b, vals[b]), ob) < TOL, (b, rel(dense(a, b, vals[b]), ob))
    assert rel(ru, oru) < TOL and rel(rp, orp) < TOL


def test_generalized_newtonian_element_matrices(F):
    model, prm = LAWS[0]
    xyz2, el2 = F.structured_mesh(2, 2, seed=4)
    xyz1, el1 = F.structured_mesh(2, 1, seed=4)
    u = F.fourier_field(xyz2, seed=4)
    p = F.uniform_field(4, xyz1.shape[0])
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                    density=1.0, newton=True)
    a.set_viscosity_law(model, prm)
    K, r = a.element_matrices(u=u, p=p, first=0, count=12)
    L = O.visc_law(model, prm)
    for e in range(12):
        Jo, ro = O.elem_gn(xyz2[el2[e]], u.reshape(-1, 3)[el2[e]].ravel(), p[el1[e]], L, 1.0, True)
        assert rel(K[e], Jo) < 2e-6 and rel(r[e], ro) < 2e-6
    # back to the Newtonian fluid: the Navier-Stokes element again
    a.set_viscosity_law(-1)
    K2, _ = a.element_matrices(u=u, p=p, first=0, count=2)
    Jn, _ = O.elem_ns(xyz2[el2[0]], u.reshape(-1, 3)[el2[0]].ravel(), p[el1[0]], 0.01, 1.0, True)
    assert rel(K2[0], Jn) < 2e-6


def test_generalized_newtonian_rejected_by_noalloc_variant(F):
    import torch
    from feddlib_gb300 import _capi as A
    xyz2, el2 = F.structured_mesh(1, 2, seed=1)
    xyz1, el1 = F.structured_mesh(1, 1, seed=1)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0])
    a.set_viscosity_law(*LAWS[0])
    d_u = torch.zeros(a.n_u, dtype=torch.float64, device="cuda")
    K = np.zeros((1, 34, 34)); r = np.zeros((1, 34))
    st = A.lib().fedd_element_matrices_noalloc(a.h, d_u.data_ptr(), None, 0, 1, K.ctypes.data, r.ctypes.data, None)
    assert st == A.ERR_UNSUPPORTED


def test_generalized_newtonian_host_path_matches_device_path(F):
    """The host-buffer call overlaps its copies with the rows in node ranges
    (viscous rows added per range after the Navier-Stokes rows); the device
    call runs each stage once over all nodes.  Same values, bit for bit."""
    torch = pytest.importorskip("torch")
    model, prm = LAWS[0]
    xyz2, el2 = F.structured_mesh(3, 2, seed=5)
    xyz1, el1 = F.structured_mesh(3, 1, seed=5)
    u = F.fourier_field(xyz2, seed=5) * 0.5
    p = F.uniform_field(5, xyz1.shape[0])
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                    density=1.0, newton=True)
    a.set_viscosity_law(model, prm, gamma_min=1e-12)
    hv, hru, hrp = a.assemble(u=u, p=p)
    dev = torch.device("cuda:0")
    dv = [torch.empty(a.block_info(b)[2], dtype=torch.float64, device=dev) for b in range(3)]
    dru = torch.empty(a.n_u, dtype=torch.float64, device=dev)
    drp = torch.empty(a.n_p, dtype=torch.float64, device=dev)
    du, dp = torch.from_numpy(u).to(dev), torch.from_numpy(p).to(dev)  # kept alive across the call
    a.assemble_device(du.data_ptr(), dp.data_ptr(), [t.data_ptr() for t in dv], dru.data_ptr(), drp.data_ptr(),
                      stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for b in range(3):
        assert np.array_equal(dv[b].cpu().numpy(), hv[b])
    assert np.array_equal(dru.cpu().numpy(), hru) and np.array_equal(drp.cpu().numpy(), hrp)


# ---- the outflow Neumann boundary term ----------------------------------------
def _outflow_faces(el2, xyz2, plane=0, value=1.0, flip=False):
    """Boundary faces of the structured mesh on the plane x_plane = value, as
    vertex node triples in the element's own local order (reversed with flip),
    plus one face listed twice, so that its element takes the later copy."""
    faces = []
    fv = ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3))
    for e in range(el2.shape[0]):
        v = el2[e, :4]
        for f in fv:
            ids = [int(v[i]) for i in f]
            if all(abs(xyz2[i, plane] - value) < 1e-12 for i in ids):
                faces.append(ids[::-1] if flip else ids)
    faces.append(faces[0][::-1])  # the same face again, opposite normal: it wins for its element
    return np.array(faces, dtype=np.int32)


def _oracle_outflow_residual(xyz2, el2, u, faces, L):
    owner, taken = O.outflow_owners(el2, faces)
    U = u.reshape(-1, 3)
    ru = np.zeros(u.size)
    for e, k in taken.items():
        ue = U[el2[e]].ravel()
        K = O.gn_outflow(xyz2[el2[e]], xyz2[faces[k]], ue, L)
        vd = (3 * el2[e][:, None] + np.arange(3)).ravel()
        np.add.at(ru, vd, K @ ue)
    return ru


@pytest.mark.parametrize("law", range(3))
@pytest.mark.parametrize("newton", [True, False])
def test_outflow_neumann_term(F, law, newton):
    """The outflow term on the faces of the plane x = 1 (one face listed twice,
    its element taking the later copy): the residual gains K u on the flagged
    elements, the Jacobian blocks stay those without the term, as the
    reference's element returns them."""
    model, prm = LAWS[law]
    xyz2, el2 = F.structured_mesh(2, 2, seed=6)
    xyz1, el1 = F.structured_mesh(2, 1, seed=6)
    u = F.fourier_field(xyz2, seed=6) * 0.5
    p = F.uniform_field(6, xyz1.shape[0])
    faces = _outflow_faces(el2, xyz2, flip=(law == 1))
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                    density=1.0, newton=newton)
    a.set_viscosity_law(model, prm, gamma_min=1e-12)
    a.set_outflow_faces(faces)
    vals, ru, rp = a.assemble(u=u, p=p)
    L = O.visc_law(model, prm, 1e-12)
    (o00, o01, o10), oru, orp = oracle_blocks(xyz2, el2, el1, xyz1.shape[0], u, p, L, 1.0, newton)
    term = _oracle_outflow_residual(xyz2, el2, u, faces, L)
    assert np.linalg.norm(term) > 1e-3 * np.linalg.norm(oru)
    for b, ob in enumerate((o00, o01, o10)):
        assert rel(dense(a, b, vals[b]), ob) < TOL, (b, rel(dense(a, b, vals[b]), ob))
    assert rel(ru, oru + term) < TOL, rel(ru, oru + term)
    assert rel(rp, orp) < TOL
    # cleared: the residual without the term again
    a.set_outflow_faces([])
    _, ru0, _ = a.assemble(u=u, p=p)
    assert rel(ru0, oru) < TOL


def test_outflow_term_in_element_vectors_and_host_path(F):
    """The element vectors of the flagged elements carry the term, their
    matrices do not; the host-buffer path with its chunked element stage
    equals the device path bit for bit."""
    import torch
    model, prm = LAWS[0]
    xyz2, el2 = F.structured_mesh(3, 2, seed=2)
    xyz1, el1 = F.structured_mesh(3, 1, seed=2)
    u = F.fourier_field(xyz2, seed=2) * 0.5
    p = F.uniform_field(2, xyz1.shape[0])
    faces = _outflow_faces(el2, xyz2, plane=2, value=0.0)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                    density=1.0, newton=True)
    a.set_viscosity_law(model, prm)
    a.set_outflow_faces(faces)
    L = O.visc_law(model, prm)
    _, taken = O.outflow_owners(el2, faces)
    els = sorted(taken)[:6]
    for e in els:
        K, r = a.element_matrices(u=u, p=p, first=e, count=1)
        ue = u.reshape(-1, 3)[el2[e]].ravel()
        Jo, ro = O.elem_gn(xyz2[el2[e]], ue, p[el1[e]], L, 1.0, True)
        ro = ro.copy()
        ro[:30] += O.gn_outflow(xyz2[el2[e]], xyz2[faces[taken[e]]], ue, L) @ ue
        assert rel(K[0], Jo) < 2e-6 and rel(r[0], ro) < 2e-6, e
    hv, hru, hrp = a.assemble(u=u, p=p)
    dev = torch.device("cuda:0")
    dv = [torch.empty(a.block_info(b)[2], dtype=torch.float64, device=dev) for b in range(3)]
    dru = torch.empty(a.n_u, dtype=torch.float64, device=dev)
    drp = torch.empty(a.n_p, dtype=torch.float64, device=dev)
    du = torch.from_numpy(u).to(dev)  # kept alive: the call reads them on the stream
    dp = torch.from_numpy(p).to(dev)
    a.assemble_device(du.data_ptr(), dp.data_ptr(), [t.data_ptr() for t in dv], dru.data_ptr(), drp.data_ptr(),
                      stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for b in range(3):
        assert np.array_equal(dv[b].cpu().numpy(), hv[b])
    assert np.array_equal(dru.cpu().numpy(), hru) and np.array_equal(drp.cpu().numpy(), hrp)


def test_outflow_faces_rejected(F):
    from feddlib_gb300 import _capi as A
    xyz2, el2 = F.structured_mesh(2, 2, seed=1)
    xyz1, el1 = F.structured_mesh(2, 1, seed=1)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0])
    v = el2[0, :4]
    for bad in ([[int(v[0]), int(v[1]), 10 ** 6]], [[0, 1, 2]]):
        f = np.ascontiguousarray(np.asarray(bad, dtype=np.int32))
        assert A.lib().fedd_set_outflow_faces(a.h, f.ctypes.data, 1) == A.ERR_ARG
    # an interior face (shared by two elements)
    count = {}
    for e in range(el2.shape[0]):
        w = el2[e, :4]
        for f in ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)):
            count.setdefault(tuple(sorted(int(w[i]) for i in f)), []).append(e)
    inner = next(k for k, es in count.items() if len(es) == 2)
    f = np.ascontiguousarray(np.asarray([inner], dtype=np.int32))
    assert A.lib().fedd_set_outflow_faces(a.h, f.ctypes.data, 1) == A.ERR_ARG


@pytest.mark.parametrize("law", range(3))
def test_outflow_term_in_the_fixed_point_matrix(F, law):
    """FE::assemblyNavierStokes' "FixedPoint" mode (linearization 2) takes the
    element's fixed-point matrix, which holds the outflow term: block (0,0)
    gains K on the flagged elements, the residual is the same as in the other
    modes; the element matrices carry it too."""
    model, prm = LAWS[law]
    xyz2, el2 = F.structured_mesh(2, 2, seed=5)
    xyz1, el1 = F.structured_mesh(2, 1, seed=5)
    u = F.fourier_field(xyz2, seed=5) * 0.5
    p = F.uniform_field(5, xyz1.shape[0])
    faces = _outflow_faces(el2, xyz2, plane=1, value=1.0)
    a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                    density=1.0, newton=False, fixed_point_matrix=True)
    a.set_viscosity_law(model, prm, gamma_min=1e-12)
    a.set_outflow_faces(faces)
    vals, ru, rp = a.assemble(u=u, p=p)
    L = O.visc_law(model, prm, 1e-12)
    (o00, o01, o10), oru, orp = oracle_blocks(xyz2, el2, el1, xyz1.shape[0], u, p, L, 1.0, False)
    _, taken = O.outflow_owners(el2, faces)
    U = u.reshape(-1, 3)
    o00 = o00.copy()
    for e, k in taken.items():
        K = O.gn_outflow(xyz2[el2[e]], xyz2[faces[k]], U[el2[e]].ravel(), L)
        vd = (3 * el2[e][:, None] + np.arange(3)).ravel()
        o00[np.ix_(vd, vd)] += K
    term = _oracle_outflow_residual(xyz2, el2, u, faces, L)
    for b, ob in enumerate((o00, o01, o10)):
        assert rel(dense(a, b, vals[b]), ob) < TOL, (b, rel(dense(a, b, vals[b]), ob))
    assert rel(ru, oru + term) < TOL and rel(rp, orp) < TOL
    e = sorted(taken)[0]
    Ke, _ = a.element_matrices(u=u, p=p, first=e, count=1)
    Jo, _ = O.elem_gn(xyz2[el2[e]], U[el2[e]].ravel(), p[el1[e]], L, 1.0, False)
    Jo = Jo.copy()
    Jo[:30, :30] += O.gn_outflow(xyz2[el2[e]], xyz2[faces[taken[e]]], U[el2[e]].ravel(), L)
    assert rel(Ke[0], Jo) < 2e-6


def test_linearization_out_of_range_rejected(F):
    import ctypes as C
    from feddlib_gb300 import _capi as A
    xyz2, el2 = F.structured_mesh(1, 2, seed=1)
    xyz1, el1 = F.structured_mesh(1, 1, seed=1)
    x = np.ascontiguousarray(xyz2)
    c = np.ascontiguousarray(el2, dtype=np.int32)
    c1 = np.ascontiguousarray(el1, dtype=np.int32)
    m = A.Mesh()
    m.num_nodes, m.num_elements, m.fe_order = xyz2.shape[0], el2.shape[0], 2
    m.coords, m.elements = x.ctypes.data, c.ctypes.data
    m.num_nodes_p, m.elements_p = xyz1.shape[0], c1.ctypes.data
    p = A.Params()
    p.problem = F.NAVIER_STOKES
    p.linearization = 3
    h = C.c_void_p()
    assert A.lib().fedd_create(C.byref(m), C.byref(p), 0, C.byref(h)) == A.ERR_ARG
