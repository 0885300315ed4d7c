"""CPU tests of the FP64 oracle: pinned against FEDDLib's own element code
(golden fixtures made by tests/golden/make_golden.py), the cross-path
identities the reference's assembly tests print (asserted here), and
known-answer tests."""
import math
import os

import numpy as np
import pytest

from oracle import oracle as O


def test_quadrature_matches_reference(golden):
    for deg in (1, 2, 3, 4, 5):
        n = O.lib().orc_quad_points_for_degree(deg)
        pts, w = O.quad(n)
        np.testing.assert_array_equal(pts, golden[f"quad_deg{deg}_pts"])
        np.testing.assert_array_equal(w, golden[f"quad_deg{deg}_w"])


def test_basis_matches_reference(golden):
    for fe, order in (("P1", 1), ("P2", 2)):
        for deg in (1, 3, 5):
            pts, _ = O.quad(O.lib().orc_quad_points_for_degree(deg))
            D = np.array([O.dphi(order, x) for x in pts])
            P = np.array([O.phi(order, x) for x in pts])
            np.testing.assert_allclose(D, golden[f"dphi_{fe}_deg{deg}"], rtol=0, atol=1e-15)
            np.testing.assert_allclose(P, golden[f"phi_{fe}_deg{deg}"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("newton", [True, False])
def test_ns_element_matches_reference(golden, newton):
    key = "ns_J_newton" if newton else "ns_J_fixedpoint"
    for k in range(golden["ns_x"].shape[0]):
        sol = golden["ns_sol"][k]
        J, r = O.elem_ns(golden["ns_x"][k], sol[:30], sol[30:], float(golden["ns_visc"]),
                         float(golden["ns_dens"]), newton)
        Jr = golden[key][k]
        assert np.abs(J - Jr).max() <= 1e-14 * np.abs(Jr).max()
        assert np.abs(r - golden["ns_res"][k]).max() <= 1e-14 * np.abs(golden["ns_res"][k]).max()


def test_laplace_element_matches_reference(golden):
    for fe, order, npts in (("P1", 1, 5), ("P2", 2, 15)):
        for k in range(golden[f"lap_{fe}_x"].shape[0]):
            K = O.elem_laplace(order, npts, golden[f"lap_{fe}_x"][k])
            Kr = golden[f"lap_{fe}_K"][k]
            assert np.abs(K - Kr).max() <= 1e-14 * np.abs(Kr).max()
            b = np.zeros(K.shape[0])
            O.lib().orc_elem_rhs_const(order, npts, O.p(np.ascontiguousarray(golden[f"lap_{fe}_x"][k])),
                                       O.C.c_double(1.0), O.p(b))
            np.testing.assert_allclose(b, golden[f"lap_{fe}_b"][k], rtol=1e-13, atol=1e-18)


def test_reference_live_if_built():
    """When oracle/_ref was compiled here, check a fresh random case too."""
    path = os.path.join(os.path.dirname(O.__file__), "_ref", "libfeddref.so")
    if not os.path.exists(path):
        pytest.skip("oracle/_ref not built (reference tree absent)")
    import ctypes as C
    R = C.CDLL(path)
    xyz, conn, _ = O.mesh(3, 2, seed=11)
    rng = np.random.default_rng(5)
    for e in rng.integers(0, conn.shape[0], 6):
        xe = np.ascontiguousarray(xyz[conn[e]])
        sol = rng.uniform(-2, 2, 34)
        J = np.zeros(34 * 34); r = np.zeros(34)
        assert R.ref_ns_element(O.p(xe), O.p(sol), C.c_double(0.03), C.c_double(1.7), 1, O.p(J), O.p(r)) == 0
        Jo, ro = O.elem_ns(xe, sol[:30], sol[30:], 0.03, 1.7, True)
        assert np.abs(J.reshape(34, 34) - Jo).max() <= 1e-13 * np.abs(Jo).max()
        assert np.abs(r - ro).max() <= 1e-13 * np.abs(ro).max()


# ---- known-answer tests ------------------------------------------------------
def _monomials(deg):
    for a in range(deg + 1):
        for b in range(deg + 1 - a):
            for c in range(deg + 1 - a - b):
                yield a, b, c


@pytest.mark.parametrize("npts,deg", [(1, 1), (4, 2), (5, 3), (15, 5)])
def test_quadrature_exactness(npts, deg):
    pts, w = O.quad(npts)
    assert abs(w.sum() - 1 / 6) < 1e-15
    for a, b, c in _monomials(deg):
        exact = math.factorial(a) * math.factorial(b) * math.factorial(c) / math.factorial(a + b + c + 3)
        got = np.sum(w * pts[:, 0] ** a * pts[:, 1] ** b * pts[:, 2] ** c)
        assert abs(got - exact) < 1e-14, (a, b, c)


def test_mesh_numbering_and_orientation():
    M = 3
    xyz, conn, nflip = O.mesh(M, 2, amp=0, orient=False)
    E = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]
    for k, (a, b) in enumerate(E):
        np.testing.assert_allclose(xyz[conn[:, 4 + k]], 0.5 * (xyz[conn[:, a]] + xyz[conn[:, b]]), atol=1e-15)
    xyz, conn, nflip = O.mesh(M, 2, seed=7)
    assert nflip == 4 * M ** 3  # 4 of the 6 tets per hex are flipped
    for e in range(conn.shape[0]):
        det, _, _ = O.geometry(xyz[conn[e, :4]])
        assert det > 0
    # P1 mesh of the same seed shares the vertices and element order
    xyz1, conn1, _ = O.mesh(M, 1, seed=7)
    P = 2 * M + 1
    idx = np.array([2 * r + P * 2 * s + P * P * 2 * t for t in range(M + 1) for s in range(M + 1) for r in range(M + 1)])
    np.testing.assert_array_equal(xyz[idx], xyz1)
    inv = {v: i for i, v in enumerate(idx)}
    assert all(inv[a] == b for a, b in zip(conn[:, :4].ravel(), conn1.ravel()))


@pytest.mark.parametrize("M", [2, 3, 4])
def test_pattern_sizes(M):
    xyz1, conn1, _ = O.mesh(M, 1, seed=1)
    rp, ci, _ = O.assemble_laplace(1, 1, xyz1, conn1)
    assert rp[-1] == 15 * M ** 3 + 21 * M ** 2 + 9 * M + 1
    xyz2, conn2, _ = O.mesh(M, 2, seed=1)
    L = O.law_from_E_nu(O.LAW_SKR1, 1000, 0.3)
    (rp2, ci2, _), _ = O.assemble_vec(0, L, 5, xyz2, conn2)
    assert rp2[-1] == 9 * (230 * M ** 3 + 138 * M ** 2 + 24 * M + 1)
    blocks, _ = O.assemble_ns(xyz2, conn2, conn1, xyz1.shape[0], np.zeros(3 * xyz2.shape[0]),
                              np.zeros(xyz1.shape[0]), 0.01, 1.0, True)
    assert blocks[1][0][-1] == 195 * M ** 3 + 171 * M ** 2 + 45 * M + 3
    assert blocks[2][0][-1] == blocks[1][0][-1]
    assert blocks[3][0][-1] == 0  # (1,1) empty after the 1e-13 filter


def test_laplace_kats():
    xyz, conn, _ = O.mesh(3, 2, seed=4)
    for e in (0, 33, 100):
        xe = xyz[conn[e]]
        K = O.elem_laplace(2, 15, xe)
        assert np.abs(K.sum(axis=1)).max() < 1e-14 * np.abs(K).max()
        assert np.abs(K - K.T).max() == 0
        det, _, _ = O.geometry(xe[:4])
        b = np.zeros(10)
        O.lib().orc_elem_rhs_const(2, 15, O.p(np.ascontiguousarray(xe)), O.C.c_double(1.0), O.p(b))
        np.testing.assert_allclose(b[:4], -det / 6 / 20, rtol=1e-12)
        np.testing.assert_allclose(b[4:], det / 6 / 5, rtol=1e-12)
    xyz1, conn1, _ = O.mesh(3, 1, seed=4)
    b1 = O.assemble_rhs(1, 1, xyz1, conn1, 1.0)
    assert abs(b1.sum() - 1.0) < 1e-13  # volume of the unit cube


def test_classic_linelas_equals_skr1_at_zero():
    """fe_test_linElas.cpp:120-136 prints the difference between the classic
    linear-elasticity assembly and skr1 at d = 0; assert it vanishes."""
    xyz, conn, _ = O.mesh(2, 2, seed=2)
    L = O.law_from_E_nu(O.LAW_SKR1, 1000, 0.3)
    (rc, cc, vc), _ = O.assemble_vec(0, L, 5, xyz, conn)
    (rs, cs, vs), res = O.assemble_vec(1, L, 4, xyz, conn, None)
    np.testing.assert_array_equal(rc, rs)
    np.testing.assert_array_equal(cc, cs)
    assert np.abs(vc - vs).max() < 1e-12 * np.abs(vc).max()
    assert np.abs(res).max() == 0


def test_rigid_body_modes_in_null_space():
    xyz, conn, _ = O.mesh(2, 2, seed=2)
    L = O.law_from_E_nu(O.LAW_SKR1, 1000, 0.3)
    xe = xyz[conn[3]]
    K, _ = O.elem_hyper(L, 4, xe, None)
    modes = []
    for d in range(3):
        v = np.zeros(30); v[d::3] = 1; modes.append(v)
    for axis in np.eye(3):
        modes.append(np.cross(axis, xe).ravel())
    for v in modes:
        assert np.abs(K @ v).max() < 1e-10 * np.abs(K).max()


def test_classic_linelas_equals_skr3_at_zero():
    """skr3's split law (mu, kappa) linearises at d = 0 to the classic
    linear-elastic element with Lame lambda = E nu / ((1 + nu)(1 - 2 nu)),
    the pin fe_test_linElas.cpp:120-136 makes for skr1."""
    xyz, conn, _ = O.mesh(2, 2, seed=2)
    E, nu = 1000.0, 0.3
    Lc = O.law_from_E_nu(O.LAW_SKR1, E, nu)      # classic element's (mu, lambda)
    L3 = O.law_from_E_nu(O.LAW_SKR3, E, nu)      # (mu, kappa)
    assert abs(L3.s.lam - (Lc.s.lam + 2.0 / 3.0 * Lc.s.mu)) < 1e-9 * L3.s.lam
    (rc, cc, vc), _ = O.assemble_vec(0, Lc, 5, xyz, conn)
    (rs, cs, vs), res = O.assemble_vec(1, L3, 5, xyz, conn, None)
    np.testing.assert_array_equal(rc, rs)
    np.testing.assert_array_equal(cc, cs)
    assert np.abs(vc - vs).max() < 1e-12 * np.abs(vc).max()
    assert np.abs(res).max() < 1e-12 * np.abs(vc).max()


def test_skr3_law_derivatives():
    """Psi = mu/2 (J^-2/3 I1 - 3) + kappa/2 (J - 1)^2 (NeoHookQuadraticTets3.f:
    25-31, 491-496): first and second derivatives against central differences,
    and dPsi/dI3 (I3 = J^2) against the AceGen intermediate v(208)/E."""
    L = O.LawSpec(O.LAW_SKR3, mu=1.3, lam=7.0)
    inv = np.array([3.4, 1.12, 1.0, 1.0])
    psi, d1, d2 = O.law_dpsi(L, inv)
    mu, kap = 1.3, 7.0
    I1, J = inv[0], inv[1]
    assert abs(psi - (0.5 * mu * (J ** (-2 / 3) * I1 - 3) + 0.5 * kap * (J - 1) ** 2)) < 1e-14
    h = 1e-6
    for k in (0, 1):
        e = np.zeros(4); e[k] = h
        assert abs(d1[k] - (O.law_dpsi(L, inv + e)[0] - O.law_dpsi(L, inv - e)[0]) / (2 * h)) < 1e-8
        for l in (0, 1):
            assert abs(d2[k, l] - (O.law_dpsi(L, inv + e)[1][l] - O.law_dpsi(L, inv - e)[1][l]) / (2 * h)) < 1e-7
    # AceGen: dPsi/dI3 = -mu I1 / (6 I3^(4/3)) + kappa (J - 1) / (2 J)
    dI3 = d1[1] / (2 * J)
    assert abs(dI3 - (-mu * I1 / (6 * (J * J) ** (4 / 3)) + kap * (J - 1) / (2 * J))) < 1e-13


@pytest.mark.parametrize("law,npts", [(O.LAW_SKR1, 4), (O.LAW_SKR2, 5), (O.LAW_ANISO, 4), (O.LAW_SKR3, 5)])
def test_hyperelastic_tangent_is_residual_derivative(law, npts):
    xyz, conn, _ = O.mesh(2, 2, seed=5)
    xe = xyz[conn[7]]
    rng = np.random.default_rng(3)
    u = 0.03 * rng.standard_normal(30)
    L = O.LawSpec(law, mu=1.0, lam=10.0)
    K, r = O.elem_hyper(L, npts, xe, u)
    eps = 1e-6
    Kfd = np.zeros((30, 30))
    for j in range(30):
        up = u.copy(); up[j] += eps; um = u.copy(); um[j] -= eps
        Kfd[:, j] = -(O.elem_hyper(L, npts, xe, up)[1] - O.elem_hyper(L, npts, xe, um)[1]) / (2 * eps)
    assert np.abs(K - Kfd).max() < 1e-7 * np.abs(K).max()
    assert np.abs(K - K.T).max() < 1e-13 * np.abs(K).max()


def test_skr1_stress_formula():
    """P = mu F + (lambda J/2 - (lambda+2mu)/(2J)) cof F (NeoHookQuadraticTets.f:481-483)."""
    L = O.LawSpec(O.LAW_SKR1, mu=1.3, lam=7.0)
    rng = np.random.default_rng(0)
    F = np.eye(3) + 0.2 * rng.standard_normal((3, 3))
    J = np.linalg.det(F)
    cof = J * np.linalg.inv(F).T
    _, P, _ = O.law_PA(L, F)
    np.testing.assert_allclose(P, 1.3 * F + (7.0 * J / 2 - (7.0 + 2.6) / (2 * J)) * cof, rtol=1e-13)
    L2 = O.LawSpec(O.LAW_SKR2, mu=1.3, lam=7.0)
    _, P2, _ = O.law_PA(L2, F)
    S = 1.3 * np.eye(3) + (7.0 * np.log(J) - 1.3) * np.linalg.inv(F.T @ F)
    np.testing.assert_allclose(P2, F @ S, rtol=1e-12)


def test_ns_newton_term_is_derivative_of_advection():
    xyz, conn, _ = O.mesh(2, 2, seed=3)
    xe = xyz[conn[9]]
    rng = np.random.default_rng(7)
    u = rng.standard_normal(30); pr = rng.standard_normal(4)
    J, r, A, N, W, B = O.elem_ns(xe, u, pr, 0.01, 1.0, True, parts=True)

    def Nu(v):
        return O.elem_ns(xe, v, pr, 0.01, 1.0, True, parts=True)[3][:30, :30] @ v
    eps = 1e-6
    fd = np.zeros((30, 30))
    for j in range(30):
        up = u.copy(); up[j] += eps; um = u.copy(); um[j] -= eps
        fd[:, j] = (Nu(up) - Nu(um)) / (2 * eps)
    assert np.abs(N[:30, :30] + W[:30, :30] - fd).max() < 1e-8 * np.abs(fd).max()


def test_ns_constant_velocity_identity():
    """fe_test_navierstokes.cpp:119-263 compares the classic A+N+W and B with the
    AssembleFE element at u = 100, p = 0: with a constant field W vanishes and
    N equals the advection matrix of the constant field."""
    xyz, conn, _ = O.mesh(2, 2, seed=3)
    xe = xyz[conn[2]]
    u = np.full(30, 100.0)
    J, r, A, N, W, B = O.elem_ns(xe, u, np.zeros(4), 1.0, 1.0, True, parts=True)
    assert np.abs(W).max() < 1e-10 * np.abs(N).max()
    np.testing.assert_allclose(J, A - B + N + W, rtol=0, atol=1e-12 * np.abs(J).max())


def test_coo_to_csr_tpetra_semantics():
    rows = np.array([1, 0, 1, 1, 0], dtype=np.int64)
    cols = np.array([2, 0, 0, 2, 0], dtype=np.int64)
    vals = np.array([1.0, 2.0, 0.0, 3.0, 4.0])
    rp, ci, v = O.coo_to_csr(3, rows, cols, vals)
    np.testing.assert_array_equal(rp, [0, 1, 3, 3])
    np.testing.assert_array_equal(ci, [0, 0, 2])
    np.testing.assert_array_equal(v, [6.0, 0.0, 4.0])  # explicit zero kept


def test_mlp_gradients_match_finite_differences():
    rng = np.random.default_rng(1)
    H = 8
    m = {"W1": rng.standard_normal((H, 4)) * 0.5, "b1": rng.standard_normal(H) * 0.1,
         "W2": rng.standard_normal((H, H)) * 0.3, "b2": rng.standard_normal(H) * 0.1,
         "w3": rng.standard_normal(H) * 0.3, "b3": 0.2}
    x = rng.standard_normal(4) * 0.5
    y, g, h = O.mlp_eval(m, x)
    eps = 1e-5
    for k in range(4):
        xp = x.copy(); xp[k] += eps; xm = x.copy(); xm[k] -= eps
        yp, gp, _ = O.mlp_eval(m, xp); ym, gm, _ = O.mlp_eval(m, xm)
        assert abs((yp - ym) / (2 * eps) - g[k]) < 1e-8
        np.testing.assert_allclose((gp - gm) / (2 * eps), h[k], atol=1e-7)
    X = rng.standard_normal((5, 4)) * 0.5
    tp = rng.standard_normal(5); tg = rng.standard_normal((5, 4))
    loss, grads = O.mlp_loss(m, X, tp, tg, 1.0, 0.5)
    for name in ("W1", "b1", "W2", "b2", "w3"):
        arr = np.asarray(m[name], dtype=np.float64)
        flat = arr.ravel()
        for idx in rng.choice(flat.size, min(6, flat.size), replace=False):
            old = flat[idx]
            flat[idx] = old + eps; m[name] = flat.reshape(arr.shape)
            lp = O.mlp_loss(m, X, tp, tg, 1.0, 0.5, grads=False)
            flat[idx] = old - eps; m[name] = flat.reshape(arr.shape)
            lm = O.mlp_loss(m, X, tp, tg, 1.0, 0.5, grads=False)
            flat[idx] = old; m[name] = flat.reshape(arr.shape)
            assert abs((lp - lm) / (2 * eps) - grads[name].ravel()[idx]) < 1e-6 * max(1, abs(grads[name].ravel()[idx]))


def test_dirichlet_restatement_known_answers():
    """BCBuilder's row replacement on a hand-made CSR: identity rows in the
    diagonal block, zero rows off it, a row without a diagonal entry zeroed."""
    # 3x3 block, row 2 has no diagonal entry
    rp = np.array([0, 2, 4, 5])
    ci = np.array([0, 1, 0, 1, 0])
    v = np.array([4.0, -1.0, -1.0, 4.0, 2.5])
    mask = np.array([1, 0, 1], dtype=np.uint8)
    np.testing.assert_array_equal(O.dirichlet_rows(rp, ci, v, mask, True), [1.0, 0.0, -1.0, 4.0, 0.0])
    np.testing.assert_array_equal(O.dirichlet_rows(rp, ci, v, mask, False), [0.0, 0.0, -1.0, 4.0, 0.0])
    res = np.array([1.0, 2.0, 3.0])
    np.testing.assert_array_equal(O.dirichlet_rhs(res, mask, g=[7.0, 8.0, 9.0]), [7.0, 2.0, 9.0])
    np.testing.assert_array_equal(O.dirichlet_rhs(res, mask, g=[7.0, 8.0, 9.0], sub=[1.0, 1.0, 2.0]),
                                  [6.0, 2.0, 7.0])
    np.testing.assert_array_equal(O.dirichlet_rhs(res, mask), [0.0, 2.0, 0.0])


def test_generalized_newtonian_element_matches_reference(golden):
    """AssembleFEGeneralizedNewtonian (three viscosity laws, Newton and
    FixedPoint) from the reference's own code, against the restatement."""
    for k in range(len(golden["gn_x"])):
        m = golden["gn_model"][k]
        L = O.visc_law(int(m[0]), m[1:6])
        x, sol = golden["gn_x"][k], golden["gn_sol"][k]
        for newton, key in ((True, "gn_J_newton"), (False, "gn_J_fixedpoint")):
            J, r = O.elem_gn(x, sol[:30], sol[30:], L, 1.0, newton)
            ref = golden[key][k]
            assert np.abs(J - ref).max() <= 1e-13 * np.abs(ref).max(), (k, newton)
            assert np.abs(r - golden["gn_res"][k]).max() <= 1e-13 * np.abs(golden["gn_res"][k]).max()


def test_generalized_newtonian_live_if_built():
    """Fresh cases against the reference library when it was compiled here,
    including shear rates below 1, where the reference's integer abs floors
    them, and a Carreau-Yasuda exponent a in (1, 3)."""
    path = os.path.join(os.path.dirname(O.__file__), "_ref", "libfeddref.so")
    if not os.path.exists(path):
        pytest.skip("oracle/_ref not built (reference tree absent)")
    import ctypes as C
    R = C.CDLL(path)
    xyz, conn, _ = O.mesh(2, 2, seed=5)
    rng = np.random.default_rng(9)
    cases = [(0, [1.902, 0.22, 0.056, 0.00345, 1.25]), (0, [0.5, 0.6, 0.05, 0.005, 3.5]),
             (1, [0.035, 0.61, 0.35, 1e-10, 0.0]), (2, [0.8, 0.45, 230.6, 3.37, 0.0012])]
    for model, prm in cases:
        for amp in (0.6, 0.03):
            e = int(rng.integers(0, conn.shape[0]))
            xe = np.ascontiguousarray(xyz[conn[e]])
            sol = np.concatenate([rng.uniform(-amp, amp, 30), rng.uniform(-1, 1, 4)])
            mp = np.array(prm, dtype=np.float64)
            J = np.zeros(34 * 34); r = np.zeros(34)
            assert R.ref_gn_element(O.p(xe), O.p(sol), model, O.p(mp), C.c_double(1.3), 1, O.p(J), O.p(r)) == 0
            Jo, ro = O.elem_gn(xe, sol[:30], sol[30:], O.visc_law(model, prm), 1.3, True)
            assert np.abs(J.reshape(34, 34) - Jo).max() <= 1e-12 * np.abs(Jo).max(), (model, amp)
            assert np.abs(r - ro).max() <= 1e-12 * np.abs(ro).max()


def test_gn_outflow_term_matches_reference():
    """The generalized-Newtonian element flagged for the outflow Neumann term
    on one face (AssembleFEGeneralizedNewtonian::
    assemblyOutflowNeumannBoundaryTerm, with the surface data FEDDLib's Domain
    attaches), from the reference's own code: the term enters the element
    residual as K u, while the Jacobian the element returns is the one without
    it (assembleJacobian forms the Jacobian from its fixed-point matrix before
    it adds the boundary term to that matrix)."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_gn_outflow.npz"))
    for k in range(len(g["x"])):
        m = g["model"][k]
        L = O.visc_law(int(m[0]), m[1:6])
        x, face, sol = g["x"][k], g["face"][k], g["sol"][k]
        K = O.gn_outflow(x, face, sol[:30], L)
        assert np.abs(K).max() > 0
        for newton, key in ((True, "J_newton"), (False, "J_fixedpoint")):
            J, r = O.elem_gn(x, sol[:30], sol[30:], L, 1.0, newton)
            assert np.abs(J - g[key][k]).max() <= 1e-13 * np.abs(g[key][k]).max(), (k, newton)
        r = r.copy()
        r[:30] += K @ sol[:30]
        assert np.abs(r - g["res"][k]).max() <= 1e-13 * np.abs(g["res"][k]).max(), k
        # FE::assemblyNavierStokes' "FixedPoint" mode takes assembleFixedPoint's
        # matrix, which holds the term: the FixedPoint Jacobian plus K
        Jp, _ = O.elem_gn(x, sol[:30], sol[30:], L, 1.0, False)
        Jp = Jp.copy()
        Jp[:30, :30] += K
        ref = g["J_fixed_point_matrix"][k]
        assert np.abs(Jp - ref).max() <= 1e-13 * np.abs(ref).max(), k


def test_gn_outflow_live_if_built():
    """Fresh elements, faces in every node order and all three laws against the
    reference library when it was compiled here."""
    path = os.path.join(os.path.dirname(O.__file__), "_ref", "libfeddref.so")
    if not os.path.exists(path):
        pytest.skip("oracle/_ref not built (reference tree absent)")
    import ctypes as C
    R = C.CDLL(path)
    xyz, conn, _ = O.mesh(2, 2, seed=8)
    rng = np.random.default_rng(21)
    cases = [(0, [1.902, 0.22, 0.056, 0.00345, 1.25]), (1, [0.035, 0.61, 0.35, 1e-10, 0.0]),
             (2, [0.8, 0.45, 230.6, 3.37, 0.0012])]
    orders = [(0, 1, 2), (2, 1, 0), (1, 3, 2), (3, 0, 2), (0, 3, 1), (2, 3, 1)]
    for model, prm in cases:
        for fo in orders:
            e = int(rng.integers(0, conn.shape[0]))
            xe = np.ascontiguousarray(xyz[conn[e]])
            face = np.ascontiguousarray(xe[list(fo)])
            sol = np.concatenate([rng.uniform(-0.6, 0.6, 30), rng.uniform(-1, 1, 4)])
            mp = np.array(prm, dtype=np.float64)
            J = np.zeros(34 * 34); r = np.zeros(34)
            assert R.ref_gn_element_outflow(O.p(xe), O.p(face), O.p(sol), model, O.p(mp), C.c_double(1.3), 1,
                                            O.p(J), O.p(r)) == 0
            L = O.visc_law(model, prm)
            Jo, ro = O.elem_gn(xe, sol[:30], sol[30:], L, 1.3, True)
            ro[:30] += O.gn_outflow(xe, face, sol[:30], L) @ sol[:30]
            assert np.abs(J.reshape(34, 34) - Jo).max() <= 1e-12 * np.abs(Jo).max(), (model, fo)
            assert np.abs(r - ro).max() <= 1e-12 * np.abs(ro).max(), (model, fo)


def test_outflow_owner_rule():
    """Each face belongs to exactly one element; an element with two listed
    faces takes the last one; a face of no element or an interior face (two
    elements) is rejected."""
    xyz, conn, _ = O.mesh(2, 2, seed=1)
    count = {}
    for e in range(conn.shape[0]):
        v = conn[e, :4]
        for f in ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)):
            count.setdefault(tuple(sorted(int(v[i]) for i in f)), []).append((e, f))
    boundary = {k: v[0] for k, v in count.items() if len(v) == 1}
    interior = [k for k, v in count.items() if len(v) == 2]
    per_elem = {}
    for k, (e, f) in boundary.items():
        per_elem.setdefault(e, []).append(k)
    e2 = next(e for e, fs in per_elem.items() if len(fs) >= 2)
    fa, fb = per_elem[e2][:2]
    owner, taken = O.outflow_owners(conn, [fa[::-1], fb])
    assert owner.tolist() == [e2, e2] and taken == {e2: 1}
    with pytest.raises(ValueError):
        O.outflow_owners(conn, [interior[0]])
    with pytest.raises(ValueError):
        O.outflow_owners(conn, [(0, 1, 10 ** 6)])


def test_viscosity_laws_and_their_derivative_term():
    """eta and -(2/gamma) deta/dgamma against finite differences where the
    reference takes the smooth branch (Power-Law above shear rate 1, the
    Dimless-Carreau law everywhere)."""
    for model, prm in ((1, [0.035, 0.61, 100.0, 1e-10]), (2, [0.8, 0.45, 230.6, 3.37, 0.0012])):
        L = O.visc_law(model, prm)
        for g in (1.5, 4.0, 20.0):
            h = 1e-6 * g
            deta = (O.gn_eta(L, g + h) - O.gn_eta(L, g - h)) / (2 * h)
            assert abs(O.gn_dterm(L, g) - (-2.0 / g) * deta) <= 1e-6 * abs(O.gn_dterm(L, g))


def test_gn_row_checker_matches_dense_assembly():
    """The full-size row checker with a viscosity law (the generalized-Newtonian
    element) reproduces a dense assembly of the same element exactly."""
    from oracle import parity as P
    xyz2, el2, _ = O.mesh(2, 2, seed=6)
    xyz1, el1, _ = O.mesh(2, 1, seed=6)
    nn, n1 = xyz2.shape[0], xyz1.shape[0]
    u = O.field_fourier(xyz2, 6) * 0.5
    p = O.field_uniform(6, n1)
    L = O.visc_law(0, [1.902, 0.22, 0.056, 0.00345, 1.25], 1e-12)
    vsel, psel = np.arange(0, nn, 7), np.arange(0, n1, 5)
    o = P.rows_ns(xyz2, el2, el1, u, p, 0.0, 1.0, True, P.node_elements(el2, nn), P.node_elements(el1, n1),
                  vsel, psel, law=L)
    J00 = np.zeros((3 * nn, 3 * nn)); ru = np.zeros(3 * nn)
    U = u.reshape(-1, 3)
    for e in range(el2.shape[0]):
        Je, re = O.elem_gn(xyz2[el2[e]], U[el2[e]].ravel(), p[el1[e]], L, 1.0, True)
        vd = (3 * el2[e][:, None] + np.arange(3)).ravel()
        J00[np.ix_(vd, vd)] += Je[:30, :30]
        np.add.at(ru, vd, re[:30])
    for k, n in enumerate(vsel):
        np.testing.assert_allclose(o["ru"][k], ru[3 * n:3 * n + 3], rtol=0, atol=1e-14)
        for s, c in enumerate(o["c00"][k]):
            if c >= 0:
                np.testing.assert_allclose(o["v00"][k, :, s, :], J00[3 * n:3 * n + 3, 3 * c:3 * c + 3], rtol=0,
                                           atol=1e-14)


def test_full_size_row_checker_matches_whole_assembly():
    """The full-size parity checker (oracle/parity.py): the rows it rebuilds
    from each node's incident elements equal the whole-mesh COO assembly
    (Tpetra semantics), and its pattern check accepts the assembled pattern
    and rejects a perturbed one."""
    from oracle import parity as P
    xyz2, el2, _ = O.mesh(3, 2, seed=3)
    xyz1, el1, _ = O.mesh(3, 1, seed=3)
    u = O.field_fourier(xyz2, 3)
    pr = O.field_uniform(3, xyz1.shape[0])
    blocks, (ou, op) = O.assemble_ns(xyz2, el2, el1, xyz1.shape[0], u, pr, 0.01, 1.0, True, blocks=(0, 1, 2))
    n2, n1 = xyz2.shape[0], xyz1.shape[0]
    inc2, inc1 = P.node_elements(el2, n2), P.node_elements(el1, n1)
    specs = [(el2, el2, n2, inc2, 3, 3), (el2, el1, n2, inc2, 3, 1), (el1, el2, n1, inc1, 1, 3)]
    for b, (rc, cc, nr, inc, dr, dc) in enumerate(specs):
        assert P.check_pattern(rc, cc, nr, inc, dr, dc, blocks[b][0], blocks[b][1]) == -1
    bad = blocks[0][1].copy()
    bad[1000] += 3
    assert P.check_pattern(el2, el2, n2, inc2, 3, 3, blocks[0][0], bad) >= 0
    vsel, psel = np.arange(n2), np.arange(n1)
    o = P.rows_ns(xyz2, el2, el1, u, pr, 0.01, 1.0, True, inc2, inc1, vsel, psel)
    err = P.compare_ns(blocks, ou, op, o, vsel, psel)
    for k in ("00", "01", "10", "res_u", "res_p"):
        assert err[k] <= 1e-14, (k, err[k])
    L = O.law_from_E_nu(O.LAW_SKR2, 32.0 / 11.0, 5.0 / 11.0)
    uh = O.field_fourier(xyz2, 4, kmin=1, kmax=2, scale=0.02)
    (rp, ci, v), res = O.assemble_vec(1, L, 5, xyz2, el2, uh)
    sel = P.sample_nodes(n2, 0.2, seed=1)
    ev = P.compare_vec(rp, ci, v, res, P.rows_vec(1, L, 5, xyz2, el2, uh, inc2, sel), sel)
    assert ev["block"] <= 1e-14 and ev["residual"] <= 1e-14


# ---- elasticity pinned to the reference's classic C++ elements -------------
@pytest.fixture(scope="module")
def golden_elas():
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_elasticity.npz"))


def _relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(b).max())


def test_linear_elasticity_matches_reference(golden_elas):
    """FE::assemblyLinElasXDim (feddlib/core/FE/FE_def.hpp:4701-5071) run by
    the reference's own code on single jittered P2 elements: the oracle's
    classic element equals it, and so does skr1 at u = 0 (the reference's
    own pin, AceFemAssembly/tests/fe_test_linElas.cpp:120-136)."""
    g = golden_elas
    E, nu = 1000.0, 0.3
    mu = E / (2 * (1 + nu)); lam = nu * 2 * mu / (1 - 2 * nu)
    L1 = O.law_from_E_nu(O.LAW_SKR1, E, nu)
    for xe, Kref in zip(g["el_x"], g["linear_K"]):
        xe = np.ascontiguousarray(xe)
        assert _relmax(O.elem_linelas_classic(5, xe, lam, mu), Kref) <= 1e-13
        assert _relmax(O.elem_hyper(L1, 4, xe, None)[0], Kref) <= 1e-13


def test_neo_hooke_matches_reference_nh3d(golden_elas):
    """FE::nh3d through FE::assemblyElasticityJacobianAceFEM /
    assemblyElasticityStressesAceFEM (FE_def.hpp:3257-3460, 3461-3650,
    9665-9954): the reference's classic neo-Hooke element equals skr2 (the
    reference's own pin, AceFemAssembly/tests/fe_test_nonLinElas.cpp:118-141):
    tangent at a smooth and at a constant displacement, element stresses
    (= minus the AceGen residual), and P, A pointwise."""
    g = golden_elas
    L2 = O.law_from_E_nu(O.LAW_SKR2, 32.0 / 11.0, 5.0 / 11.0)
    for xe, ue, Kref, fref, Kc in zip(g["el_x"], g["el_u"], g["nh_K"], g["nh_f"], g["nh_K_const"]):
        xe = np.ascontiguousarray(xe)
        K, r = O.elem_hyper(L2, 5, xe, np.ascontiguousarray(ue))
        assert _relmax(K, Kref) <= 1e-13
        assert _relmax(-r, fref) <= 1e-13
        K0, _ = O.elem_hyper(L2, 5, xe, np.full(30, 0.1))
        assert _relmax(K0, Kc) <= 1e-13
    for F, P, A in zip(g["nh_F"], g["nh_P"], g["nh_A"]):
        _, Po, Ao = O.law_PA(L2, F)
        assert _relmax(Po, P) <= 1e-13 and _relmax(Ao, A) <= 1e-13


def test_elasticity_reference_live_if_built():
    """The whole jittered M = 2 P2 mesh assembled by the reference's own FE
    members (when oracle/_ref was built here) against the oracle's Tpetra-
    semantics assembly: linear elasticity and the nh3d tangent."""
    path = os.path.join(os.path.dirname(O.__file__), "_ref", "libfeddref.so")
    if not os.path.exists(path):
        pytest.skip("oracle/_ref not built (reference tree absent)")
    import ctypes as C
    R = C.CDLL(path)
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    R.ref_linelas_xdim.argtypes = [i, vp, i, vp, d, d, vp, vp, vp, i]
    R.ref_nh3d_acefem.argtypes = [i, vp, i, vp, vp, d, d, vp, vp, vp, i, vp]
    xyz, el, _ = O.mesh(2, 2, seed=8)
    nn, ne = xyz.shape[0], el.shape[0]
    el32 = np.ascontiguousarray(el, dtype=np.int32)
    cap = ne * 900
    rows = np.zeros(cap, dtype=np.int64); cols = np.zeros(cap, dtype=np.int64); vals = np.zeros(cap)
    E, nu = 1000.0, 0.3
    mu = E / (2 * (1 + nu)); lam = nu * 2 * mu / (1 - 2 * nu)
    k = R.ref_linelas_xdim(nn, O.p(xyz), ne, O.p(el32, O.I32), lam, mu, O.p(rows, O.I64), O.p(cols, O.I64),
                           O.p(vals), cap)
    ref = O.coo_to_csr(3 * nn, rows[:k].copy(), cols[:k].copy(), vals[:k].copy())
    (rp, ci, v), _ = O.assemble_vec(0, O.law_from_E_nu(O.LAW_SKR1, E, nu), 5, xyz, el, None)
    assert np.array_equal(rp, ref[0]) and np.array_equal(ci, ref[1]) and _relmax(v, ref[2]) <= 1e-13
    u = O.field_fourier(xyz, 9, kmin=1, kmax=2, scale=0.03)
    f = np.zeros(3 * nn)
    k = R.ref_nh3d_acefem(nn, O.p(xyz), ne, O.p(el32, O.I32), O.p(u), 32.0 / 11.0, 5.0 / 11.0, O.p(rows, O.I64),
                          O.p(cols, O.I64), O.p(vals), cap, O.p(f))
    ref = O.coo_to_csr(3 * nn, rows[:k].copy(), cols[:k].copy(), vals[:k].copy())
    (rp, ci, v), _ = O.assemble_vec(1, O.law_from_E_nu(O.LAW_SKR2, 32.0 / 11.0, 5.0 / 11.0), 5, xyz, el, u)
    assert np.array_equal(ci, ref[1]) and _relmax(v, ref[2]) <= 1e-13


def test_surrogate_targets_from_law_evaluations():
    """The surrogate's training targets from plain-law evaluations (energy and
    stress of the two-fibre law minus those of its neo-Hooke matrix, invariant
    derivatives by least squares; feddlib_gb300.surrogate.fibre_targets),
    fed with the oracle's law here, equal the fibre energy and its
    derivatives; the quadrature-point deformation gradients match the
    oracle's element kinematics."""
    from feddlib_gb300 import surrogate as S
    La = O.LawSpec(O.LAW_ANISO, mu=1.0, lam=10.0, k1=2.0, k2=1.0, angle_deg=40.0)
    Lm = O.LawSpec(O.LAW_SKR1, mu=1.0, lam=10.0)
    rng = np.random.default_rng(5)
    F = np.array([np.eye(3) + 0.12 * rng.standard_normal((3, 3)) for _ in range(200)])
    ev = lambda L: [O.law_PA(L, f) for f in F]
    pa, pm = ev(La), ev(Lm)
    inv, psi, g = S.fibre_targets(F, np.array([x[0] for x in pa]), np.array([x[1] for x in pa]),
                                  np.array([x[0] for x in pm]), np.array([x[1] for x in pm]))
    psi_ref, g_ref = S.fibre_energy(inv)
    assert np.abs(psi - psi_ref).max() <= 1e-12 * np.abs(psi_ref).max()
    assert np.abs(g - g_ref).max() <= 1e-10 * np.abs(g_ref).max()
    inv_o = np.array([O.law_invariants(La, f) for f in F])
    assert np.abs(inv - inv_o).max() <= 1e-13
    # deformation gradients at quadrature points, against the oracle's element residual
    # (r = -sum_q w det B P(F_q) : grad phi; here with one point's F rebuilt per element)
    xyz, el, _ = O.mesh(2, 2, seed=4)
    u = O.field_fourier(xyz, 4, kmin=1, kmax=2, scale=0.05)
    es = np.arange(el.shape[0]); qs = es % 4
    Fq = S.qp_F(xyz, el, u, es, qs)
    pts, _ = O.quad(4)
    for e in (0, 17, 33):
        g_ref = O.dphi(2, pts[qs[e]])
        xe = xyz[el[e]]
        B = np.stack([xe[1] - xe[0], xe[2] - xe[0], xe[3] - xe[0]], axis=1)
        Fe = np.eye(3) + u.reshape(-1, 3)[el[e]].T @ (g_ref @ np.linalg.inv(B))
        assert np.abs(Fq[e] - Fe).max() <= 1e-14


def test_rhs_function_restatement():
    """The oracle's FE::assemblyRHS with a source function (FE_def.hpp:7303-7400):
    a constant function gives the compiled restatement's constant-source load
    (pinned by the Laplace goldens), a Vector source is three Scalar ones, and
    the physical points are B xhat + x_0 of each element."""
    for fe, npts in ((1, 1), (2, 5)):
        xyz, el, _ = O.mesh(2, fe, seed=5)
        b = O.assemble_rhs_func(fe, npts, xyz, el, lambda x: 1.75, 1)
        assert np.abs(b - O.assemble_rhs(fe, npts, xyz, el, 1.75)).max() < 1e-15
        f3 = lambda x: [np.cos(x[0]), x[1] * x[2], 2.0 + x[0] * x[1]]
        bv = O.assemble_rhs_func(fe, npts, xyz, el, f3, 3).reshape(-1, 3)
        for c in range(3):
            bc = O.assemble_rhs_func(fe, npts, xyz, el, lambda x, c=c: f3(x)[c], 1)
            assert np.array_equal(bv[:, c], bc)
        xq = O.rhs_points(npts, xyz, el)
        pts, _ = O.quad(npts)
        e = 3
        v = xyz[el[e, :4]]
        assert np.allclose(xq[e], v[0] + pts @ (v[1:] - v[0]), rtol=0, atol=1e-15)


def test_ns_residual_coefficients_live_if_built():
    """The oracle's residual with FE::assemblyNavierStokes' coeff against the
    reference's own AssembleFENavierStokes after setCoeff
    (AssembleFENavierStokes_def.hpp:56-64, 199-224), compiled here."""
    path = os.path.join(os.path.dirname(O.__file__), "_ref", "libfeddref.so")
    if not os.path.exists(path):
        pytest.skip("oracle/_ref not built (reference tree absent)")
    import ctypes as C
    R = C.CDLL(path)
    if not hasattr(R, "ref_ns_element_coeff"):
        pytest.skip("oracle/_ref predates ref_ns_element_coeff")
    xyz, conn, _ = O.mesh(3, 2, seed=12)
    rng = np.random.default_rng(6)
    for e, co in zip(rng.integers(0, conn.shape[0], 4), ((0.5, 2.0, -1.5, 3.0), (1.0, 0.0, 0.0, 1.0),
                                                         (-0.25, 1.0, 4.0, 0.0), (1.0, 1.0, 1.0, 1.0))):
        xe = np.ascontiguousarray(xyz[conn[e]])
        sol = rng.uniform(-2, 2, 34)
        r = np.zeros(34)
        c = np.ascontiguousarray(co, dtype=np.float64)
        assert R.ref_ns_element_coeff(O.p(xe), O.p(sol), C.c_double(0.03), C.c_double(1.7), O.p(c), O.p(r)) == 0
        _, ro = O.elem_ns(xe, sol[:30], sol[30:], 0.03, 1.7, True, coeff=co)
        assert np.abs(r - ro).max() <= 1e-13 * max(np.abs(ro).max(), 1e-300), co


def test_rhs_function_live_if_built():
    """The oracle's load vector with a source function against the
    reference's own FE::assemblyRHS (FE_def.hpp:7303-7400), extracted and
    compiled here, Scalar on P1 and Vector on P2."""
    path = os.path.join(os.path.dirname(O.__file__), "_ref", "libfeddref.so")
    if not os.path.exists(path):
        pytest.skip("oracle/_ref not built (reference tree absent)")
    import ctypes as C
    R = C.CDLL(path)
    if not hasattr(R, "ref_assembly_rhs"):
        pytest.skip("oracle/_ref predates ref_assembly_rhs")
    fs = lambda x: np.sin(3.0 * x[0]) + 0.5
    fv = lambda x: [x[0] * x[0], 2.0 * x[0] * 0.5, 1.0 + x[0]]
    for fe, npts, nc, f in ((1, 1, 1, fs), (2, 5, 3, fv), (2, 5, 1, fs)):
        xyz, el, _ = O.mesh(2, fe, seed=7)
        out = np.zeros(xyz.shape[0] * nc)
        conn = np.ascontiguousarray(el, dtype=np.int32)
        assert R.ref_assembly_rhs(el.shape[1], xyz.shape[0], O.p(xyz), el.shape[0], O.p(conn, O.I32), nc,
                                  O.p(out)) == 0
        ob = O.assemble_rhs_func(fe, npts, xyz, el, f, nc)
        assert np.abs(out - ob).max() <= 1e-13 * np.abs(ob).max(), (fe, nc)
