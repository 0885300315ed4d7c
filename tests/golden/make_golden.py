"""Generates tests/golden/ref_elements.npz, ref_elasticity.npz and
ref_gn_outflow.npz from FEDDLib's own element code.

Run in a container that has the reference tree: it builds oracle/_ref
(oracle/build_ref.sh compiles FEDDLib's Helper.cpp and the AssembleFE_Laplace /
AssembleFENavierStokes / AssembleFEGeneralizedNewtonian element classes
against stub Trilinos headers) and
records, for seeded inputs, the reference's quadrature tables, basis tables and
element matrices.  The fixtures travel with the repository; the reference tree
does not.

    python tests/golden/make_golden.py
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402  (only for the seeded mesh)


def main():
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")])
    R = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libfeddref.so"))
    Dp = C.POINTER(C.c_double)

    def p(a):
        return a.ctypes.data_as(Dp)

    out = {}
    for deg in (1, 2, 3, 4, 5):
        pts = np.zeros((32, 3)); w = np.zeros(32)
        n = R.ref_quad(deg, p(pts), p(w))
        out[f"quad_deg{deg}_pts"] = pts[:n].copy()
        out[f"quad_deg{deg}_w"] = w[:n].copy()
    for fe in ("P1", "P2"):
        nb = 4 if fe == "P1" else 10
        for deg in (1, 3, 5):
            dphi = np.zeros(32 * nb * 3); phi = np.zeros(32 * nb)
            nq = R.ref_dphi(fe.encode(), deg, p(dphi), p(phi))
            out[f"dphi_{fe}_deg{deg}"] = dphi[:nq * nb * 3].reshape(nq, nb, 3).copy()
            out[f"phi_{fe}_deg{deg}"] = phi[:nq * nb].reshape(nq, nb).copy()
    # Navier-Stokes elements of a jittered P2 mesh (M=2, seed 3), random fields
    xyz, conn, _ = O.mesh(2, 2, seed=3)
    rng = np.random.default_rng(2024)
    els = [0, 5, 17, 40]
    xs, sols, Jn, Jf, rn = [], [], [], [], []
    for e in els:
        xe = np.ascontiguousarray(xyz[conn[e]])
        sol = np.concatenate([rng.uniform(-1, 1, 30), rng.uniform(-1, 1, 4)])
        J1 = np.zeros(34 * 34); J0 = np.zeros(34 * 34); r = np.zeros(34); r0 = np.zeros(34)
        assert R.ref_ns_element(p(xe), p(sol), C.c_double(0.01), C.c_double(1.0), 1, p(J1), p(r)) == 0
        assert R.ref_ns_element(p(xe), p(sol), C.c_double(0.01), C.c_double(1.0), 0, p(J0), p(r0)) == 0
        xs.append(xe); sols.append(sol); Jn.append(J1.reshape(34, 34)); Jf.append(J0.reshape(34, 34))
        rn.append(r)
    out["ns_x"] = np.array(xs); out["ns_sol"] = np.array(sols)
    out["ns_J_newton"] = np.array(Jn); out["ns_J_fixedpoint"] = np.array(Jf)
    out["ns_res"] = np.array(rn)
    out["ns_visc"] = np.array(0.01); out["ns_dens"] = np.array(1.0)
    # generalized-Newtonian elements (AssembleFEGeneralizedNewtonian), three
    # viscosity laws, Newton and FixedPoint, velocity of modest amplitude
    gn_models = [(0, [0.5, 0.6, 0.05, 0.005, 1.5]), (1, [0.02, 0.7, 1.0, 1e-4, 0.0]),
                 (2, [0.8, 0.5, 1.0, 0.1, 0.03])]
    gx, gs, gm, gJn, gJf, gr = [], [], [], [], [], []
    for mi, (model, prm) in enumerate(gn_models):
        for e in (3, 22):
            xe = np.ascontiguousarray(xyz[conn[e]])
            sol = np.concatenate([rng.uniform(-0.5, 0.5, 30), rng.uniform(-1, 1, 4)])
            mp = np.array(prm, dtype=np.float64)
            J1 = np.zeros(34 * 34); J0 = np.zeros(34 * 34); r = np.zeros(34); r0 = np.zeros(34)
            assert R.ref_gn_element(p(xe), p(sol), model, p(mp), C.c_double(1.0), 1, p(J1), p(r)) == 0
            assert R.ref_gn_element(p(xe), p(sol), model, p(mp), C.c_double(1.0), 0, p(J0), p(r0)) == 0
            gx.append(xe); gs.append(sol); gm.append(np.concatenate([[model], mp]))
            gJn.append(J1.reshape(34, 34)); gJf.append(J0.reshape(34, 34)); gr.append(r)
    out["gn_x"] = np.array(gx); out["gn_sol"] = np.array(gs); out["gn_model"] = np.array(gm)
    out["gn_J_newton"] = np.array(gJn); out["gn_J_fixedpoint"] = np.array(gJf); out["gn_res"] = np.array(gr)
    # Laplace elements (AssembleFE_Laplace), P1 and P2, f = 1
    for fe, order in (("P1", 1), ("P2", 2)):
        xyzl, connl, _ = O.mesh(2, order, seed=1)
        nb = connl.shape[1]
        Ks, bs, xl = [], [], []
        for e in (1, 9, 30):
            xe = np.ascontiguousarray(xyzl[connl[e]])
            K = np.zeros(nb * nb); b = np.zeros(nb)
            assert R.ref_laplace_element(fe.encode(), p(xe), C.c_double(1.0), p(K), p(b)) == 0
            Ks.append(K.reshape(nb, nb)); bs.append(b); xl.append(xe)
        out[f"lap_{fe}_x"] = np.array(xl); out[f"lap_{fe}_K"] = np.array(Ks)
        out[f"lap_{fe}_b"] = np.array(bs)
    np.savez_compressed(os.path.join(HERE, "ref_elements.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_elements.npz"))
    elasticity(R)
    gn_outflow(R)


def ref_bind(R):
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    R.ref_linelas_xdim.argtypes = [i, vp, i, vp, d, d, vp, vp, vp, i]
    R.ref_nh3d_acefem.argtypes = [i, vp, i, vp, vp, d, d, vp, vp, vp, i, vp]
    R.ref_nh3d.argtypes = [d, d, vp, vp, vp]
    return R


def ref_element_elasticity(R, xe, ue, E, nu, kind):
    """FE::assemblyLinElasXDim (kind "linear", lambda/mu from E, nu) or
    FE::assemblyElasticityJacobianAceFEM + assemblyElasticityStressesAceFEM
    with "Neo-Hooke" (kind "nh3d") run on a one-element mesh: the element
    matrix (30 x 30, node-wise dofs) and, for nh3d, the element stresses."""
    cap = 900
    rows = np.zeros(cap, dtype=np.int64); cols = np.zeros(cap, dtype=np.int64); vals = np.zeros(cap)
    conn = np.arange(10, dtype=np.int32)
    x = np.ascontiguousarray(xe, dtype=np.float64)
    f = np.zeros(30)
    if kind == "linear":
        mu = E / (2 * (1 + nu)); lam = nu * 2 * mu / (1 - 2 * nu)
        k = R.ref_linelas_xdim(10, x.ctypes.data, 1, conn.ctypes.data, lam, mu, rows.ctypes.data, cols.ctypes.data,
                               vals.ctypes.data, cap)
    else:
        u = np.ascontiguousarray(ue, dtype=np.float64)
        k = R.ref_nh3d_acefem(10, x.ctypes.data, 1, conn.ctypes.data, u.ctypes.data, E, nu, rows.ctypes.data,
                              cols.ctypes.data, vals.ctypes.data, cap, f.ctypes.data)
    assert k == cap
    K = np.zeros((30, 30))
    K[rows[:k], cols[:k]] = vals[:k]
    return K, f


def elasticity(R):
    """tests/golden/ref_elasticity.npz: the reference's classic elasticity
    elements (FE_def.hpp members, extracted and compiled by oracle/build_ref.sh)
    on jittered P2 elements -- linear elasticity (E = 1000, nu = 0.3) at u = 0,
    the nh3d neo-Hooke law (E = 32/11, nu = 5/11, i.e. mu = 1, lambda = 10) at a
    smooth displacement and at a constant one -- and nh3d's P and A at given
    deformation gradients."""
    ref_bind(R)
    xyz, conn, _ = O.mesh(2, 2, seed=5)
    u = O.field_fourier(xyz, 4, kmin=1, kmax=2, scale=0.03).reshape(-1, 3)
    els = [0, 9, 21, 26, 38, 47]
    out = {"el_x": np.array([xyz[conn[e]] for e in els]), "el_u": np.array([u[conn[e]].ravel() for e in els])}
    out["linear_K"] = np.array([ref_element_elasticity(R, xyz[conn[e]], None, 1000.0, 0.3, "linear")[0] for e in els])
    KS, FS, KC = [], [], []
    for k, e in enumerate(els):
        K, f = ref_element_elasticity(R, xyz[conn[e]], out["el_u"][k], 32.0 / 11.0, 5.0 / 11.0, "nh3d")
        KS.append(K); FS.append(f)
        KC.append(ref_element_elasticity(R, xyz[conn[e]], np.full(30, 0.1), 32.0 / 11.0, 5.0 / 11.0, "nh3d")[0])
    out["nh_K"], out["nh_f"], out["nh_K_const"] = np.array(KS), np.array(FS), np.array(KC)
    rng = np.random.default_rng(11)
    Fs = np.array([np.eye(3) + 0.15 * rng.standard_normal((3, 3)) for _ in range(4)])
    P = np.zeros((4, 9)); A = np.zeros((4, 81))
    for k in range(4):
        Fk = np.ascontiguousarray(Fs[k].ravel())
        R.ref_nh3d(32.0 / 11.0, 5.0 / 11.0, Fk.ctypes.data, P[k].ctypes.data, A[k].ctypes.data)
    out["nh_F"], out["nh_P"], out["nh_A"] = Fs, P.reshape(4, 3, 3), A.reshape(4, 3, 3, 3, 3)
    np.savez_compressed(os.path.join(HERE, "ref_elasticity.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_elasticity.npz"))


def gn_outflow(R):
    """AssembleFEGeneralizedNewtonian elements flagged for the outflow
    Neumann term on one face (oracle/ref_driver.cpp sets the surface data as
    FEDDLib's Domain does): Jacobian (Newton and FixedPoint), the fixed-point
    matrix (assembleFixedPoint) and residual,
    three viscosity laws, faces given in several node orders (the order sets
    the normal's sign)."""
    def p(a):
        return a.ctypes.data_as(C.POINTER(C.c_double))

    xyz, conn, _ = O.mesh(2, 2, seed=3)
    rng = np.random.default_rng(77)
    models = [(0, [1.902, 0.22, 0.056, 0.00345, 1.25]), (1, [0.035, 0.61, 0.35, 1e-10, 0.0]),
              (2, [0.8, 0.45, 230.633, 3.3707, 0.0012])]
    faces = [(0, 1, 2), (0, 3, 1), (1, 2, 3), (3, 2, 0)]
    X, FC, S, M, Jn, Jf, RR, JP = [], [], [], [], [], [], [], []
    for k, (model, prm) in enumerate(models):
        for j, e in enumerate((4, 29)):
            xe = np.ascontiguousarray(xyz[conn[e]])
            face = np.ascontiguousarray(xe[list(faces[(2 * k + j) % 4])])
            sol = np.concatenate([rng.uniform(-0.5, 0.5, 30), rng.uniform(-1, 1, 4)])
            mp = np.array(prm, dtype=np.float64)
            J1 = np.zeros(34 * 34); J0 = np.zeros(34 * 34); r = np.zeros(34); r0 = np.zeros(34)
            assert R.ref_gn_element_outflow(p(xe), p(face), p(sol), model, p(mp), C.c_double(1.0), 1, p(J1),
                                            p(r)) == 0
            assert R.ref_gn_element_outflow(p(xe), p(face), p(sol), model, p(mp), C.c_double(1.0), 0, p(J0),
                                            p(r0)) == 0
            Jp = np.zeros(34 * 34); rp_ = np.zeros(34)
            assert R.ref_gn_element_fixed_point(p(xe), p(face), p(sol), model, p(mp), C.c_double(1.0), p(Jp),
                                                p(rp_)) == 0
            X.append(xe); FC.append(face); S.append(sol); M.append(np.concatenate([[model], mp]))
            Jn.append(J1.reshape(34, 34)); Jf.append(J0.reshape(34, 34)); RR.append(r)
            JP.append(Jp.reshape(34, 34))
    out = {"x": np.array(X), "face": np.array(FC), "sol": np.array(S), "model": np.array(M),
           "J_newton": np.array(Jn), "J_fixedpoint": np.array(Jf), "res": np.array(RR),
           "J_fixed_point_matrix": np.array(JP)}
    np.savez_compressed(os.path.join(HERE, "ref_gn_outflow.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_gn_outflow.npz"))


if __name__ == "__main__":
    main()
