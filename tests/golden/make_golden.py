"""Generates tests/golden/ref_elements.npz from FEDDLib's own element code.

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


if __name__ == "__main__":
    main()
