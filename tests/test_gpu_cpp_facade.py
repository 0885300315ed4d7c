"""GPU test of the C++ facade (include/feddgpu_fe.hpp): tests/cpp/facade_main.cpp
drives feddgpu::FE and feddgpu::AssembleFEFactory as FEDDLib's drivers drive
FE::assembly* and AssembleFE; its outputs are checked against the FP64
oracle (patterns bit-exact, values within the FP32 / FP64 tolerances) and
against the Python binding of the same engine (bitwise)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL_FP32, TOL_FP64 = 1e-6, 1e-12


def build_facade_program(dst):
    """g++ the facade test program against the in-tree engine library."""
    lib = os.path.join(ROOT, "feddlib_gb300")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "facade_main.cpp"), "-L", lib, "-lfeddgpu",
           f"-Wl,-rpath,{lib}", "-o", dst]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def read_records(path):
    types = {0: np.float64, 1: np.int64, 2: np.int32}
    out = {}
    with open(path, "rb") as f:
        while True:
            head = f.read(32)
            if not head:
                break
            name = head.rstrip(b"\0").decode()
            t = int(np.frombuffer(f.read(4), np.int32)[0])
            n = int(np.frombuffer(f.read(8), np.int64)[0])
            dt = np.dtype(types[t])
            out[name] = np.frombuffer(f.read(n * dt.itemsize), dt).copy()
    return out


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def res(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("facade")
    exe, data = str(d / "facade_main"), str(d / "out.bin")
    build_facade_program(exe)
    p = subprocess.run([exe, data], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    return read_records(data)


def test_facade_navier_stokes(res):
    xyz2, el2, _ = O.mesh(2, 2, seed=3)
    xyz1, el1, _ = O.mesh(2, 1, seed=3)
    u = O.field_fourier(xyz2, 3)
    p = O.field_uniform(3, xyz1.shape[0])
    blocks, (ou, op) = O.assemble_ns(xyz2, el2, el1, xyz1.shape[0], u, p, 0.01, 1.0, True, blocks=(0, 1, 2, 3))
    for b, name in enumerate(("ns00", "ns01", "ns10")):
        np.testing.assert_array_equal(res[name + "_rowptr"], blocks[b][0])
        np.testing.assert_array_equal(res[name + "_colind"], blocks[b][1])
        assert rel(res[name + "_values"], blocks[b][2]) < TOL_FP32, name
    assert res["ns11_nnz"][0] == 0
    assert rel(res["ns_res_u"], ou) < TOL_FP32
    assert rel(res["ns_res_p"], op) < TOL_FP32
    fp, _ = O.assemble_ns(xyz2, el2, el1, xyz1.shape[0], u, p, 0.01, 1.0, False, blocks=(0,))
    assert rel(res["nsfp00_values"], fp[0][2]) < TOL_FP32
    assert np.array_equal(res["ns00_reassembled"], res["ns00_values"])


def test_facade_generalized_newtonian(res):
    """FE::assemblyNavierStokes with Material/Newtonian = false (Carreau-Yasuda)
    and outflow faces on the plane x = 1: the Newton Jacobian's block (0,0)
    without the outflow term, the residual with it, and the "FixedPoint"
    mode's fixed-point matrix with it."""
    xyz2, el2, _ = O.mesh(2, 2, seed=6)
    xyz1, el1, _ = O.mesh(2, 1, seed=6)
    u = O.field_fourier(xyz2, 6, scale=0.5)
    p = O.field_uniform(6, xyz1.shape[0])
    L = O.visc_law(0, [1.902, 0.22, 0.056, 0.00345, 1.25], 1e-12)
    faces = res["gn_faces"].reshape(-1, 3)
    assert faces.shape[0] == 8
    _, taken = O.outflow_owners(el2, faces)
    n_u = 3 * xyz2.shape[0]
    U = u.reshape(-1, 3)

    def dense00(newton, with_k):
        J = np.zeros((n_u, n_u))
        r = np.zeros(n_u)
        for e in range(el2.shape[0]):
            ue = U[el2[e]].ravel()
            Je, re = O.elem_gn(xyz2[el2[e]], ue, p[el1[e]], L, 1.0, newton)
            vd = (3 * el2[e][:, None] + np.arange(3)).ravel()
            J[np.ix_(vd, vd)] += Je[:30, :30]
            np.add.at(r, vd, re[:30])
            if e in taken:
                K = O.gn_outflow(xyz2[el2[e]], xyz2[faces[taken[e]]], ue, L)
                np.add.at(r, vd, K @ ue)
                if with_k:
                    J[np.ix_(vd, vd)] += K
        return J, r

    def csr_dense(prefix, values):
        rp, ci = res[prefix + "_rowptr"], res[prefix + "_colind"]
        M = np.zeros((n_u, n_u))
        M[np.repeat(np.arange(n_u), np.diff(rp)), ci] = values
        return M

    J, r = dense00(True, False)
    assert rel(csr_dense("gn00", res["gn00_values"]), J) < TOL_FP32
    assert rel(res["gn_res_u"], r) < TOL_FP32
    Jfp, _ = dense00(False, True)
    assert rel(csr_dense("gn00", res["gnfp00_values"]), Jfp) < TOL_FP32
    # the factory's "GeneralizedNewtonian" elements (no outflow flag on them)
    K4 = res["assfe_gn_K"].reshape(4, 34, 34)
    r4 = res["assfe_gn_r"].reshape(4, 34)
    for e in range(4):
        Jo, ro = O.elem_gn(xyz2[el2[e]], U[el2[e]].ravel(), p[el1[e]], L, 1.0, True)
        assert rel(K4[e], Jo) < 2e-6 and rel(r4[e], ro) < 2e-6, e


def test_facade_assemble_fe_elements(res):
    xyz2, el2, _ = O.mesh(2, 2, seed=3)
    xyz1, el1, _ = O.mesh(2, 1, seed=3)
    u = O.field_fourier(xyz2, 3)
    p = O.field_uniform(3, xyz1.shape[0])
    K = res["assfe_ns_K"].reshape(-1, 34, 34)
    r = res["assfe_ns_r"].reshape(-1, 34)
    assert K.shape[0] == 6
    for e in range(6):
        Jo, ro = O.elem_ns(xyz2[el2[e]], u.reshape(-1, 3)[el2[e]].ravel(), p[el1[e]], 0.01, 1.0, True)
        assert rel(K[e], Jo) < 2e-6
        assert rel(r[e], ro) < 2e-6


def test_facade_laplace_and_load(res):
    xyz, el, _ = O.mesh(2, 1, seed=1)
    orp, oci, ov = O.assemble_laplace(1, 1, xyz, el)
    np.testing.assert_array_equal(res["lap_rowptr"], orp)
    np.testing.assert_array_equal(res["lap_colind"], oci)
    assert rel(res["lap_values"], ov) < TOL_FP64
    assert rel(res["lap_rhs"], O.assemble_rhs(1, 1, xyz, el, 1.0)) < TOL_FP64
    # assemblyLaplaceAssFE gives assemblyLaplace's matrix (fe_test_laplace.cpp:104-161)
    for k in ("rowptr", "colind", "values"):
        assert np.array_equal(res["lapassfe_" + k], res["lap_" + k]), k


def test_facade_rhs_source_functions(res):
    """FE::assemblyRHS with an RhsFunc_Type source, Scalar (P1) and Vector (P2)."""
    xyz, el, _ = O.mesh(2, 1, seed=1)
    ob = O.assemble_rhs_func(1, 1, xyz, el, lambda x: 2.0 * x[0] + np.sin(x[1]), 1)
    assert rel(res["lap_rhs_func"], ob) < TOL_FP64
    xyz, el, _ = O.mesh(2, 2, seed=4)
    ob = O.assemble_rhs_func(2, 5, xyz, el, lambda x: [x[0] * x[0], 0.5 * x[1], 1.0 + x[2]], 3)
    assert rel(res["nh_rhs_vector"], ob) < TOL_FP64


def test_facade_nonlinear_elasticity(res):
    xyz, el, _ = O.mesh(2, 2, seed=4)
    u = O.field_fourier(xyz, 4, kmin=1, kmax=2, scale=0.004)
    L = O.law_from_E_nu(O.LAW_SKR2, 32.0 / 11.0, 5.0 / 11.0)
    (orp, oci, ov), ores = O.assemble_vec(1, L, 5, xyz, el, u)
    np.testing.assert_array_equal(res["nh_rowptr"], orp)
    np.testing.assert_array_equal(res["nh_colind"], oci)
    assert rel(res["nh_values"], ov) < TOL_FP32
    assert rel(res["nh_res"], ores) < 1e-5


def test_facade_nonlinear_elasticity_modulus_field(res):
    """FE::assemblyNonLinearElasticity's E-field variant (FE_def.hpp:538-614)."""
    xyz, el, _ = O.mesh(2, 2, seed=4)
    U = O.field_fourier(xyz, 4, kmin=1, kmax=2, scale=0.004).reshape(-1, 3)
    emod = 0.5 + 0.25 * (np.arange(el.shape[0]) % 7)
    n = 3 * xyz.shape[0]
    Kd, rd = np.zeros((n, n)), np.zeros(n)
    for e in range(el.shape[0]):
        Ko, ro = O.elem_hyper(O.law_from_E_nu(O.LAW_SKR2, emod[e], 5.0 / 11.0), 5, xyz[el[e]], U[el[e]].ravel())
        d = (3 * el[e][:, None] + np.arange(3)).ravel()
        Kd[np.ix_(d, d)] += Ko
        rd[d] += ro
    rp, ci = res["nhE_rowptr"], res["nhE_colind"]
    rows = np.repeat(np.arange(n), np.diff(rp))
    assert rel(res["nhE_values"], Kd[rows, ci]) < TOL_FP32
    assert rel(res["nhE_res"], rd) < 1e-5


def test_facade_same_values_as_python_binding(res):
    import feddlib_gb300 as F
    xyz, el = F.structured_mesh(2, 2, seed=4)
    u = F.fourier_field(xyz, seed=4, kmin=1, kmax=2, scale=0.004)
    a = F.Assembler(F.NONLINEAR_ELASTICITY, xyz, el, E=32.0 / 11.0, poisson_ratio=5.0 / 11.0)
    (v,), r, _ = a.assemble(u=u)
    assert np.array_equal(v, res["nh_values"]) and np.array_equal(r, res["nh_res"])


def test_facade_errors_are_exceptions(res):
    from feddlib_gb300 import _capi as A
    assert list(res["error_codes"]) == [A.ERR_ARG, A.ERR_ARG]


def test_facade_assemble_fe_controls(res):
    """AssembleFE's per-element controls: changeLinearization (FixedPoint from
    the parameter list, then Newton), updateParameter("E") on neo-Hooke
    elements (AssembleFE_NonLinElas_def.hpp:175-180; other names ignored),
    the time and Newton counters (AssembleFE_def.hpp:79-101), and the
    batch's refusal of elements that disagree on E or the linearization."""
    from feddlib_gb300 import _capi as A
    xyz2, el2, _ = O.mesh(2, 2, seed=3)
    xyz1, el1, _ = O.mesh(2, 1, seed=3)
    u = O.field_fourier(xyz2, 3).reshape(-1, 3)
    p = O.field_uniform(3, xyz1.shape[0])
    Kfp = res["assfe_ns_fp_K"].reshape(-1, 34, 34)
    Knt = res["assfe_ns_newton_K"].reshape(-1, 34, 34)
    for e in range(6):
        Jf, _ = O.elem_ns(xyz2[el2[e]], u[el2[e]].ravel(), p[el1[e]], 0.01, 1.0, False)
        Jn, _ = O.elem_ns(xyz2[el2[e]], u[el2[e]].ravel(), p[el1[e]], 0.01, 1.0, True)
        assert rel(Kfp[e], Jf) < 2e-6 and rel(Knt[e], Jn) < 2e-6, e
    assert rel(Kfp[0], Knt[0]) > 1e-4  # the W term is there
    xyz, el, _ = O.mesh(2, 2, seed=4)
    d = O.field_fourier(xyz, 4, kmin=1, kmax=2, scale=0.004).reshape(-1, 3)
    L = O.law_from_E_nu(O.LAW_SKR2, 5.0, 5.0 / 11.0)
    K5 = res["assfe_nhE5_K"].reshape(-1, 30, 30)
    r5 = res["assfe_nhE5_r"].reshape(-1, 30)
    for e in range(4):
        Ko, ro = O.elem_hyper(L, 5, xyz[el[e]], d[el[e]].ravel())
        assert rel(K5[e], Ko) < 2e-6 and rel(r5[e], ro) < 1e-5, e
    assert list(res["assfe_ctl_codes"]) == [A.ERR_UNSUPPORTED, A.ERR_UNSUPPORTED]
    assert list(res["assfe_gn_block_code"]) == [A.ERR_UNSUPPORTED]
    assert list(res["assfe_counters"]) == [0.75, 0.25, 2.0, 0.0]
    co = (0.5, 2.0, -1.5, 3.0)
    rco = res["assfe_ns_coeff_r"].reshape(-1, 34)
    for e in range(6):
        _, ro = O.elem_ns(xyz2[el2[e]], u[el2[e]].ravel(), p[el1[e]], 0.01, 1.0, True, coeff=co)
        assert rel(rco[e], ro) < 2e-6, e


def test_facade_navier_stokes_residual_coefficients(res):
    """FE::assemblyNavierStokes' coeff scales the residual's blocks as the
    reference's elements do after setCoeff (AssembleFENavierStokes_def.hpp:199-224)."""
    xyz2, el2, _ = O.mesh(2, 2, seed=3)
    xyz1, el1, _ = O.mesh(2, 1, seed=3)
    U = O.field_fourier(xyz2, 3).reshape(-1, 3)
    p = O.field_uniform(3, xyz1.shape[0])
    co = (0.5, 2.0, -1.5, 3.0)
    ru, rp = np.zeros(U.size), np.zeros(p.size)
    for e in range(el2.shape[0]):
        _, r = O.elem_ns(xyz2[el2[e]], U[el2[e]].ravel(), p[el1[e]], 0.01, 1.0, True, coeff=co)
        for a in range(10):
            ru[3 * el2[e, a]:3 * el2[e, a] + 3] += r[3 * a:3 * a + 3]
        rp[el1[e]] += r[30:]
    assert rel(res["ns_res_u_coeff"], ru) < TOL_FP32
    assert rel(res["ns_res_p_coeff"], rp) < TOL_FP32
