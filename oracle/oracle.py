"""Python side of the FP64 CPU oracle (test infrastructure only).

Loads ``oracle/liboracle.so`` (built by ``oracle/Makefile``) and exposes the
FEDDLib restatement with numpy arrays.  Only tests/, ``__graft_entry__.smoke``
and bench.py's cpu_baseline leg import this module; the engine never does.
"""
import ctypes as C
import math
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

D = C.POINTER(C.c_double)
I32 = C.POINTER(C.c_int32)
I64 = C.POINTER(C.c_int64)

LAW_SKR1, LAW_SKR2, LAW_ANISO, LAW_MLP, LAW_SKR3 = 1, 2, 3, 4, 5


class Law(C.Structure):
    _fields_ = [("law", C.c_int), ("mu", C.c_double), ("lam", C.c_double),
                ("k1", C.c_double), ("k2", C.c_double),
                ("a1", C.c_double * 3), ("a2", C.c_double * 3),
                ("hidden", C.c_int), ("W1", D), ("b1", D), ("W2", D), ("b2", D),
                ("w3", D), ("b3", C.c_double), ("in_shift", D), ("in_scale", D),
                ("out_scale", C.c_double), ("mlp_add_matrix", C.c_int), ("in_clamp", C.c_int)]


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            import subprocess
            subprocess.check_call(["make", "-s", "-C", _HERE])
        L = C.CDLL(path)
        L.orc_quad.restype = C.c_int
        L.orc_quad_points_for_degree.restype = C.c_int
        L.orc_degree_un.restype = C.c_int
        L.orc_degree_pair.restype = C.c_int
        L.orc_mesh_orient.restype = C.c_int64
        L.orc_geometry.restype = C.c_double
        L.orc_coo_to_csr.restype = C.c_int64
        L.orc_assemble_laplace_coo.restype = C.c_int64
        L.orc_assemble_vec_coo.restype = C.c_int64
        L.orc_assemble_ns_coo.restype = C.c_int64
        L.orc_mlp_loss.restype = C.c_double
        L.orc_cpu_baseline_ns.restype = C.c_double
        L.orc_cpu_baseline_vec.restype = C.c_double
        i, i64, d, u64, vp = C.c_int, C.c_int64, C.c_double, C.c_uint64, C.c_void_p
        sig = {
            "orc_quad": [i, vp, vp], "orc_quad_points_for_degree": [i],
            "orc_degree_un": [i, C.c_uint], "orc_degree_pair": [i, i, i, i, i],
            "orc_phi": [i, vp, vp], "orc_dphi": [i, vp, vp],
            "orc_mesh_sizes": [i, i, vp, vp], "orc_mesh_structured": [i, i, vp, vp],
            "orc_mesh_jitter": [i, i, u64, d, vp], "orc_mesh_p2_midpoints": [i64, vp, vp],
            "orc_mesh_orient": [i, i64, vp, vp], "orc_geometry": [vp] * 6,
            "orc_elem_laplace": [i, i, vp, vp], "orc_elem_rhs_const": [i, i, vp, d, vp],
            "orc_elem_ns": [vp, vp, vp, d, d, i, vp, vp, vp, vp, vp, vp, vp],
            "orc_elem_linelas_classic": [i, vp, d, d, vp],
            "orc_law_invariants": [vp, vp, vp], "orc_law_dpsi": [vp, vp, vp, vp, vp],
            "orc_law_PA": [vp, vp, vp, vp, vp], "orc_elem_hyper": [vp, i, vp, vp, vp, vp],
            "orc_mlp_eval": [i, vp, vp, vp, vp, vp, d, vp, vp, vp, vp],
            "orc_mlp_loss": [i, vp, vp, vp, vp, vp, d, i64, vp, vp, vp, d, d] + [vp] * 6,
            "orc_coo_to_csr": [i64, i64, vp, vp, vp, vp, vp, vp],
            "orc_assemble_laplace_coo": [i, i, i64, vp, vp, vp, vp, vp],
            "orc_assemble_rhs": [i, i, i64, vp, vp, d, vp],
            "orc_assemble_vec_coo": [i, vp, i, i64, vp, vp, vp, vp, vp, vp, vp],
            "orc_assemble_ns_coo": [i64, vp, vp, vp, vp, vp, d, d, i, i, vp, vp, vp, vp, vp],
            "orc_cpu_baseline_ns": [i64, vp, vp, vp, vp, vp, d, d, i64, i64],
            "orc_cpu_baseline_vec": [vp, i, i64, vp, vp, vp, i, i64],
            "orc_detF_range": [i, i64, vp, vp, vp, vp, vp],
            "orc_field_fourier": [u64, i, i, i64, vp, d, vp],
            "orc_field_uniform": [u64, i64, d, d, vp],
        }
        for name, args in sig.items():
            getattr(L, name).argtypes = args
        _LIB = L
    return _LIB


def p(a, t=D):
    """ctypes pointer to a C-contiguous array (any other layout would hand the
    C restatement the wrong element order)."""
    if a is None:
        return None
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("oracle arrays must be C-contiguous")
    return a.ctypes.data_as(C.c_void_p)


def quad(npts):
    pts = np.zeros((npts, 3)); w = np.zeros(npts)
    n = lib().orc_quad(npts, p(pts), p(w))
    assert n == npts
    return pts, w


def phi(fe, x):
    v = np.zeros(4 if fe == 1 else 10)
    lib().orc_phi(fe, p(np.ascontiguousarray(x, dtype=np.float64)), p(v))
    return v


def dphi(fe, x):
    v = np.zeros((4 if fe == 1 else 10, 3))
    lib().orc_dphi(fe, p(np.ascontiguousarray(x, dtype=np.float64)), p(v))
    return v


def mesh(M, fe, seed=0, amp=0.1, orient=True):
    """Structured unit-cube mesh in FEDDLib's numbering (buildMesh3D), interior
    P1 vertices jittered by (2u-1)*amp*h, P2 edge nodes at edge midpoints,
    elements oriented to det B > 0 (flipElement)."""
    nn = C.c_int64(); ne = C.c_int64()
    lib().orc_mesh_sizes(M, fe, C.cast(C.pointer(nn), C.c_void_p), C.cast(C.pointer(ne), C.c_void_p))
    npe = 4 if fe == 1 else 10
    xyz = np.zeros((nn.value, 3)); conn = np.zeros((ne.value, npe), dtype=np.int32)
    lib().orc_mesh_structured(M, fe, p(xyz), p(conn, I32))
    if amp:
        lib().orc_mesh_jitter(M, fe, C.c_uint64(seed), C.c_double(amp), p(xyz))
        if fe == 2:
            lib().orc_mesh_p2_midpoints(ne.value, p(conn, I32), p(xyz))
    nflip = 0
    if orient:
        nflip = lib().orc_mesh_orient(fe, ne.value, p(xyz), p(conn, I32))
    return xyz, conn, nflip


# local vertex pairs of a tetrahedron's edges in the order
# MeshPartitioner::setLocalEdgeIndices lists them (MeshPartitioner_def.hpp:
# 795-812), and the P2 position of each pair (determinePositionInElementP2,
# MeshUnstructured_def.hpp:690-736; the local ids are sorted first)
P2_EDGE_PAIRS = ((0, 1), (0, 2), (1, 2), (0, 3), (1, 3), (2, 3))
P2_EDGE_POS = {(0, 1): 4, (1, 2): 5, (0, 2): 6, (0, 3): 7, (1, 3): 8, (2, 3): 9}


def p2_of_p1(xyz1, tets):
    """P2 mesh of a P1 tetrahedral mesh as MeshUnstructured::buildP2ofP1MeshEdge
    builds it (feddlib/core/Mesh/MeshUnstructured_def.hpp:122-233): each
    element edge as its (min, max) vertex pair (MeshPartitioner::
    buildEdgeListParallel, MeshPartitioner_def.hpp:737-775), sorted and made
    unique with global id = rank (EdgeElements::sortUniqueAndSetGlobalIDs,
    EdgeElements.cpp:105-130); P2 nodes = the P1 nodes then node nn1 + id at
    the edge midpoint (:160-171, 215-226); the P2 element lists the P1 element
    then the edge nodes at their determinePositionInElementP2 slots (:186-199)."""
    xyz1 = np.asarray(xyz1, dtype=np.float64)
    tets = np.asarray(tets, dtype=np.int64)
    nn1, ne = xyz1.shape[0], tets.shape[0]
    a = tets[:, [pq[0] for pq in P2_EDGE_PAIRS]]
    b = tets[:, [pq[1] for pq in P2_EDGE_PAIRS]]
    key = np.minimum(a, b) * nn1 + np.maximum(a, b)
    uniq, inv = np.unique(key.ravel(), return_inverse=True)
    eid = inv.reshape(ne, 6)
    conn2 = np.zeros((ne, 10), dtype=np.int32)
    conn2[:, :4] = tets
    for k, pq in enumerate(P2_EDGE_PAIRS):
        conn2[:, P2_EDGE_POS[pq]] = nn1 + eid[:, k]
    lo, hi = uniq // nn1, uniq % nn1
    xyz2 = np.vstack([xyz1, 0.5 * (xyz1[lo] + xyz1[hi])])
    return xyz2, conn2


def geometry(xe):
    B = np.zeros(9); Bi = np.zeros(9)
    det = lib().orc_geometry(p(xe[0]), p(xe[1]), p(xe[2]), p(xe[3]), p(B), p(Bi))
    return det, B.reshape(3, 3), Bi.reshape(3, 3)


def elem_laplace(fe, npts, xe):
    n = 4 if fe == 1 else 10
    K = np.zeros((n, n))
    lib().orc_elem_laplace(fe, npts, p(np.ascontiguousarray(xe)), p(K))
    return K


def elem_ns(xe, u, pr, visc, dens, newton=True, coeff=(1, 1, 1, 1), parts=False):
    J = np.zeros((34, 34)); r = np.zeros(34)
    co = np.asarray(coeff, dtype=np.float64)
    if parts:
        A, N, W, B = (np.zeros((34, 34)) for _ in range(4))
    else:
        A = N = W = B = None
    lib().orc_elem_ns(p(np.ascontiguousarray(xe)), p(np.ascontiguousarray(u, dtype=np.float64)),
                      p(np.ascontiguousarray(pr, dtype=np.float64)), C.c_double(visc),
                      C.c_double(dens), int(newton), p(co), p(J), p(r), p(A), p(N), p(W), p(B))
    if parts:
        return J, r, A, N, W, B
    return J, r


GN_CARREAU_YASUDA, GN_POWER_LAW, GN_DIMLESS_CARREAU = 0, 1, 2


class ViscLaw(C.Structure):
    _fields_ = [("model", C.c_int), ("prm", C.c_double * 5), ("gamma_min", C.c_double)]


def visc_law(model, prm, gamma_min=1e-8):
    L = ViscLaw()
    L.model = model
    for k, v in enumerate(list(prm)[:5]):
        L.prm[k] = float(v)
    L.gamma_min = gamma_min
    return L


def gn_eta(L, gamma):
    f = lib().orc_gn_eta
    f.restype = C.c_double
    return f(C.byref(L), C.c_double(gamma))


def gn_dterm(L, gamma):
    f = lib().orc_gn_dterm
    f.restype = C.c_double
    return f(C.byref(L), C.c_double(gamma))


def elem_gn(xe, u, pr, L, dens, newton=True):
    """AssembleFEGeneralizedNewtonian element (no outflow Neumann term):
    34x34 Jacobian and residual."""
    J = np.zeros((34, 34)); r = np.zeros(34)
    lib().orc_elem_gn(p(np.ascontiguousarray(xe)), p(np.ascontiguousarray(u, dtype=np.float64)),
                      p(np.ascontiguousarray(pr, dtype=np.float64)), C.byref(L), C.c_double(dens), int(newton),
                      p(J), p(r))
    return J, r


def gn_outflow(xe, face, u, L):
    """Outflow Neumann boundary term of one generalized-Newtonian element with
    one flagged face (face: its 3 vertex coordinates, 3x3, in the face's node
    order): the 30x30 matrix that enters the Jacobian and the residual's
    operator."""
    K = np.zeros((30, 30))
    lib().orc_gn_outflow(p(np.ascontiguousarray(xe, dtype=np.float64)),
                         p(np.ascontiguousarray(face, dtype=np.float64)),
                         p(np.ascontiguousarray(u, dtype=np.float64)), C.byref(L), p(K))
    return K


def outflow_owners(conn, faces):
    """The element that holds each face (three vertex ids, any order) among
    its four vertex faces, and per element the face it takes: the last one
    listed (the reference's loop over an element's flagged sub-elements keeps
    the last one's surface data).  Returns (owner per face, {element: face})."""
    where = {}
    for e in range(conn.shape[0]):
        v = conn[e, :4]
        for f in ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)):
            where.setdefault(tuple(sorted(int(v[i]) for i in f)), []).append(e)
    owner = []
    taken = {}
    for k, f in enumerate(faces):
        es = where.get(tuple(sorted(int(x) for x in f)), [])
        if len(es) != 1:
            raise ValueError(f"face {k} belongs to {len(es)} elements, not to exactly one")
        owner.append(es[0])
        taken[es[0]] = k
    return np.array(owner), taken


def elem_linelas_classic(npts, xe, lam, mu):
    K = np.zeros((30, 30))
    lib().orc_elem_linelas_classic(npts, p(np.ascontiguousarray(xe)), C.c_double(lam),
                                   C.c_double(mu), p(K))
    return K


class LawSpec:
    """Holds a Law struct plus the numpy arrays it points into."""

    def __init__(self, law, mu=1.0, lam=10.0, k1=2.0, k2=1.0, angle_deg=40.0, mlp=None):
        self.s = Law()
        self.s.law = law; self.s.mu = mu; self.s.lam = lam; self.s.k1 = k1; self.s.k2 = k2
        a = math.radians(angle_deg)
        for i, v in enumerate((math.cos(a), math.sin(a), 0.0)):
            self.s.a1[i] = v
        for i, v in enumerate((math.cos(a), -math.sin(a), 0.0)):
            self.s.a2[i] = v
        self._keep = []
        if mlp is not None:
            self.set_mlp(mlp)

    def set_mlp(self, m):
        arrs = {k: np.ascontiguousarray(np.asarray(m[k], dtype=np.float64))
                for k in ("W1", "b1", "W2", "b2", "w3", "in_shift", "in_scale")}
        self._keep = list(arrs.values())
        self.s.hidden = int(arrs["b1"].shape[0])
        for k, v in arrs.items():
            setattr(self.s, k, v.ctypes.data_as(D))
        self.s.b3 = float(m["b3"]); self.s.out_scale = float(m.get("out_scale", 1.0))
        self.s.mlp_add_matrix = int(m.get("add_matrix", 1))
        self.s.in_clamp = int(m.get("in_clamp", 0))

    @property
    def ptr(self):
        return C.cast(C.pointer(self.s), C.c_void_p)


def law_from_E_nu(law, E, nu, **kw):
    """(mu, lambda) from E and nu as the AceGen kernels do (NeoHookQuadraticTets*.f);
    skr3 takes the bulk modulus kappa = E / (3 (1 - 2 nu)) in the lambda slot
    (NeoHookQuadraticTets3.f:25-31: 1 / (6 (1 - 2 nu)) times 2 E)."""
    mu = E / (2 * (1 + nu))
    lam = E / (3 * (1 - 2 * nu)) if law == LAW_SKR3 else nu * 2 * mu / (1 - 2 * nu)
    return LawSpec(law, mu=mu, lam=lam, **kw)


def law_PA(L, F):
    psi = C.c_double(); P = np.zeros(9); A = np.zeros(81)
    lib().orc_law_PA(L.ptr, p(np.ascontiguousarray(F, dtype=np.float64).ravel()), C.cast(C.pointer(psi), C.c_void_p),
                     p(P), p(A))
    return psi.value, P.reshape(3, 3), A.reshape(3, 3, 3, 3)


def law_dpsi(L, inv):
    psi = C.c_double(); d1 = np.zeros(4); d2 = np.zeros(16)
    lib().orc_law_dpsi(L.ptr, p(np.ascontiguousarray(inv, dtype=np.float64)), C.cast(C.pointer(psi), C.c_void_p),
                       p(d1), p(d2))
    return psi.value, d1, d2.reshape(4, 4)


def law_invariants(L, F):
    inv = np.zeros(4)
    lib().orc_law_invariants(L.ptr, p(np.ascontiguousarray(F, dtype=np.float64).ravel()), p(inv))
    return inv


def elem_hyper(L, npts, xe, u):
    K = np.zeros((30, 30)); r = np.zeros(30)
    uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
    lib().orc_elem_hyper(L.ptr, npts, p(np.ascontiguousarray(xe)), p(uu), p(K), p(r))
    return K, r


def coo_to_csr(nrows, rows, cols, vals):
    n = rows.shape[0]
    rowptr = np.zeros(nrows + 1, dtype=np.int64)
    colind = np.zeros(max(n, 1), dtype=np.int32)
    values = np.zeros(max(n, 1))
    nnz = lib().orc_coo_to_csr(nrows, n, p(rows, I64), p(cols, I64), p(vals), p(rowptr, I64),
                               p(colind, I32), p(values))
    return rowptr, colind[:nnz].copy(), values[:nnz].copy()


def assemble_laplace(fe, npts, xyz, conn):
    ne, n = conn.shape
    m = ne * n * n
    rows = np.zeros(m, dtype=np.int64); cols = np.zeros(m, dtype=np.int64); vals = np.zeros(m)
    lib().orc_assemble_laplace_coo(fe, npts, ne, p(xyz), p(conn, I32), p(rows, I64),
                                   p(cols, I64), p(vals))
    return coo_to_csr(xyz.shape[0], rows, cols, vals)


def assemble_rhs(fe, npts, xyz, conn, f=1.0):
    rhs = np.zeros(xyz.shape[0])
    lib().orc_assemble_rhs(fe, npts, conn.shape[0], p(xyz), p(conn, I32), C.c_double(f), p(rhs))
    return rhs


def rhs_points(npts, xyz, conn):
    """FE::assemblyRHS's physical quadrature points (FE_def.hpp:7355-7364):
    x_q = B xhat_q + x_0 with B = [x_1 - x_0, x_2 - x_0, x_3 - x_0];
    (num_elements, npts, 3)."""
    pts, _ = quad(npts)
    v = xyz[conn[:, :4]]                                  # (ne, 4, 3)
    B = np.transpose(v[:, 1:] - v[:, :1], (0, 2, 1))      # B[e][j][k] = (x_{k+1} - x_0)_j
    return np.einsum("ejk,qk->eqj", B, pts) + v[:, :1]


def assemble_rhs_func(fe, npts, xyz, conn, f, ncomp=1):
    """FE::assemblyRHS (FE_def.hpp:7303-7400) with a source function, in
    FP64: b[ncomp node(a) + c] += |det B| sum_q w_q phi_a(q) f_c(x_q), f
    taking one point and returning ncomp values."""
    pts, w = quad(npts)
    ph = np.array([phi(fe, x) for x in pts])              # (nq, npe)
    xq = rhs_points(npts, xyz, conn)
    out = np.zeros(xyz.shape[0] * ncomp)
    for e in range(conn.shape[0]):
        v = xyz[conn[e, :4]]
        det = np.linalg.det((v[1:] - v[0]).T)
        fv = np.array([np.atleast_1d(f(x)) for x in xq[e]]).reshape(npts, ncomp)
        val = np.einsum("q,qa,qc->ac", w, ph, fv) * abs(det)
        for a in range(conn.shape[1]):
            out[ncomp * conn[e, a]:ncomp * conn[e, a] + ncomp] += val[a]
    return out


def assemble_vec(kind, L, npts, xyz, conn, u=None, want_matrix=True):
    ne = conn.shape[0]
    m = ne * 900 if want_matrix else 0
    rows = np.zeros(max(m, 1), dtype=np.int64); cols = np.zeros(max(m, 1), dtype=np.int64)
    vals = np.zeros(max(m, 1))
    res = np.zeros(3 * xyz.shape[0]) if kind == 1 else None
    uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64).ravel()
    lib().orc_assemble_vec_coo(kind, L.ptr, npts, ne, p(xyz), p(conn, I32), p(uu),
                               p(rows, I64) if want_matrix else None,
                               p(cols, I64) if want_matrix else None,
                               p(vals) if want_matrix else None, p(res))
    csr = coo_to_csr(3 * xyz.shape[0], rows[:m], cols[:m], vals[:m]) if want_matrix else None
    return csr, res


def assemble_ns(xyz2, conn2, conn1, n1, u, pr, visc, dens, newton=True, blocks=(0, 1, 2, 3)):
    """Returns {block: (rowptr, colind, values)} and (res_u, res_p)."""
    ne = conn2.shape[0]
    n2 = xyz2.shape[0]
    out = {}
    res_u = np.zeros(3 * n2); res_p = np.zeros(n1)
    sizes = {0: 900, 1: 120, 2: 120, 3: 16}
    nrows = {0: 3 * n2, 1: 3 * n2, 2: n1, 3: n1}
    uu = np.ascontiguousarray(u, dtype=np.float64).ravel()
    pp = np.ascontiguousarray(pr, dtype=np.float64)
    first = True
    for b in blocks:
        m = ne * sizes[b]
        rows = np.zeros(m, dtype=np.int64); cols = np.zeros(m, dtype=np.int64); vals = np.zeros(m)
        c = lib().orc_assemble_ns_coo(ne, p(xyz2), p(conn2, I32), p(conn1, I32), p(uu), p(pp),
                                      C.c_double(visc), C.c_double(dens), int(newton), b,
                                      p(rows, I64), p(cols, I64), p(vals),
                                      p(res_u) if first else None, p(res_p) if first else None)
        first = False
        out[b] = coo_to_csr(nrows[b], rows[:c], cols[:c], vals[:c])
    return out, (res_u, res_p)


def mlp_eval(m, x):
    y = C.c_double(); g = np.zeros(4); h = np.zeros(16)
    a = {k: np.ascontiguousarray(np.asarray(m[k], dtype=np.float64)) for k in ("W1", "b1", "W2", "b2", "w3")}
    H = a["b1"].shape[0]
    lib().orc_mlp_eval(H, p(a["W1"]), p(a["b1"]), p(a["W2"]), p(a["b2"]), p(a["w3"]),
                       C.c_double(float(m["b3"])), p(np.ascontiguousarray(x, dtype=np.float64)),
                       C.cast(C.pointer(y), C.c_void_p), p(g), p(h))
    return y.value, g, h.reshape(4, 4)


def mlp_loss(m, X, tpsi, tgrad, wpsi, wgrad, grads=True):
    a = {k: np.ascontiguousarray(np.asarray(m[k], dtype=np.float64)) for k in ("W1", "b1", "W2", "b2", "w3")}
    H = a["b1"].shape[0]
    g = {k: np.zeros_like(v) for k, v in a.items()} if grads else None
    gb3 = C.c_double()
    X = np.ascontiguousarray(X, dtype=np.float64)
    loss = lib().orc_mlp_loss(H, p(a["W1"]), p(a["b1"]), p(a["W2"]), p(a["b2"]), p(a["w3"]),
                              C.c_double(float(m["b3"])), X.shape[0], p(X),
                              p(np.ascontiguousarray(tpsi, dtype=np.float64)),
                              p(np.ascontiguousarray(tgrad, dtype=np.float64)),
                              C.c_double(wpsi), C.c_double(wgrad),
                              p(g["W1"]) if grads else None, p(g["b1"]) if grads else None,
                              p(g["W2"]) if grads else None, p(g["b2"]) if grads else None,
                              p(g["w3"]) if grads else None, C.cast(C.pointer(gb3), C.c_void_p) if grads else None)
    if grads:
        g["b3"] = gb3.value
        return loss, g
    return loss


def field_fourier(xyz, seed, kmin=1, kmax=4, scale=1.0):
    u = np.zeros(3 * xyz.shape[0])
    lib().orc_field_fourier(C.c_uint64(seed), kmin, kmax, xyz.shape[0], p(np.ascontiguousarray(xyz)),
                            C.c_double(scale), p(u))
    return u


def field_uniform(seed, n, lo=-1.0, hi=1.0):
    v = np.zeros(n)
    lib().orc_field_uniform(C.c_uint64(seed), n, C.c_double(lo), C.c_double(hi), p(v))
    return v


def cpu_baseline_ns(xyz2, conn2, conn1, u, pr, visc, dens, n1):
    """Reference-shaped single-thread Navier-Stokes Jacobian + residual over
    the given elements (per-element table rebuild, heap element matrices,
    row-wise inserts, sort + merge); returns a checksum."""
    c2 = np.ascontiguousarray(conn2, dtype=np.int32); c1 = np.ascontiguousarray(conn1, dtype=np.int32)
    return lib().orc_cpu_baseline_ns(c2.shape[0], p(xyz2), p(c2), p(c1), p(np.ascontiguousarray(u)),
                                     p(np.ascontiguousarray(pr)), C.c_double(visc), C.c_double(dens),
                                     3 * xyz2.shape[0], n1)


def cpu_baseline_vec(L, npts, xyz, conn, u, want_res):
    """Reference-shaped single-thread elasticity Jacobian (+ residual: a
    second kernel call per element, as AssembleFE_NonLinElas does) over the
    given elements, with row-wise inserts and sort + merge; returns a
    checksum."""
    c = np.ascontiguousarray(conn, dtype=np.int32)
    uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64).ravel()
    return lib().orc_cpu_baseline_vec(L.ptr, npts, c.shape[0], p(xyz), p(c), p(uu), int(want_res),
                                      3 * xyz.shape[0])


def detF_range(npts, xyz, conn, u):
    """(min, max) of det F over the quadrature points of the given elements."""
    c = np.ascontiguousarray(conn, dtype=np.int32)
    lo, hi = C.c_double(), C.c_double()
    lib().orc_detF_range(npts, c.shape[0], p(xyz), p(c), p(np.ascontiguousarray(u, dtype=np.float64).ravel()),
                         C.cast(C.pointer(lo), C.c_void_p), C.cast(C.pointer(hi), C.c_void_p))
    return lo.value, hi.value


# ---------------------------------------------------------------- Dirichlet --
def dirichlet_rows(rowptr, colind, vals, mask, diagonal_block):
    """BCBuilder::setDirichletBC with setLocalRowOne / setLocalRowZero
    (feddlib/core/General/BCBuilder_def.hpp:620-700) on one CSR block: the rows
    of Dirichlet dofs become zero; in a diagonal block the entry in the
    diagonal column becomes one (a row without that entry stays zero, as
    setLocalRowOne then finds nothing to set)."""
    out = np.array(vals, dtype=np.float64, copy=True)
    for r in np.nonzero(np.asarray(mask))[0]:
        lo, hi = int(rowptr[r]), int(rowptr[r + 1])
        out[lo:hi] = 0.0
        if diagonal_block:
            hit = np.nonzero(np.asarray(colind[lo:hi]) == r)[0]
            if hit.size:
                out[lo + hit[0]] = 1.0
    return out


def dirichlet_rhs(res, mask, g=None, sub=None):
    """BCBuilder::setRHS (BCBuilder_def.hpp:93-200; sub None) and
    setBCMinusVector (:232-350): at Dirichlet dofs the entry becomes the
    boundary value g (zero when None) minus sub; other entries keep their value."""
    out = np.array(res, dtype=np.float64, copy=True)
    m = np.asarray(mask) != 0
    gv = np.zeros_like(out) if g is None else np.asarray(g, dtype=np.float64)
    sv = np.zeros_like(out) if sub is None else np.asarray(sub, dtype=np.float64)
    out[m] = gv[m] - sv[m]
    return out
