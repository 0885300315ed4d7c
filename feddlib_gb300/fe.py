"""Python side of the engine: the C ABI handle and an FE facade shaped like
FEDDLib's FE::assembly* drivers (feddlib/core/FE/FE_decl.hpp).

Parameters follow FEDDLib's ParameterList keys as nested dicts:
    {"Parameter": {"Viscosity": 0.01, "Density": 1.0, "E": 1000.0,
                   "Poisson Ratio": 0.3},
     "General": {"Linearization": "Newton"}}
Matrices come back as CsrMatrix (Tpetra layout: int64 row offsets, int32
columns sorted per row, float64 values, node-wise dofs).
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _capi as A


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


@dataclass
class CsrMatrix:
    rowptr: np.ndarray
    colind: np.ndarray
    values: np.ndarray
    shape: tuple

    @property
    def nnz(self):
        return int(self.rowptr[-1])

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.values, self.colind, self.rowptr), shape=self.shape)


# ---------------------------------------------------------------- inputs ----
def structured_mesh(M, fe_order, seed=0, amp=0.1):
    """FEDDLib's buildMesh3D unit cube (M^3 hexes x 6 tets), jittered and
    oriented; returns (coords [n,3] float64, elements [ne, 4|10] int32)."""
    L = A.lib()
    nn, ne = C.c_int64(), C.c_int64()
    A.check(L.fedd_mesh_sizes(M, fe_order, C.byref(nn), C.byref(ne)))
    xyz = np.zeros((nn.value, 3))
    conn = np.zeros((ne.value, 4 if fe_order == 1 else 10), dtype=np.int32)
    A.check(L.fedd_mesh_structured(M, fe_order, seed, amp, _p(xyz), _p(conn)))
    return xyz, conn


def _is_cuda(x):
    return getattr(x, "is_cuda", False)


def structured_mesh_device(M, fe_order, seed=0, amp=0.1, device=0):
    """structured_mesh made on the device: (coords, elements) as CUDA tensors
    (float64 [n, 3], int32 [ne, 4|10]), bit-identical to structured_mesh."""
    import torch
    L = A.lib()
    nn, ne = C.c_int64(), C.c_int64()
    A.check(L.fedd_mesh_sizes(M, fe_order, C.byref(nn), C.byref(ne)))
    dev = torch.device("cuda", device)
    xyz = torch.empty((nn.value, 3), dtype=torch.float64, device=dev)
    conn = torch.empty((ne.value, 4 if fe_order == 1 else 10), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    A.check(L.fedd_mesh_structured_device(M, fe_order, seed, amp, xyz.data_ptr(), conn.data_ptr(), stream))
    return xyz, conn


def p2_of_p1(coords, elements, device=0):
    """P2 mesh of a P1 tetrahedral mesh (buildP2ofP1MeshEdge), built on the
    device: host arrays in -> host arrays out, CUDA tensors in -> CUDA tensors
    out.  Returns (coords2 [n2, 3], elements2 [ne, 10])."""
    L = A.lib()
    ne, nn1 = elements.shape[0], coords.shape[0]
    h, nn2 = C.c_void_p(), C.c_int64()
    if _is_cuda(coords):
        import torch
        c1, e1 = coords.contiguous(), elements.contiguous()
        A.check(L.fedd_p2_of_p1(nn1, ne, c1.data_ptr(), e1.data_ptr(), A.MESH_DEVICE, device, C.byref(h),
                                C.byref(nn2)))
        try:
            xyz = torch.empty((nn2.value, 3), dtype=torch.float64, device=coords.device)
            conn = torch.empty((ne, 10), dtype=torch.int32, device=coords.device)
            A.check(L.fedd_p2_copy(h, xyz.data_ptr(), conn.data_ptr(), A.MESH_DEVICE))
        finally:
            L.fedd_p2_destroy(h)
        return xyz, conn
    c1 = np.ascontiguousarray(coords, dtype=np.float64)
    e1 = np.ascontiguousarray(elements, dtype=np.int32)
    A.check(L.fedd_p2_of_p1(nn1, ne, _p(c1), _p(e1), 0, device, C.byref(h), C.byref(nn2)))
    try:
        xyz = np.zeros((nn2.value, 3))
        conn = np.zeros((ne, 10), dtype=np.int32)
        A.check(L.fedd_p2_copy(h, _p(xyz), _p(conn), 0))
    finally:
        L.fedd_p2_destroy(h)
    return xyz, conn


def medit_read(path):
    """A medit (.mesh) file as FEDDLib reads it: dict with coords [n, 3],
    node_flags, tets [nt, 4] (zero-based), tet_flags, tris [ntri, 3], tri_flags."""
    L = A.lib()
    nn, nt, ntri = C.c_int64(), C.c_int64(), C.c_int64()
    A.check(L.fedd_medit_sizes(str(path).encode(), C.byref(nn), C.byref(nt), C.byref(ntri)))
    out = dict(coords=np.zeros((nn.value, 3)), node_flags=np.zeros(nn.value, dtype=np.int32),
               tets=np.zeros((nt.value, 4), dtype=np.int32), tet_flags=np.zeros(nt.value, dtype=np.int32),
               tris=np.zeros((ntri.value, 3), dtype=np.int32), tri_flags=np.zeros(ntri.value, dtype=np.int32))
    A.check(L.fedd_medit_read(str(path).encode(), _p(out["coords"]), _p(out["node_flags"]), _p(out["tets"]),
                              _p(out["tet_flags"]), _p(out["tris"]), _p(out["tri_flags"])))
    return out


def medit_write(path, coords, tets, node_flags=None, tet_flags=None, tris=None, tri_flags=None):
    """Writes a medit (.mesh) file (ids zero-based in, one-based on disk)."""
    c = np.ascontiguousarray(coords, dtype=np.float64)
    t = np.ascontiguousarray(tets, dtype=np.int32)
    nf = None if node_flags is None else np.ascontiguousarray(node_flags, dtype=np.int32)
    tf = None if tet_flags is None else np.ascontiguousarray(tet_flags, dtype=np.int32)
    tr = None if tris is None else np.ascontiguousarray(tris, dtype=np.int32)
    trf = None if tri_flags is None else np.ascontiguousarray(tri_flags, dtype=np.int32)
    A.check(A.lib().fedd_medit_write(str(path).encode(), c.shape[0], _p(c), _p(nf), t.shape[0], _p(t), _p(tf),
                                     0 if tr is None else tr.shape[0], _p(tr), _p(trf)))


def fourier_field(coords, seed, kmin=1, kmax=4, scale=1.0):
    u = np.zeros(coords.shape[0] * 3)
    A.check(A.lib().fedd_field_fourier(seed, kmin, kmax, coords.shape[0],
                                       _p(np.ascontiguousarray(coords)), scale, _p(u)))
    return u


def uniform_field(seed, n, lo=-1.0, hi=1.0):
    v = np.zeros(n)
    A.check(A.lib().fedd_field_uniform(seed, n, lo, hi, _p(v)))
    return v


def detF_scaled_field(asm, coords, seed, lo_j=0.7, hi_j=1.4, iters=24, kmin=1, kmax=2):
    """The seeded smooth displacement field (8 Fourier modes, kmin <= k <=
    kmax) at the largest amplitude s for which det F stays in [lo_j, hi_j]
    at every quadrature point of `asm`'s mesh: bisection on the engine's own
    quadrature-point invariants.  Returns (u, s, (min det F, max det F))."""
    base = fourier_field(coords, seed=seed, kmin=kmin, kmax=kmax, scale=1.0)

    def jr(s):
        J = asm.qp_invariants(base * s)[..., 1]
        return float(J.min()), float(J.max())

    lo, hi = 0.0, 1e-3
    while True:
        jmin, jmax = jr(hi)
        if jmin < lo_j or jmax > hi_j:
            break
        lo, hi = hi, 2 * hi
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        jmin, jmax = jr(mid)
        if jmin < lo_j or jmax > hi_j:
            hi = mid
        else:
            lo = mid
    return base * lo, lo, jr(lo)


# ------------------------------------------------------------- assembler ----
class Assembler:
    """One mesh + problem on one GPU (a fedd_assembler handle)."""

    def __init__(self, problem, coords, elements, fe_order=2, elements_p=None, num_nodes_p=0,
                 viscosity=1.0, density=1.0, E=1000.0, poisson_ratio=0.3, newton=True,
                 quad_points=0, surrogate=False, k1=2.0, k2=1.0, fiber_angle_deg=40.0,
                 source=1.0, device=0, fixed_point_matrix=False):
        """newton: FEDDLib's Linearization Newton (True) or FixedPoint;
        fixed_point_matrix (with newton False): the matrix of
        FE::assemblyNavierStokes' assembleMode "FixedPoint", which for a
        generalized-Newtonian fluid also holds the outflow term."""
        m = A.Mesh()
        m.num_nodes = coords.shape[0]
        m.num_elements = elements.shape[0]
        m.fe_order = fe_order
        m.num_nodes_p = num_nodes_p
        if _is_cuda(coords):
            # a device-resident mesh (CUDA tensors): the handle copies and
            # transposes it on the device
            self._keep = (coords.contiguous(), elements.contiguous(),
                          None if elements_p is None else elements_p.contiguous())
            m.flags = A.MESH_DEVICE
            m.coords, m.elements = self._keep[0].data_ptr(), self._keep[1].data_ptr()
            m.elements_p = None if elements_p is None else self._keep[2].data_ptr()
        else:
            self._keep = (np.ascontiguousarray(coords, dtype=np.float64),
                          np.ascontiguousarray(elements, dtype=np.int32),
                          None if elements_p is None else np.ascontiguousarray(elements_p, dtype=np.int32))
            m.coords = self._keep[0].ctypes.data
            m.elements = self._keep[1].ctypes.data
            m.elements_p = None if elements_p is None else self._keep[2].ctypes.data
        p = A.Params()
        p.problem = problem
        p.linearization = 1 if newton else (2 if fixed_point_matrix else 0)
        p.quad_points = quad_points
        p.surrogate = 1 if surrogate else 0
        p.viscosity, p.density, p.E, p.poisson_ratio = viscosity, density, E, poisson_ratio
        p.k1, p.k2, p.fiber_angle_deg, p.source = k1, k2, fiber_angle_deg, source
        self.problem = problem
        # quadrature points per element of the elasticity laws (the engine's
        # default rule: skr2 5 points, skr1 and the fibre law 4)
        self.nq = quad_points or (5 if problem in (A.NONLINEAR_ELASTICITY, A.NONLINEAR_ELASTICITY2) else 4)
        self.h = C.c_void_p()
        st = A.lib().fedd_create(C.byref(m), C.byref(p), device, C.byref(self.h))
        if st != A.OK:
            h, self.h = self.h, C.c_void_p()
            try:
                A.check(st, h)
            finally:
                if h:
                    A.lib().fedd_destroy(h)
        self.nblocks = 3 if problem == A.NAVIER_STOKES else 1
        nu, np_ = C.c_int64(), C.c_int64()
        A.check(A.lib().fedd_residual_sizes(self.h, C.byref(nu), C.byref(np_)), self.h)
        self.n_u, self.n_p = nu.value, np_.value

    def close(self):
        if self.h:
            A.lib().fedd_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def block_info(self, block=0):
        r, c, n = C.c_int64(), C.c_int64(), C.c_int64()
        A.check(A.lib().fedd_block_info(self.h, block, C.byref(r), C.byref(c), C.byref(n)), self.h)
        return r.value, c.value, n.value

    def pattern(self, block=0):
        nr, nc, nnz = self.block_info(block)
        rp = np.zeros(nr + 1, dtype=np.int64)
        ci = np.zeros(max(nnz, 1), dtype=np.int32)
        A.check(A.lib().fedd_get_pattern(self.h, block, _p(rp), _p(ci)), self.h)
        return rp, ci[:nnz], (nr, nc)

    def device_pattern(self, block=0):
        rp, ci = C.c_void_p(), C.c_void_p()
        A.check(A.lib().fedd_device_pattern(self.h, block, C.byref(rp), C.byref(ci)), self.h)
        return rp.value, ci.value

    def assemble(self, u=None, p=None, jacobian=True, residual=True, stream=None):
        """Host-buffer path: returns (list of value arrays per block, res_u, res_p)."""
        what = (A.JACOBIAN if jacobian else 0) | (A.RESIDUAL if residual else 0)
        vals = [np.zeros(max(self.block_info(b)[2], 1)) if jacobian else None for b in range(self.nblocks)]
        while len(vals) < 3:
            vals.append(None)
        ru = np.zeros(self.n_u) if residual else None
        rp = np.zeros(self.n_p) if (residual and self.n_p) else None
        uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        pp = None if p is None else np.ascontiguousarray(p, dtype=np.float64)
        A.check(A.lib().fedd_assemble(self.h, what, _p(uu), _p(pp), _p(vals[0]), _p(vals[1]), _p(vals[2]),
                                      _p(ru), _p(rp), stream), self.h)
        out = []
        for b in range(self.nblocks):
            out.append(None if vals[b] is None else vals[b][:self.block_info(b)[2]])
        return out, ru, rp

    def assemble_device(self, d_u, d_p, d_vals, d_res_u, d_res_p, jacobian=True, residual=True, stream=None):
        """Device path: arguments are raw device pointers (ints) or None."""
        what = (A.JACOBIAN if jacobian else 0) | (A.RESIDUAL if residual else 0)
        v = list(d_vals) + [None] * (3 - len(d_vals))
        A.check(A.lib().fedd_assemble_device(self.h, what, d_u, d_p, v[0], v[1], v[2], d_res_u, d_res_p,
                                             stream), self.h)

    CARREAU_YASUDA, POWER_LAW, DIMLESS_CARREAU = 0, 1, 2

    def set_viscosity_law(self, model, prm=(0.0,) * 5, gamma_min=1e-8):
        """Generalized-Newtonian fluid (FEDDLib's AssembleFEGeneralizedNewtonian):
        model 0 Carreau-Yasuda (lambda, n, eta0, etaInf, a), 1 Power-Law
        (K, n, eta_max, eta_min), 2 Dimless-Carreau (lambda, n, eta0, etaInf,
        reference viscosity); model < 0 restores the Newtonian fluid."""
        arr = np.zeros(5)
        arr[:len(prm)] = np.asarray(prm, dtype=np.float64)
        A.check(A.lib().fedd_set_viscosity_law(self.h, int(model), _p(arr), float(gamma_min)), self.h)

    def rhs_points(self):
        """The physical quadrature points of FE::assemblyRHS's rule, element-
        major: (num_elements, nq, 3)."""
        nq = C.c_int32()
        A.check(A.lib().fedd_rhs_points(self.h, None, C.byref(nq)), self.h)
        x = np.zeros((self._keep[1].shape[0], nq.value, 3))
        A.check(A.lib().fedd_rhs_points(self.h, _p(x), C.byref(nq)), self.h)
        return x

    def assemble_rhs(self, f, ncomp=1):
        """FE::assemblyRHS's load vector from a source function f(xq) (xq of
        shape (n, 3); n values for ncomp 1, (n, 3) for ncomp 3), or from its
        values at rhs_points() given as an array."""
        xq = self.rhs_points()
        ne, nq = xq.shape[:2]
        fq = np.asarray(f(xq.reshape(-1, 3)) if callable(f) else f, dtype=np.float64)
        fq = np.ascontiguousarray(fq.reshape(ne, nq, ncomp))
        out = np.zeros(self._keep[0].shape[0] * ncomp)
        A.check(A.lib().fedd_assemble_rhs(self.h, _p(fq), ncomp, _p(out)), self.h)
        return out

    def set_element_moduli(self, E):
        """A Young's modulus per element (the E-field variant of
        FE::assemblyNonLinearElasticity); None returns to the handle's E."""
        if E is None:
            A.check(A.lib().fedd_set_element_moduli(self.h, None), self.h)
            return
        e = np.ascontiguousarray(E, dtype=np.float64)
        if e.shape != (self._keep[1].shape[0],):
            raise ValueError("one modulus per element")
        A.check(A.lib().fedd_set_element_moduli(self.h, _p(e)), self.h)

    def set_coeff(self, coeff):
        """FE::assemblyNavierStokes' coeff (AssembleFENavierStokes::setCoeff):
        the 2x2 block factors [[c_uu, c_up], [c_pu, c_pp]] of the residual;
        the matrices are not scaled."""
        c = np.ascontiguousarray(np.asarray(coeff, dtype=np.float64).reshape(4))
        A.check(A.lib().fedd_set_coeff(self.h, _p(c)), self.h)

    def set_outflow_faces(self, faces):
        """Faces flagged for the generalized-Newtonian outflow Neumann term
        (FEDDLib's boundary sub-elements with the outflow flag): n x 3 vertex
        node ids in the face's own order (it sets the normal's sign); an empty
        list clears.  The term enters the velocity residual while a viscosity
        law is set."""
        f = np.ascontiguousarray(np.asarray(faces, dtype=np.int32).reshape(-1, 3))
        A.check(A.lib().fedd_set_outflow_faces(self.h, _p(f) if f.size else None, f.shape[0]), self.h)

    def set_dirichlet(self, mask_u, mask_p=None):
        """Dirichlet dofs (nonzero mask entries) of block rows 0 and 1; the
        BC flags of FEDDLib's BCBuilder resolved to dofs."""
        mu = np.ascontiguousarray(np.asarray(mask_u) != 0, dtype=np.uint8)
        mp = None if mask_p is None else np.ascontiguousarray(np.asarray(mask_p) != 0, dtype=np.uint8)
        A.check(A.lib().fedd_dirichlet_set(self.h, _p(mu), _p(mp)), self.h)

    def dirichlet_system_device(self, d_vals, stream=None):
        """BCBuilder::setSystem on device CSR values (pointers of the blocks)."""
        v = list(d_vals) + [None] * (3 - len(d_vals))
        A.check(A.lib().fedd_dirichlet_system(self.h, v[0], v[1], v[2], stream), self.h)

    def dirichlet_rhs_device(self, d_res_u, d_res_p=None, d_g_u=None, d_g_p=None, d_sub_u=None, d_sub_p=None,
                             stream=None):
        """BCBuilder::setRHS (sub None) / setBCMinusVector on device vectors."""
        A.check(A.lib().fedd_dirichlet_rhs(self.h, d_g_u, d_g_p, d_sub_u, d_sub_p, d_res_u, d_res_p, stream), self.h)

    def check(self, stream=None):
        A.check(A.lib().fedd_check(self.h, stream), self.h)

    def launch_count(self):
        n = C.c_int64()
        A.check(A.lib().fedd_launch_count(self.h, C.byref(n)), self.h)
        return n.value

    def set_profiling(self, on=True):
        A.check(A.lib().fedd_set_profiling(self.h, 1 if on else 0), self.h)

    def stage_times(self):
        """{stage name: (total ms, calls)} over the calls since profiling began."""
        ms = (C.c_double * 8)()
        ns, calls = C.c_int(), C.c_int64()
        A.check(A.lib().fedd_stage_times(self.h, 8, ms, C.byref(ns), C.byref(calls)), self.h)
        return {A.lib().fedd_stage_name(self.h, k).decode(): (ms[k], calls.value) for k in range(ns.value)}

    def element_matrices(self, u=None, p=None, first=0, count=None, nd=None):
        ne = self._keep[1].shape[0]
        count = ne - first if count is None else count
        if nd is None:
            nd = {A.LAPLACE: self._keep[1].shape[1], A.NAVIER_STOKES: 34}.get(self.problem, 30)
        K = np.zeros((count, nd, nd)); r = np.zeros((count, nd))
        uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        pp = None if p is None else np.ascontiguousarray(p, dtype=np.float64)
        A.check(A.lib().fedd_element_matrices(self.h, _p(uu), _p(pp), first, count, _p(K), _p(r)), self.h)
        return K, r

    def set_surrogate(self, m, inv_lo=(-1e30,) * 4, inv_hi=(1e30,) * 4):
        d = A.MLPDesc()
        arrs = {k: np.ascontiguousarray(np.asarray(m[k], dtype=np.float32)) for k in ("W1", "b1", "W2", "b2", "w3")}
        self._mlp_keep = arrs
        d.hidden = arrs["b1"].shape[0]
        for k, v in arrs.items():
            setattr(d, k, v.ctypes.data)
        d.b3 = float(m["b3"]); d.out_scale = float(m.get("out_scale", 1.0))
        d.in_clamp = int(m.get("in_clamp", 0))
        for k in range(4):
            d.in_shift[k] = float(m["in_shift"][k]); d.in_scale[k] = float(m["in_scale"][k])
            d.inv_lo[k] = float(inv_lo[k]); d.inv_hi[k] = float(inv_hi[k])
        A.check(A.lib().fedd_set_surrogate(self.h, C.byref(d)), self.h)

    def surrogate_fallbacks(self):
        c, t = C.c_int64(), C.c_int64()
        A.check(A.lib().fedd_surrogate_fallbacks(self.h, C.byref(c), C.byref(t)), self.h)
        return c.value, t.value

    def qp_invariants(self, u):
        """(num_elements, quadrature points, 4) float32 invariants
        (I1, J, I4a, I4b) at the quadrature points for displacement u."""
        ne = self._keep[1].shape[0]
        out = np.zeros((ne, self.nq, 4), dtype=np.float32)
        A.check(A.lib().fedd_qp_invariants(self.h, _p(np.ascontiguousarray(u, dtype=np.float64)), _p(out)), self.h)
        return out

    def element_geometry(self, first=0, count=None):
        """(det B (count,), B^-1 (count, 3, 3) float32) of elements
        [first, first + count) as the element kernels form them."""
        ne = self._keep[1].shape[0]
        count = ne - first if count is None else count
        det = np.zeros(count)
        binv = np.zeros((count, 3, 3), dtype=np.float32)
        A.check(A.lib().fedd_element_geometry(self.h, first, count, _p(det), _p(binv)), self.h)
        return det, binv

    def law_eval(self, F):
        F = np.ascontiguousarray(F, dtype=np.float64).reshape(-1, 9)
        n = F.shape[0]
        psi = np.zeros(n); P = np.zeros((n, 9)); Am = np.zeros((n, 81))
        A.check(A.lib().fedd_law_eval(self.h, n, _p(F), _p(psi), _p(P), _p(Am)), self.h)
        return psi, P.reshape(n, 3, 3), Am.reshape(n, 3, 3, 3, 3)


# ------------------------------------------------------------- trainer ------
class Trainer:
    """Surrogate training on the device (forward, Sobolev-loss backward, Adam)."""

    def __init__(self, hidden, x, tpsi, tgrad, device=0):
        self._keep = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, tpsi, tgrad)]
        self.H = hidden
        self.h = C.c_void_p()
        A.check(A.lib().fedd_trainer_create(hidden, self._keep[0].shape[0], _p(self._keep[0]),
                                            _p(self._keep[1]), _p(self._keep[2]), device, C.byref(self.h)))

    def close(self):
        if self.h:
            A.lib().fedd_trainer_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, m):
        a = {k: np.ascontiguousarray(np.asarray(m[k], dtype=np.float32)) for k in ("W1", "b1", "W2", "b2", "w3")}
        A.check(A.lib().fedd_trainer_set_params(self.h, _p(a["W1"]), _p(a["b1"]), _p(a["W2"]), _p(a["b2"]),
                                                _p(a["w3"]), float(m["b3"])))

    def get_params(self):
        H = self.H
        m = {"W1": np.zeros((H, 4), np.float32), "b1": np.zeros(H, np.float32), "W2": np.zeros((H, H), np.float32),
             "b2": np.zeros(H, np.float32), "w3": np.zeros(H, np.float32)}
        b3 = C.c_float()
        A.check(A.lib().fedd_trainer_get_params(self.h, _p(m["W1"]), _p(m["b1"]), _p(m["W2"]), _p(m["b2"]),
                                                _p(m["w3"]), C.byref(b3)))
        m["b3"] = b3.value
        return m

    def run(self, steps, batch, lr, wpsi=1.0, wgrad=1.0, seed=0):
        loss = C.c_float()
        A.check(A.lib().fedd_trainer_run(self.h, steps, batch, lr, wpsi, wgrad, seed, C.byref(loss)))
        return loss.value

    def grad(self, wpsi=1.0, wgrad=1.0):
        H = self.H
        g = {"W1": np.zeros((H, 4), np.float32), "b1": np.zeros(H, np.float32), "W2": np.zeros((H, H), np.float32),
             "b2": np.zeros(H, np.float32), "w3": np.zeros(H, np.float32)}
        loss, gb3 = C.c_float(), C.c_float()
        A.check(A.lib().fedd_trainer_grad(self.h, wpsi, wgrad, C.byref(loss), _p(g["W1"]), _p(g["b1"]),
                                          _p(g["W2"]), _p(g["b2"]), _p(g["w3"]), C.byref(gb3)))
        g["b3"] = gb3.value
        return loss.value, g


# ------------------------------------------------------ FEDDLib-shaped FE ----
def _param(params, sub, key, default):
    return (params or {}).get(sub, {}).get(key, default)


class FE:
    """FE::assembly* with plain CSR outputs.  `domain` is (coords, elements)
    of the velocity/displacement/scalar mesh; `domain_p` the P1 pressure mesh
    for Navier-Stokes.  One engine handle per (problem, parameters) is cached,
    like FEDDLib's assemblyFEElements_."""

    def __init__(self, domain, domain_p=None, device=0):
        self.coords, self.elements = domain
        self.domain_p = domain_p
        self.device = device
        self._asm = {}

    def _get(self, key, **kw):
        if key not in self._asm:
            self._asm[key] = Assembler(coords=self.coords, elements=self.elements, device=self.device, **kw)
        return self._asm[key]

    @staticmethod
    def _order(FEType):
        if FEType not in ("P1", "P2"):
            raise ValueError(f"FEType {FEType!r} not supported (P1, P2)")
        return 1 if FEType == "P1" else 2

    def assemblyLaplace(self, dim, FEType, degree, callFillComplete=True):
        """FE::assemblyLaplace (FE_def.hpp:2437-2500)."""
        if dim != 3:
            raise ValueError("dim must be 3")
        a = self._get(("Laplace", FEType), problem=A.LAPLACE, fe_order=self._order(FEType))
        (v,), _, _ = a.assemble(jacobian=True, residual=False)
        rp, ci, shape = a.pattern(0)
        return CsrMatrix(rp, ci, v, shape)

    def assemblyLaplaceAssFE(self, dim, FEType, degree, dofs=1, callFillComplete=True):
        """FE::assemblyLaplaceAssFE (FE_def.hpp:1818-1853): the stiffness of
        assemblyLaplace through FEDDLib's AssembleFE_Laplace elements.  Both
        rules integrate the gradient products exactly and the engine forms
        them in closed form, so the values are assemblyLaplace's."""
        if dofs != 1:
            raise ValueError("scalar Laplace: dofs = 1")
        return self.assemblyLaplace(dim, FEType, degree, callFillComplete)

    def assemblyRHS(self, dim, FEType, fieldType="Scalar", f=1.0):
        """FE::assemblyRHS (FE_def.hpp:7303-7400).  f: a constant (Scalar),
        or a function evaluated at the rule's physical quadrature points,
        f(xq) with xq of shape (n, 3) returning n values (Scalar) or (n, 3)
        (Vector, node-wise dofs)."""
        if fieldType not in ("Scalar", "Vector"):
            raise ValueError("fieldType 'Scalar' or 'Vector'")
        if not callable(f):
            if fieldType != "Scalar":
                raise ValueError("a constant source is scalar")
            a = self._get(("Laplace", FEType, f), problem=A.LAPLACE, fe_order=self._order(FEType), source=f)
            _, ru, _ = a.assemble(jacobian=False, residual=True)
            return ru
        a = self._get(("Laplace", FEType), problem=A.LAPLACE, fe_order=self._order(FEType))
        return a.assemble_rhs(f, 1 if fieldType == "Scalar" else 3)

    def _elasticity(self, problem, d_rep, params, assembleMode, quad, eModVec=None):
        E = _param(params, "Parameter", "E", 1000.0)
        nu = _param(params, "Parameter", "Poisson Ratio", 0.4)
        a = self._get(("Elas", problem, E, nu), problem=problem, E=E, poisson_ratio=nu, quad_points=quad)
        a.set_element_moduli(eModVec)
        jac = assembleMode in ("Jacobian", "Newton-Residual", "Jacobian+Residual")
        res = assembleMode in ("Rhs", "Newton-Residual", "Jacobian+Residual")
        vals, ru, _ = a.assemble(u=d_rep, jacobian=jac, residual=res)
        mat = None
        if jac:
            rp, ci, shape = a.pattern(0)
            mat = CsrMatrix(rp, ci, vals[0], shape)
        return mat, ru

    def assemblyLinearElasticity(self, dim, FEType, degree, dofs, d_rep, params=None, reAssemble=False,
                                 assembleMode="Jacobian", callFillComplete=True):
        """FE::assemblyLinearElasticity (FE_def.hpp:362-434): AceGen skr1."""
        return self._elasticity(A.LINEAR_ELASTICITY, d_rep, params, assembleMode, 0)

    def assemblyNonLinearElasticity(self, dim, FEType, degree, dofs, d_rep, params=None, reAssemble=False,
                                    assembleMode="Jacobian", callFillComplete=True, eModVec=None):
        """FE::assemblyNonLinearElasticity (FE_def.hpp:449-523): "Parameter/
        Neo-Hooke Modell" 1 (the default) is "NonLinearElasticity" (AceGen
        skr2), any other value "NonLinearElasticity2" (skr3) (:483-487).
        eModVec: a Young's modulus per element, the E-field variant
        (:538-614)."""
        if d_rep is None:
            d_rep = np.zeros(3 * self.coords.shape[0])
        model = _param(params, "Parameter", "Neo-Hooke Modell", 1)
        prob = A.NONLINEAR_ELASTICITY if model == 1 else A.NONLINEAR_ELASTICITY2
        return self._elasticity(prob, d_rep, params, assembleMode, 0, eModVec)

    def assemblyNavierStokes(self, dim, FETypeVelocity, FETypePressure, degree, dofsVelocity, dofsPressure,
                             u_rep, p_rep, params=None, reAssemble=False, assembleMode="Jacobian",
                             callFillComplete=True, coeff=((1.0, 1.0), (1.0, 1.0))):
        """FE::assemblyNavierStokes (FE_def.hpp:1078-1239).  Returns a 2x2
        list of CsrMatrix (block (1,1) empty) for "Jacobian", the residual
        pair (res_u, res_p) for "Rhs"; coeff scales the residual's blocks
        (the reference's argument, handed to each element by setCoeff)."""
        if (FETypeVelocity, FETypePressure) != ("P2", "P1"):
            raise ValueError("Taylor-Hood P2-P1 only")
        visc = _param(params, "Parameter", "Viscosity", 1.0)
        dens = _param(params, "Parameter", "Density", 1.0)
        newton = _param(params, "General", "Linearization", "FixedPoint") != "FixedPoint"
        xyz_p, el_p = self.domain_p
        a = self._get(("NS", visc, dens, newton), problem=A.NAVIER_STOKES, elements_p=el_p,
                      num_nodes_p=xyz_p.shape[0], viscosity=visc, density=dens, newton=newton)
        if assembleMode == "Rhs":
            a.set_coeff(coeff)
            _, ru, rp = a.assemble(u=u_rep, p=p_rep, jacobian=False, residual=True)
            return ru, rp
        vals, _, _ = a.assemble(u=u_rep, p=p_rep, jacobian=True, residual=False)
        blocks = [[None, None], [None, None]]
        for b, (i, j) in enumerate([(0, 0), (0, 1), (1, 0)]):
            rp, ci, shape = a.pattern(b)
            blocks[i][j] = CsrMatrix(rp, ci, vals[b], shape)
        rp, ci, shape = a.pattern(3)
        blocks[1][1] = CsrMatrix(rp, ci, np.zeros(0), shape)
        if reAssemble:  # FEDDLib re-assembles only block (0,0) in Newton steps
            return blocks[0][0]
        return blocks
