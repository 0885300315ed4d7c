"""Parity at the configurations' full sizes (test infrastructure only).

The checker side of the full-size parity tests and of the bench's parity
report: the engine's complete CSR pattern is checked node by node against
the element adjacency, and the complete rows of a seeded sample of nodes
(>= 1 % of each row-node set) are rebuilt by the FP64 oracle from all of
their incident elements and compared with the engine's rows, block by
block.  Only tests/ and bench.py's CPU leg import this module.
"""
import math

import numpy as np

from . import oracle as O

I64 = np.int64


def _lib():
    L = O.lib()
    if not getattr(L, "_parity_sigs", False):
        import ctypes as C
        i, i64, d, vp = C.c_int, C.c_int64, C.c_double, C.c_void_p
        L.orc_node_elements.argtypes = [i64, vp, i, i64, vp, vp]
        L.orc_check_block_pattern.argtypes = [i64, vp, i, vp, i, i64, vp, vp, i, i, vp, vp]
        L.orc_check_block_pattern.restype = i64
        L.orc_rows_vec.argtypes = [i, vp, i, i64, vp, vp, vp, vp, vp, i64, vp, i, vp, vp, vp]
        L.orc_rows_vec.restype = i
        L.orc_rows_ns.argtypes = [i64, vp, vp, vp, vp, vp, d, d, i, vp, vp, vp, vp, i64, vp, i64, vp, i, i,
                                  vp, vp, vp, vp, vp, vp, vp, vp]
        L.orc_rows_ns.restype = i
        L.orc_rows_gn.argtypes = [i64, vp, vp, vp, vp, vp, vp, d, i, vp, vp, vp, vp, i64, vp, i64, vp, i, i,
                                  vp, vp, vp, vp, vp, vp, vp, vp]
        L.orc_rows_gn.restype = i
        L._parity_sigs = True
    return L


def node_elements(conn, nn):
    """(ptr, elems): the elements incident to each node, ascending."""
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    ne, npe = conn.shape
    ptr = np.zeros(nn + 1, dtype=I64)
    el = np.zeros(ne * npe, dtype=I64)
    _lib().orc_node_elements(ne, O.p(conn, O.I32), npe, nn, O.p(ptr, O.I64), O.p(el, O.I64))
    return ptr, el


def sample_nodes(nn, frac=0.01, seed=0):
    """A seeded sample of ceil(frac * nn) distinct nodes (at least 64, at most
    all), sorted, always holding the first and the last node."""
    k = min(nn, max(64, int(math.ceil(frac * nn))))
    rng = np.random.default_rng(seed)
    s = rng.choice(nn, size=k, replace=False).astype(I64)
    s[0], s[-1] = 0, nn - 1
    return np.unique(s)


def check_pattern(row_conn, col_conn, nrow_nodes, node_inc, dofs_r, dofs_c, rowptr, colind):
    """-1 when the CSR block (rowptr, colind) is exactly the node adjacency of
    the elements (rows (row node, dr), columns (column node, dc), node-wise,
    ascending) at every row; else the first row that differs."""
    rc = np.ascontiguousarray(row_conn, dtype=np.int32)
    cc = np.ascontiguousarray(col_conn, dtype=np.int32)
    ptr, el = node_inc
    rowptr = np.ascontiguousarray(rowptr, dtype=I64)
    colind = np.ascontiguousarray(colind, dtype=np.int32)
    if rowptr.shape[0] != dofs_r * nrow_nodes + 1:
        return 0
    return int(_lib().orc_check_block_pattern(rc.shape[0], O.p(rc, O.I32), rc.shape[1], O.p(cc, O.I32),
                                              cc.shape[1], nrow_nodes, O.p(ptr, O.I64), O.p(el, O.I64),
                                              dofs_r, dofs_c, O.p(rowptr, O.I64), O.p(colind, O.I32)))


def _rows_of(rowptr, vals, rows):
    return [vals[rowptr[r]:rowptr[r + 1]] for r in rows]


def _rel(num, den):
    return float(math.sqrt(num) / max(math.sqrt(den), 1e-300))


def rows_vec(kind, law, npts, xyz, conn, u, node_inc, sel, kmax=160):
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    sel = np.ascontiguousarray(sel, dtype=I64)
    n = sel.shape[0]
    cols = np.zeros(n * kmax, dtype=I64)
    vals = np.zeros(n * 9 * kmax)
    res = np.zeros(3 * n)
    uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64).ravel()
    rc = _lib().orc_rows_vec(kind, law.ptr, npts, conn.shape[0], O.p(xyz), O.p(conn, O.I32), O.p(uu),
                             O.p(node_inc[0], O.I64), O.p(node_inc[1], O.I64), n, O.p(sel, O.I64), kmax,
                             O.p(cols, O.I64), O.p(vals), O.p(res))
    if rc:
        raise RuntimeError("a sampled node has more columns than kmax")
    return cols.reshape(n, kmax), vals.reshape(n, 3, kmax, 3), res.reshape(n, 3)


def compare_vec(rowptr, colind, vals, res, oracle_rows, sel):
    """Relative Frobenius errors of the sampled rows of a 3-dof block and of
    their residual entries: {"block": e, "residual": e or None, "rows": n}.
    Raises if a sampled row's columns differ from the oracle's."""
    cols, ov, ores = oracle_rows
    num = den = rnum = rden = 0.0
    for k, n in enumerate(sel):
        K = int((cols[k] >= 0).sum())
        want_c = (3 * cols[k, :K, None] + np.arange(3)).ravel()
        for di in range(3):
            r = 3 * n + di
            a, b = rowptr[r], rowptr[r + 1]
            if b - a != 3 * K or not np.array_equal(colind[a:b], want_c):
                raise AssertionError(f"row {r}: columns differ from the oracle's")
            o = ov[k, di, :K, :].ravel()
            num += float(((vals[a:b] - o) ** 2).sum()); den += float((o ** 2).sum())
        if res is not None:
            e = res[3 * n:3 * n + 3]
            rnum += float(((e - ores[k]) ** 2).sum()); rden += float((ores[k] ** 2).sum())
    return {"block": _rel(num, den), "residual": _rel(rnum, rden) if res is not None else None,
            "rows": int(3 * len(sel))}


def rows_ns(xyz2, conn2, conn1, u, pr, visc, dens, newton, inc2, inc1, vsel, psel, kmax=160, kpmax=64, law=None):
    """Complete rows of the sampled velocity nodes (vsel) and pressure nodes
    (psel), each rebuilt from all of its incident elements; with `law` (an
    oracle.ViscLaw) the generalized-Newtonian element, visc ignored."""
    conn2 = np.ascontiguousarray(conn2, dtype=np.int32)
    conn1 = np.ascontiguousarray(conn1, dtype=np.int32)
    vsel = np.ascontiguousarray(vsel, dtype=I64)
    psel = np.ascontiguousarray(psel, dtype=I64)
    nv, npr = vsel.shape[0], psel.shape[0]
    c00 = np.zeros(nv * kmax, dtype=I64); v00 = np.zeros(nv * 9 * kmax)
    c01 = np.zeros(nv * kpmax, dtype=I64); v01 = np.zeros(nv * 3 * kpmax)
    ru = np.zeros(3 * nv)
    c10 = np.zeros(max(npr, 1) * kmax, dtype=I64); v10 = np.zeros(max(npr, 1) * 3 * kmax)
    rp = np.zeros(max(npr, 1))
    uu = np.ascontiguousarray(u, dtype=np.float64).ravel()
    pp = np.ascontiguousarray(pr, dtype=np.float64)
    import ctypes as C
    head = ((_lib().orc_rows_gn, C.cast(C.pointer(law), C.c_void_p)) if law is not None
            else (_lib().orc_rows_ns, float(visc)))
    rc = head[0](conn2.shape[0], O.p(xyz2), O.p(conn2, O.I32), O.p(conn1, O.I32), O.p(uu), O.p(pp),
                            head[1], float(dens), int(newton), O.p(inc2[0], O.I64), O.p(inc2[1], O.I64),
                            O.p(inc1[0], O.I64), O.p(inc1[1], O.I64), nv, O.p(vsel, O.I64), npr,
                            O.p(psel, O.I64), kmax, kpmax, O.p(c00, O.I64), O.p(v00), O.p(c01, O.I64), O.p(v01),
                            O.p(ru), O.p(c10, O.I64), O.p(v10), O.p(rp))
    if rc:
        raise RuntimeError("a sampled node has more columns than kmax / kpmax")
    return dict(c00=c00.reshape(nv, kmax), v00=v00.reshape(nv, 3, kmax, 3), c01=c01.reshape(nv, kpmax),
                v01=v01.reshape(nv, 3, kpmax), ru=ru.reshape(nv, 3), c10=c10.reshape(-1, kmax)[:npr],
                v10=v10.reshape(-1, kmax, 3)[:npr], rp=rp[:npr])


def compare_ns(csr, res_u, res_p, o, vsel, psel):
    """Per-block relative Frobenius errors of the sampled Navier-Stokes rows:
    {"00", "01", "10", "res_u", "res_p", "rows_u", "rows_p"}.  csr[b] =
    (rowptr, colind, vals) of block b; columns must equal the oracle's."""
    acc = {k: [0.0, 0.0] for k in ("00", "01", "10", "res_u", "res_p")}

    def add(key, got, want):
        acc[key][0] += float(((got - want) ** 2).sum()); acc[key][1] += float((want ** 2).sum())

    (rp0, ci0, v0), (rp1, ci1, v1), (rp2, ci2, v2) = csr[0], csr[1], csr[2]
    for k, n in enumerate(vsel):
        K = int((o["c00"][k] >= 0).sum()); Kp = int((o["c01"][k] >= 0).sum())
        c3 = (3 * o["c00"][k, :K, None] + np.arange(3)).ravel()
        for di in range(3):
            r = 3 * n + di
            a, b = rp0[r], rp0[r + 1]
            if b - a != 3 * K or not np.array_equal(ci0[a:b], c3):
                raise AssertionError(f"block (0,0) row {r}: columns differ from the oracle's")
            add("00", v0[a:b], o["v00"][k, di, :K, :].ravel())
            a, b = rp1[r], rp1[r + 1]
            if b - a != Kp or not np.array_equal(ci1[a:b], o["c01"][k, :Kp]):
                raise AssertionError(f"block (0,1) row {r}: columns differ from the oracle's")
            add("01", v1[a:b], o["v01"][k, di, :Kp])
        if res_u is not None:
            add("res_u", res_u[3 * n:3 * n + 3], o["ru"][k])
    for k, q in enumerate(psel):
        K = int((o["c10"][k] >= 0).sum())
        c3 = (3 * o["c10"][k, :K, None] + np.arange(3)).ravel()
        a, b = rp2[q], rp2[q + 1]
        if b - a != 3 * K or not np.array_equal(ci2[a:b], c3):
            raise AssertionError(f"block (1,0) row {q}: columns differ from the oracle's")
        add("10", v2[a:b], o["v10"][k, :K, :].ravel())
        if res_p is not None:
            add("res_p", res_p[q:q + 1], o["rp"][k:k + 1])
    out = {k: (_rel(*v) if v[1] > 0 else None) for k, v in acc.items()}
    out["rows_u"] = int(3 * len(vsel)); out["rows_p"] = int(len(psel))
    return out
