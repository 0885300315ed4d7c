"""Small Newton driver for hyperelastic load stepping on the engine.

Only for comparing laws (plain vs surrogate) by their Newton iteration
counts; FEDDLib's own nonlinear solvers (NOX / NonLinearSolver, with Belos /
FROSch underneath) stay outside the engine.  Conventions follow FEDDLib's
elasticity elements: the engine returns r = -f_int and K = -dr/du, so a
Newton step solves K du = r at the free dofs.  The linear solve is a direct
sparse solve on the host (scipy), adequate for the small meshes used here.
"""
import numpy as np


def box_bc(coords, axis=0, tol=1e-9):
    """Dofs on the faces x_axis = 0 (clamped) and x_axis = 1 (pulled)."""
    lo = np.where(np.abs(coords[:, axis]) < tol)[0]
    hi = np.where(np.abs(coords[:, axis] - 1.0) < tol)[0]
    clamped = np.concatenate([3 * lo, 3 * lo + 1, 3 * lo + 2])
    pulled = 3 * hi + axis
    return clamped, pulled


def solve_load_steps(asm, coords, stretch=0.2, steps=5, axis=0, tol=1e-6, max_iter=25, on_iterate=None):
    """Pull the face x_axis = 1 to `stretch` in `steps` increments with the
    opposite face clamped.  A step has converged when the free-dof residual
    norm is below tol * max(r0, 1), r0 being the step's first residual; the
    default tolerance sits above the noise of FP32 element accumulation.
    `on_iterate(step, it, u)` sees every iterate (e.g. to collect surrogate
    training samples).  Returns (u, iterations per step, residual
    histories)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    n = 3 * coords.shape[0]
    clamped, pulled = box_bc(coords, axis)
    fixed = np.zeros(n, dtype=bool)
    fixed[clamped] = True
    fixed[pulled] = True
    free = ~fixed
    u = np.zeros(n)
    rp, ci, shape = asm.pattern(0)
    its, hist = [], []
    for s in range(1, steps + 1):
        u[pulled] = stretch * s / steps
        u[clamped] = 0.0
        h = []
        r0 = None
        for it in range(max_iter + 1):
            if on_iterate is not None:
                on_iterate(s, it, u.copy())
            (vals,), r, _ = asm.assemble(u=u)
            rn = float(np.linalg.norm(r[free]))
            h.append(rn)
            if r0 is None:
                r0 = max(rn, 1e-300)
            if rn <= tol * max(r0, 1.0):
                break
            K = sp.csr_matrix((vals, ci, rp), shape=shape)[free][:, free]
            du = spla.spsolve(K.tocsc(), r[free])
            u[free] += du
        its.append(len(h) - 1)
        hist.append(h)
    return u, its, hist
