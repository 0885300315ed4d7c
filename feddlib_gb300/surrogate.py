"""Strain-energy surrogate for the two-fibre exponential law (no FEDDLib
counterpart; it stands in for an expensive anisotropic law).

The network learns the fibre part of the energy,
    Psi_fib(I4a, I4b) = sum_f k1 / (2 k2) (exp(k2 (I4f - 1)^2) - 1),  I4f > 1,
from invariants x = (I1, J, I4a, I4b); the compressible neo-Hooke matrix
(skr1) stays analytic.  Samples are the deformation gradients at the
quadrature points of the simulation's own load steps (the plain law's
deformations, e.g. the Newton iterates of a load-stepping run).  Targets
come from the engine's plain-law kernel (fedd_law_eval): the energy and the
first Piola-Kirchhoff stress of the two-fibre law minus those of its
neo-Hooke matrix give Psi_fib and P_fib, and P_fib, which lies in the span
of dI4a/dF and dI4b/dF, gives dPsi_fib/dinv by least squares per sample.
Training minimises the Sobolev loss with the engine's own device kernels
(fedd_trainer_*).  Inputs on which the sampled targets show no
dependence (I1 and J for this law) are frozen: their normalisation scale is
zero, so the network's derivative with respect to them is exactly zero and
the trained box does not restrict them.  The fibre invariants enter as
max(I4 - 1, 0)^2: the law's one-sidedness at I4 = 1 (fibres in tension only)
is part of the input map, not something the network has to fit.  At inference the weights are rounded
to bf16 and evaluated on the tensor cores; quadrature points whose invariants
leave the training box fall back to the plain law.
"""
import math
import time

import numpy as np

from . import _capi as A
from .fe import Trainer


def fibre_energy(inv, k1=2.0, k2=1.0):
    """Psi_fib and its gradient with respect to (I1, J, I4a, I4b)."""
    inv = np.asarray(inv, dtype=np.float64)
    psi = np.zeros(inv.shape[0])
    g = np.zeros((inv.shape[0], 4))
    for f in (2, 3):
        e = inv[:, f] - 1.0
        act = e > 0
        ex = np.exp(k2 * e * e)
        psi += np.where(act, k1 / (2 * k2) * (ex - 1.0), 0.0)
        g[:, f] = np.where(act, k1 * e * ex, 0.0)
    return psi, g


def state_samples(asm, states, n_samples=2_000_000, seed=0):
    """Invariants at every quadrature point of each displacement state, then a
    seeded subsample of n_samples points."""
    allinv = np.concatenate([asm.qp_invariants(u).reshape(-1, 4) for u in states])
    rng = np.random.default_rng(seed)
    idx = rng.choice(allinv.shape[0], size=min(n_samples, allinv.shape[0]), replace=False)
    return allinv[idx].astype(np.float64)


def load_step_samples(asm, u_full, steps=10, n_samples=2_000_000, seed=0):
    """Invariants at the quadrature points of load steps l/steps * u_full,
    l = 1..steps (seeded subsample of n_samples points)."""
    return state_samples(asm, [u_full * (l / steps) for l in range(1, steps + 1)], n_samples, seed)


# the 4-point rule of the fibre law's elements (AceGen code 18) and the P2
# reference gradients at a point (FEDDLib local node order)
_Q4A, _Q4B = 0.585410196624968454, 0.138196601125010515
_Q4 = np.array([[_Q4A, _Q4B, _Q4B], [_Q4B, _Q4A, _Q4B], [_Q4B, _Q4B, _Q4A], [_Q4B, _Q4B, _Q4B]])


def _p2_ref_grad(p):
    x, y, z = p
    t = -3 + 4 * (x + y + z)
    return np.array([[t, t, t], [4 * x - 1, 0, 0], [0, 4 * y - 1, 0], [0, 0, 4 * z - 1],
                     [4 - 8 * x - 4 * y - 4 * z, -4 * x, -4 * x], [4 * y, 4 * x, 0],
                     [-4 * y, 4 - 4 * x - 8 * y - 4 * z, -4 * y], [-4 * z, -4 * z, 4 - 4 * x - 4 * y - 8 * z],
                     [4 * z, 0, 4 * x], [0, 4 * z, 4 * y]])


def qp_F(coords, elements, u, es, qs):
    """Deformation gradients F = I + grad u (FP64, host) at quadrature points
    qs (4-point rule) of elements es, for displacement u (3 per node)."""
    G = np.stack([_p2_ref_grad(p) for p in _Q4])          # (4, 10, 3)
    c = elements[es]                                      # (n, 10)
    x = coords[c]                                         # (n, 10, 3)
    B = np.stack([x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]], axis=2)
    Bi = np.linalg.inv(B)                                 # (n, 3, 3)
    Gp = np.einsum("nak,nkj->naj", G[qs], Bi)              # physical gradients (n, 10, 3)
    U = np.asarray(u).reshape(-1, 3)[c]                   # (n, 10, 3)
    return np.eye(3)[None] + np.einsum("nai,naj->nij", U, Gp)


def law_samples(plain, matrix, states, n_samples=2_000_000, seed=0, chunk=250_000):
    """Training samples from the plain law's own kernel: deformation
    gradients at a seeded subsample of the quadrature points of the given
    displacement states, the fibre law's energy and stress there
    (fedd_law_eval of `plain`) minus those of its neo-Hooke matrix
    (fedd_law_eval of `matrix`, the same E and nu).  Returns (inv, psi_fib,
    g_fib): invariants (I1, J, I4a, I4b), fibre energy and its derivatives
    with respect to the invariants (least squares on P_fib per sample)."""
    coords, elements = plain._keep[0], plain._keep[1]
    ne = elements.shape[0]
    rng = np.random.default_rng(seed)
    tot = len(states) * ne * 4
    pick = rng.choice(tot, size=min(n_samples, tot), replace=False)
    st, rem = pick // (ne * 4), pick % (ne * 4)
    es, qs = rem // 4, rem % 4
    inv_l, psi_l, g_l = [], [], []
    for k0 in range(0, len(pick), chunk):
        sl = slice(k0, k0 + chunk)
        F = np.empty((len(pick[sl]), 3, 3))
        for s_ in np.unique(st[sl]):
            m = st[sl] == s_
            F[m] = qp_F(coords, elements, states[s_], es[sl][m], qs[sl][m])
        psi_p, P_p, _ = plain.law_eval(F)
        psi_m, P_m, _ = matrix.law_eval(F)
        inv, psi, g = fibre_targets(F, psi_p, P_p, psi_m, P_m)
        inv_l.append(inv); psi_l.append(psi); g_l.append(g)
    return np.concatenate(inv_l), np.concatenate(psi_l), np.concatenate(g_l)


def fibre_targets(F, psi_p, P_p, psi_m, P_m, angle_deg=40.0):
    """Invariants of F and the fibre part of a plain-law evaluation: psi_fib
    = psi_p - psi_m and dPsi_fib/dinv from P_fib = P_p - P_m, which equals
    dPsi/dI4a 2 F a (x) a + dPsi/dI4b 2 F b (x) b (fibres a, b at +-angle in
    the xy-plane), by least squares per sample."""
    a = np.radians(angle_deg)
    fa = np.array([np.cos(a), np.sin(a), 0.0]); fb = np.array([np.cos(a), -np.sin(a), 0.0])
    C = np.einsum("nki,nkj->nij", F, F)
    J = np.linalg.det(F)
    I4a = np.einsum("i,nij,j->n", fa, C, fa); I4b = np.einsum("i,nij,j->n", fb, C, fb)
    inv = np.stack([np.einsum("nii->n", C), J, I4a, I4b], axis=1)
    Da = 2 * np.einsum("nij,j,k->nik", F, fa, fa).reshape(-1, 9)
    Db = 2 * np.einsum("nij,j,k->nik", F, fb, fb).reshape(-1, 9)
    Pf = (np.asarray(P_p) - np.asarray(P_m)).reshape(-1, 9)
    Maa, Mab, Mbb = (Da * Da).sum(1), (Da * Db).sum(1), (Db * Db).sum(1)
    ra, rb = (Da * Pf).sum(1), (Db * Pf).sum(1)
    det = Maa * Mbb - Mab * Mab
    g = np.zeros((len(Pf), 4))
    g[:, 2] = (Mbb * ra - Mab * rb) / det
    g[:, 3] = (Maa * rb - Mab * ra) / det
    return inv, np.asarray(psi_p) - np.asarray(psi_m), g


def init_params(H, seed=0):
    rng = np.random.default_rng(seed)
    return {"W1": rng.standard_normal((H, 4)) * math.sqrt(1.0 / 4),
            "b1": np.zeros(H),
            "W2": rng.standard_normal((H, H)) * math.sqrt(1.0 / H),
            "b2": np.zeros(H),
            "w3": rng.standard_normal(H) * math.sqrt(1.0 / H),
            "b3": 0.0}


def train_surrogate(inv, k1=2.0, k2=1.0, hidden=64, steps=3000, batch=65536, lr=3e-3, lr_final=1e-4,
                    wpsi=1.0, wgrad=1.0, seed=0, device=0, log=None, targets=None, clamp=(2, 3), clamp_at=1.0):
    """Trains on the device; returns the model dict (FP32 master weights plus
    normalisation) and a training report.  targets = (psi_fib, g_fib) from
    law_samples; without them the fibre energy is evaluated from the
    invariants (fibre_energy).  The inputs listed in `clamp` (the fibre
    invariants: the fibres carry load in tension only) enter the network as
    max(I4 - clamp_at, 0)^2: the one-sidedness of the law is then part of the
    input map, the surrogate and its stress vanish continuously in
    compression (dx/dI4 -> 0 at I4 = 1), and the network fits a function
    that is smooth where it is used (the exponential law is a smooth function
    of (I4 - 1)^2)."""
    psi, g = fibre_energy(inv, k1, k2) if targets is None else targets
    gmax = np.abs(g).max(axis=0)
    active = gmax > 1e-9 * max(gmax.max(), 1e-300)
    g = np.where(active, g, 0.0)
    cl = np.zeros(4, dtype=bool)
    for k in clamp:
        cl[k] = active[k]
    shift = np.where(cl, clamp_at, inv.mean(axis=0))
    e = inv - shift
    ep = np.maximum(e, 0.0)
    # clamped inputs enter as max(I4 - 1, 0)^2 (the law is a smooth function of it)
    z = np.where(cl[None, :], ep * ep, e)
    # the clamped inputs share one scale (the two fibres obey one law): a
    # fibre that is barely stretched in the samples would otherwise get a huge
    # scale, and its tiny share of the output would be lost to bf16 rounding
    # and then multiplied by that scale in the tangent
    pooled = np.sqrt((z[:, cl] ** 2).mean()) if cl.any() else 1.0
    spread = np.where(cl, pooled, inv.std(axis=0))
    scale = np.where(active, 1.0 / np.maximum(spread, 1e-12), 0.0)
    out_scale = float(max(np.abs(psi).max(), 1e-6))
    x = z * scale
    ty = psi / out_scale
    # dPsi/dx = dPsi/dinv / (dx/dinv); for a clamped input dx/dinv = 2 (I4 - 1)
    # scale, and the quotient is kept finite where I4 - 1 is tiny (there the
    # stress it multiplies vanishes with I4 - 1)
    emin = 1e-3 * np.sqrt(np.maximum((ep * ep).mean(axis=0), 1e-30))
    dxdi = np.where(cl[None, :], 2.0 * np.maximum(ep, emin[None, :]), 1.0) * np.where(active, scale, 1.0)
    tg = np.where(active[None, :], g / (out_scale * dxdi), 0.0)
    # in compression a clamped input sits at x = 0 and its chain factor is
    # zero, so the network's slope there never reaches the stress; its target
    # is the slope's right limit (the median over the 2 % of samples closest
    # above the shift), which keeps the targets at x = 0 consistent
    for k in np.flatnonzero(cl):
        pos = ep[:, k] > 0
        if pos.any():
            near = pos & (ep[:, k] <= np.quantile(ep[pos, k], 0.02))
            tg[~pos, k] = np.median(tg[near, k])
    tr = Trainer(hidden, x, ty, tg, device=device)
    m = init_params(hidden, seed)
    tr.set_params(m)
    t0 = time.time()
    chunk = 100
    # loss of the untrained network (full data set when it is small)
    if x.shape[0] <= 262144:
        losses = [float(tr.grad(wpsi, wgrad)[0])]
    else:
        losses = [float(tr.run(1, min(batch, x.shape[0]), 0.0, wpsi, wgrad, seed=seed))]
    done = 0
    while done < steps:
        n = min(chunk, steps - done)
        frac = done / max(steps - 1, 1)
        cur = lr * (lr_final / lr) ** frac  # geometric decay
        losses.append(tr.run(n, min(batch, x.shape[0]), cur, wpsi, wgrad, seed=seed))
        done += n
        if log:
            log(f"step {done} lr {cur:.2e} loss {losses[-1]:.3e}")
    params = tr.get_params()
    tr.close()
    model = dict(params)
    model.update({"in_shift": shift, "in_scale": scale, "out_scale": out_scale,
                  "in_clamp": int(sum(1 << k for k in range(4) if cl[k])),
                  # a clamped input below its shift maps to 0, inside the training data
                  "inv_lo": np.where(active & ~cl, inv.min(axis=0), -1e30),
                  "inv_hi": np.where(active, inv.max(axis=0), 1e30), "add_matrix": 1})
    report = {"samples": int(inv.shape[0]), "steps": steps, "batch": batch, "seconds": time.time() - t0,
              "targets": "fedd_law_eval of the plain law (energy, stress)" if targets is not None else
                         "fibre energy of the invariants",
              "final_loss": float(losses[-1]) if losses else None, "loss_history": [float(v) for v in losses]}
    return model, report


def bf16_round(a):
    """Round-to-nearest-even to bf16, returned as float64 (what the device
    evaluates)."""
    a = np.asarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def stress_tangent_errors(asm_plain, asm_surr, F):
    """Relative Frobenius errors of P and A = dP/dF of the surrogate against
    the plain law at deformation gradients F (n x 3 x 3), both evaluated by
    the engine (fedd_law_eval)."""
    _, Pp, Ap = asm_plain.law_eval(F)
    _, Ps, As = asm_surr.law_eval(F)
    dP = np.linalg.norm((Ps - Pp).reshape(len(F), -1), axis=1)
    nP = np.linalg.norm(Pp.reshape(len(F), -1), axis=1)
    dA = np.linalg.norm((As - Ap).reshape(len(F), -1), axis=1)
    nA = np.linalg.norm(Ap.reshape(len(F), -1), axis=1)
    return {"stress_rel_fro": float(np.linalg.norm(Ps - Pp) / np.linalg.norm(Pp)),
            "stress_rel_max": float((dP / np.maximum(nP, 1e-30)).max()),
            "stress_rel_median": float(np.median(dP / np.maximum(nP, 1e-30))),
            "tangent_rel_fro": float(np.linalg.norm(As - Ap) / np.linalg.norm(Ap)),
            "tangent_rel_max": float((dA / np.maximum(nA, 1e-30)).max())}


def sample_F(inv_source_asm, u, n, seed=0):
    """Deformation gradients at random quadrature points of the mesh for
    displacement u, rebuilt from element data on the host (FP64)."""
    coords, elements = inv_source_asm._keep[0], inv_source_asm._keep[1]
    rng = np.random.default_rng(seed)
    es = rng.integers(0, elements.shape[0], n)
    a, b = 0.585410196624968454, 0.138196601125010515
    pts = np.array([[a, b, b], [b, a, b], [b, b, a], [b, b, b]])
    qs = rng.integers(0, 4, n)
    F = np.zeros((n, 3, 3))
    U = np.asarray(u).reshape(-1, 3)
    for t in range(n):
        c = elements[es[t]]
        x = coords[c]
        B = np.stack([x[1] - x[0], x[2] - x[0], x[3] - x[0]], axis=1)
        Bi = np.linalg.inv(B)
        p = pts[qs[t]]
        x_, y_, z_ = p
        tt = -3 + 4 * (x_ + y_ + z_)
        G = np.array([[tt, tt, tt], [4 * x_ - 1, 0, 0], [0, 4 * y_ - 1, 0], [0, 0, 4 * z_ - 1],
                      [4 - 8 * x_ - 4 * y_ - 4 * z_, -4 * x_, -4 * x_], [4 * y_, 4 * x_, 0],
                      [-4 * y_, 4 - 4 * x_ - 8 * y_ - 4 * z_, -4 * y_], [-4 * z_, -4 * z_, 4 - 4 * x_ - 4 * y_ - 8 * z_],
                      [4 * z_, 0, 4 * x_], [0, 4 * z_, 4 * y_]])
        Gp = G @ Bi
        F[t] = np.eye(3) + U[c].T @ Gp
    return F
