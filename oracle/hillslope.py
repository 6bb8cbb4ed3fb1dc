"""FP64 restatement of the reference's implicit hillslope step -- TEST
INFRASTRUCTURE ONLY.

The reference solves the backward-Euler Roering step with Newton and Eigen's
SparseLU (src/cpu/lsdtt_hillslope_newton_cpu.cpp:196-675, 690-788) on the
shared operator of src/cpu/lsdtt_hillslope_operator_cpu.hpp:83-322. Eigen is
not available here, so this module restates the linear case (alpha = 1):
the residual F, the constant Jacobian J (triplets summed like
setFromTriplets) and one Newton step solved exactly by scipy's SuperLU,
iterated until ||F||_inf <= residual_tol as the reference does. Parity with
the Eigen build itself is unpinned; the restatement is checked by the
reference's own analytic properties (volume conservation under no-flux,
Dirichlet cells untouched, linear steady state) in tests/test_hillslope_oracle.py.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def _neighbours(nr, nc, bc, mask):
    """Index of the N, E, S, W neighbour of every cell under the domain rule
    (operator_cpu.hpp:163-175): 'p' wraps, other edges and masked cells
    resolve to the cell itself."""
    r = np.arange(nr)[:, None].repeat(nc, 1)
    c = np.arange(nc)[None, :].repeat(nr, 0)
    out = []
    for dr, dc in ((-1, 0), (0, 1), (1, 0), (0, -1)):
        rr = r + dr
        cc = c + dc
        rr = np.where(rr < 0, (nr - 1) if bc[0] == "p" else r, rr)
        rr = np.where(rr >= nr, 0 if bc[2] == "p" else r, rr)
        cc = np.where(cc < 0, (nc - 1) if bc[3] == "p" else c, cc)
        cc = np.where(cc >= nc, 0 if bc[1] == "p" else c, cc)
        j = rr * nc + cc
        self_i = r * nc + c
        j = np.where(mask.ravel()[j.ravel()].reshape(nr, nc) != 0, j, self_i)
        out.append(j.ravel())
    return out


def dofs(nr, nc, bc, mask, is_channel=None):
    r = np.arange(nr)[:, None].repeat(nc, 1)
    c = np.arange(nc)[None, :].repeat(nr, 0)
    dirichlet = ((r == 0) & (bc[0] == "o")) | ((r == nr - 1) & (bc[2] == "o")) | \
                ((c == 0) & (bc[3] == "o")) | ((c == nc - 1) & (bc[1] == "o"))
    d = (mask != 0) & ~dirichlet
    if is_channel is not None:
        d &= (is_channel == 0)
    return d.ravel()


def linear_step(z, mask, cell, bc, D, dt, U=0.0, residual_tol=1e-12, max_newton=50, is_channel=None,
                solver="direct", rel_tol=1e-8):
    """One backward-Euler step of linear hillslope diffusion over dt.
    Returns (z_new float32, n_newton, final ||F||_inf).

    solver="direct" (the parity oracle): sparse LU, Newton to residual_tol.
    solver="pcg": one Newton step solved by FP64 Jacobi-preconditioned CG to
    ||r|| <= rel_tol ||b|| (scipy), the iterative form of the reference's
    Eigen solve; the timed CPU baseline uses it."""
    bc = (bc + "oooo")[:4]
    z = np.asarray(z, np.float32)
    nr, nc = z.shape
    n = nr * nc
    mask = np.asarray(mask, np.uint8)
    nb = _neighbours(nr, nc, bc, mask)
    dof = dofs(nr, nc, bc, mask, is_channel)
    idx = np.nonzero(dof)[0]
    dof_of = np.full(n, -1, np.int64)
    dof_of[idx] = np.arange(idx.size)
    DA = float(D) / (cell * cell)
    inv_dt = 1.0 / float(dt)
    zn = z.ravel().astype(np.float64)

    def residual(zz):
        flux = np.zeros(idx.size)
        for j in nb:
            flux += zz[j[idx]] - zz[idx]
        F = -U - DA * flux + inv_dt * (zz[idx] - zn[idx])
        return F

    rows, cols, vals = [idx * 0 + np.arange(idx.size)], [np.arange(idx.size)], [np.full(idx.size, inv_dt)]
    for j in nb:
        jj = j[idx]
        rows.append(np.arange(idx.size)); cols.append(np.arange(idx.size)); vals.append(np.full(idx.size, DA))
        ok = dof_of[jj] >= 0
        rows.append(np.arange(idx.size)[ok]); cols.append(dof_of[jj[ok]]); vals.append(np.full(ok.sum(), -DA))
    J = sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(idx.size, idx.size))
    if solver == "pcg":
        zz = zn.copy()
        F = residual(zz)
        if F.size and np.any(F != 0):
            Jr = J.tocsr()
            dinv = 1.0 / Jr.diagonal()
            M = spla.LinearOperator(Jr.shape, matvec=lambda v: dinv * v)
            dz, info = spla.cg(Jr, -F, rtol=rel_tol, atol=0.0, M=M, maxiter=10000)
            zz[idx] += dz
            F = residual(zz)
        return zz.astype(np.float32).reshape(nr, nc), 1, float(np.max(np.abs(F))) if F.size else 0.0
    lu = spla.splu(J)
    zz = zn.copy()
    F = residual(zz)
    it = 0
    while np.max(np.abs(F)) > residual_tol and it < max_newton:
        zz[idx] += lu.solve(-F)
        F = residual(zz)
        it += 1
    return zz.astype(np.float32).reshape(nr, nc), it, float(np.max(np.abs(F))) if F.size else 0.0


# ---------------------------------------------------------------------------
# Nonlinear (Roering) case: compute_hillslope_newton / _transient restated.
# ---------------------------------------------------------------------------
def _nb_index(nr, nc, bc, mask):
    """nb[(dr,dc)] -> flat index array of the domain neighbour for every cell
    (operator_cpu.hpp:163-175), for the 4 faces and the 4 tangential probes."""
    r = np.arange(nr)[:, None].repeat(nc, 1)
    c = np.arange(nc)[None, :].repeat(nr, 0)
    self_i = (r * nc + c)

    def nb(rr0, cc0, dr, dc):
        rr = rr0 + dr
        cc = cc0 + dc
        rr = np.where(rr < 0, (nr - 1) if bc[0] == "p" else rr0, rr)
        rr = np.where(rr >= nr, 0 if bc[2] == "p" else rr0, rr)
        cc = np.where(cc < 0, (nc - 1) if bc[3] == "p" else cc0, cc)
        cc = np.where(cc >= nc, 0 if bc[1] == "p" else cc0, cc)
        j = rr * nc + cc
        ok = mask.ravel()[j.ravel()].reshape(j.shape) != 0
        return np.where(ok, j, rr0 * nc + cc0)
    return nb, r, c, self_i


def _faces(z, nr, nc, bc, mask, h, Sc, nonlinear, cap):
    """Per cell and face (N, E, S, W): neighbour index, s_n, s_t, alpha,
    whether the cap binds (face_alphas, operator_cpu.hpp:290-321)."""
    nb, r, c, self_i = _nb_index(nr, nc, bc, mask)
    zf = z.ravel()
    E = nb(r, c, 0, 1).ravel(); Wd = nb(r, c, 0, -1).ravel()
    S = nb(r, c, 1, 0).ravel(); N = nb(r, c, -1, 0).ravel()
    sx = (zf[E] - zf[Wd]) / (2.0 * h)
    sy = (zf[S] - zf[N]) / (2.0 * h)
    out = []
    for k, (dr, dc) in enumerate(((-1, 0), (0, 1), (1, 0), (0, -1))):
        j = nb(r, c, dr, dc).ravel()
        sn = (zf[j] - zf) / h
        if not nonlinear:
            out.append((j, sn, np.zeros_like(sn), np.ones_like(sn), np.zeros(sn.shape, bool), k))
            continue
        st = 0.5 * (sx + sx[j]) if k in (0, 2) else 0.5 * (sy + sy[j])
        raw = (sn * sn + st * st) / (Sc * Sc)
        s2 = np.minimum(raw, cap)
        out.append((j, sn, st, 1.0 / (1.0 - s2), raw >= cap, k))
    return out, nb, r, c


def newton_step(z_in, zn_in, mask, cell, bc, D, Sc, inv_dt, nonlinear=True, U=0.0, residual_tol=1e-12,
                max_iterations=50, cap=0.9999, max_line_search=30):
    """compute_hillslope_newton (newton_cpu.cpp:196-675) on one sub-step.
    Returns (z float64, converged, iterations, final ||F||inf)."""
    bc = (bc + "oooo")[:4]
    nr, nc = z_in.shape
    n = nr * nc
    mask = np.asarray(mask, np.uint8)
    h = float(cell)
    DA = float(D) / (h * h)
    z = z_in.astype(np.float64).ravel().copy()
    zn = zn_in.astype(np.float64).ravel()
    dof = dofs(nr, nc, bc, mask)
    idx = np.nonzero(dof)[0]
    dof_of = np.full(n, -1, np.int64)
    dof_of[idx] = np.arange(idx.size)

    def residual(zz):
        faces, _, _, _ = _faces(zz.reshape(nr, nc), nr, nc, bc, mask, h, Sc, nonlinear, cap)
        flux = np.zeros(n)
        for (j, sn, st, a, capped, k) in faces:
            flux += a * sn * h
        F = -U - DA * flux
        if inv_dt > 0:
            F = F + inv_dt * (zz - zn)
        return F[idx]

    def max_ratio(zz):
        nb, r, c, _ = _nb_index(nr, nc, bc, mask)
        zf = zz
        sx = (zf[nb(r, c, 0, 1).ravel()] - zf[nb(r, c, 0, -1).ravel()]) / (2.0 * h)
        sy = (zf[nb(r, c, 1, 0).ravel()] - zf[nb(r, c, -1, 0).ravel()]) / (2.0 * h)
        v = np.sqrt(sx * sx + sy * sy)[idx] / Sc
        return float(v.max()) if v.size else 0.0

    def jacobian(zz):
        faces, nb, r, c = _faces(zz.reshape(nr, nc), nr, nc, bc, mask, h, Sc, nonlinear, cap)
        rows, cols, vals = [], [], []
        P = idx
        if inv_dt > 0:
            rows.append(P); cols.append(P); vals.append(np.full(P.size, inv_dt))
        for (j, sn, st, a, capped, k) in faces:
            rows.append(P); cols.append(j[P]); vals.append(-DA * a[P])
            rows.append(P); cols.append(P); vals.append(DA * a[P])
            if nonlinear:
                ok = ~capped[P]
                pref = a[P] * a[P] * 2.0 / (Sc * Sc)
                dzf = sn[P] * h
                coef = np.where(ok, -DA * dzf, 0.0)
                rows.append(P); cols.append(P); vals.append(coef * pref * sn[P] * (-1.0 / h))
                rows.append(P); cols.append(j[P]); vals.append(coef * pref * sn[P] * (1.0 / h))
                wt = pref * st[P] * (1.0 / (4.0 * h))
                rr, cc = r.ravel()[P], c.ravel()[P]
                jr, jc = j[P] // nc, j[P] % nc
                if k in (0, 2):
                    probes = [(rr, cc, 0, 1, 1.0), (rr, cc, 0, -1, -1.0), (jr, jc, 0, 1, 1.0), (jr, jc, 0, -1, -1.0)]
                else:
                    probes = [(rr, cc, 1, 0, 1.0), (rr, cc, -1, 0, -1.0), (jr, jc, 1, 0, 1.0), (jr, jc, -1, 0, -1.0)]
                for (pr, pc, dr, dc, sgn) in probes:
                    q = nb(pr, pc, dr, dc)
                    rows.append(P); cols.append(q); vals.append(coef * sgn * wt)
        R = np.concatenate(rows); Cq = np.concatenate(cols); V = np.concatenate(vals)
        keep = dof_of[Cq] >= 0
        return sp.csc_matrix((V[keep], (dof_of[R[keep]], dof_of[Cq[keep]])), shape=(idx.size, idx.size))

    if idx.size == 0:
        return z.reshape(nr, nc), True, 0, 0.0
    F = residual(z)
    fnorm = np.max(np.abs(F))
    feasible = np.sqrt(cap)
    it = 0
    converged = False
    while it < max_iterations:
        if fnorm <= residual_tol:
            converged = True
            break
        J = jacobian(z)
        step = spla.splu(J).solve(-F)
        lam = 1.0
        ratio_now = max_ratio(z) if nonlinear else 0.0
        restoring = nonlinear and ratio_now > feasible
        accepted = False
        for _ in range(max_line_search):
            zt = z.copy()
            zt[idx] += lam * step
            if nonlinear:
                rt = max_ratio(zt)
                if restoring:
                    if rt >= ratio_now:
                        lam *= 0.5
                        continue
                    Ft = residual(zt); accepted = True; break
                if rt > feasible:
                    lam *= 0.5
                    continue
            Ft = residual(zt)
            if np.max(np.abs(Ft)) < fnorm:
                accepted = True
                break
            lam *= 0.5
        if not accepted:
            break
        z, F = zt, Ft
        fnorm = np.max(np.abs(F))
        if fnorm <= residual_tol:
            converged = True
            it += 1
            break
        it += 1
    return z.reshape(nr, nc), converged, it, float(fnorm)


def transient(z_in, mask, cell, bc, D, Sc, dt_total, nonlinear=True, **kw):
    """compute_hillslope_newton_transient (newton_cpu.cpp:690-788) with the
    default controller: dt_init = dt_max = dt_total, grow x1.7 at <= 4
    iterations, shrink x0.5 at >= 15 or on rejection. Returns
    (z float32, n_substeps, total_iterations)."""
    total = float(dt_total)
    dt = total
    dt_min = total * 1e-9
    zn = np.asarray(z_in, np.float32)
    cur = zn.copy()
    remaining = total
    n_sub = 0
    iters = 0
    rejects = 0
    while remaining > 0.0:
        step = min(dt, remaining)
        znew, ok, it, _ = newton_step(cur, zn, mask, cell, bc, D, Sc, 1.0 / step, nonlinear, **kw)
        iters += it
        if not ok:
            rejects += 1
            if rejects > 40 or step <= dt_min:
                raise RuntimeError("Newton failed at the minimum sub-step")
            dt = max(dt_min, step * 0.5)
            continue
        cur = znew.astype(np.float32)
        zn = cur.copy()
        remaining -= step
        n_sub += 1
        if it <= 4:
            dt = min(total, step * 1.7)
        elif it >= 15:
            dt = max(dt_min, step * 0.5)
    return cur, n_sub, iters
