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


def linear_step(z, mask, cell, bc, D, dt, U=0.0, residual_tol=1e-12, max_newton=50, is_channel=None):
    """One backward-Euler step of linear hillslope diffusion over dt.
    Returns (z_new float32, n_newton, final ||F||_inf)."""
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
    lu = spla.splu(J)
    zz = zn.copy()
    F = residual(zz)
    it = 0
    while np.max(np.abs(F)) > residual_tol and it < max_newton:
        zz[idx] += lu.solve(-F)
        F = residual(zz)
        it += 1
    return zz.astype(np.float32).reshape(nr, nc), it, float(np.max(np.abs(F))) if F.size else 0.0
