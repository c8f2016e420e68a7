"""FP64 CPU reference gradients of the density map w -> rho (the pullback of density!) and of
free_energy at fixed fields.

TEST INFRASTRUCTURE ONLY, like pf_oracle.py: the checker the GPU adjoint is compared
against.  PolyFields.jl has no derivative code; this module differentiates the oracle's
restatement of density! (src/species/multiblock.jl:125-231, src/system/system.jl:266-289,
src/species/point.jl:36-58) by hand and is itself pinned to central finite differences of
that density in tests/test_adjoint_oracle.py.

Given rho_bar[m] = dL/drho_m for the pooled densities rho_m of a FieldSystem after
density_update(), ``density_pullback`` returns dL/dw_m for every monomer, dL/dtheta for the
cell parameters, dL/dNref_b for every block of every Multiblock species (block lengths
varied with the contour step counts held fixed, ds_b = Nref_b / Ns_b -- the continuous
relaxation of the composition f), and dL/dchi = 0 (chi does not enter rho at fixed w).

The chain operator of a block is A = LW . irfft(LD . rfft(LW . )) with LW = exp(-ds vol w/2)
and LD = exp(-ds b^2 k^2 / 6).  It is symmetric (LD is real and even in k), so the adjoint
of q_{t+1} = A q_t runs the same operator backward: lambda_t = A lambda_{t+1} + dL/dq_t.
For one application y = A x with adjoint ybar:
    dL/dw      += -(ds vol / 2) (ybar * y + x * A ybar)
    dL/dLD_k   += (c_k / Ng) Re(rfft(LW x)_k conj(rfft(LW ybar)_k)),
c_k = 1 on the kx = 0 and kx = Nx/2 planes and 2 elsewhere (the Hermitian multiplicity).
"""
from __future__ import annotations

from typing import Dict

import numpy as np

import pf_oracle as O


def simpson_weights(n: int) -> np.ndarray:
    """Weights of the reference's block Simpson sum over n+1 contour points
    (multiblock.jl:209-222): 1 at both ends, 4 at odd offsets, 2 at even interior offsets."""
    w = np.zeros(n + 1)
    w[0] += 1.0
    w[n] += 1.0
    for s in range(1, n, 2):
        w[s] += 4.0
    for s in range(2, n - 1, 2):
        w[s] += 2.0
    return w


def hermitian_multiplicity(shape) -> np.ndarray:
    """c_k of the half spectrum of a real grid of `shape` (Nz, Ny, Nx): 1 on kx = 0 and
    kx = Nx/2 (Nx even), 2 elsewhere."""
    nx = shape[2]
    kx = nx // 2 + 1
    c = np.full(kx, 2.0)
    c[0] = 1.0
    if nx % 2 == 0:
        c[-1] = 1.0
    return np.broadcast_to(c, (shape[0], shape[1], kx))


def _apply(sys, w, vol, b, ds, x):
    solver = O.PseudoSpectralSolver(sys.dims)
    solver.update(w, sys.cell.ksq, vol, b, ds)
    y = np.empty_like(x)
    solver.propagate(x, y)
    return y, solver


def _step_grads(sys, solver, vol, b, ds, w, x, y, ybar, ax_ybar, grads, m, iblk, kshape, cmult):
    """Accumulate the gradients of one application y = A x (A ybar = ax_ybar)."""
    ng = sys.ngrid
    prod = ybar * y + x * ax_ybar
    grads["w"][m] += -(ds * vol / 2.0) * prod
    gds = float(np.sum(-(vol * w / 2.0) * prod))
    X = O._rfftn(solver.LW1 * x, 1)
    Y = O._rfftn(solver.LW1 * ybar, 1)
    dld = cmult * (X.real * Y.real + X.imag * Y.imag) / ng          # dL/dLD_k
    ksq = np.broadcast_to(sys.cell.ksq, kshape)
    gds += float(np.sum(dld * solver.LD1 * (-(b * b) * ksq / 6.0)))
    for p in range(sys.cell.nparams):
        dk = np.broadcast_to(sys.cell.dksq[p], kshape)
        grads["cell"][p] += float(np.sum(dld * solver.LD1 * (-(ds * b * b / 6.0)) * dk))
    return gds


def density_pullback(sys, rho_bar: Dict[int, np.ndarray]) -> Dict:
    """dL/d(w, cell, Nref_b, chi) for a loss L with dL/drho_m = rho_bar[m] (pooled densities).
    ``sys`` must have run density_update() for its current fields and cell."""
    kshape = sys.kshape
    cmult = hermitian_multiplicity(sys.shape)
    grads = {"w": {mid: np.zeros(sys.shape) for mid in sys.monomers},
             "cell": np.zeros(sys.cell.nparams), "Nref_block": [], "chi": {}}
    for itx in sys.interactions:
        for key in getattr(itx, "chis", {}):
            grads["chi"][key] = 0.0
    for isp, sp in enumerate(sys.species):
        phi = sys.phi_species[isp]
        g = {mid: phi * np.asarray(rho_bar.get(mid, np.zeros(sys.shape)), dtype=np.float64) for mid in sp.mids}
        if isinstance(sp, O.Point):
            mid = sp.mids[0]
            vol = sys.monomers[mid].vol
            rho = sp.density[mid]
            S = float(np.sum(g[mid] * rho))
            boltz = np.exp(-vol * sys.fields[mid])
            grads["w"][mid] += -vol * rho * g[mid] + S * vol * boltz / (sys.ngrid * sp.Q)
            grads["Nref_block"].append([])
            continue
        q, qc, Q, Nref, Ns = sp.q, sp.qc, sp.Q, sp.Nref, sp.Ns
        nb = sp.nblocks
        bounds = [(sp.begin_block[i] - 1, sp.begin_block[i + 1] - 1) for i in range(nb)]  # 0-based [bgn, end]
        # direct sources dL/dq_s and dL/dqc_s from the Simpson sums
        a = [np.zeros(sys.shape) for _ in range(Ns + 1)]
        c = [np.zeros(sys.shape) for _ in range(Ns + 1)]
        S = 0.0
        dds = [0.0] * nb
        for i, (b0, b1) in enumerate(bounds):
            m = sp.mid_block[i]
            kap = sp.ds_block[i] / 3.0 / (Q * Nref)
            wts = simpson_weights(b1 - b0)
            rho_blk = np.zeros(sys.shape)
            for s in range(b0, b1 + 1):
                coef = kap * wts[s - b0]
                a[s] += coef * g[m] * qc[s]
                c[s] += coef * g[m] * q[s]
                rho_blk += coef * q[s] * qc[s]
            contrib = float(np.sum(g[m] * rho_blk))
            S += contrib
            dds[i] += contrib / sp.ds_block[i]  # Simpson prefactor ds/3
        a[Ns] += (-S / Q) / sys.ngrid  # through Q = mean(q_Ns)
        if nb == 1:  # homopolymer: qc_s = q_{Ns-s}
            for s in range(Ns + 1):
                a[Ns - s] += c[s]
        # forward chain, adjoint walks t = Ns-1 .. 0
        lam = a[Ns].copy()
        for t in range(Ns - 1, -1, -1):
            i = next(k for k, (b0, b1) in enumerate(bounds) if b0 <= t < b1)
            m = sp.mid_block[i]
            vol = sys.monomers[m].vol
            w = sys.fields[m]
            r, solver = _apply(sys, w, vol, sp.b_block[i], sp.ds_block[i], lam)
            dds[i] += _step_grads(sys, solver, vol, sp.b_block[i], sp.ds_block[i], w, q[t], q[t + 1], lam, r,
                                  grads, m, i, kshape, cmult)
            lam = r + a[t]
        if nb > 1:
            # backward chain qc_{s-1} = A qc_s, adjoint walks s = 1 .. Ns
            mu = c[0].copy()
            for s in range(1, Ns + 1):
                i = next(k for k, (b0, b1) in enumerate(bounds) if b0 < s <= b1)
                m = sp.mid_block[i]
                vol = sys.monomers[m].vol
                w = sys.fields[m]
                r, solver = _apply(sys, w, vol, sp.b_block[i], sp.ds_block[i], mu)
                dds[i] += _step_grads(sys, solver, vol, sp.b_block[i], sp.ds_block[i], w, qc[s], qc[s - 1], mu, r,
                                      grads, m, i, kshape, cmult)
                mu = r + c[s]
        # ds_b = Nref_b / Ns_b and rho ~ 1 / Nref with Nref = sum_b Nref_b
        grads["Nref_block"].append([dds[i] / (bounds[i][1] - bounds[i][0]) - S / Nref for i in range(nb)])
    return grads


def free_energy_pullback(sys) -> Dict:
    """d free_energy / d(w, cell, Nref_b, chi, u) at fixed fields, for a canonical system that
    has run density_update().  free_energy (src/system/system.jl:402-433, as restated in
    pf_oracle: translational term with mu = phi, -<rho w>, interaction energies) depends on w
    directly through -sum rho w / Ng and through rho(w); on chi and u only through the
    interaction energies (src/interactions/flory.jl:39-59, edwards.jl:34-60); on the block
    lengths through rho and through the translational term phi (phi - 1) / Nref."""
    ng = sys.ngrid
    vol = {m: sys.monomers[m].vol for m in sys.monomers}
    rho = sys.density
    rbar = {m: -sys.fields[m] / ng for m in sys.monomers}
    chi_bar, u_bar = {}, {}
    for itx in sys.interactions:
        if isinstance(itx, O.FloryInteraction):
            for (a, b), chi in itx.chis.items():
                if a in sys.monomers and b in sys.monomers:
                    rbar[a] = rbar[a] + chi * rho[b] / (vol[a] * vol[b]) / ng
                    rbar[b] = rbar[b] + chi * rho[a] / (vol[a] * vol[b]) / ng
                    chi_bar[(a, b)] = float(np.sum(rho[a] * rho[b])) / (vol[a] * vol[b]) / ng
        elif isinstance(itx, O.EdwardsInteraction):
            for m, u in itx.uvals.items():
                if m in sys.monomers:
                    rbar[m] = rbar[m] + u * rho[m] / vol[m] ** 2 / ng
                    u_bar[m] = float(np.sum(0.5 * (rho[m] / vol[m]) ** 2)) / ng
    g = density_pullback(sys, rbar)
    for m in sys.monomers:
        g["w"][m] = g["w"][m] - rho[m] / ng
    g["chi"] = chi_bar
    g["u"] = u_bar
    for isp, sp in enumerate(sys.species):
        phi = sys.phi_species[isp]
        if isinstance(sp, O.Multiblock) and phi > 1e-8:
            g["Nref_block"][isp] = [v - phi * (phi - 1.0) / sp.Nref ** 2 for v in g["Nref_block"][isp]]
    return g


def density_loss(sys, mid: int, target: np.ndarray):
    """L = sum_x (rho_mid - target)^2 and its rho_bar."""
    d = sys.density[mid] - target
    return float(np.sum(d * d)), {mid: 2.0 * d}


def smooth_target(shape, mean: float, amp: float = 0.2, nmodes: int = 5, seed: int = 12345) -> np.ndarray:
    """A seeded smooth field: `mean` plus the `nmodes` lowest-|k| cosine modes (excluding
    k = 0; ties broken by index order) with PCG64 amplitudes and phases, scaled so that the
    largest deviation from the mean is `amp`."""
    nz, ny, nx = shape
    rng = np.random.Generator(np.random.PCG64(seed))
    ks = []
    for kz in range(-(nz // 2), nz // 2 + 1):
        for ky in range(-(ny // 2), ny // 2 + 1):
            for kx in range(0, nx // 2 + 1):
                if (kx, ky, kz) == (0, 0, 0):
                    continue
                if kx == 0 and (ky < 0 or (ky == 0 and kz < 0)):
                    continue  # one of each +-k pair
                if (nz == 1 and kz != 0) or (ny == 1 and ky != 0):
                    continue
                ks.append((kx * kx + ky * ky + kz * kz, kx, ky, kz))
    ks.sort()
    z, y, x = np.meshgrid(np.arange(nz) / nz, np.arange(ny) / ny, np.arange(nx) / nx, indexing="ij")
    f = np.zeros(shape)
    for _, kx, ky, kz in ks[:nmodes]:
        f += rng.uniform(0.5, 1.0) * np.cos(2 * np.pi * (kx * x + ky * y + kz * z) + rng.uniform(0, 2 * np.pi))
    f *= amp / max(np.max(np.abs(f)), 1e-300)
    return mean + f
