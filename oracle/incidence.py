"""Expected incidence and its vector-Jacobian product, in numpy (FP64).

Test infrastructure: the checker of the device kernels in
laser_polio_gb300/csrc/lpg_adjoint.cu.  It restates the node-level part of
the transmission step (model.py:1315-1363) with the agent state held fixed:
per tick t, node n, strain s

    N       = rownorm(gravity(p, d, k, a, b, c) / (sum p)^c, m)          model.py:1250-1258
    u[t,n,s] = beta[t,n,s] (1 - sum_k N[n,k]) + sum_i N[i,n] beta[t,i,s]  model.py:1335-1338
    seas[t] = 1 + amp cos(2 pi (doy[t] - peak) / year[t])                 utils.py:589-625
    r       = u seas[t] r0s[n] R / max(pop[t,n], 1)                       model.py:1339-1347
    lam[t,n] = srisk[t,n] sum_s (1 - exp(-r))                             model.py:1348-1363

(R scales every agent's infectivity: R0 / R0_ref).  Pinned against the C oracle
of the agent step (lpg_oracle.c, lpo_record_aggregates): on the aggregates
that oracle mixes, forward() reproduces its expected exposures per tick and
node (tests/test_adjoint.py).  The reverse pass gives,
for an upstream gradient g[t,n] = dL/dlam[t,n], the gradients of L with
respect to R, amp, peak, r0s[n], the network N[a,b] and the gravity
parameters k, a, b, c.  gravity[i,j] = k p_i^a p_j^b / d_ij^c with a zero
diagonal; rownorm scales a row whose sum exceeds m down to m.
"""

from __future__ import annotations

import numpy as np


def network(pops, dist, k, a, b, c, max_frac):
    """(N, G, rs, capped): the normalised network, the scaled gravity flows
    G = gravity / P^c, their row sums and the rows that were scaled down."""
    p = np.asarray(pops, np.float64)
    d = np.asarray(dist, np.float64)
    n = len(p)
    P = p.sum()
    off = ~np.eye(n, dtype=bool)
    G = np.zeros((n, n))
    with np.errstate(divide="ignore", invalid="ignore"):
        val = k * p[:, None] ** a * p[None, :] ** b / d**c / P**c
    G[off] = val[off]
    G[~np.isfinite(G)] = 0.0
    rs = G.sum(axis=1)
    capped = rs > max_frac
    N = G.copy()
    N[capped] = G[capped] * (max_frac / rs[capped])[:, None]
    return N, G, rs, capped


def forward(srisk, beta, pop, doy, year, r0s, R, amp, peak, N):
    """lam [T, G] and the intermediates of the reverse pass."""
    rsN = N.sum(axis=1)
    # sum_i N[i,n] beta[t,i,s] as one BLAS product (np.tensordot), not einsum's loops
    u = beta * (1.0 - rsN)[None, :, None] + np.tensordot(N, beta, axes=([0], [1])).transpose(1, 0, 2)
    ang = 2.0 * np.pi * (doy - peak) / year
    seas = 1.0 + amp * np.cos(ang)
    q = seas[:, None] * r0s[None, :] * R / np.maximum(pop, 1.0)
    r = u * q[:, :, None]
    e = np.exp(-r)
    lam = srisk * (1.0 - e).sum(axis=2)
    return lam, dict(u=u, ang=ang, seas=seas, q=q, e=e)


def backward(g, srisk, beta, pop, doy, year, r0s, R, amp, peak, N, mid, pops, dist, k, a, b, c, max_frac, G, rs, capped):
    """Gradients of L = sum g * lam."""
    u, e, q, seas, ang = mid["u"], mid["e"], mid["q"], mid["seas"], mid["ang"]
    gr = (g * srisk)[:, :, None] * e  # dL/dr
    gu = gr * q[:, :, None]
    gq = (gr * u).sum(axis=2)  # [T, G]
    popc = np.maximum(pop, 1.0)
    g_seas = (gq * r0s[None, :] * R / popc).sum(axis=1)
    g_r0s = (gq * seas[:, None] * R / popc).sum(axis=0)
    g_R = (gq * seas[:, None] * r0s[None, :] / popc).sum()
    g_amp = (g_seas * np.cos(ang)).sum()
    g_peak = (g_seas * amp * np.sin(ang) * 2.0 * np.pi / year).sum()
    # u[n] = beta[n] (1 - sum_k N[n,k]) + sum_i N[i,n] beta[i]
    gN = np.tensordot(beta, gu, axes=([0, 2], [0, 2])) - np.einsum("tas,tas->a", beta, gu)[:, None]
    np.fill_diagonal(gN, 0.0)
    # through rownorm: capped rows N = m G / rs
    gG = gN.copy()
    if capped.any():
        rc = rs[capped]
        gNc = gN[capped]
        Gc = G[capped]
        gG[capped] = (max_frac / rc)[:, None] * (gNc - ((gNc * Gc).sum(axis=1) / rc)[:, None])
    p = np.asarray(pops, np.float64)
    d = np.asarray(dist, np.float64)
    P = p.sum()
    n = len(p)
    off = ~np.eye(n, dtype=bool)
    with np.errstate(divide="ignore"):
        lp = np.log(p)
    with np.errstate(divide="ignore"):
        ld = np.where(off, np.log(np.where(off, d, 1.0)), 0.0)
    w = gG * G
    nz = w != 0.0  # a zero flow contributes nothing; its logs may be infinite
    with np.errstate(invalid="ignore"):
        g_k = w.sum() / k
        g_a = np.where(nz, w * lp[:, None], 0.0).sum()
        g_b = np.where(nz, w * lp[None, :], 0.0).sum()
        g_c = np.where(nz, w * (-ld - np.log(P)), 0.0).sum()
    return dict(R=g_R, amp=g_amp, peak=g_peak, r0s=g_r0s, network=gN, k=g_k, a=g_a, b=g_b, c=g_c)


def incidence(inp, g=None):
    """lam and, with g, the gradients: inp holds srisk [T,G], beta [T,G,S],
    pop [T,G], doy [T], year [T], r0s [G], R, amp, peak, pops [G],
    dist [G,G], k, a, b, c, max_frac."""
    N, G, rs, capped = network(inp["pops"], inp["dist"], inp["k"], inp["a"], inp["b"], inp["c"], inp["max_frac"])
    args = (inp["srisk"], inp["beta"], inp["pop"], inp["doy"], inp["year"], inp["r0s"], inp["R"], inp["amp"],
            inp["peak"], N)
    lam, mid = forward(*args)
    if g is None:
        return lam, None
    grads = backward(g, *args, mid, inp["pops"], inp["dist"], inp["k"], inp["a"], inp["b"], inp["c"],
                     inp["max_frac"], G, rs, capped)
    return lam, grads


def random_inputs(T, Gn, S, seed=0):
    """Seeded node-level aggregates of the shapes a replayed run produces."""
    rng = np.random.default_rng(seed)
    pops = rng.lognormal(np.log(5e4), 0.7, Gn)
    xy = rng.uniform(0, 300, (Gn, 2))
    dist = np.sqrt(((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1))
    dist[np.eye(Gn, dtype=bool)] = 0.0
    dist = np.where(np.eye(Gn, dtype=bool), 0.0, np.maximum(dist, 1.0))
    pop = pops[None, :] * (1.0 + 0.001 * np.arange(T))[:, None]
    return dict(
        srisk=pop * rng.uniform(0.1, 0.6, (T, Gn)),
        beta=rng.gamma(0.5, 20.0, (T, Gn, S)) * (rng.uniform(size=(T, Gn, S)) < 0.7),
        pop=pop,
        doy=(np.arange(T) % 365).astype(np.float64) + 1.0,
        year=np.full(T, 365.0),
        r0s=rng.lognormal(0.0, 0.3, Gn),
        R=1.1,
        amp=0.4,
        peak=180.0,
        pops=pops,
        dist=dist,
        k=0.5,
        a=1.0,
        b=1.0,
        c=2.0,
        max_frac=0.2,
    )
