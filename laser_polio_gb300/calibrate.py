"""Gradient-based calibration on the expected-incidence adjoint.

No counterpart in the reference: its calibration (calib/objective.py:9-82)
samples parameters with Optuna and scores whole simulations.  Here the
loss L = sum (log1p(lam) - log1p(target))^2 of an IncidencePlan (the
transmission step's expected exposures over replayed aggregates) and its
gradient drive scipy's L-BFGS-B over any subset of R, amp, peak, k, a, b, c
and, optionally, the per-node r0 scalars.
"""

from __future__ import annotations

import numpy as np

SCALARS = ("R", "amp", "peak", "k", "a", "b", "c")


def fit_incidence(plan, params: dict, free=("R", "amp", "peak"), fit_r0s: bool = False, bounds: dict | None = None,
                  r0s_bounds=(1e-6, None), maxiter: int = 200, tol: float = 1e-12):
    """Minimise ``plan``'s target loss from ``params`` (R, amp, peak, k, a,
    b, c, max_frac, r0s) over the ``free`` scalars and, with ``fit_r0s``, the
    r0 scalars.  ``plan`` is an ``ops.IncidencePlan`` made with a target (or
    any object with its ``evaluate`` method).  ``bounds`` maps a free name to
    (low, high), None for unbounded.

    Returns (params at the minimum, scipy OptimizeResult)."""
    from scipy.optimize import minimize

    free = tuple(free)
    unknown = [n for n in free if n not in SCALARS]
    if unknown:
        raise ValueError(f"fit_incidence: unknown parameters {unknown}; choose from {SCALARS}")
    if not free and not fit_r0s:
        raise ValueError("fit_incidence: nothing to fit")
    base = dict(params)
    r0s0 = np.asarray(base["r0s"], np.float64)
    bounds = dict(bounds or {})

    def unpack(x):
        p = dict(base)
        for i, name in enumerate(free):
            p[name] = float(x[i])
        p["r0s"] = np.asarray(x[len(free):], np.float64) if fit_r0s else r0s0
        return p

    def fun(x):
        out = plan.evaluate(unpack(x), network_grad=False)
        g = [out["grad"][name] for name in free]
        if fit_r0s:
            g = np.concatenate([np.asarray(g, np.float64), out["grad"]["r0s"]])
        return out["loss"], np.asarray(g, np.float64)

    x0 = [float(base[name]) for name in free]
    bnd = [bounds.get(name, (None, None)) for name in free]
    if fit_r0s:
        x0 = np.concatenate([np.asarray(x0, np.float64), r0s0])
        bnd += [r0s_bounds] * len(r0s0)
    res = minimize(fun, np.asarray(x0, np.float64), jac=True, method="L-BFGS-B", bounds=bnd,
                   options={"maxiter": maxiter, "ftol": tol, "gtol": tol})
    return unpack(res.x), res
