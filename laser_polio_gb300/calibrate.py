"""Calibration around the per-tick step.

  - replicate_objective: the reference's objective (calib/objective.py:9-82)
    runs a trial's replicates one after another, each in its own
    try/except, scores each and returns the mean.  Here the replicates run
    as one batch (engine.run_replicates: one handle, one launch sequence a
    tick), with the same per-replicate reporting and the same mean.
  - fit_incidence: no counterpart in the reference.  The loss L = sum
    (log1p(lam) - log1p(target))^2 of an IncidencePlan (the transmission
    step's expected exposures over replayed aggregates) and its gradient
    drive scipy's L-BFGS-B over any subset of R, amp, peak, k, a, b, c and,
    optionally, the per-node r0 scalars.
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


def replicate_objective(make_sim, params: dict, score, n_replicates: int = 1, autotune: bool = False,
                        log=print) -> dict:
    """One calibration trial: ``n_replicates`` simulations of the suggested
    ``params``, run as one batch, each scored.

    ``make_sim(params, rep)`` returns a SEIR_ABM with the drop-in
    components (its own seed for each replicate); ``score(sim)`` returns the
    replicate's fit score (the reference's total log-likelihood).  As in the
    reference's objective loop, a replicate whose construction, run or
    scoring fails is reported through ``log`` and left out, and the trial's
    value is the mean of the others' scores (NaN when none is left).

    Returns {"value", "scores", "seeds", "errors"}: the mean, the scores
    and seeds of the replicates that scored, and (replicate, exception) for
    the others."""
    from . import engine

    sims, reps, errors = [], [], []
    for rep in range(int(n_replicates)):
        try:
            sims.append(make_sim(dict(params), rep))
            reps.append(rep)
        except Exception as exc:  # noqa: BLE001 - reported and skipped, as the reference does
            log(f"replicate {rep}: could not be built: {exc}")
            errors.append((rep, exc))
    run_errors = engine.run_replicates(sims, autotune=autotune) if sims else []
    scores, seeds = [], []
    for rep, sim, err in zip(reps, sims, run_errors):
        if err is not None:
            log(f"replicate {rep}: the simulation failed: {err}")
            errors.append((rep, err))
            continue
        try:
            scores.append(float(score(sim)))
            seeds.append(getattr(getattr(sim, "pars", None), "seed", None))
        except Exception as exc:  # noqa: BLE001
            log(f"replicate {rep}: scoring failed: {exc}")
            errors.append((rep, exc))
    value = float(np.mean(scores)) if scores else float("nan")
    return {"value": value, "scores": scores, "seeds": seeds, "errors": sorted(errors, key=lambda e: e[0])}
