"""Distribution objects for timer parameters (laser_polio/distributions.py:17-151).

``Distribution.sample`` draws with numpy on the host, as the reference does at
initialisation (model.py:575-587).  ``Distribution.spec`` is the same
distribution as plain numbers for the C ABI (lpg_dist), used where the device
must draw from it during a run (timers of seeded agents, model.py:777).
"""

from __future__ import annotations

import numpy as np

from ._abi import DIST_KINDS

dist_list = ["constant", "exponential", "gamma", "lognormal", "normal", "poisson", "uniform"]
__all__ = ["Distribution", *dist_list, "lognormal_int"]


class Distribution:
    def __init__(self, dist_type, **pars):
        self.dist_type = dist_type
        self.pars = pars
        supported = {"constant", "exponential", "gamma", "lognormal", "normal", "poisson", "uniform", "lognormal_int"}
        if dist_type not in supported:
            raise ValueError(f"Unsupported distribution: {dist_type}. Supported: {supported}")

    def sample(self, size=1):
        dist = self.dist_type
        if dist == "constant":
            return np.full(size, self.pars.get("value", 1))
        if dist == "exponential":
            return np.random.exponential(self.pars.get("scale", 1.0), size)
        if dist == "gamma":
            return np.random.gamma(self.pars.get("shape", 2.0), self.pars.get("scale", 1.0), size)
        if dist in ("lognormal", "lognormal_int"):
            par1 = self.pars.get("mean", 1.0)
            par2 = self.pars.get("sigma", 0.5)
            if par1 > 0:
                mean = np.log(par1**2 / np.sqrt(par2**2 + par1**2))
                sigma = np.sqrt(np.log(par2**2 / par1**2 + 1))
                samples = np.random.lognormal(mean=mean, sigma=sigma, size=size)
            else:
                samples = np.zeros(size)
            if dist == "lognormal_int":
                samples = np.round(samples)
            return samples
        if dist == "normal":
            return np.random.normal(self.pars.get("mean", 0.0), self.pars.get("std", 1.0), size)
        if dist == "poisson":
            return np.random.poisson(self.pars.get("lam", 5), size)
        if dist == "uniform":
            return np.random.randint(self.pars.get("min", 2), self.pars.get("max", 10), size)
        raise ValueError(f"Unsupported distribution type: {dist}")

    def __call__(self, size=1):
        return self.sample(size)

    def spec(self):
        """(kind, p1, p2) in the layout of lpg_dist."""
        d, p = self.dist_type, self.pars
        if d == "constant":
            return DIST_KINDS[d], float(p.get("value", 1)), 0.0
        if d == "exponential":
            return DIST_KINDS[d], float(p.get("scale", 1.0)), 0.0
        if d == "gamma":
            return DIST_KINDS[d], float(p.get("shape", 2.0)), float(p.get("scale", 1.0))
        if d in ("lognormal", "lognormal_int"):
            return DIST_KINDS[d], float(p.get("mean", 1.0)), float(p.get("sigma", 0.5))
        if d == "normal":
            return DIST_KINDS[d], float(p.get("mean", 0.0)), float(p.get("std", 1.0))
        if d == "poisson":
            return DIST_KINDS[d], float(p.get("lam", 5)), 0.0
        if d == "uniform":
            return DIST_KINDS[d], float(p.get("min", 2)), float(p.get("max", 10))
        raise ValueError(d)

    def __repr__(self):
        return f"Distribution(type={self.dist_type}, pars={self.pars})"


def constant(value):
    return Distribution("constant", value=value)


def exponential(scale):
    return Distribution("exponential", scale=scale)


def gamma(shape, scale):
    return Distribution("gamma", shape=shape, scale=scale)


def lognormal(mean, sigma):
    return Distribution("lognormal", mean=mean, sigma=sigma)


def lognormal_int(mean, sigma):
    return Distribution("lognormal_int", mean=mean, sigma=sigma)


def normal(mean, std):
    return Distribution("normal", mean=mean, std=std)


def poisson(lam):
    return Distribution("poisson", lam=lam)


def uniform(min, max):
    return Distribution("uniform", min=min, max=max)
