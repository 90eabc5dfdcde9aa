"""Standalone GPU ops with the reference's function signatures.

count_SEIRP mirrors laser_polio.model.count_SEIRP (model.py:869-899): same
name, arguments and result tuple.  It runs the CUDA entry point
lpg_count_seirp (include/lpg.h) on the current device and stream; there is
no CPU fallback.

expected_incidence and IncidencePlan have no counterpart in the reference:
the expected-exposure map of the transmission step with the agent state
held fixed, and its vector-Jacobian product, for gradient-based
calibration (lpg_expected_incidence, lpg_incidence_plan_*).
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _abi
from . import _lib


def _dev(x, dtype):
    if isinstance(x, torch.Tensor):
        if not x.is_cuda:
            raise ValueError("count_SEIRP: tensors must be on a CUDA device")
        t = x
    else:
        t = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    if t.dtype != dtype:
        raise ValueError(f"count_SEIRP: expected {dtype}, got {t.dtype}")
    return t.contiguous()


def count_SEIRP(node_id, disease_state, strain, potentially_paralyzed, paralyzed, n_nodes: int, n_strains: int,
                n_people: int, *, n_invalid: list | None = None):
    """Per-node counts of slots [0, n_people) with disease_state >= 0.

    Returns (S, E, I, R, E_by_strain, I_by_strain, potentially_paralyzed,
    paralyzed) as int32 arrays of shape [n_nodes] or [n_nodes, n_strains]:
    torch CUDA tensors when the columns are torch tensors, numpy arrays when
    they are numpy arrays.  Slots with a node id outside [0, n_nodes) or an
    E/I strain outside [0, n_strains) are skipped; pass a list as
    ``n_invalid`` to receive their number.
    """
    host = not isinstance(disease_state, torch.Tensor)
    cols = [
        _dev(node_id, torch.int16),
        _dev(disease_state, torch.int8),
        _dev(strain, torch.int8),
        _dev(potentially_paralyzed, torch.int8),
        _dev(paralyzed, torch.int8),
    ]
    n_people = int(n_people)
    if any(c.numel() < n_people for c in cols):
        raise ValueError("count_SEIRP: a column is shorter than n_people")
    device = cols[1].device
    with torch.cuda.device(device):
        outs = [torch.empty(int(n_nodes), dtype=torch.int32, device=device) for _ in range(4)]
        ebs = torch.empty((int(n_nodes), int(n_strains)), dtype=torch.int32, device=device)
        ibs = torch.empty_like(ebs)
        potp = torch.empty(int(n_nodes), dtype=torch.int32, device=device)
        par = torch.empty_like(potp)
        bad = torch.zeros(1, dtype=torch.int64, device=device)
        lib = _lib.load()
        stream = torch.cuda.current_stream(device).cuda_stream
        S, E, I, R = outs
        rc = lib.lpg_count_seirp(*[c.data_ptr() for c in cols], int(n_nodes), int(n_strains), n_people,
                                 S.data_ptr(), E.data_ptr(), I.data_ptr(), R.data_ptr(), ebs.data_ptr(),
                                 ibs.data_ptr(), potp.data_ptr(), par.data_ptr(), bad.data_ptr(),
                                 C.c_void_p(stream))
        if rc != 0:
            msg = lib.lpg_op_last_error().decode()
            if rc == -1:
                raise ValueError(msg)
            raise _lib.LpgError(rc, msg)
    res = (S, E, I, R, ebs, ibs, potp, par)
    if n_invalid is not None:
        n_invalid.append(int(bad.item()))
    if host:
        return tuple(t.cpu().numpy() for t in res)
    return res


INCIDENCE_ARRAYS = {"srisk": 2, "beta": 3, "pop": 2, "doy": 1, "year": 1, "r0s": 1, "pops": 1, "dist": 2}
INCIDENCE_SCALARS = ("R", "amp", "peak", "k", "a", "b", "c", "max_frac")
_DP = C.POINTER(C.c_double)


def _raise(lib, rc):
    msg = lib.lpg_op_last_error().decode()
    if rc == -1:
        raise ValueError(msg)
    raise _lib.LpgError(rc, msg)


def _incidence_desc(inp: dict, need_r0s: bool):
    """(lpg_incidence_in, the arrays it points into, (T, G, S)) after shape checks."""
    arrs = {}
    for name, nd in INCIDENCE_ARRAYS.items():
        if name == "r0s" and not need_r0s and inp.get("r0s") is None:
            continue
        a = np.ascontiguousarray(np.asarray(inp[name], dtype=np.float64))
        if a.ndim != nd:
            raise ValueError(f"expected_incidence: {name} must have {nd} dimensions, got {a.ndim}")
        arrs[name] = a
    T, G, S = arrs["beta"].shape
    want = {"srisk": (T, G), "pop": (T, G), "doy": (T,), "year": (T,), "r0s": (G,), "pops": (G,), "dist": (G, G)}
    for name, shape in want.items():
        if name in arrs and arrs[name].shape != shape:
            raise ValueError(f"expected_incidence: {name} has shape {arrs[name].shape}, expected {shape}")
    desc = _abi.lpg_incidence_in(T=T, G=G, S=S)
    for name, a in arrs.items():
        setattr(desc, name, _abi.ptr(a, _DP))
    for name in INCIDENCE_SCALARS:
        if name in inp:
            setattr(desc, name, float(inp[name]))
    return desc, arrs, (T, G, S)


def _grad_out(G):
    out = {"r0s": np.empty(G, np.float64), "network": np.empty((G, G), np.float64)}
    grad = _abi.lpg_incidence_grad(r0s=_abi.ptr(out["r0s"], _DP), network=_abi.ptr(out["network"], _DP))
    return out, grad


def _grad_dict(out, grad):
    for name in _abi.INCIDENCE_SCALAR_GRADS:
        out[name] = float(getattr(grad, name))
    return out


def _check_g(g, T, G):
    gvec = np.ascontiguousarray(np.asarray(g, dtype=np.float64))
    if gvec.shape != (T, G):
        raise ValueError(f"expected_incidence: g has shape {gvec.shape}, expected {(T, G)}")
    return gvec


def expected_incidence(inp: dict, g=None):
    """Expected new exposures lam [T, G] of a replayed tick range and, given
    g = dL/dlam [T, G], the gradients of L = sum(g * lam).

    ``inp`` holds srisk [T, G], beta [T, G, S], pop [T, G], doy [T],
    year [T], r0s [G], pops [G], dist [G, G] and the scalars R, amp, peak,
    k, a, b, c, max_frac; the formula is the transmission step's node-level
    part with the agent state held fixed (model.py:1250-1258, 1315-1363).
    Runs lpg_expected_incidence (include/lpg.h) on the current CUDA device.
    Returns (lam, grads): grads is None without g, else a dict with the
    scalars' gradients and arrays ``r0s`` [G] and ``network`` [G, G] (dL/dN,
    the normalised network).
    """
    desc, _keep, (T, G, _) = _incidence_desc(inp, need_r0s=True)
    lam = np.empty((T, G), np.float64)
    gvec, out, grad = None, None, None
    if g is not None:
        gvec = _check_g(g, T, G)
        out, grad = _grad_out(G)
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream if torch.cuda.is_available() else 0
    rc = lib.lpg_expected_incidence(C.byref(desc), _abi.ptr(lam, _DP), _abi.ptr(gvec, _DP),
                                    C.byref(grad) if grad is not None else None, C.c_void_p(stream))
    if rc != 0:
        _raise(lib, rc)
    return lam, (_grad_dict(out, grad) if grad is not None else None)


class IncidencePlan:
    """The replayed aggregates (and an optional target curve [T, G]) kept
    resident on the current CUDA device (lpg_incidence_plan_* in
    include/lpg.h); ``evaluate`` runs the expected-incidence map and its
    reverse pass at new parameters without re-uploading them."""

    def __init__(self, inp: dict, target=None):
        desc, keep, (T, G, S) = _incidence_desc(inp, need_r0s=False)
        self.T, self.G, self.S = T, G, S
        tgt = None
        if target is not None:
            tgt = _check_g(target, T, G)
        self._lib = _lib.load()
        h = C.c_void_p()
        rc = self._lib.lpg_incidence_plan_create(C.byref(desc), _abi.ptr(tgt, _DP), None, C.byref(h))
        if rc != 0:
            _raise(self._lib, rc)
        self._h = h
        self.has_target = tgt is not None
        del keep

    def evaluate(self, params: dict, g=None, *, lam=False, loss=None, grad=True, network_grad=True):
        """One evaluation at ``params`` (R, amp, peak, k, a, b, c, max_frac,
        r0s [G]).  Returns a dict with ``lam`` (if asked), ``loss`` (a target
        plan; default: when there is a target) and ``grad`` (the gradients of
        sum(g * lam) when g is given, else of the target loss)."""
        r0s = np.ascontiguousarray(np.asarray(params["r0s"], np.float64))
        if r0s.shape != (self.G,):
            raise ValueError(f"expected_incidence: r0s has shape {r0s.shape}, expected {(self.G,)}")
        prm = _abi.lpg_incidence_params(**{n: float(params[n]) for n in INCIDENCE_SCALARS},
                                        r0s=_abi.ptr(r0s, _DP))
        gvec = _check_g(g, self.T, self.G) if g is not None else None
        want_loss = self.has_target if loss is None else loss
        lam_out = np.empty((self.T, self.G), np.float64) if lam else None
        loss_out = C.c_double(0.0)
        out, gstruct = (None, None)
        if grad:
            out, gstruct = _grad_out(self.G)
            if not network_grad:
                gstruct.network = None
                del out["network"]
        rc = self._lib.lpg_incidence_plan_eval(self._h, C.byref(prm), _abi.ptr(gvec, _DP), _abi.ptr(lam_out, _DP),
                                               C.byref(loss_out) if want_loss else None,
                                               C.byref(gstruct) if gstruct is not None else None)
        if rc != 0:
            _raise(self._lib, rc)
        res = {}
        if lam:
            res["lam"] = lam_out
        if want_loss:
            res["loss"] = loss_out.value
        if grad:
            res["grad"] = _grad_dict(out, gstruct)
        return res

    def stream(self) -> int:
        return self._lib.lpg_incidence_plan_stream(self._h) or 0

    def set_profiling(self, enable: bool):
        self._lib.lpg_incidence_plan_set_profiling(self._h, int(enable))

    def profile(self) -> dict:
        """{kernel: (total ms, launches)} of the evaluations since profiling was enabled."""
        pr = _abi.lpg_profile()
        rc = self._lib.lpg_incidence_plan_read_profile(self._h, C.byref(pr))
        if rc != 0:
            _raise(self._lib, rc)
        return {pr.names[i].decode(): (pr.total_ms[i], pr.launches[i]) for i in range(pr.n_kernels)}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lpg_incidence_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


_AUTOGRAD_SCALARS = ("R", "amp", "peak", "k", "a", "b", "c")


class ExpectedIncidence(torch.autograd.Function):
    """lam [T, G] of an IncidencePlan as a differentiable function of the
    scalars R, amp, peak, k, a, b, c (0-dim float64 tensors) and r0s [G].
    forward() evaluates the map; backward() runs the plan's reverse pass
    with the incoming dL/dlam (one lpg_incidence_plan_eval each), so any
    torch loss over lam and any torch optimiser can drive a calibration.
    Use through expected_incidence_torch."""

    @staticmethod
    def forward(ctx, plan, max_frac, R, amp, peak, k, a, b, c, r0s):
        values = (R, amp, peak, k, a, b, c)
        params = {name: float(v) for name, v in zip(_AUTOGRAD_SCALARS, values)}
        params["max_frac"] = float(max_frac)
        params["r0s"] = r0s.detach().to("cpu", torch.float64).contiguous().numpy()
        out = plan.evaluate(params, lam=True, loss=False, grad=False)
        ctx.plan, ctx.params, ctx.device = plan, params, r0s.device
        return torch.as_tensor(out["lam"], dtype=torch.float64, device=r0s.device)

    @staticmethod
    def backward(ctx, g_lam):
        g = g_lam.detach().to("cpu", torch.float64).contiguous().numpy()
        gr = ctx.plan.evaluate(ctx.params, g, loss=False, network_grad=False)["grad"]
        scalars = [torch.tensor(gr[name], dtype=torch.float64, device=ctx.device) for name in _AUTOGRAD_SCALARS]
        return (None, None, *scalars, torch.as_tensor(gr["r0s"], dtype=torch.float64, device=ctx.device))


def expected_incidence_torch(plan, params: dict) -> torch.Tensor:
    """lam = ExpectedIncidence.apply over ``params``: R, amp, peak, k, a, b,
    c as 0-dim tensors (or floats, then constant), r0s as a [G] tensor (or
    array), and max_frac a float.  Gradients flow to every tensor that
    requires them."""

    def t(x):
        return x if isinstance(x, torch.Tensor) else torch.tensor(x, dtype=torch.float64)

    args = [t(params[name]) for name in _AUTOGRAD_SCALARS]
    return ExpectedIncidence.apply(plan, float(params["max_frac"]), *args, t(params["r0s"]))
