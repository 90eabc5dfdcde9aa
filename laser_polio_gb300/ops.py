"""Standalone GPU ops with the reference's function signatures.

count_SEIRP mirrors laser_polio.model.count_SEIRP (model.py:869-899): same
name, arguments and result tuple.  It runs the CUDA entry point
lpg_count_seirp (include/lpg.h) on the current device and stream; there is
no CPU fallback.
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
    arrs = {}
    for name, nd in INCIDENCE_ARRAYS.items():
        a = np.ascontiguousarray(np.asarray(inp[name], dtype=np.float64))
        if a.ndim != nd:
            raise ValueError(f"expected_incidence: {name} must have {nd} dimensions, got {a.ndim}")
        arrs[name] = a
    T, G, S = arrs["beta"].shape
    want = {"srisk": (T, G), "pop": (T, G), "doy": (T,), "year": (T,), "r0s": (G,), "pops": (G,), "dist": (G, G)}
    for name, shape in want.items():
        if arrs[name].shape != shape:
            raise ValueError(f"expected_incidence: {name} has shape {arrs[name].shape}, expected {shape}")
    desc = _abi.lpg_incidence_in(T=T, G=G, S=S)
    dp = C.POINTER(C.c_double)
    for name, a in arrs.items():
        setattr(desc, name, _abi.ptr(a, dp))
    for name in INCIDENCE_SCALARS:
        setattr(desc, name, float(inp[name]))
    lam = np.empty((T, G), np.float64)
    grad = None
    gvec = None
    out = None
    if g is not None:
        gvec = np.ascontiguousarray(np.asarray(g, dtype=np.float64))
        if gvec.shape != (T, G):
            raise ValueError(f"expected_incidence: g has shape {gvec.shape}, expected {(T, G)}")
        out = {"r0s": np.empty(G, np.float64), "network": np.empty((G, G), np.float64)}
        grad = _abi.lpg_incidence_grad(r0s=_abi.ptr(out["r0s"], dp), network=_abi.ptr(out["network"], dp))
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream if torch.cuda.is_available() else 0
    rc = lib.lpg_expected_incidence(C.byref(desc), _abi.ptr(lam, dp), _abi.ptr(gvec, dp),
                                    C.byref(grad) if grad is not None else None, C.c_void_p(stream))
    if rc != 0:
        msg = lib.lpg_op_last_error().decode()
        if rc == -1:
            raise ValueError(msg)
        raise _lib.LpgError(rc, msg)
    if grad is None:
        return lam, None
    for name in _abi.INCIDENCE_SCALAR_GRADS:
        out[name] = float(getattr(grad, name))
    return lam, out
