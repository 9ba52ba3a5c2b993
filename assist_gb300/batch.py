"""Batched device API: many independent particles, each with its own time,
adaptive IAS15 step and integration length (no ASSIST counterpart: ASSIST
integrates one REBOUND simulation at a time on one CPU core).

Host-array entry points take numpy arrays; ``*_device`` entry points take
torch CUDA tensors (torch is used only for device memory and streams).
"""
from __future__ import annotations

from ctypes import byref, c_int, c_void_p
from typing import Optional

import numpy as np

from ._lib import BatchStats, D, I, Options, TuneResult, clib, last_error
from .ephem import Ephem


def options(**kw) -> Options:
    """ASSIST's defaults (src/assist.c:408-447) overridden by keyword arguments:
    forces, gr_eih_sources, geocentric, alpha, nk, nm, nn, r0, epsilon, min_dt,
    dt0, max_steps, warm_start, threads_per_block, group_steps, dt_floor,
    group_order, blocks_per_sm, ephem_staging (struct assist_gb300_options in assist.h)."""
    o = Options()
    clib.assist_gb300_default_options(byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError("unknown option %r" % k)
        setattr(o, k, v)
    return o


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(D)


def integrate_batch(ephem: Ephem, t0, t_end, state, params=None, var_state=None, opts: Optional[Options] = None):
    """Integrate n independent particles (state: (n, 6) barycentric AU, AU/day)
    from t0[i] to t_end[i] (days relative to ephem.jd_ref).  var_state, if
    given, is (n, 6, 6): six first-order variational states per particle.
    Returns (state_out, var_out, status, stats_dict)."""
    o = opts or options()
    st = np.ascontiguousarray(state, dtype=np.float64).reshape(-1, 6).copy()
    n = st.shape[0]
    t0 = np.ascontiguousarray(np.broadcast_to(np.asarray(t0, np.float64), (n,))).copy()
    te = np.ascontiguousarray(np.broadcast_to(np.asarray(t_end, np.float64), (n,))).copy()
    prm = None if params is None else np.ascontiguousarray(params, dtype=np.float64).reshape(n, 3).copy()
    nv = 0
    var = None
    if var_state is not None:
        var = np.ascontiguousarray(var_state, dtype=np.float64).reshape(n, 6, 6).copy()
        nv = 6
    status = np.zeros(n, dtype=np.int32)
    stats = BatchStats()
    rc = clib.assist_gb300_integrate_batch(byref(ephem), byref(o), n, _p(t0), _p(te), _p(st), _p(prm), nv,
                                           _p(var), status.ctypes.data_as(I), byref(stats))
    if rc != 0:
        raise RuntimeError("assist_gb300_integrate_batch failed (%d): %s" % (rc, last_error()))
    return st, var, status, {f: getattr(stats, f) for f, _ in BatchStats._fields_}


def _ptr(t):
    return None if t is None else c_void_p(t.data_ptr())


def integrate_batch_device(ephem: Ephem, t0, t_end, state, params=None, var_state=None, status=None,
                           opts: Optional[Options] = None, stream=None):
    """Device-resident variant: torch CUDA float64 tensors, state overwritten in place."""
    o = opts or options()
    n = state.shape[0]
    nv = 0 if var_state is None else 6
    stats = BatchStats()
    s = None if stream is None else c_void_p(stream.cuda_stream)
    rc = clib.assist_gb300_integrate_batch_device(byref(ephem), byref(o), n, _ptr(t0), _ptr(t_end), _ptr(state),
                                                  _ptr(params), nv, _ptr(var_state), _ptr(status), s, byref(stats))
    if rc != 0:
        raise RuntimeError("assist_gb300_integrate_batch_device failed (%d): %s" % (rc, last_error()))
    return {f: getattr(stats, f) for f, _ in BatchStats._fields_}


def autotune_device(ephem: Ephem, t0, t_end, state, params=None, var_state=None, opts: Optional[Options] = None,
                    stream=None) -> dict:
    """Time the default batched kernel's builds on this batch (torch CUDA
    tensors; the states are copied, not changed) and record the fastest for
    batches of its signature (assist_gb300_autotune_device).  Returns the
    chosen build (2, 3: plain, blocks per SM; 4: plain, two with the staged
    .440 record; 5: the learned warm start, a candidate when opts.warm_start
    is set), each candidate's kernel time and the signature."""
    o = opts or options()
    r = TuneResult()
    s = None if stream is None else c_void_p(stream.cuda_stream)
    rc = clib.assist_gb300_autotune_device(byref(ephem), byref(o), state.shape[0], _ptr(t0), _ptr(t_end), _ptr(state),
                                           _ptr(params), 0 if var_state is None else 6, _ptr(var_state), s, byref(r))
    if rc != 0:
        raise RuntimeError("assist_gb300_autotune_device failed (%d): %s" % (rc, last_error()))
    names = {2: "2 blocks/SM", 3: "3 blocks/SM", 4: "2 blocks/SM + staged .440 record", 5: "learned warm start"}
    return {"chosen": r.chosen, "chosen_name": names.get(r.chosen, "?"),
            "candidates_ms": {names[r.candidate[k]]: r.kernel_ms[k] for k in range(r.n_candidates)},
            "signature": r.signature.decode()}


class Plan:
    """A batch integrated repeatedly (assist_gb300_plan_*): the host work of a
    call done once, each launch a CUDA-graph replay over the same device
    tensors.  Write the next initial states into ``state`` (in place) between
    launches."""

    def __init__(self, ephem: Ephem, t0, t_end, state, params=None, var_state=None, status=None,
                 opts: Optional[Options] = None, stream=None):
        o = opts or options()
        self._keep = (ephem, t0, t_end, state, params, var_state, status)
        self._h = c_void_p()
        s = None if stream is None else c_void_p(stream.cuda_stream)
        rc = clib.assist_gb300_plan_create(byref(ephem), byref(o), state.shape[0], _ptr(t0), _ptr(t_end), _ptr(state),
                                           _ptr(params), 0 if var_state is None else 6, _ptr(var_state), _ptr(status),
                                           s, byref(self._h))
        if rc != 0:
            raise RuntimeError("assist_gb300_plan_create failed (%d): %s" % (rc, last_error()))

    def launch(self, stream=None) -> None:
        s = None if stream is None else c_void_p(stream.cuda_stream)
        rc = clib.assist_gb300_plan_launch(self._h, s)
        if rc != 0:
            raise RuntimeError("assist_gb300_plan_launch failed (%d): %s" % (rc, last_error()))

    def stats(self) -> dict:
        st = BatchStats()
        rc = clib.assist_gb300_plan_stats(self._h, byref(st))
        if rc != 0:
            raise RuntimeError("assist_gb300_plan_stats failed (%d): %s" % (rc, last_error()))
        return {f: getattr(st, f) for f, _ in BatchStats._fields_}

    def close(self) -> None:
        if self._h:
            clib.assist_gb300_plan_free(self._h)
            self._h = c_void_p()

    def __del__(self):
        self.close()


def integrate_batch_dense_device(ephem: Ephem, t0, t_end, state, out_start, out_t, out_state, params=None,
                                 status=None, opts: Optional[Options] = None, stream=None):
    """integrate_batch_device plus dense output: particle i's state at
    out_t[out_start[i]:out_start[i+1]] (sorted along its integration, within
    its span) into out_state [*, 6] (torch CUDA tensors; out_start int32)."""
    o = opts or options()
    n = state.shape[0]
    stats = BatchStats()
    s = None if stream is None else c_void_p(stream.cuda_stream)
    rc = clib.assist_gb300_integrate_batch_dense_device(byref(ephem), byref(o), n, _ptr(t0), _ptr(t_end), _ptr(state),
                                                        _ptr(params), _ptr(out_start), _ptr(out_t), _ptr(out_state),
                                                        _ptr(status), s, byref(stats))
    if rc != 0:
        raise RuntimeError("assist_gb300_integrate_batch_dense_device failed (%d): %s" % (rc, last_error()))
    return {f: getattr(stats, f) for f, _ in BatchStats._fields_}


def integrate_batch_device_static(ephem: Ephem, t0, t_end, state, params=None, status=None,
                                  opts: Optional[Options] = None, stream=None):
    """integrate_batch_device with independent steps and no variational
    particles, through the entry point that allocates nothing (its scratch is
    a fixed device array; at most STATIC_MAX_PARTICLES particles; one call at a
    time per device)."""
    o = opts or options()
    n = state.shape[0]
    stats = BatchStats()
    s = None if stream is None else c_void_p(stream.cuda_stream)
    rc = clib.assist_gb300_integrate_batch_device_static(byref(ephem), byref(o), n, _ptr(t0), _ptr(t_end), _ptr(state),
                                                         _ptr(params), _ptr(status), s, byref(stats))
    if rc != 0:
        raise RuntimeError("assist_gb300_integrate_batch_device_static failed (%d): %s" % (rc, last_error()))
    return {f: getattr(stats, f) for f, _ in BatchStats._fields_}


def forces_device(ephem: Ephem, t, state, params=None, var_state=None, acc=None, var_acc=None, status=None,
                  opts: Optional[Options] = None, stream=None):
    """One force evaluation of n particles at their own times t[i] (torch CUDA tensors)."""
    import torch
    o = opts or options()
    n = state.shape[0]
    if acc is None:
        acc = torch.empty((n, 3), dtype=torch.float64, device=state.device)
    nv = 0 if var_state is None else 6
    if nv and var_acc is None:
        var_acc = torch.empty((n, 6, 3), dtype=torch.float64, device=state.device)
    s = None if stream is None else c_void_p(stream.cuda_stream)
    rc = clib.assist_gb300_forces_device(byref(ephem), byref(o), n, _ptr(t), _ptr(state), _ptr(params), nv,
                                         _ptr(var_state), _ptr(acc), _ptr(var_acc), _ptr(status), s)
    if rc != 0:
        raise RuntimeError("assist_gb300_forces_device failed (%d): %s" % (rc, last_error()))
    return acc, var_acc


def forces_shared_time_device(ephem: Ephem, t: float, state, params=None, acc=None, status=None,
                              opts: Optional[Options] = None, stream=None):
    """One force evaluation of n particles at one time t (torch CUDA tensors)
    by the block-cooperative evaluation of the batched and shared-step
    integrators."""
    import torch
    o = opts or options()
    n = state.shape[0]
    if acc is None:
        acc = torch.empty((n, 3), dtype=torch.float64, device=state.device)
    s = None if stream is None else c_void_p(stream.cuda_stream)
    rc = clib.assist_gb300_forces_shared_time_device(byref(ephem), byref(o), n, float(t), _ptr(state), _ptr(params),
                                                     _ptr(acc), _ptr(status), s)
    if rc != 0:
        raise RuntimeError("assist_gb300_forces_shared_time_device failed (%d): %s" % (rc, last_error()))
    return acc


def bodies_device(ephem: Ephem, t, out=None, status=None, stream=None):
    """All bodies at n times: (n, n_bodies, 10) = GM, x, v, a (torch CUDA)."""
    import torch
    n = t.shape[0]
    nb = clib.assist_gb300_n_bodies(byref(ephem))
    if out is None:
        out = torch.empty((n, nb, 10), dtype=torch.float64, device=t.device)
    s = None if stream is None else c_void_p(stream.cuda_stream)
    rc = clib.assist_gb300_ephem_device(byref(ephem), n, _ptr(t), _ptr(out), _ptr(status), s)
    if rc != 0:
        raise RuntimeError("assist_gb300_ephem_device failed (%d): %s" % (rc, last_error()))
    return out


def encounter_ratio_device(ephem: Ephem, t0, t_end, state, out=None, stream=None):
    """Close-encounter cost ratio per particle (torch CUDA float32): the IAS15
    steps close planetary encounters add over [t0, t_end], as a fraction of
    the particle's plain steps (the estimate the grouped kernels queue by)."""
    import torch
    n = state.shape[0]
    if out is None:
        out = torch.empty(n, dtype=torch.float32, device=state.device)
    s = None if stream is None else c_void_p(stream.cuda_stream)
    rc = clib.assist_gb300_encounter_ratio_device(byref(ephem), n, _ptr(t0), _ptr(t_end), _ptr(state), _ptr(out), s)
    if rc != 0:
        raise RuntimeError("assist_gb300_encounter_ratio_device failed (%d): %s" % (rc, last_error()))
    return out


def group_plan(t0, t_end, state, params=None, ratio=None, group_order: int = 0,
               gm_sun: float = 2.9591220828411951e-04):
    """The grouped kernels' grouping on host arrays: (order, groups) with
    groups a list of index arrays into the batch, most expensive first."""
    t0 = np.ascontiguousarray(t0, np.float64)
    n = t0.shape[0]
    te = np.ascontiguousarray(t_end, np.float64)
    st = np.ascontiguousarray(state, np.float64).reshape(n, 6)
    prm = None if params is None else np.ascontiguousarray(params, np.float64).reshape(n, 3)
    rat = None if ratio is None else np.ascontiguousarray(ratio, np.float32).reshape(n)
    order = np.empty(n, np.int32); gs = np.empty(max(n, 1), np.int32); gz = np.empty(max(n, 1), np.int32)
    ng = c_int(0)
    rc = clib.assist_gb300_group_plan(n, t0.ctypes.data, te.ctypes.data, st.ctypes.data,
                                      None if prm is None else prm.ctypes.data,
                                      None if rat is None else rat.ctypes.data, group_order, gm_sun,
                                      order.ctypes.data, gs.ctypes.data, gz.ctypes.data, byref(ng))
    if rc != 0:
        raise RuntimeError("assist_gb300_group_plan failed (%d): %s" % (rc, last_error()))
    return order, [order[s:s + z] for s, z in zip(gs[:ng.value], gz[:ng.value])]


def fp64_peak_gflops() -> float:
    """Measured FP64 FMA throughput of the current device (GFLOP/s)."""
    return float(clib.assist_gb300_fp64_peak_gflops())
