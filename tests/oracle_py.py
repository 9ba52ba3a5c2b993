"""ctypes wrapper of the oracle (oracle/liboracle.so) -- test infrastructure.

The oracle is the CPU restatement of ASSIST's force model, ephemerides and
IAS15 (oracle/assist_oracle.cpp), pinned against the reference build.  Only
tests, smoke() and bench.py's CPU baseline use it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "liboracle.so")
REFLIB = os.path.join(ROOT, "oracle", "_ref", "libassist_ref.so")
D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)
L = C.POINTER(C.c_longlong)
DEFAULT_LAW = (1.0, 0.0, 2.0, 5.093, 1.0)


def _p(a):
    return None if a is None else a.ctypes.data_as(D)


def load_lib():
    if not os.path.exists(LIB):
        import subprocess
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    lib = C.CDLL(LIB)
    lib.orc_ephem_load.restype = C.c_void_p
    lib.orc_ephem_load.argtypes = [C.c_char_p, C.c_char_p]
    lib.orc_ephem_free.argtypes = [C.c_void_p]
    lib.orc_n_bodies.argtypes = [C.c_void_p]
    lib.orc_body.argtypes = [C.c_void_p, C.c_int, C.c_double, D]
    lib.orc_time_bounds.argtypes = [C.c_void_p, D, D]
    lib.orc_constants.argtypes = [C.c_void_p, D]
    lib.orc_forces.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, D, C.c_double, C.c_int, D, D, C.c_int, I, D, D, D, D]
    lib.orc_forces_dd.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, D, C.c_double, C.c_int, D, D, C.c_int, I, D, D,
                                  D, D, D]
    lib.orc_warm_start_study.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, D, C.c_int, C.c_int, D, D, D, D,
                                         C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, D, C.c_ulonglong, L]
    lib.orc_count_ops.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, D, C.c_double, D, D, C.c_int, D, D, D, L]
    lib.orc_integrate.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, D, C.c_double, C.c_double, C.c_int, C.c_int, I,
                                  D, D, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, C.c_int, L, D, D]
    lib.orc_integrate_batch.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, D, C.c_int, D, D, D, D, C.c_int, D, I,
                                        C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, C.c_int, L]
    lib.orc_ias15_constants.argtypes = [D, D, D]
    return lib


class Oracle:
    def __init__(self, planets: str, asteroids: str):
        self.lib = load_lib()
        self.h = self.lib.orc_ephem_load(planets.encode(), asteroids.encode())
        if not self.h:
            raise RuntimeError("oracle could not load %s / %s" % (planets, asteroids))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_ephem_free(self.h)
            self.h = None

    @property
    def n_bodies(self) -> int:
        return self.lib.orc_n_bodies(self.h)

    def body(self, i: int, t: float):
        out = np.zeros(10)
        st = self.lib.orc_body(self.h, i, float(t), _p(out))
        return st, out

    def time_bounds(self):
        a, b = C.c_double(), C.c_double()
        self.lib.orc_time_bounds(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def forces(self, t, state, params=None, var_state=None, var_tp=None, forces=0x7F, gr_eih_sources=1,
               geocentric=0, law=DEFAULT_LAW, dd=False):
        """state: (n, 6); var_state: (m, 6) with var_tp: (m,) owner indices.
        params: (n + m, 3) rows (real rows first) or (n, 3).  Returns (n + m, 3)."""
        st = np.ascontiguousarray(state, np.float64).reshape(-1, 6)
        n = st.shape[0]
        x = np.ascontiguousarray(st[:, :3]).ravel()
        v = np.ascontiguousarray(st[:, 3:]).ravel()
        m = 0
        vx = vv = None
        tp = None
        if var_state is not None:
            vs = np.ascontiguousarray(var_state, np.float64).reshape(-1, 6)
            m = vs.shape[0]
            vx = np.ascontiguousarray(vs[:, :3]).ravel()
            vv = np.ascontiguousarray(vs[:, 3:]).ravel()
            tp = np.ascontiguousarray(var_tp, np.int32)
        prm = None
        if params is not None:
            p = np.asarray(params, np.float64).reshape(-1, 3)
            if p.shape[0] == n and m:
                p = np.concatenate([p, np.zeros((m, 3))])
            prm = np.ascontiguousarray(p).ravel()
        law = np.asarray(law, np.float64)
        tpp = None if tp is None else tp.ctypes.data_as(I)
        if not dd:
            acc = np.zeros(3 * (n + m))
            r = self.lib.orc_forces(self.h, forces, gr_eih_sources, geocentric, _p(law), float(t), n, _p(x), _p(v), m,
                                    tpp, _p(vx), _p(vv), _p(prm), _p(acc))
            if r != 0:
                raise RuntimeError("oracle forces status %d" % r)
            return acc.reshape(-1, 3)
        hi = np.zeros(3 * (n + m)); lo = np.zeros(3 * (n + m))
        r = self.lib.orc_forces_dd(self.h, forces, gr_eih_sources, geocentric, _p(law), float(t), n, _p(x), _p(v), m,
                                   tpp, _p(vx), _p(vv), _p(prm), _p(hi), _p(lo))
        if r != 0:
            raise RuntimeError("oracle forces status %d" % r)
        return hi.reshape(-1, 3), lo.reshape(-1, 3)

    def count_ops(self, t, state, params=None, var_state=None, forces=0x7F, gr_eih_sources=1, law=DEFAULT_LAW):
        st = np.ascontiguousarray(state, np.float64).reshape(6)
        x = st[:3].copy(); v = st[3:].copy()
        m = 0
        vx = vv = None
        if var_state is not None:
            vs = np.ascontiguousarray(var_state, np.float64).reshape(-1, 6)
            m = vs.shape[0]
            vx = np.ascontiguousarray(vs[:, :3]).ravel(); vv = np.ascontiguousarray(vs[:, 3:]).ravel()
        prm = None
        if params is not None:
            prm = np.concatenate([np.asarray(params, np.float64).reshape(3), np.zeros(3 * m)])
        out = np.zeros(15, dtype=np.int64)
        law = np.asarray(law, np.float64)
        r = self.lib.orc_count_ops(self.h, forces, gr_eih_sources, 0, _p(law), float(t), _p(x), _p(v), m, _p(vx),
                                   _p(vv), _p(prm), out.ctypes.data_as(L))
        if r != 0:
            raise RuntimeError("oracle count status %d" % r)
        names = ["add", "mul", "div", "sqrt", "pow"]
        d = dict(zip(names, out[:5].tolist()))
        d["bodies"] = dict(zip(names, out[5:10].tolist()))    # the part of d that forms the body states
        # force-term work that does not depend on the particle (origin-minus-body
        # offsets, EIH source-source sums); counted apart from d
        d["shared"] = dict(zip(names, out[10:15].tolist()))
        return d

    def integrate(self, t0, t_end, state, var_state=None, var_tp=None, params=None, epsilon=1e-9, min_dt=0.0,
                  dt0=0.001, max_steps=0, dd=False, forces=0x7F, gr_eih_sources=1, geocentric=0, law=DEFAULT_LAW,
                  dt_floor=0.0):
        """One shared-step simulation (real particles then variational ones)."""
        st = np.ascontiguousarray(state, np.float64).reshape(-1, 6)
        n = st.shape[0]
        m = 0
        tp = None
        allst = st
        if var_state is not None:
            vs = np.ascontiguousarray(var_state, np.float64).reshape(-1, 6)
            m = vs.shape[0]
            allst = np.concatenate([st, vs])
            tp = np.ascontiguousarray(var_tp, np.int32)
        buf = np.ascontiguousarray(allst).ravel().copy()
        prm = None
        if params is not None:
            p = np.asarray(params, np.float64).reshape(-1, 3)
            if p.shape[0] == n and m:
                p = np.concatenate([p, np.zeros((m, 3))])
            prm = np.ascontiguousarray(p).ravel()
        stats = np.zeros(5, dtype=np.int64)
        tout, dtout = C.c_double(), C.c_double()
        law = np.asarray(law, np.float64)
        r = self.lib.orc_integrate(self.h, forces, gr_eih_sources, geocentric, _p(law), float(t0), float(t_end), n, m,
                                   None if tp is None else tp.ctypes.data_as(I), _p(buf), _p(prm), epsilon, min_dt,
                                   dt0, max_steps, dt_floor, 1 if dd else 0, stats.ctypes.data_as(L), C.byref(tout),
                                   C.byref(dtout))
        out = buf.reshape(-1, 6)
        return out[:n], out[n:], dict(status=r, accepted=int(stats[0]), rejected=int(stats[1]), evals=int(stats[2]),
                                      iterations=int(stats[3]), t=tout.value, dt=dtout.value)

    def warm_start_study(self, t0, t_end, state, rel_err, group=1, params=None, epsilon=1e-9, dt0=0.001,
                         dt_floor=1e-8, threads=None, seed=1, forces=0x7F, gr_eih_sources=1, law=DEFAULT_LAW):
        """Corrector iterations per accepted step of the plain predictor and
        of replays of each step started from the converged b with relative
        error rel_err[k] (shared-step groups of `group` particles).  Returns
        an int array (1 + len(rel_err), 13) of step counts by iterations."""
        st = np.ascontiguousarray(state, np.float64).reshape(-1, 6)
        n = st.shape[0]
        t0 = np.ascontiguousarray(np.broadcast_to(np.asarray(t0, np.float64), (n,))).copy()
        te = np.ascontiguousarray(np.broadcast_to(np.asarray(t_end, np.float64), (n,))).copy()
        prm = None if params is None else np.ascontiguousarray(params, np.float64).reshape(n, 3)
        errs = np.ascontiguousarray(rel_err, np.float64)
        hist = np.zeros((1 + errs.size, 13), np.int64)
        law = np.asarray(law, np.float64)
        r = self.lib.orc_warm_start_study(self.h, forces, gr_eih_sources, 0, _p(law), n, group, _p(t0), _p(te), _p(st),
                                          _p(prm), epsilon, dt0, dt_floor, threads or os.cpu_count() or 1, errs.size,
                                          _p(errs), seed, hist.ctypes.data_as(L))
        if r != 0:
            raise RuntimeError("warm-start study status %d" % r)
        return hist

    def integrate_batch(self, t0, t_end, state, params=None, var_state=None, epsilon=1e-9, min_dt=0.0, dt0=0.001,
                        max_steps=0, threads=None, forces=0x7F, gr_eih_sources=1, geocentric=0, law=DEFAULT_LAW,
                        return_all=False, dt_floor=1e-8):
        st = np.ascontiguousarray(state, np.float64).reshape(-1, 6).copy()
        n = st.shape[0]
        t0 = np.ascontiguousarray(np.broadcast_to(np.asarray(t0, np.float64), (n,))).copy()
        te = np.ascontiguousarray(np.broadcast_to(np.asarray(t_end, np.float64), (n,))).copy()
        prm = None if params is None else np.ascontiguousarray(params, np.float64).reshape(n, 3).copy()
        nv = 0
        var = None
        if var_state is not None:
            var = np.ascontiguousarray(var_state, np.float64).reshape(n, 6, 6).copy()
            nv = 6
        status = np.zeros(n, dtype=np.int32)
        stats = np.zeros(4, dtype=np.int64)
        law = np.asarray(law, np.float64)
        self.lib.orc_integrate_batch(self.h, forces, gr_eih_sources, geocentric, _p(law), n, _p(t0), _p(te), _p(st),
                                     _p(prm), nv, _p(var), status.ctypes.data_as(I), epsilon, min_dt, dt0, max_steps,
                                     dt_floor, threads or os.cpu_count() or 1, stats.ctypes.data_as(L))
        if return_all:
            return st, var, status, dict(accepted=int(stats[0]), rejected=int(stats[1]), evals=int(stats[2]),
                                         iterations=int(stats[3]))
        return st
