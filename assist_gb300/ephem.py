"""``Ephem``: ctypes mirror of struct assist_ephem, same interface as ASSIST's
assist/ephem.py (Ephem(planets_path, asteroids_path), get_particle, time_bounds).
"""
from __future__ import annotations

from ctypes import Structure, byref, c_char_p, c_double, c_int, c_void_p
from typing import Optional, Union

from ._lib import assist_error_messages, clib
from .rebound import Particle

ASSIST_BODY_IDS = {0: "Sun", 1: "Mercury", 2: "Venus", 3: "Earth", 4: "Moon", 5: "Mars", 6: "Jupiter",
                   7: "Saturn", 8: "Uranus", 9: "Neptune", 10: "Pluto", 11: "Camilla", 12: "Ceres", 13: "Cybele",
                   14: "Davida", 15: "Eunomia", 16: "Euphrosyne", 17: "Europa", 18: "Hygiea", 19: "Interamnia",
                   20: "Iris", 21: "Juno", 22: "Pallas", 23: "Psyche", 24: "Sylvia", 25: "Thisbe", 26: "Vesta"}


class Ephem(Structure):
    """Ephemeris handle (planets .440/.441 + asteroid SPK), not tied to a simulation."""

    def __init__(self, planets_path: Optional[str] = None, asteroids_path: Optional[str] = None):
        p = c_char_p(str(planets_path).encode("ascii")) if planets_path is not None else c_char_p(None)
        a = c_char_p(str(asteroids_path).encode("ascii")) if asteroids_path is not None else c_char_p(None)
        clib.assist_ephem_init.restype = c_int
        ret = clib.assist_ephem_init(byref(self), p, a)
        if ret != 0:
            raise RuntimeError(assist_error_messages(ret))
        self._live = True

    def get_particle(self, body: Union[int, str], t: float) -> Particle:
        if isinstance(body, str):
            name = body.lower()
            ids = [k for k, v in ASSIST_BODY_IDS.items() if v.lower() == name]
            if not ids:
                raise ValueError("Cannot find body '" + name + "'. Needs to be one of: " +
                                 ", ".join(ASSIST_BODY_IDS.values()) + ".")
            body = ids[0]
        if not isinstance(body, int):
            raise ValueError("Expecting integer for body id.")
        clib.assist_get_particle_with_error.restype = Particle
        e = c_int(0)
        p = clib.assist_get_particle_with_error(byref(self), c_int(body), c_double(t), byref(e))
        if e.value:
            raise RuntimeError(assist_error_messages(e.value))
        return p

    def time_bounds(self) -> tuple:
        tb, te = c_double(0.0), c_double(0.0)
        clib.assist_ephem_time_bounds(byref(self), byref(tb), byref(te))
        return (tb.value, te.value)

    def __del__(self) -> None:
        if getattr(self, "_live", False):
            clib.assist_ephem_free_pointers(byref(self))
            self._live = False

    _fields_ = [("jd_ref", c_double), ("spk_planets", c_void_p), ("spk_asteroids", c_void_p),
                ("ascii_planets", c_void_p), ("planets_source", c_int), ("planets_calc", c_void_p),
                ("spk_target_index", c_int * 11), ("spk_emb_index", c_int),
                ("AU", c_double), ("EMRAT", c_double), ("J2E", c_double), ("J3E", c_double), ("J4E", c_double),
                ("J2SUN", c_double), ("RE", c_double), ("CLIGHT", c_double), ("ASUN", c_double),
                ("Re_eq", c_double), ("Rs_eq", c_double), ("c_AU_per_day", c_double), ("c_squared", c_double),
                ("over_c_squared", c_double)]
