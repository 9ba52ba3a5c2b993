"""``Extras``: ctypes mirror of struct assist_extras, same interface as
ASSIST's assist/extras.py (forces list, particle_params, integrate_or_interpolate).
"""
from __future__ import annotations

from ctypes import POINTER, Structure, byref, c_double, c_int, c_void_p
from typing import List

import numpy as np

from ._lib import clib
from .ephem import Ephem
from .rebound import Particle, Simulation

ASSIST_FORCES = {"SUN": 0x01, "PLANETS": 0x02, "ASTEROIDS": 0x04, "NON_GRAVITATIONAL": 0x08,
                 "EARTH_HARMONICS": 0x10, "SUN_HARMONICS": 0x20, "GR_EIH": 0x40, "GR_SIMPLE": 0x80,
                 "GR_POTENTIAL": 0x100}


class Extras(Structure):
    """ASSIST attached to one simulation."""

    def __init__(self, sim: Simulation, ephem: Ephem):
        sim._extras_ref = self
        self._ephem_ref = ephem
        clib.assist_init(byref(self), byref(sim), byref(ephem))
        self.extras_should_free_ephem = 0
        self._live = True

    def __del__(self) -> None:
        if getattr(self, "_live", False):
            clib.assist_free_pointers(byref(self))
            self._live = False

    def detach(self, sim: Simulation) -> None:
        sim._extras_ref = None
        clib.assist_detach(byref(sim), byref(self))

    def integrate_or_interpolate(self, t: float) -> None:
        clib.assist_integrate_or_interpolate(byref(self), c_double(t))

    @property
    def forces(self) -> List[str]:
        return [k for k, v in ASSIST_FORCES.items() if self._forces & v]

    @forces.setter
    def forces(self, value: List[str]) -> None:
        if not isinstance(value, list):
            raise AttributeError("Forces need to be a list.")
        for elem in value:
            if not isinstance(elem, str):
                raise AttributeError("Each force needs to be a string.")
            if elem.upper() not in ASSIST_FORCES:
                raise AttributeError("Force '" + elem + "' not recognized. Needs to be one of the following: " +
                                     ", ".join(ASSIST_FORCES))
        v = 0
        for k in ASSIST_FORCES:
            if k in value:
                v |= ASSIST_FORCES[k]
        self._forces = c_int(v)

    @property
    def particle_params(self):
        raise AttributeError("Cannot get particle_params. Only setting is supported.")

    @particle_params.setter
    def particle_params(self, value) -> None:
        self._particle_params_reference = np.ascontiguousarray(value, dtype=np.float64).copy()
        self._particle_params = self._particle_params_reference.ctypes.data_as(POINTER(c_double))

    _fields_ = [("_sim", POINTER(Simulation)), ("ephem", POINTER(Ephem)), ("_ephem_cache", c_void_p),
                ("extras_should_free_ephem", c_int), ("geocentric", c_int),
                ("last_state", POINTER(Particle)), ("current_state", POINTER(Particle)),
                ("_particle_params", POINTER(c_double)), ("steps_done", c_int), ("_forces", c_int),
                ("gr_eih_sources", c_int), ("alpha", c_double), ("nk", c_double), ("nm", c_double),
                ("nn", c_double), ("r0", c_double)]


clib.assist_init.argtypes = [POINTER(Extras), POINTER(Simulation), POINTER(Ephem)]
clib.assist_free_pointers.argtypes = [POINTER(Extras)]
clib.assist_detach.argtypes = [POINTER(Simulation), POINTER(Extras)]
clib.assist_integrate_or_interpolate.argtypes = [POINTER(Extras), c_double]
