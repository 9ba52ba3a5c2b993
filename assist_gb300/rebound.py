"""ctypes mirror of the REBOUND subset in include/rebound.h.

``Particle`` follows REBOUND 4.x's ``rebound.Particle`` layout; ``Simulation``
mirrors this library's compact ``struct reb_simulation`` (same member names as
REBOUND for everything ASSIST touches) and drives the device IAS15.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_char, c_double, c_int, c_uint, c_uint32, c_ulong, c_ulonglong, c_void_p

from ._lib import clib


class Particle(ctypes.Structure):
    _fields_ = [("x", c_double), ("y", c_double), ("z", c_double),
                ("vx", c_double), ("vy", c_double), ("vz", c_double),
                ("ax", c_double), ("ay", c_double), ("az", c_double),
                ("m", c_double), ("r", c_double), ("last_collision", c_double),
                ("c", c_void_p), ("hash", c_uint32), ("ap", c_void_p), ("_sim", c_void_p)]

    @property
    def xyz(self):
        return [self.x, self.y, self.z]

    @property
    def vxyz(self):
        return [self.vx, self.vy, self.vz]


class VarConfig(ctypes.Structure):
    _fields_ = [("sim", c_void_p), ("order", c_int), ("index", c_int), ("testparticle", c_int),
                ("index_1st_order_a", c_int), ("index_1st_order_b", c_int), ("lrescale", c_double)]


class DP7(ctypes.Structure):
    _fields_ = [("p%d" % k, POINTER(c_double)) for k in range(7)]


class IAS15(ctypes.Structure):
    _fields_ = [("epsilon", c_double), ("min_dt", c_double), ("adaptive_mode", c_uint),
                ("iterations_max_exceeded", c_ulong), ("N_allocated", c_int),
                ("x0", POINTER(c_double)), ("v0", POINTER(c_double)), ("a0", POINTER(c_double)),
                ("br", DP7), ("dt_last_success", c_double)]


class Simulation(ctypes.Structure):
    _fields_ = [("t", c_double), ("G", c_double), ("dt", c_double), ("dt_last_done", c_double),
                ("steps_done", c_ulonglong), ("N", c_int), ("N_var", c_int), ("N_var_config", c_int),
                ("N_active", c_int), ("N_allocated", c_int), ("N_allocated_var_config", c_int),
                ("var_config", POINTER(VarConfig)), ("_particles", POINTER(Particle)),
                ("exact_finish_time", c_int), ("force_is_velocity_dependent", c_int), ("status", c_int),
                ("integrator", c_int), ("gravity", c_int), ("ri_ias15", IAS15),
                ("additional_forces", c_void_p), ("pre_timestep_modifications", c_void_p),
                ("post_timestep_modifications", c_void_p), ("extras", c_void_p), ("extras_cleanup", c_void_p),
                ("error_message", c_char * 1024), ("gb300", c_void_p)]

    @staticmethod
    def create() -> "Simulation":
        return clib.reb_simulation_create().contents

    def add(self, x=0.0, y=0.0, z=0.0, vx=0.0, vy=0.0, vz=0.0, m=0.0):
        p = Particle(x=x, y=y, z=z, vx=vx, vy=vy, vz=vz, m=m)
        clib.reb_simulation_add(byref(self), p)

    def add_variation(self, testparticle: int) -> int:
        return clib.reb_simulation_add_variation_1st_order(byref(self), testparticle)

    @property
    def particles(self):
        return [self._particles[i] for i in range(self.N)]

    def particle(self, i: int) -> Particle:
        return self._particles[i]

    def integrate(self, tmax: float) -> int:
        return clib.reb_simulation_integrate(byref(self), c_double(tmax))

    def step(self) -> None:
        clib.reb_simulation_step(byref(self))

    def update_acceleration(self) -> None:
        clib.reb_simulation_update_acceleration(byref(self))

    def free(self) -> None:
        clib.reb_simulation_free(byref(self))


clib.reb_simulation_create.restype = POINTER(Simulation)
clib.reb_simulation_add.argtypes = [POINTER(Simulation), Particle]
clib.reb_simulation_add_variation_1st_order.argtypes = [POINTER(Simulation), c_int]
clib.reb_simulation_add_variation_1st_order.restype = c_int
clib.reb_simulation_integrate.argtypes = [POINTER(Simulation), c_double]
clib.reb_simulation_integrate.restype = c_int
clib.reb_simulation_step.argtypes = [POINTER(Simulation)]
clib.reb_simulation_update_acceleration.argtypes = [POINTER(Simulation)]
clib.reb_simulation_free.argtypes = [POINTER(Simulation)]
