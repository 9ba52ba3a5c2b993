"""assist_gb300: ASSIST's test-particle equations of motion on GB300 (sm_103a).

Drop-in surface (mirrors ASSIST's Python wrapper): ``Ephem``, ``Extras`` and
the REBOUND subset ``Simulation``/``Particle``; batched device API in
``assist_gb300.batch``.  Synthetic ephemerides and populations in
``assist_gb300.synth``.
"""
from ._lib import __build__, __githash__, __libpath__, __version__, assist_error_messages, clib
from .ephem import ASSIST_BODY_IDS, Ephem
from .extras import ASSIST_FORCES, Extras
from .rebound import Particle, Simulation

__all__ = ["__libpath__", "__version__", "__build__", "__githash__", "assist_error_messages", "clib", "Ephem",
           "Extras", "Simulation", "Particle", "ASSIST_FORCES", "ASSIST_BODY_IDS"]
