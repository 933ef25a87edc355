"""micmec_gb300: GB300-native (sm_103a) force evaluation and integration for MicMec.

Mirrors the reference package layout for the hot path: ``micmec_gb300.system``
(``System``), ``micmec_gb300.pes.mmff`` (``MicMecForceField``, ``ForcePart``,
``ForcePartMechanical``, ``ForcePartPressure``) and ``micmec_gb300.sampling``
(Verlet integrator, thermostats, barostat, optimisers). The compute runs in
``lib/libmicmec_gb300.so`` (C ABI: ``include/micmec_gb300.h``).
"""

__version__ = "0.1.0"
