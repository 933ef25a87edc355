"""molmod.units stand-in: re-exports the product's restatement of molmod's factors."""
from micmec_gb300.units import *  # noqa: F401,F403
from micmec_gb300.units import boltzmann  # noqa: F401
