"""Minimal stand-in for molmod 1.4.8: the names the reference imports from it."""
from .units import *  # noqa: F401,F403
from .units import boltzmann  # noqa: F401
