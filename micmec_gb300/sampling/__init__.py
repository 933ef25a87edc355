"""Phase-space sampling: Verlet MD with thermostats/barostat, and optimisers."""
