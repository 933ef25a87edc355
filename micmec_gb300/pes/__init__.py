"""Micromechanical potential energy surfaces (GPU force parts)."""
