"""Integrators: the leapfrog halves (leapfrog)."""
