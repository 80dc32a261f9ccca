"""Leapfrog integrator entry points."""
