"""Gravity solvers: direct N^2 (gravity) and LBVH Barnes-Hut (barnes_hut)."""
