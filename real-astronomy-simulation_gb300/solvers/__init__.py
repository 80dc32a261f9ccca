"""Gravity solvers: direct N^2 (gravity), LBVH Barnes-Hut (barnes_hut), the
analytic galaxy potential (external) and the SPH neighbour grid
(neighbor_grid)."""
