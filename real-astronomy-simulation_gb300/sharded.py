"""Direct N^2 KDK stepping with the targets split across the ranks of a
process group, one GPU per rank.

The target loop ``for i in range(n)`` of compute_acc_direct
(core/solvers/gravity.py:18-26) is cut into W contiguous slices of
``chunk = ceil(n / W)`` targets: rank r owns particles r*chunk ..
min((r + 1) * chunk, n) - 1, their positions, velocities and
accelerations.  One KDK step (core/engine.py:108-116 with the kick and drift
of core/integrators/leapfrog.py:11-22):

1. kick   v += a dt/2                      own slice
2. drift  x += v dt                        own slice
3. all-gather of the 16-byte {x, y, z, m} records: every rank then holds
   all n positions (the step's only exchange)
4. force on the own targets from all n sources (gb_direct_acc_range)
5. kick   v += a dt/2                      own slice

Each target's force sums the same terms in the same order whatever the
split, so a sharded run follows the single-rank run.  Energies need one
all-reduce of the slices' FP64 (kinetic, potential) sums.

The device work goes through an ``ops`` object (kick, drift, acc_range,
energies, alloc); the default one calls the CUDA library.  A caller can hand
in another implementation of the same five methods (the CPU tests use the
FP64 oracle that way to check the exchange logic over gloo).

ShardedBarnesHut does the same for the tree path.  The tree is global, so
every rank builds the whole of it and walks one slice of the key order; one
all-reduce of the accelerations joins the slices.
"""
from __future__ import annotations

import numpy as np
import torch

from ._dev import require_cuda


def shard_range(n: int, rank: int, world: int) -> tuple[int, int, int]:
    """(t0, nt, chunk): the first target, target count and slice stride of
    rank `rank` of `world` for an n-particle system."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError(f"bad rank {rank} of {world}")
    chunk = -(-n // world) if n > 0 else 0
    t0 = min(rank * chunk, n)
    return t0, max(0, min(chunk, n - t0)), chunk


class CudaOps:
    """The device work of a sharded step through the C ABI (float32 float4
    records on the rank's GPU)."""

    def __init__(self, n: int, G: float, eps2: float, device, plain_fp32: bool = False):
        from .integrators import leapfrog
        from .solvers.gravity import DirectGravity

        self.device = require_cuda(device)
        self.G, self.eps2, self.plain = float(G), float(eps2), bool(plain_fp32)
        self._lf = leapfrog
        self._g = DirectGravity(max(n, 1), self.device)

    def alloc(self, rows: int) -> torch.Tensor:
        return torch.zeros((rows, 4), dtype=torch.float32, device=self.device)

    def alloc_phi(self, rows: int) -> torch.Tensor:
        return torch.zeros(rows, dtype=torch.float32, device=self.device)

    def kick(self, v, a, nt: int, h: float) -> None:
        if nt:
            self._lf.kick(v, a, nt, h)

    def drift(self, x, v, nt: int, dt: float) -> None:
        if nt:
            self._lf.drift(x, v, nt, dt)

    def acc_range(self, x_all, n: int, t0: int, nt: int, a, phi=None) -> None:
        if nt:
            self._g.acc_range(x_all, n, t0, nt, a, self.G, self.eps2, phi=phi, plain=self.plain)

    def energies(self, x, v, phi, nt: int) -> torch.Tensor:
        """(KE, PE) of the slice as a float64 tensor on the device."""
        if nt == 0:
            return torch.zeros(2, dtype=torch.float64, device=self.device)
        ke, pe, _ = self._g.energies_from_phi(x[:nt], v[:nt], phi[:nt], self.G)
        return torch.tensor([ke, pe], dtype=torch.float64, device=self.device)

    def close(self) -> None:
        self._g.close()


class ShardedDirect:
    """Direct-sum KDK integration of one system, targets split across the
    ranks of ``group`` (torch.distributed; None or a one-rank world runs
    alone).  pos, vel (n, 3) and mass (n,) are the whole system's initial
    state on every rank (each rank keeps its own slice)."""

    def __init__(self, pos, vel, mass, *, G: float = 1.0, softening: float = 0.05, group=None,
                 device=None, ops=None, plain_fp32: bool = False):
        import torch.distributed as dist

        self._dist = dist if (dist.is_available() and dist.is_initialized()) else None
        self.group = group
        self.world = self._dist.get_world_size(group) if self._dist else 1
        self.rank = self._dist.get_rank(group) if self._dist else 0
        pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
        vel = np.asarray(vel, dtype=np.float64).reshape(-1, 3)
        mass = np.asarray(mass, dtype=np.float64).reshape(-1)
        self.n = pos.shape[0]
        self.G = float(G)
        self.eps2 = float(softening) ** 2
        self.t0, self.nt, self.chunk = shard_range(self.n, self.rank, self.world)
        self.ops = ops if ops is not None else CudaOps(self.n, self.G, self.eps2, device, plain_fp32)
        rows = max(self.chunk, 1)
        # x_all: every rank's slice at rank * chunk (padded tail rows: zero
        # mass, never a source: the force reads the first n rows only).
        self.x_all = self.ops.alloc(self.world * rows)
        self.x = self.ops.alloc(rows)      # own positions and masses (the master copy)
        self.v = self.ops.alloc(rows)
        self.a = self.ops.alloc(rows)
        self.phi = self.ops.alloc_phi(rows)
        self._phi_valid = False
        s = slice(self.t0, self.t0 + self.nt)
        host = torch.zeros((rows, 4), dtype=self.x.dtype)
        host[: self.nt, :3] = torch.from_numpy(pos[s])
        host[: self.nt, 3] = torch.from_numpy(mass[s])
        self.x.copy_(host)
        host.zero_()
        host[: self.nt, :3] = torch.from_numpy(vel[s])
        self.v.copy_(host)
        self.time = 0.0
        self.step_count = 0
        self._gather()
        self._force(phi=True)

    # ------------------------------------------------------------ exchange
    def _gather(self) -> None:
        """x_all <- every rank's own slice (one all-gather of float4 records)."""
        if self.world == 1:
            self.x_all.copy_(self.x)
            return
        rows = self.x.shape[0]
        views = [self.x_all[r * rows:(r + 1) * rows] for r in range(self.world)]
        self._dist.all_gather(views, self.x, group=self.group)

    def _force(self, phi: bool = False) -> None:
        self.ops.acc_range(self.x_all, self.n, self.t0, self.nt, self.a,
                           self.phi if phi else None)
        self._phi_valid = phi

    # ------------------------------------------------------------ stepping
    def step(self, dt: float) -> None:
        self.run(dt, 1)

    def run(self, dt: float, nsteps: int) -> None:
        """nsteps KDK steps; the last step's force pass also writes the
        potential sums of the own targets (for energies())."""
        h = 0.5 * float(dt)
        for k in range(int(nsteps)):
            self.ops.kick(self.v, self.a, self.nt, h)
            self.ops.drift(self.x, self.v, self.nt, float(dt))
            self._gather()
            self._force(phi=k == nsteps - 1)
            self.ops.kick(self.v, self.a, self.nt, h)
            self.time += float(dt)
            self.step_count += 1

    # --------------------------------------------------------- diagnostics
    def energies(self) -> tuple[float, float, float]:
        """(kinetic, potential, total) of the whole system (FP64 sums of the
        slices, all-reduced; core/solvers/gravity.py:29-57)."""
        if not self._phi_valid:
            scratch = torch.empty_like(self.a)
            self.ops.acc_range(self.x_all, self.n, self.t0, self.nt, scratch, self.phi)
            self._phi_valid = True
        e = self.ops.energies(self.x, self.v, self.phi, self.nt)
        if self.world > 1:
            self._dist.all_reduce(e, group=self.group)
        ke, pe = float(e[0]), float(e[1])
        return ke, pe, ke + pe

    def gather_state(self):
        """(pos, vel, acc) of the whole system as float64 numpy arrays, on
        every rank (an all-gather of the slices; for checks and snapshots)."""
        def full(t):
            if self.world == 1:
                out = t.clone()
            else:
                rows = t.shape[0]
                out = torch.empty((self.world * rows, 4), dtype=t.dtype, device=t.device)
                self._dist.all_gather([out[r * rows:(r + 1) * rows] for r in range(self.world)], t,
                                      group=self.group)
            return out[: self.n, :3].double().cpu().numpy()
        return full(self.x), full(self.v), full(self.a)

    def close(self) -> None:
        if hasattr(self.ops, "close"):
            self.ops.close()


# ------------------------------------------------------------------- tree
class CudaTreeOps:
    """The device work of a tree-sharded step through the C ABI."""

    def __init__(self, n: int, theta: float, softening: float, G: float, key_bits: int, max_stack: int,
                 traversal: int, device):
        from .integrators import leapfrog
        from .solvers.barnes_hut import BarnesHut

        self.device = require_cuda(device)
        self._lf = leapfrog
        self._bh = BarnesHut(max(n, 1), theta=theta, softening=softening, max_stack=max_stack,
                             key_bits=key_bits, G=G, device=self.device)
        if traversal != -1:
            self._bh.set_traversal(traversal)

    def alloc(self, rows: int) -> torch.Tensor:
        return torch.zeros((rows, 4), dtype=torch.float32, device=self.device)

    def alloc_phi(self, rows: int) -> torch.Tensor:
        return torch.zeros(rows, dtype=torch.float32, device=self.device)

    def kick(self, v, a, n: int, h: float) -> None:
        if n:
            self._lf.kick(v, a, n, h)

    def drift(self, x, v, n: int, dt: float) -> None:
        if n:
            self._lf.drift(x, v, n, dt)

    def tree_acc(self, x, n: int, s0: int, ns: int, a, phi=None) -> None:
        """Builds the tree of all n particles and writes the accelerations
        (and potentials) of the key-order slice [s0, s0 + ns) into a zeroed
        a (and phi)."""
        a.zero_()
        if phi is not None:
            phi.zero_()
        if n:
            self._bh.build(x[:n])
            self._bh.accel_range(a, s0, ns, phi=phi)

    def energies(self, x, v, phi, n: int) -> torch.Tensor:
        if n == 0:
            return torch.zeros(2, dtype=torch.float64, device=self.device)
        ke, pe, _ = self._bh.energies_from_phi(x[:n], v[:n], phi[:n])
        return torch.tensor([ke, pe], dtype=torch.float64, device=self.device)

    def close(self) -> None:
        self._bh.close()


class ShardedBarnesHut:
    """Tree KDK integration with the tree replicated and the targets split
    across the ranks of ``group``.  Every rank holds the whole state, makes
    the same kick and drift and builds the same tree; it walks only the
    targets of its slice of the key order (``gb_bh_accel_range``), and one
    all-reduce (sum) of the zero-filled acceleration array, 16 bytes per
    particle, gives every rank all of them: each sum has one non-zero term,
    so the result is exact and the ranks stay identical.  The build (about
    a tenth of a step at 1M particles) is repeated on every rank; the
    traversal, the rest, is split.  pos, vel (n, 3) and mass (n,) are the
    whole system's initial state on every rank."""

    def __init__(self, pos, vel, mass, *, theta: float = 0.5, softening: float = 0.05, G=None,
                 key_bits: int = 21, max_stack: int = 64, traversal: int = -1, group=None, device=None,
                 ops=None):
        import torch.distributed as dist

        from . import units

        self._dist = dist if (dist.is_available() and dist.is_initialized()) else None
        self.group = group
        self.world = self._dist.get_world_size(group) if self._dist else 1
        self.rank = self._dist.get_rank(group) if self._dist else 0
        pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
        vel = np.asarray(vel, dtype=np.float64).reshape(-1, 3)
        mass = np.asarray(mass, dtype=np.float64).reshape(-1)
        self.n = pos.shape[0]
        self.G = units.G if G is None else float(G)
        self.s0, self.ns, _ = shard_range(self.n, self.rank, self.world)
        self.ops = ops if ops is not None else CudaTreeOps(self.n, theta, softening, self.G, key_bits,
                                                           max_stack, traversal, device)
        rows = max(self.n, 1)
        self.x = self.ops.alloc(rows)
        self.v = self.ops.alloc(rows)
        self.a = self.ops.alloc(rows)
        self.phi = self.ops.alloc_phi(rows)
        host = torch.zeros((rows, 4), dtype=self.x.dtype)
        host[: self.n, :3] = torch.from_numpy(pos)
        host[: self.n, 3] = torch.from_numpy(mass)
        self.x.copy_(host)
        host.zero_()
        host[: self.n, :3] = torch.from_numpy(vel)
        self.v.copy_(host)
        self.time = 0.0
        self.step_count = 0
        self._phi_valid = False
        self._force(phi=True)

    def _sum(self, t) -> None:
        if self.world > 1:
            self._dist.all_reduce(t, group=self.group)

    def _force(self, phi: bool = False) -> None:
        self.ops.tree_acc(self.x, self.n, self.s0, self.ns, self.a, self.phi if phi else None)
        self._sum(self.a)
        if phi:
            self._sum(self.phi)
        self._phi_valid = phi

    def step(self, dt: float) -> None:
        self.run(dt, 1)

    def run(self, dt: float, nsteps: int) -> None:
        """nsteps KDK steps; the last one's traversal also writes the tree
        potential (for energies())."""
        h = 0.5 * float(dt)
        for k in range(int(nsteps)):
            self.ops.kick(self.v, self.a, self.n, h)
            self.ops.drift(self.x, self.v, self.n, float(dt))
            self._force(phi=k == nsteps - 1)
            self.ops.kick(self.v, self.a, self.n, h)
            self.time += float(dt)
            self.step_count += 1

    def energies(self) -> tuple[float, float, float]:
        """(kinetic, potential, total), the potential from the tree (the same
        on every rank: the state and the summed potentials are replicated)."""
        if not self._phi_valid:
            scratch = torch.empty_like(self.a)
            self.ops.tree_acc(self.x, self.n, self.s0, self.ns, scratch, self.phi)
            self._sum(self.phi)
            self._phi_valid = True
        e = self.ops.energies(self.x, self.v, self.phi, self.n)
        ke, pe = float(e[0]), float(e[1])
        return ke, pe, ke + pe

    def gather_state(self):
        """(pos, vel, acc) as float64 numpy arrays (every rank holds them)."""
        def host(t):
            return t[: self.n, :3].double().cpu().numpy()
        return host(self.x), host(self.v), host(self.a)

    def close(self) -> None:
        if hasattr(self.ops, "close"):
            self.ops.close()
