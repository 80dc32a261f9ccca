"""Sharded direct-sum stepping on CPU (gloo, world_size 2): the target split,
the per-step all-gather of the position records and the slice-local KDK
updates of ShardedDirect, with the FP64 oracle doing the device work.  Each
target's force is the oracle's sum over all sources in index order, so the
two-rank run must equal the one-rank run bit for bit, and both must equal
the oracle's own KDK loop (core/engine.py:108-116).  No GPU involved."""
import importlib
import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import PKG_NAME, ROOT


class OracleOps:
    """The five device operations of a sharded step in FP64 on the CPU
    (oracle forces, elementwise kick/drift)."""

    def __init__(self, G, eps2):
        from oracle import oracle

        self.orc = oracle
        self.G, self.eps2 = G, eps2

    def alloc(self, rows):
        return torch.zeros((rows, 4), dtype=torch.float64)

    def alloc_phi(self, rows):
        return torch.zeros(rows, dtype=torch.float64)

    def kick(self, v, a, nt, h):
        v[:nt, :3] += a[:nt, :3] * h

    def drift(self, x, v, nt, dt):
        x[:nt, :3] += v[:nt, :3] * dt

    def acc_range(self, x_all, n, t0, nt, a, phi=None):
        if nt == 0:
            return
        xs = x_all[:n].numpy()
        t = np.arange(t0, t0 + nt)
        a[:nt, :3] = torch.from_numpy(self.orc.direct_acc(xs[:, :3], xs[:, 3], self.G, self.eps2, t))
        if phi is not None:
            phi[:nt] = torch.from_numpy(self.orc.phi_targets(xs[:, :3], xs[:, 3], self.eps2, t))

    def energies(self, x, v, phi, nt):
        if nt == 0:
            return torch.zeros(2, dtype=torch.float64)
        m = x[:nt, 3].numpy()
        ke = self.orc.kinetic_energy(v[:nt, :3].numpy(), m)
        pe = -0.5 * self.G * float(np.sum(m * phi[:nt].numpy()))
        return torch.tensor([ke, pe], dtype=torch.float64)


def _system(n, seed=3):
    ic = importlib.import_module(PKG_NAME + ".ic")
    pos, vel, mass = ic.plummer(n, seed=seed)
    return pos, vel, mass


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


STEPS = 4
DT = 1e-3
EPS = 0.05


def _worker(rank, world, port, out_dir, n):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sh = importlib.import_module(PKG_NAME + ".sharded")
        pos, vel, mass = _system(n)
        s = sh.ShardedDirect(pos, vel, mass, G=1.0, softening=EPS, ops=OracleOps(1.0, EPS * EPS))
        s.run(DT, STEPS)
        p, v, a = s.gather_state()
        e = s.energies()
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), p=p, v=v, a=a, e=np.array(e),
                 t0=s.t0, nt=s.nt)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("n", [301, 1])
def test_two_ranks_equal_one_rank(tmp_path, n):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path), n), nprocs=world, join=True)
    sh = importlib.import_module(PKG_NAME + ".sharded")
    pos, vel, mass = _system(n)
    one = sh.ShardedDirect(pos, vel, mass, G=1.0, softening=EPS, ops=OracleOps(1.0, EPS * EPS))
    one.run(DT, STEPS)
    p1, v1, a1 = one.gather_state()
    e1 = one.energies()
    r = [np.load(tmp_path / f"rank{k}.npz") for k in range(world)]
    # The slices tile the system.
    assert [int(x["t0"]) for x in r] == [0, min(-(-n // 2), n)]
    assert sum(int(x["nt"]) for x in r) == n
    for x in r:
        assert np.array_equal(x["p"], p1) and np.array_equal(x["v"], v1) and np.array_equal(x["a"], a1)
        # The potential sum is all-reduced over slices: FP64 order differs.
        assert np.allclose(x["e"], np.array(e1), rtol=1e-12, atol=0)
    # Both equal the oracle's own KDK loop.
    from oracle import oracle

    acc0 = oracle.direct_acc(pos, mass, 1.0, EPS * EPS)
    pr, vr, ar = oracle.kdk_direct(pos, vel, acc0, mass, 1.0, EPS * EPS, DT, STEPS)
    assert np.array_equal(p1, pr) and np.array_equal(v1, vr) and np.array_equal(a1, ar)


def test_shard_range_tiles_the_system():
    sh = importlib.import_module(PKG_NAME + ".sharded")
    for n in (0, 1, 7, 8, 1000, 1001):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                t0, nt, chunk = sh.shard_range(n, r, world)
                assert nt >= 0 and t0 == min(r * chunk, n)
                seen.extend(range(t0, t0 + nt))
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        sh.shard_range(10, 2, 2)


# ------------------------------------------------------------------- tree
class OracleTreeOps(OracleOps):
    """The tree step's device work in FP64 on the CPU: the oracle's tree
    (keys, order, topology, summaries) and its per-particle traversal for
    the targets of one slice of the key order."""

    def __init__(self, theta, softening, G, bits):
        super().__init__(G, softening * softening)
        self.theta, self.bits = theta, bits

    def tree_acc(self, x, n, s0, ns, a, phi=None):
        a.zero_()
        if phi is not None:
            phi.zero_()
        if ns == 0:
            return
        xs = x[:n].numpy()
        t = self.orc.bh_tree(xs[:, :3], xs[:, 3], self.bits)
        sel = np.asarray(t["order"][s0:s0 + ns], dtype=np.int64)
        args = (xs[:, :3], t["order"], t["com"], t["nmass"], t["nmin"], t["nmax"], t["left"], t["right"],
                self.theta, self.eps2)
        acc, _ = self.orc.traverse(*args, self.G, 64, sel)
        a[torch.as_tensor(sel), :3] = torch.from_numpy(acc)
        if phi is not None:
            p, _ = self.orc.traverse_phi(*args, 64, sel)
            phi[torch.as_tensor(sel)] = torch.from_numpy(p)


TREE = dict(theta=0.5, softening=0.05, G=1.0, bits=10)


def _tree_worker(rank, world, port, out_dir, n):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sh = importlib.import_module(PKG_NAME + ".sharded")
        pos, vel, mass = _system(n)
        s = sh.ShardedBarnesHut(pos, vel, mass, theta=TREE["theta"], softening=TREE["softening"],
                                G=TREE["G"], key_bits=TREE["bits"], ops=OracleTreeOps(**TREE))
        s.run(DT, STEPS)
        p, v, a = s.gather_state()
        np.savez(os.path.join(out_dir, f"tree{rank}.npz"), p=p, v=v, a=a, e=np.array(s.energies()),
                 s0=s.s0, ns=s.ns)
    finally:
        dist.destroy_process_group()


def test_tree_two_ranks_equal_one_rank(tmp_path):
    """ShardedBarnesHut over two gloo ranks (replicated tree, key-order
    slices, one all-reduce of the accelerations per step) equals the one-rank
    run bit for bit, and both equal the
    oracle's own BH KDK loop; energies agree to FP64 rounding."""
    world, n = 2, 700
    mp.spawn(_tree_worker, args=(world, _free_port(), str(tmp_path), n), nprocs=world, join=True)
    sh = importlib.import_module(PKG_NAME + ".sharded")
    pos, vel, mass = _system(n)
    one = sh.ShardedBarnesHut(pos, vel, mass, theta=TREE["theta"], softening=TREE["softening"], G=TREE["G"],
                              key_bits=TREE["bits"], ops=OracleTreeOps(**TREE))
    one.run(DT, STEPS)
    p1, v1, a1 = one.gather_state()
    e1 = np.array(one.energies())
    r = [np.load(tmp_path / f"tree{k}.npz") for k in range(world)]
    assert [int(x["s0"]) for x in r] == [0, 350] and [int(x["ns"]) for x in r] == [350, 350]
    for x in r:
        assert np.array_equal(x["p"], p1) and np.array_equal(x["v"], v1) and np.array_equal(x["a"], a1)
        # The oracle's FP64 energy sums are OpenMP reductions: their order
        # follows the thread count of each process.
        assert np.allclose(x["e"], e1, rtol=1e-13, atol=0)
    from oracle import oracle

    p, v = pos.copy(), vel.copy()
    a, _, _ = oracle.bh_compute(p, mass, TREE["theta"], TREE["softening"], TREE["G"], bits=TREE["bits"])
    for _ in range(STEPS):
        v = v + a * (0.5 * DT)
        p = p + v * DT
        a, _, _ = oracle.bh_compute(p, mass, TREE["theta"], TREE["softening"], TREE["G"], bits=TREE["bits"])
        v = v + a * (0.5 * DT)
    assert np.array_equal(p1, p) and np.array_equal(v1, v) and np.array_equal(a1, a)
