"""Snapshots written off the critical path (snapshot.py) against the
engine's synchronous to_state at the same steps, and device-resident state
access.  The snapshot holds the same float32 records, so comparisons are
exact."""
import importlib
import os

import numpy as np
import pytest
import torch

from conftest import PKG_NAME

pytestmark = pytest.mark.gpu


def _mods():
    return (importlib.import_module(PKG_NAME), importlib.import_module(PKG_NAME + ".snapshot"),
            importlib.import_module(PKG_NAME + ".ic"), importlib.import_module(PKG_NAME + ".state"))


def _state(kind, n):
    pkg, _, ic, st = _mods()
    if kind == "direct":
        p, v, m = ic.plummer(n, seed=3)
    else:
        p, v, m = ic.exponential_disk(n, seed=4)
    return st.State.from_arrays(p, v, m, meta={"scene": kind})


def _load(path):
    _, snap, _, st = _mods()
    return st.State.load_npz(path) if path.endswith(".npz") else st.State.load(path)


@pytest.mark.parametrize("mode,n", [("direct", 1500), ("bh", 4000)])
def test_async_snapshots_equal_synchronous_states(cuda_dev, tmp_path, mode, n):
    pkg, snap, _, _ = _mods()
    s0 = _state(mode, n)
    e1 = pkg.Engine(softening=0.05, gravity_mode=mode, theta=0.5, device=cuda_dev)
    e1.load_state(s0)
    last = snap.run_with_snapshots(e1, 1e-4, 50, str(tmp_path), snap_every=20, meta={"run": "a"})
    assert last == 2
    e2 = pkg.Engine(softening=0.05, gravity_mode=mode, theta=0.5, device=cuda_dev)
    e2.load_state(s0)
    ext = ".h5" if snap.has_h5py() else ".npz"
    for frame, steps in ((0, 0), (1, 20), (2, 20)):
        e2.run(1e-4, steps)
        ref = e2.to_state()
        got = _load(os.path.join(str(tmp_path), f"snap_{frame:04d}{ext}"))
        for name in ("pos", "vel", "mass", "ptype", "ids"):
            np.testing.assert_array_equal(getattr(got, name), getattr(ref, name))
        assert got.step == ref.step == 20 * frame
        assert got.time == pytest.approx(ref.time, abs=0.0)
        assert got.meta["run"] == "a" and got.meta["scene"] == mode
    assert e1.step_count == 50


def test_writer_error_is_raised_on_close(cuda_dev, tmp_path):
    pkg, snap, _, _ = _mods()
    e = pkg.Engine(softening=0.05, device=cuda_dev)
    e.load_state(_state("direct", 300))

    def bad_writer(state, path):
        raise OSError("disk full")

    w = snap.SnapshotWriter(e, writer=bad_writer)
    w.request(str(tmp_path / "x.npz"))
    with pytest.raises(OSError):
        w.close()


def test_device_state_round_trip(cuda_dev):
    pkg, _, _, _ = _mods()
    s0 = _state("bh", 3000)
    a = pkg.Engine(softening=0.05, gravity_mode="bh", theta=0.5, device=cuda_dev)
    a.load_state(s0)
    a.run(1e-4, 5)
    d = a.to_device_state()
    host = a.to_state()
    np.testing.assert_array_equal(d["pos"].double().cpu().numpy(), host.pos)
    assert d["pos"].data_ptr() == a.xm.data_ptr()  # a view, no copy
    b = pkg.Engine(softening=0.05, gravity_mode="bh", theta=0.5, device=cuda_dev)
    b.load_device_state(d["pos"], d["vel"], d["mass"], time=d["time"], step=d["step"])
    c = pkg.Engine(softening=0.05, gravity_mode="bh", theta=0.5, device=cuda_dev)
    c.load_state(host)
    b.run(1e-4, 5)
    c.run(1e-4, 5)
    assert torch.equal(b.xm, c.xm) and torch.equal(b.v4, c.v4) and b.step_count == c.step_count == 10
