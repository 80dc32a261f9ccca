"""Host state container with the reference's contract (core/state.py:26-110):
float64 (N,3) positions/velocities, (N,) masses, int32 particle types, int64
ids, time/step/seed and free-form meta.  HDF5 I/O keeps the reference's file
layout and needs h5py (imported lazily, as in the reference)."""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

PTYPE_DM = 0
PTYPE_STAR = 1
PTYPE_GAS = 2

_OPTIONAL = ("age", "temperature", "metallicity", "u", "rho")


@dataclass
class State:
    pos: np.ndarray
    vel: np.ndarray
    mass: np.ndarray
    ptype: np.ndarray
    ids: np.ndarray
    time: float = 0.0
    step: int = 0
    seed: int = 0
    age: Optional[np.ndarray] = None
    temperature: Optional[np.ndarray] = None
    metallicity: Optional[np.ndarray] = None
    u: Optional[np.ndarray] = None
    rho: Optional[np.ndarray] = None
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.pos.shape[0]

    def __post_init__(self) -> None:
        self.pos = np.ascontiguousarray(self.pos, dtype=np.float64).reshape(-1, 3)
        self.vel = np.ascontiguousarray(self.vel, dtype=np.float64).reshape(-1, 3)
        self.mass = np.ascontiguousarray(self.mass, dtype=np.float64).reshape(-1)
        self.ptype = np.ascontiguousarray(self.ptype, dtype=np.int32).reshape(-1)
        self.ids = np.ascontiguousarray(self.ids, dtype=np.int64).reshape(-1)

    @classmethod
    def from_arrays(cls, pos, vel, mass, **kw) -> "State":
        n = np.asarray(pos).reshape(-1, 3).shape[0]
        kw.setdefault("ptype", np.zeros(n, np.int32))
        kw.setdefault("ids", np.arange(n, dtype=np.int64))
        return cls(pos=pos, vel=vel, mass=mass, **kw)

    def save(self, path: str) -> None:
        import h5py

        with h5py.File(path, "w") as f:
            f.attrs["time"] = float(self.time)
            f.attrs["step"] = int(self.step)
            f.attrs["seed"] = int(self.seed)
            f.attrs["n"] = int(self.n)
            f.attrs["units"] = "kpc, km/s, 1e10 Msun"
            for k, v in self.meta.items():
                f.attrs[f"meta_{k}"] = v if np.isscalar(v) else str(v)
            for name in ("pos", "vel", "mass", "ptype", "ids"):
                f.create_dataset(name, data=getattr(self, name), compression="gzip")
            for name in _OPTIONAL:
                arr = getattr(self, name)
                if arr is not None:
                    f.create_dataset(name, data=np.asarray(arr, dtype=np.float64),
                                     compression="gzip")

    def save_npz(self, path: str) -> None:
        """The same datasets and attributes as save(), in a numpy .npz file
        (for hosts without h5py)."""
        arrays = {name: getattr(self, name) for name in ("pos", "vel", "mass", "ptype", "ids")}
        for name in _OPTIONAL:
            arr = getattr(self, name)
            if arr is not None:
                arrays[name] = np.asarray(arr, dtype=np.float64)
        attrs = {"time": float(self.time), "step": int(self.step), "seed": int(self.seed),
                 "n": int(self.n)}
        for k, v in attrs.items():
            arrays[f"attr_{k}"] = np.asarray(v)
        for k, v in self.meta.items():
            arrays[f"meta_{k}"] = np.asarray(v if np.isscalar(v) else str(v))
        with open(path, "wb") as f:
            np.savez(f, **arrays)

    @classmethod
    def load_npz(cls, path: str) -> "State":
        with np.load(path, allow_pickle=False) as z:
            meta = {k[len("meta_"):]: z[k].item() for k in z.files if k.startswith("meta_")}
            optional = {name: z[name] for name in _OPTIONAL if name in z.files}
            return cls(pos=z["pos"], vel=z["vel"], mass=z["mass"], ptype=z["ptype"], ids=z["ids"],
                       time=float(z["attr_time"]), step=int(z["attr_step"]), seed=int(z["attr_seed"]),
                       meta=meta, **optional)

    @classmethod
    def load(cls, path: str) -> "State":
        import h5py

        with h5py.File(path, "r") as f:
            meta = {k[len("meta_"):]: f.attrs[k] for k in f.attrs if k.startswith("meta_")}
            optional = {name: f[name][:] for name in _OPTIONAL if name in f}
            return cls(pos=f["pos"][:], vel=f["vel"][:], mass=f["mass"][:],
                       ptype=f["ptype"][:], ids=f["ids"][:],
                       time=float(f.attrs["time"]), step=int(f.attrs["step"]),
                       seed=int(f.attrs["seed"]), meta=meta, **optional)
