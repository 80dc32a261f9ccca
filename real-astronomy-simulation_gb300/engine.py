"""Drop-in ``Engine`` for the reference's core/engine.py:32-124.

Same constructor (softening, gravity_mode, theta), same methods (load_state,
to_state, step, energies, _compute_acc) and attributes (n, time, step_count,
seed, meta, pos/vel/acc/mass), with the state resident on the GPU as float32
float4 records and every force evaluation running in the sm_103a CUDA
library.  Extra keyword arguments: ``G`` (default core/units.py:21),
``key_bits`` (Morton key width of the tree path; the reference uses 21),
``max_stack`` (traversal stack rule, reference default 64), ``plain_fp32``
(disable Kahan accumulation; ``precision="fp32"`` says the same,
``precision="fp32-kahan"`` the default), ``symmetric`` (direct sum: evaluate each
unordered pair once and update both particles, default; False runs one pass
per target), ``check`` (tree mode: every step waits for the device and
raises GravityError when the traversal's max_stack rule dropped work or a
position is not finite; the reference drops such work silently),
``bh_traversal`` (tree mode: traversal shape, default -1, the per-particle
walk of the reference; 3 selects the group walk, see
BarnesHut.set_traversal), ``fused_potential`` (whether the force pass
also writes the potential of its positions, so that ``energies()`` after it
runs only the O(N) FP64 reductions instead of a potential pass of its own;
the potential costs about a tenth of a step.  True: the last step of every
``step``/``run`` call and the priming in ``load_state``; False: never;
"auto" (default): the priming, and the step that ends where the cadence of
the last two ``energies()`` calls puts the next one, as a run loop that
prints every k steps does), ``device``.

Energies (core/engine.py:119-124): the direct mode's potential is the
potential_energy sum (core/solvers/gravity.py:39-57); the tree mode's is the
tree potential of the traversal (monopole terms of the accepted nodes),
which agrees with that sum within the tree's own error.
``energies(exact=True)`` runs the O(N^2) sum in either mode, as the
reference does at every call.

As in the reference (core/engine.py:75-80), gravity_mode="bh" uses the tree
only for n >= 256; smaller systems use the direct sum.
"""
from __future__ import annotations

import numpy as np
import torch

from . import units
from ._dev import FieldView, empty4, pack_vec, pack_xm, require_cuda
from .solvers.gravity import DirectGravity
from .state import State

BH_MIN_N = 256


def init_taichi(arch: str = "cuda") -> None:
    """Accepted for call-site compatibility with core/engine.py:21-29; the
    engine always runs on the CUDA device."""
    require_cuda()


class Engine:
    def __init__(self, softening: float = 0.05, gravity_mode: str = "direct",
                 theta: float = 0.6, *, G: float = units.G, key_bits: int = 21,
                 max_stack: int = 64, plain_fp32: bool = False, symmetric: bool = True,
                 check: bool = False, fused_potential="auto", bh_traversal: int = -1,
                 precision: str | None = None, device=None):
        if gravity_mode not in ("direct", "bh"):
            raise ValueError(f"gravity_mode must be 'direct' or 'bh', got {gravity_mode!r}")
        if fused_potential not in (True, False, "auto"):
            raise ValueError(f"fused_potential must be True, False or 'auto', got {fused_potential!r}")
        if precision is not None:
            if precision not in ("fp32-kahan", "fp32"):
                raise ValueError(f"precision must be 'fp32-kahan' or 'fp32', got {precision!r}")
            plain_fp32 = precision == "fp32"
        self.softening = float(softening)
        self.gravity_mode = gravity_mode
        self.theta = float(theta)
        self.G = float(G)
        self.key_bits = int(key_bits)
        self.max_stack = int(max_stack)
        self.plain_fp32 = bool(plain_fp32)
        self.symmetric = bool(symmetric)
        self.check = bool(check)
        self.fused_potential = fused_potential
        self._e_steps: list = []     # step counts of the last energies() calls
        self.potential_passes = 0    # potential passes energies() had to run itself
        self.bh_traversal = int(bh_traversal)
        self.phi = None          # potential sums (no G) of the current positions, when valid
        self._phi_valid = False
        self.device = require_cuda(device)
        self._bh = None
        self._direct = None
        self.n = 0
        self.time = 0.0
        self.step_count = 0
        self.seed = 0
        self.meta: dict = {}
        self.xm = self.v4 = self.a4 = None
        self._ptype = self._ids = None
        self._age = self._temperature = self._metallicity = None

    # ---------------------------------------------------------------- fields
    @property
    def pos(self):
        return None if self.xm is None else FieldView(self.xm, slice(0, 3), self._invalidate_phi)

    @property
    def mass(self):
        return None if self.xm is None else FieldView(self.xm, 3, self._invalidate_phi)

    def _invalidate_phi(self) -> None:
        """Positions or masses were written: the stored potential is stale."""
        self._phi_valid = False

    @property
    def vel(self):
        return None if self.v4 is None else FieldView(self.v4, slice(0, 3))

    @property
    def acc(self):
        return None if self.a4 is None else FieldView(self.a4, slice(0, 3))

    @property
    def eps2(self) -> float:
        return self.softening ** 2

    # ----------------------------------------------------------------- setup
    def load_state(self, state: State) -> None:
        """Upload a State and prime the accelerations (core/engine.py:53-81)."""
        self.n = state.n
        self.time = state.time
        self.step_count = state.step
        self._e_steps = []  # the energies() cadence restarts with a new state
        self.seed = state.seed
        self.meta = dict(state.meta)
        self._ptype = state.ptype.copy()
        self._ids = state.ids.copy()
        self._age = state.age
        self._temperature = state.temperature
        self._metallicity = state.metallicity
        with torch.cuda.device(self.device):
            self.xm = pack_xm(state.pos, state.mass, self.device)
            self.v4 = pack_vec(state.vel, self.device)
            self.a4 = empty4(self.n, self.device)
            self.phi = torch.zeros(self.n, dtype=torch.float32, device=self.device)
            self._make_solvers()
            self._compute_acc()

    def _make_solvers(self) -> None:
        if self.gravity_mode == "bh" and self.n >= BH_MIN_N:
            from .solvers.barnes_hut import BarnesHut
            self._bh = BarnesHut(self.n, theta=self.theta, softening=self.softening,
                                 max_stack=self.max_stack, key_bits=self.key_bits,
                                 G=self.G, check=self.check, device=self.device)
            if self.bh_traversal != -1:
                self._bh.set_traversal(self.bh_traversal)
        else:
            self._bh = None
            self._direct_solver()

    def _direct_solver(self) -> DirectGravity:
        """The direct-sum solver, made on first use: the direct mode steps with
        it; the tree mode needs it only for a potential its steps did not
        provide."""
        if self._direct is None or self._direct.n_max < max(self.n, 1):
            self._direct = DirectGravity(max(self.n, 1), self.device)
            self._direct.set_variant(2 if self.symmetric else 0)
        return self._direct

    def to_state(self) -> State:
        """Download the state into a host State (core/engine.py:83-98)."""
        xm = self.xm.detach().cpu().numpy().astype(np.float64)
        vel = self.v4.detach().cpu().numpy().astype(np.float64)
        return State(pos=xm[:, :3], vel=vel[:, :3], mass=xm[:, 3], ptype=self._ptype,
                     ids=self._ids, time=self.time, step=self.step_count, seed=self.seed,
                     age=self._age, temperature=self._temperature,
                     metallicity=self._metallicity, meta=dict(self.meta))

    def to_device_state(self) -> dict:
        """The state without a host copy: device tensor views of the engine's
        float32 records (pos, vel, acc: (n, 3); mass: (n,)) plus time and
        step.  The views change as the engine steps; copy them to keep a
        snapshot (see snapshot.SnapshotWriter)."""
        return {"pos": self.xm[:, :3], "vel": self.v4[:, :3], "mass": self.xm[:, 3],
                "acc": self.a4[:, :3], "time": self.time, "step": self.step_count}

    def load_device_state(self, pos: torch.Tensor, vel: torch.Tensor, mass: torch.Tensor, *,
                          time: float = 0.0, step: int = 0, seed: int = 0, ptype=None, ids=None,
                          meta: dict | None = None) -> None:
        """load_state from device tensors (copied device to device, no host
        round trip) and prime the accelerations."""
        n = int(pos.shape[0])
        self.n = n
        self.time = float(time)
        self.step_count = int(step)
        self._e_steps = []
        self.seed = int(seed)
        self.meta = dict(meta or {})
        self._ptype = np.zeros(n, np.int32) if ptype is None else np.asarray(ptype, np.int32).copy()
        self._ids = np.arange(n, dtype=np.int64) if ids is None else np.asarray(ids, np.int64).copy()
        self._age = self._temperature = self._metallicity = None
        with torch.cuda.device(self.device):
            self.xm = empty4(n, self.device)
            self.xm[:, :3] = pos.to(self.device, torch.float32)
            self.xm[:, 3] = mass.to(self.device, torch.float32)
            self.v4 = empty4(n, self.device)
            self.v4[:, :3] = vel.to(self.device, torch.float32)
            self.a4 = empty4(n, self.device)
            self.phi = torch.zeros(n, dtype=torch.float32, device=self.device)
            self._make_solvers()
            self._compute_acc()

    # -------------------------------------------------------------- stepping
    def _compute_acc(self) -> None:
        """core/engine.py:101-106 (with fused_potential the same pass also
        writes the potential)."""
        self._phi_valid = False
        if self.n == 0:
            return
        phi = self.phi if self.fused_potential in (True, "auto") else None
        with torch.cuda.device(self.device):
            if self._bh is not None:
                self._bh.compute(self.xm, self.a4, phi=phi)
            elif phi is not None:
                self._direct.acc_phi(self.xm, self.a4, phi, self.G, self.eps2, plain=self.plain_fp32)
            else:
                self._direct.acc(self.xm, self.a4, self.G, self.eps2, plain=self.plain_fp32)
        self._phi_valid = phi is not None

    def _fuse_at(self, end_step: int) -> bool:
        """Whether the run ending at end_step writes the potential."""
        if self.fused_potential in (True, False):
            return self.fused_potential
        if len(self._e_steps) < 2:
            return False
        last, k = self._e_steps[-1], self._e_steps[-1] - self._e_steps[-2]
        return k > 0 and end_step > last and (end_step - last) % k == 0

    def step(self, dt: float) -> None:
        """One KDK step (core/engine.py:108-116); kick and drift are fused
        into the force pass."""
        self.run(dt, 1)

    def run(self, dt: float, nsteps: int) -> None:
        """nsteps KDK steps without returning to Python in between."""
        if nsteps <= 0:
            return
        if self.n > 0:
            self._phi_valid = False
            phi = self.phi if self._fuse_at(self.step_count + nsteps) else None
            with torch.cuda.device(self.device):
                if self._bh is not None:
                    self._bh.kdk(self.xm, self.v4, self.a4, dt, nsteps, phi=phi)
                else:
                    self._direct.kdk(self.xm, self.v4, self.a4, self.G, self.eps2, dt, nsteps,
                                     plain=self.plain_fp32, graph=True, phi=phi)
            self._phi_valid = phi is not None
        self.time += dt * nsteps
        self.step_count += nsteps

    # ----------------------------------------------------------- diagnostics
    def energies(self, exact: bool = False) -> tuple[float, float, float]:
        """(kinetic, potential, total) in code units (core/engine.py:119-124),
        FP64 reductions.  The potential is the one the last force pass wrote
        (fused_potential) when it is current, else a pass of its own: the
        tree potential in tree mode, the FP32-Kahan pair sum otherwise.
        exact=True always runs the O(N^2) pair sum, as the reference does."""
        if self.n == 0:
            return 0.0, 0.0, 0.0
        with torch.cuda.device(self.device):
            if exact:
                return self._direct_solver().energies(self.xm, self.v4, self.G, self.eps2)
            if not self._e_steps or self._e_steps[-1] != self.step_count:
                self._e_steps = (self._e_steps + [self.step_count])[-2:]
            if not self._phi_valid:
                self.potential_passes += 1
                if self._bh is not None:
                    self._bh.compute(self.xm, torch.empty_like(self.a4), phi=self.phi)
                else:
                    self._direct.phi(self.xm, self.eps2, out=self.phi, plain=self.plain_fp32)
                self._phi_valid = True
            if self._bh is not None:
                return self._bh.energies_from_phi(self.xm, self.v4, self.phi)
            return self._direct.energies_from_phi(self.xm, self.v4, self.phi, self.G)

    def diagnostics(self) -> dict:
        """The energy / virial record a simulation controller shows
        (core/sim_controller.py:288-293 builds it from energies() for an
        engine without its own diagnostics): kinetic, potential, thermal (0:
        no gas here), total and the virial ratio 2 KE / |PE| (0 when PE is
        0)."""
        ke, pe, tot = self.energies()
        return dict(kinetic=ke, potential=pe, thermal=0.0, total=tot,
                    virial=(2.0 * ke / abs(pe) if pe else 0.0))

    def diag(self) -> dict:
        d = self._direct.diag() if self._direct is not None else {}
        if self._bh is not None:
            for k, v in self._bh.diag().items():
                d[k] = d.get(k, 0) + v
        return d
