"""Batched ECMC chains on the GPU: the host side of ``jfgpu_engine_*`` / ``jfgpu_chains_*``.

A ``ChainBatch`` holds thousands of independent chains (each with its own number of particles, box, cell system
and potential) in flat device pools owned by PyTorch tensors, and advances them with one kernel launch whose
event loop runs on the device.  It replaces, for the event-time path, the reference's mediator loop
(``jellyfysh/mediator/single_process_mediator.py:91-156``), tree state handler
(``jellyfysh/state_handler/tree_state_handler.py``), heap scheduler
(``jellyfysh/scheduler/heap_scheduler/heap_scheduler.py``) and single-active cell occupancy
(``jellyfysh/activator/internal_state/single_active_cell_occupancy.py``).
"""
import ctypes
import dataclasses
import json
import math
from typing import List, Optional, Sequence

import numpy as np

from . import _lib

MASK64 = (1 << 64) - 1
GOLDEN = 0x9E3779B97F4A7C15


def _mix64(z: int) -> int:
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def chain_key(seed: int, chain: int) -> int:
    """Key of a chain's keyed random numbers (SplitMix64 output of a Weyl state)."""
    return _mix64((seed + (chain + 1) * GOLDEN) & MASK64)


POTENTIALS = {"hard_sphere": _lib.POT_HARD_SPHERE, "lennard_jones": _lib.POT_LENNARD_JONES,
              "coulomb": _lib.POT_COULOMB}
FAR_FIELDS = {"none": _lib.FAR_NONE, "cell_veto": _lib.FAR_CELL_VETO, "cell_bounding": _lib.FAR_CELL_BOUNDING}
MODES = {"exact": _lib.MODE_EXACT, "mixed": _lib.MODE_MIXED}
# kernel kinds of jfgpu_engine_kernel_times, in JFGPU_KERNEL_* order
KERNEL_KINDS = ("screen", "refine", "resolve", "chains", "init", "observe")

EVENT_DTYPE = np.dtype([("kind", np.int32), ("moved", np.int32), ("target", np.int32), ("new_active", np.int32),
                        ("new_direction", np.int32), ("accepted", np.int32), ("time_q", np.float64),
                        ("time_r", np.float64), ("x", np.float64), ("y", np.float64), ("z", np.float64)])
STATE_DTYPE = np.dtype([("time_q", np.float64), ("time_r", np.float64), ("eoc_q", np.float64),
                        ("eoc_r", np.float64), ("events", np.int64), ("bound_warnings", np.int64),
                        ("refine_fallbacks", np.int64), ("candidates", np.int64), ("refined", np.int64),
                        ("active", np.int32), ("direction", np.int32),
                        ("eoc_new_active", np.int32), ("occ_active", np.int32), ("occ_cell", np.int32),
                        ("n_surplus", np.int32), ("status", np.int32), ("stopped", np.int32),
                        ("lift_sum", np.float64), ("liftings", np.int64), ("far_lookups", np.int64)])
assert EVENT_DTYPE.itemsize == ctypes.sizeof(_lib.Event)
assert STATE_DTYPE.itemsize == ctypes.sizeof(_lib.ChainState)


@dataclasses.dataclass
class ChainSpec:
    """Parameters of one chain, in the reference's vocabulary (INI sections named in brackets).

    potential: "hard_sphere" [HardSpherePotential], "lennard_jones" [LennardJonesPotential] or "coulomb"
    ([MergedImageCoulombPotential] bounded by [InversePowerCoulombBoundingPotential], optional hard core);
    far: "none", "cell_veto" [LeafUnitCellVetoEventHandler] or "cell_bounding" [CellBoundingPotential].
    """
    n: int
    system_length: float
    cells_per_side: int
    potential: str = "hard_sphere"
    far: str = "none"
    neighbor_layers: int = 1
    max_occupants: int = 1
    beta: float = 1.0
    chain_time: float = 1.0
    speed: float = 1.0
    hs_radius: float = 0.0
    lj_prefactor: float = 1.0
    lj_sigma: float = 1.0
    coulomb_prefactor: float = 1.0
    bound_prefactor: float = 1.5837
    ewald_alpha: float = 3.45
    fourier_cutoff: int = 6
    position_cutoff: int = 2
    estimator_points: int = 10
    estimator_prefactor: float = 1.5
    initial_active: int = 0
    initial_direction: int = 0
    rng_key: Optional[int] = None

    def desc(self, key: int) -> _lib.ChainDesc:
        return _lib.ChainDesc(potential=POTENTIALS[self.potential], far=FAR_FIELDS[self.far], n=self.n,
                              cells_per_side=self.cells_per_side, neighbor_layers=self.neighbor_layers,
                              max_occupants=self.max_occupants, initial_active=self.initial_active,
                              initial_direction=self.initial_direction, fourier_cutoff=self.fourier_cutoff,
                              position_cutoff=self.position_cutoff, estimator_points=self.estimator_points,
                              reserved=0, system_length=float(self.system_length), beta=float(self.beta),
                              chain_time=float(self.chain_time), speed=float(self.speed),
                              hs_radius=float(self.hs_radius), lj_prefactor=float(self.lj_prefactor),
                              lj_sigma=float(self.lj_sigma), coulomb_prefactor=float(self.coulomb_prefactor),
                              bound_prefactor=float(self.bound_prefactor), ewald_alpha=float(self.ewald_alpha),
                              estimator_prefactor=float(self.estimator_prefactor), rng_key=key)


def _ptr(tensor) -> Optional[int]:
    return None if tensor is None else tensor.data_ptr()


def check_positions(positions, length: float, what: str) -> None:
    """Refuse positions the device cannot take, before they reach it: not finite, or outside [0, L).  The
    reference's cells map a position by int(x / side) (cuboid_cells.py:190-211), which raises IndexError past the
    box and indexes from the other end below it; on the device such a position would land in a wrong cell."""
    p = np.asarray(positions, dtype=np.float64)
    if not np.isfinite(p).all():
        raise ValueError("%s: positions must be finite" % what)
    if (p < 0.0).any() or (p >= length).any():
        raise ValueError("%s: positions must lie in [0, %r)" % (what, float(length)))


def check_charges(charges, what: str) -> None:
    if not np.isfinite(np.asarray(charges, dtype=np.float64)).all():
        raise ValueError("%s: charges must be finite" % what)


class ChainBatch:
    """Independent ECMC chains advanced together on one GPU."""

    def __init__(self, specs: Sequence[ChainSpec], positions: Sequence[np.ndarray],
                 charges: Optional[Sequence[Optional[np.ndarray]]] = None, seed: int = 0, device: str = "cuda"):
        import torch
        self._torch = torch
        self.specs = list(specs)
        if len(positions) != len(self.specs):
            raise ValueError("one position array per chain is required")
        for c, spec in enumerate(self.specs):
            check_positions(positions[c], spec.system_length, "chain %d" % c)
            if charges is not None and charges[c] is not None:
                check_charges(charges[c], "chain %d" % c)
        self.lib = _lib.load()
        self.device = torch.device(device)
        self.n_chains = len(self.specs)
        descs = (_lib.ChainDesc * self.n_chains)()
        self.keys = []
        for c, spec in enumerate(self.specs):
            key = spec.rng_key if spec.rng_key is not None else chain_key(seed, c)
            self.keys.append(key)
            descs[c] = spec.desc(key)
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device).cuda_stream
            _lib.check(self.lib.jfgpu_engine_create(descs, self.n_chains, stream, ctypes.byref(handle)),
                       "jfgpu_engine_create")
        self._engine = handle
        layout = _lib.Layout()
        _lib.check(self.lib.jfgpu_engine_layout(self._engine, ctypes.byref(layout)), "jfgpu_engine_layout")
        self.layout = layout
        self.particle_offset = np.zeros(self.n_chains, dtype=np.int64)
        self.occupancy_offset = np.zeros(self.n_chains, dtype=np.int64)
        _lib.check(self.lib.jfgpu_engine_offsets(self._engine, self.particle_offset.ctypes.data,
                                                 self.occupancy_offset.ctypes.data), "jfgpu_engine_offsets")
        P, O = int(layout.particles), int(layout.occupancy_slots)
        host_positions = np.zeros((P, 3), dtype=np.float64)
        for c, spec in enumerate(self.specs):
            p = np.asarray(positions[c], dtype=np.float64).reshape(spec.n, 3)
            host_positions[self.particle_offset[c]:self.particle_offset[c] + spec.n] = p
        charged = charges is not None and any(q is not None for q in charges)
        host_charges = None
        if charged:
            host_charges = np.ones(P, dtype=np.float64)
            for c, spec in enumerate(self.specs):
                if charges[c] is not None:
                    host_charges[self.particle_offset[c]:self.particle_offset[c] + spec.n] = np.asarray(
                        charges[c], dtype=np.float64)
        t = torch
        self.positions_dev = t.from_numpy(host_positions).to(self.device)
        self.positions32_dev = t.zeros((P, 4), dtype=t.float32, device=self.device)
        self.charges_dev = None if host_charges is None else t.from_numpy(host_charges).to(self.device)
        self.occupancy_dev = t.full((O,), -1, dtype=t.int32, device=self.device)
        self.surplus_dev = t.zeros((P,), dtype=t.int32, device=self.device)
        self.roles_dev = t.zeros((P,), dtype=t.int32, device=self.device)
        self.cell_slots_dev = t.zeros((O, 4), dtype=t.float32, device=self.device)
        self.state_dev = t.zeros((self.n_chains * STATE_DTYPE.itemsize,), dtype=t.uint8, device=self.device)
        self._buffers = _lib.Buffers(positions=_ptr(self.positions_dev), positions32=_ptr(self.positions32_dev),
                                     charges=_ptr(self.charges_dev), occupancy=_ptr(self.occupancy_dev),
                                     surplus=_ptr(self.surplus_dev), roles=_ptr(self.roles_dev),
                                     state=_ptr(self.state_dev), cell_slots=_ptr(self.cell_slots_dev))
        with torch.cuda.device(self.device):
            _lib.check(self.lib.jfgpu_chains_init(self._engine, ctypes.byref(self._buffers), self._stream()),
                       "jfgpu_chains_init")

    def _stream(self) -> int:
        return self._torch.cuda.current_stream(self.device).cuda_stream

    def close(self) -> None:
        if getattr(self, "_engine", None):
            self._torch.cuda.synchronize(self.device)
            self.lib.jfgpu_engine_destroy(self._engine)
            self._engine = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------------------------------------
    def set_block_warps(self, warps: int) -> None:
        _lib.check(self.lib.jfgpu_chains_set_block_warps(self._engine, int(warps)), "jfgpu_chains_set_block_warps")

    def set_refine_limit(self, limit: int) -> None:
        """Mixed mode: events with more than ``limit`` near-winners (1..28) are re-solved entirely in FP64 (the
        results do not depend on it; a small limit exercises the whole-event FP64 re-solve)."""
        _lib.check(self.lib.jfgpu_chains_set_refine_limit(self._engine, int(limit)), "jfgpu_chains_set_refine_limit")

    # ------------------------------------------------------------------------------------------------
    # checkpoint / resume (the reference dumps its whole mediator with dill, dumping_output_handler.py:70-90, and
    # resumes from it, resume.py:63-105; the device state of a batch is its buffers)
    def checkpoint(self, path: str) -> None:
        """Write the batch (chain parameters with their random-number keys, and every device buffer) to `path`
        (numpy .npz).  ``ChainBatch.restore(path)`` continues it exactly where it stopped."""
        self._torch.cuda.synchronize(self.device)
        specs = [dict(dataclasses.asdict(spec), rng_key=int(key)) for spec, key in zip(self.specs, self.keys)]
        arrays = {name: getattr(self, name + "_dev").cpu().numpy()
                  for name in ("positions", "positions32", "occupancy", "surplus", "roles", "state", "cell_slots")}
        if self.charges_dev is not None:
            arrays["charges"] = self.charges_dev.cpu().numpy()
        np.savez(path, specs=json.dumps(specs), **arrays)

    @classmethod
    def restore(cls, path: str, device: str = "cuda") -> "ChainBatch":
        """The batch written by `checkpoint`: the engine's tables are rebuilt from the chain parameters (they are
        deterministic) and every buffer is loaded back."""
        data = np.load(path)
        specs = [ChainSpec(**entry) for entry in json.loads(str(data["specs"]))]
        batch = cls.__new__(cls)
        positions = np.asarray(data["positions"])
        charges = np.asarray(data["charges"]) if "charges" in data.files else None
        # construct from the saved positions (any valid start), then replace every buffer by the saved one
        offsets = np.concatenate([[0], np.cumsum([spec.n for spec in specs])])
        per_chain = [positions[offsets[c]:offsets[c + 1]] for c in range(len(specs))]
        per_charges = None if charges is None else [charges[offsets[c]:offsets[c + 1]] for c in range(len(specs))]
        batch.__init__(specs, per_chain, per_charges, device=device)
        for name in ("positions", "positions32", "occupancy", "surplus", "roles", "state", "cell_slots"):
            target = getattr(batch, name + "_dev")
            source = batch._torch.from_numpy(np.ascontiguousarray(data[name])).to(batch.device)
            if source.shape != target.shape or source.dtype != target.dtype:
                raise ValueError("checkpoint buffer %s does not match the batch layout" % name)
            target.copy_(source)
        batch._torch.cuda.synchronize(batch.device)
        return batch

    def refresh_mirror(self, first: int = 0, count: Optional[int] = None) -> None:
        """Rewrite the FP32 mirrors of chains [first, first + count) (positions32 from the FP64 positions, the
        cell slots from the occupancy and positions32), after the host has written positions_dev and occupancy_dev."""
        count = self.n_chains - first if count is None else count
        with self._torch.cuda.device(self.device):
            _lib.check(self.lib.jfgpu_chains_refresh_mirror(self._engine, ctypes.byref(self._buffers), int(first),
                                                            int(count), self._stream()),
                       "jfgpu_chains_refresh_mirror")

    def input_tensors(self):
        """The device buffers a host uploads to set the batch's state: FP64 positions, occupancy, surplus lists,
        role words and chain states (the FP32 mirrors follow from them: ``refresh_mirror``)."""
        return [self.positions_dev, self.occupancy_dev, self.surplus_dev, self.roles_dev, self.state_dev]

    def set_graphs(self, enable: bool) -> None:
        """Replay the event rounds of the mixed mode from captured CUDA graphs (default) or launch them plainly."""
        _lib.check(self.lib.jfgpu_chains_set_graphs(self._engine, 1 if enable else 0), "jfgpu_chains_set_graphs")

    def set_groups(self, groups: int) -> None:
        """Split the chains of every mixed-mode run into ``groups`` groups on streams of their own."""
        with self._torch.cuda.device(self.device):
            _lib.check(self.lib.jfgpu_chains_set_groups(self._engine, int(groups)), "jfgpu_chains_set_groups")

    def launch_count(self) -> int:
        return int(self.lib.jfgpu_engine_launch_count(self._engine))

    def observe(self, bins: int = 0, r_max: float = 0.0, first: int = 0, count: Optional[int] = None,
                histogram=None):
        """Potential energy of every chain's configuration (device tensor [count], NaN for Coulomb chains) and,
        with bins > 0, its pair-distance histogram over [0, r_max) ADDED to ``histogram`` (a device int64 tensor
        [count, bins], created when None).  Returns (energy, histogram)."""
        torch = self._torch
        count = self.n_chains - first if count is None else count
        energy = torch.empty(count, dtype=torch.float64, device=self.device)
        if bins and histogram is None:
            histogram = torch.zeros((count, bins), dtype=torch.int64, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self.lib.jfgpu_chains_observe(self._engine, ctypes.byref(self._buffers), int(first), int(count),
                                                     int(bins), float(r_max), _ptr(energy),
                                                     _ptr(histogram) if bins else None, self._stream()),
                       "jfgpu_chains_observe")
        return energy, histogram

    def set_timing(self, enable: bool, stride: int = 1) -> None:
        """Bracket the chain launches by CUDA events on their streams (read back by kernel_times); in the mixed
        mode every `stride`-th event round only."""
        _lib.check(self.lib.jfgpu_engine_set_timing(self._engine, int(stride) if enable else 0),
                   "jfgpu_engine_set_timing")

    def kernel_times(self, reset: bool = True) -> dict:
        """Device milliseconds and launches per kernel kind since the last reset (waits for the events)."""
        ms = (ctypes.c_double * len(KERNEL_KINDS))()
        n = (ctypes.c_int64 * len(KERNEL_KINDS))()
        _lib.check(self.lib.jfgpu_engine_kernel_times(self._engine, ms, n, 1 if reset else 0),
                   "jfgpu_engine_kernel_times")
        return {name: {"ms": ms[k], "launches": int(n[k])} for k, name in enumerate(KERNEL_KINDS)}

    def run(self, max_events: int, stop_time: Optional[float] = None, mode: str = "mixed", first: int = 0,
            count: Optional[int] = None, log_capacity: int = 0, sync: bool = True):
        """Advance chains [first, first + count) by at most ``max_events`` events each (or to ``stop_time``).

        Returns the device event log as a numpy structured array [count, log_capacity] when log_capacity > 0."""
        torch = self._torch
        count = self.n_chains - first if count is None else count
        stop_q, stop_r = (math.inf, math.inf) if stop_time is None else divmod(float(stop_time), 1.0)
        log = None
        if log_capacity:
            log = torch.zeros((count * log_capacity * EVENT_DTYPE.itemsize,), dtype=torch.uint8, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self.lib.jfgpu_chains_run(self._engine, ctypes.byref(self._buffers), int(first), int(count),
                                                 int(max_events), stop_q, stop_r, MODES[mode], _ptr(log),
                                                 int(log_capacity), self._stream()), "jfgpu_chains_run")
        if sync:
            torch.cuda.synchronize(self.device)
        if log is not None:
            return np.frombuffer(log.cpu().numpy().tobytes(), dtype=EVENT_DTYPE).reshape(count, log_capacity)
        return None

    # ------------------------------------------------------------------------------------------------
    def state(self) -> np.ndarray:
        raw = self.state_dev.cpu().numpy().tobytes()
        return np.frombuffer(raw, dtype=STATE_DTYPE).copy()

    def positions(self, chain: Optional[int] = None):
        host = self.positions_dev.cpu().numpy()
        if chain is not None:
            o = self.particle_offset[chain]
            return host[o:o + self.specs[chain].n].copy()
        return [host[o:o + s.n].copy() for o, s in zip(self.particle_offset, self.specs)]

    def occupancy(self, chain: int) -> np.ndarray:
        spec = self.specs[chain]
        o = self.occupancy_offset[chain]
        host = self.occupancy_dev[o:o + spec.cells_per_side ** 3 * spec.max_occupants].cpu().numpy()
        return host.reshape(spec.cells_per_side ** 3, spec.max_occupants)

    def surplus(self, chain: int) -> np.ndarray:
        n_surplus = int(self.state()[chain]["n_surplus"])
        o = self.particle_offset[chain]
        return self.surplus_dev[o:o + n_surplus].cpu().numpy().copy()

    def roles(self, chain: int) -> np.ndarray:
        """Role word of every unit (cell axes x | y << 8 | z << 16; surplus units: bit 24 and their index in the
        surplus list; the occupancy's active unit: bit 25)."""
        o = self.particle_offset[chain]
        return self.roles_dev[o:o + self.specs[chain].n].cpu().numpy().copy()

    def bounds(self, chain: int):
        spec = self.specs[chain]
        cells = spec.cells_per_side ** 3
        upper = np.zeros(cells * 3, dtype=np.float64)
        lower = np.zeros(cells * 3, dtype=np.float64)
        _lib.check(self.lib.jfgpu_engine_bounds(self._engine, chain, upper.ctypes.data, lower.ctypes.data,
                                                cells * 3), "jfgpu_engine_bounds")
        return upper.reshape(cells, 3), lower.reshape(cells, 3)

    def check_status(self) -> None:
        state = self.state()
        bad = np.nonzero(state["status"])[0]
        if bad.size:
            c = int(bad[0])
            raise _lib.JfgpuError("chain %d stopped: %s" % (c, _lib.STATUS_NAMES.get(int(state["status"][c]),
                                                                                      state["status"][c])))

    # ---- host <-> device state transfer (the end-to-end path of a caller holding host buffers) ----
    def state_tensors(self):
        return [self.positions_dev, self.positions32_dev, self.cell_slots_dev, self.occupancy_dev, self.surplus_dev,
                self.roles_dev, self.state_dev]
