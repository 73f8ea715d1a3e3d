"""Batched chains of flexible water on the GPU (``jfgpu_water_*`` in ``include/jfgpu.h``).

A chain holds ``molecules`` water molecules as composite objects of three point charges (hydrogen, oxygen,
hydrogen; unit ``3 m + t``).  Its factors are those of the reference's water built from a factor-set file
(``activator/tagger/factor_type_maps.py``): harmonic O–H and H–H bonds (``DisplacedEvenPowerPotential``),
Lennard-Jones between oxygens (``TwoLeafUnitEventHandler``) and one Coulomb factor per pair of molecules
(``TwoCompositeObjectSummedBoundingPotentialEventHandler`` with merged-image Coulomb, the summed inverse-power
Coulomb bound and a lifting scheme), for every pair of molecules; chains end by the periodic-direction end of
chain.  One block advances one chain with the event loop on the device, in FP64 with the reference's arithmetic.  In
the mixed mode (the default) the Coulomb candidates are screened in FP32 with error bounds and only those that may
come first are solved in FP64, and the thinning of a Coulomb event first tries FP32 merged-image sums with an
error bound; every outcome is the exact mode's.
"""
import ctypes
import json
import math
from dataclasses import asdict, dataclass
from typing import Optional

import numpy as np

from . import _lib
from .chains import EVENT_DTYPE

KILOCALORIE_PER_MOLE_KELVIN = 0.0019872041
LIFTING = {"inside_first": _lib.LIFTING_INSIDE_FIRST, "outside_first": _lib.LIFTING_OUTSIDE_FIRST,
           "ratio": _lib.LIFTING_RATIO}
STATE_DTYPE = np.dtype([("time_q", np.float64), ("time_r", np.float64), ("eoc_q", np.float64), ("eoc_r", np.float64),
                        ("active", np.int32), ("direction", np.int32), ("eoc_new_active", np.int32),
                        ("status", np.int32), ("stopped", np.int32), ("reserved", np.int32), ("events", np.int64),
                        ("composite_events", np.int64),
                        ("composite_accepted", np.int64), ("bond_events", np.int64), ("lj_events", np.int64),
                        ("eoc_events", np.int64), ("thinning_exact", np.int64), ("refined_items", np.int64)])
MODES = {"exact": _lib.MODE_EXACT, "mixed": _lib.MODE_MIXED}
CELL_STATE_DTYPE = np.dtype([("pair_q", np.float64), ("pair_r", np.float64), ("snap_leaf", np.float64, 3),
                             ("snap_root", np.float64, 3), ("snap_q", np.float64), ("snap_r", np.float64),
                             ("pair_kind", np.int32), ("pair_target", np.int32), ("pairs_valid", np.int32),
                             ("occ_active", np.int32), ("occ_cell", np.int32), ("reserved", np.int32),
                             ("boundary_events", np.int64), ("veto_events", np.int64), ("veto_targets", np.int64)])


@dataclass
class WaterCells:
    """The molecular cells of the reference's water cell-veto configuration
    (``config_files/2018_JCP_149_064113/water/coulomb_cell_veto_lj_inverted.ini``): cells_per_side^3 cuboid periodic
    cells of the molecules' root units with neighbor_layers layers of nearby cells, one occupant per cell, and the
    molecular cell veto's bound tables [cells][3] (upper and negated lower derivative bound of every relative cell
    and direction; NaN for the nearby cells).  keep_pairs: the cell boundary's tagger trashes only the cell-based
    factors (the reference's configuration: the bond and Lennard-Jones candidates outlive it); False: it trashes them
    too.  far: "cell_veto", or "cell_bounding" (``TwoCompositeObjectCellBoundingPotentialEventHandler`` with its tagger:
    a factor for every occupied far cell, as the reference's dipole configuration ``dipoles/cell_bounded.ini`` sets it
    up; the charge factor divides by the estimator's ``dipole_charge``)."""

    cells_per_side: int
    neighbor_layers: int
    bounds_upper: np.ndarray
    bounds_lower: np.ndarray
    keep_pairs: bool = True
    far: str = "cell_veto"
    dipole_charge: float = 1.0

    @property
    def cells(self) -> int:
        return self.cells_per_side ** 3


def dipole_cell_veto_bounds(model: "WaterModel", cells_per_side: int, neighbor_layers: int,
                            dipole_separation: float = 0.5, dipole_charge: float = 0.82, prefactor: float = 1.5,
                            number_trials: int = 1000, empirical_bound: float = 30.0, seed: int = 0,
                            keep_pairs: bool = True, far: str = "cell_veto") -> WaterCells:
    """The bound tables of the molecular cell veto as the reference's ``CellVetoEventHandler.initialize``
    (``event_handler/abstracts/cell_veto_event_handler.py:93-160``), and of the molecular cell-bounding factor as
    ``CellBoundingPotential.initialize`` (``potential/cell_bounding_potential.py:70-126``), fill them with the
    ``DipoleMonteCarloEstimator`` (``estimator/dipole_monte_carlo_estimator.py:74-155``): for every relative cell
    that is not nearby and every direction, ``number_trials`` dipoles of two charges ``±dipole_charge`` at distance
    ``dipole_separation`` (centre uniform in the cell separation's box widened by half the separation, direction
    uniform on the sphere by rejection from the cube, both ends wrapped into the box), the largest absolute summed
    merged-image derivative against a unit charge times ``prefactor``, capped by ``empirical_bound``; upper bound
    that value, lower bound its negative (stored negated).  The trials draw from ``numpy.random.default_rng(seed)``
    (not the reference's stream: equal in distribution) and every derivative is evaluated by one batched GPU call
    (``jfgpu_merged_image_coulomb_derivative``)."""
    from . import potentials
    m = int(cells_per_side)
    length = float(model.system_length)
    lo, hi = _cell_bounds(length, m)
    near = np.zeros(m, dtype=bool)
    for o in range(-neighbor_layers, neighbor_layers + 1):
        near[o % m] = True
    cells = m ** 3
    far_cells = [c for c in range(cells) if not (near[c % m] and near[(c // m) % m] and near[c // (m * m)])]
    rng = np.random.default_rng(seed)
    half = dipole_separation / 2.0
    n_far = len(far_cells)
    lower_corner = np.empty((n_far, 3))
    upper_corner = np.empty((n_far, 3))
    for i, c in enumerate(far_cells):
        axes = (c % m, (c // m) % m, c // (m * m))
        for d in range(3):
            lower_corner[i, d] = lo[axes[d]] - hi[0] - half
            upper_corner[i, d] = hi[axes[d]] - lo[0] + half
    # [far cell][direction][trial]: centres and directions on the sphere
    shape = (n_far, 3, int(number_trials))
    centres = lower_corner[:, None, None, :] + (upper_corner - lower_corner)[:, None, None, :] * rng.random(shape + (3,))
    directions = np.empty(shape + (3,))
    pending = np.ones(shape, dtype=bool)
    while pending.any():
        trial = rng.uniform(-1.0, 1.0, (int(pending.sum()), 3))
        norms = np.sqrt((trial * trial).sum(axis=1))
        ok = (norms > 0.0) & (norms <= 1.0)
        index = np.argwhere(pending)[ok]
        directions[tuple(index.T)] = trial[ok] / norms[ok, None]
        pending[tuple(index.T)] = False
    ends = np.stack([centres + directions * half, centres - directions * half])  # [2][far][dir][trial][3]
    ends = np.mod(ends + length / 2.0, length) - length / 2.0
    velocities = np.zeros(ends.shape)
    for d in range(3):
        velocities[:, :, d, :, d] = 1.0
    charges = np.empty(ends.shape[:-1] + (2,))
    charges[..., 0] = 1.0
    charges[0, ..., 1] = dipole_charge
    charges[1, ..., 1] = -dipole_charge
    values, status = potentials.merged_image_coulomb_derivative(
        model.alpha, model.fourier_cutoff, model.position_cutoff, model.coulomb_prefactor, length,
        velocities.reshape(-1, 3), ends.reshape(-1, 3), charges.reshape(-1, 2))
    if np.any(status != 0):
        raise RuntimeError("merged-image derivative failed in the dipole estimator")
    values = values.reshape(2, n_far, 3, int(number_trials))
    upper = np.abs(values[0] + values[1]).max(axis=2) * prefactor
    upper = np.minimum(empirical_bound, upper)
    bounds_upper = np.full((cells, 3), np.nan)
    bounds_lower = np.full((cells, 3), np.nan)
    bounds_upper[far_cells] = upper
    bounds_lower[far_cells] = -np.maximum(-empirical_bound, -upper)
    return WaterCells(m, int(neighbor_layers), bounds_upper, bounds_lower, bool(keep_pairs), far,
                      float(dipole_charge))


def _cell_bounds(length: float, m: int):
    """Exact float bounds of the cells along one axis (``cuboid_cells.py:115-131``)."""
    side = length / m
    lo, hi = [], []
    for i in range(m):
        lower, upper = i * side, (i + 1) * side
        if lower > 0.0:
            while int(lower / side) == i:
                lower = np.nextafter(lower, -np.inf)
            while int(lower / side) < i:
                lower = np.nextafter(lower, np.inf)
        while int(upper / side) == i:
            upper = np.nextafter(upper, np.inf)
        while int(upper / side) > i:
            upper = np.nextafter(upper, -np.inf)
        lo.append(float(lower))
        hi.append(float(upper))
    return lo, hi


@dataclass
class WaterModel:
    """Flexible water in kcal/mol, Å and e.  Defaults: 64 molecules in a 12.42 Å box at 300 K, O–H bonds
    r0 = 1.0 Å with k = 1059 kcal/mol/Å² and H–H r0 = 1.633 Å with k = 684 (prefactor k/2 of (r - r0)^2),
    Lennard-Jones on oxygen ε = 0.1554 kcal/mol (prefactor 4ε), σ = 3.166 Å, charges O −0.82 e, H +0.41 e with
    merged-image Coulomb (332.0637 kcal Å/mol/e²) bounded by 1.6 times its prefactor, inside-first lifting."""

    molecules: int = 64
    system_length: float = 12.42
    beta: float = 1.0 / (KILOCALORIE_PER_MOLE_KELVIN * 300.0)
    chain_time: float = 2.0
    speed: float = 1.0
    initial_active: int = 1
    initial_direction: int = 0
    oh_r0: float = 1.0
    oh_prefactor: float = 1059.0 / 2.0
    hh_r0: float = 1.633
    hh_prefactor: float = 684.0 / 2.0
    lj_prefactor: float = 4.0 * 0.1554
    lj_sigma: float = 3.166
    coulomb_prefactor: float = 332.0637
    bound_prefactor: float = 1.6 * 332.0637
    alpha: float = 3.45
    fourier_cutoff: int = 6
    position_cutoff: int = 2
    lifting: str = "inside_first"
    charge_oxygen: float = -0.82
    charge_hydrogen: float = 0.41
    mode: str = "mixed"

    @classmethod
    def from_spec(cls, spec: dict) -> "WaterModel":
        """The model of a specification with these field names (``molecules_per_side`` counts as
        ``molecules_per_side``^3 molecules); other keys are ignored."""
        values = {key: spec[key] for key in cls.__dataclass_fields__ if key in spec}
        if "molecules" not in values and "molecules_per_side" in spec:
            values["molecules"] = int(spec["molecules_per_side"]) ** 3
        return cls(**values)

    def charges(self) -> np.ndarray:
        return np.tile(np.array([self.charge_hydrogen, self.charge_oxygen, self.charge_hydrogen]), self.molecules)

    def desc(self, seed: int) -> "_lib.WaterDesc":
        values = asdict(self)
        values.pop("charge_oxygen")
        values.pop("charge_hydrogen")
        values["lifting"] = LIFTING[self.lifting]
        values["mode"] = MODES[self.mode]
        return _lib.WaterDesc(seed=int(seed), **values)


class WaterBatch:
    """Independent water chains: positions [chains][3 molecules][3], the same charges for every chain; chain c draws
    its random numbers with the key of (seed, first_chain + c)."""

    def __init__(self, model: WaterModel, positions, seed: int = 0, first_chain: int = 0, charges=None,
                 warps_per_block: int = 3, cells: Optional[WaterCells] = None, roots=None):
        import torch
        from .chains import check_charges, check_positions
        self._torch = torch
        if isinstance(positions, torch.Tensor):
            inside = torch.isfinite(positions).all() and bool(((positions >= 0) & (positions < model.system_length))
                                                              .all())
            if not inside:
                raise ValueError("water positions must be finite and lie in [0, %r)" % float(model.system_length))
        else:
            check_positions(positions, model.system_length, "water positions")
        if charges is not None:
            check_charges(charges, "water charges")
        self.lib = _lib.load()
        self.device = torch.device("cuda", torch.cuda.current_device())
        self.model = model
        self.seed = int(seed)
        self.first_chain = int(first_chain)
        self.warps_per_block = int(warps_per_block)
        if isinstance(positions, torch.Tensor) and positions.is_cuda:
            self.positions_dev = positions.to(torch.float64).contiguous().reshape(-1, 3 * model.molecules, 3)
        else:
            host = np.ascontiguousarray(np.asarray(positions, dtype=np.float64)).reshape(-1, 3 * model.molecules, 3)
            self.positions_dev = torch.from_numpy(host).to(self.device)
        self.chains = self.positions_dev.shape[0]
        charges = model.charges() if charges is None else np.asarray(charges, dtype=np.float64)
        self.charges_dev = torch.from_numpy(np.ascontiguousarray(charges)).to(self.device)
        self.state_dev = torch.zeros(max(self.chains, 1) * STATE_DTYPE.itemsize, dtype=torch.uint8,
                                     device=self.device)
        handle = ctypes.c_void_p()
        desc = model.desc(self.seed)
        _lib.check(self.lib.jfgpu_water_create(ctypes.byref(desc), ctypes.byref(handle)), "jfgpu_water_create")
        self._handle = handle
        _lib.check(self.lib.jfgpu_water_init(self._handle, self.state_dev.data_ptr(), self.chains, self.first_chain,
                                             self._stream()), "jfgpu_water_init")
        self.cells = cells
        if cells is not None:
            self._init_cells(cells, roots)

    def _init_cells(self, cells: WaterCells, roots) -> None:
        """Attach the molecular cells: the tables on the model, the roots (default: the barycentres of the
        positions), the occupancy and a fresh cell state of every chain."""
        torch = self._torch
        from . import systems
        upper = np.ascontiguousarray(cells.bounds_upper, dtype=np.float64).reshape(cells.cells, 3)
        lower = np.ascontiguousarray(cells.bounds_lower, dtype=np.float64).reshape(cells.cells, 3)
        far = {"cell_veto": _lib.FAR_CELL_VETO, "cell_bounding": _lib.FAR_CELL_BOUNDING}[cells.far]
        _lib.check(self.lib.jfgpu_water_set_cells(self._handle, int(cells.cells_per_side), int(cells.neighbor_layers),
                                                  upper.ctypes.data, lower.ctypes.data, int(bool(cells.keep_pairs)),
                                                  far, float(cells.dipole_charge)), "jfgpu_water_set_cells")
        M = self.model.molecules
        if roots is None:
            host = self.positions_dev.cpu().numpy()
            roots = np.stack([systems.water_roots(host[c], self.model.system_length) for c in range(self.chains)])
        roots = np.ascontiguousarray(np.asarray(roots, dtype=np.float64)).reshape(self.chains, M, 3)
        self.roots_dev = torch.from_numpy(roots).to(self.device)
        self.occupancy_dev = torch.full((self.chains, cells.cells), -1, dtype=torch.int32, device=self.device)
        self.surplus_dev = torch.full((self.chains, M), -1, dtype=torch.int32, device=self.device)
        self.cell_state_dev = torch.zeros(max(self.chains, 1) * CELL_STATE_DTYPE.itemsize, dtype=torch.uint8,
                                          device=self.device)
        buffers = self._cell_buffers(None)
        _lib.check(self.lib.jfgpu_water_cells_init(self._handle, ctypes.byref(buffers), self.chains, self._stream()),
                   "jfgpu_water_cells_init")
        if np.any(self.cell_states()["reserved"]):
            raise ValueError("a root unit lies outside the cell system")

    def _cell_buffers(self, root_log) -> "_lib.WaterCellBuffers":
        return _lib.WaterCellBuffers(self.roots_dev.data_ptr(), self.occupancy_dev.data_ptr(),
                                     self.surplus_dev.data_ptr(), self.cell_state_dev.data_ptr(),
                                     root_log.data_ptr() if root_log is not None else None)

    def _stream(self):
        return self._torch.cuda.current_stream(self.device).cuda_stream

    def run(self, events: int, record: bool = False, stop_time: Optional[float] = None, record_roots: bool = False):
        """Advance every chain by up to ``events`` events, stopping at ``stop_time`` (the active unit time-sliced to
        it, ``stopped`` set); with ``record`` returns the event log [chains][events] (zero rows after a stop), with
        ``record_roots`` (molecular cells) also the root of the moved unit's molecule after every event
        [chains][events][3]."""
        torch = self._torch
        log = None
        if record:
            log = torch.zeros(max(self.chains * events, 1) * EVENT_DTYPE.itemsize, dtype=torch.uint8,
                              device=self.device)
        stop_q, stop_r = (math.inf, math.inf) if stop_time is None else divmod(float(stop_time), 1.0)
        if self.cells is None:
            if record_roots:
                raise ValueError("root positions exist with molecular cells only")
            _lib.check(self.lib.jfgpu_water_run(self._handle, self.positions_dev.data_ptr(),
                                                self.charges_dev.data_ptr(), self.state_dev.data_ptr(), self.chains,
                                                self.first_chain, int(events), stop_q, stop_r,
                                                log.data_ptr() if record else None, self.warps_per_block,
                                                self._stream()), "jfgpu_water_run")
            root_log = None
        else:
            root_log = (torch.zeros((max(self.chains * events, 1), 3), dtype=torch.float64, device=self.device)
                        if record_roots else None)
            buffers = self._cell_buffers(root_log)
            _lib.check(self.lib.jfgpu_water_cells_run(self._handle, self.positions_dev.data_ptr(),
                                                      self.charges_dev.data_ptr(), self.state_dev.data_ptr(),
                                                      ctypes.byref(buffers), self.chains, self.first_chain,
                                                      int(events), stop_q, stop_r,
                                                      log.data_ptr() if record else None, self.warps_per_block,
                                                      self._stream()), "jfgpu_water_cells_run")
        result = None
        if record:
            host = log.cpu().numpy()[:self.chains * events * EVENT_DTYPE.itemsize]
            result = host.view(EVENT_DTYPE).reshape(self.chains, events)
        if record_roots:
            roots = root_log.cpu().numpy()[:self.chains * events].reshape(self.chains, events, 3)
            return result, roots
        return result

    def checkpoint(self, path: str) -> None:
        """Write the batch (model, seed, first chain, charges, positions and chain states; with molecular cells also
        the cell tables, roots, occupancy and cell states) to `path` (numpy .npz); ``WaterBatch.restore(path)``
        continues it exactly where it stopped (the random numbers are keyed by chain and event)."""
        self._torch.cuda.synchronize(self.device)
        extra = {}
        if self.cells is not None:
            extra = dict(cells=json.dumps([self.cells.cells_per_side, self.cells.neighbor_layers,
                                           bool(self.cells.keep_pairs), self.cells.far, self.cells.dipole_charge]),
                         bounds_upper=self.cells.bounds_upper, bounds_lower=self.cells.bounds_lower,
                         roots=self.roots_dev.cpu().numpy(), occupancy=self.occupancy_dev.cpu().numpy(),
                         surplus=self.surplus_dev.cpu().numpy(), cell_state=self.cell_state_dev.cpu().numpy())
        np.savez(path, model=json.dumps(asdict(self.model)), seed=self.seed, first_chain=self.first_chain,
                 warps_per_block=self.warps_per_block, charges=self.charges_dev.cpu().numpy(),
                 positions=self.positions_dev.cpu().numpy(), state=self.state_dev.cpu().numpy(), **extra)

    @classmethod
    def restore(cls, path: str) -> "WaterBatch":
        data = np.load(path)
        cells = None
        if "cells" in data.files:
            m, layers, keep_pairs, far, dipole_charge = json.loads(str(data["cells"]))
            cells = WaterCells(int(m), int(layers), np.asarray(data["bounds_upper"]), np.asarray(data["bounds_lower"]),
                               bool(keep_pairs), far, float(dipole_charge))
        batch = cls(WaterModel(**json.loads(str(data["model"]))), np.asarray(data["positions"]), seed=int(data["seed"]),
                    first_chain=int(data["first_chain"]), charges=np.asarray(data["charges"]),
                    warps_per_block=int(data["warps_per_block"]), cells=cells,
                    roots=np.asarray(data["roots"]) if cells is not None else None)
        torch = batch._torch
        pairs = [(batch.state_dev, "state")]
        if cells is not None:
            pairs += [(batch.occupancy_dev, "occupancy"), (batch.surplus_dev, "surplus"),
                      (batch.cell_state_dev, "cell_state")]
        for target, name in pairs:
            source = torch.from_numpy(np.ascontiguousarray(data[name])).to(batch.device)
            if source.shape != target.shape:
                raise ValueError("checkpoint %s does not match the batch layout" % name)
            target.copy_(source)
        torch.cuda.synchronize(batch.device)
        return batch

    def positions(self) -> np.ndarray:
        return self.positions_dev.cpu().numpy()

    def states(self) -> np.ndarray:
        return self.state_dev.cpu().numpy()[:self.chains * STATE_DTYPE.itemsize].view(STATE_DTYPE)

    def cell_states(self) -> np.ndarray:
        return self.cell_state_dev.cpu().numpy()[:self.chains * CELL_STATE_DTYPE.itemsize].view(CELL_STATE_DTYPE)

    def roots(self) -> np.ndarray:
        return self.roots_dev.cpu().numpy()

    def check_status(self) -> None:
        states = self.states()
        bad = np.nonzero(states["status"])[0]
        if len(bad):
            chain = int(bad[0])
            raise RuntimeError("water chain %d stopped: %s" % (chain, _lib.STATUS_NAMES.get(
                int(states["status"][chain]), str(int(states["status"][chain])))))

    def close(self) -> None:
        handle = getattr(self, "_handle", None)
        if handle and handle.value:
            self.lib.jfgpu_water_destroy(handle)
        self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lattice_positions(model: WaterModel, chains: int, seed: int, rng_offset: int = 0) -> np.ndarray:
    """Seeded water lattices of ``model.molecules`` = k^3 molecules for ``chains`` chains, chain c from
    ``numpy.random.default_rng((seed, rng_offset + c))``: [chains][3 molecules][3]."""
    from . import systems
    side = int(round(model.molecules ** (1.0 / 3.0)))
    if side ** 3 != model.molecules:
        raise ValueError("a lattice start needs k^3 molecules")
    out = np.empty((chains, 3 * model.molecules, 3), dtype=np.float64)
    for c in range(chains):
        rng = np.random.default_rng((seed, rng_offset + c))
        out[c] = systems.water_lattice(side, model.system_length, model.oh_r0, model.hh_r0, rng,
                                       model.charge_oxygen, model.charge_hydrogen)[0]
    return out
