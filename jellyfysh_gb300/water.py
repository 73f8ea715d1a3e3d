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
                 warps_per_block: int = 3):
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

    def _stream(self):
        return self._torch.cuda.current_stream(self.device).cuda_stream

    def run(self, events: int, record: bool = False, stop_time: Optional[float] = None):
        """Advance every chain by up to ``events`` events, stopping at ``stop_time`` (the active unit time-sliced to
        it, ``stopped`` set); with ``record`` returns the event log [chains][events] (zero rows after a stop)."""
        torch = self._torch
        log = None
        if record:
            log = torch.zeros(max(self.chains * events, 1) * EVENT_DTYPE.itemsize, dtype=torch.uint8,
                              device=self.device)
        stop_q, stop_r = (math.inf, math.inf) if stop_time is None else divmod(float(stop_time), 1.0)
        _lib.check(self.lib.jfgpu_water_run(self._handle, self.positions_dev.data_ptr(), self.charges_dev.data_ptr(),
                                            self.state_dev.data_ptr(), self.chains, self.first_chain, int(events),
                                            stop_q, stop_r, log.data_ptr() if record else None,
                                            self.warps_per_block, self._stream()), "jfgpu_water_run")
        if not record:
            return None
        host = log.cpu().numpy()[:self.chains * events * EVENT_DTYPE.itemsize]
        return host.view(EVENT_DTYPE).reshape(self.chains, events)

    def checkpoint(self, path: str) -> None:
        """Write the batch (model, seed, first chain, charges, positions and chain states) to `path` (numpy .npz);
        ``WaterBatch.restore(path)`` continues it exactly where it stopped (the random numbers are keyed by chain and
        event)."""
        self._torch.cuda.synchronize(self.device)
        np.savez(path, model=json.dumps(asdict(self.model)), seed=self.seed, first_chain=self.first_chain,
                 warps_per_block=self.warps_per_block, charges=self.charges_dev.cpu().numpy(),
                 positions=self.positions_dev.cpu().numpy(), state=self.state_dev.cpu().numpy())

    @classmethod
    def restore(cls, path: str) -> "WaterBatch":
        data = np.load(path)
        batch = cls(WaterModel(**json.loads(str(data["model"]))), np.asarray(data["positions"]), seed=int(data["seed"]),
                    first_chain=int(data["first_chain"]), charges=np.asarray(data["charges"]),
                    warps_per_block=int(data["warps_per_block"]))
        state = batch._torch.from_numpy(np.ascontiguousarray(data["state"])).to(batch.device)
        if state.shape != batch.state_dev.shape:
            raise ValueError("checkpoint state does not match the batch layout")
        batch.state_dev.copy_(state)
        batch._torch.cuda.synchronize(batch.device)
        return batch

    def positions(self) -> np.ndarray:
        return self.positions_dev.cpu().numpy()

    def states(self) -> np.ndarray:
        return self.state_dev.cpu().numpy()[:self.chains * STATE_DTYPE.itemsize].view(STATE_DTYPE)

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
