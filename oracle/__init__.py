"""CPU oracle of the ECMC event-time path: ctypes front end of ``oracle/jf_oracle.c``.

TEST INFRASTRUCTURE ONLY.  This package is the CPU oracle the GPU product is tested against.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import it; the product package
``jellyfysh_gb300`` never does.

The C library restates JeLLyFysh's arithmetic with CPython 3.12 float semantics; see the header of
``jf_oracle.c`` for the file-by-file map onto the reference.
"""
import ctypes
import math
from typing import Optional, Sequence

import numpy as np

from .build_oracle import build as _build

EV_PAIR, EV_BOUNDED, EV_HARDCORE, EV_CELL_BOUNDING, EV_CELL_VETO, EV_BOUNDARY, EV_END_OF_CHAIN, EV_STOP = range(8)
EV_BOND, EV_COMPOSITE = 8, 9
POT_HARD_SPHERE, POT_LENNARD_JONES, POT_COULOMB = range(3)
FAR_NONE, FAR_CELL_VETO, FAR_CELL_BOUNDING = range(3)
RNG_PAIR, RNG_THIN, RNG_VETO_TIME, RNG_VETO_CHOICE, RNG_VETO_UNIFORM, RNG_NEW_ACTIVE, RNG_COMPOSITE, RNG_LIFT = range(8)
RNG_CELL_BOUND = 8  # potential change of a molecular cell-bounding factor, by target molecule

STATUS_NAMES = {0: "ok", 1: "ValueError", 2: "AssertionError", 3: "ZeroDivisionError", 4: "complex result",
                5: "bad configuration", 6: "allocation failure", 7: "cell index out of range",
                9: "LiftingSchemeError", 10: "IndexError"}
LIFTING_SCHEMES = {"inside_first": 0, "outside_first": 1, "ratio": 2}


class OracleError(RuntimeError):
    pass


class JfoSystem(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("system_length", ctypes.c_double), ("cells_per_side", ctypes.c_int),
                ("neighbor_layers", ctypes.c_int), ("max_occupants", ctypes.c_int), ("beta", ctypes.c_double),
                ("chain_time", ctypes.c_double), ("speed", ctypes.c_double), ("initial_direction", ctypes.c_int),
                ("initial_active", ctypes.c_int), ("potential", ctypes.c_int), ("hs_radius", ctypes.c_double),
                ("lj_prefactor", ctypes.c_double), ("lj_sigma", ctypes.c_double),
                ("coulomb_prefactor", ctypes.c_double), ("bound_prefactor", ctypes.c_double),
                ("ewald_alpha", ctypes.c_double), ("fourier_cutoff", ctypes.c_int),
                ("position_cutoff", ctypes.c_int), ("far", ctypes.c_int), ("estimator_points", ctypes.c_int),
                ("estimator_prefactor", ctypes.c_double), ("rng_key", ctypes.c_uint64)]


class JfoWaterSystem(ctypes.Structure):
    _fields_ = [("molecules", ctypes.c_int), ("system_length", ctypes.c_double), ("beta", ctypes.c_double),
                ("chain_time", ctypes.c_double), ("speed", ctypes.c_double), ("initial_direction", ctypes.c_int),
                ("initial_active", ctypes.c_int), ("oh_r0", ctypes.c_double), ("oh_prefactor", ctypes.c_double),
                ("hh_r0", ctypes.c_double), ("hh_prefactor", ctypes.c_double), ("lj_prefactor", ctypes.c_double),
                ("lj_sigma", ctypes.c_double), ("coulomb_prefactor", ctypes.c_double),
                ("bound_prefactor", ctypes.c_double), ("ewald_alpha", ctypes.c_double),
                ("fourier_cutoff", ctypes.c_int), ("position_cutoff", ctypes.c_int), ("lifting", ctypes.c_int),
                ("rng_key", ctypes.c_uint64)]


EVENT_DTYPE = np.dtype([("kind", np.int32), ("moved", np.int32), ("target", np.int32), ("new_active", np.int32),
                        ("new_direction", np.int32), ("accepted", np.int32), ("time_q", np.float64),
                        ("time_r", np.float64), ("x", np.float64), ("y", np.float64), ("z", np.float64)])

_LIB = None
_D = ctypes.c_double
_PD = ctypes.POINTER(ctypes.c_double)


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        handle = ctypes.CDLL(_build())
        handle.jfo_py_mod.restype = _D
        handle.jfo_py_mod.argtypes = [_D, _D]
        handle.jfo_py_divmod.argtypes = [_D, _D, _PD, _PD]
        handle.jfo_py_sum.restype = _D
        handle.jfo_py_sum.argtypes = [_PD, ctypes.c_int]
        handle.jfo_time_add.argtypes = [_D, _D, _D, _PD, _PD]
        handle.jfo_time_sub.restype = _D
        handle.jfo_time_sub.argtypes = [_D, _D, _D, _D]
        handle.jfo_chain_key.restype = ctypes.c_uint64
        handle.jfo_chain_key.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        handle.jfo_draw.restype = ctypes.c_uint64
        handle.jfo_draw.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32]
        handle.jfo_uniform.restype = _D
        handle.jfo_uniform.argtypes = [ctypes.c_uint64]
        handle.jfo_log.restype = _D
        handle.jfo_log.argtypes = [_D]
        handle.jfo_expovariate.restype = _D
        handle.jfo_expovariate.argtypes = [ctypes.c_uint64, _D]
        handle.jfo_randbelow.restype = ctypes.c_uint32
        handle.jfo_randbelow.argtypes = [ctypes.c_uint64, ctypes.c_uint32]
        handle.jfo_hs_displacement.argtypes = [_D, _PD, _PD, _PD]
        _I = ctypes.c_int
        handle.jfo_composite_event_time.argtypes = [_I, _D, _I, _I, _D, _D, _D, _PD, _PD, _D, _PD, _PD, _PD, _PD]
        handle.jfo_composite_out_state.argtypes = [_I, _I, _I, _D, _I, _I, _D, _D, _D, _PD, _PD, _PD, _I, _PD, _PD,
                                                   _I, _PD, ctypes.POINTER(ctypes.c_int), _PD, _PD]
        handle.jfo_composite_bounded_out_state.argtypes = [_I, _I, _I, _D, _I, _I, _D, _D, _PD, _PD, _PD, _I, _PD,
                                                           _PD, _I, _D, _PD, ctypes.POINTER(ctypes.c_int), _PD]
        handle.jfo_composite_cell_bound_time.argtypes = [_PD, _PD, _PD, _D, _PD, _I, _D, _D, _PD, _PD]
        handle.jfo_composite_cell_veto_time.argtypes = [_PD, _PD, _PD, _PD, _PD, _D, _D, _PD, _PD]
        _PI = ctypes.POINTER(ctypes.c_int)
        handle.jfo_walker_table.argtypes = [_PI, _PD, _I, _PI, _PD, _PI, _PD, _PD]
        handle.jfo_walker_pick.argtypes = [_PI, _PD, _PI, _I, _I, _D]
        handle.jfo_lifting.argtypes = [ctypes.c_int, ctypes.c_int, _PD, ctypes.POINTER(ctypes.c_int32), ctypes.c_int,
                                       _D, ctypes.POINTER(ctypes.c_int64), _PD]
        handle.jfo_ip_displacement.argtypes = [_D, _D, _PD, _PD, _D, _D, _D, _PD]
        handle.jfo_ip_derivative.argtypes = [_D, _D, _PD, _PD, _D, _D, _PD]
        handle.jfo_lj_displacement.argtypes = [_D, _D, _PD, _PD, _D, _PD]
        handle.jfo_lj_derivative.argtypes = [_D, _D, _PD, _PD, _PD]
        handle.jfo_dep_displacement.argtypes = [_D, ctypes.c_int, _D, _PD, _PD, _D, _PD]
        handle.jfo_dep_derivative.argtypes = [_D, ctypes.c_int, _D, _PD, _PD, _PD]
        handle.jfo_ipcb_displacement.argtypes = [_D, _D, _PD, _PD, _D, _D, _D, _PD]
        handle.jfo_ipcb_derivative.argtypes = [_D, _PD, _PD, _D, _D, _PD]
        handle.jfo_mic_x_derivative.restype = _D
        handle.jfo_mic_x_derivative.argtypes = [_D, ctypes.c_int, ctypes.c_int, _D, _D, _D, _D]
        handle.jfo_mic_derivative.argtypes = [_D, ctypes.c_int, ctypes.c_int, _D, _D, _PD, _PD, _D, _D, _PD]
        handle.jfo_cell_bounds.argtypes = [_D, ctypes.c_int, _PD, _PD]
        handle.jfo_water_create.restype = ctypes.c_void_p
        handle.jfo_water_create.argtypes = [ctypes.POINTER(JfoWaterSystem), _PD, _PD, ctypes.POINTER(ctypes.c_int)]
        handle.jfo_water_destroy.argtypes = [ctypes.c_void_p]
        handle.jfo_water_run.restype = ctypes.c_int64
        handle.jfo_water_run.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        handle.jfo_water_positions.argtypes = [ctypes.c_void_p, _PD]
        handle.jfo_water_run_roots.restype = ctypes.c_int64
        handle.jfo_water_run_roots.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.POINTER(ctypes.c_int)]
        handle.jfo_water_cells_create.restype = ctypes.c_void_p
        handle.jfo_water_cells_create.argtypes = [ctypes.POINTER(JfoWaterSystem), ctypes.c_int, ctypes.c_int, _PD,
                                                  _PD, _PD, _PD, _PD, ctypes.c_int, ctypes.c_int, _D,
                                                  ctypes.POINTER(ctypes.c_int)]
        handle.jfo_water_roots.argtypes = [ctypes.c_void_p, _PD]
        handle.jfo_chain_create.restype = ctypes.c_void_p
        handle.jfo_chain_create.argtypes = [ctypes.POINTER(JfoSystem), _PD, _PD, ctypes.POINTER(ctypes.c_int)]
        handle.jfo_chain_destroy.argtypes = [ctypes.c_void_p]
        handle.jfo_chain_run.restype = ctypes.c_int64
        handle.jfo_chain_run.argtypes = [ctypes.c_void_p, ctypes.c_int64, _D, _D, ctypes.c_void_p,
                                         ctypes.POINTER(ctypes.c_int)]
        handle.jfo_chain_positions.argtypes = [ctypes.c_void_p, _PD]
        handle.jfo_chain_state.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                           ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), _PD, _PD]
        handle.jfo_chain_occupancy.restype = ctypes.c_int
        handle.jfo_chain_occupancy.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]
        handle.jfo_chain_liftings.argtypes = [ctypes.c_void_p, _PD, ctypes.POINTER(ctypes.c_int64)]
        handle.jfo_chain_bounds.restype = ctypes.c_int
        handle.jfo_chain_bounds.argtypes = [ctypes.c_void_p, _PD, ctypes.c_int]
        handle.jfo_chain_walker.restype = ctypes.c_int
        handle.jfo_chain_walker.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_int32), _PD, ctypes.c_int, _PD]
        _LIB = handle
    return _LIB


def _vec(values: Sequence[float]):
    return (ctypes.c_double * 3)(*[float(v) for v in values])


def _call(fn, *args) -> float:
    out = ctypes.c_double()
    status = fn(*args, ctypes.byref(out))
    if status != 0:
        raise OracleError(STATUS_NAMES.get(status, str(status)))
    return out.value


# ---- primitives ---------------------------------------------------------------------------------
def py_mod(x: float, y: float) -> float:
    return lib().jfo_py_mod(x, y)


def py_divmod(x: float, y: float):
    q, r = ctypes.c_double(), ctypes.c_double()
    lib().jfo_py_divmod(x, y, ctypes.byref(q), ctypes.byref(r))
    return q.value, r.value


def py_sum(values: Sequence[float]) -> float:
    array = (ctypes.c_double * len(values))(*values)
    return lib().jfo_py_sum(array, len(values))


def time_add(q: float, r: float, dt: float):
    oq, orr = ctypes.c_double(), ctypes.c_double()
    lib().jfo_time_add(q, r, dt, ctypes.byref(oq), ctypes.byref(orr))
    return oq.value, orr.value


def chain_key(seed: int, chain: int) -> int:
    return lib().jfo_chain_key(seed, chain)


def draw(key: int, event: int, kind: int, target: int) -> int:
    return lib().jfo_draw(key, event, kind, target)


def uniform(bits: int) -> float:
    return lib().jfo_uniform(bits)


def log(x: float) -> float:
    return lib().jfo_log(x)


def expovariate(bits: int, beta: float) -> float:
    return lib().jfo_expovariate(bits, beta)


def randbelow(bits: int, n: int) -> int:
    return lib().jfo_randbelow(bits, n)


# ---- lifting schemes ----
def lifting(scheme: str, rates: Sequence[float], active: Sequence[bool], draw: float, unit_draw: bool = False):
    """(status, table index of the new active unit, b of the deciding random.uniform(0.0, b)) of one table."""
    count = len(rates)
    r = (ctypes.c_double * max(count, 1))(*[float(x) for x in rates])
    a = (ctypes.c_int32 * max(count, 1))(*[1 if x else 0 for x in active])
    selected = ctypes.c_int64(-1)
    bound = ctypes.c_double(0.0)
    status = lib().jfo_lifting(LIFTING_SCHEMES[scheme], 1 if unit_draw else 0, r, a, count, float(draw),
                               ctypes.byref(selected), ctypes.byref(bound))
    return status, selected.value, bound.value


# ---- composite objects ----
def _doubles(values):
    flat = [float(x) for x in np.asarray(values, dtype=np.float64).reshape(-1)]
    return (ctypes.c_double * max(len(flat), 1))(*flat)


def composite_event_time(model: dict, velocity, active_position, active_charge, target_positions, target_charges,
                         potential_changes):
    """(status, displacement) of send_event_time of two composite objects; model holds units, alpha,
    fourier_cutoff, position_cutoff, coulomb_prefactor, bound_prefactor, system_length."""
    out = ctypes.c_double(0.0)
    status = lib().jfo_composite_event_time(
        model["units"], model["alpha"], model["fourier_cutoff"], model["position_cutoff"],
        model["coulomb_prefactor"], model["bound_prefactor"], model["system_length"], _doubles(velocity),
        _doubles(active_position), float(active_charge), _doubles(target_positions), _doubles(target_charges),
        _doubles(potential_changes), ctypes.byref(out))
    return status, out.value


def composite_out_state(model: dict, scheme: str, velocity, local_positions, local_charges, active_index,
                        target_positions, target_charges, local_first, draws, unit_draw: bool = False):
    """(status, new active, bounding rate, event rate) of send_out_state of two composite objects."""
    new_active = ctypes.c_int(-1)
    bounding = ctypes.c_double(0.0)
    rate = ctypes.c_double(0.0)
    status = lib().jfo_composite_out_state(
        model["units"], LIFTING_SCHEMES[scheme], 1 if unit_draw else 0, model["alpha"], model["fourier_cutoff"],
        model["position_cutoff"], model["coulomb_prefactor"], model["bound_prefactor"], model["system_length"],
        _doubles(velocity), _doubles(local_positions), _doubles(local_charges), int(active_index),
        _doubles(target_positions), _doubles(target_charges), 1 if local_first else 0, _doubles(draws),
        ctypes.byref(new_active), ctypes.byref(bounding), ctypes.byref(rate))
    return status, new_active.value, bounding.value, rate.value


def composite_bounded_out_state(model: dict, scheme: str, velocity, local_positions, local_charges, active_index,
                                target_positions, target_charges, local_first, bounding_rate, draws,
                                unit_draw: bool = False):
    """(status, new active, event rate) of send_out_state of the molecular cell-bounding or cell-veto handler: the
    thinning draws against the given bounding event rate."""
    new_active = ctypes.c_int(-1)
    rate = ctypes.c_double(0.0)
    status = lib().jfo_composite_bounded_out_state(
        model["units"], LIFTING_SCHEMES[scheme], 1 if unit_draw else 0, model["alpha"], model["fourier_cutoff"],
        model["position_cutoff"], model["coulomb_prefactor"], model["system_length"], _doubles(velocity),
        _doubles(local_positions), _doubles(local_charges), int(active_index), _doubles(target_positions),
        _doubles(target_charges), 1 if local_first else 0, float(bounding_rate), _doubles(draws),
        ctypes.byref(new_active), ctypes.byref(rate))
    return status, new_active.value, rate.value


def composite_cell_bound_time(upper, lower, velocity, active_charge, target_charges, dipole_charge,
                              potential_change):
    """(status, bounding event rate, time displacement) of the molecular cell-bounding handler's event time; upper
    and lower are the relative cell's bounds in the three directions."""
    rate = ctypes.c_double(0.0)
    time = ctypes.c_double(0.0)
    charges = [float(q) for q in target_charges]
    status = lib().jfo_composite_cell_bound_time(
        _doubles(upper), _doubles(lower), _doubles(velocity), float(active_charge), _doubles(charges), len(charges),
        float(dipole_charge), float(potential_change), ctypes.byref(rate), ctypes.byref(time))
    return status, rate.value, time.value


def composite_cell_veto_time(upper, lower, walker_upper, walker_lower, velocity, active_charge, potential_change):
    """(status, bounding event rate, time displacement) of the molecular cell veto's event time for a sampled
    relative cell (bounds upper / lower in the three directions; Walker totals per direction)."""
    rate = ctypes.c_double(0.0)
    time = ctypes.c_double(0.0)
    status = lib().jfo_composite_cell_veto_time(
        _doubles(upper), _doubles(lower), _doubles(walker_upper), _doubles(walker_lower), _doubles(velocity),
        float(active_charge), float(potential_change), ctypes.byref(rate), ctypes.byref(time))
    return status, rate.value, time.value


def walker_table(items, rates):
    """(status, first_item, first_rate, second_item, total rate, mean rate) of Walker's alias table."""
    n = len(items)
    size = max(n, 1)
    first_item = (ctypes.c_int * size)()
    second_item = (ctypes.c_int * size)()
    first_rate = (ctypes.c_double * size)()
    total, mean = ctypes.c_double(0.0), ctypes.c_double(0.0)
    status = lib().jfo_walker_table((ctypes.c_int * size)(*[int(i) for i in items]), _doubles(rates), n,
                                    first_item, first_rate, second_item, ctypes.byref(total), ctypes.byref(mean))
    return status, list(first_item)[:n], list(first_rate)[:n], list(second_item)[:n], total.value, mean.value


def walker_pick(first_item, first_rate, second_item, choice, uniform):
    """The item Walker.sample_cell returns for the table index of random.choice and the random.uniform value."""
    n = len(first_item)
    return lib().jfo_walker_pick((ctypes.c_int * n)(*first_item), _doubles(first_rate),
                                 (ctypes.c_int * n)(*second_item), n, int(choice), float(uniform))


# ---- potentials (reference argument order: velocity, separation, [charges], [potential_change]) ----
def hs_displacement(radius, velocity, separation) -> float:
    return _call(lib().jfo_hs_displacement, radius, _vec(velocity), _vec(separation))


def ip_displacement(power, prefactor, velocity, separation, charge_one, charge_two, potential_change) -> float:
    return _call(lib().jfo_ip_displacement, power, prefactor, _vec(velocity), _vec(separation), charge_one,
                 charge_two, potential_change)


def ip_derivative(power, prefactor, velocity, separation, charge_one, charge_two) -> float:
    return _call(lib().jfo_ip_derivative, power, prefactor, _vec(velocity), _vec(separation), charge_one,
                 charge_two)


def lj_displacement(prefactor, sigma, velocity, separation, potential_change) -> float:
    return _call(lib().jfo_lj_displacement, prefactor, sigma, _vec(velocity), _vec(separation), potential_change)


def lj_derivative(prefactor, sigma, velocity, separation) -> float:
    return _call(lib().jfo_lj_derivative, prefactor, sigma, _vec(velocity), _vec(separation))


def dep_displacement(r0, power, prefactor, velocity, separation, potential_change) -> float:
    return _call(lib().jfo_dep_displacement, r0, int(power), prefactor, _vec(velocity), _vec(separation),
                 potential_change)


def dep_derivative(r0, power, prefactor, velocity, separation) -> float:
    return _call(lib().jfo_dep_derivative, r0, int(power), prefactor, _vec(velocity), _vec(separation))


def ipcb_displacement(prefactor, system_length, velocity, separation, charge_one, charge_two,
                      potential_change) -> float:
    return _call(lib().jfo_ipcb_displacement, prefactor, system_length, _vec(velocity), _vec(separation),
                 charge_one, charge_two, potential_change)


def ipcb_derivative(prefactor, velocity, separation, charge_one, charge_two) -> float:
    return _call(lib().jfo_ipcb_derivative, prefactor, _vec(velocity), _vec(separation), charge_one, charge_two)


def mic_derivative(alpha, fourier_cutoff, position_cutoff, prefactor, system_length, velocity, separation,
                   charge_one, charge_two) -> float:
    return _call(lib().jfo_mic_derivative, alpha, fourier_cutoff, position_cutoff, prefactor, system_length,
                 _vec(velocity), _vec(separation), charge_one, charge_two)


def mic_x_derivative(alpha, fourier_cutoff, position_cutoff, system_length, sx, sy, sz) -> float:
    return lib().jfo_mic_x_derivative(alpha, fourier_cutoff, position_cutoff, system_length, sx, sy, sz)


def cell_bounds(system_length: float, cells_per_side: int):
    lo = (ctypes.c_double * cells_per_side)()
    hi = (ctypes.c_double * cells_per_side)()
    lib().jfo_cell_bounds(system_length, cells_per_side, lo, hi)
    return list(lo), list(hi)


# ---- chains -------------------------------------------------------------------------------------
SYSTEM_DEFAULTS = dict(neighbor_layers=1, max_occupants=1, beta=1.0, chain_time=1.0, speed=1.0,
                       initial_direction=0, initial_active=0, potential=POT_HARD_SPHERE, hs_radius=0.0,
                       lj_prefactor=1.0, lj_sigma=1.0, coulomb_prefactor=1.0, bound_prefactor=1.5837,
                       ewald_alpha=3.45, fourier_cutoff=6, position_cutoff=2, far=FAR_NONE, estimator_points=10,
                       estimator_prefactor=1.5, rng_key=0)


def make_system(**kwargs) -> JfoSystem:
    values = dict(SYSTEM_DEFAULTS)
    values.update(kwargs)
    return JfoSystem(**values)


class Chain:
    """One ECMC chain run by the oracle (single thread; ctypes releases the GIL during runs)."""

    def __init__(self, system: JfoSystem, positions: np.ndarray, charges: Optional[np.ndarray] = None):
        positions = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        assert positions.shape[0] == system.n
        self.system = system
        self._positions_in = positions
        charge_pointer = None
        if charges is not None:
            self._charges_in = np.ascontiguousarray(charges, dtype=np.float64)
            charge_pointer = self._charges_in.ctypes.data_as(_PD)
        status = ctypes.c_int()
        self._handle = lib().jfo_chain_create(ctypes.byref(system), positions.ctypes.data_as(_PD), charge_pointer,
                                              ctypes.byref(status))
        if not self._handle:
            raise OracleError("chain creation failed: " + STATUS_NAMES.get(status.value, str(status.value)))

    def __del__(self):
        handle = getattr(self, "_handle", None)
        if handle:
            lib().jfo_chain_destroy(handle)
            self._handle = None

    def run(self, max_events: int, stop_time: Optional[float] = None, record: bool = True):
        """Advance by at most ``max_events`` events; returns the event log (or the count)."""
        stop_q, stop_r = (math.inf, math.inf) if stop_time is None else divmod(stop_time, 1.0)
        log_array = np.zeros(max_events if record else 0, dtype=EVENT_DTYPE)
        status = ctypes.c_int()
        done = lib().jfo_chain_run(self._handle, max_events, stop_q, stop_r,
                                   log_array.ctypes.data if record else None, ctypes.byref(status))
        if status.value != 0:
            raise OracleError("chain run stopped after %d events: %s"
                              % (done, STATUS_NAMES.get(status.value, str(status.value))))
        return log_array[:done] if record else done

    def positions(self) -> np.ndarray:
        out = np.zeros((self.system.n, 3), dtype=np.float64)
        lib().jfo_chain_positions(self._handle, out.ctypes.data_as(_PD))
        return out

    def state(self):
        event, active, direction = ctypes.c_int64(), ctypes.c_int(), ctypes.c_int()
        q, r = ctypes.c_double(), ctypes.c_double()
        lib().jfo_chain_state(self._handle, ctypes.byref(event), ctypes.byref(active), ctypes.byref(direction),
                              ctypes.byref(q), ctypes.byref(r))
        return dict(events=event.value, active=active.value, direction=direction.value, time_q=q.value,
                    time_r=r.value)

    def liftings(self):
        """(sum of the lifting separations along the direction of motion, number of liftings)."""
        total = ctypes.c_double()
        count = ctypes.c_int64()
        lib().jfo_chain_liftings(self._handle, ctypes.byref(total), ctypes.byref(count))
        return total.value, count.value

    def occupancy(self):
        """owner[i]: cell of particle i among the occupants, -2 - cell for a surplus unit, -1 for the active unit."""
        owner = np.zeros(self.system.n, dtype=np.int32)
        cell = lib().jfo_chain_occupancy(self._handle, owner.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        return owner, cell

    def bounds(self) -> np.ndarray:
        need = -lib().jfo_chain_bounds(self._handle, None, 0)
        if need <= 0:
            return np.zeros((0,))
        out = np.zeros(need, dtype=np.float64)
        lib().jfo_chain_bounds(self._handle, out.ctypes.data_as(_PD), need)
        cells = need // 6
        return out.reshape(2, cells, 3)

    def walker(self, direction: int, which: int = 0):
        size = -lib().jfo_chain_walker(self._handle, direction, which, None, None, 0, None)
        cells = np.zeros((size, 2), dtype=np.int32)
        rates = np.zeros(size, dtype=np.float64)
        total = ctypes.c_double()
        lib().jfo_chain_walker(self._handle, direction, which, cells.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                               rates.ctypes.data_as(_PD), size, ctypes.byref(total))
        return cells, rates, total.value


# ---- flexible water -----------------------------------------------------------------------------
WATER_FIELDS = [name for name, _ in JfoWaterSystem._fields_]


def make_water_system(spec: dict, rng_key: int) -> JfoWaterSystem:
    """The oracle's water system from a specification with the keys of the water trajectories (molecules_per_side or
    molecules, system_length, beta, chain_time, speed, initial_direction, initial_active, oh_r0, oh_prefactor,
    hh_r0, hh_prefactor, lj_prefactor, lj_sigma, coulomb_prefactor, bound_prefactor, alpha, fourier_cutoff,
    position_cutoff, lifting)."""
    molecules = spec.get("molecules", spec.get("molecules_per_side", 0) ** 3)
    lifting = {"inside_first": 0, "outside_first": 1, "ratio": 2}[spec.get("lifting", "inside_first")]
    return JfoWaterSystem(molecules=molecules, system_length=float(spec["system_length"]), beta=float(spec["beta"]),
                          chain_time=float(spec["chain_time"]), speed=float(spec["speed"]),
                          initial_direction=int(spec["initial_direction"]), initial_active=int(spec["initial_active"]),
                          oh_r0=float(spec["oh_r0"]), oh_prefactor=float(spec["oh_prefactor"]),
                          hh_r0=float(spec["hh_r0"]), hh_prefactor=float(spec["hh_prefactor"]),
                          lj_prefactor=float(spec["lj_prefactor"]), lj_sigma=float(spec["lj_sigma"]),
                          coulomb_prefactor=float(spec["coulomb_prefactor"]),
                          bound_prefactor=float(spec["bound_prefactor"]), ewald_alpha=float(spec["alpha"]),
                          fourier_cutoff=int(spec["fourier_cutoff"]), position_cutoff=int(spec["position_cutoff"]),
                          lifting=lifting, rng_key=int(rng_key))


class Water:
    """One chain of flexible water molecules run by the oracle.  With ``cells`` (cells_per_side, neighbor_layers,
    roots [molecules][3], bounds_upper [cells][3], bounds_lower [cells][3][, keep_pairs[, far, dipole_charge]])
    the Coulomb interaction between molecules goes through the molecular cells of the root units: nearby and surplus
    factors, the far field ("cell_veto", the default, or "cell_bounding" with the estimator's dipole charge) with the
    given bound tables and the cell-boundary events of the active root unit (across which the bond and Lennard-Jones
    candidates persist unless keep_pairs is False)."""

    def __init__(self, system: JfoWaterSystem, positions: np.ndarray, charges: np.ndarray, cells=None):
        self.system = system
        self._positions_in = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        self._charges_in = np.ascontiguousarray(charges, dtype=np.float64)
        assert self._positions_in.shape[0] == 3 * system.molecules == len(self._charges_in)
        status = ctypes.c_int()
        self.has_cells = cells is not None
        if cells is None:
            self._handle = lib().jfo_water_create(ctypes.byref(system), self._positions_in.ctypes.data_as(_PD),
                                                  self._charges_in.ctypes.data_as(_PD), ctypes.byref(status))
        else:
            m, layers, roots, upper, lower = cells[:5]
            keep_pairs = bool(cells[5]) if len(cells) > 5 else True
            far = {"cell_veto": 1, "cell_bounding": 2}[cells[6] if len(cells) > 6 else "cell_veto"]
            dipole_charge = float(cells[7]) if len(cells) > 7 else 1.0
            self._cells_in = [np.ascontiguousarray(a, dtype=np.float64) for a in (roots, upper, lower)]
            assert self._cells_in[0].shape == (system.molecules, 3)
            assert self._cells_in[1].shape == self._cells_in[2].shape == (m ** 3, 3)
            self._handle = lib().jfo_water_cells_create(
                ctypes.byref(system), int(m), int(layers), self._positions_in.ctypes.data_as(_PD),
                self._charges_in.ctypes.data_as(_PD), *[a.ctypes.data_as(_PD) for a in self._cells_in],
                int(keep_pairs), far, dipole_charge, ctypes.byref(status))
        if not self._handle:
            raise OracleError("water creation failed: " + STATUS_NAMES.get(status.value, str(status.value)))

    def __del__(self):
        handle = getattr(self, "_handle", None)
        if handle:
            lib().jfo_water_destroy(handle)
            self._handle = None

    def run(self, max_events: int, record: bool = True, roots: bool = False):
        """Advance by ``max_events`` events; returns the event log (or the count without ``record``); with ``roots``
        also the root position of the moved unit's molecule after every event ([events][3], molecular cells)."""
        log_array = np.zeros(max_events if record else 0, dtype=EVENT_DTYPE)
        root_array = np.zeros((max_events if roots else 0, 3), dtype=np.float64)
        status = ctypes.c_int()
        done = lib().jfo_water_run_roots(self._handle, max_events, log_array.ctypes.data if record else None,
                                         root_array.ctypes.data if roots else None, ctypes.byref(status))
        if status.value != 0:
            raise OracleError("water run stopped after %d events: %s"
                              % (done, STATUS_NAMES.get(status.value, str(status.value))))
        result = log_array[:done] if record else done
        return (result, root_array[:done]) if roots else result

    def roots(self) -> np.ndarray:
        """Root positions [molecules][3] (molecular cells)."""
        out = np.zeros((self.system.molecules, 3), dtype=np.float64)
        lib().jfo_water_roots(self._handle, out.ctypes.data_as(_PD))
        return out

    def positions(self) -> np.ndarray:
        out = np.zeros((3 * self.system.molecules, 3), dtype=np.float64)
        lib().jfo_water_positions(self._handle, out.ctypes.data_as(_PD))
        return out
