"""The oracle's merged-image Coulomb and inverse-power Coulomb bound against the reference's own C code, compiled from
its sources into ``oracle/_ref/`` by ``oracle/build_ref.py`` (skipped where the reference tree is absent).

Bar: bit for bit, on seeded separations across the box (the oracle restates the same C arithmetic), and on the
reference's default parameters as well as the water and dipole configurations' ones.
"""
import ctypes
import os

import numpy as np
import pytest

import oracle

REF = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref")
MIC_PATH = os.path.join(REF, "libref_merged_image_coulomb.so")
IPCB_PATH = os.path.join(REF, "libref_inverse_power_coulomb_bound.so")

pytestmark = pytest.mark.skipif(not (os.path.exists(MIC_PATH) and os.path.exists(IPCB_PATH)),
                                reason="the reference's C code is not built (oracle/build_ref.py)")

_D = ctypes.c_double


def _mic():
    lib = ctypes.CDLL(MIC_PATH)
    lib.construct_merged_image_coulomb_potential.restype = ctypes.c_void_p
    lib.construct_merged_image_coulomb_potential.argtypes = [ctypes.c_int, ctypes.c_int, _D, _D]
    lib.destroy_merged_image_coulomb_potential.argtypes = [ctypes.c_void_p]
    lib.derivative.restype = _D
    lib.derivative.argtypes = [ctypes.c_void_p, _D, _D, _D]
    return lib


def _ipcb():
    lib = ctypes.CDLL(IPCB_PATH)
    lib.derivative.restype = _D
    lib.derivative.argtypes = [_D, _D, _D, _D]
    lib.displacement.restype = _D
    lib.displacement.argtypes = [_D, _D, _D, _D, _D, _D]
    return lib


@pytest.mark.parametrize("alpha, fourier_cutoff, position_cutoff, length",
                         [(3.45, 6, 2, 1.0), (3.45, 6, 2, 12.42), (3.45, 6, 2, 10.0), (5.0, 4, 1, 2.0)])
def test_merged_image_derivative_equals_the_reference_c(alpha, fourier_cutoff, position_cutoff, length):
    lib = _mic()
    potential = lib.construct_merged_image_coulomb_potential(fourier_cutoff, position_cutoff, alpha, length)
    assert potential
    try:
        rng = np.random.default_rng(int(100 * alpha) + fourier_cutoff + int(length))
        separations = rng.uniform(-0.5 * length, 0.5 * length, (400, 3))
        separations[:20] *= 1e-3  # close pairs
        for sx, sy, sz in separations:
            want = lib.derivative(potential, sx, sy, sz)
            got = oracle.lib().jfo_mic_x_derivative(alpha, fourier_cutoff, position_cutoff, length, sx, sy, sz)
            assert got == want, (sx, sy, sz)
    finally:
        lib.destroy_merged_image_coulomb_potential(potential)


@pytest.mark.parametrize("length", [1.0, 12.42])
def test_inverse_power_coulomb_bound_equals_the_reference_c(length):
    lib = _ipcb()
    rng = np.random.default_rng(int(length * 100))
    for _ in range(600):
        sx, sy, sz = rng.uniform(-0.5 * length, 0.5 * length, 3)
        prefactor = float(rng.choice([-1.0, 1.0]) * rng.uniform(0.1, 600.0))
        du = float(rng.exponential(1.0) * rng.choice([0.01, 1.0, 100.0]))
        want_d = lib.derivative(prefactor, sx, sy, sz)
        want_t = lib.displacement(prefactor, sx, sy, sz, du, length)
        got_d = oracle.ipcb_derivative(prefactor, [1.0, 0.0, 0.0], [sx, sy, sz], 1.0, 1.0)
        got_t = oracle.ipcb_displacement(prefactor, length, [1.0, 0.0, 0.0], [sx, sy, sz], 1.0, 1.0, du)
        assert got_d == want_d, (prefactor, sx, sy, sz)
        assert got_t == want_t, (prefactor, sx, sy, sz, du)
