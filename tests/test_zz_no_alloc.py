"""The allocation-free merged-image Coulomb derivative against the allocating entry point (GPU).

Some callers cannot allocate device memory: hosts that must not enter the CUDA allocator while they run (real-time
loops, a fixed memory budget), plug-ins that live inside another framework's memory pool.
``jfgpu_merged_image_coulomb_derivative_noalloc`` serves them with its Fourier table in a fixed device array, filled
on the device.
This test calls it through the C ABI twice in a row, with different Ewald parameters (so the second call must
rewrite the shared table), and compares each result with ``jfgpu_merged_image_coulomb_derivative`` at the
tolerance of the other potential tests (1e-12 relative).  It lives in a file of its own that pytest collects last.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = 1e-12


def _inputs(n, length, seed):
    rng = np.random.default_rng(seed)
    velocity = np.zeros((n, 3))
    velocity[np.arange(n), rng.integers(0, 3, n)] = rng.uniform(0.5, 2.0, n)
    separation = rng.uniform(-0.5 * length, 0.5 * length, (n, 3))
    charges = rng.choice([-1.0, 1.0], (n, 2))
    to = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")  # noqa: E731
    return to(velocity), to(separation), to(charges)


def _call(fn, alpha, fourier_cutoff, position_cutoff, prefactor, length, velocity, separation, charges):
    n = velocity.shape[0]
    out = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    status = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    code = fn(alpha, fourier_cutoff, position_cutoff, prefactor, length, velocity.data_ptr(), separation.data_ptr(),
              charges.data_ptr(), n, out.data_ptr(), status.data_ptr(), None)
    torch.cuda.synchronize()
    return code, out.cpu().numpy(), status.cpu().numpy()


def test_no_alloc_entry_point_matches_the_allocating_one_on_two_calls_in_a_row():
    from jellyfysh_gb300 import _lib
    lib = _lib.load()
    calls = [(3.45, 6, 2, 1.0, 1.0, 11), (5.0, 9, 2, 1.3, 2.0, 12)]
    for alpha, fc, pc, prefactor, length, seed in calls:
        velocity, separation, charges = _inputs(512, length, seed)
        code, expected, st_expected = _call(lib.jfgpu_merged_image_coulomb_derivative, alpha, fc, pc, prefactor,
                                            length, velocity, separation, charges)
        assert code == 0 and (st_expected == 0).all()
        code, got, st_got = _call(lib.jfgpu_merged_image_coulomb_derivative_noalloc, alpha, fc, pc, prefactor,
                                  length, velocity, separation, charges)
        assert code == 0 and (st_got == 0).all()
        scale = np.maximum(np.abs(expected), 1e-300)
        assert np.all(np.abs(got - expected) <= REL * scale), float(np.max(np.abs(got - expected) / scale))


def test_no_alloc_entry_point_rejects_cutoffs_beyond_its_table():
    from jellyfysh_gb300 import _lib
    lib = _lib.load()
    velocity, separation, charges = _inputs(4, 1.0, 13)
    code, _, _ = _call(lib.jfgpu_merged_image_coulomb_derivative_noalloc, 3.45, 16, 2, 1.0, 1.0, velocity,
                       separation, charges)
    assert code == 2  # JFGPU_ERROR_ARGUMENT
