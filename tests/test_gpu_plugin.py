"""The drop-in classes of ``jellyfysh_gb300.plugin`` on the GPU, without the reference.

* Each GPU potential class, called one row at a time with the reference's method signature, reproduces every
  value of the reference's potential test suites (``golden/potential_known_answers.json``) to 1e-12 relative.
* A batch plan (what the drop-in mediator builds from a configuration) runs to its end-of-run time and equals the
  oracle run to the same time: hard spheres bit for bit, Lennard-Jones to 1e-12 of the box.
"""
import math

import numpy as np
import pytest

import oracle
from tests.potential_cases import load_cases, normalise
from tests.trajectory_cases import load_trajectory, oracle_system

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = 1e-12


def plugin_call(case):
    from jellyfysh_gb300.plugin.potential import (gpu_displaced_even_power_potential, gpu_hard_sphere_potential,
                                                  gpu_inverse_power_coulomb_bounding_potential,
                                                  gpu_inverse_power_potential, gpu_lennard_jones_potential,
                                                  gpu_merged_image_coulomb_potential)
    name, method = case["potential"], case["method"]
    v, s, du = case["velocity"], list(case["separation"]), case["potential_change"]
    c1, c2 = case["charges"]
    if name == "HardSpherePotential":
        return gpu_hard_sphere_potential.GpuHardSpherePotential(case["radius"]).displacement(v, s)
    if name == "InversePowerPotential":
        p = gpu_inverse_power_potential.GpuInversePowerPotential(case["power"], case["prefactor"])
        return p.displacement(v, s, c1, c2, potential_change=du) if method == "displacement" else \
            p.derivative(v, s, c1, c2)
    if name == "LennardJonesPotential":
        p = gpu_lennard_jones_potential.GpuLennardJonesPotential(case["prefactor"], case["sigma"])
        return p.displacement(v, s, potential_change=du) if method == "displacement" else p.derivative(v, s)
    if name == "DisplacedEvenPowerPotential":
        p = gpu_displaced_even_power_potential.GpuDisplacedEvenPowerPotential(case["r0"], case["power"],
                                                                              case["prefactor"])
        return p.displacement(v, s, potential_change=du) if method == "displacement" else p.derivative(v, s)
    if name == "InversePowerCoulombBoundingPotential":
        p = gpu_inverse_power_coulomb_bounding_potential.GpuInversePowerCoulombBoundingPotential(case["prefactor"])
        p._system_length = case["system_length"]  # the reference reads it from its hypercubic setting
        return p.displacement(v, s, c1, c2, potential_change=du) if method == "displacement" else \
            p.derivative(v, s, c1, c2)
    p = gpu_merged_image_coulomb_potential.GpuMergedImageCoulombPotential(
        case["alpha"], case["fourier_cutoff"], case["position_cutoff"], case["prefactor"])
    p._system_length = case["system_length"]
    return p.derivative(v, s, c1, c2)


def test_gpu_potential_classes_reproduce_the_reference_values():
    failures = []
    for raw in load_cases():
        case = normalise(raw)
        value = plugin_call(case)
        reference = case["reference"]
        same = (math.isinf(value) and math.isinf(reference) and (value > 0) == (reference > 0)) or \
            abs(value - reference) <= REL * max(abs(reference), 1e-300)
        if not same:
            failures.append((case["test"], value, reference))
    assert failures == []


def test_potential_classes_declare_the_reference_argument_counts():
    from jellyfysh_gb300.plugin.potential import (gpu_hard_sphere_potential, gpu_inverse_power_potential,
                                                  gpu_lennard_jones_potential)
    hs = gpu_hard_sphere_potential.GpuHardSpherePotential(0.5)
    assert (hs.number_separation_arguments, hs.number_charge_arguments, hs.potential_change_required) == \
        (1, 0, False)
    lj = gpu_lennard_jones_potential.GpuLennardJonesPotential()
    assert (lj.number_separation_arguments, lj.number_charge_arguments, lj.potential_change_required) == \
        (1, 0, True)
    ip = gpu_inverse_power_potential.GpuInversePowerPotential(1.0, 1.0)
    assert ip.number_charge_arguments == 2
    with pytest.raises(NotImplementedError):
        hs.derivative([1.0, 0.0, 0.0], [0.5, 0.0, 0.0])
    # the reference's exceptions come back from the device status codes (sqrt of a negative number)
    from jellyfysh_gb300 import potentials
    with pytest.raises(ValueError):
        potentials.raise_status(1)


@pytest.mark.parametrize("name", ["hard_spheres_n64", "lennard_jones_n64_cell_veto"])
def test_batch_plan_runs_to_the_end_of_run_time_like_the_oracle(name):
    from jellyfysh_gb300.chains import ChainSpec
    from jellyfysh_gb300.plugin.plan import BatchPlan, run_plan
    spec, initial, charges, events, final = load_trajectory(name)
    t_end = float(events["time_q"][299] + events["time_r"][299]) + 1e-9
    chain_spec = ChainSpec(n=spec["n"], system_length=spec["system_length"], cells_per_side=spec["cells_per_side"],
                           potential=spec["potential"], far=spec["far"], neighbor_layers=spec["neighbor_layers"],
                           beta=spec["beta"], chain_time=spec["chain_time"], hs_radius=spec.get("radius", 0.0),
                           estimator_points=spec.get("estimator_points", 10),
                           estimator_prefactor=spec.get("estimator_prefactor", 1.5), rng_key=spec["rng_key"])
    plan = BatchPlan(spec=chain_spec, positions=initial, charges=None, end_of_run_time=t_end, chains=2,
                     events_per_launch=64)
    batch = run_plan(plan)
    chain = oracle.Chain(oracle_system(spec), initial)
    chain.run(10 ** 6, stop_time=t_end, record=False)
    for c in range(2):  # both chains carry the fixture's key
        state = batch.state()[c]
        assert state["events"] == chain.state()["events"] == 300
        if spec["potential"] == "hard_sphere":
            assert np.array_equal(batch.positions(c), chain.positions())
        else:
            assert np.allclose(batch.positions(c), chain.positions(), rtol=0, atol=1e-12 * spec["system_length"])
    batch.close()
