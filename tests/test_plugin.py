"""The drop-in classes against the reference's own factory (CPU only; needs the reference's source tree).

Set JELLYFYSH_TREE to a JeLLyFysh source tree (with its cffi extensions built for the Coulomb systems) to run
these tests; without it they are skipped.  They check that a configuration file in the reference's vocabulary
selects the GPU classes by name:

* ``potential = gpu_lennard_jones_potential`` (and the other GPU potentials) builds the GPU class inside the
  reference's own event handler;
* ``lifting = gpu_inside_first_lifting`` (and the other schemes) builds the GPU lifting inside the reference's
  composite-object event handler;
* ``mediator = gpu_chain_batch_mediator`` builds the drop-in mediator from the same object graph, and its batch
  plan (atoms) or water plan (water molecules through factor-type-map taggers) is the system of the configuration (the chain parameters that the GPU trajectory tests run, the injected
  initial positions and charges).
"""
import configparser
import dataclasses
import importlib
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from tests.trajectory_cases import load_trajectory, trajectory_names

TREE = os.environ.get("JELLYFYSH_TREE")
pytestmark = pytest.mark.skipif(not TREE or not os.path.isdir(os.path.join(TREE or "", "jellyfysh")),
                                reason="JELLYFYSH_TREE does not name a JeLLyFysh source tree")


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference():
    if TREE not in sys.path:
        sys.path.insert(0, TREE)
    from jellyfysh.base import factory
    from jellyfysh.base.strings import to_camel_case
    from jellyfysh_gb300 import plugin
    plugin.install()
    return factory, to_camel_case


def _in_child(function, *args):
    """The reference keeps its setting in module globals (one per process): every build runs in its own
    interpreter, as the reference's own runs do.  Returns the child's JSON result."""
    code = "import json, sys; import tests.test_plugin as t; print(json.dumps(t.%s(*sys.argv[1:])))" % function
    done = subprocess.run([sys.executable, "-c", code, *args], cwd=ROOT, capture_output=True, text=True,
                          timeout=300)
    assert done.returncode == 0, done.stderr[-3000:]
    return json.loads(done.stdout.strip().splitlines()[-1])


def build_handler_with_gpu_potential():
    factory, camel = _reference()
    config = configparser.ConfigParser()
    config.read_string("""
[Run]
setting = hypercubic_setting
[HypercubicSetting]
system_length = 4.0
beta = 1.0
dimension = 3
[TwoLeafUnitEventHandler]
potential = gpu_lennard_jones_potential
[GpuLennardJonesPotential]
prefactor = 2.0
characteristic_length = 1.1
""")
    factory.build_from_config(config, "HypercubicSetting", "jellyfysh.setting")
    handler = factory.build_from_config(config, "TwoLeafUnitEventHandler", "jellyfysh.event_handler")
    potential = handler._potential
    modules = []
    for module in ("gpu_hard_sphere_potential", "gpu_inverse_power_potential", "gpu_displaced_even_power_potential",
                   "gpu_inverse_power_coulomb_bounding_potential", "gpu_merged_image_coulomb_potential"):
        modules.append(importlib.import_module("jellyfysh.potential." + module).__name__)
    return [type(potential).__name__, potential._prefactor, potential._characteristic_length, modules]


def translate_configuration(name):
    factory, camel = _reference()
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_reference_trajectories as trajectories
    spec, initial, charges, events, final = load_trajectory(name)
    text = trajectories.config_text(spec, spec["system_length"])
    text = text.replace("mediator = single_process_mediator", "mediator = gpu_chain_batch_mediator")
    text = text.replace("[SingleProcessMediator]", "[GpuChainBatchMediator]\nchains = 3\nmode = exact\nseed = 5")
    config = configparser.ConfigParser()
    config.read_string(text)
    # the reference's input handler places random units; inject the fixture's, as the trajectory recorder does
    from jellyfysh.base.particle import Particle
    from jellyfysh.input_output_handler.input_handler.random_node_creator import atom_random_node_creator
    queue = list(range(spec["n"]))

    def fill_root_node(self, node):
        i = queue.pop(0)
        charge = {} if charges is None else {"electric_charge": float(charges[i])}
        node.value = Particle([float(v) for v in initial[i]], charge)
    atom_random_node_creator.AtomRandomNodeCreator.fill_root_node = fill_root_node
    factory.build_from_config(config, camel(config.get("Run", "setting")), "jellyfysh.setting")
    mediator = factory.build_from_config(config, camel(config.get("Run", "mediator")), "jellyfysh.mediator")
    plan = mediator.plan
    return {"spec": dataclasses.asdict(plan.spec), "positions": plan.positions.tolist(),
            "charges": None if plan.charges is None else plan.charges.tolist(),
            "end_of_run_time": plan.end_of_run_time, "chains": plan.chains, "mode": plan.mode, "seed": plan.seed}


def build_composite_handler_with_gpu_lifting(scheme):
    factory, camel = _reference()
    config = configparser.ConfigParser()
    config.read_string("""
[Run]
setting = hypercubic_setting
[HypercubicSetting]
system_length = 10.0
beta = 1.679
dimension = 3
[TwoCompositeObjectSummedBoundingPotentialEventHandler]
potential = merged_image_coulomb_potential
bounding_potential = inverse_power_coulomb_bounding_potential
lifting = gpu_%s_lifting
charge = electric_charge
[MergedImageCoulombPotential]
prefactor = 332
[InversePowerCoulombBoundingPotential]
prefactor = 531.2
""" % scheme)
    factory.build_from_config(config, camel(config.get("Run", "setting")), "jellyfysh.setting")
    from jellyfysh import setting
    # two water molecules, as the reference's water node creator sets them: the handler wants composite objects
    setting.set_number_of_root_nodes(2)
    setting.set_number_of_nodes_per_root_node(3)
    setting.set_number_of_node_levels(2)
    handler = factory.build_from_config(config, "TwoCompositeObjectSummedBoundingPotentialEventHandler",
                                        "jellyfysh.event_handler")
    return [type(handler._lifting).__name__, type(handler._lifting).__module__]


@pytest.mark.parametrize("scheme", ["inside_first", "outside_first", "ratio"])
def test_gpu_lifting_is_built_inside_the_reference_composite_handler(scheme):
    name, module = _in_child("build_composite_handler_with_gpu_lifting", scheme)
    camel = "".join(part.capitalize() for part in scheme.split("_"))
    assert name == "Gpu%sLifting" % camel
    assert module == "jellyfysh.lifting.gpu_%s_lifting" % scheme


def test_gpu_potentials_are_built_inside_the_reference_event_handler():
    name, prefactor, sigma, modules = _in_child("build_handler_with_gpu_potential")
    assert (name, prefactor, sigma) == ("GpuLennardJonesPotential", 2.0, 1.1)
    assert len(modules) == 5


@pytest.mark.parametrize("name", trajectory_names())
def test_mediator_translates_the_reference_configuration(name):
    spec, initial, charges, events, final = load_trajectory(name)
    plan = _in_child("translate_configuration", name)
    assert (plan["chains"], plan["mode"], plan["seed"]) == (3, "exact", 5)
    s = plan["spec"]
    expected = dict(n=spec["n"], system_length=spec["system_length"], cells_per_side=spec["cells_per_side"],
                    neighbor_layers=spec["neighbor_layers"], beta=spec["beta"], chain_time=spec["chain_time"],
                    far=spec["far"], initial_active=0, initial_direction=0, speed=1.0, potential=spec["potential"],
                    max_occupants=1)
    for key, value in expected.items():
        assert s[key] == value, key
    if spec["potential"] in ("hard_sphere", "coulomb"):
        assert s["hs_radius"] == spec["radius"]
    if spec["far"] != "none":
        assert (s["estimator_points"], s["estimator_prefactor"]) == (spec["estimator_points"],
                                                                    spec["estimator_prefactor"])
    assert np.array_equal(np.array(plan["positions"]), initial)
    if charges is not None:
        assert np.array_equal(np.array(plan["charges"]), charges)
    assert plan["end_of_run_time"] == 1e9


def translate_water_configuration(name):
    """The reference's factory builds the drop-in mediator from the water configuration of the water trajectories
    (run in a child); returns the water plan."""
    factory, camel = _reference()
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import tempfile
    import make_water_trajectories as waters
    from tests.water_cases import load_water
    spec, initial, charges, events, final = load_water(name)
    scratch = tempfile.mkdtemp()
    factor_file = os.path.join(scratch, "factors.txt")
    with open(factor_file, "w") as handle:
        handle.write(waters.FACTORS)
    text = waters.config_text(spec, factor_file)
    text = text.replace("mediator = single_process_mediator", "mediator = gpu_chain_batch_mediator")
    text = text.replace("[SingleProcessMediator]", "[GpuChainBatchMediator]\nchains = 4\nmode = exact\nseed = 7")
    config = configparser.ConfigParser()
    config.read_string(text)
    from jellyfysh.base.node import Node
    from jellyfysh.base.particle import Particle
    from jellyfysh.input_output_handler.input_handler.random_node_creator import water_random_node_creator
    queue = list(range(len(initial) // 3))

    def fill_root_node(self, node):
        m = queue.pop(0)
        for t in range(3):
            node.add_child(Node(Particle([float(v) for v in initial[3 * m + t]],
                                         {"electric_charge": float(charges[3 * m + t])})))
        node.value = Particle(position=[float(v) for v in initial[3 * m + 1]])
    water_random_node_creator.WaterRandomNodeCreator.fill_root_node = fill_root_node
    factory.build_from_config(config, camel(config.get("Run", "setting")), "jellyfysh.setting")
    mediator = factory.build_from_config(config, camel(config.get("Run", "mediator")), "jellyfysh.mediator")
    plan = mediator.plan
    return {"type": type(plan).__name__, "model": dataclasses.asdict(plan.model), "positions": plan.positions.tolist(),
            "charges": plan.charges.tolist(), "end_of_run_time": plan.end_of_run_time, "chains": plan.chains,
            "mode": plan.mode, "seed": plan.seed}


@pytest.mark.parametrize("name", ["water_n8"])
def test_mediator_translates_the_reference_water_configuration(name):
    from tests.water_cases import load_water
    spec, initial, charges, events, final = load_water(name)
    plan = _in_child("translate_water_configuration", name)
    assert plan["type"] == "WaterPlan" and (plan["chains"], plan["mode"], plan["seed"]) == (4, "exact", 7)
    model = plan["model"]
    for key in ("system_length", "beta", "chain_time", "speed", "oh_r0", "oh_prefactor", "hh_r0", "hh_prefactor",
                "lj_prefactor", "lj_sigma", "coulomb_prefactor", "bound_prefactor", "alpha", "fourier_cutoff",
                "position_cutoff", "initial_direction", "initial_active", "lifting"):
        assert model[key] == spec[key], key
    assert model["molecules"] == spec["molecules_per_side"] ** 3 and model["mode"] == "exact"
    assert np.array_equal(np.array(plan["positions"]), initial)
    assert np.array_equal(np.array(plan["charges"]), charges)
    assert plan["end_of_run_time"] == 1e9


def translate_water_cell_configuration(name, boundary_trashes_pairs="0"):
    """The reference's factory builds the drop-in mediator from the water cell-veto configuration of a recorded
    trajectory (run in a child); with boundary_trashes_pairs the molecule cell boundary trashes the pair factors too.
    Returns the water plan."""
    factory, camel = _reference()
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import tempfile
    import make_water_cell_trajectories as cells
    from tests.water_cases import load_water_cells
    spec, data = load_water_cells(name)
    initial, charges, roots = data["initial"], data["charges"], data["initial_roots"]
    scratch = tempfile.mkdtemp()
    factor_file = os.path.join(scratch, "factors.txt")
    with open(factor_file, "w") as handle:
        handle.write(cells.FACTORS.replace("[0, 1, 2, 3, 4, 5], Coulomb\n", ""))
    text = cells.config_text(spec, factor_file)
    text = text.replace("mediator = single_process_mediator", "mediator = gpu_chain_batch_mediator")
    text = text.replace("[SingleProcessMediator]", "[GpuChainBatchMediator]\nchains = 3\nmode = mixed\nseed = 5")
    if boundary_trashes_pairs == "1":
        tags = cells.cell_tags(spec)
        every = ", ".join(cells.PAIR_TAGS + tags)
        text = text.replace("[MoleculeCellBoundary]\ntrash = %s" % ", ".join(tags),
                            "[MoleculeCellBoundary]\ntrash = %s" % every)
    config = configparser.ConfigParser()
    config.read_string(text)
    from jellyfysh.base.node import Node
    from jellyfysh.base.particle import Particle
    from jellyfysh.input_output_handler.input_handler.random_node_creator import water_random_node_creator
    queue = list(range(len(initial) // 3))

    def fill_root_node(self, node):
        m = queue.pop(0)
        for t in range(3):
            node.add_child(Node(Particle([float(v) for v in initial[3 * m + t]],
                                         {"electric_charge": float(charges[3 * m + t])})))
        node.value = Particle(position=[float(v) for v in roots[m]])
    water_random_node_creator.WaterRandomNodeCreator.fill_root_node = fill_root_node
    factory.build_from_config(config, camel(config.get("Run", "setting")), "jellyfysh.setting")
    mediator = factory.build_from_config(config, camel(config.get("Run", "mediator")), "jellyfysh.mediator")
    plan = mediator.plan
    return {"type": type(plan).__name__, "model": dataclasses.asdict(plan.model), "positions": plan.positions.tolist(),
            "roots": plan.roots.tolist(), "cell_veto": plan.cell_veto, "charges": plan.charges.tolist()}


@pytest.mark.parametrize("name", ["water_n8_cell_veto", "water_n64_cell_veto", "water_n8_cell_bounding"])
def test_mediator_translates_the_reference_water_cell_veto_configuration(name):
    """The reference's water cell-veto configuration (with this project's water model) becomes a water plan with
    molecular cells: the cell system, the dipole estimator's parameters, the root units, and the pair candidates kept
    across cell boundaries exactly when the boundary's tagger leaves them out of its trash list."""
    from tests.water_cases import load_water_cells
    spec, data = load_water_cells(name)
    plan = _in_child("translate_water_cell_configuration", name)
    assert plan["type"] == "WaterPlan"
    for key in ("system_length", "beta", "chain_time", "oh_r0", "hh_prefactor", "lj_sigma", "coulomb_prefactor",
                "bound_prefactor", "alpha", "fourier_cutoff", "position_cutoff", "initial_active", "lifting"):
        assert plan["model"][key] == spec[key], key
    cell_veto = plan["cell_veto"]
    assert (cell_veto["cells_per_side"], cell_veto["neighbor_layers"]) == (spec["cells_per_side"],
                                                                           spec["neighbor_layers"])
    assert (cell_veto["dipole_separation"], cell_veto["dipole_charge"], cell_veto["prefactor"],
            cell_veto["number_trials"], cell_veto["empirical_bound"]) == (
        spec["dipole_separation"], spec["dipole_charge"], spec["estimator_prefactor"], spec["number_trials"],
        spec["empirical_bound"])
    assert cell_veto["keep_pairs"] is True and cell_veto["far"] == spec.get("far", "cell_veto")
    assert np.array_equal(np.array(plan["roots"]), data["initial_roots"])
    assert np.array_equal(np.array(plan["positions"]), data["initial"])
    trashing = _in_child("translate_water_cell_configuration", name, "1")
    assert trashing["cell_veto"]["keep_pairs"] is False


def reference_separation_file(path):
    """The reference's SeparationOutputHandler writing one sample of a fixed configuration (run in a child)."""
    if TREE not in sys.path:
        sys.path.insert(0, TREE)
    import configparser as cp
    from jellyfysh.base import factory
    from jellyfysh.base.node import Node
    from jellyfysh.base.particle import Particle
    from jellyfysh.base.unit import Unit
    config = cp.ConfigParser()
    config.read_string("[Run]\nsetting = hypercubic_setting\n[HypercubicSetting]\nsystem_length = 4.308869380063767\n"
                       "beta = 1.0\ndimension = 3\n[SeparationOutputHandler]\nfilename = %s\n" % path)
    factory.build_from_config(config, "HypercubicSetting", "jellyfysh.setting")
    from jellyfysh import setting
    positions = np.random.default_rng(9).uniform(0.0, 4.308869380063767, size=(20, 3))
    setting.set_number_of_root_nodes(20)
    setting.set_number_of_nodes_per_root_node(1)
    setting.set_number_of_node_levels(1)
    handler = factory.build_from_config(config, "SeparationOutputHandler",
                                        "jellyfysh.input_output_handler.output_handler")
    nodes = [Node(Unit(identifier=(i,), position=[float(v) for v in positions[i]], charge=None))
             for i in range(20)]
    handler.write(nodes)
    handler.post_run()
    return positions.tolist()


def reference_oxygen_separation_file(path):
    """The reference's OxygenOxygenSeparationOutputHandler writing one sample of a water configuration (child)."""
    if TREE not in sys.path:
        sys.path.insert(0, TREE)
    import configparser as cp
    from jellyfysh.base import factory
    from jellyfysh.base.node import Node
    from jellyfysh.base.unit import Unit
    from jellyfysh_gb300 import systems
    config = cp.ConfigParser()
    config.read_string("[Run]\nsetting = hypercubic_setting\n[HypercubicSetting]\nsystem_length = 12.42\n"
                       "beta = 1.0\ndimension = 3\n[OxygenOxygenSeparationOutputHandler]\nfilename = %s\n" % path)
    factory.build_from_config(config, "HypercubicSetting", "jellyfysh.setting")
    from jellyfysh import setting
    positions, _ = systems.water_lattice(4, 12.42, 1.0, 1.633, np.random.default_rng(10))
    setting.set_number_of_root_nodes(64)
    setting.set_number_of_nodes_per_root_node(3)
    setting.set_number_of_node_levels(2)
    handler = factory.build_from_config(config, "OxygenOxygenSeparationOutputHandler",
                                        "jellyfysh.input_output_handler.output_handler")
    roots = []
    for m in range(64):
        root = Node(Unit(identifier=(m,), position=[float(v) for v in positions[3 * m + 1]], charge=None))
        for t in range(3):
            root.add_child(Node(Unit(identifier=(m, t), position=[float(v) for v in positions[3 * m + t]],
                                     charge=None)))
        roots.append(root)
    handler.write(roots)
    handler.post_run()
    return positions.tolist()


def test_oxygen_separation_samples_equal_the_reference_output_handler(tmp_path):
    from jellyfysh_gb300 import outputs
    reference_path = str(tmp_path / "reference.dat")
    positions = np.array(_in_child("reference_oxygen_separation_file", reference_path))
    ours_path = str(tmp_path / "ours.dat")
    with outputs.OxygenSeparationWriter(ours_path) as writer:
        writer.write(positions, 12.42)
    reference = open(reference_path).read().splitlines()
    ours = open(ours_path).read().splitlines()
    assert reference[0].startswith("# Run identification hash") and ours[0].startswith("# Run identification hash")
    assert len(ours) == 1 + 64 * 63 // 2 and reference[1:] == ours[1:]


def test_separation_samples_equal_the_reference_output_handler(tmp_path):
    from jellyfysh_gb300 import outputs
    reference_path = str(tmp_path / "reference.dat")
    positions = np.array(_in_child("reference_separation_file", reference_path))
    ours_path = str(tmp_path / "ours.dat")
    with outputs.SeparationWriter(ours_path) as writer:
        writer.write(positions, 4.308869380063767)
    reference = open(reference_path).read().splitlines()
    ours = open(ours_path).read().splitlines()
    assert reference[0].startswith("# Run identification hash") and ours[0].startswith("# Run identification hash")
    assert reference[1:] == ours[1:]



NEIGHBOURHOOD_SECTION = """
[PairNeighbourhood]
create = {create}
trash = {create}
internal_state_label = single_active_cell_occupancy
event_handler = gpu_neighbourhood_event_handler
number_event_handlers = 2

[GpuNeighbourhoodEventHandler]
potential = {potential}

[{potential_section}]
{parameters}
"""


def neighbourhood_configuration(text, spec):
    """The trajectory configuration with the pairwise nearby and surplus taggers (one TwoLeafUnitEventHandler per
    target) replaced by the GPU neighbourhood tagger and its event handler, which take the same targets as one
    in-state.  Everything else of the configuration stays."""
    import re
    text = text.replace("pair_nearby (excluded_cells_tagger),\n    pair_surplus (surplus_cells_tagger)",
                        "pair_neighbourhood (gpu_neighbourhood_tagger)")
    text = text.replace("pair_nearby, pair_surplus", "pair_neighbourhood")
    create = re.search(r"\[CellBoundary\]\ncreate = ([^\n]*)\n", text).group(1)
    if spec["potential"] == "hard_sphere":
        potential, section, parameters = "gpu_hard_sphere_potential", "GpuHardSpherePotential", "radius = %r" % (
            spec["radius"],)
    else:
        potential, section, parameters = ("gpu_lennard_jones_potential", "GpuLennardJonesPotential",
                                          "prefactor = 1.0\ncharacteristic_length = 1.0")
    start = text.index("\n[PairNearby]")
    end = text.index("\n[TwoLeafUnitEventHandler]")
    end = text.index("\n[", end + 1)
    return text[:start] + NEIGHBOURHOOD_SECTION.format(create=create, potential=potential,
                                                       potential_section=section, parameters=parameters) + text[end:]


def run_neighbourhood_handler(name):
    """The reference's SingleProcessMediator on a trajectory configuration whose pair taggers are the GPU
    neighbourhood tagger and event handler, built by the reference's factory (run in a child).  The random numbers are
    the trajectory's keyed draws.  The batched solve of the handler (one GPU launch of the potential for all targets,
    tested against the oracle on the GPU in tests/test_gpu_neighbourhood.py) is taken by a stand-in that solves the
    same pairs with the oracle, so that this test runs the reference's CPU-only loop with the drop-in's tagger,
    in-states, time slicing and out-states.  Returns the logged events and final positions."""
    factory, camel = _reference()
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_reference_trajectories as trajectories
    import oracle
    spec = dict(trajectories.SYSTEMS[name])

    def solve_with_oracle(potential, velocity, separations, charges, potential_changes):
        if spec["potential"] == "hard_sphere":
            times = [oracle.hs_displacement(spec["radius"], velocity, s) for s in separations]
        else:
            times = [oracle.lj_displacement(1.0, 1.0, velocity, s, du) for s, du in zip(separations, potential_changes)]
        if not times:
            return -1, float("inf")
        index = int(np.argmin(times))
        return (-1, float("inf")) if np.isinf(times[index]) else (index, float(times[index]))

    calls = {"solves": 0, "targets": 0}

    def counted_solve(potential, velocity, separations, charges, potential_changes):
        calls["solves"] += 1
        calls["targets"] += len(separations)
        return solve_with_oracle(potential, velocity, separations, charges, potential_changes)

    def prepare(context):
        import jellyfysh.event_handler.gpu_neighbourhood_event_handler as handler_module
        handler_module.earliest = counted_solve

        def keyed_change(self, unit):
            return oracle.expovariate(oracle.draw(context["key"], context["event_index"](), oracle.RNG_PAIR,
                                                  unit.identifier[0]), context["beta"])
        handler_module.GpuNeighbourhoodEventHandler._potential_change = keyed_change
        context["kinds"]["GpuNeighbourhoodEventHandler"] = oracle.EV_PAIR

    def transform(text):
        text = neighbourhood_configuration(text, spec)
        assert "[PairNearby]" not in text and "two_leaf_unit_event_handler" not in text
        return text

    events, _, final, _, _, _ = trajectories.record(TREE, spec, transform=transform, prepare=prepare)
    return {"events": {field: events[field].tolist() for field in events.dtype.names}, "final": final.tolist(),
            "calls": calls}


@pytest.mark.parametrize("name", ["hard_spheres_n64", "lennard_jones_n64_cell_veto"])
def test_neighbourhood_event_handler_reproduces_the_reference_trajectory(name):
    """The GPU neighbourhood tagger and event handler, selected by name in the reference's configuration and run in
    the reference's own mediator, reproduce the committed trajectory of the reference's pairwise handlers event for
    event: the same events, targets, liftings and times, and the same final positions."""
    result = _in_child("run_neighbourhood_handler", name)
    spec, initial, charges, events, final = load_trajectory(name)
    for field in events.dtype.names:
        assert np.array_equal(np.array(result["events"][field]), events[field]), field
    assert np.array_equal(np.array(result["final"]), final)
    # one batched solve per event of the neighbourhood handler, over all targets of the neighbourhood
    assert result["calls"]["solves"] >= len(events)
    assert result["calls"]["targets"] > 3 * result["calls"]["solves"]
