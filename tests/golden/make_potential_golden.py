"""Generate ``potential_known_answers.json`` from the reference's own potential unit tests.

Run in a container that holds the JeLLyFysh source tree with its two cffi extensions built:

    python tests/golden/make_potential_golden.py /path/to/jellyfysh/tree

The script runs the reference's ``unittests/test_potential`` test cases unchanged, records every top-level
``displacement`` / ``derivative`` call of the potentials on this path (arguments before the call, the value the
reference returned) and pairs it with the ``assertAlmostEqual`` that checks it (the known answer the test holds and
its number of places).  The fixture therefore pins the oracle to the reference's arithmetic (bit-exact value) and to
the tests' independent known answers.
"""
import copy
import functools
import json
import os
import sys
import unittest


def main(tree: str, output: str) -> None:
    sys.path.insert(0, tree)
    sys.path.insert(0, os.path.join(tree, "unittests"))
    import jellyfysh.setting as setting
    from jellyfysh.potential.hard_sphere_potential import HardSpherePotential
    from jellyfysh.potential.inverse_power_potential import InversePowerPotential
    from jellyfysh.potential.lennard_jones_potential import LennardJonesPotential
    from jellyfysh.potential.displaced_even_power_potential import DisplacedEvenPowerPotential
    from jellyfysh.potential.inverse_power_coulomb_bounding_potential import InversePowerCoulombBoundingPotential
    from jellyfysh.potential.merged_image_coulomb_potential import MergedImageCoulombPotential

    classes = [HardSpherePotential, InversePowerPotential, LennardJonesPotential, DisplacedEvenPowerPotential,
               InversePowerCoulombBoundingPotential, MergedImageCoulombPotential]
    state = {"depth": 0, "calls": [], "cases": []}

    def wrap_init(cls):
        original = cls.__init__

        @functools.wraps(original)
        def init(self, *args, **kwargs):
            if not hasattr(self, "_golden_params"):
                self._golden_params = dict(kwargs, _args=list(args))
            original(self, *args, **kwargs)
        cls.__init__ = init

    def wrap_method(cls, name):
        original = getattr(cls, name)

        @functools.wraps(original)
        def method(self, *args, **kwargs):
            top = state["depth"] == 0
            recorded_args = copy.deepcopy(args)
            recorded_kwargs = copy.deepcopy(kwargs)
            state["depth"] += 1
            try:
                result = original(self, *args, **kwargs)
            finally:
                state["depth"] -= 1
            if top and type(self) in classes:
                length = None
                if hasattr(self, "_system_length"):
                    length = self._system_length
                else:
                    try:
                        from jellyfysh.setting import hypercubic_setting
                        length = hypercubic_setting.system_length
                    except ImportError:
                        length = None
                attributes = {key: value for key, value in vars(self).items()
                              if isinstance(value, (int, float)) and not isinstance(value, bool)}
                state["calls"].append(dict(potential=type(self).__name__, params=self._golden_params,
                                           attributes=attributes,
                                           system_length=length, method=name, args=list(recorded_args),
                                           kwargs=recorded_kwargs, result=result, result_id=id(result)))
            return result
        setattr(cls, name, method)

    for cls in classes:
        wrap_init(cls)
    for cls in classes:
        for name in ("displacement", "derivative"):
            if name in cls.__dict__ or any(name in base.__dict__ for base in cls.__mro__[1:]):
                wrap_method(cls, name)

    original_almost_equal = unittest.TestCase.assertAlmostEqual

    def almost_equal(self, first, second, places=None, msg=None, delta=None):
        for call in reversed(state["calls"]):
            if call["result_id"] == id(first) and call["result"] is first:
                case = {key: value for key, value in call.items() if key != "result_id"}
                case["reference"] = case.pop("result")
                case["expected"] = second
                case["places"] = places
                case["test"] = self.id()
                case["reference_meets_known_answer"] = True
                state["cases"].append(case)
                try:
                    return original_almost_equal(self, first, second, places=places, msg=msg, delta=delta)
                except AssertionError:
                    # the reference test tolerates this miss (it catches the AssertionError itself)
                    case["reference_meets_known_answer"] = False
                    raise
        return original_almost_equal(self, first, second, places=places, msg=msg, delta=delta)
    unittest.TestCase.assertAlmostEqual = almost_equal

    loader = unittest.TestLoader()
    suite = unittest.TestSuite()
    for module in ("test_hard_sphere_potential", "test_inverse_power_potential", "test_lennard_jones_potential",
                   "test_displaced_even_power_potential", "test_inverse_power_coulomb_bounding_potential",
                   "test_merged_image_coulomb_potential"):
        suite.addTests(loader.loadTestsFromName("test_potential." + module))
    result = unittest.TextTestRunner(verbosity=0).run(suite)
    if not result.wasSuccessful():
        raise SystemExit("reference potential tests failed")
    setting.reset() if hasattr(setting, "reset") else None
    with open(output, "w") as handle:
        json.dump({"source": "reference unittests/test_potential (known answers calculated in the tests)",
                   "cases": state["cases"]}, handle, indent=1)
    print("wrote %d cases to %s" % (len(state["cases"]), output))


if __name__ == "__main__":
    from _tree import tree_argument
    tree_path = tree_argument(sys.argv)
    main(tree_path, os.path.join(os.path.dirname(os.path.abspath(__file__)), "potential_known_answers.json"))
