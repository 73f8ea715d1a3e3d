"""Generate ``lifting_known_answers.json`` from the reference's lifting schemes.

Run in a container that holds the JeLLyFysh source tree:

    python tests/golden/make_lifting_golden.py /path/to/jellyfysh/tree

Three kinds of cases, each a lifting table (factor derivatives in insertion order, the active flag of each entry),
the draw that decides the outcome and what the reference returned or raised:

* ``unittests/test_lifting`` run unchanged: every ``get_active_identifier`` call of the three schemes, with the
  table filled since the last ``reset`` and the value the tests' mocked ``random.uniform`` returned (draw mode
  "value"), together with the arguments the reference passed to ``random.uniform`` (the tests assert them);
* seeded random tables run through the reference's classes with Python's real ``random`` (draw mode "unit"): the
  unit draw is the first ``random()`` of the seed, from which the reference's ``random.uniform(0.0, b)`` formed its
  value.  The tables mix positive, negative and zero derivatives, missing and misplaced active units and empty
  negative sides, so the errors the reference raises are covered as well;
* hand-made tables with mocked draws that land exactly on cumulative sums of the negative side (the reference
  selects with ``<=``), run through the reference's classes.

The draw that decides the outcome is the one of the active unit's ``insert`` for the inside-first and
outside-first schemes (``lifting/lifting.py:47-80``) and the one of ``get_active_identifier`` for the ratio scheme
(``lifting/ratio_lifting.py:38-56``).
"""
import json
import os
import random
import sys
import unittest

SCHEMES = {"InsideFirstLifting": "inside_first", "OutsideFirstLifting": "outside_first", "RatioLifting": "ratio"}
RANDOM_CASES = 400


def _outcome(call, identifiers):
    """{"index": table index} of the returned identifier, or {"error": exception class name}."""
    try:
        identifier = call()
    except Exception as error:  # the reference's LiftingSchemeError, AssertionError, IndexError
        return {"error": type(error).__name__}
    return {"index": identifiers.index(identifier)}


def record_unittests(tree):
    """Cases of the reference's own lifting unit tests (mocked random.uniform)."""
    sys.path.insert(0, os.path.join(tree, "unittests"))
    from jellyfysh.lifting.lifting import Lifting
    import jellyfysh.lifting.lifting as lifting_module

    cases = []
    tables = {}
    original_reset, original_insert = Lifting.reset, Lifting.insert

    def reset(self):
        tables[id(self)] = {"rates": [], "active": [], "identifiers": [], "draw": None, "uniform_args": None}
        original_reset(self)

    def insert(self, lifting_rate, associated_identifier, is_active):
        table = tables.setdefault(id(self), {"rates": [], "active": [], "identifiers": [], "draw": None,
                                             "uniform_args": None})
        table["rates"].append(lifting_rate)
        table["active"].append(bool(is_active))
        table["identifiers"].append(associated_identifier)
        uniform = lifting_module.random.uniform
        before = getattr(uniform, "call_count", None)
        try:
            original_insert(self, lifting_rate, associated_identifier, is_active)
        except AssertionError:
            table["insert_error"] = "AssertionError"
            raise
        if before is not None and uniform.call_count > before:
            table["draw"] = uniform.return_value
            table["uniform_args"] = list(uniform.call_args[0])

    originals = {}

    def wrap(cls):
        original = originals[cls] = cls.get_active_identifier

        def get_active_identifier(self):
            table = tables[id(self)]
            scheme = SCHEMES[type(self).__name__]
            uniform = lifting_module.random.uniform
            before = uniform.call_count
            case = {"scheme": scheme, "draw_mode": "value", "rates": list(table["rates"]),
                    "active": list(table["active"])}
            try:
                result = original(self)
            except Exception as error:
                case.update(draw=None, uniform_args=None, expected={"error": type(error).__name__})
                cases.append(case)
                raise
            if scheme == "ratio":
                assert uniform.call_count == before + 1
                case.update(draw=uniform.return_value, uniform_args=list(uniform.call_args[0]))
            else:
                case.update(draw=table["draw"], uniform_args=table["uniform_args"])
            case["expected"] = {"index": table["identifiers"].index(result)}
            cases.append(case)
            return result
        cls.get_active_identifier = get_active_identifier

    Lifting.reset, Lifting.insert = reset, insert
    from jellyfysh.lifting.inside_first_lifting import InsideFirstLifting
    from jellyfysh.lifting.outside_first_lifting import OutsideFirstLifting
    from jellyfysh.lifting.ratio_lifting import RatioLifting
    for cls in (InsideFirstLifting, OutsideFirstLifting, RatioLifting):
        wrap(cls)
    suite = unittest.TestSuite()
    loader = unittest.TestLoader()
    for module in ("test_inside_first_lifting", "test_outside_first_lifting", "test_ratio_lifting"):
        suite.addTests(loader.loadTestsFromName("test_lifting." + module))
    result = unittest.TextTestRunner(verbosity=0).run(suite)
    if not result.wasSuccessful():
        raise SystemExit("reference lifting tests failed")
    Lifting.reset, Lifting.insert = original_reset, original_insert
    for cls, original in originals.items():
        cls.get_active_identifier = original
    for case in cases:
        case["source"] = "unittests/test_lifting"
    return cases


def _random_table(rng):
    """A table of 0..10 entries: positive, negative and zero derivatives, usually one active positive entry."""
    count = rng.randrange(0, 11)
    rates = []
    for _ in range(count):
        kind = rng.random()
        if kind < 0.08:
            rates.append(0.0)
        elif kind < 0.12:
            rates.append(-0.0)
        elif kind < 0.55:
            rates.append(-rng.choice([rng.uniform(0.0, 2.0), rng.uniform(0.0, 1e-6), float(rng.randrange(1, 5))]))
        else:
            rates.append(rng.choice([rng.uniform(0.0, 2.0), rng.uniform(0.0, 1e-6), float(rng.randrange(1, 5)) / 4]))
    active = [False] * count
    positives = [i for i, r in enumerate(rates) if r > 0.0]
    mode = rng.random()
    if positives and mode < 0.85:
        active[rng.choice(positives)] = True
    elif count and mode < 0.93:
        # an active entry with a non-positive derivative: the reference's insert asserts
        active[rng.randrange(count)] = True
    return rates, active


def record_random(seed=20240611):
    """Seeded random tables through the reference's classes with Python's real random numbers."""
    from jellyfysh.lifting.inside_first_lifting import InsideFirstLifting
    from jellyfysh.lifting.outside_first_lifting import OutsideFirstLifting
    from jellyfysh.lifting.ratio_lifting import RatioLifting
    classes = {"inside_first": InsideFirstLifting, "outside_first": OutsideFirstLifting, "ratio": RatioLifting}
    rng = random.Random(seed)
    cases = []
    for k in range(RANDOM_CASES):
        scheme = ("inside_first", "outside_first", "ratio")[k % 3]
        rates, active = _random_table(rng)
        draw_seed = rng.randrange(1 << 30)
        # the reference consumes one random() per random.uniform call: the inside-first and outside-first
        # schemes draw in the active insert, the ratio scheme draws in the active insert and again in
        # get_active_identifier
        draws = random.Random(draw_seed)
        unit = draws.random()
        if scheme == "ratio":
            unit = draws.random() if any(a and r > 0.0 for r, a in zip(rates, active)) else unit
        identifiers = [(i, 0) for i in range(len(rates))]
        lifting = classes[scheme]()
        random.seed(draw_seed)
        lifting.reset()
        try:
            for rate, identifier, is_active in zip(rates, identifiers, active):
                lifting.insert(rate, identifier, is_active)
        except AssertionError:
            expected = {"error": "AssertionError"}
        else:
            expected = _outcome(lifting.get_active_identifier, identifiers)
        cases.append({"scheme": scheme, "draw_mode": "unit", "rates": rates, "active": active, "draw": unit,
                      "uniform_args": None, "expected": expected, "source": "generated, reference classes"})
    return cases


def record_ties():
    """Draws that land exactly on a cumulative sum of the negative side (the reference selects with <=)."""
    from unittest import mock
    from jellyfysh.lifting.inside_first_lifting import InsideFirstLifting
    from jellyfysh.lifting.outside_first_lifting import OutsideFirstLifting
    from jellyfysh.lifting.ratio_lifting import RatioLifting
    classes = {"inside_first": InsideFirstLifting, "outside_first": OutsideFirstLifting, "ratio": RatioLifting}
    tables = [([0.25, -0.5, -0.25, 1.0, -0.75], [False, False, False, True, False]),
              ([-0.1, -0.2, -0.3, 0.6], [False, False, False, True]),
              ([0.5, -1.0, -1.0, -1.0, 0.5], [True, False, False, False, False]),
              ([-0.3, 0.3, -0.0, -0.7], [False, True, False, False])]
    draws = [0.0, 0.1, 0.25, 0.3, 0.5, 0.6, 0.75, 1.0, 1.5, 2.0, 3.0, 0.30000000000000004]
    cases = []
    for scheme, cls in classes.items():
        for rates, active in tables:
            for draw in draws:
                identifiers = [(i, 1) for i in range(len(rates))]
                with mock.patch("jellyfysh.lifting.lifting.random.uniform") as uniform:
                    uniform.return_value = draw
                    lifting = cls()
                    lifting.reset()
                    for rate, identifier, is_active in zip(rates, identifiers, active):
                        lifting.insert(rate, identifier, is_active)
                    expected = _outcome(lifting.get_active_identifier, identifiers)
                    args = list(uniform.call_args[0])
                cases.append({"scheme": scheme, "draw_mode": "value", "rates": rates, "active": active, "draw": draw,
                              "uniform_args": args, "expected": expected, "source": "generated ties, reference classes"})
    return cases


def main(tree, output):
    sys.path.insert(0, tree)
    import logging
    logging.disable(logging.ERROR)
    cases = record_unittests(tree) + record_ties() + record_random()
    with open(output, "w") as handle:
        json.dump({"source": "reference lifting schemes: unittests/test_lifting and seeded tables through the "
                             "reference's classes", "cases": cases}, handle, indent=None)
        handle.write("\n")
    print("wrote %d cases to %s" % (len(cases), output))


if __name__ == "__main__":
    from _tree import tree_argument
    tree_path = tree_argument(sys.argv)
    main(tree_path, os.path.join(os.path.dirname(os.path.abspath(__file__)), "lifting_known_answers.json"))
