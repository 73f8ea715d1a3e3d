"""Lifting schemes on the CPU: the oracle against the reference's recorded tables, and the host-side table layout
of the GPU entry point (no compute)."""
import math

import numpy as np
import pytest

import oracle
from jellyfysh_gb300 import lifting
from tests.lifting_cases import draw_of, expected_status, load_cases

CASES = load_cases()


def test_fixture_covers_every_scheme_outcome_and_draw_mode():
    seen = {(c["scheme"], c["draw_mode"], expected_status(c)) for c in CASES}
    for scheme in ("inside_first", "outside_first", "ratio"):
        assert (scheme, "value", 0) in seen and (scheme, "unit", 0) in seen
        for status in (2, 9, 10):
            assert (scheme, "unit", status) in seen
    assert sum(c["source"] == "unittests/test_lifting" for c in CASES) == 18


@pytest.mark.parametrize("index", range(len(CASES)))
def test_oracle_matches_the_reference(index):
    case = CASES[index]
    status, selected, bound = oracle.lifting(case["scheme"], case["rates"], case["active"], draw_of(case),
                                             unit_draw=case["draw_mode"] == "unit")
    assert status == expected_status(case)
    if status == 0:
        assert selected == case["expected"]["index"]
    if case["uniform_args"] is not None:
        assert case["uniform_args"][0] == 0.0
        assert bound == case["uniform_args"][1]  # the reference's random.uniform bound, bit for bit


def test_oracle_reports_no_bound_when_the_reference_raises_first():
    status, selected, bound = oracle.lifting("ratio", [0.5, -0.5], [False, False], 0.3)
    assert (status, selected) == (9, -1) and math.isnan(bound)


def test_pack_lays_tables_back_to_back():
    rates, active, offsets = lifting.pack([([0.5, -1.0], [True, False]), ([], []), ([-0.25, 0.75, -0.5],
                                                                                    [False, True, False])])
    assert offsets.tolist() == [0, 2, 2, 5]
    assert rates.tolist() == [0.5, -1.0, -0.25, 0.75, -0.5]
    assert active.tolist() == [1, 0, 0, 1, 0]
    rates, active, offsets = lifting.pack([([], []), ([], [])])
    assert offsets.tolist() == [0, 0, 0] and len(rates) == 1  # room for a valid pointer
    with pytest.raises(ValueError):
        lifting.pack([([0.5, -1.0], [True])])


def test_class_interface_raises_at_the_reference_calls():
    # errors raised on the host before any device work, as the reference raises them in insert / get
    scheme = lifting.InsideFirstLifting()
    with pytest.raises(AssertionError):
        scheme.insert(-0.5, (1, 2), True)
    scheme.reset()
    scheme.insert(0.5, (1, 2), False)
    scheme.insert(-0.5, (3, 4), False)
    with pytest.raises(lifting.LiftingSchemeError):
        scheme.get_active_identifier()
    ratio = lifting.RatioLifting()
    ratio.insert(-0.3, (1, 2), False)
    with pytest.raises(lifting.LiftingSchemeError):
        ratio.get_active_identifier()


def test_plugin_modules_name_the_reference_classes():
    import importlib
    import os
    from jellyfysh_gb300 import plugin
    directory = plugin.PACKAGES["lifting"]
    for scheme, name in (("inside_first", "InsideFirstLifting"), ("outside_first", "OutsideFirstLifting"),
                         ("ratio", "RatioLifting")):
        assert os.path.exists(os.path.join(directory, "gpu_%s_lifting.py" % scheme))
        module = importlib.import_module("jellyfysh_gb300.plugin.lifting.gpu_%s_lifting" % scheme)
        cls = getattr(module, "Gpu" + name)
        assert issubclass(cls, getattr(lifting, name)) and cls.scheme == scheme
