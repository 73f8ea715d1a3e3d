"""GPU lifting schemes through the C ABI (``jfgpu_lifting``) against the reference's recorded tables and the oracle.

The decision is integer (the table index of the new active unit, or the reference's exception): bit-exact.  The
bound of the deciding random.uniform call is compared bit for bit as well.
"""
import random
from unittest import mock

import numpy as np
import pytest

import oracle
from tests.lifting_cases import draw_of, expected_status, load_cases

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = load_cases()


@pytest.fixture(scope="module")
def lifting():
    from jellyfysh_gb300 import _lib, lifting as module
    _lib.load()
    return module


@pytest.mark.parametrize("scheme", ["inside_first", "outside_first", "ratio"])
@pytest.mark.parametrize("draw_mode", ["value", "unit"])
def test_batched_tables_match_the_reference(lifting, scheme, draw_mode):
    cases = [c for c in CASES if c["scheme"] == scheme and c["draw_mode"] == draw_mode]
    assert cases
    rates, active, offsets = lifting.pack([(c["rates"], c["active"]) for c in cases])
    selected, bound, status = lifting.select(scheme, rates, active, offsets, [draw_of(c) for c in cases],
                                             unit_draws=draw_mode == "unit")
    for k, case in enumerate(cases):
        assert status[k] == expected_status(case), case
        if status[k] == 0:
            assert selected[k] == case["expected"]["index"], case
        else:
            assert selected[k] == -1
        if case["uniform_args"] is not None:
            assert bound[k] == case["uniform_args"][1], case


@pytest.mark.parametrize("index", range(len(CASES)))
def test_class_interface_matches_the_reference(lifting, index):
    """One table at a time through the reference's interface, random.uniform mocked as the reference's tests do."""
    case = CASES[index]
    classes = {"inside_first": lifting.InsideFirstLifting, "outside_first": lifting.OutsideFirstLifting,
               "ratio": lifting.RatioLifting}
    identifiers = [(i, 7) for i in range(len(case["rates"]))]
    with mock.patch("jellyfysh_gb300.lifting.random.uniform") as uniform:
        if case["draw_mode"] == "value":
            uniform.return_value = draw_of(case)
        else:  # random.uniform(a, b) of Python from the recorded unit draw
            uniform.side_effect = lambda a, b: a + (b - a) * draw_of(case)
        scheme = classes[case["scheme"]]()
        scheme.reset()
        error = case["expected"].get("error")
        if error == "AssertionError":  # the reference asserts in insert
            with pytest.raises(AssertionError):
                for rate, identifier, is_active in zip(case["rates"], identifiers, case["active"]):
                    scheme.insert(rate, identifier, is_active)
            return
        for rate, identifier, is_active in zip(case["rates"], identifiers, case["active"]):
            scheme.insert(rate, identifier, is_active)
        if error is None:
            assert scheme.get_active_identifier() == identifiers[case["expected"]["index"]]
            if case["uniform_args"] is not None:
                assert list(uniform.call_args[0]) == case["uniform_args"]
        else:
            expected = {"LiftingSchemeError": lifting.LiftingSchemeError, "IndexError": IndexError}[error]
            with pytest.raises(expected):
                scheme.get_active_identifier()


def _random_tables(rng, count):
    tables = []
    for _ in range(count):
        size = rng.randrange(0, 17)
        rates = []
        for _ in range(size):
            u = rng.random()
            if u < 0.05:
                rates.append(0.0)
            elif u < 0.5:
                rates.append(-rng.choice([rng.uniform(0, 3), rng.uniform(0, 1e-9), float(rng.randrange(1, 9)) / 8]))
            else:
                rates.append(rng.choice([rng.uniform(0, 3), rng.uniform(0, 1e-9), float(rng.randrange(1, 9)) / 8]))
        active = [False] * size
        positives = [i for i, r in enumerate(rates) if r > 0.0]
        if positives and rng.random() < 0.95:
            active[rng.choice(positives)] = True
        elif size and rng.random() < 0.5:
            active[rng.randrange(size)] = True
        tables.append((rates, active))
    return tables


@pytest.mark.parametrize("scheme", ["inside_first", "outside_first", "ratio"])
def test_large_ragged_batch_matches_the_oracle(lifting, scheme):
    rng = random.Random({"inside_first": 1, "outside_first": 2, "ratio": 3}[scheme])
    tables = _random_tables(rng, 20000)
    draws = [rng.random() for _ in tables]
    rates, active, offsets = lifting.pack(tables)
    selected, bound, status = lifting.select(scheme, rates, active, offsets, draws, unit_draws=True)
    for k, (table, draw) in enumerate(zip(tables, draws)):
        want = oracle.lifting(scheme, table[0], table[1], draw, unit_draw=True)
        assert (int(status[k]), int(selected[k])) == want[:2], (table, draw)
        assert bound[k] == want[2] or (np.isnan(bound[k]) and np.isnan(want[2]))


def test_device_resident_inputs_and_empty_tables(lifting):
    device = torch.device("cuda")
    rates = torch.tensor([0.5, -1.0, -1.0], dtype=torch.float64, device=device)
    active = torch.tensor([1, 0, 0], dtype=torch.int32, device=device)
    offsets = torch.tensor([0, 3, 3], dtype=torch.int64, device=device)
    draws = torch.tensor([0.25, 0.5], dtype=torch.float64, device=device)
    selected, bound, status = lifting.select("outside_first", rates, active, offsets, draws)
    # outside-first: position 2.0 - 0.25 = 1.75 falls into the second negative entry
    assert selected.tolist() == [2, -1] and status.tolist() == [0, 9] and bound[0] == 0.5
    selected, bound, status = lifting.select("ratio", [], [], [0], [])
    assert len(selected) == 0 and len(status) == 0


def test_invalid_scheme_and_draw_mode_are_argument_errors(lifting):
    from jellyfysh_gb300 import _lib
    lib = _lib.load()
    device = torch.device("cuda")
    buffers = [torch.zeros(4, dtype=dtype, device=device)
               for dtype in (torch.float64, torch.int32, torch.int64, torch.float64, torch.int64, torch.float64,
                             torch.int32)]
    pointers = [b.data_ptr() for b in buffers]
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.jfgpu_lifting(3, 0, pointers[0], pointers[1], pointers[2], 1, pointers[3], pointers[4], pointers[5],
                             pointers[6], stream) == 2
    assert lib.jfgpu_lifting(0, 2, pointers[0], pointers[1], pointers[2], 1, pointers[3], pointers[4], pointers[5],
                             pointers[6], stream) == 2
    torch.cuda.synchronize()
