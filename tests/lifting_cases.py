"""Lifting tables recorded from the reference's lifting schemes (``golden/lifting_known_answers.json``, written by
``golden/make_lifting_golden.py``) and the status each expected outcome maps to."""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
STATUS = {None: 0, "AssertionError": 2, "LiftingSchemeError": 9, "IndexError": 10}


def load_cases():
    with open(os.path.join(HERE, "golden", "lifting_known_answers.json")) as handle:
        return json.load(handle)["cases"]


def expected_status(case) -> int:
    return STATUS[case["expected"].get("error")]


def draw_of(case) -> float:
    """The deciding draw (0.0 where the reference raises before drawing)."""
    return 0.0 if case["draw"] is None else float(case["draw"])
