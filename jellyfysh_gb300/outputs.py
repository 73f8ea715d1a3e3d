"""Sampling outputs in the reference's file formats, written from configurations of the GPU engine.

``SeparationWriter`` writes what the reference's ``SeparationOutputHandler`` writes for systems of point masses
(``input_output_handler/output_handler/separation_output_handler.py:75-97``): a first line with a run
identification hash, then for every sample the norm of the shortest separation of every pair of units (first unit
before second, in identifier order), one per line, as Python prints a float.  The numbers are computed with the
reference's operations on the same doubles: the separation ``target - reference`` corrected as
``(s + L/2) % L - L/2`` (``setting/hypercubic_setting.py:120-172``) and the norm ``sum(c * c) ** 0.5``
(``base/vectors.py:29-43``, ``sum`` with CPython 3.12's compensation, ``**`` with the C library's ``pow``), so that
the reference's analysis scripts read the files unchanged.  ``OxygenSeparationWriter`` writes the water samples of
``OxygenOxygenSeparationOutputHandler`` (``oxygen_oxygen_separation_output_handler.py:67-88``): the same norms for the
oxygens, the second unit of every molecule.  Like the reference's writer (``output_handler.py:90-125``), a file is
written under a temporary name and renamed when closed.
"""
import os
import uuid

import numpy as np


def _python_sum3(a: np.ndarray, b: np.ndarray, c: np.ndarray) -> np.ndarray:
    """sum((a, b, c)) elementwise with CPython 3.12's Neumaier compensation (starting from the integer 0)."""
    f = a + 0.0
    t = f + b
    comp = np.where(np.abs(f) >= np.abs(b), (f - t) + b, (b - t) + f)
    f = t
    t = f + c
    comp = comp + np.where(np.abs(f) >= np.abs(c), (f - t) + c, (c - t) + f)
    f = t
    use = (comp != 0.0) & np.isfinite(comp)
    return np.where(use, f + comp, f)


def pair_separation_norms(positions: np.ndarray, system_length: float) -> np.ndarray:
    """Norms of the corrected separations of all pairs (i < j), in the reference's order and arithmetic."""
    p = np.ascontiguousarray(positions, dtype=np.float64)
    half = system_length / 2.0
    i, j = np.triu_indices(len(p), k=1)
    s = p[j] - p[i]
    s = np.mod(s + half, system_length) - half
    squares = _python_sum3(s[:, 0] * s[:, 0], s[:, 1] * s[:, 1], s[:, 2] * s[:, 2])
    # ``** 0.5`` of Python floats calls the C library's pow, which is not always the correctly rounded square root
    # (numpy's power may take a square-root shortcut or its own vector routines): one Python power per pair
    return np.array([x ** 0.5 for x in squares.tolist()], dtype=np.float64)


class SeparationWriter:
    """The reference's separation samples file for point masses, one sample per ``write``."""

    def __init__(self, filename: str) -> None:
        self._filename = filename
        self._file = open(filename + ".tmp", "w")
        self._file.write("# Run identification hash: {0}\n".format(uuid.uuid4().hex))

    def write(self, positions: np.ndarray, system_length: float) -> None:
        norms = pair_separation_norms(positions, system_length)
        self._file.write("".join(repr(x) + "\n" for x in norms.tolist()))

    def close(self) -> None:
        self._file.close()
        os.replace(self._filename + ".tmp", self._filename)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class OxygenSeparationWriter(SeparationWriter):
    """The reference's oxygen-oxygen separation samples file for water, one sample per ``write`` of the positions of
    all units (hydrogen, oxygen, hydrogen per molecule)."""

    def write(self, positions: np.ndarray, system_length: float) -> None:
        units = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        if len(units) % 3:
            raise ValueError("water positions come in molecules of three units")
        super().write(units[1::3], system_length)
