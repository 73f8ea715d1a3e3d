"""Sampling outputs in the reference's file formats (CPU).

The separation samples of ``jellyfysh_gb300.outputs`` equal, line for line, the reference's arithmetic written out
with Python floats: separation target - reference corrected by ``(s + L/2) % L - L/2``
(``setting/hypercubic_setting.py:120-172``), norm ``sum(c * c for c in s) ** 0.5`` (``base/vectors.py:29-43``),
printed as Python prints a float (``separation_output_handler.py:75-97``).
"""
import numpy as np
import pytest

from jellyfysh_gb300 import outputs


def reference_lines(positions, length):
    half = length / 2.0
    lines = []
    units = [[float(v) for v in p] for p in positions]
    for i in range(len(units)):
        for j in range(i + 1, len(units)):
            separation = [(units[j][k] - units[i][k] + half) % length - half for k in range(3)]
            lines.append(repr(sum(c * c for c in separation) ** 0.5))
    return lines


def test_separation_norms_follow_the_reference_arithmetic():
    rng = np.random.default_rng(5)
    for n, length in ((40, 1.0), (64, 4.308869380063767), (30, 10.857)):
        positions = rng.uniform(0.0, length, size=(n, 3))
        positions[3] = positions[4] + [length * 0.5, 0.0, -length * 0.5]  # separations at +-L/2
        positions[5] = positions[6]                                      # zero separation
        positions %= length
        ours = [repr(x) for x in outputs.pair_separation_norms(positions, length).tolist()]
        assert ours == reference_lines(positions, length)


def test_separation_writer_file_layout(tmp_path):
    rng = np.random.default_rng(6)
    length = 3.0
    samples = [rng.uniform(0.0, length, size=(12, 3)) for _ in range(3)]
    path = str(tmp_path / "separations.dat")
    with outputs.SeparationWriter(path) as writer:
        for positions in samples:
            writer.write(positions, length)
    lines = open(path).read().splitlines()
    assert lines[0].startswith("# Run identification hash: ")
    expected = sum((reference_lines(p, length) for p in samples), [])
    assert lines[1:] == expected


def test_oxygen_separation_writer_takes_the_second_unit_of_every_molecule(tmp_path):
    from jellyfysh_gb300 import outputs, systems
    positions, _ = systems.water_lattice(2, 6.21, 1.0, 1.633, np.random.default_rng(3))
    path = str(tmp_path / "oo.dat")
    with outputs.OxygenSeparationWriter(path) as writer:
        writer.write(positions, 6.21)
    lines = open(path).read().splitlines()
    expected = outputs.pair_separation_norms(positions[1::3], 6.21)
    assert [float(x) for x in lines[1:]] == expected.tolist()
    with pytest.raises(ValueError):
        with outputs.OxygenSeparationWriter(str(tmp_path / "bad.dat")) as writer:
            writer.write(positions[:4], 6.21)
