"""Water trajectories recorded from the reference's event loop: every pair of molecules with a Coulomb factor
(``golden/water_n*.npz`` without ``cell`` in the name, written by ``golden/make_water_trajectories.py``) and with the
molecular cells of its water cell-veto configuration (``golden/water_*cell*.npz``, written by
``golden/make_water_cell_trajectories.py``)."""
import glob
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIELDS = ("kind", "moved", "target", "new_active", "new_direction", "accepted")


def water_names():
    return sorted(os.path.basename(p)[:-len(".npz")] for p in glob.glob(os.path.join(HERE, "golden", "water_*.npz"))
                  if "cell" not in os.path.basename(p))


def water_cell_names():
    return sorted(os.path.basename(p)[:-len(".npz")]
                  for p in glob.glob(os.path.join(HERE, "golden", "water_*cell*.npz")))


def load_water_cells(name):
    """(spec, fixture arrays) of a trajectory with molecular cells."""
    data = np.load(os.path.join(HERE, "golden", name + ".npz"))
    return json.loads(str(data["spec"])), data


def load_water(name):
    data = np.load(os.path.join(HERE, "golden", name + ".npz"))
    spec = json.loads(str(data["spec"]))
    return spec, data["initial"], data["charges"], data["events"], data["final"]
