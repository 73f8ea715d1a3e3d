"""Water trajectories recorded from the reference's event loop (``golden/water_*.npz``, written by
``golden/make_water_trajectories.py``)."""
import glob
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIELDS = ("kind", "moved", "target", "new_active", "new_direction", "accepted")


def water_names():
    return sorted(os.path.basename(p)[:-len(".npz")] for p in glob.glob(os.path.join(HERE, "golden", "water_*.npz")))


def load_water(name):
    data = np.load(os.path.join(HERE, "golden", name + ".npz"))
    spec = json.loads(str(data["spec"]))
    return spec, data["initial"], data["charges"], data["events"], data["final"]
