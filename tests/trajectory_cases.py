"""Load the reference trajectories of ``golden/trajectory_*.npz`` and map their specs onto chain systems."""
import glob
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def trajectory_names():
    return sorted(os.path.basename(p)[len("trajectory_"):-len(".npz")]
                  for p in glob.glob(os.path.join(HERE, "golden", "trajectory_*.npz")))


def load_trajectory(name):
    data = np.load(os.path.join(HERE, "golden", "trajectory_%s.npz" % name))
    spec = json.loads(str(data["spec"]))
    charges = data["charges"] if data["charges"].size else None
    return spec, data["initial"], charges, data["events"], data["final"]


def oracle_system(spec):
    import oracle
    potential = {"hard_sphere": oracle.POT_HARD_SPHERE, "lennard_jones": oracle.POT_LENNARD_JONES,
                 "coulomb": oracle.POT_COULOMB}[spec["potential"]]
    far = {"none": oracle.FAR_NONE, "cell_veto": oracle.FAR_CELL_VETO,
           "cell_bounding": oracle.FAR_CELL_BOUNDING}[spec["far"]]
    return oracle.make_system(n=spec["n"], system_length=spec["system_length"], cells_per_side=spec["cells_per_side"],
                              neighbor_layers=spec["neighbor_layers"], max_occupants=1, beta=spec["beta"],
                              chain_time=spec["chain_time"], speed=1.0, initial_direction=0, initial_active=0,
                              potential=potential, hs_radius=spec.get("radius", 0.0), lj_prefactor=1.0, lj_sigma=1.0,
                              coulomb_prefactor=1.0, bound_prefactor=1.5837, ewald_alpha=3.45, fourier_cutoff=6,
                              position_cutoff=2, far=far, estimator_points=spec.get("estimator_points", 10),
                              estimator_prefactor=spec.get("estimator_prefactor", 1.5), rng_key=spec["rng_key"])
