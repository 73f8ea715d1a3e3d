"""Drop-in classes for the reference's INI factory.

The reference builds every object of a run from its configuration file with ``base/factory.py:22-135``: a class
``CamelName`` is found as ``jellyfysh.<package>.camel_name`` (``factory.py:111-122``) and constructed from the keys
of its section, typed by the constructor's annotations (``factory.py:180-235``).  ``install()`` appends this
package's directories to the search paths of ``jellyfysh.potential``, ``jellyfysh.lifting``, ``jellyfysh.mediator``,
``jellyfysh.event_handler`` and ``jellyfysh.activator.tagger``, so that a configuration names the GPU classes exactly
like the reference's own:

    [TwoLeafUnitEventHandler]
    potential = gpu_lennard_jones_potential          ; instead of lennard_jones_potential

    [TwoCompositeObjectSummedBoundingPotentialEventHandler]
    lifting = gpu_inside_first_lifting               ; instead of inside_first_lifting

    [Run]
    mediator = gpu_chain_batch_mediator              ; instead of single_process_mediator

    [TagActivator]
    taggers = pair_neighbourhood (gpu_neighbourhood_tagger), ...   ; instead of the pairwise nearby/surplus taggers
    [PairNeighbourhood]
    event_handler = gpu_neighbourhood_event_handler  ; one GPU launch for all pairs of the neighbourhood

The potentials evaluate the reference's displacement / derivative and the lifting schemes decide the new active
unit on the GPU one call at a time (drop-ins for the reference's own event handlers); the neighbourhood event handler
solves all pair candidates of the active unit in one launch inside the reference's own mediator loop; the mediator
runs the whole configured system as a batch of chains on the GPU.
Nothing here needs the reference to be importable except ``install()`` and the mediator's translation of a
configured run.
"""
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PACKAGES = {"potential": os.path.join(HERE, "potential"), "mediator": os.path.join(HERE, "mediator"),
            "lifting": os.path.join(HERE, "lifting"), "event_handler": os.path.join(HERE, "event_handler"),
            "activator.tagger": os.path.join(HERE, "tagger")}


def install() -> None:
    """Make the GPU classes resolvable by the reference's factory (requires the ``jellyfysh`` package)."""
    import importlib
    for package, directory in PACKAGES.items():
        module = importlib.import_module("jellyfysh." + package)
        if directory not in module.__path__:
            module.__path__.append(directory)
