"""Build recipe of the reference's own C code for the event-time path, for cross-checks of the oracle (test
infrastructure).

JeLLyFysh's merged-image Coulomb potential and inverse-power Coulomb bounding potential are plain C files that its
cffi builders compile (``jellyfysh/potential/merged_image_coulomb_potential/merged_image_coulomb_potential.c``,
``jellyfysh/potential/inverse_power_coulomb_bounding_potential/inverse_power_coulomb_bounding_potential.c``).  This
recipe compiles each, where it lies in the reference tree, into its own shared library under ``oracle/_ref/`` (both
define ``derivative``), with floating-point contraction off as on the x86-64 baseline the reference is built for.
The reference tree is the ``tree`` argument of ``build`` or the ``JELLYFYSH_REFERENCE`` environment variable (there
is no default); without one nothing is built.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SOURCES = {
    "libref_merged_image_coulomb.so":
        "jellyfysh/potential/merged_image_coulomb_potential/merged_image_coulomb_potential.c",
    "libref_inverse_power_coulomb_bound.so":
        "jellyfysh/potential/inverse_power_coulomb_bounding_potential/inverse_power_coulomb_bounding_potential.c",
}


def reference_tree(tree=None):
    tree = tree or os.environ.get("JELLYFYSH_REFERENCE")
    return tree if tree and os.path.isdir(os.path.join(tree, "jellyfysh", "potential")) else None


def build(tree=None, force: bool = False):
    """Compile the reference's C files of the tree ``tree`` (or JELLYFYSH_REFERENCE) into oracle/_ref/; returns the
    built paths (empty without a reference tree)."""
    tree = reference_tree(tree)
    if tree is None:
        return []
    os.makedirs(REF_DIR, exist_ok=True)
    built = []
    for name, relative in SOURCES.items():
        source = os.path.join(tree, relative)
        target = os.path.join(REF_DIR, name)
        if force or not os.path.exists(target) or os.path.getmtime(target) < os.path.getmtime(source):
            temporary = target + ".%d.tmp" % os.getpid()
            subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off",
                            "-fno-fast-math", "-I", os.path.dirname(source), "-o", temporary, source, "-lm"],
                           check=True)
            os.replace(temporary, target)
        built.append(target)
    return built


if __name__ == "__main__":
    trees = [a for a in sys.argv[1:] if not a.startswith("--")]
    print("\n".join(build(trees[0] if trees else None, force="--force" in sys.argv)) or "no reference tree: nothing built")
