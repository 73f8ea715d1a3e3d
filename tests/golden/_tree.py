"""Where the fixture scripts find the reference: a JeLLyFysh source tree with its cffi extensions built, named by
the first command-line argument or by the JELLYFYSH_TREE environment variable (there is no default)."""
import os
import sys


def tree_argument(argv) -> str:
    tree = argv[1] if len(argv) > 1 else os.environ.get("JELLYFYSH_TREE")
    if not tree or not os.path.isdir(os.path.join(tree, "jellyfysh")):
        raise SystemExit("usage: %s JELLYFYSH_TREE [name ...]  (or set JELLYFYSH_TREE): a JeLLyFysh source tree "
                         "with its cffi extensions built" % os.path.basename(argv[0]))
    return tree
