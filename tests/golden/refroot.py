"""The command-line argument of the fixture generators: the reference project's checkout."""
import sys


def reference_root() -> str:
    """The reference project's checkout, the generator's one argument (its methods are read from there)."""
    if len(sys.argv) < 2:
        sys.exit(f"usage: python {sys.argv[0]} REFERENCE_ROOT   (a checkout of the DiffTactile project)")
    return sys.argv[1]
