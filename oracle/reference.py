"""Where the HEAL reference sources are, for the recipes that read them.

Only the checker's recipes use this: oracle/build_ref.sh (compiles HEAL's
example_impl into oracle/_ref/), the CPU tests that build HEAL's C++ suite or
import HEAL's Python runtime, and __graft_entry__.build().  The location is
the HEAL_REFERENCE environment variable, else the development container's
checkout; `path()` is None when neither holds HEAL's sources, and those
recipes then skip.  Nothing on the GPU host or in the product reads it.
"""
import os

_DEFAULT = "/root/reference"


def path():
    """The reference checkout, or None when HEAL's sources are not present."""
    for cand in (os.environ.get("HEAL_REFERENCE"), _DEFAULT):
        if cand and os.path.isdir(os.path.join(cand, "example_impl")):
            return cand
    return None
