"""Where the AFEPack source tree is, for the recipes that read it.

Only the oracle recipes, the fixture generator and the CPU tests that compile
against the AFEPack sources use this; nothing on the GPU path does.  The tree
is taken from AFEPACK_SOURCE, else from the read-only mount of the build
container; `source()` returns None where neither exists (the GPU machine).
"""
import os

_MOUNT = "/root/reference"


def source():
    for cand in (os.environ.get("AFEPACK_SOURCE"), _MOUNT):
        if cand and os.path.isdir(os.path.join(cand, "src")):
            return cand
    return None


def template_dir():
    s = source()
    return None if s is None else os.path.join(s, "include", "AFEPack", "template")
