"""CPU checker for the GB300 mobility library.  TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this package.  The product library never links, calls or
falls back to anything here.
"""

import os as _os


def reference_dir() -> str:
    """The reference source tree the CPU checker builds from: the directory
    named by GMI_REFERENCE_DIR, else a directory called ``reference`` next
    to this repository's root.  The path may not exist (the GPU machine has no
    reference tree); callers check for the files they need."""
    env = _os.environ.get("GMI_REFERENCE_DIR")
    if env:
        return env
    repo = _os.path.dirname(_os.path.dirname(_os.path.abspath(__file__)))
    return _os.path.join(_os.path.dirname(repo), "reference")
