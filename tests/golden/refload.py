"""Import the reference's MC/tools modules in this container (fixture generation only).

The reference is read from /root/reference (read-only).  Missing third-party
modules are replaced by the stubs in tests/golden/refshim, and the two NumPy 2
renames the reference still uses (np.trapz, np.NaN) are aliased.  The
reference's table module configures logging to ../logs at import time, so the
working directory is switched to a scratch tree that has ../logs and
../tables/integration.
"""
import os
import sys
import tempfile

import numpy as np

REF_ROOT = "/root/reference"
HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    sys.dont_write_bytecode = True
    if not hasattr(np, "trapz"):
        np.trapz = np.trapezoid
    if not hasattr(np, "NaN"):
        np.NaN = np.nan
    shim = os.path.join(HERE, "refshim")
    if shim not in sys.path:
        sys.path.insert(0, shim)
    import quaternion  # noqa: F401  (registers np.quaternion)
    mc = os.path.join(REF_ROOT, "MC")
    if mc not in sys.path:
        sys.path.insert(0, mc)
    scratch = tempfile.mkdtemp(prefix="mcref_")
    for d in ("logs", "tables/integration", "run"):
        os.makedirs(os.path.join(scratch, d), exist_ok=True)
    os.chdir(os.path.join(scratch, "run"))
    import importlib
    mods = {}
    for name in ("parameters", "crossSections", "stoppingPowers", "extFunctions",
                 "material", "probTables", "scattering", "electron", "rotation",
                 "singleScatter", "multiScatter", "fileTools"):
        mods[name] = importlib.import_module("tools." + name)
    return mods, scratch
