"""Import the reference's MC/tools modules in this container (fixture generation only).

The reference checkout is named by the MCD_REFERENCE_ROOT environment
variable (the directory holding MC/tools).  Missing third-party
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

HERE = os.path.dirname(os.path.abspath(__file__))


def ref_root():
    root = os.environ.get("MCD_REFERENCE_ROOT")
    if not root or not os.path.isdir(os.path.join(root, "MC", "tools")):
        raise RuntimeError("set MCD_REFERENCE_ROOT to a checkout of the reference (the directory holding "
                           "MC/tools)")
    return root


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
    mc = os.path.join(ref_root(), "MC")
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
