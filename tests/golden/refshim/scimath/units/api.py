"""Identity stand-ins for scimath's unit machinery (fixture generation only)."""
import numpy as np


def has_units(func=None, **_kw):
    if func is None:
        return lambda f: f
    return func


def UnitScalar(value, units=None):  # noqa: N802 - mirrors the scimath name
    return float(value)


def UnitArray(value, units=None):  # noqa: N802
    return np.asarray(value)
