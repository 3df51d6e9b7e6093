"""Shared parity helpers: run the device path and the oracle side by side."""
import numpy as np

from adaptivemerging_gb300 import abi

DT = 0.01


def params(**over):
    base = dict(gravity_amount=9.81, friction_override=1, friction=0.6, restitution_override=1,
                restitution=0.0, iterations=100, enable_merging=0)
    base.update(over)
    return abi.default_params(**base)


def first_diff(a, b):
    a = np.asarray(a); b = np.asarray(b)
    if a.shape != b.shape:
        return f"shape {a.shape} vs {b.shape}"
    bad = np.argwhere(~((a == b) | (np.isnan(a) & np.isnan(b))) if a.dtype.kind == "f" else (a != b))
    if len(bad) == 0:
        return None
    i = tuple(bad[0])
    return f"first mismatch at {i}: {a[i]!r} vs {b[i]!r} ({len(bad)} entries differ)"


def compare_contacts(cg, co, fields=("body1", "body2", "bv1", "bv2", "info", "frame", "jac", "violation",
                                     "lambda", "state", "fresh")):
    for f in fields:
        d = first_diff(cg[f], co[f])
        if d:
            return f"{f}: {d}"
    return None


def compare_bodies(bg, bo, fields=("x", "R", "v", "omega", "sleeping")):
    for f in fields:
        d = first_diff(bg[f], bo[f])
        if d:
            return f"{f}: {d}"
    return None
