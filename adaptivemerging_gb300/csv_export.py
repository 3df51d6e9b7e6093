"""Per-step metrics CSV with the reference's columns and format
(RigidBodySystem.exportDataToFile, RigidBodySystem.java:495-542).

The reference opens `<scene>_merged.csv` (merging on) or `<scene>.csv`, and
its first call writes only the header; every later call appends one row for
the step just taken, so row k of the file is step k + 1.  Values are printed
with Java's Double.toString and separated by ", "; every line after the
header starts with a space (the reference prints "\\n " after each line).

    exporter = CsvExporter(system, "tower25", merging=True)
    for _ in range(n):
        system.step(dt)
        exporter.record()
    exporter.close()

`system` is a native.System or native.BatchSystem; phase timing is switched
on for it.  "#bodies" counts top-level bodies (a collection counts once, as
RigidBodySystem.bodies does) and "#contacts" the contacts of the step.
"""
import decimal
import math
import os

from . import abi

HEADER = ["#bodies", "#contacts"] + list(abi.PHASES)


def java_double(x):
    """Java's Double.toString: shortest round-trip digits; plain decimal for
    1e-3 <= |x| < 1e7 (at least one digit after the point), otherwise
    computerized scientific notation d.dddE<n>."""
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "Infinity" if x > 0 else "-Infinity"
    if x == 0.0:
        return "-0.0" if math.copysign(1.0, x) < 0 else "0.0"
    a = abs(x)
    sign = "-" if x < 0 else ""
    digits, exp = _shortest(a)
    if 1e-3 <= a < 1e7:
        point = exp + 1                          # digits before the decimal point
        if point <= 0:
            s = "0." + "0" * (-point) + digits
        elif point >= len(digits):
            s = digits + "0" * (point - len(digits)) + ".0"
        else:
            s = digits[:point] + "." + digits[point:]
        return sign + s
    mant = digits[0] + "." + (digits[1:] if len(digits) > 1 else "0")
    return f"{sign}{mant}E{exp}"


def _shortest(a):
    """Shortest round-trip decimal digits of a > 0 (as repr) and the decimal
    exponent of the first digit: a = d1.d2d3... x 10^exp."""
    t = decimal.Decimal(repr(a)).normalize().as_tuple()
    digits = "".join(str(d) for d in t.digits)
    return digits, len(digits) + t.exponent - 1


class CsvExporter:
    def __init__(self, system, scene_name, merging, directory="."):
        name = f"{scene_name}_merged.csv" if merging else f"{scene_name}.csv"
        self.path = os.path.join(directory, name)
        self.system = system
        self.system.set_phase_timing(True)
        self._f = None

    def record(self):
        """One call after each step: the first writes the header, the others a
        row for the step just taken."""
        if self._f is None:
            self._f = open(self.path, "w")
            self._f.write(", ".join(HEADER) + "\n ")
            return
        n_bodies = len(self.system.topology())
        n_contacts = self.system.num_contacts()
        t = self.system.phase_times()
        row = [str(n_bodies), str(n_contacts)] + [java_double(v) for v in t]
        self._f.write(", ".join(row) + "\n ")

    def close(self):
        if self._f is not None:
            self._f.close()
            self._f = None
