"""The per-step metrics CSV: the reference's columns, Java number format and
header-first behaviour (RigidBodySystem.exportDataToFile,
RigidBodySystem.java:495-542), checked on the host with a stand-in system."""
import numpy as np

from adaptivemerging_gb300 import abi
from adaptivemerging_gb300.csv_export import HEADER, CsvExporter, java_double


def test_java_double_format():
    cases = {0.0: "0.0", 1.0: "1.0", 0.5: "0.5", 0.001: "0.001", 0.00099: "9.9E-4", 1e-4: "1.0E-4",
             1.2345e-5: "1.2345E-5", 12.5: "12.5", 1234567.0: "1234567.0", 1e7: "1.0E7", 0.0123: "0.0123",
             2.5e-10: "2.5E-10", -0.25: "-0.25", 123456789.0: "1.23456789E8"}
    for v, s in cases.items():
        assert java_double(v) == s, (v, java_double(v), s)


def test_header_matches_reference_columns():
    assert HEADER == ["#bodies", "#contacts", "detection", "warmstart", "LCPSolve", "updateCollections",
                      "contactOrdering", "singleItPGS", "merging", "mergingBuild", "unmerging", "unmergingBuild",
                      "computeTime"]
    assert len(abi.PHASES) == abi.AM_NUM_PHASES == 11


class _Stand:
    def __init__(self):
        self.on = False
        self.k = 0

    def set_phase_timing(self, on):
        self.on = on

    def topology(self):
        return [0, (1, 2), 3]

    def num_contacts(self):
        return 7 + self.k

    def phase_times(self):
        self.k += 1
        return np.array([1e-4 * self.k] * 10 + [2e-3 * self.k])


def test_first_record_is_header_only(tmp_path):
    st = _Stand()
    ex = CsvExporter(st, "tower", merging=True, directory=str(tmp_path))
    assert st.on
    for _ in range(3):
        ex.record()
    ex.close()
    text = (tmp_path / "tower_merged.csv").read_text()
    lines = text.split("\n ")
    assert lines[0] == ", ".join(HEADER)
    rows = [l for l in lines[1:] if l]
    assert len(rows) == 2
    f = rows[0].split(", ")
    assert len(f) == 13 and f[0] == "3" and f[1] == "7" and f[2] == "1.0E-4" and f[12] == "0.002"
    ex2 = CsvExporter(_Stand(), "wall", merging=False, directory=str(tmp_path))
    ex2.record()
    ex2.close()
    assert (tmp_path / "wall.csv").exists()
