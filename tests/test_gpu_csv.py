"""Per-phase step times and the metrics CSV on the device path (the
reference's RigidBodySystem.exportDataToFile columns)."""
import numpy as np
import pytest

from adaptivemerging_gb300 import abi, scenes
from adaptivemerging_gb300.csv_export import HEADER, CsvExporter
from helpers import params

pytestmark = pytest.mark.gpu


def test_phase_times_and_csv_with_merging(gpu_lib, tmp_path):
    """A tower with merging on: every row has the 13 columns; the step's wall
    time covers its timed phases; merge steps show collection building; the
    body count drops as collections form; results equal an untimed run."""
    from adaptivemerging_gb300 import native
    sc = scenes.tower(12, seed=4, density=1.0)
    P = params(enable_merging=1, friction=0.6, iterations=60)
    g = native.System(sc, P)
    ref = native.System(sc, P)
    ex = CsvExporter(g, "tower12", merging=True, directory=str(tmp_path))
    ex.record()
    rows = []
    for _ in range(160):
        g.step(0.01)
        ref.step(0.01)
        ex.record()
        rows.append(g.phase_times())
    ex.close()
    t = np.array(rows)
    assert (t >= 0).all()
    main = t[:, [abi.PHASES.index(k) for k in ("detection", "warmstart", "LCPSolve", "updateCollections",
                                               "merging", "unmerging")]].sum(axis=1)
    assert (t[:, abi.PHASES.index("computeTime")] >= main).all()
    assert (t[:, abi.PHASES.index("detection")] > 0).all() and (t[:, abi.PHASES.index("LCPSolve")] > 0).all()
    assert (t[:, abi.PHASES.index("mergingBuild")] > 0).any()
    assert (t[:, abi.PHASES.index("contactOrdering")] <= t[:, abi.PHASES.index("updateCollections")]).all()
    assert np.array_equal(g.bodies()["x"], ref.bodies()["x"])     # timing changes nothing
    lines = (tmp_path / "tower12_merged.csv").read_text().split("\n ")
    assert lines[0] == ", ".join(HEADER)
    data = [l.split(", ") for l in lines[1:] if l]
    assert len(data) == 160 and all(len(r) == 13 for r in data)
    nb = [int(r[0]) for r in data]
    assert nb[0] == sc.n and min(nb) < sc.n


def test_phase_times_batched(gpu_lib):
    """Batched steps time detection, warm start and the solve; the collection
    phases stay 0 (merging is off in batched mode)."""
    from adaptivemerging_gb300 import native
    sc = [scenes.bin_scene(n, 40 + n, gap=-0.001) for n in (30, 80)]
    g = native.BatchSystem(sc, params(friction_override=0, iterations=2000), threads=0, residual_target=1e-6,
                           check_every=10)
    g.set_phase_timing(True)
    for _ in range(3):
        g.step(0.005)
    t = g.phase_times()
    for k in ("detection", "warmstart", "LCPSolve", "computeTime"):
        assert t[abi.PHASES.index(k)] > 0, k
    for k in ("updateCollections", "contactOrdering", "singleItPGS", "mergingBuild", "unmergingBuild"):
        assert t[abi.PHASES.index(k)] == 0, k
    g.set_phase_timing(False)
    g.step(0.005)
    assert (g.phase_times() == 0).all()
