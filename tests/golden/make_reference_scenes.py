"""Regenerates tests/golden/reference_scenes.json from the reference's own
scene files.

    python tests/golden/make_reference_scenes.py [reference project root]

Two of the reference's XML scenes, `scenes3D/tower30.xml` (135 boxes in a
ring tower on a plane) and `scenes3D/denseTower25.xml` (78 boxes), are parsed
by this repository's loader (adaptivemerging_gb300.scene_xml) and stored as
the loader's output: the am_scene arrays, the am_params fields the scene sets,
and the body names.  A third, "meshes", is `scenes3D/allBodyTypes.xml`
without its first body (a platform hung on four springs, which this
implementation does not model): two boxes, a sphere, a plane and four mesh
bodies whose sphere trees come from the reference's `data/*.sph` files and
whose mass properties come from its `data/*.obj` meshes.  Two more,
`scenes3D/seesaw.xml` and `scenes3D/chariot.xml`, hold composite bodies
(RigidBodyGeomComposite) without springs; their arrays include the
composite sub-bodies (am_scene's sub_* arrays), which only the oracle steps so far.  The reference tree is not present where the GPU tests
run, so the tests read this fixture instead of the XML files.  The first rows
(#bodies, #contacts) of the reference's recorded metrics for tower30
(`scenes3D/csv/conditional_acceptance_revisions/tower30_merged.csv`, and an
earlier run's `scenes3D/csv/old/tower30_merged.csv`) are kept beside them as
recorded.
"""
import csv
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from adaptivemerging_gb300 import abi, scene_xml  # noqa: E402

SCENES = ("tower30", "denseTower25")
COMPOSITE_SCENES = ("seesaw", "chariot")   # composites without springs
MESHES_FROM = "allBodyTypes"
CSV = "scenes3D/csv/conditional_acceptance_revisions/tower30_merged.csv"
CSV_OLD = "scenes3D/csv/old/tower30_merged.csv"


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    out = {"source": "reference scenes3D/*.xml parsed by adaptivemerging_gb300.scene_xml", "scenes": {}}
    for name in SCENES:
        sc, P, names = scene_xml.load(os.path.join(root, "scenes3D", name + ".xml"))
        arrays = {k: v.tolist() for k, v in sc.a.items()}
        prm = {f: getattr(P, f) for f, _ in abi.am_params._fields_}
        out["scenes"][name] = {"arrays": arrays, "params": prm, "names": names}
    with open(os.path.join(root, "scenes3D", MESHES_FROM + ".xml")) as f:
        doc = f.read()
    doc = re.sub(r'<body type="box" name="platform".*?</body>', "", doc, count=1, flags=re.S)
    sc, P, names = scene_xml.load(doc, data_root=root)
    out["scenes"]["meshes"] = {"arrays": {k: v.tolist() for k, v in sc.a.items()},
                               "params": {f: getattr(P, f) for f, _ in abi.am_params._fields_}, "names": names}
    for name in COMPOSITE_SCENES:
        sc, P, names = scene_xml.load(os.path.join(root, "scenes3D", name + ".xml"), composites=True)
        out["scenes"][name] = {"arrays": {k: v.tolist() for k, v in sc.a.items()},
                               "params": {f: getattr(P, f) for f, _ in abi.am_params._fields_}, "names": names}
    with open(os.path.join(root, CSV)) as f:
        rows = list(csv.reader(f))[1:]
    out["tower30_csv_bodies_contacts"] = [[int(r[0]), int(r[1])] for r in rows[:60] if len(r) > 2]
    with open(os.path.join(root, CSV_OLD)) as f:
        rows = list(csv.reader(f))[1:]
    out["tower30_old_csv_bodies_contacts"] = [[int(r[0]), int(r[1])] for r in rows[:20] if len(r) > 2]
    with open(os.path.join(HERE, "reference_scenes.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
