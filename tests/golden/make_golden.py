"""Regenerates the oracle golden fixtures (tests/golden/*.json).

    python tests/golden/make_golden.py

The fixture records, for the first steps of the 25-box tower workload with
merging on, a digest of the oracle's state after every step: contact count,
a weighted sum of the contact keys, the bits of the multiplier sum and of the
position sum, and the top-level list with collection members.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from adaptivemerging_gb300 import abi, scenes  # noqa: E402
from oracle_binding import Oracle  # noqa: E402
from test_oracle_cpu import _digest  # noqa: E402


def main():
    scene = {"n_boxes": 25, "seed": 1, "density": 1.0}
    prm = dict(gravity_amount=9.81, friction_override=1, friction=0.6, restitution_override=1,
               restitution=0.0, iterations=100)
    dt = 0.01
    o = Oracle(scenes.tower(**scene), abi.default_params(**prm))
    steps = []
    for _ in range(120):
        o.step(dt)
        steps.append(_digest(o))
    out = {"scene": scene, "params": prm, "dt": dt, "steps": steps,
           "counters": o.counters()}
    with open(os.path.join(HERE, "tower_c1.json"), "w") as f:
        json.dump(out, f, indent=0)
    print("merges", o.counters())


if __name__ == "__main__":
    main()
