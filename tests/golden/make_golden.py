"""Regenerates tests/golden/frames.json: digests of oracle frames.

The reference has no golden vectors, so these fixtures pin the oracle itself
(its outputs for seeded scenes) against accidental change; the GPU tests
compare the CUDA path with the oracle directly.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests.golden_scenes import GOLDEN_SCENES  # noqa: E402
from oracle import oracle  # noqa: E402


def digest(a):
    return hashlib.sha256(a.tobytes()).hexdigest()


def main():
    oracle.build()
    out = {}
    for name, make in GOLDEN_SCENES.items():
        sc = make()
        rgba, z, tpf, st = oracle.draw_scene(sc, nthreads=4)
        assert st == 0, (name, st)
        out[name] = {"rgba_sha256": digest(rgba), "z_sha256": digest(z), "tpf": tpf,
                     "covered": int((z > -1).sum()), "width": sc.width, "height": sc.height}
        print(name, out[name]["tpf"], out[name]["covered"])
    with open(os.path.join(HERE, "frames.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
