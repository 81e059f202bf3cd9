"""The oracle's frames for the seeded golden scenes match the committed
digests (tests/golden/frames.json, made by tests/golden/make_golden.py)."""
import hashlib
import json
import os

import pytest

from oracle import oracle
from tests.golden_scenes import GOLDEN_SCENES

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "frames.json")))


@pytest.mark.parametrize("name", sorted(GOLDEN_SCENES))
def test_oracle_matches_golden(oracle_lib, name):
    g = GOLDEN[name]
    rgba, z, tpf, st = oracle.draw_scene(GOLDEN_SCENES[name](), nthreads=2)
    assert st == 0
    assert tpf == g["tpf"]
    assert int((z > -1).sum()) == g["covered"]
    assert hashlib.sha256(rgba.tobytes()).hexdigest() == g["rgba_sha256"]
    assert hashlib.sha256(z.tobytes()).hexdigest() == g["z_sha256"]
