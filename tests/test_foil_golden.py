"""The oracle on the reference's real flapping-foil frame (fixture made by
tests/golden/make_foil_golden.py from examples/data/flapping_foil_216000.bin)
against the numbers the reference prints for it (README.md:146-172): the
PCG iteration counts 8,450 and 11,150 and the four force terms per
direction to their printed digits."""
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "foil_frame_oracle.json")

# README.md:166-171 (x = drag direction, y = lift)
README_TERMS = {
    "x": [1.900e-2, -4.606e-2, 9.73e-4, -3.61e-4],
    "y": [-1.480e-1, 7.444e-1, 7.33e-3, 3.31e-3],
}
README_ITERS = {"x": 8450, "y": 11150}


@pytest.mark.parametrize("axis", ["x", "y"])
def test_foil_frame_oracle_matches_readme(axis):
    gold = json.load(open(GOLD))
    assert gold["nx"] == 600 and gold["ny"] == 1250 and gold["solid_cells"] == 3321
    d = [x for x in gold["directions"] if x["axis"] == axis][0]
    assert d["iterations"] == README_ITERS[axis]
    for got, ref in zip(d["terms"], README_TERMS[axis]):
        # significant figures as printed in the README
        sig = {1.900e-2: 4, -4.606e-2: 4, 9.73e-4: 3, -3.61e-4: 3, -1.480e-1: 4, 7.444e-1: 4, 7.33e-3: 3,
               3.31e-3: 3}[ref]
        assert f"{got:.{sig - 1}e}" == f"{ref:.{sig - 1}e}", (axis, got, ref)
