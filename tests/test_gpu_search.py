"""The weight-bounded search with its probes answered in waves by the device completion table:
the reference's own search distances (tests/golden/search.json) and known code distances."""
import json
import os

import pytest

from helpers import ROOT
from tropidist_gb300 import search
from tropidist_gb300.problem import Problem

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(ROOT, "tests", "golden", "search.json")))
CODES = json.load(open(os.path.join(ROOT, "tests", "golden", "codes.json")))


def test_reference_search_distances_on_device():
    for c in GOLD:
        p = Problem("g", c["m"], c["nobs"], c["h"], c["l"], [(i, 0) for i in range(c["m"])])
        for wave in (3, 1 << 16):
            r = search.distance(p, k_table=c["k_table"], kmax=c["kmax"], wave=wave)
            assert r["distance"] == c["distance"] and r["lower_bound"] == c["lower_bound"]
            for s in r["solutions"]:
                syn, lg = p.check(list(s))
                assert syn == 0 and lg != 0


@pytest.mark.parametrize("name", ["bb72_Z", "surface_d9_Z", "surface_d15_Z"])
def test_known_code_distances_on_device(name):
    c = next(x for x in CODES if x["name"] == name)
    h = [int(x, 16) if isinstance(x, str) else int(x) for x in c["h"]]
    l = [int(x, 16) if isinstance(x, str) else int(x) for x in c["l"]]
    p = Problem(name, c["nrows"], c["nobs"], h, l, [(i, 0) for i in range(c["nrows"])])
    r = search.distance(p, k_table=2, kmax=c["distance"])
    assert r["distance"] == c["distance"]
