"""Loader of the golden fixtures written by tests/golden/gen_golden.py."""
import json
import os

import numpy as np

from tests.golden.gen_golden import mp_from, params_from  # noqa: F401

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(fname):
    z = np.load(os.path.join(GOLDEN, fname), allow_pickle=False)
    n = int(z["ncases"])
    cases = []
    for i in range(n):
        pre = f"{i}:"
        c = {k[len(pre):]: z[k] for k in z.files if k.startswith(pre)}
        for k in ("name", "kind", "params", "minimiser"):
            if k in c:
                c[k] = str(c[k])
        c["params_kw"] = json.loads(c["params"])
        if "minimiser" in c:
            c["minimiser_kw"] = json.loads(c["minimiser"])
        cases.append(c)
    return cases


def case_ids(cases):
    return [f'{c["kind"]}-{c["name"]}' for c in cases]
