import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def golden():
    class G:
        boys = json.loads((GOLDEN / "boys.json").read_text())
        m8 = json.loads((GOLDEN / "primitive_eri_m8.json").read_text())
        cholesky = json.loads((GOLDEN / "cholesky.json").read_text())
        blocks = dict(np.load(GOLDEN / "eri_blocks.npz"))
        nuclear = dict(np.load(GOLDEN / "nuclear.npz"))
        derivatives = dict(np.load(GOLDEN / "derivatives.npz"))
        contraction = dict(np.load(GOLDEN / "contraction.npz"))

    return G


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    return O.Oracle()


def derivative_systems(g):
    """(name, shell specs, quartets) of the centre-derivative fixture."""
    from oracle import oracle as O

    out = []
    for name in ("molecule3", "hand"):
        specs = [O.ShellSpec(tuple(d["center"]), d["l"], d["exponents"], d["coefficients"], d["normalize"])
                 for d in json.loads(str(g[f"{name}_shells"]))]
        out.append((name, specs, g[f"{name}_quartets"]))
    return out


def contraction_setup():
    """Systems and closed-form densities of the contraction fixture."""
    sys.path.insert(0, str(GOLDEN))
    import make_golden as mg

    return mg
