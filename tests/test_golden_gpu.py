"""The CUDA path against the committed golden fixtures (tests/golden/*.npz).

FP64 path: |dF| <= 1e-10, max|dG| / max|G| <= 1e-8 for every gradient mode.
Mixed path (gate targets): |dF| <= 1e-8, max|dG| / max|G| <= 1e-4.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import make_golden  # noqa: E402

from test_parity_gpu import to_gpu  # noqa: E402

pytestmark = pytest.mark.gpu

FIXTURES = sorted((Path(__file__).resolve().parent / "golden").glob("*.npz"))


def _check(F, G, Fw, Gw, ftol, grtol):
    assert abs(F - Fw) <= ftol, (F, Fw, abs(F - Fw))
    err = np.max(np.abs(G - Gw)) / max(np.max(np.abs(Gw)), 1e-300)
    assert err <= grtol, err


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: p.stem)
def test_fp64_path_matches_fixture(pg, path):
    prob, u, modes, want = make_golden.load(path)
    for mode in modes:
        p = to_gpu(pg, prob, mode, "fp64")
        F, G = p.eval(u)
        p.close()
        _check(F, G, *want[mode], 1e-10, 1e-8)


@pytest.mark.parametrize("path", [p for p in FIXTURES if "quickstart" not in p.stem and "states" not in p.stem],
                         ids=lambda p: p.stem)
def test_mixed_path_matches_fixture(pg, path):
    prob, u, modes, want = make_golden.load(path)
    for mode in modes:
        p = to_gpu(pg, prob, mode, "mixed")
        F, G = p.eval(u)
        p.close()
        _check(F, G, *want[mode], 1e-8, 1e-4)
