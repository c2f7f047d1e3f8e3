"""The oracle against the committed golden fixtures (tests/golden/*.npz).

The fixtures freeze the oracle's (F, G) on small seeded problems of every
kind the path serves: state and gate targets, the three metrics, padded odd
dimensions, offset x B1 members, Liouvillian superoperators at D = 16 and 64.
The numpy oracle must reproduce them up to LAPACK rounding.  Where the C
restatement covers the case (Hermitian generators), it must reproduce them
too.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import make_golden  # noqa: E402

from oracle import members as mb  # noqa: E402

FIXTURES = sorted((Path(__file__).resolve().parent / "golden").glob("*.npz"))


def test_fixture_set_is_complete():
    names = {p.stem for p in FIXTURES}
    assert names == set(make_golden.cases().keys())


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: p.stem)
def test_oracle_reproduces_fixture(path):
    prob, u, modes, want = make_golden.load(path)
    for mode in modes:
        F, G = mb.eval_problem(prob, u, mode)
        Fw, Gw = want[mode]
        assert abs(F - Fw) <= 1e-13, (mode, F, Fw)
        assert np.max(np.abs(G - Gw)) <= 1e-12 * max(np.max(np.abs(Gw)), 1e-300), mode


@pytest.mark.parametrize("backend", ["lapack", "jacobi"])
@pytest.mark.parametrize("path", [p for p in FIXTURES if "lindblad" not in p.stem], ids=lambda p: p.stem)
def test_c_restatement_reproduces_fixture(path, backend):
    """Both arithmetic backends of the C restatement: LAPACK zheevr + BLAS zgemm
    (the reference's stack, used by the timed CPU baseline) and the built-in
    Jacobi eigensolver with plain loops."""
    from oracle import cpu_port
    if backend == "lapack" and not cpu_port.lapack_pointers():
        pytest.skip("SciPy's cython_lapack is not available")
    cpu_port.set_backend(backend)
    try:
        prob, u, modes, want = make_golden.load(path)
        for mode in modes:
            F, G = cpu_port.CpuProblem(prob, mode).eval(u, threads=2)
            Fw, Gw = want[mode]
            assert abs(F - Fw) <= 1e-12, (mode, F, Fw)
            assert np.max(np.abs(G - Gw)) <= 1e-10 * max(np.max(np.abs(Gw)), 1e-300), mode
    finally:
        cpu_port.set_backend("lapack" if cpu_port.lapack_pointers() else "jacobi")
