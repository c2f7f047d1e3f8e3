"""Textbook known answers of the reference's test/Physics/PhysicsValidation.jl
on the device: the propagator entry points (FP64) and whole problem
evaluations through the C ABI in both precisions (the mixed one takes the
register-resident d = 2 expm and the df state chain).
"""
import numpy as np
import pytest

from oracle import ref_semantics as rs
from test_oracle_kats import ECHO_DOMEGA, ECHO_T_FREE, RABI_OMEGA, SX, SZ, phys_echo, phys_rabi
from test_parity_gpu import to_gpu

pytestmark = pytest.mark.gpu

PSI0 = np.array([1, 0], complex)


def test_pi_pulses_and_not_gate_propagators(pg):           # :24-48, :104-106
    U = pg.compute_propagator(np.pi / 2 * SX, 1.0)
    out = U @ PSI0
    assert abs(out[0]) ** 2 < 1e-10 and abs(abs(out[1]) ** 2 - 1) < 1e-10
    assert abs(pg.gate_fidelity(U, SX) - 1.0) < 1e-10
    Uh = pg.compute_propagator(np.pi / 4 * SX, 1.0)
    out2 = Uh @ (Uh @ PSI0)
    assert abs(out2[0]) ** 2 < 1e-10 and abs(abs(out2[1]) ** 2 - 1) < 1e-10


@pytest.mark.parametrize("theta,p1", [(np.pi, 1.0), (2 * np.pi, 0.0), (np.pi / 2, 0.5)])
def test_rabi_propagators(pg, theta, p1):                   # :280-308
    U = pg.compute_propagator(RABI_OMEGA * SX / 2, theta / RABI_OMEGA)
    assert abs(abs((U @ PSI0)[1]) ** 2 - p1) < 1e-10


def test_spin_echo_propagator_stack(pg):                    # :50-73
    T = ECHO_T_FREE
    ref = None
    for dw in ECHO_DOMEGA:
        H = np.stack([np.pi / 4 / T * SX, dw * SZ, np.pi / 2 / T * SX, dw * SZ, np.pi / 4 / T * SX])
        props = pg.compute_propagators(H, T)
        Uo = rs.compute_propagators(H, T)
        assert np.max(np.abs(props - Uo)) < 1e-12
        U = pg.compute_total_propagator(props)
        assert np.max(np.abs(U - rs.compute_total_propagator(Uo))) < 1e-12
        pops = np.abs(U @ PSI0) ** 2
        if ref is None:
            ref = pops
        assert np.max(np.abs(pops - ref)) < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rabi_and_echo_problems(pg, precision):
    for theta, p1 in ((np.pi, 1.0), (2 * np.pi, 0.0), (np.pi / 2, 0.5)):
        prob, u = phys_rabi(theta)
        p = to_gpu(pg, prob, "exact", precision=precision)
        F, _ = p.eval(u)
        p.close()
        assert abs(F - p1) < 1e-10, (theta, F)
    F0 = None
    for dw in ECHO_DOMEGA:
        prob, u = phys_echo(dw)
        p = to_gpu(pg, prob, "exact", precision=precision)
        F, _ = p.eval(u)
        p.close()
        if F0 is None:
            F0 = F
            assert abs(F0) < 1e-10
        assert abs(F - F0) < 1e-6, (dw, F, F0)
