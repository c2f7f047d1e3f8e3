"""pgx_total_propagator_noalloc, the entry point for callers that cannot
allocate device memory (real-time loops that forbid allocation once started,
hosts whose device memory all belongs to their own pool allocator).  It must
give the same U_total as the regular entry point (pgx_total_propagator through
a problem) and as the oracle's product of slice exponentials, on two calls in
a row -- the second call reuses the static scratch the first one left behind --
and refuse sizes beyond its static scratch with a clear error.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest
import scipy.linalg as sla

from oracle import ref_semantics as rs

pytestmark = pytest.mark.gpu

TOL = 1e-12         # against the regular entry point (same Taylor method)
ORACLE_TOL = 1e-10  # against the oracle (eigendecomposition / Pade slice exponentials)


def _rand_herm(rng, d, s=1.0):
    A = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    return s * (A + A.conj().T) / 2


def _dev(torch, host: np.ndarray):
    return torch.tensor(np.ascontiguousarray(host).ravel(), dtype=torch.float64, device="cuda:0")


def _noalloc(pg, torch, dim, generator, gens, dt):
    """Call the entry point with device buffers the test owns."""
    A = pg._abi
    d_g = _dev(torch, A.cmat_buf(gens))
    d_dt = _dev(torch, np.asarray(dt, np.float64))
    d_U = torch.full((2 * dim * dim,), np.nan, dtype=torch.float64, device="cuda:0")
    err = C.create_string_buffer(256)
    st = A.lib().pgx_total_propagator_noalloc(dim, A.GEN[generator], len(dt), d_g.data_ptr(),
                                              d_dt.data_ptr(), d_U.data_ptr(), None, err, 256)
    torch.cuda.synchronize()
    return st, err.value.decode(), A.cmat_from_buf(d_U.cpu().numpy(), dim)


@pytest.mark.parametrize("dim,n_t,generator", [(2, 100, "hermitian"), (5, 37, "hermitian"),
                                               (16, 300, "hermitian"), (32, 64, "hermitian"),
                                               (64, 24, "liouvillian")])
def test_noalloc_matches_regular_entry_point_twice(pg, dim, n_t, generator):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(dim)
    Hd = _rand_herm(rng, dim)
    Hc = np.stack([_rand_herm(rng, dim), _rand_herm(rng, dim)])
    if generator == "liouvillian":   # a dissipative generator: -i[H,.] plus damping
        Hd = -1j * Hd - 0.05 * np.eye(dim)
        Hc = -1j * Hc
    dt = rng.uniform(0.02, 0.05, n_t) / np.sqrt(dim)
    prob = pg.Problem(Hd, Hc, dt, generator=generator, target="gate", target_op=np.eye(dim),
                      grad_mode="exact")
    for call in range(2):   # second call reuses whatever the first left in the scratch
        u = rng.uniform(-1, 1, (2, n_t))
        gens = Hd[None] + np.einsum("jk,jab->kab", u, Hc)
        st, msg, U = _noalloc(pg, torch, dim, generator, gens, dt)
        assert st == 0, msg
        U_ref = prob.total_propagator(u, 0)
        assert np.max(np.abs(U - U_ref)) <= TOL * max(1.0, np.max(np.abs(U_ref))), call
        # the oracle: U_total = U_{n-1} ... U_0 with eigendecomposition (Hermitian)
        # or Pade (Liouvillian) slice exponentials
        if generator == "hermitian":
            props = rs.compute_propagators(gens, dt)
        else:
            props = np.stack([sla.expm(gens[k] * dt[k]) for k in range(n_t)])
        U_or = rs.compute_total_propagator(props)
        assert np.max(np.abs(U - U_or)) <= ORACLE_TOL * max(1.0, np.max(np.abs(U_or))), call
    prob.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(pg):
    torch = pytest.importorskip("torch")
    dim, n_t = 64, 400                    # 400 x 64 KB > 16 MiB
    gens = np.zeros((1, dim, dim))
    A = pg._abi
    d_g = torch.zeros(2 * dim * dim, dtype=torch.float64, device="cuda:0")
    d_dt = torch.zeros(n_t, dtype=torch.float64, device="cuda:0")
    d_U = torch.zeros(2 * dim * dim, dtype=torch.float64, device="cuda:0")
    err = C.create_string_buffer(256)
    st = A.lib().pgx_total_propagator_noalloc(dim, 0, n_t, d_g.data_ptr(), d_dt.data_ptr(),
                                              d_U.data_ptr(), None, err, 256)
    assert st == 4   # PGX_ERR_BUDGET
    assert b"static scratch" in err.value
    del gens
