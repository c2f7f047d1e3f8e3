"""Checkpoint blobs without a GPU: the C codec (pgx_checkpoint_create /
_parse / _set_metadata, host code only) against an independent restatement
of the documented byte layout in this file, corruption detection, the
problem fingerprint, and the Python mirror of IO/Checkpoint.jl (save / load /
list / summary / compatible, CheckpointHierarchyTests.jl and the
checkpoint block of EndToEndTests.jl:108-130)."""
import os
import struct

import numpy as np
import pytest

HEADER = 208
MAGIC = b"PGXCKPT\0"


def fnv1a64(data: bytes) -> int:
    h = 0xcbf29ce484222325
    for b in data:
        h = ((h ^ b) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return h


OPT_I = ("method", "max_iter", "adapt_step_size", "lbfgs_memory")
OPT_F = ("convergence_tol", "step_size", "min_step_size", "max_step_size", "gradient_norm_tol",
         "amplitude_limit", "l_bound", "u_bound")


def py_encode(f: dict) -> bytes:
    """Writer of the layout documented in include/pgx.h / pgx_checkpoint.cpp."""
    n = f["n_controls"] * f["n_timesteps"]
    hdr = MAGIC + struct.pack("<II", 1, HEADER)
    hdr += struct.pack("<14i", f["flags"], f["system_dim"], f["n_controls"], f["n_timesteps"], f["n_members"],
                       f["iteration"], len(f["fh"]), len(f["gh"]), f["prior_iteration"], f["prior_history_len"],
                       f["prior_gnorm_len"], f["pairs"], f["round"], f["step_iter"])
    hdr += struct.pack("<dddQ", f["F_opt"], f["F"], f["timestamp"], f["fingerprint"])
    hdr += struct.pack("<4i", *[f["opt"][k] for k in OPT_I])
    hdr += struct.pack("<8d", *[f["opt"][k] for k in OPT_F])
    hdr += struct.pack("<dd", f["step"], f["F_prev"])
    arrays = [f["w"], f["fh"], f["gh"]] + ([f["u"], f["g"]] if f["flags"] & 1 else []) + \
             ([f["rho"], f["S"], f["Y"]] if f["flags"] & 1 and f["opt"]["method"] == 1 else [])
    payload = b"".join(np.asarray(a, "<f8").tobytes() for a in arrays)
    assert len(f["w"]) == n
    hdr += struct.pack("<Q", len(payload))
    assert len(hdr) == HEADER
    body = hdr + payload + struct.pack("<Q", len(f["meta"])) + f["meta"]
    return body + struct.pack("<Q", fnv1a64(body))


def py_decode(b: bytes) -> dict:
    assert b[:8] == MAGIC
    version, hb = struct.unpack_from("<II", b, 8)
    assert (version, hb) == (1, HEADER)
    (flags, sdim, nc, nt, nm, it, nf, ng, piter, pf, pg_, pairs, rnd, siter) = struct.unpack_from("<14i", b, 16)
    F_opt, F, ts, fp = struct.unpack_from("<dddQ", b, 72)
    opt = dict(zip(OPT_I, struct.unpack_from("<4i", b, 104)))
    opt.update(zip(OPT_F, struct.unpack_from("<8d", b, 120)))
    step, F_prev = struct.unpack_from("<dd", b, 184)
    (payload,) = struct.unpack_from("<Q", b, 200)
    (ck,) = struct.unpack_from("<Q", b, len(b) - 8)
    assert ck == fnv1a64(b[:-8])
    n = nc * nt
    pos = HEADER

    def take(k):
        nonlocal pos
        a = np.frombuffer(b, "<f8", count=k, offset=pos).astype(np.float64)
        pos += 8 * k
        return a

    out = dict(flags=flags, system_dim=sdim, n_controls=nc, n_timesteps=nt, n_members=nm, iteration=it,
               prior_iteration=piter, prior_history_len=pf, prior_gnorm_len=pg_, pairs=pairs, round=rnd,
               step_iter=siter, F_opt=F_opt, F=F, timestamp=ts, fingerprint=fp, opt=opt, step=step, F_prev=F_prev)
    out["w"], out["fh"], out["gh"] = take(n), take(nf), take(ng)
    if flags & 1:
        out["u"], out["g"] = take(n), take(n)
        if opt["method"] == 1:
            out["rho"], out["S"], out["Y"] = take(pairs), take(pairs * n), take(pairs * n)
    assert pos == HEADER + payload
    (m,) = struct.unpack_from("<Q", b, pos)
    out["meta"] = b[pos + 8:pos + 8 + m]
    assert pos + 16 + m == len(b)
    return out


def _opt(method=0, **kw):
    o = dict(method=method, max_iter=100, adapt_step_size=1, lbfgs_memory=10, convergence_tol=1e-8, step_size=0.01,
             min_step_size=1e-10, max_step_size=10.0, gradient_norm_tol=1e-6, amplitude_limit=float("inf"),
             l_bound=-1.0, u_bound=1.0)
    o.update(kw)
    return o


def test_c_writer_matches_the_documented_layout(pg):
    rng = np.random.default_rng(1)
    w = rng.normal(size=(3, 11))
    fh, gh = rng.random(9).tolist(), rng.random(8).tolist()
    blob = pg.checkpoint_create(w, 0.8125, iteration=8, fidelity_history=fh, gradient_norm_history=gh,
                                system_dim=4, n_members=6, converged=True, timestamp=1.5e9, fingerprint=0xDEADBEEF,
                                method="ensemble_lbfgs", opt={"max_iter": 77, "lbfgs_memory": 5},
                                metadata=b'{"k": 1}')
    d = py_decode(blob)
    assert d["flags"] == 2 and d["system_dim"] == 4 and d["n_members"] == 6 and d["iteration"] == 8
    assert (d["n_controls"], d["n_timesteps"]) == (3, 11)
    assert d["F_opt"] == 0.8125 and d["timestamp"] == 1.5e9 and d["fingerprint"] == 0xDEADBEEF
    assert d["opt"]["method"] == 1 and d["opt"]["max_iter"] == 77 and d["opt"]["lbfgs_memory"] == 5
    assert np.array_equal(d["w"], w.T.ravel())          # column-major [n_c x n_t]
    assert d["fh"].tolist() == fh and d["gh"].tolist() == gh
    assert d["meta"] == b'{"k": 1}'
    # the Python writer of the same fields gives the same bytes
    f = dict(d, fh=list(d["fh"]), gh=list(d["gh"]))
    assert py_encode(f) == blob


def test_c_reader_reads_an_exact_lbfgs_blob_written_from_the_spec(pg):
    rng = np.random.default_rng(2)
    nc, nt, pairs = 2, 5, 3
    n = nc * nt
    f = dict(flags=1, system_dim=4, n_controls=nc, n_timesteps=nt, n_members=2, iteration=12, prior_iteration=4,
             prior_history_len=5, prior_gnorm_len=4, pairs=pairs, round=9, step_iter=0, F_opt=0.75, F=0.7,
             timestamp=1.7e9, fingerprint=12345, opt=_opt(1, lbfgs_memory=4), step=0.0, F_prev=0.0,
             w=rng.normal(size=n), fh=rng.random(13).tolist(), gh=rng.random(11).tolist(), u=rng.normal(size=n),
             g=rng.normal(size=n), rho=rng.random(pairs), S=rng.normal(size=pairs * n), Y=rng.normal(size=pairs * n),
             meta=b"")
    blob = py_encode(f)
    d = pg.checkpoint_parse(blob)
    assert d["exact"] and d["lbfgs_pairs"] == pairs and d["iteration"] == 12 and d["F"] == 0.7
    assert np.array_equal(d["w_opt"], f["w"].reshape(nt, nc).T)
    assert d["fidelity_history"] == f["fh"] and d["gradient_norm_history"] == f["gh"]
    assert d["optimizer"]["method"] == "ensemble_lbfgs" and d["optimizer"]["lbfgs_memory"] == 4
    # re-wrapping the metadata keeps every other byte of the payload
    b2 = pg.checkpoint_set_metadata(blob, b'{"note": "x"}')
    d2 = py_decode(b2)
    assert d2["meta"] == b'{"note": "x"}'
    for k in ("u", "g", "rho", "S", "Y", "w"):
        assert np.array_equal(d2[k], np.asarray(f[k])), k
    assert d2["round"] == 9 and d2["prior_history_len"] == 5 and d2["fingerprint"] == 12345


@pytest.mark.parametrize("damage", ["flip_payload", "flip_header", "truncate", "magic", "version", "extra"])
def test_corrupted_blobs_are_refused(pg, damage):
    w = np.arange(6.0).reshape(2, 3)
    blob = bytearray(pg.checkpoint_create(w, 0.5, fidelity_history=[0.1, 0.5], system_dim=2))
    if damage == "flip_payload":
        blob[HEADER + 3] ^= 0x10
    elif damage == "flip_header":
        blob[36] ^= 0x01                      # iteration
    elif damage == "truncate":
        blob = blob[:-9]
    elif damage == "magic":
        blob[0:8] = b"PGXCKPX\0"
    elif damage == "version":                 # a consistent blob of an unknown version
        blob[8:12] = struct.pack("<I", 2)
        blob[-8:] = struct.pack("<Q", fnv1a64(bytes(blob[:-8])))
    else:
        blob += b"\0"
    with pytest.raises(pg._abi.PgxError) as e:
        pg.checkpoint_parse(bytes(blob))
    assert e.value.status == 1


def test_inconsistent_header_with_valid_checksum_is_refused(pg):
    """A well-formed checksum does not make a blob valid: sizes must agree."""
    w = np.zeros((2, 3))
    d = py_decode(pg.checkpoint_create(w, 0.5, fidelity_history=[0.5]))
    d["prior_history_len"] = 2                # more prior entries than history
    with pytest.raises(pg._abi.PgxError):
        pg.checkpoint_parse(py_encode(dict(d, fh=list(d["fh"]), gh=list(d["gh"]))))
    d["prior_history_len"] = 0
    d["pairs"] = 2                            # pairs in a non-exact blob
    with pytest.raises(pg._abi.PgxError):
        pg.checkpoint_parse(py_encode(dict(d, fh=list(d["fh"]), gh=list(d["gh"]))))


def test_create_refuses_exact_flag_and_bad_sizes(pg):
    A = pg._abi
    import ctypes as C
    info = A.CheckpointInfo()
    info.struct_size = C.sizeof(A.CheckpointInfo)
    info.n_controls, info.n_timesteps, info.flags = 1, 2, A.CKPT_EXACT
    info.opt = pg.opt_desc("grape")
    w = np.zeros(2)
    n = C.c_uint64()
    assert A.lib().pgx_checkpoint_create(C.byref(info), A.as_dptr(w), None, None, None, None, 0, C.byref(n)) == 1
    info.flags = 0
    info.history_len = 3                      # history without a buffer
    assert A.lib().pgx_checkpoint_create(C.byref(info), A.as_dptr(w), None, None, None, None, 0, C.byref(n)) == 1
    info.history_len = 0
    assert A.lib().pgx_checkpoint_create(C.byref(info), A.as_dptr(w), None, None, None, None, 0, C.byref(n)) == 0
    small = C.create_string_buffer(16)
    assert A.lib().pgx_checkpoint_create(C.byref(info), A.as_dptr(w), None, None, None, small, 16,
                                         C.byref(n)) == 2


def test_problem_fingerprint_tracks_the_problem(pg):
    from pulsar_gb300 import workloads as W
    spec, _ = W.spin4_ensemble(n_t=6, n_off=2, n_b1=2)
    kw = dict(spec.problem_kwargs())
    f0 = pg.problem_fingerprint(**kw)
    assert f0 == pg.problem_fingerprint(**dict(kw, dt=spec.dt.copy()))
    dt2 = spec.dt.copy()
    dt2[3] = np.nextafter(dt2[3], 1.0)
    assert pg.problem_fingerprint(**dict(kw, dt=dt2)) != f0
    assert pg.problem_fingerprint(**dict(kw, precision="mixed")) != f0


def test_checkpoint_round_trip_like_the_reference(pg, tmp_path):
    """CheckpointHierarchyTests.jl 'Round-trip' and 'Kwargs constructor'."""
    rng = np.random.default_rng(3)
    w = rng.normal(size=(2, 50))
    c0 = pg.Checkpoint(w, 0.987, 2, 50)
    assert c0.iteration == 0 and not c0.fidelity_history and not c0.optimizer_state and c0.system_dim == 0
    assert c0.domain == "generic" and c0.system_kind == "generic" and isinstance(c0.metadata, dict)
    assert pg.checkpoint_compatible(c0, 2, 50) and not pg.checkpoint_compatible(c0, 3, 50)
    fh = list(np.linspace(0.5, 0.987, 20))
    gn = list(np.linspace(0.2, 0.001, 20))
    c = pg.Checkpoint(w, 0.987, 2, 50, iteration=200, fidelity_history=fh, gradient_norm_history=gn,
                      optimizer_state={"method": "lbfgs"}, system_dim=4, domain="qc", drive_max_hz=200e6,
                      T_pulse=5e-8, system_kind="transmon", metadata={"note": "test", "dt": 1e-8})
    fp = tmp_path / "a.ckpt"
    pg.save_checkpoint(str(fp), c)
    assert not (tmp_path / "a.ckpt.tmp").exists()
    L = pg.load_checkpoint(str(fp))
    assert np.array_equal(L.w_opt, w) and L.F_opt == 0.987 and (L.n_controls, L.n_timesteps) == (2, 50)
    assert L.iteration == 200 and L.fidelity_history == fh and L.gradient_norm_history == gn
    assert L.optimizer_state["method"] == "lbfgs" and L.system_dim == 4 and L.domain == "qc"
    assert L.drive_max_hz == 200e6 and L.T_pulse == 5e-8 and L.system_kind == "transmon"
    assert L.metadata == {"note": "test", "dt": 1e-8} and L.timestamp == c.timestamp
    # an unchanged load re-saves to the same bytes
    assert L.to_bytes() == fp.read_bytes()
    # editing a field re-encodes it
    L.F_opt = 0.5
    assert pg.Checkpoint.from_bytes(L.to_bytes()).F_opt == 0.5


def test_load_missing_or_foreign_file(pg, tmp_path):
    with pytest.raises(ValueError):
        pg.load_checkpoint(str(tmp_path / "missing.ckpt"))
    bad = tmp_path / "junk.ckpt"
    bad.write_bytes(b"not a checkpoint at all" * 20)
    with pytest.raises(ValueError):
        pg.load_checkpoint(str(bad))
    assert pg.checkpoint_summary(str(bad)).startswith("Could not read checkpoint")
    assert pg.checkpoint_summary(str(tmp_path / "nope.ckpt")).startswith("File not found")


def test_list_checkpoints_and_summary(pg, tmp_path):
    c = pg.Checkpoint(np.zeros((2, 50)), 0.987, 2, 50, iteration=7)
    pg.save_checkpoint(str(tmp_path / "b.ckpt"), c)
    pg.save_checkpoint(str(tmp_path / "a.jls"), c)      # the reference's naming keeps working
    (tmp_path / "notes.txt").write_text("x")
    files = pg.list_checkpoints(str(tmp_path))
    assert [os.path.basename(f) for f in files] == ["a.jls", "b.ckpt"]
    s = pg.checkpoint_summary(files[1])
    assert s.startswith("b.ckpt | iter=7 | F=0.987000 | saved ")
    assert pg.list_checkpoints(str(tmp_path / "absent")) == []


def test_auto_checkpoint_callback(pg, tmp_path):
    sysm = pg.quantum_system(np.diag([1.0, -1.0]).astype(complex), [np.array([[0, 1], [1, 0]], complex)])
    cb = pg.auto_checkpoint_callback(str(tmp_path / "auto.ckpt"), 5)
    cb(3, np.ones((1, 4)), 0.5, 0.1, sysm)
    assert not (tmp_path / "auto.ckpt").exists()
    cb(10, np.ones((1, 4)), 0.6, 0.2, sysm)
    L = pg.load_checkpoint(str(tmp_path / "auto.ckpt"))
    assert L.iteration == 10 and L.fidelity_history == [0.6] and L.gradient_norm_history == [0.2]
    assert L.system_dim == 2 and L.metadata == {"callback_interval": 5}


def test_resume_validation_happens_before_any_device_work(pg):
    """resume_optimization's ArgumentErrors (Checkpoint.jl:236-247)."""
    X = np.array([[0, 1], [1, 0]], complex)
    sys2 = pg.quantum_system(np.diag([1.0, -1.0]).astype(complex), [X])
    tgt = pg.unitary_target(X)
    c = pg.Checkpoint(np.zeros((1, 8)), 0.5, 1, 8, system_dim=3)
    with pytest.raises(ValueError, match="dimension mismatch"):
        pg.resume_optimization(c, sys2, tgt, verbose=False)
    c = pg.Checkpoint(np.zeros((2, 8)), 0.5, 2, 8, system_dim=2)
    with pytest.raises(ValueError, match="n_controls mismatch"):
        pg.resume_optimization(c, sys2, tgt, verbose=False)
