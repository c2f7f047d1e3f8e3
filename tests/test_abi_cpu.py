"""C-ABI checks that need no GPU: the library loads, exports every symbol
include/pgx.h declares, and the ctypes mirror has the C struct layouts."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(pgx_\w+)\s*\(", txt, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("pgx_ctx_create", "pgx_problem_create", "pgx_eval", "pgx_eval_device",
                 "pgx_optimize", "pgx_propagator", "pgx_total_propagator"):
        assert must in names


def test_library_exports_every_declared_symbol(pg):
    lib = C.CDLL(str(pg.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert pg._abi.lib().pgx_abi_version() == 1
    assert pg._abi.lib().pgx_status_string(4) == b"HBM budget exceeded"


def test_ctypes_layout_matches_c(tmp_path, pg):
    A = pg._abi
    src = tmp_path / "layout.c"
    fields = {"pgx_problem_desc": A.ProblemDesc, "pgx_eval_stats": A.EvalStats,
              "pgx_opt_desc": A.OptDesc, "pgx_opt_result": A.OptResult,
              "pgx_server_desc": A.ServerDesc, "pgx_job_status": A.JobStatus,
              "pgx_serve_stats": A.ServeStats, "pgx_penalty": A.Penalty,
              "pgx_checkpoint_info": A.CheckpointInfo, "pgx_job_extras": A.JobExtras}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "pgx.h"', "int main(void){"]
    for cname, py in fields.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            a, b, c = ln.split()
            got[(a, b)] = int(c)
    for cname, py in fields.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_no_device_means_loud_failure(pg):
    """Without a GPU the product path raises; it never falls back to the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pg._abi.PgxError):
        pg.Context(0)


def test_c_oracle_matches_numpy_oracle():
    from oracle import cpu_port, members as mb
    import fx
    prob, u0 = fx.spin4_ensemble(n_t=12, n_off=2, n_b1=2)
    for mode in ("ref_grape", "ref_mr", "exact"):
        F, G = cpu_port.CpuProblem(prob, mode).eval(u0, threads=2)
        Fo, Go = mb.eval_problem(prob, u0, mode)
        assert abs(F - Fo) < 1e-13
        assert np.max(np.abs(G - Go)) < 1e-11 * np.max(np.abs(Go))
    prob, u0 = fx.single_qubit_transfer(explicit_init=True)
    for mode in ("ref_grape", "exact"):
        F, G = cpu_port.CpuProblem(prob, mode).eval(u0, threads=1)
        Fo, Go = mb.eval_problem(prob, u0, mode)
        assert abs(F - Fo) < 1e-13 and np.max(np.abs(G - Go)) < 1e-11 * np.max(np.abs(Go))


def test_plan_cache_is_host_side(pg):
    """pgx_plan_lookup / pgx_plan_clear touch no device: an unknown key reports
    PGX_ERR_STATE, and invalid descriptors are refused."""
    from pulsar_gb300 import workloads as W
    spec, _ = W.spin4_ensemble(n_t=4, n_off=1, n_b1=1)
    pg.plan_clear()
    assert pg.plan_lookup(**spec.problem_kwargs("exact", "mixed")) is None
    A = pg._abi
    t1, t2 = C.c_int32(), C.c_int32()
    assert A.lib().pgx_plan_lookup(0, None, C.byref(t1), C.byref(t2)) == 1


def test_taylor_table_is_the_generators_output():
    """csrc/taylor_table.h is exactly what csrc/gen_taylor_table.py prints
    (the thresholds the expm kernels choose degrees with)."""
    import io
    import importlib.util
    gen = ROOT / "pulsar.jl_gb300" / "csrc" / "gen_taylor_table.py"
    spec = importlib.util.spec_from_file_location("gen_taylor_table", gen)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    buf = io.StringIO()
    mod.main(out=buf)
    assert buf.getvalue() == (ROOT / "pulsar.jl_gb300" / "csrc" / "taylor_table.h").read_text()


def test_df_thresholds_bound_the_taylor_tail():
    """Every df threshold theta_m (degrees 1..20) keeps the Taylor tail
    sum_{k>m} theta^k/k! at or below 2^-47, and is increasing in m."""
    import math
    txt = (ROOT / "pulsar.jl_gb300" / "csrc" / "taylor_table.h").read_text()
    vals = [float(v) for v in re.search(r"PGX_THETADF_ALL_INIT \{([^}]*)\}", txt).group(1).split(",")]
    assert len(vals) == 20 and all(a < b for a, b in zip(vals, vals[1:]))
    for m, th in enumerate(vals, start=1):
        tail = sum(th ** k / math.factorial(k) for k in range(m + 1, m + 60))
        assert tail <= 2.0 ** -47 * (1 + 1e-9), (m, th, tail)
