"""The C ABI library loads and exports every function include/seiswg.h
declares, and the Python binding declares a prototype for each of them."""
import ctypes
import os
import re
import subprocess
import sys

import seiswg_gb300 as sw

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(seiswg_\w+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_the_api():
    names = declared_functions()
    for n in ("seiswg_config_load", "seiswg_solver_new", "seiswg_solver_run_forward", "seiswg_solver_run_adjoint",
              "seiswg_sim_forward", "seiswg_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(sw.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_has_prototypes_for_every_symbol():
    bound = {p[0] for p in sw.PROTOTYPES}
    assert set(declared_functions()) <= bound


def test_exports_are_c_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", sw.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (seiswg_\w+)$", out, flags=re.M))
    assert set(declared_functions()) <= exported


def test_cli_prints_usage():
    r = subprocess.run([sw.CLI_PATH], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage" in r.stderr


NULL_PROBE = r"""
import ctypes, sys
sys.path.insert(0, sys.argv[1])
import seiswg_gb300 as sw
lib = sw.lib()
# Calls that return a value rather than a status (0 for a null handle), and a
# Ricker wavelet of zero samples (a valid empty request).
values = {"seiswg_sim_checkpoint_interval", "seiswg_batch_chunk_rows", "seiswg_batch_two_step",
          "seiswg_batch_concurrent", "seiswg_batch_stream_groups", "seiswg_batch_tma_jobs", "seiswg_ricker"}
for name, res, args in sw.PROTOTYPES:
    if res is not ctypes.c_int or name in values:
        continue
    vals = [a(0) if a in (ctypes.c_float, ctypes.c_int32, ctypes.c_size_t, ctypes.c_int64, ctypes.c_uint64)
            else None for a in args]
    rc = getattr(lib, name)(*vals)
    msg = lib.seiswg_last_error() or b""
    print(name, rc, len(msg), flush=True)
"""


def test_null_arguments_give_error_codes():
    """Every status-returning call of the C ABI, given null handles and null
    pointers (and zero sizes), returns an error code with a message; none
    crashes (run in a child process so that a crash fails only this test).
    Without a GPU none of these reaches the device."""
    r = subprocess.run([sys.executable, "-c", NULL_PROBE, ROOT], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout[-2000:], r.stderr[-2000:])
    lines = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("seiswg_")]
    assert len(lines) >= 40
    bad = [(n, rc, m) for (n, rc, m) in lines if int(rc) == 0 or int(m) == 0]
    assert not bad, bad
