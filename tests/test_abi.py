"""The C ABI library loads and exports every function include/seiswg.h
declares, and the Python binding declares a prototype for each of them."""
import ctypes
import os
import re
import subprocess

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
