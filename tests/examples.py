"""Test inputs: the reference's examples rebuilt from tests/golden/*.npz in
the reference's own file formats (model .bin with int32 header, sources.dat,
stations.dat, config.ini), plus the FP32/FP64 oracle run on the same inputs."""
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def write_bin(path, data):
    a = np.ascontiguousarray(data, np.float32).reshape(-1)
    with open(path, "wb") as f:
        np.array([a.size], np.int32).tofile(f)
        a.tofile(f)


def write_example(name, dest):
    """Writes examples/<name> into dest; returns the path of config.ini."""
    g = golden(name)
    os.makedirs(dest, exist_ok=True)
    open(os.path.join(dest, "config.ini"), "w").write(str(g["config_ini"]))
    open(os.path.join(dest, "sources.dat"), "w").write(str(g["sources_dat"]))
    open(os.path.join(dest, "stations.dat"), "w").write(str(g["stations_dat"]))
    if name in ("forward", "spin"):
        md = os.path.join(dest, "model")
        os.makedirs(md, exist_ok=True)
        for k in g.files:
            if k.startswith("model_"):
                write_bin(os.path.join(md, f"proc000000_{k[6:]}.bin"), g[k])
    else:
        open(os.path.join(dest, "config_true.ini"), "w").write(str(g["config_true_ini"]))
        for pre, sub in (("init_", "model_init"), ("true_", "model_true")):
            md = os.path.join(dest, sub)
            os.makedirs(md, exist_ok=True)
            for k in g.files:
                if k.startswith(pre):
                    write_bin(os.path.join(md, f"proc000000_{k[len(pre):]}.bin"), g[k])
    return os.path.join(dest, "config.ini")


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def max_rel(a, b):
    """tests/integration.rs:153-175: max |got-ref| / peak |ref|."""
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    peak = np.abs(b).max()
    return float(np.abs(a - b).max() / (peak if peak > np.finfo(np.float32).eps else 1.0))


def read_npy_payload(b):
    """Payload of a .npy v1 file as flat float32 (tests/integration.rs:116-142)."""
    hl = int.from_bytes(b[8:10], "little")
    return np.frombuffer(b[10 + hl:], "<f4")


# ---------------------------------------------------------------------------
# oracle set-ups for the examples
# ---------------------------------------------------------------------------

def oracle_example(name, precision=32, model="init"):
    """(oracle instance, setup, src_k, rec_k) for an example, built with the
    oracle's own restatement of the reference's host set-up."""
    import configparser

    from oracle import oracle as O

    g = golden(name)
    c = configparser.ConfigParser()
    c.read_string(str(g["config_ini"]))
    sol = c["solver"]
    yes = lambda k, d: sol.get(k, "yes" if d else "no").strip().lower() == "yes"  # noqa: E731
    if name == "adjoint":
        pre = "init_" if model == "init" else "true_"
        x, z = g[pre + "x"], g[pre + "z"]
    else:
        pre = "model_"
        x, z = g["model_x"], g["model_z"]
    nx, nz, dx, dz = O.infer_grid(x, z)
    nt = int(sol["nt"])
    dt = float(np.float32(sol["dt"]))
    s = O.Setup(nx, nz, nt, dx, dz, dt, sh=yes("sh", False), psv=yes("psv", True), spin=yes("spin", False),
                abs_left=yes("abs_left", False), abs_right=yes("abs_right", False),
                abs_bottom=yes("abs_bottom", False), abs_top=yes("abs_top", False),
                abs_width=int(sol.get("abs_width", 20)), abs_alpha=float(np.float32(sol.get("abs_alpha", 0.015))))
    src = O.source_params(O.parse_table(str(g["sources_dat"])))
    rec = O.parse_table(str(g["stations_dat"]))
    sk = O.locate([r[0] for r in src], [r[1] for r in src], dx, dz, nz)
    rk = O.locate([r[0] for r in rec], [r[1] for r in rec], dx, dz, nz)
    stf = O.stf_table(src, nt, dt, precision)
    o = O.FD2DOracle(s, sk, stf, rk, precision)
    if s.spin:
        for n, f in [("rho", "RHO"), ("lambda", "LAM"), ("mu", "MU"), ("nu", "NU"), ("j", "J"),
                     ("lambda_c", "LAM_C"), ("mu_c", "MU_C"), ("nu_c", "NU_C")]:
            o.set_field(f, g[pre + n])
    else:
        o.set_field("LAM", g[pre + "vp"])
        o.set_field("MU", g[pre + "vs"])
        o.set_field("RHO", g[pre + "rho"])
    o.init_model()
    return o, s, sk, rk
