"""Regenerate the golden fixtures under tests/golden/ from a checkout of seiswg.

The reference's integration tests (tests/integration.rs:202-282) pin three
WGSL-path outputs; this script packs those outputs, together with the example
inputs that produced them, into compressed .npz files so that the parity tests
run without the reference checkout (it is absent on the GPU machines).

    python tests/golden/make_golden.py /path/to/seiswg
    SEISWG_REFERENCE=/path/to/seiswg python tests/golden/make_golden.py

Contents
--------
forward.npz   examples/forward inputs + tests/fixtures/forward/{proc000100_vy.bin,uy_000000.npy}
spin.npz      examples/spin inputs    + tests/fixtures/spin/{proc000200_vx.bin,ry_000000.npy}
adjoint.npz   examples/adjoint inputs (model_init, model_true) + tests/fixtures/adjoint/proc000000_kmu.bin
              + a slice of examples/adjoint/obs_traces (the WGSL forward run on model_true):
                shots 0 and 11, every 6th receiver, all 4800 samples.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_model_bin(path):
    b = open(path, "rb").read()
    n = int(np.frombuffer(b[:4], "<i4")[0])
    return np.frombuffer(b[4:4 + 4 * n], "<f4").copy()


def read_raw(path):
    return np.fromfile(path, "<f4")


def read_npy(path):
    return np.load(path).astype(np.float32)


def text(path):
    return np.array(open(path).read())


def model_dir(d, names, prefix):
    return {f"{prefix}{n}": read_model_bin(os.path.join(d, f"proc000000_{n}.bin")) for n in names}


def main(ref):
    ex = os.path.join(ref, "examples")
    fx = os.path.join(ref, "tests", "fixtures")

    d = os.path.join(ex, "forward")
    arrs = dict(config_ini=text(os.path.join(d, "config.ini")),
                sources_dat=text(os.path.join(d, "sources.dat")),
                stations_dat=text(os.path.join(d, "stations.dat")))
    arrs.update(model_dir(os.path.join(d, "model"), ["x", "z", "vp", "vs", "rho"], "model_"))
    arrs["fix_proc000100_vy"] = read_raw(os.path.join(fx, "forward", "proc000100_vy.bin"))
    arrs["fix_uy_000000"] = read_npy(os.path.join(fx, "forward", "uy_000000.npy"))
    np.savez_compressed(os.path.join(HERE, "forward.npz"), **arrs)

    d = os.path.join(ex, "spin")
    arrs = dict(config_ini=text(os.path.join(d, "config.ini")),
                sources_dat=text(os.path.join(d, "sources.dat")),
                stations_dat=text(os.path.join(d, "stations.dat")))
    arrs.update(model_dir(os.path.join(d, "model"),
                          ["x", "z", "rho", "lambda", "mu", "nu", "j", "lambda_c", "mu_c", "nu_c"], "model_"))
    arrs["fix_proc000200_vx"] = read_raw(os.path.join(fx, "spin", "proc000200_vx.bin"))
    arrs["fix_ry_000000"] = read_npy(os.path.join(fx, "spin", "ry_000000.npy"))
    np.savez_compressed(os.path.join(HERE, "spin.npz"), **arrs)

    d = os.path.join(ex, "adjoint")
    arrs = dict(config_ini=text(os.path.join(d, "config.ini")),
                config_true_ini=text(os.path.join(d, "config_true.ini")),
                sources_dat=text(os.path.join(d, "sources.dat")),
                stations_dat=text(os.path.join(d, "stations.dat")))
    names = ["x", "z", "vp", "vs", "rho"]
    arrs.update(model_dir(os.path.join(d, "model_init"), names, "init_"))
    arrs.update(model_dir(os.path.join(d, "model_true"), names, "true_"))
    arrs["fix_proc000000_kmu"] = read_raw(os.path.join(fx, "adjoint", "proc000000_kmu.bin"))
    shots = np.array([0, 11], np.int32)
    recs = np.arange(0, 144, 6, dtype=np.int32)
    obs = np.stack([read_npy(os.path.join(d, "obs_traces", f"uy_{s:06d}.npy"))[recs] for s in shots])
    arrs.update(obs_shots=shots, obs_recs=recs, obs_uy=obs)
    np.savez_compressed(os.path.join(HERE, "adjoint.npz"), **arrs)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SEISWG_REFERENCE", "")
    if not src:
        sys.exit("usage: make_golden.py <seiswg checkout> (or set SEISWG_REFERENCE)")
    main(src)
