"""The reference-side binding (include/gpu_bridge.c) compiled against a
stand-in of CoLoRe's ParamCoLoRe (src/common.h:208-381, restated in
tests/bridge/common.h) and run with cg_create replaced by a recorder: the
cg_config it builds from ParamCoLoRe must equal, field by field, the one
the host side builds from the same param file (cg_read_run_params +
cg_params_to_config).  Shell and plane distances pass through flouble in the
reference and are compared at float precision; everything else exactly.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "colore_gb300", "csrc", "host")
SRCS = [os.path.join(ROOT, "include", "gpu_bridge.c"), os.path.join(ROOT, "tests", "bridge", "bridge_check.c")] + \
       [os.path.join(HOST, f) for f in ("host_cosmo.c", "host_params.c", "host_io.c", "host_pred.c")]

SPECS = {
    "sources": dict(n_grid=64, z_min=0.05, z_max=0.6, r_smooth=2.0, seed=11, dens_type=0, bias_model=2,
                    srcs=[dict(nz=("gauss", 0.3, 0.1), density=40.0, bias=("1+z",), lensing=True, skewers=True),
                          dict(nz=("flat", 0.0, 0.5), density=30.0, bias=("const", 2.0), skewers=True,
                               gaussian_skewers=True)]),
    "maps": dict(n_grid=128, z_min=0.05, z_max=1.5, r_smooth=2.0, seed=4001, dens_type=1, bias_model=3,
                 lpt_interp_type=0,
                 srcs=[dict(nz=("gauss", 0.8, 0.3), density=100.0, bias=("1+z",))],
                 imap=[dict(tz=0.1, bias=("const", 1.0), z_range=(0.05, 1.5), nbands=64, nside=512),
                       dict(tz=0.2, bias=("1+z",), z_range=(0.3, 0.9), nbands=7, nside=64)],
                 custom=[dict(kz=("gauss", 0.5, 0.2), bias=("const", 1.0), nside=128)],
                 kappa=dict(z_out=[0.3, 0.7, 1.1, 1.5], nside=256),
                 isw=dict(z_out=[0.4, 0.9], nside=128)),
    "powerlaw": dict(n_grid=32, z_min=0.1, z_max=0.5, r_smooth=1.0, seed=7, dens_type=0, bias_model=1,
                     srcs=[dict(nz=("gauss", 0.3, 0.05), density=100.0, bias=("const", 1.5))]),
}


@pytest.mark.parametrize("name", sorted(SPECS))
def test_binding_fills_the_same_config(tmp_path, name):
    if shutil.which("gcc") is None:
        pytest.skip("gcc absent")
    from colore_gb300 import inputs
    spec = SPECS[name]
    cfg = inputs.write_inputs(str(tmp_path), spec)
    exe = str(tmp_path / "bridge_check")
    flag = {1: [], 2: ["-D_BIAS_MODEL_2"], 3: ["-D_BIAS_MODEL_3"]}[spec["bias_model"]]
    cmd = ["gcc", "-std=gnu11", "-O1", "-Wall", "-Werror", "-Wno-unused-function", "-fopenmp"] + flag + \
          ["-I" + os.path.join(ROOT, "tests", "bridge"), "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "colore_gb300", "csrc"), "-o", exe] + SRCS + ["-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([exe, cfg], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fields differing: 0" in r.stdout
