"""Synthetic inputs for CoLoRe runs: linear P(k), N(z), b(z), T(z), frequency
tables and the param file, in the text formats the reference reads
(cosmo.c:452-465, 549-666, 497-514).

P(k) is the Eisenstein & Hu (1998, ApJ 496, 605) no-wiggle transfer function,
eqs. (26) and (28)-(31), times k^ns; the run renormalises it to sigma_8.
The public datasets of the reference's examples are not shipped, so every
benchmark and test configuration is generated here with the shapes the run
configurations describe.
"""
import os

import numpy as np

TCMB = 2.7255


def eh_nowiggle_pk(k, om, ob, h, ns, tcmb=TCMB):
    """Unnormalised P(k) = k^ns T_nw(k)^2, k in h/Mpc."""
    k = np.asarray(k, float)
    theta = tcmb / 2.7
    omh2, obh2 = om * h * h, ob * h * h
    fb = ob / om
    s = 44.5 * np.log(9.83 / omh2) / np.sqrt(1 + 10 * obh2 ** 0.75)          # Mpc, eq. (26)
    alpha = 1 - 0.328 * np.log(431 * omh2) * fb + 0.38 * np.log(22.3 * omh2) * fb * fb  # eq. (31)
    kmpc = k * h
    gamma = om * h * (alpha + (1 - alpha) / (1 + (0.43 * kmpc * s) ** 4))    # eq. (30)
    q = k * theta * theta / gamma                                             # eq. (28)
    L0 = np.log(2 * np.e + 1.8 * q)
    C0 = 14.2 + 731.0 / (1 + 62.5 * q)
    T = L0 / (L0 + C0 * q * q)                                                # eq. (29)
    return k ** ns * T * T


COSMO = dict(omega_M=0.3, omega_L=0.7, omega_B=0.05, h=0.7, w=-1.0, ns=0.96, sigma_8=0.8)


def _nz_shape(z, shape):
    kind = shape[0]
    if kind == "gauss":
        return np.exp(-0.5 * ((z - shape[1]) / shape[2]) ** 2)
    if kind == "flat":  # top hat with 0.005-wide tanh edges (no spline ringing)
        w = 0.005
        return 0.5 * (np.tanh((z - shape[1]) / w) - np.tanh((z - shape[2]) / w))
    raise ValueError(shape)


def _bias(z, b):
    if b[0] == "const":
        return np.full_like(z, b[1])
    if b[0] == "1+z":
        return 1 + z
    raise ValueError(b)


# Run configurations c1-c5 of the benchmark suite, as their text states them
# (nside choices where the text leaves them open are written beside them).
CONFIGS = {
    "c1": dict(n_grid=128, z_min=0.1, z_max=0.5, r_smooth=2.0, seed=1001, dens_type=0, bias_model=1,
               srcs=[dict(nz=("gauss", 0.3, 0.05), density=100.0, bias=("const", 1.5), nside_count=64)]),
    "c2": dict(n_grid=512, z_min=0.05, z_max=1.0, r_smooth=2.0, seed=2001, dens_type=0, bias_model=2,
               srcs=[dict(nz=("flat", 0.2, 0.8), density=500.0, bias=("1+z",), nside_count=256),
                     dict(nz=("gauss", 0.7, 0.1), density=50.0, bias=("const", 2.0), nside_count=256)]),
    "c4": dict(n_grid=1024, z_min=0.05, z_max=1.5, r_smooth=2.0, seed=4001, dens_type=1, bias_model=2,
               srcs=[dict(nz=("gauss", 0.8, 0.3), density=1000.0, bias=("1+z",), nside_count=512)],
               imap=[dict(tz=0.1, bias=("const", 1.0), z_range=(0.05, 1.5), nbands=64, nside=512)],
               kappa=dict(z_out=list(np.linspace(0.3, 1.5, 8)), nside=512)),
    "c5": dict(n_grid=2048, z_min=0.05, z_max=2.0, r_smooth=2.0, seed=5001, dens_type=0, bias_model=2,
               srcs=[dict(nz=("gauss", 0.4, 0.15), density=2000.0, bias=("const", 1.2), nside_count=1024),
                     dict(nz=("gauss", 0.9, 0.15), density=500.0, bias=("const", 1.8), nside_count=1024),
                     dict(nz=("gauss", 1.4, 0.15), density=100.0, bias=("const", 2.5), nside_count=1024)],
               kappa=dict(z_out=[0.5, 1.0, 1.5, 1.9], nside=1024)),
}


def batch_specs(n=48, seed=3000):
    """The batched workload: n independent realisations, a third each at
    128^3, 256^3 and 384^3, seeds 3001 + i, z_min 0.05 and z_max drawn
    uniformly in [0.1, 1.2] from `seed`; one population with b = 1.5 and a
    flat dN/dz of 200 per deg^2 between z_min and z_max."""
    rng = np.random.default_rng(seed)
    zmax = rng.uniform(0.1, 1.2, n)
    grids = [128, 256, 384]
    out = []
    for i in range(n):
        out.append(dict(n_grid=grids[min(3 * i // n, 2)], z_min=0.05, z_max=float(zmax[i]), r_smooth=2.0,
                        seed=3001 + i, dens_type=0, bias_model=2,
                        srcs=[dict(nz=("flat", 0.05, float(zmax[i])), density=200.0, bias=("const", 1.5),
                                   nside_count=0)]))
    return out


def scaled(name, n_grid, **over):
    """A configuration with another grid size (and optional overrides)."""
    spec = dict(CONFIGS[name])
    spec["n_grid"] = n_grid
    spec.update(over)
    return spec


def write_inputs(dirname, spec, prefix="run"):
    """Write every input file and the param file; returns the param path."""
    os.makedirs(dirname, exist_ok=True)
    z_end = spec["z_max"] * 1.3 + 0.3
    zs = np.linspace(0.0, z_end, 2001)
    k = np.logspace(-4, 2, 1000)
    cos = dict(COSMO, **spec.get("cosmo", {}))
    pk = eh_nowiggle_pk(k, cos["omega_M"], cos["omega_B"], cos["h"], cos["ns"])
    pkf = os.path.join(dirname, "pk.txt")
    np.savetxt(pkf, np.transpose([k, pk]), fmt="%.10e")
    lines = []
    add = lines.append
    add("global:\n{\n  prefix_out= \"%s\";\n  output_format= \"%s\";\n  output_density= %s;" %
        (os.path.join(dirname, prefix), spec.get("output_format", "ASCII"),
         "true" if spec.get("output_density") else "false"))
    pred = spec.get("pred")
    pred_txt = ("write_pred= true;\n  just_write_pred= %s;\n  pred_dz= %r;" %
                ("true" if pred.get("just") else "false", float(pred["dz"]))) if pred else "write_pred= false;"
    add("  pk_filename= \"%s\";\n  z_min= %r;\n  z_max= %r;\n  seed= %d;\n  %s" %
        (pkf, float(spec["z_min"]), float(spec["z_max"]), spec["seed"], pred_txt))
    add("  bias_model= %d;\n}\n" % spec.get("bias_model", 2))
    add("field_par:\n{\n  r_smooth= %r;\n  smooth_potential= true;\n  n_grid= %d;\n  dens_type= %d;" %
        (float(spec["r_smooth"]), spec["n_grid"], spec.get("dens_type", 0)))
    add("  lpt_buffer_fraction= 0.6;\n  lpt_interp_type= %d;\n  output_lpt= 0;\n}\n" % spec.get("lpt_interp_type", 1))
    add("cosmo_par:\n{\n" + "".join("  %s= %r;\n" % (kk, float(v)) for kk, v in cos.items()) + "}\n")
    for i, s in enumerate(spec.get("srcs", [])):
        nz = _nz_shape(zs, s["nz"])
        nz *= s["density"] / np.trapezoid(nz, zs)
        fnz = os.path.join(dirname, "nz_%d.txt" % (i + 1))
        fbz = os.path.join(dirname, "bz_%d.txt" % (i + 1))
        np.savetxt(fnz, np.transpose([zs, nz]), fmt="%.10e")
        np.savetxt(fbz, np.transpose([zs, _bias(zs, s["bias"])]), fmt="%.10e")
        tf = lambda b: "true" if b else "false"  # noqa: E731
        gs = "  gaussian_skewers= %s;\n" % tf(s["gaussian_skewers"]) if "gaussian_skewers" in s else ""
        add("srcs%d:\n{\n  nz_filename= \"%s\";\n  bias_filename= \"%s\";\n  include_lensing= %s;\n"
            "  store_skewers= %s;\n%s  nside_count= %d;\n}\n" %
            (i + 1, fnz, fbz, tf(s.get("lensing")), tf(s.get("skewers")), gs, s.get("nside_count", 0)))
    for i, m in enumerate(spec.get("imap", [])):
        ftz = os.path.join(dirname, "tz_%d.txt" % (i + 1))
        fbz = os.path.join(dirname, "bzi_%d.txt" % (i + 1))
        fnu = os.path.join(dirname, "nu_%d.txt" % (i + 1))
        np.savetxt(ftz, np.transpose([zs, m["tz"] * (1 + zs)]), fmt="%.10e")
        np.savetxt(fbz, np.transpose([zs, _bias(zs, m["bias"])]), fmt="%.10e")
        nu_rest = 1420.405
        z0, z1 = m["z_range"]
        edges = np.linspace(nu_rest / (1 + z1), nu_rest / (1 + z0), m["nbands"] + 1)
        np.savetxt(fnu, np.transpose([edges[:-1], edges[1:]]), fmt="%.10f")
        add("imap%d:\n{\n  tbak_filename= \"%s\";\n  bias_filename= \"%s\";\n  freq_list= \"%s\";\n"
            "  freq_rest= %r;\n  nside= %d;\n}\n" % (i + 1, ftz, fbz, fnu, nu_rest, m["nside"]))
    for i, m in enumerate(spec.get("custom", [])):
        fkz = os.path.join(dirname, "kzc_%d.txt" % (i + 1))
        fbz = os.path.join(dirname, "bzc_%d.txt" % (i + 1))
        np.savetxt(fkz, np.transpose([zs, m.get("amp", 1.0) * _nz_shape(zs, m["kz"])]), fmt="%.10e")
        np.savetxt(fbz, np.transpose([zs, _bias(zs, m["bias"])]), fmt="%.10e")
        add("custom%d:\n{\n  kz_filename= \"%s\";\n  bias_filename= \"%s\";\n  nside= %d;\n}\n" %
            (i + 1, fkz, fbz, m["nside"]))
    if "kappa" in spec:
        kz = ", ".join("%r" % float(z) for z in spec["kappa"]["z_out"])
        add("kappa:\n{\n  z_out= [%s];\n  nside= %d;\n}\n" % (kz, spec["kappa"]["nside"]))
    if "isw" in spec:
        iz = ", ".join("%r" % float(z) for z in spec["isw"]["z_out"])
        add("isw:\n{\n  z_out= [%s];\n  nside= %d;\n}\n" % (iz, spec["isw"]["nside"]))
    fcfg = os.path.join(dirname, prefix + ".cfg")
    with open(fcfg, "w") as f:
        f.write("\n".join(lines))
    return fcfg
