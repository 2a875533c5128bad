"""Benchmark: end-to-end cells/s of CoLoRe's mock-generation path.

One step is the whole driver sequence of src/main.c:66-125 on one
realisation: Gaussian density and potential (fill + 3-D c2r), physical
density (1LPT + CIC for the 1024^3 configuration), redshift-bin bias
normalisation, Poisson sources with their local properties and count map,
the 64-shell intensity map and the 8 convergence planes.

  value : N^3 * steps / device time, inputs (tables) resident on the GPU;
  e2e   : the same through the C ABI with host buffers: every step uploads
          the tables and downloads the catalogue, count map, intensity and
          convergence maps into pinned host memory inside the timed region.

--impl reference times the CPU restatement of the reference (the oracle,
FP64, OpenMP on all host cores) on a bounded sample of the same workload.
Multi-GPU runs are independent replicas (one realisation per rank, seed +
rank): the path has no exchange step on one node.
"""
import argparse
import json
import numpy as np
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# the headline metric of the 1024^3 workload
METRIC = "end-to-end cells/s at 1024\u00b3, FP32/split vs FP64 on same GPU at P(k) err\u22641e-4"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d["hbm_gbs"], "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    def __init__(self, dev):
        self.dev = dev
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                self.samples.append(f)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        import numpy as np
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if "Active" in s[5 + i]
                          and "Not" not in s[5 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def config_spec(name, n):
    from colore_gb300 import inputs
    spec = inputs.scaled(name, n) if n else dict(inputs.CONFIGS[name])
    return spec


# Algorithmic HBM bytes per cell of each launch group (FP32 grids; per pass
# and field one read and one write of 4 bytes per cell; the fill+z pass only
# writes).  fields: fill+z 2x4 W, y 2x(4R+4W), x 2x(4R+4W) = 40 B/cell.
ALGO_BYTES_PER_CELL = {"field_fft": 40.0, "lpt_fft": 60.0, "dens_bins": 8.0, "srcs_count": 6.0,
                       "field_fill": 8.0, "field_y": 16.0, "field_x": 16.0,
                       "lpt_fill": 12.0, "lpt_y": 24.0, "lpt_x": 24.0}
# passes whose bound is HBM traffic: the y and x transform passes.  The
# fills generate their modes, the density/bins pass evaluates exp/log per
# cell and tracer, the Poisson count draws per cell: those are issue bound
# (ncu: 5-18 % of DRAM peak) and are reported under "kernels" only.
HBM_PASSES = ("lpt_y", "lpt_x", "field_y", "field_x")
# DRAM bytes (read + write) per cell of the same groups measured by ncu on the
# 512^3 case of config c4 (grids larger than L2; dram__bytes_read.sum +
# dram__bytes_write.sum of one launch over the cell count); traffic grows with
# the cell count, so a launch at N^3 moves N^3 times these.
MEASURED_DRAM_BYTES_PER_CELL = {"field_fft": 38.5, "lpt_fft": 59.8, "dens_bins": 7.6, "field_fill": 7.6,
                                "field_y": 15.65, "field_x": 15.2, "lpt_fill": 11.8, "lpt_y": 23.68, "lpt_x": 23.7}


# Thread-instructions per unit of work of the intensity-map stage's kernels,
# from one-kernel ncu captures at 512^3 (smsp__inst_executed.sum x
# smsp__thread_inst_executed_per_inst_executed.ratio over the units): the
# listing kernel per cell in the shells' radial range, the painting kernel per
# sub-sample.  The stage is bound by instruction issue, not HBM, so its
# roofline is the issue rate: 4 schedulers x 32 lanes per SM and cycle.
IMAP_INSTR_PER_CELL = 688.9
IMAP_INSTR_PER_SAMPLE = 176.5


def issue_roofline(dom, t_step, cfg, m, clocks):
    """The step's largest launch group and what bounds it."""
    name, ms = dom
    out = {"kernel": name, "ms": round(ms, 3), "share": round(ms / (t_step * 1e3), 3)}
    if name != "imap_paint":
        out["bound"] = "see kernels"
        return out
    import math
    import torch
    n = cfg.n_grid
    # cells in the shells' radial range: the ball of radius r_max in a box of
    # side l_box (the shells reach r_max), pi/6 of the cells when it fits
    frac = min(1.0, 4.0 / 3.0 * math.pi * (cfg.r_max / cfg.l_box) ** 3)
    cells = frac * float(n) ** 3
    samples = float(sum(m.imap_samples(i) for i in range(cfg.n_imap)))
    instr = IMAP_INSTR_PER_CELL * cells + IMAP_INSTR_PER_SAMPLE * samples
    mhz = clocks.get("sm_mhz") or 2070.0
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    peak = sms * 4 * 32 * mhz * 1e6
    achieved = instr / (ms / 1e3)
    out.update({"bound": "instruction issue", "achieved": achieved, "peak": peak, "unit": "thread-instructions/s",
                "frac": round(achieved / peak, 4),
                "basis": "ncu thread-instructions per unit at 512^3 (listing %.0f per cell in range, painting %.1f "
                         "per sub-sample) x this step's cells and sub-samples / the stage's CUDA-event time; peak "
                         "= SMs x 4 schedulers x 32 lanes x median SM clock; DRAM at 1-4 %% of peak"
                         % (IMAP_INSTR_PER_CELL, IMAP_INSTR_PER_SAMPLE)})
    return out


# ---- replicas: one realisation per rank, no exchange on the data path ----
def rank_seed(seed, rank):
    """Each rank runs its own realisation."""
    return seed + rank


def max_over_ranks(times, dist, device):
    """The slowest rank bounds the job: max of each timing over the ranks."""
    if dist is None:
        return [float(t) for t in times]
    import torch
    tt = torch.tensor([float(t) for t in times], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return tt.tolist()


def job_cells_per_s(ncell, world, t_step):
    """Whole-job throughput: the cells of all ranks over the slowest rank's time."""
    return world * ncell / t_step


def run_ours(args):
    import numpy as np
    import torch
    import colore_gb300 as cg

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    torch.cuda.set_device(local)
    spec = config_spec(args.config, args.n)
    spec["seed"] = rank_seed(spec["seed"], rank)
    d = tempfile.mkdtemp(prefix="colore_bench_%d_" % rank)
    from colore_gb300 import inputs
    prm = cg.Params(inputs.write_inputs(d, spec))
    cfg = prm.config
    n = cfg.n_grid
    ncell = float(n) ** 3
    m = cg.Mock(prm, device=local)
    stream = torch.cuda.Stream()
    m.set_stream(stream.cuda_stream)

    def barrier():
        if dist:
            dist.barrier()

    for _ in range(args.warmup):
        m.run()
    m.sync()
    m.exact_stats(reset=True)
    # device-timed region (inputs resident; grids of 4.3 GB per field >> 129 MB L2)
    m.set_profiling(True)
    l0 = m.launches()
    barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        with torch.cuda.stream(stream):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            t0 = time.perf_counter()
            for _ in range(args.steps):
                m.run()
            e1.record(stream)
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t0
    barrier()
    launches = m.launches() - l0
    ms = e0.elapsed_time(e1)
    groups = {}
    for name, t in m.kernel_times():
        g = groups.setdefault(name, [0.0, 0])
        g[0] += t
        g[1] += 1
    m.set_profiling(False)
    nsrc = [m.num_sources(i) for i in range(cfg.n_srcs)]
    # what the timed steps left to double arithmetic (cg_exact_stats)
    exact = m.exact_stats(reset=True)
    # end-to-end through the C ABI with host buffers: the outputs the
    # reference's writers take (the catalogue's Src array, src/common.h:169-179;
    # the intensity maps as data/nadd; the convergence maps) are registered as
    # page-locked host destinations that the stages fill as each output is
    # final, overlapping the later stages (cg_set_host_*); the small count
    # maps are downloaded after the run
    outs = {}
    cats = {}
    for i in range(cfg.n_srcs):
        k = int(nsrc[i] * 1.25) + 1024
        outs["src%d" % i] = torch.empty((k, 9), dtype=torch.float32, pin_memory=True).numpy()
        outs["n%d" % i] = torch.empty(1, dtype=torch.int64, pin_memory=True).numpy()
        cats[i] = (outs["src%d" % i], outs["n%d" % i])
        if cfg.nside_count[i]:
            outs["cmap%d" % i] = torch.empty(12 * cfg.nside_count[i] ** 2, dtype=torch.int32,
                                             pin_memory=True).numpy()
    imaps = {}
    for i in range(cfg.n_imap):
        imaps[i] = outs["imap%d" % i] = torch.empty((cfg.imap_nr[i], 12 * cfg.nside_imap[i] ** 2),
                                                    dtype=torch.float32, pin_memory=True).numpy()
    if cfg.do_kappa:
        outs["kappa"] = torch.empty((cfg.n_kappa, 12 * cfg.nside_kappa ** 2), dtype=torch.float32,
                                    pin_memory=True).numpy()
    m.set_host_outputs(catalogs=cats, imaps=imaps, kappa=outs.get("kappa"))

    def e2e_step():
        m.upload_tables()
        m.run()
        m.sync()
        t1 = time.perf_counter()
        nb = 0
        for i in range(cfg.n_srcs):
            ns = int(outs["n%d" % i][0])
            if ns > outs["src%d" % i].shape[0]:
                raise RuntimeError("host catalogue buffer too short")
            nb += ns * 36 + 8
            if cfg.nside_count[i]:
                m.count_map(i, out=outs["cmap%d" % i])
                nb += outs["cmap%d" % i].nbytes
        for i in range(cfg.n_imap):
            nb += outs["imap%d" % i].nbytes
        if cfg.do_kappa:
            nb += outs["kappa"].nbytes
        return nb, time.perf_counter() - t1

    # untimed steps first: the first steps after registering the host
    # outputs set up the copy stream and the maps' staging buffers
    for _ in range(max(1, min(args.warmup, 3))):
        e2e_step()
    e2e_steps = max(10, args.steps)
    d2h = 0
    h2d = 0
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    t_dl = 0.0
    for _ in range(e2e_steps):
        d2h, dt = e2e_step()
        t_dl += dt
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    t_dl /= e2e_steps
    barrier()
    na = cg.NA
    h2d = 8 * (9 * na + 2 * na * (cfg.n_srcs + cfg.n_imap) + cfg.numk) // 2  # tables as float
    t_step = ms / 1e3 / args.steps
    if dist:
        t_step, t_e2e = max_over_ranks([t_step, t_e2e], dist, "cuda")
    hbm, peak_kind = peaks()
    # roofline of the dominant HBM-bound group
    rl = None
    avg = {k: v[0] / max(v[1], 1) for k, v in groups.items()}
    for name in HBM_PASSES:
        if avg.get(name, 0) > 0:
            bytes_launch = ALGO_BYTES_PER_CELL[name] * ncell
            a = bytes_launch / (avg[name] / 1e3) / 1e9
            if rl is None or avg[name] > rl["_t"]:
                tr = MEASURED_DRAM_BYTES_PER_CELL.get(name)
                rl = {"kernel": name, "bound": "hbm", "achieved": round(a, 1), "peak": hbm, "unit": "GB/s",
                      "frac": round(a / hbm, 4), "traffic": tr * ncell if tr else None,
                      "traffic_source": "ncu DRAM bytes per cell at 512^3 x cells" if tr else None,
                      "peak_kind": peak_kind,
                      "algorithmic_bytes_per_launch": bytes_launch, "avg_launch_ms": round(avg[name], 3),
                      "note": "the HBM-bound pass with the most time per step (fills, bins, Poisson count, "
                              "deposit and painting are issue bound: see kernels and roofline_dominant)",
                      "_t": avg[name]}
    if rl:
        rl.pop("_t")
    # the step's largest launch group and what bounds it
    dom = max(avg.items(), key=lambda kv: kv[1]) if avg else None
    # per group: GB/s of the HBM-bound passes, samples/s where atomics or
    # gathers bound the kernel (intensity-map sub-samples, kappa ray steps)
    kern = {}
    for name, t in avg.items():
        if name in ALGO_BYTES_PER_CELL and t > 0:
            gbs = ALGO_BYTES_PER_CELL[name] * ncell / (t / 1e3) / 1e9
            kern[name] = {"ms": round(t, 3), "GB/s": round(gbs, 1), "frac_hbm": round(gbs / hbm, 4)}
        else:
            kern[name] = {"ms": round(t, 3)}
    if "imap_paint" in avg:
        smp = sum(m.imap_samples(i) for i in range(cfg.n_imap))
        kern["imap_paint"]["samples"] = smp
        kern["imap_paint"]["samples/s"] = smp / (avg["imap_paint"] / 1e3)
    if "kappa" in avg and cfg.do_kappa:
        st = _kappa_steps(cfg)
        kern["kappa"]["ray_steps"] = st
        kern["kappa"]["ray_steps/s"] = st / (avg["kappa"] / 1e3)
    if rank != 0:
        return
    out = {
        "metric": METRIC if args.config == "c4" and not args.n else "end-to-end cells/s, %s %d^3" % (args.config, n),
        "value": job_cells_per_s(ncell, world, t_step), "unit": "cells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (EH98 no-wiggle P(k), analytic N(z)/b(z)/T(z); random seeds per rank)",
        "config": workload_config(args, cfg),
        "e2e": {"value": job_cells_per_s(ncell, world, t_e2e), "unit": "cells/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": t_e2e * 1e3,
                "download_ms_per_step": t_dl * 1e3,
                "overlapped_copies": "catalogue Src arrays, intensity maps and convergence maps are copied to "
                                     "page-locked host memory during the run (cg_set_host_*); download_ms_per_step "
                                     "is the count maps read after it"},
        "gpu_launches": int(launches),
        "kernel_ms": {k: round(v, 3) for k, v in avg.items()},
        "kernels": kern,
        "sources": nsrc,
        "wall_s_timed": t_wall,
        "roofline": rl,
        "fft_plan": m.field_plan(),
        "exact_decisions": {"per_step": {k: v / max(args.steps, 1) for k, v in exact.items()},
                            "note": "decisions taken in double per step (cells' counts, source pixels, "
                                    "intensity-map cells and sub-samples); every other decision in single "
                                    "precision with a proven margin, or in float-float for the intensity-map "
                                    "sub-samples that margin leaves open"},
        "roofline_dominant": issue_roofline(dom, t_step, cfg, m, clk.summary()) if dom else None,
        "clocks": clk.summary(),
    }
    if not args.no_fp64:
        # the metric's gate: the Gaussian field and potential of this
        # realisation against the FP64 path's, mode for mode, on the device
        # (relative rms and the P(k) error per shell of width k_f)
        from colore_gb300 import validate
        m.create_cartesian_fields()
        f64 = cg.Mock64(prm, device=local)
        f64.create_cartesian_fields()
        fe = validate.field_errors(m, f64)
        f64.close()
        torch.cuda.empty_cache()
        out["pk_max_rel_err"] = max(fe[0]["pk_max_rel_err"], fe[1]["pk_max_rel_err"])
        out["field_errors_vs_fp64"] = {
            lab: {"rel_rms": fe[w]["rel_rms"], "pk_max_rel_err": fe[w]["pk_max_rel_err"],
                  "shells": len(fe[w]["pk_rel_err"])} for w, lab in ((0, "delta_G"), (1, "phi"))}
    if world == 1 and not args.no_fp64:
        # the plain FP64 path of the same sequence on the same GPU (first run
        # allocates; the second is timed with CUDA events)
        m64 = cg.Mock64(prm, device=local)
        m64.run()
        t64 = m64.run()
        m64.close()
        v64 = ncell / (t64 / 1e3)
        out["fp64_gpu"] = {"value": v64, "unit": "cells/s", "ms_per_step": t64,
                           "speedup_of_value": out["value"] / v64,
                           "path": "plain FP64 kernels + cuFFT, no fusion, same GPU"}
    if world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args)
    if world == 1 and not args.no_batched:
        # the batching pattern on the 48-realisation workload, after this
        # configuration's context is released
        m.close()
        bt = batched_measure(args, rank, world, local, None, baselines=not args.no_fp64)
        keep = ("metric", "value", "unit", "ms_per_step", "cells_per_s", "e2e", "gpu_launches", "fp64_seq", "clocks")
        out["batched"] = {k: bt[k] for k in keep if k in bt}
        out["batched"]["streams"] = bt["config"]["streams"]
        out["batched"]["workload"] = bt["config"]["workload"]
    print(json.dumps(out))


def run_batched(args):
    """The batched workload on its own JSON line (`--config c3`)."""
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    torch.cuda.set_device(local)
    out = batched_measure(args, rank, world, local, dist, baselines=True)
    if out is not None:
        print(json.dumps(out))


def batched_measure(args, rank, world, local, dist, baselines):
    """The batched workload (48 independent realisations at 128^3, 256^3 and
    384^3, one source population each): one captured graph per realisation,
    dealt over autotuned streams.  value = realisations/s of whole passes,
    device-timed; e2e adds, every pass, the copy of every catalogue's Src array
    into pinned host memory; fp64_seq runs the plain FP64 path over the same
    48 configurations one after the other.  Returns the result (rank 0)."""
    import torch
    import colore_gb300 as cg
    from colore_gb300 import inputs

    specs = inputs.batch_specs()
    nreal = len(specs)
    for s in specs:
        s["seed"] = rank_seed(s["seed"], rank * nreal)
    d = tempfile.mkdtemp(prefix="colore_batch_%d_" % rank)
    t = time.perf_counter()
    prms = [cg.Params(inputs.write_inputs(os.path.join(d, "r%02d" % i), s)) for i, s in enumerate(specs)]
    t_params = time.perf_counter() - t
    t = time.perf_counter()
    b = cg.Batch(prms, device=local, nstreams=args.streams)
    t_setup = time.perf_counter() - t
    cells = sum(float(p.config.n_grid) ** 3 for p in prms)

    def barrier():
        if dist:
            dist.barrier()

    for _ in range(args.warmup):
        b.run()
    l0 = sum(m.launches() for m in b.mocks)
    barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        ms = [b.run() for _ in range(args.steps)]
        t_wall = time.perf_counter() - t0
    launches = sum(m.launches() for m in b.mocks) - l0
    t_step = sum(ms) / len(ms) / 1e3
    nsrc = [m.num_sources(0) for m in b.mocks]
    # end to end: every pass also copies each realisation's catalogue (its
    # Src array, the columns the reference's writers take) into pinned host
    # memory, behind the realisation's graph on its stream
    # (cg_batch_set_host_catalog), so the copies overlap the other graphs
    hosts = []
    for i, n in enumerate(nsrc):
        # replays of a realisation repeat its catalogue, so the count of the
        # first pass sizes the buffer (the copy moves up to its size)
        src_i = torch.empty((n + 1024, 9), dtype=torch.float32, pin_memory=True).numpy()
        cnt_i = torch.empty(1, dtype=torch.int64, pin_memory=True).numpy()
        b.set_host_catalog(i, 0, src_i, cnt_i)
        hosts.append((src_i, cnt_i))
    for _ in range(2):  # warm the copies
        b.run()
    e2e_steps = max(10, args.steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d2h = 0
    for _ in range(e2e_steps):
        b.run()
        d2h = sum(int(c[0]) * 36 + 8 for _, c in hosts)
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    if any(int(c[0]) > h.shape[0] for h, c in hosts):
        raise RuntimeError("a host catalogue buffer was too short")
    if dist:
        t_step, t_e2e = max_over_ranks([t_step, t_e2e], dist, "cuda")
    if rank != 0:
        b.close()
        return None
    sizes = sorted({p.config.n_grid for p in prms})
    out = {
        "metric": "realisations/s, batched uneven grids (48 x {128^3, 256^3, 384^3}), FP32 vs sequential FP64",
        "value": world * nreal / t_step, "unit": "realisations/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (EH98 no-wiggle P(k), flat dN/dz, seeds 3001+i, z_max ~ U[0.1,1.2] from seed 3000)",
        "config": {"workload": "c3: %d realisations, grids %s, one population b=1.5, 200/deg^2" % (nreal, sizes),
                   "cells_per_pass": cells, "streams": b.streams, "stream_tuning_ms": b.tuning(),
                   "l2": "inputs larger than L2 for the 256^3 and 384^3 grids (0.07-0.23 GB per field)",
                   "parallelism": "graphs over streams on one GPU; replicas across GPUs"},
        "cells_per_s": world * cells / t_step,
        "e2e": {"value": world * nreal / t_e2e, "unit": "realisations/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(d2h), "ms_per_step": t_e2e * 1e3},
        "gpu_launches": int(launches), "sources_per_realisation": [int(min(nsrc)), int(max(nsrc))],
        "setup_s": {"params_and_tables": round(t_params, 2), "contexts_capture_autotune": round(t_setup, 2)},
        "wall_s_timed": t_wall, "roofline": None,
        "roofline_note": "graph replays carry no per-kernel events; the per-kernel roofline is the 1024^3 line's",
        "clocks": clk.summary(),
    }
    b.close()
    if world == 1 and not args.no_fp64 and baselines:
        t64 = 0.0
        warm = set()
        for p in prms:
            m64 = cg.Mock64(p, device=local)
            if p.config.n_grid not in warm:  # first run of a size loads cuFFT plans
                m64.run()
                warm.add(p.config.n_grid)
            t64 += m64.run()
            m64.close()
        out["fp64_seq"] = {"value": nreal / (t64 / 1e3), "unit": "realisations/s", "ms_per_pass": t64,
                           "speedup_of_value": out["value"] / (nreal / (t64 / 1e3)),
                           "path": "plain FP64 kernels + cuFFT, one realisation after another, same GPU"}
    if world == 1 and not args.no_cpu_baseline and baselines:
        out["cpu_baseline"] = cpu_baseline_batched(args)
    return out


def cpu_baseline_batched(args):
    """The FP64 oracle on one realisation of each grid size of the batch
    (field, density, bins, Poisson totals; OpenMP on every host core),
    scaled to the 48 realisations (16 of each size)."""
    from colore_gb300 import inputs
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    specs = inputs.batch_specs()
    per = {}
    d = tempfile.mkdtemp(prefix="colore_cpub_")
    for s in specs:
        n = s["n_grid"]
        if n in per:
            continue
        c = orc.Params(inputs.write_inputs(os.path.join(d, str(n)), s))
        cfg = c.config
        t = time.perf_counter()
        dens, npot, st = orc.field64(cfg)
        dens = orc.density64(cfg, dens, st[3])
        tabs, e0f, nz = orc.norm_tables64(cfg, dens)
        lam = orc.lambda64(cfg, 0, dens, tabs[0], e0f[0])
        orc.poisson_total64(cfg, 0, lam)
        per[n] = time.perf_counter() - t
    counts = {}
    for s in specs:
        counts[s["n_grid"]] = counts.get(s["n_grid"], 0) + 1
    est = sum(per[n] * counts[n] for n in per)
    cores = os.cpu_count()
    return {"value": len(specs) / est, "unit": "realisations/s", "cores": cores, "kind": "port",
            "sample": "FP64 oracle, %d OpenMP threads, one realisation per grid size timed (%s s) and scaled to "
                      "the 48 (catalogue positions not drawn)" % (cores, {k: round(v, 2) for k, v in per.items()})}


def _kappa_steps(cfg):
    """Ray steps of kappa_get_beam_properties (kappa.c:146-162) for cfg."""
    nr = cfg.n_grid // 2
    dr = cfg.r_max / nr
    rmax = max(float(np.float32(cfg.kappa_r[i])) for i in range(cfg.n_kappa))
    last = min(int(rmax / dr + 0.5), nr - 1)
    return 12 * cfg.nside_kappa ** 2 * (last + 1)


def cpu_baseline(args):
    """The FP64 oracle (the reference's arithmetic; OpenMP on every host core)
    timed stage by stage on a sample of the workload and scaled to it:
      field/1LPT FFT stages at cpu_n^3, scaled by cells x log2 N;
      density, bins and Poisson stages at cpu_n^3, scaled by cells;
      intensity maps: every iz_stride-th plane of the cpu_n^3 grid gives the
        sub-samples/s, times the exact sub-sample count of the full grid;
      kappa: every pix_stride-th pixel gives the ray steps/s, times the full
        grid's ray steps."""
    import numpy as np
    from colore_gb300 import inputs
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    full = config_spec(args.config, args.n)
    ns_ = args.cpu_n
    d = tempfile.mkdtemp(prefix="colore_cpu_")
    prm_f = orc.Params(inputs.write_inputs(os.path.join(d, "full"), full))
    cf = prm_f.config
    nf = cf.n_grid
    prm = orc.Params(inputs.write_inputs(os.path.join(d, "sample"), config_spec(args.config, ns_)))
    c = prm.config
    T = {}
    t = time.perf_counter()
    dens, npot, st = orc.field64(c)
    T["field"] = time.perf_counter() - t
    t = time.perf_counter()
    if c.dens_type == 1:
        dens, _ = orc.lpt64(c, dens)
    else:
        dens = orc.density64(c, dens, st[3])
    T["density"] = time.perf_counter() - t
    t = time.perf_counter()
    tabs, e0f, nz = orc.norm_tables64(c, dens)
    T["bins"] = time.perf_counter() - t
    t = time.perf_counter()
    nsrc = 0
    for i in range(c.n_srcs):
        lam = orc.lambda64(c, i, dens, tabs[i], e0f[i])
        nsrc += orc.poisson_total64(c, i, lam)
    T["sources"] = time.perf_counter() - t
    R = (nf / ns_) ** 3
    lg = np.log2(nf) / np.log2(ns_)
    parts = {"field": T["field"] * R * lg, "density": T["density"] * R * (lg if c.dens_type == 1 else 1),
             "bins": T["bins"] * R, "sources": T["sources"] * R}
    est = sum(parts.values())
    if c.n_imap:
        stride = max(1, ns_ // 16)
        t = time.perf_counter()
        done = 0
        for i in range(c.n_imap):
            done += orc.imap64_part(c, i, dens, npot, tabs[c.n_srcs + i], e0f[c.n_srcs + i], stride)
        ti = time.perf_counter() - t
        need = sum(orc.imap_samples(cf, i) for i in range(cf.n_imap))
        parts["imap"] = need / max(done, 1) * ti
        est += parts["imap"]
    if c.do_kappa:
        ps = 64
        t = time.perf_counter()
        orc.kappa64_part(c, npot, ps)
        tk = time.perf_counter() - t
        parts["kappa"] = _kappa_steps(cf) / (_kappa_steps(c) / ps) * tk
        est += parts["kappa"]
    cores = os.cpu_count()
    return {"value": nf ** 3 / est, "unit": "cells/s", "cores": cores, "kind": "port",
            "sample": ("FP64 oracle of the reference path, %d OpenMP threads: stages timed at %d^3 and scaled to "
                       "%d^3 (FFT by N^3 log N, cell stages by N^3), imap by sub-sample count, kappa by ray steps; "
                       "estimated %.1f s per full step") % (cores, ns_, nf, est),
            "stage_s_full_step": {k: round(v, 3) for k, v in parts.items()},
            "stage_s_sample": {k: round(v, 4) for k, v in T.items()}}


def workload_config(args, cfg):
    """The `config` object of both arms: the workload and its sizes."""
    n = cfg.n_grid
    gb = (n * n * 2 * (n // 2 + 1) * 4) / 1e9
    return {"workload": "%s: %d^3, dens_type %d, %d source pops, %d imap shells nside %s, %d kappa planes"
                        % (args.config, n, cfg.dens_type, cfg.n_srcs, sum(cfg.imap_nr[i] for i in range(cfg.n_imap)),
                           [cfg.nside_imap[i] for i in range(cfg.n_imap)], cfg.n_kappa if cfg.do_kappa else 0),
            "n_grid": n, "l2": "inputs larger than L2 (%.1f GB per field)" % gb, "parallelism": "replicas"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from colore_gb300 import inputs
    # the CPU arm loads the oracle library alone (its own build of the host
    # param reader and tables), never the GPU library
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    prm = orc.Params(inputs.write_inputs(tempfile.mkdtemp(prefix="colore_ref_"), config_spec(args.config, args.n)))
    # warm-up steps: the oracle library loaded and its OpenMP pool running, on
    # the same configuration at 64^3 (each timed step is a bounded sample of
    # the full workload)
    small = orc.Params(inputs.write_inputs(tempfile.mkdtemp(prefix="colore_refw_"), config_spec(args.config, 64)))
    for _ in range(args.warmup):
        orc.field64(small.config)
    vals = []
    cb = None
    for _ in range(max(1, args.steps)):
        cb = cpu_baseline(args)
        vals.append(cb["value"])
    v = sum(vals) / len(vals)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cells/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": workload_config(args, prm.config),
           "cpu_baseline": dict(cb, value=v),
           "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c4")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 baseline path")
    ap.add_argument("--n", type=int, default=0, help="override the grid size")
    ap.add_argument("--cpu-n", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--streams", type=int, default=0, help="batched workload: streams (0 autotunes)")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-workload measurement")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "c3":
        run_batched(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
