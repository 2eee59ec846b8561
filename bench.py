#!/usr/bin/env python
"""Benchmark of the GB300 elastic time step: grid-point-steps/s on the 512^3
layer-over-halfspace workload (free surface on top, supergrid on the other five
sides, moment-tensor point source), FP64, one GPU.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A "step" is one full time step of the fused path (predictor stage, one-sided rows,
forcing, boundary closures, corrector stage with supergrid damping).  Inputs are
resident in HBM (3.3 GB per 3-component field, far above the 129 MB L2, so no L2
flush is needed between steps).  Prints one JSON line on rank 0.

--impl reference times the reference's own CPU implementation of the step on the
host cores (oracle/_ref where it was built here, else the oracle restatement of
the reference kernels) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid-pt-steps/s FP64 vs mixed at stated L2 err; HBM GB/s vs peak; adjoint/fwd time"
UNIT = "grid-pt-steps/s"


# --------------------------------------------------------------------------
# Workload: 512^3, h = 50 m, 1 km layer (vp 4000, vs 2000, rho 2600) over a
# half-space (vp 6000, vs 3464, rho 2700); free surface on top, supergrid (30
# points) on the other sides; Mxy = 1e18 N m at 2 km depth, Gaussian moment rate
# with sigma = 0.05 s (freq 20), t0 = 0.3 s; dt from CFL 1.3.
# --------------------------------------------------------------------------
def c2_config(n=512):
    return dict(nx=n, ny=n, nz=n, h=50.0, bc=(2, 2, 2, 2, 0, 2), sg_gp=30, sg_damping=0.02,
                layer_depth=1000.0, layer=(4000.0, 2000.0, 2600.0), half=(6000.0, 3464.0, 2700.0),
                src=dict(x=(n - 1) * 50.0 / 2, y=(n - 1) * 50.0 / 2, z=2000.0,
                         moment=(0.0, 1e18, 0.0, 0.0, 0.0, 0.0), freq=20.0, t0=0.3),
                cfl=1.3)


def layered_material(cfg):
    nx, ny, nz, h = cfg["nx"], cfg["ny"], cfg["nz"], cfg["h"]
    kk = np.arange(-1, nz + 3)
    z = (kk - 1) * h
    vp = np.where(z <= cfg["layer_depth"], cfg["layer"][0], cfg["half"][0])
    vs = np.where(z <= cfg["layer_depth"], cfg["layer"][1], cfg["half"][1])
    rh = np.where(z <= cfg["layer_depth"], cfg["layer"][2], cfg["half"][2])
    mu_k = rh * vs * vs
    la_k = rh * vp * vp - 2 * mu_k
    plane = (ny + 4) * (nx + 4)
    rho = np.repeat(rh, plane)
    mu = np.repeat(mu_k, plane)
    la = np.repeat(la_k, plane)
    return rho, mu, la


def cfl_dt(cfg):
    vmax2 = max(cfg["layer"][0] ** 2 + 2 * cfg["layer"][1] ** 2,
                cfg["half"][0] ** 2 + 2 * cfg["half"][1] ** 2)
    return cfg["cfl"] * cfg["h"] / np.sqrt(vmax2)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# algorithmic bytes per interior point of one corrector stage: reads Up, U, Um (9
# words) and mu, lambda, rho (3), writes the new level (3): 15 FP64 words
CORR_STAGE_WORDS = 15
# DRAM bytes per interior point of the FP64 corrector stage kernel, from one ncu
# capture of the 192^3 case (dram__bytes_read.sum + dram__bytes_write.sum = 2.1133e9 B
# over 7,077,888 interior points); traffic grows with the point count, so a launch
# moves this many bytes per point at any size
CORR_STAGE_DRAM_BYTES_PER_PT = 298.6
# FP64-pipe warp instructions per interior point of the FP64 stage kernels on the
# 512^3 workload (smsp__inst_executed_pipe_fp64.sum, single-pass ncu captures of the
# full-size run: corrector 830,809,640 and predictor 671,186,048 over 512^3 points).  The pipe issues
# 2 FP64 thread instructions per clock per SM, i.e. one warp instruction per 16 clocks.
FP64_WARP_INST_PER_PT = {"corr": 830809640 / 512 ** 3, "pred": 671186048 / 512 ** 3}
FP64_THREAD_INST_PER_CLK_PER_SM = 2
# mixed form, corrector stage: reads Up, U, Um as double-float pairs (9 x 8 B), mu,
# lambda, rho in FP32 (3 x 4 B), writes the new level (3 x 8 B): the compulsory bytes
# of an all-FP32-coefficient stage
MIXED_CORR_STAGE_BYTES = 9 * 8 + 3 * 4 + 3 * 8
# DRAM bytes per interior point the tensor-copy corrector stage moves (ncu, 256^3:
# 3.445e9 read + 0.394e9 written over 256^3 points): the levels, the (hi, lo)
# coefficient pairs of mu, lambda, 1/rho and the twelve weight arrays
MIXED_CORR_STAGE_DRAM_BYTES_PER_PT = 228.8


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------------------
# CPU baseline: the reference's CPU step on the host cores, on the same workload.
# Built from oracle/ alone (no product code): the reference's own kernels
# (oracle/_ref, compiled from the reference sources where they are present) or
# else the oracle's restatement of them, both OpenMP over every host core.
# --------------------------------------------------------------------------
def cpu_rate(n, steps, warmup=1, which=None):
    """Grid-point-steps/s of `steps` CPU time steps of the C2 workload at n^3 after
    `warmup` untimed ones, on the reference's kernels where they were built here
    (which="ref") or else on the oracle restatement ("oracle"); returns (rate,
    seconds, kind, cores)."""
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    from oracle import oracle as O
    O.lib()
    if which is None:
        which = "ref" if O.ref_available() else "oracle"
    cfg = c2_config(n)
    rho, mu, la = layered_material(cfg)
    sc = cfg["src"]
    src = O.PointSource(sc["x"], sc["y"], sc["z"], moment=sc["moment"], freq=sc["freq"], t0=sc["t0"],
                        kind=0)  # Gaussian
    prob = O.CartProblem(n, n, n, cfg["h"], cfg["bc"], rho, mu, la, cfl_dt(cfg), [src],
                         sg_gp=cfg["sg_gp"], sg_damping=cfg["sg_damping"])
    n3 = 3 * prob.npts
    u, um, up, lu, f, uacc = (np.zeros(n3) for _ in range(6))
    t = 0.0
    for _ in range(warmup):
        O.step(prob.P, 1, t, up, u, um, lu, f, uacc, which=which)
        um, u, up = u, up, um
        t += prob.P.dt
    t0 = time.perf_counter()
    for _ in range(steps):
        O.step(prob.P, 1, t, up, u, um, lu, f, uacc, which=which)
        um, u, up = u, up, um
        t += prob.P.dt
    el = time.perf_counter() - t0
    kind = "reference" if which == "ref" else "port"
    return n ** 3 * steps / el, el, kind, int(os.environ["OMP_NUM_THREADS"])


def run_reference(args, rank, world):
    """Reference arm: the reference's CPU step on the host cores, same workload."""
    if rank != 0:
        return 0
    n = args.n
    rate, el, kind, cores = cpu_rate(n, args.steps, args.warmup)
    src = ("the reference's own kernels (oracle/_ref)" if kind == "reference"
           else "the oracle restatement of the reference kernels")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"C2 layer-over-halfspace {n}^3 h=50, FP64 time step (CPU)",
                   "grid": [n, n, n]},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"{args.steps} time steps of the {n}^3 workload after "
                                   f"{args.warmup} untimed ({el:.1f} s; {src}, OpenMP)"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def _make_ew(sg, cfg, n, precision, stream):
    g = sg.grid_desc(n, n, n, cfg["h"], bc=cfg["bc"], sg_gp=cfg["sg_gp"],
                     sg_damping=cfg["sg_damping"], precision=precision)
    ew = sg.EW(g, stream=stream)
    rho, mu, la = layered_material(cfg)
    ew.set_material(rho, mu, la)
    ew.add_source(sg.source_desc(cfg["src"]["x"], cfg["src"]["y"], cfg["src"]["z"],
                                 moment=cfg["src"]["moment"], freq=cfg["src"]["freq"],
                                 t0=cfg["src"]["t0"], kind=sg.GAUSSIAN))
    ew.set_time_step(cfl_dt(cfg), 0.0)
    return ew


def _time_form(args, sg, torch, precision, stream, world, local):
    """Warm up, then time args.steps steps of one form (CUDA events on its stream);
    per-kernel times; end-to-end run through the C ABI with pinned host buffers."""
    n = args.n
    cfg = c2_config(n)
    ew = _make_ew(sg, cfg, n, precision, stream)
    mode = sg.MODE_FUSED if args.mode == "fused" else sg.MODE_PHASES
    npts_int = n ** 3
    with torch.cuda.stream(stream):
        ew.step(args.warmup, mode)
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clocks:
            torch.cuda.synchronize()
            e0.record(stream)
            ew.step(args.steps, mode)
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
    barrier(world)
    ms = max_over_ranks(ms, world)
    ms_step = ms / args.steps
    out = {"value": world * npts_int / (ms_step * 1e-3), "ms_per_step": ms_step,
           "clocks": clocks.summary(), "gpu_launches": ew.launches_per_step(mode) * args.steps}
    out["kernel_ms"] = ew.profile_kernels(nrep=3)
    if not args.no_e2e:
        n3 = 3 * ew.npts
        hu = torch.zeros(n3, dtype=torch.float64, pin_memory=True)
        hum = torch.zeros(n3, dtype=torch.float64, pin_memory=True)
        ew.get_fields(hu, hum)
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        with torch.cuda.stream(stream):
            ew.set_fields(hu, hum)
            ew.step(args.steps, mode)
            ew.get_fields(hu, None)
        torch.cuda.synchronize()
        el = max_over_ranks(time.perf_counter() - t0, world)
        out["e2e"] = {"value": world * npts_int * args.steps / el, "unit": UNIT,
                      "h2d_bytes_per_step": int(2 * n3 * 8 / args.steps),
                      "d2h_bytes_per_step": int(n3 * 8 / args.steps)}
        del hu, hum
    ew.close()
    torch.cuda.empty_cache()
    return out


def c3_config(nx=384, ny=384, nz_total=128):
    """Topography workload: a curvilinear grid over a 1 km Gaussian hill (width
    3 km) at the domain centre on top of a Cartesian grid, 384 x 384 x 128 points
    in all at h = 50 m; the interface between the grids at z = 2000 m.  Material
    vs = 2000 + 0.5 depth, vp = sqrt(3) vs, rho = 2500 below the surface.  A
    vertical point force 3 km below the datum z = 0 under the hill top (in the
    Cartesian grid), Gaussian (sigma 0.05 s)."""
    h = 50.0
    return dict(nx=nx, ny=ny, nz_total=nz_total, h=h, zmax_topo=2000.0, amp=1000.0,
                xc=(nx - 1) * h / 2, yc=(ny - 1) * h / 2, lx=3000.0, ly=3000.0, vs0=2000.0,
                grad=0.5, rho=2500.0, gp=30, damping=0.02,
                src=dict(x=(nx - 1) * h / 2, y=(ny - 1) * h / 2, z=3000.0, force=(0.0, 0.0, 1e15),
                         freq=20.0, t0=0.3),
                cfl=1.3)


def _make_topo_ew(sg, cfg, stream, precision=0):
    """The C3 EW object: the curvilinear grid's point count comes from the
    topography (1 + round((zmax - z_avg)/h)); the Cartesian grid takes the rest of
    the nz_total planes (the grids share the interface plane)."""
    import torch
    h, nx, ny = cfg["h"], cfg["nx"], cfg["ny"]
    topo = sg.topo_desc(cfg["amp"], cfg["xc"], cfg["yc"], cfg["lx"], cfg["ly"])
    i = np.arange(-1, nx + 3)
    j = np.arange(-1, ny + 3)
    X, Y = np.meshgrid((i - 1) * h, (j - 1) * h, indexing="xy")
    zs = -cfg["amp"] * np.exp(-((X - cfg["xc"]) / cfg["lx"]) ** 2 - ((Y - cfg["yc"]) / cfg["ly"]) ** 2)
    nc = 1 + int(round((cfg["zmax_topo"] - 0.5 * (zs.min() + zs.max())) / h))
    ncart = cfg["nz_total"] - (nc - 1)
    g = sg.grid_desc(nx, ny, ncart, h, bc=(2, 2, 2, 2, sg.INTERFACE, 2), zmin=cfg["zmax_topo"],
                     sg_gp=cfg["gp"], sg_damping=cfg["damping"], precision=precision)
    ew = sg.EW(g, stream=stream, topo=topo)
    assert ew.grid_dims(1)[2] == nc

    def material(z_planes, grid_shape):
        depth = torch.clamp(z_planes - torch.from_numpy(zs).to("cuda"), min=0.0)
        vs = cfg["vs0"] + cfg["grad"] * depth
        rho = torch.full_like(vs, cfg["rho"])
        mu = rho * vs * vs
        la = rho * 3.0 * vs * vs - 2 * mu
        return [a.reshape(-1).contiguous() for a in (rho, mu, la)]

    kk = torch.arange(-1, ncart + 3, dtype=torch.float64, device="cuda")
    zc = (cfg["zmax_topo"] + (kk - 1) * h)[:, None, None].expand(ncart + 4, ny + 4, nx + 4)
    ew.set_material(*material(zc, None))
    n1 = ew.grid_dims(1)[3]
    z1 = torch.zeros(n1, dtype=torch.float64, device="cuda")
    ew.curvilinear_arrays(z=z1)
    ew.set_material_grid(1, *material(z1.reshape(nc + 4, ny + 4, nx + 4), None))
    sc = cfg["src"]
    ew.add_source(sg.source_desc(sc["x"], sc["y"], sc["z"], force=sc["force"], freq=sc["freq"],
                                 t0=sc["t0"], kind=sg.GAUSSIAN))
    # dt from the CFL number of both grids, landing on t = 1 s
    dt, _ = ew.compute_time_step(cfg["cfl"], 1.0)
    ew.set_time_step(dt, 0.0)
    return ew, nc, ncart, dt


def _time_topo(args, sg, torch, stream, world, precision=0):
    """C3: timed fused steps of both grids (FP64, or FP32-mixed: FP32 interior
    stencils, FP64 SBP top rows, curvilinear free surface and metric
    coefficients, double-float levels); end-to-end through the C ABI with both
    grids' levels in pinned host memory."""
    cfg = c3_config(args.topo_nx, args.topo_nx, args.topo_nz)
    ew, nc, ncart, dt = _make_topo_ew(sg, cfg, stream, precision)
    nx, ny = cfg["nx"], cfg["ny"]
    pts = nx * ny * (ncart + nc)  # interior points of both grids
    with torch.cuda.stream(stream):
        ew.step(args.warmup, sg.MODE_FUSED)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ew.step(args.steps, sg.MODE_FUSED)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1), world) / args.steps
    out = {"value": world * pts / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms,
           "grids": {"cartesian": [nx, ny, ncart], "curvilinear": [nx, ny, nc]},
           "dt": dt, "gpu_launches": ew.launches_per_step(sg.MODE_FUSED) * args.steps,
           "workload": f"C3 Gaussian-hill topography {nx}x{ny}x{cfg['nz_total']} h=50, "
                       + ("FP64" if precision == 0 else "FP32-mixed") +
                       ", fused Cartesian and curvilinear stage kernels"}
    if not args.no_e2e:
        n0, n1 = 3 * ew.grid_dims(0)[3], 3 * ew.grid_dims(1)[3]
        hb = [torch.zeros(n, dtype=torch.float64, pin_memory=True) for n in (n0, n0, n1, n1)]
        ew.get_fields(hb[0], hb[1])
        ew.get_fields_grid(1, hb[2], hb[3])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(stream):
            ew.set_fields(hb[0], hb[1])
            ew.set_fields_grid(1, hb[2], hb[3])
            ew.step(args.steps, sg.MODE_FUSED)
            ew.get_fields(hb[0], None)
            ew.get_fields_grid(1, hb[2], None)
        torch.cuda.synchronize()
        el = max_over_ranks(time.perf_counter() - t0, world)
        out["e2e"] = {"value": world * pts * args.steps / el, "unit": UNIT,
                      "h2d_bytes_per_step": int(2 * (n0 + n1) * 8 / args.steps),
                      "d2h_bytes_per_step": int((n0 + n1) * 8 / args.steps)}
    ew.close()
    torch.cuda.empty_cache()
    return out


def _topo_mixed_error(args, sg, torch, stream, nsteps):
    """Relative L2 error of the FP32-mixed two-grid run against the FP64 run after
    nsteps steps from rest (the C3 shot), over both grids' fields."""
    cfg = c3_config(args.topo_nx, args.topo_nx, args.topo_nz)
    res = []
    for prec in (0, 1):
        ew, nc, ncart, dt = _make_topo_ew(sg, cfg, stream, prec)
        with torch.cuda.stream(stream):
            ew.step(nsteps, sg.MODE_FUSED)
        n0, n1 = 3 * ew.grid_dims(0)[3], 3 * ew.grid_dims(1)[3]
        u0 = torch.zeros(n0, dtype=torch.float64, device="cuda")
        u1 = torch.zeros(n1, dtype=torch.float64, device="cuda")
        ew.get_fields(u0, None)
        ew.get_fields_grid(1, u1, None)
        torch.cuda.synchronize()
        res.append((u0, u1))
        ew.close()
    (a0, a1), (b0, b1) = res
    num = float(torch.sum((b0 - a0) ** 2) + torch.sum((b1 - a1) ** 2))
    den = float(torch.sum(a0 ** 2) + torch.sum(a1 ** 2))
    lin = max(float(torch.max(torch.abs(b0 - a0))), float(torch.max(torch.abs(b1 - a1))))
    amax = max(float(torch.max(torch.abs(a0))), float(torch.max(torch.abs(a1))))
    del res, a0, a1, b0, b1
    torch.cuda.empty_cache()
    return {"steps": nsteps, "l2_rel": (num / den) ** 0.5 if den > 0 else None,
            "linf_rel": lin / amax if amax > 0 else None,
            "against": "FP64 two-grid run, both grids' final displacement"}


def c4_config(n=256):
    """Adjoint workload: a 5% log-normal medium (Gaussian correlation length 10h,
    seeded) around vp 6000, vs 3464, rho 2700 on an n^3 grid at h = 50 m with
    supergrid on all sides; one vertical point force at the centre (Gaussian,
    sigma 0.05 s); 16 receivers at seeded interior points; the observed data are
    the records of the same shot in the homogeneous background."""
    return dict(n=n, h=50.0, vp=6000.0, vs=3464.0, rho=2700.0, std=0.05, corr=10.0, seed=4242,
                gp=30, src=dict(force=(0.0, 0.0, 1e15), freq=20.0, t0=0.3), nrec=16, cfl=1.3)


def _lognormal(torch, shape, std, corr, seed):
    """exp(std * g), g a unit-variance Gaussian random field with Gaussian
    correlation length `corr` points (white noise filtered in Fourier space)."""
    gen = torch.Generator(device="cuda").manual_seed(seed)
    w = torch.randn(shape, generator=gen, dtype=torch.float64, device="cuda")
    f = torch.fft.rfftn(w)
    ks = [torch.fft.fftfreq(s, device="cuda", dtype=torch.float64) for s in shape[:-1]]
    ks.append(torch.fft.rfftfreq(shape[-1], device="cuda", dtype=torch.float64))
    K = sum(k.reshape([-1 if d == a else 1 for d in range(3)]) ** 2 for a, k in enumerate(ks))
    g = torch.fft.irfftn(f * torch.exp(-0.5 * (2 * np.pi * corr) ** 2 * K), s=shape)
    g = (g - g.mean()) / g.std()
    return torch.exp(std * g)


def _make_c4(sg, torch, cfg, stream, nsteps, homogeneous=False, dt=None, precision=None):
    n, h = cfg["n"], cfg["h"]
    g = sg.grid_desc(n, n, n, h, bc=(2,) * 6, sg_gp=cfg["gp"],
                     precision=sg.FP64 if precision is None else precision)
    shape = (n + 4, n + 4, n + 4)
    if homogeneous:
        pr = ps = pv = torch.ones(shape, dtype=torch.float64, device="cuda")
    else:
        pr, ps, pv = (_lognormal(torch, shape, cfg["std"], cfg["corr"], cfg["seed"] + q)
                      for q in range(3))
    rho = cfg["rho"] * pr
    vs = cfg["vs"] * ps
    vp = cfg["vp"] * pv
    mu = rho * vs * vs
    la = rho * vp * vp - 2 * mu
    ew = sg.EW(g, stream=stream)
    mat = [a.reshape(-1).contiguous() for a in (rho, mu, la)]
    ew.set_material(*mat)
    c = (n - 1) * h / 2
    sc = cfg["src"]
    ew.add_source(sg.source_desc(c, c, c, force=sc["force"], freq=sc["freq"], t0=sc["t0"],
                                 kind=sg.GAUSSIAN))
    if dt is None:
        dt = cfg["cfl"] * h / float(torch.sqrt(((4 * mu + la) / rho).max()))
    ew.set_time_step(dt, 0.0)
    rng = np.random.default_rng(cfg["seed"])
    rec = [tuple(int(x) for x in rng.integers(cfg["gp"] + 2, n - cfg["gp"], size=3))
           for _ in range(cfg["nrec"])]
    ew.set_receivers(rec, [sg.REC_DISPLACEMENT] * len(rec), nsteps + 1)
    return ew, dt


def _time_adjoint(args, sg, torch, stream):
    """Forward solve and misfit gradient of the adjoint workload, each timed with
    CUDA events on the EW stream; the ratio is the gradient's cost in forward
    solves.  The gradient keeps as many segments of its forward run as the free
    device memory holds (the rest are recomputed from checkpoints), so the ratio is
    measured at the workload's full length.  The observed data (records of the same
    shot in the homogeneous background) come from the FP32-mixed solver: any data
    serve, and the timed runs are FP64."""
    cfg = c4_config(args.adj_n)
    N, C = args.adj_steps, args.adj_ckpt
    with torch.cuda.stream(stream):
        ew, dt = _make_c4(sg, torch, cfg, stream, N)
        ew.close()
        ew0, _ = _make_c4(sg, torch, cfg, stream, N, homogeneous=True, dt=dt, precision=sg.MIXED)
        ew0.step(N, sg.MODE_FUSED)
        obs = torch.zeros(ew0.record_shape(), dtype=torch.float64, device="cuda")
        ew0.records(obs)
        torch.cuda.synchronize()
        ew0.close()
        ew, _ = _make_c4(sg, torch, cfg, stream, N, dt=dt)
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        torch.cuda.synchronize()
        e[0].record(stream)
        ew.step(N, sg.MODE_FUSED)
        e[1].record(stream)
        torch.cuda.synchronize()
        ew.close()
        ew, _ = _make_c4(sg, torch, cfg, stream, N, dt=dt)
        g = [torch.zeros(ew.npts, dtype=torch.float64, device="cuda") for _ in range(3)]
        torch.cuda.synchronize()
        e[2].record(stream)
        J = ew.gradient(N, C, obs, *g)
        e[3].record(stream)
        torch.cuda.synchronize()
        ew.close()
    fwd_ms, grad_ms = e[0].elapsed_time(e[1]), e[2].elapsed_time(e[3])
    n = cfg["n"]
    return {"workload": f"C4 adjoint {n}^3, 5% log-normal medium, 1 point force, 16 receivers, "
                        f"{N} steps, checkpoints every {C}",
            "forward_ms": fwd_ms, "gradient_ms": grad_ms, "gradient_over_forward": grad_ms / fwd_ms,
            "misfit": J, "grad_norms": [float(x.norm()) for x in g],
            "forward_value": n ** 3 * N / (fwd_ms * 1e-3), "unit": UNIT}


def c5_config(n=256):
    """Multi-shot workload: the adjoint workload's medium, receivers and source time
    function, 16 vertical point forces at seeded interior points outside the
    supergrid layers; observed data are each shot's records in the homogeneous
    background (FP32-mixed forward)."""
    cfg = c4_config(n)
    rng = np.random.default_rng(cfg["seed"] + 100)
    lo, hi = (cfg["gp"] + 4) * cfg["h"], (n - 5 - cfg["gp"]) * cfg["h"]
    cfg["shots"] = [tuple(float(x) for x in rng.uniform(lo, hi, size=3)) for _ in range(16)]
    return cfg


def _c5_ew(sg, torch, cfg, stream, nsteps, precision, mat, dt):
    n, h = cfg["n"], cfg["h"]
    g = sg.grid_desc(n, n, n, h, bc=(2,) * 6, sg_gp=cfg["gp"], precision=precision)
    ew = sg.EW(g, stream=stream)
    ew.set_material(*mat)
    ew.set_time_step(dt, 0.0)
    rng = np.random.default_rng(cfg["seed"])
    rec = [tuple(int(x) for x in rng.integers(cfg["gp"] + 2, n - cfg["gp"], size=3))
           for _ in range(cfg["nrec"])]
    ew.set_receivers(rec, [sg.REC_DISPLACEMENT] * len(rec), nsteps + 1)
    ew.set_graphs(True)
    return ew


def _c5_medium(torch, cfg, homogeneous):
    n = cfg["n"]
    shape = (n + 4, n + 4, n + 4)
    if homogeneous:
        pr = ps = pv = torch.ones(shape, dtype=torch.float64, device="cuda")
    else:
        pr, ps, pv = (_lognormal(torch, shape, cfg["std"], cfg["corr"], cfg["seed"] + q) for q in range(3))
    rho = cfg["rho"] * pr
    mu = rho * (cfg["vs"] * ps) ** 2
    la = rho * (cfg["vp"] * pv) ** 2 - 2 * mu
    return [a.reshape(-1).contiguous() for a in (rho, mu, la)]


def _c5_shot(sg, ew, cfg, s):
    sc = cfg["src"]
    x, y, z = cfg["shots"][s]
    ew.clear_sources()
    ew.add_source(sg.source_desc(x, y, z, force=sc["force"], freq=sc["freq"], t0=sc["t0"],
                                 kind=sg.GAUSSIAN))


def _c5_observed(sg, torch, cfg, stream, N, shots, dt):
    """Observed data of the shots: FP32-mixed forward runs in the homogeneous background."""
    ew0 = _c5_ew(sg, torch, cfg, stream, N, sg.MIXED, _c5_medium(torch, cfg, True), dt)
    zero = torch.zeros(3 * ew0.npts, dtype=torch.float64, device="cuda")
    obs = []
    for s in shots:
        _c5_shot(sg, ew0, cfg, s)
        ew0.set_time_step(dt, 0.0)
        ew0.set_receivers(*_c5_receivers(cfg), N + 1)
        ew0.set_fields(zero, zero)
        ew0.step(N, sg.MODE_FUSED)
        o = torch.zeros(ew0.record_shape(), dtype=torch.float64, device="cuda")
        ew0.records(o)
        obs.append(o)
    ew0.close()
    return obs


def _c5_gradients(sg, torch, cfg, stream, mat, dt, N, C, shots, obs, prec, keep_after=0):
    """The summed gradient over the shots in one precision (FP64 accumulation on the
    device), each shot's gradient() timed by CUDA events; with keep_after = E > 0 also
    a copy of the sum after the first E shots."""
    ew = _c5_ew(sg, torch, cfg, stream, N, prec, mat, dt)
    zero = torch.zeros(3 * ew.npts, dtype=torch.float64, device="cuda")
    tot = [torch.zeros(ew.npts, dtype=torch.float64, device="cuda") for _ in range(3)]
    g = [torch.zeros(ew.npts, dtype=torch.float64, device="cuda") for _ in range(3)]
    ms, J, part = [], 0.0, None
    for n, (s, o) in enumerate(zip(shots, obs)):
        _c5_shot(sg, ew, cfg, s)
        ew.set_time_step(dt, 0.0)
        ew.set_fields(zero, zero)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        J += ew.gradient(N, C, o, *g)
        for q in range(3):
            tot[q] += g[q]  # FP64 accumulation over shots, on the device
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
        if n + 1 == keep_after:
            part = [x.clone() for x in tot]
    ew.close()
    return dict(ms=ms, J=J, tot=tot, part=part)


def _time_multishot(args, sg, torch, stream):
    """C5: the summed misfit gradient over point-force shots, FP32-mixed (double-float
    levels, FP32 stencils and gradient terms) with FP64 accumulation, every time loop
    replayed as CUDA graphs.  Per-shot time from CUDA events on args.ms_shots shots at
    the workload's length (args.ms_steps); the error of the mixed sum over the first
    args.ms_err_shots shots against the FP64 gradients of the same shots at
    args.ms_err_steps steps (the timed run's partial sum when the lengths agree)."""
    cfg = c5_config(args.adj_n)
    N, C, S = args.ms_steps, args.adj_ckpt, args.ms_shots
    E = min(args.ms_err_shots, len(cfg["shots"]))
    n = cfg["n"]
    with torch.cuda.stream(stream):
        mat = _c5_medium(torch, cfg, False)
        dt = cfg["cfl"] * cfg["h"] / float(torch.sqrt(((4 * mat[1] + mat[2]) / mat[0]).max()))
        shots = list(range(S))
        obs = _c5_observed(sg, torch, cfg, stream, N, shots, dt)
        reuse = E > 0 and E <= S and args.ms_err_steps == N
        mx = _c5_gradients(sg, torch, cfg, stream, mat, dt, N, C, shots, obs, sg.MIXED,
                           keep_after=E if reuse else 0)
        res = {"workload": f"C5 multi-shot gradient {n}^3, C4 medium, point-force shots, 16 receivers, "
                           f"{N} steps, checkpoints every {C}, FP32-mixed with FP64 accumulation, "
                           "time loops as CUDA graphs",
               "shots": S, "of_shots": len(cfg["shots"]), "steps": N,
               "per_shot_ms": sum(mx["ms"]) / len(mx["ms"]), "total_ms": sum(mx["ms"]),
               "misfit": mx["J"], "grad_norms": [float(x.norm()) for x in mx["tot"]]}
        if E > 0:
            M = args.ms_err_steps
            if reuse:
                a_tot, a_ms = mx["part"], sum(mx["ms"][:E]) / E
                eobs = obs[:E]
            else:
                eobs = _c5_observed(sg, torch, cfg, stream, M, list(range(E)), dt)
                a = _c5_gradients(sg, torch, cfg, stream, mat, dt, M, C, list(range(E)), eobs, sg.MIXED)
                a_tot, a_ms = a["tot"], sum(a["ms"]) / E
            del mx, obs
            b = _c5_gradients(sg, torch, cfg, stream, mat, dt, M, C, list(range(E)), eobs, sg.FP64)
            res["error_vs_fp64"] = {
                "shots": E, "steps": M,
                "mixed_per_shot_ms": a_ms, "fp64_per_shot_ms": sum(b["ms"]) / E,
                "l2_rel": [float((x - y).norm() / y.norm()) for x, y in zip(a_tot, b["tot"])],
                "linf_rel": [float((x - y).abs().max() / y.abs().max()) for x, y in zip(a_tot, b["tot"])],
                "against": "sum of the FP64 gradients of the same shots (rho, mu, lambda)"}
            del b
        torch.cuda.empty_cache()
    return res


def _c5_receivers(cfg):
    n = cfg["n"]
    rng = np.random.default_rng(cfg["seed"])
    rec = [tuple(int(x) for x in rng.integers(cfg["gp"] + 2, n - cfg["gp"], size=3))
           for _ in range(cfg["nrec"])]
    import sw4lite_gb300 as sg
    return rec, [sg.REC_DISPLACEMENT] * len(rec)


RECEIVER_SEED = 20240611


def c2_receivers(cfg, n, nrec=8):
    """The workload's 8 surface receivers: (x, y) uniform over the interior outside
    the supergrid layers, z = 0, from a fixed seed."""
    rng = np.random.default_rng(RECEIVER_SEED)
    h, gp = cfg["h"], cfg["sg_gp"]
    lo, hi = gp * h, (n - 1 - gp) * h
    return [(float(x), float(y), 0.0) for x, y in rng.uniform(lo, hi, size=(nrec, 2))]


def _mixed_l2_error(args, sg, torch, stream):
    """The mixed form against the FP64 form over args.err_steps steps of the
    workload at args.err_n^3: relative L2 and Linf difference of the surface
    receivers' displacement traces (all receivers, components and steps), and the
    absolute L2 norms of the whole-field difference at the end beside the FP64
    field's own norm at the end and at its peak."""
    n = args.err_n
    cfg = c2_config(n)
    rec_xyz = c2_receivers(cfg, n)
    res, traces, peak = [], [], 0.0
    every = max(1, args.err_steps // 10)
    for prec in (sg.FP64, sg.MIXED):
        ew = _make_ew(sg, cfg, n, prec, stream)
        ijk = [sg.nearest_grid_point(ew.grid, *p) for p in rec_xyz]
        ew.set_receivers(ijk, [sg.REC_DISPLACEMENT] * len(ijk), args.err_steps + 1)
        with torch.cuda.stream(stream):
            u = torch.zeros(3 * ew.npts, dtype=torch.float64, device="cuda")
            done = 0
            while done < args.err_steps:
                k = min(every, args.err_steps - done)
                ew.step(k, sg.MODE_FUSED)
                done += k
                if prec == sg.FP64:
                    ew.get_fields(u, None)
                    peak = max(peak, float(torch.linalg.norm(u)))
            ew.get_fields(u, None)
        torch.cuda.synchronize()
        res.append(u)
        traces.append(ew.records())
        ew.close()
    a, b = res
    ta, tb = traces
    d = float(torch.linalg.norm(b - a))
    # the workload's measure is the receiver traces; the whole field is reported as
    # absolute L2 norms (the difference at the end, the FP64 field at the end and at
    # its largest during the run), since the supergrid has absorbed most of the wave
    # energy by the end and a ratio to the remainder says little
    return {"receivers_l2_rel": float(np.linalg.norm(tb - ta) / np.linalg.norm(ta)),
            "receivers_linf_rel": float(np.abs(tb - ta).max() / np.abs(ta).max()),
            "field_diff_l2_end": d, "field_l2_end": float(torch.linalg.norm(a)),
            "field_l2_peak": peak,
            "receivers": {"n": len(rec_xyz), "seed": RECEIVER_SEED, "z": 0.0,
                          "mode": "displacement"},
            "grid": [n, n, n], "steps": args.err_steps, "t_end": args.err_steps * cfl_dt(cfg)}


def _guarded(world, name, fn, *a, **k):
    """One secondary workload of the line.  On one GPU a failure is reported in its
    place on the line instead of taking the headline figures with it; with several
    ranks it propagates, so that no rank waits at a barrier another rank has left."""
    if world > 1:
        return fn(*a, **k)
    try:
        return fn(*a, **k)
    except Exception as e:  # noqa: BLE001 -- reported on the line and on stderr
        import traceback
        traceback.print_exc(file=sys.stderr)
        try:
            import torch
            torch.cuda.empty_cache()
        except Exception:  # noqa: BLE001
            pass
        return {"failed": f"{name}: {type(e).__name__}: {e}"}


def run_ours(args, rank, world):
    import torch
    import sw4lite_gb300 as sg

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    sg.build()
    n = args.n
    npts_int = n ** 3
    stream = torch.cuda.Stream()
    if args.only_c2:
        # one form of the C2 workload alone (launch lists and kernel captures)
        f = _time_form(args, sg, torch, sg.FP64 if args.only_c2 == "fp64" else sg.MIXED, stream,
                       world, local)
        if rank == 0:
            print(json.dumps({"only": "C2 " + args.only_c2, "ms_per_step": f["ms_per_step"],
                              "value": f["value"], "kernel_ms": f["kernel_ms"]}), flush=True)
        return 0
    if args.only_topo:
        # the topography workload alone (launch lists and kernel captures)
        prec = 0 if args.only_topo == "fp64" else 1
        t = _time_topo(args, sg, torch, stream, world, precision=prec)
        if rank == 0:
            print(json.dumps({"only": "topography " + args.only_topo, "topography": t}), flush=True)
        return 0
    fp64 = _time_form(args, sg, torch, sg.FP64, stream, world, local)
    mixed = None
    if not args.no_mixed:
        mixed = _time_form(args, sg, torch, sg.MIXED, stream, world, local)
        if not args.no_err:
            mixed["error_vs_fp64"] = _guarded(world, "mixed error run", _mixed_l2_error, args, sg,
                                              torch, stream)
        mixed["speedup_vs_fp64"] = mixed["value"] / fp64["value"]
        cm = mixed["kernel_ms"]["corr_stage"]
        mixed["roofline"] = {"bound": "hbm", "kernel": "mixed corrector stage",
                             "achieved": MIXED_CORR_STAGE_BYTES * npts_int / (cm * 1e-3) / 1e9,
                             "unit": "GB/s", "algorithmic_bytes_per_pt": MIXED_CORR_STAGE_BYTES}

    corr_ms = fp64["kernel_ms"]["corr_stage"]
    peak_hbm, peak_kind = measured_peaks()
    corr_bytes = CORR_STAGE_WORDS * 8 * npts_int
    achieved = corr_bytes / (corr_ms * 1e-3) / 1e9
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = fp64["clocks"]["sm_mhz"] or 2070.0
    fp64_peak = FP64_THREAD_INST_PER_CLK_PER_SM * nsm * mhz * 1e6 / 1e9
    fp64_rate = 32 * FP64_WARP_INST_PER_PT["corr"] * npts_int / (corr_ms * 1e-3) / 1e9
    pred_ms = fp64["kernel_ms"]["pred_stage"]
    fp64_rate_pred = 32 * FP64_WARP_INST_PER_PT["pred"] * npts_int / (pred_ms * 1e-3) / 1e9
    if mixed is not None:
        mixed["roofline"]["peak"] = peak_hbm
        mixed["roofline"]["frac"] = mixed["roofline"]["achieved"] / peak_hbm
        mb = MIXED_CORR_STAGE_DRAM_BYTES_PER_PT * npts_int / (cm * 1e-3) / 1e9
        mixed["roofline"].update({"dram_bytes_per_pt": MIXED_CORR_STAGE_DRAM_BYTES_PER_PT,
                                  "dram_achieved": mb, "dram_frac": mb / peak_hbm,
                                  "peak_source": peak_kind, "launch_ms": cm})

    topo = None if args.no_topo else _guarded(world, "topography", _time_topo, args, sg, torch,
                                              stream, world)
    topo_mixed = None
    if not args.no_topo and not args.no_mixed:
        topo_mixed = _guarded(world, "topography mixed", _time_topo, args, sg, torch, stream, world,
                              precision=1)
        if topo and "ms_per_step" in topo and "ms_per_step" in topo_mixed:
            topo_mixed["speedup_vs_fp64"] = topo["ms_per_step"] / topo_mixed["ms_per_step"]
        if not args.no_err and args.topo_err_steps > 0 and "failed" not in topo_mixed:
            topo_mixed["error"] = _guarded(world, "topography error run", _topo_mixed_error, args, sg,
                                           torch, stream, args.topo_err_steps)
    adj = None if args.no_adjoint else _guarded(world, "adjoint", _time_adjoint, args, sg, torch,
                                                stream)
    multishot = None if args.no_multishot else _guarded(world, "multi-shot", _time_multishot, args,
                                                        sg, torch, stream)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        def _cpu():
            rate, el, kind, cores = cpu_rate(args.n, args.cpu_steps, 1)
            return {"value": rate, "unit": UNIT, "cores": cores, "kind": kind,
                    "sample": f"{args.cpu_steps} time steps of the {args.n}^3 workload after 1 "
                              f"untimed ({el:.1f} s; the reference arm's timing function, OpenMP)"}
        cpu = _guarded(world, "CPU baseline", _cpu)

    if rank == 0:
        line = {
            "metric": METRIC, "value": fp64["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": fp64["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": f"C2 layer-over-halfspace {n}^3 h=50, FP64, fused time step",
                       "grid": [n, n, n], "mode": args.mode, "dt": cfl_dt(c2_config(n)),
                       "l2": "inputs larger than L2 (3.3 GB per field), no flush",
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": {
                "bound": "fp64", "kernel": "fused corrector stage (fused_stage_kernel<1>)",
                "achieved": fp64_rate, "peak": fp64_peak, "unit": "G FP64 thread-instructions/s",
                "frac": fp64_rate / fp64_peak,
                "traffic": CORR_STAGE_DRAM_BYTES_PER_PT * npts_int,
                "basis": f"{32 * FP64_WARP_INST_PER_PT['corr']:.2f} FP64-pipe thread instructions "
                         "per interior point (ncu smsp__inst_executed_pipe_fp64 x 32 at 512^3) x points "
                         f"/ launch_ms; peak = {FP64_THREAD_INST_PER_CLK_PER_SM} per clock per SM x "
                         f"{nsm} SMs x the median sampled SM clock ({mhz:.0f} MHz)",
                "launch_ms": corr_ms,
                "predictor": {"achieved": fp64_rate_pred, "frac": fp64_rate_pred / fp64_peak,
                              "launch_ms": pred_ms},
                "hbm": {"achieved": achieved, "peak": peak_hbm, "unit": "GB/s",
                        "frac": achieved / peak_hbm, "peak_source": peak_kind,
                        "algorithmic_bytes_per_launch": corr_bytes,
                        "traffic_source": "ncu capture at 192^3 scaled per point"}},
            "kernel_ms": fp64["kernel_ms"],
            "clocks": fp64["clocks"],
            "e2e": fp64.get("e2e"),
            "gpu_launches": fp64["gpu_launches"],
            "cpu_baseline": cpu,
            "mixed": mixed,
            "topography": topo,
            "topography_mixed": topo_mixed,
            "adjoint": adj,
            "multishot": multishot,
        }
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--mode", choices=["fused", "phases"], default="fused")
    ap.add_argument("--n", type=int, default=512, help="grid points per axis")
    ap.add_argument("--cpu-steps", type=int, default=4,
                    help="timed CPU steps of the in-line CPU baseline (same workload as the GPU)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the FP32-mixed form")
    ap.add_argument("--no-topo", action="store_true", help="skip the topography workload")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint workload")
    ap.add_argument("--topo-nx", type=int, default=384, help="x and y points of the topography workload")
    ap.add_argument("--topo-err-steps", type=int, default=800,
                    help="steps of the mixed-vs-FP64 error run of the topography workload (0: skip)")
    ap.add_argument("--topo-nz", type=int, default=128, help="z points of both grids together")
    ap.add_argument("--adj-n", type=int, default=256, help="grid of the adjoint workload")
    ap.add_argument("--adj-steps", type=int, default=2000, help="steps of the adjoint workload")
    ap.add_argument("--adj-ckpt", type=int, default=100, help="checkpoint spacing")
    ap.add_argument("--no-multishot", action="store_true", help="skip the multi-shot gradient workload")
    ap.add_argument("--ms-shots", type=int, default=16, help="timed shots of the multi-shot workload (of 16)")
    ap.add_argument("--ms-steps", type=int, default=1500, help="steps of the multi-shot workload")
    ap.add_argument("--ms-err-steps", type=int, default=1500, help="steps of the mixed-vs-FP64 gradient check")
    ap.add_argument("--ms-err-shots", type=int, default=2,
                    help="shots whose summed gradient is compared with FP64 (0: skip)")
    ap.add_argument("--only-c2", choices=["fp64", "mixed"], default=None,
                    help="time only the C2 workload in that form (for profiling)")
    ap.add_argument("--only-topo", choices=["fp64", "mixed"], default=None,
                    help="time only the topography workload in that form (for profiling)")
    ap.add_argument("--no-err", action="store_true", help="skip the mixed-vs-FP64 error run")
    ap.add_argument("--err-n", type=int, default=512, help="grid of the mixed-vs-FP64 error run")
    ap.add_argument("--err-steps", type=int, default=1000, help="steps of the error run")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    rank, world = dist_init(args)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world)


if __name__ == "__main__":
    sys.exit(main())
