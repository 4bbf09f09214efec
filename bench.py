"""Benchmark of the LES time step on one GB300.

Workload: the variable-density temporal mixing layer, 256 x 192 x 128
cells (one block), tanh stretching in y (beta = 2), periodic x/z, slip
walls in y, WALE eddy viscosity (Cw = 0.5), density ratio 2 carried by the
scalar through the mixing law, seeded Gaussian noise (sigma = 0.02, seed 2).
Inputs are synthetic (numpy default_rng); the working set (~2 GB of FP64
fields) is far larger than the 129 MB L2, so no L2 flush is needed between
steps.

A step is one call of lester_step: the ivar loop of code/step.F (wall ghost
velocities, eddy viscosity, scalar transport and density, momentum
predictor, pressure source, the Poisson solve to ||b - A p|| / ||b|| <= 1e-8,
extrap_p, p_ref_subtract, projection, slip faces, density rotation).  The
step is timed twice, with the mixed-precision solver (headline ``value``)
and with the plain FP64 solver; the line carries both and their ratio.

``value`` has every field resident in HBM.  ``e2e`` is the same step with
every field in pinned host memory (the strict drop-in a Fortran host sees):
each call copies the carried state in and the state the caller reads after
the step back; work arrays and the pressure coefficients (written at
istep 1) stay on the device.  ``cpu_baseline`` and ``--impl
reference`` time the oracle (the C restatement of the reference Fortran,
one thread: the reference runs one MPI rank per block and this workload is
one block) on the same workload with the reference's own solver settings.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mcell-steps/s & Poisson V-cycle ms: mixed-prec vs FP64 on GB300 at 1e-8 resid"
SHAPE = (256, 192, 128)
DOMAIN = (30.0, 30.0, 15.0)
# FP64 physics kernels: 0 = fast build (reciprocal metric tables, FMA), the
# product default; the reference arm and the CPU baseline are unaffected
EXACT = 0
WORKLOAD = ("variable-density temporal mixing layer 256x192x128, tanh y-stretch beta 2, slip y "
            "walls, WALE Cw 0.5, density ratio 2, full lester_step, Poisson to 1e-8")
# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) per launch
# of the timed kernels on the mixing-layer workload: the level-1 half sweep
# (k_rb_geo<float>) from one capture at full size (52.0 MB read + 0.16 MB
# written, against 50.3 MB algorithmic); the tile-pipeline scalar sweep from one
# capture at 128x96x64 (53.1 MB read + 0.08 MB written for 0.786 M cells)
# scaled by cells to 256x192x128
TRAFFIC = {"rb": 52.17e6, "sweep": 53.22e6 * 6291456 / 786432}
# algorithmic bytes per interior cell of one launch: a red-black half sweep
# (one colour per launch, FP32) must read x of both colours (its own points
# and their neighbours of the other colour: 4 B per cell), b of its colour
# and write x of its colour (2 + 2 B per cell);
# the tile-pipeline scalar sweep reads the FP32 skewed copies of sc1, hsc1,
# u, v, w, rho, gamsc1, gamlam and writes the new sc1 and hsc1 (10 FP32
# arrays)
ALG_BYTES = {"rb": 8.0, "sweep": 40.0}
KERNEL_NAMES = {"rb": "k_rb_geo<float> level-1 red-black SOR half sweep",
                "sweep": "set_sc1 in-place scalar sweep (one launch per step)"}
# the level-1 smoother as shared-memory tiles (k_rb_tile, when the level
# allows it): one launch is a full sweep, both colours (12 B per cell)
ALG_BYTES_TILE = 12.0
KERNEL_NAME_TILE = "k_rb_tile<float> level-1 red-black SOR sweep (both colours, shared-memory tiles)"
# other workloads (--workload): the plain channel of the reference's own
# CPU-runnable case, and the large stretched channel
WORKLOADS = {
    "mixing": dict(shape=SHAPE, desc=WORKLOAD),
    "channel64": dict(shape=(64, 64, 64), beta=None, nummgl=4, seed=1,
                      desc="plane channel 64^3 cells, 2pi x 2 x pi, walls in y, periodic x/z, uniform "
                           "grid, Re_b 2800, Smagorinsky Cs 0.1, constant density, dt from CFL 0.3 and "
                           "diffusion number 0.2, "
                           "4 multigrid levels, full lester_step, Poisson to 1e-8"),
    "poisson32": dict(shape=(0, 0, 0), seed=5,
                      desc="32 independent Poisson boxes in one solve, sides drawn from 32,40,...,128 "
                           "cells per axis (seed 5), cubic cells, periodic x/z and Neumann y, sources "
                           "N(0,1) minus their mean, to 1e-8"),
    "bl6": dict(shape=(384, 144, 64), seed=3, inflow=True,
                desc="multiblock spatially developing boundary layer: 6 uneven blocks (160,96,64) "
                     "(128,96,64) (96,96,64) below (160,48,64) (128,48,64) (96,48,64), interfaces in x "
                     "and y, fixed inflow u = tanh(y/0.5) + noise (fixed plane, no recycling), convective "
                     "outflow, wall below, slip above, periodic z, a passive scalar layer at y = 2 at "
                     "constant density (with density ratio 1.5 the reference scheme itself diverges in "
                     "its first steps at this resolution), "
                     "Smagorinsky Cs 0.1, dt from CFL 0.3 and diffusion number 0.2, full lester_step, "
                     "Poisson to 1e-8"),
    "channel512": dict(shape=(512, 384, 256), beta=2.2, nummgl=0, seed=5,
                       desc="stretched plane channel 512x384x256 cells, 2pi x 2 x pi, tanh walls "
                            "beta 2.2, periodic x/z, Re_b 2800, Smagorinsky Cs 0.1, constant "
                            "density, dt from CFL 0.3 and diffusion number 0.2, full lester_step, Poisson to 1e-8"),
}


# ----------------------------------------------------------------- helpers
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Ranks:
    """The processes of a torchrun launch, one replica of the step per GPU
    with no exchange on the data path: a host-side gloo group that starts and
    ends every timed region together (barrier) and takes the slowest rank's
    time (max).  One process: every call is a no-op."""

    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.dist = None
        if self.world > 1:
            import datetime
            import torch.distributed as dist
            # a rank that fails inside a timed region releases the others
            # within minutes, not after gloo's default 30
            dist.init_process_group("gloo", timeout=datetime.timedelta(minutes=2))
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.dist is None:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist is not None:
            try:
                self.dist.destroy_process_group()
            finally:
                self.dist = None


RANKS = None  # set by main(); run_gpu's callers outside main get one process
GPU_INDEX = 0  # physical index of this process's GPU (nvidia-smi -i)


def pick_gpu(local: int, world: int) -> int:
    """The physical GPU of this rank: the local-rank entry of an existing
    CUDA_VISIBLE_DEVICES list (the launcher's choice), else the local rank;
    CUDA_VISIBLE_DEVICES is then narrowed to that one GPU."""
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        ids = [v.strip() for v in vis.split(",") if v.strip()]
        phys = ids[local % len(ids)] if world > 1 else ids[0]
    else:
        phys = str(local)
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = phys
    try:
        return int(phys)
    except ValueError:  # a UUID: nvidia-smi -i accepts it too
        return phys


def _ranks() -> Ranks:
    global RANKS
    if RANKS is None:
        RANKS = Ranks()
    return RANKS


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._th:
            self._th.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def make_case(shape=SHAPE, wl="mixing"):
    from fortranutils_gb300 import grid, lester as L
    ni, nj, nk = shape
    if wl == "mixing":
        lx, ly, lz = DOMAIN
        return grid.box_case(ni, nj, nk, lx=lx, ly=ly, lz=lz, ybc=L.BCT_ZERO_GRAD, beta=2.0)
    if wl == "bl6":
        return grid.bl6_case(1)
    w = WORKLOADS[wl]
    return grid.box_case(ni, nj, nk, ybc=L.BCT_WALL, beta=w["beta"], nummgl=w["nummgl"])


def cfl_dt(case, s, cfl=0.3, dfs=0.2, visc=1.0 / 2800.0):
    """dt from the initial field (cflest-style): the smaller of cfl / max
    over cells of |u|/dx + |v|/dy + |w|/dz and, since the predictor's
    diffusion is explicit, dfs / max of visc (1/dx^2 + 1/dy^2 + 1/dz^2)."""
    cmax = dmax = 0.0
    for ib, b in enumerate(case.blocks):
        dx = np.diff(b.x[1:b.n[0]]).min()
        dy = np.diff(b.y[1:b.n[1]])
        dz = np.diff(b.z[1:b.n[2]]).min()
        u, v, w = (case.block_view(s[n], ib)[1:-1, 1:-1, 1:-1] for n in "uvw")
        c = np.abs(u) / dx + np.abs(v) / dy[None, :, None] + np.abs(w) / dz
        cmax = max(cmax, float(c.max()))
        dmax = max(dmax, visc * (1.0 / dx ** 2 + 1.0 / dy.min() ** 2 + 1.0 / dz ** 2))
    return min(cfl / cmax, dfs / dmax)


SMOOTHER = "auto"
RB_TILE = 0  # ctrl.rb_tile: red-black sweeps through shared-memory tiles (opt-in)
P_GUESS = 0  # ctrl.p_guess: 0 the previous pressure, 1 extrapolated in time
PHYS32 = 1


def make_ctrl(psolve, krylov=2, wl="mixing", dtime=None):
    from fortranutils_gb300 import lester as L
    sm = dict(autotune=3) if SMOOTHER == "auto" else dict(autotune=0)
    sm["rb_tile"] = RB_TILE
    sm["p_guess"] = P_GUESS
    # the mixed path's physics in FP32 arithmetic (FP64 fields)
    sm["phys32"] = PHYS32 if psolve == L.PSOLVE_MIXED else 0
    if SMOOTHER == "line":
        sm.update(rb_line=1, rb_omega=1.2, rb_sweeps=2)
    if wl == "mixing":
        return L.default_ctrl(dtime=0.01, model=2, csles=0.5, rholo=1.0, rhohi=2.0, psolve=psolve,
                              rtol=1e-8, max_outer=200, exact=EXACT, krylov=krylov, **sm)
    return L.default_ctrl(dtime=dtime, model=1, csles=0.1, rholo=1.0, rhohi=1.0,
                          visc=1.0 / 2800.0, psolve=psolve, rtol=1e-8, max_outer=200, exact=EXACT,
                          krylov=krylov, **sm)


def host_state(case, ctrl, wl="mixing"):
    """Initial fields (numpy); metrics left zero for the caller to fill."""
    from fortranutils_gb300 import lester as L, state as S
    c = case
    s = S.new_state(c, {n: np.zeros(c.n2) for n in L.METRIC_NAMES}, np.zeros(c.n1k),
                    np.zeros(c.n1k))
    if wl == "mixing":
        return S.init_mixing_layer(s, seed=2, sigma=0.02, rholo=ctrl.rholo, rhohi=ctrl.rhohi)
    if wl == "bl6":
        return S.init_bl6(s, seed=3, sigma=0.03, rholo=1.0, rhohi=1.0, width=0.25)
    return S.init_channel(s, seed=WORKLOADS[wl]["seed"], sigma=0.05)


def set_inlet(case, wl, orc=None):
    """The bl6 workload's inflow planes (fixed, no recycling): blocks 1 and
    4 in fixed_inlet's slots 1 and 4."""
    if wl != "bl6":
        return
    from fortranutils_gb300 import grid, lester as L
    up, vp = grid.bl6_inflow(case)
    if orc is not None:
        orc.set_inlet([1, 0, 0, 4], up, vp, 3)
    else:
        L.gpu_set_inlet([1, 0, 0, 4], up, vp, 3)


def device_state(case, ctrl, wl="mixing"):
    """Device-resident state: metrics by comp_metric, halos exchanged."""
    import torch
    from fortranutils_gb300 import lester as L
    g = host_state(case, ctrl, wl).to("torch")
    x, y, z = (torch.from_numpy(a).cuda() for a in case.coordinates())
    L.comp_metric(x, y, z, g["metric"], g["dkp"], g["dkw"])
    for n in ("u", "v", "w", "sc1", "rho", "rhonp1", "rhonm1"):
        L.swap_sc(0, 1, g[n], mg_or_sg=2)
    L.gpu_sync()
    return g


def step_bytes(mode: str, cycles: float, sweeps: int, krylov: int = 1) -> float:
    """Algorithmic bytes per interior cell of one step: distinct 3-D arrays
    read plus written once per kernel (8 B FP64, 4 B FP32), metric tables and
    matrix-free coefficients free.  Per V-cycle, levels sum with 8/7:
      FP64: sweeps 24, residual 24, restriction 9, prolongation 17;
      mixed: FP32 sweeps 12, restriction 4.5, prolongation 8.5.
    Per outer iteration (level 1, FP64 vectors; z the cycle's correction):
      defect correction: residual 24 + update p += z (16 + |z|);
      flexible CG: z.q and z.r (16 + |z|), direction p, q (40 + |z|),
      step x, r (48 + |z|).
    Per step: predictor 128, WALE 64, sour_p 72, projection 64, p_ref 16,
    scalar predictor 80, search_lib 32."""
    nsw = 2 * sweeps  # pre + post smoothing sweeps per level
    zb = 8 if mode == "fp64" else 4
    outer = (104 + 3 * zb) if krylov else (40 + zb)
    if mode == "fp64":
        bv = 8.0 / 7.0 * (nsw * 24 + 24 + 9 + 17) + outer
    else:
        bv = 8.0 / 7.0 * (nsw * 12 + 4.5 + 8.5) + outer
    return 128 + 64 + 72 + 64 + 16 + 80 + 32 + cycles * bv


# ------------------------------------------------------------ GPU arm
def run_gpu(args):
    import torch
    from fortranutils_gb300 import build, lester as L, state as S
    build.build()
    torch.cuda.set_device(0)
    wl = args.workload
    case = make_case(tuple(args.shape), wl)
    dtime = None if wl == "mixing" else cfl_dt(case, host_state(case, make_ctrl(0, wl=wl, dtime=1.0), wl))
    res = {}
    modes = [("fp64", L.PSOLVE_FP64), ("mixed", L.PSOLVE_MIXED)]
    modes = [m for m in modes if args.mode in ("both", m[0])]
    for mode, ps in modes:
        ctrl = make_ctrl(ps, {"dc": 0, "fcg": 1, "auto": 2}[args.outer], wl, dtime)
        L.gpu_init(case.geom(), ctrl)
        set_inlet(case, wl)
        g = device_state(case, ctrl, wl)
        stream = torch.cuda.current_stream()
        istep = 0
        for _ in range(args.warmup):
            istep += 1
            S.step(g, istep)
        L.gpu_sync()
        cyc, solve_ms, rel = [], [], []
        launches0 = L.gpu_launch_count()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        L.gpu_prof(True)
        with ClockSampler(GPU_INDEX) as clk:
            torch.cuda.synchronize()
            _ranks().barrier()
            e0.record(stream)
            for _ in range(args.steps):
                istep += 1
                rc = S.step(g, istep)
                st = L.gpu_solve_stats()
                cyc.append(st["cycles"])
                rel.append(st["relres"])
                solve_ms.append(L.gpu_solve_time())
                if rc != 0:
                    raise RuntimeError(f"{mode} solver did not reach 1e-8: {st}")
            e1.record(stream)
            torch.cuda.synchronize()
            _ranks().barrier()
        L.gpu_prof(False)
        tuned = L.gpu_tuned(32 if mode == "mixed" else 64)
        forms = L.gpu_solver_forms()
        ms = _ranks().max(e0.elapsed_time(e1))
        kms, kl = L.gpu_prof_read(L.PROF_RB)
        rb_tile = bool(L.gpu_rb_tiles() & 2)  # level 1 smoothed by k_rb_tile
        sms, sl = L.gpu_prof_read(L.PROF_SWEEP)
        res[mode] = {"ms_per_step": ms / args.steps, "cycles": float(np.mean(cyc)),
                     "relres_max": float(np.max(rel)), "solve_ms": float(np.mean(solve_ms)),
                     "launches": L.gpu_launch_count() - launches0, "rb_ms": kms, "rb_tile": rb_tile,
                     "rb_launches": kl, "sweep_ms": sms, "sweep_launches": sl,
                     "clocks": clk.summary(), "ctrl": ctrl, "tuned": tuned, "forms": forms}
        del g
        if args.step_graph:
            res[mode]["graph"] = run_graph_leg(args, case, ctrl, wl)
        if mode == "mixed" and not args.no_e2e:
            res[mode]["e2e"] = run_e2e(args, case, ctrl, wl)
        L.gpu_finalize()
        torch.cuda.empty_cache()
    return case, res


def run_graph_leg(args, case, ctrl, wl):
    """The same run again from the same initial state and step counter, the
    steps replayed from the whole-step CUDA graph (ctrl.step_graph; the
    autotuned settings kept): step 1 as launched (coeff_p), the graph
    captured at step 2, the same timed step indices as the launched leg."""
    import torch
    from fortranutils_gb300 import lester as L, state as S
    g = device_state(case, ctrl, wl)
    L.gpu_set_iststep(2)
    ctrl.step_graph = 1
    L.gpu_set_ctrl(ctrl)
    stream = torch.cuda.current_stream()
    istep = 0
    for _ in range(args.warmup):
        istep += 1
        S.step(g, istep)
    L.gpu_sync()
    info0 = L.gpu_step_graph_info()
    cyc = []
    launches0 = L.gpu_launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(GPU_INDEX) as clk:
        torch.cuda.synchronize()
        _ranks().barrier()
        e0.record(stream)
        for _ in range(args.steps):
            istep += 1
            rc = S.step(g, istep)
            st = L.gpu_solve_stats()
            cyc.append(st["cycles"])
            if rc != 0:
                raise RuntimeError(f"graph step: solver did not reach 1e-8: {st}")
        e1.record(stream)
        torch.cuda.synchronize()
        _ranks().barrier()
    info = L.gpu_step_graph_info()
    ctrl.step_graph = 0
    L.gpu_set_ctrl(ctrl)
    del g
    if info["failed"] or info["replays"] - info0["replays"] != args.steps:
        raise RuntimeError(f"whole-step graph not replayed: {info}")
    return {"ms_per_step": _ranks().max(e0.elapsed_time(e1)) / args.steps, "cycles": float(np.mean(cyc)),
            "launches": L.gpu_launch_count() - launches0, "clocks": clk.summary(),
            "handovers": info["handovers"] - info0["handovers"]}


def run_e2e(args, case, ctrl, wl="mixing"):
    """lester_step with every field in pinned host memory (strict drop-in):
    each call copies the carried state, level 1 of p, the metrics and the
    wall arrays in and the state the caller reads after a step back; the
    pressure coefficients, written at istep 1, stay mirrored on the device
    and the work arrays in library-held device memory."""
    import torch
    from fortranutils_gb300 import lester as L, state as S
    g = device_state(case, ctrl, wl)
    h = g.to("pinned")
    del g
    torch.cuda.empty_cache()
    # the same way of running the step as the headline: the whole-step
    # graph (with the host copies as its nodes) unless --step-graph 0
    graph = int(bool(args.step_graph))
    ctrl.step_graph = graph
    L.gpu_set_ctrl(ctrl)
    L.gpu_set_iststep(2)  # a run's first step
    info0 = L.gpu_step_graph_info()
    S.step(h, 1)  # coeff_p at istep 1, as the first step of a run
    S.step(h, 2)  # untimed: the first step that can be captured as a graph
    L.gpu_sync()
    k = max(1, min(args.steps, 10))
    b0 = L.gpu_xfer_bytes()
    _ranks().barrier()
    t0 = time.perf_counter()
    for it in range(k):
        S.step(h, 3 + it)
    L.gpu_sync()
    dt = _ranks().max(time.perf_counter() - t0) / k
    _ranks().barrier()
    b1 = L.gpu_xfer_bytes()
    info = L.gpu_step_graph_info()
    ctrl.step_graph = 0
    L.gpu_set_ctrl(ctrl)
    if graph and (info["failed"] or info["replays"] - info0["replays"] != k + 1):
        raise RuntimeError(f"e2e: whole-step graph not replayed: {info}")
    return {"s_per_step": dt, "steps": k, "h2d_bytes_per_step": (b1[0] - b0[0]) // k,
            "d2h_bytes_per_step": (b1[1] - b0[1]) // k,
            "step_launch": "whole-step CUDA graph" if graph else "launched"}


# ------------------------------------------------------------- CPU arm
def run_cpu_steps(case, nsteps: int, warmup: int = 0, wl: str = "mixing", dtime=None):
    """The oracle on the same workload: orc_step with the reference's own
    solver settings (nummgits 5 V(1,1) cycles of lexicographic SOR).  One
    thread.  Returns seconds per timed step."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as O
    from fortranutils_gb300 import lester as L
    ctrl = make_ctrl(L.PSOLVE_REFERENCE, wl=wl, dtime=dtime)
    orc = O.Oracle(case)
    set_inlet(case, wl, orc)
    x, y, z = case.coordinates()
    met, dkp, dkw = orc.comp_metric(x, y, z)
    s = host_state(case, ctrl, wl)
    for i, n in enumerate(L.METRIC_NAMES):
        s["metric"][n][:] = met[i]
    s["dkp"][:] = dkp
    s["dkw"][:] = dkw
    for n in ("u", "v", "w", "sc1", "rho", "rhonp1", "rhonm1"):
        orc.swap_sc(1, s[n], 2)
    orc.coeff_p(s["metric"], dkp, dkw, [s[n] for n in "ap aw ae as an al ar".split()])
    mg, k = O.mgctrl_from_ctrl(ctrl), O.phys_from_ctrl(ctrl)
    istep = 1  # coefficients exist: every oracle step runs as istep > 1
    for _ in range(warmup):
        istep += 1
        orc.step(mg, k, istep, istep, s)
    t0 = time.perf_counter()
    for _ in range(nsteps):
        istep += 1
        orc.step(mg, k, istep, istep, s)
    return (time.perf_counter() - t0) / nsteps, ctrl.nummgits


def run_poisson(args):
    """Batched Poisson solves: 32 unlinked boxes of uneven sizes as one
    multiblock grid, every multigrid operation one launch over all boxes."""
    import torch
    from fortranutils_gb300 import build, grid, lester as L
    build.build()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(WORKLOADS["poisson32"]["seed"])
    sizes = [tuple(int(v) for v in rng.choice(np.arange(32, 129, 8), 3)) for _ in range(32)]
    case = grid.boxes_case(sizes, h=1.0 / 64.0)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    b = np.zeros(case.n3_mg)
    for ib in range(len(case.blocks)):
        v = case.block_view(b, ib, 0)[1:-1, 1:-1, 1:-1]
        v[...] = rng.standard_normal(v.shape)
        v -= v.mean()
    out = {}
    for mode, ps in (("fp64", L.PSOLVE_FP64), ("mixed", L.PSOLVE_MIXED)):
        ctrl = L.default_ctrl(psolve=ps, rtol=1e-8, max_outer=200)
        L.gpu_init(case.geom(), ctrl)
        met = {n: torch.zeros(case.n2, dtype=torch.float64, device="cuda") for n in L.METRIC_NAMES}
        dkp = torch.zeros(case.n1k, dtype=torch.float64, device="cuda")
        dkw = torch.zeros_like(dkp)
        L.comp_metric(*(dev(a) for a in case.coordinates()), met, dkp, dkw)
        a = [torch.zeros(case.n3_mg, dtype=torch.float64, device="cuda") for _ in range(7)]
        L.coeff_p(met["diu"], met["djv"], met["rdiv"], met["rdju"], met["didjp"], met["rp"], dkp, dkw, *a)
        bd, rd = dev(b), torch.zeros_like(a[0])
        fd = torch.zeros_like(a[0])
        for _ in range(args.warmup):
            fd.zero_()
            L.lmg_solve(*a, fd, bd.clone(), rd)
        ms, cyc, rel = [], [], []
        for _ in range(args.steps):
            fd.zero_()
            bc = bd.clone()
            L.lmg_solve(*a, fd, bc, rd)
            st = L.gpu_solve_stats()
            ms.append(L.gpu_solve_time())
            cyc.append(st["cycles"])
            rel.append(st["relres"])
        out[mode] = {"solve_ms": float(np.mean(ms)), "cycles": float(np.mean(cyc)),
                     "relres_max": float(np.max(rel)),
                     "vcycle_ms": float(np.mean(ms)) / max(float(np.mean(cyc)), 1.0)}
        L.gpu_finalize()
        del a, bd, rd, fd, met
        torch.cuda.empty_cache()
    ncell = case.cells()
    line = {"metric": "Poisson solve ms to 1e-8, 32 independent boxes (mixed; FP64 beside)",
            "value": out["mixed"]["solve_ms"], "unit": "ms", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": False, "dtype": "f32/f64",
            "data": "synthetic (seeded numpy default_rng, seed 5)",
            "config": {"workload": WORKLOADS["poisson32"]["desc"], "cells": ncell,
                       "levels": case.levels and len(case.levels), "sizes": sizes},
            "mixed": out["mixed"], "fp64": out["fp64"],
            "solve_speedup_mixed_vs_fp64": out["fp64"]["solve_ms"] / out["mixed"]["solve_ms"],
            "mcells_per_s_mixed": ncell / (out["mixed"]["solve_ms"] * 1e-3) / 1e6}
    print(json.dumps(line), flush=True)


def reference_line(args, rank):
    """--impl reference: the oracle (the reference's algorithm on the CPU),
    the same --steps and --warmup as the GPU arm."""
    if rank != 0:
        return
    case = make_case()
    n, w = max(1, args.steps), max(0, args.warmup)
    sps, nmg = run_cpu_steps(case, n, warmup=w)
    val = case.cells() / sps / 1e6
    sample = (f"{n} full steps of the 256x192x128 workload after {w} warm-up, "
              f"reference solver settings ({nmg} V-cycles per step)")
    line = {"metric": METRIC, "value": val, "unit": "Mcell-steps/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": n, "warmup": w,
            "ms_per_step": 1e3 * sps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy default_rng)",
            "config": {"workload": WORKLOAD, "cells": case.cells()},
            "cpu_baseline": {"value": val, "unit": "Mcell-steps/s", "cores": 1, "kind": "port",
                             "sample": sample},
            "e2e": {"value": val, "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer (e2e) leg")
    ap.add_argument("--phys32", type=int, default=1, choices=[0, 1],
                    help="mixed path: predictors, scalar and eddy viscosity in FP32 arithmetic on the FP64 "
                         "fields (0: the FP64 physics of the FP64 path)")
    ap.add_argument("--step-graph", type=int, default=1, choices=[0, 1],
                    help="also time the steps replayed from the whole-step CUDA graph; the headline is "
                         "the faster of the two ways of running the same step")
    ap.add_argument("--mode", default="both", choices=["both", "mixed", "fp64"],
                    help="solvers to time (the JSON line needs both)")
    ap.add_argument("--outer", default="auto", choices=["auto", "fcg", "dc"],
                    help="fast solvers' outer loop: defect correction switching to flexible CG "
                         "when a cycle stalls (auto), flexible CG, or defect correction")
    ap.add_argument("--smoother", default="auto", choices=["auto", "point", "line"],
                    help="fast solvers' smoother: autotuned on the third solve (inside the warm-up "
                         "steps), point red-black, or y-line zebra relaxation")
    ap.add_argument("--p-guess", type=int, default=0, choices=[0, 1],
                    help="fast solves' initial pressure: 0 p(n), 1 2p(n)-p(n-1) (ctrl.p_guess)")
    ap.add_argument("--rb-tile", type=int, default=0, choices=[0, 1],
                    help="1: the FP32 solver's red-black sweeps through shared-memory tiles (ctrl.rb_tile)")
    ap.add_argument("--workload", default="mixing", choices=list(WORKLOADS),
                    help="mixing: the headline mixing layer; channel64: the 64^3 plain channel; "
                         "channel512: the 512x384x256 stretched channel")
    ap.add_argument("--shape", type=int, nargs=3, default=None,
                    help="cells per axis (other shapes than the workload's are for profiling only)")
    args = ap.parse_args()
    global SMOOTHER, PHYS32, RB_TILE, P_GUESS
    SMOOTHER = args.smoother
    RB_TILE = args.rb_tile
    P_GUESS = args.p_guess
    PHYS32 = args.phys32
    if args.shape is None:
        args.shape = list(WORKLOADS[args.workload]["shape"])
    rank, world, local = dist_env()
    # the path runs on one GPU; extra ranks are independent replicas
    global GPU_INDEX
    GPU_INDEX = pick_gpu(local, world)
    if args.impl == "reference":
        reference_line(args, rank)
        return
    if args.workload == "poisson32":
        if rank == 0:
            run_poisson(args)
        return
    global RANKS
    RANKS = Ranks()
    try:
        report(args, rank, world)
    finally:
        RANKS.close()


def report(args, rank, world):
    case, res = run_gpu(args)
    ncell = case.cells()
    wl = args.workload
    if args.mode != "both" or args.no_e2e or tuple(args.shape) != WORKLOADS[wl]["shape"]:
        print(json.dumps({k: {kk: vv for kk, vv in v.items() if kk not in ("clocks", "ctrl")}
                          for k, v in res.items()}), flush=True)
        return
    mx, fp = res["mixed"], res["fp64"]

    def best(r):
        """(ms per step, how, leg): the faster way of running the same step"""
        gr = r.get("graph")
        if gr and gr["ms_per_step"] < r["ms_per_step"]:
            return gr["ms_per_step"], "whole-step CUDA graph", gr
        return r["ms_per_step"], "launched call by call", r

    mx_ms, mx_how, mx_leg = best(mx)
    fp_ms, fp_how, _ = best(fp)
    value = ncell / (mx_ms * 1e-3) / 1e6 * world
    peaks = {}
    pf = ROOT / "MEASURED_PEAKS.json"
    if pf.exists():
        peaks = json.loads(pf.read_text())
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    # roofline of the two timed kernels (CUDA events around every launch in
    # the launched leg's timed region): algorithmic bytes per launch over the
    # average launch time; the headline entry is the one with more time
    kern = {}
    for key, ms_k, n_k in (("rb", mx["rb_ms"], mx["rb_launches"]),
                           ("sweep", mx["sweep_ms"], mx["sweep_launches"])):
        if n_k <= 0:
            continue
        avg = ms_k / n_k
        tile = key == "rb" and mx.get("rb_tile")
        ach = (ALG_BYTES_TILE if tile else ALG_BYTES[key]) * ncell / (avg * 1e-3) / 1e9
        kern[key] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                     "traffic": TRAFFIC[key] if wl == "mixing" and not tile else None,
                     "traffic_source": ({"rb": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                               "launch on this workload",
                                        "sweep": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                                 "launch at 128x96x64, scaled by cells"}[key]
                                        if TRAFFIC[key] and wl == "mixing" and not tile else None),
                     "peak_source": peak_src, "kernel": KERNEL_NAME_TILE if tile else KERNEL_NAMES[key],
                     "avg_launch_ms": avg,
                     "launches": n_k, "total_ms": ms_k,
                     "share_of_timed_steps": ms_k / (mx["ms_per_step"] * args.steps)}
    dominant = max(kern, key=lambda k: kern[k]["total_ms"])
    sweeps = mx["tuned"]["rb_sweeps"] if mx["tuned"]["done"] else mx["ctrl"].rb_sweeps
    # outer iterations counted as defect correction unless flexible CG ran
    kry = 1 if args.outer == "fcg" else 0
    step_gbs = {m: step_bytes(m, r["cycles"], sweeps, kry) * ncell / (t * 1e-3) / 1e9
                for m, r, t in (("mixed", mx, mx_ms), ("fp64", fp, fp_ms))}
    cpu = None
    if not args.no_cpu and rank == 0 and ncell <= 10_000_000:
        sps, nmg = run_cpu_steps(case, 1, wl=wl, dtime=mx["ctrl"].dtime)
        cpu = {"value": ncell / sps / 1e6, "unit": "Mcell-steps/s", "cores": 1, "kind": "port",
               "sample": f"1 full step of the same workload, reference solver settings "
                         f"({nmg} V-cycles, lexicographic SOR), {sps:.1f} s"}
    e2e = mx["e2e"]
    line = {
        "metric": METRIC, "value": value, "unit": "Mcell-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mx_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64",
        "data": f"synthetic (seeded numpy default_rng, seed {WORKLOADS[wl].get('seed', 2)})",
        "config": {"workload": WORKLOADS[wl]["desc"], "cells": ncell,
                   "l2": ("inputs larger than L2, no flush" if ncell * 8 * 20 > 129e6 else
                          "working set smaller than the 129 MB L2 (not flushed): a small-case figure"),
                   "parallelism": "replicas" if world > 1 else "1 GPU",
                   "precision": ("mixed: FP32 arithmetic in the predictors, scalar, eddy viscosity and multigrid "
                                 "cycles; FP64 fields, fine-grid residual, global sums, metrics" if args.phys32 else
                                 "mixed: FP32 multigrid cycles, FP64 physics") + "; fp64: all FP64",
                   "outer_loop": {"auto": "defect correction, flexible CG when a cycle stalls",
                                  "fcg": "flexible CG", "dc": "defect correction"}[args.outer]},
        "step_launch": mx_how,
        "mixed": {"launched_ms_per_step": mx["ms_per_step"],
                  "graph_ms_per_step": mx["graph"]["ms_per_step"] if "graph" in mx else None,
                  "graph_vcycles_per_step": mx["graph"]["cycles"] if "graph" in mx else None,
                  "vcycles_per_step": mx["cycles"], "solve_ms": mx["solve_ms"], "tuned": mx["tuned"],
                  "vcycle_ms": mx["solve_ms"] / max(mx["cycles"], 1),
                  "relres_max": mx["relres_max"], "solver_forms": mx["forms"]},
        "fp64": {"value": ncell / (fp_ms * 1e-3) / 1e6 * world, "step_launch": fp_how,
                 "ms_per_step": fp_ms, "launched_ms_per_step": fp["ms_per_step"],
                 "graph_ms_per_step": fp["graph"]["ms_per_step"] if "graph" in fp else None,
                 "vcycles_per_step": fp["cycles"],
                 "solve_ms": fp["solve_ms"], "vcycle_ms": fp["solve_ms"] / max(fp["cycles"], 1),
                 "tuned": fp["tuned"],
                 "relres_max": fp["relres_max"]},
        "speedup_mixed_vs_fp64": fp_ms / mx_ms,
        "solve_speedup_mixed_vs_fp64": fp["solve_ms"] / mx["solve_ms"],
        "roofline": kern[dominant],
        "roofline_kernels": kern,
        "step_roofline": {"mixed_gbs": step_gbs["mixed"], "fp64_gbs": step_gbs["fp64"],
                          "mixed_frac": step_gbs["mixed"] / peak,
                          "fp64_frac": step_gbs["fp64"] / peak},
        "e2e": {"value": ncell / e2e["s_per_step"] / 1e6, "unit": "Mcell-steps/s",
                "h2d_bytes_per_step": e2e["h2d_bytes_per_step"],
                "d2h_bytes_per_step": e2e["d2h_bytes_per_step"]},
        "gpu_launches": mx_leg["launches"],
        "clocks": mx_leg["clocks"],
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
