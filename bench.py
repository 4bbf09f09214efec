"""Benchmark of the LES-step hot path on one GB300.

Workload: the variable-density temporal mixing layer, 256 x 192 x 128
cells, tanh stretching in y (beta = 2), periodic x/z, slip walls in y, WALE
eddy viscosity, density ratio 2 carried by the scalar, seeded Gaussian noise
(sigma = 0.02).  Inputs are synthetic (numpy default_rng, seed 2); the
working set (~4 GB of FP64 fields) is far larger than the 129 MB L2, so no
L2 flush is needed between steps.

A step is the per-time-step hot path run through the library: eddy
viscosity (subgrid), pressure source (sour_p), the Poisson solve
(lmg_solve) to ||b - A p|| / ||b|| <= 1e-8 from a zero initial guess,
extrap_p, p_ref_subtract, the projection (uvw_adv for u, v, w, each with its
halo swap) and the slip faces (slipbc).  The step is timed twice, with the
mixed-precision solver (headline ``value``) and with the plain FP64 solver.

Output: one JSON line (rank 0).  ``--impl reference`` times the CPU oracle
(the C restatement of the reference Fortran, one thread: the reference runs
one MPI rank per block and this workload is one block) on the same workload.
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


# ----------------------------------------------------------------- helpers
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


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


def make_case():
    from fortranutils_gb300 import grid, lester as L
    ni, nj, nk = SHAPE
    lx, ly, lz = DOMAIN
    return grid.box_case(ni, nj, nk, lx=lx, ly=ly, lz=lz, ybc=L.BCT_ZERO_GRAD, beta=2.0)


def initial_fields(case, seed=2):
    """u = 0.5 tanh(2y/delta), scalar 0.5(1 + tanh(2y)), noise sigma = 0.02."""
    rng = np.random.default_rng(seed)
    b = case.blocks[0]
    nip1, njp1, nkp1 = b.n
    yv = b.y.copy()
    yv[0] = 2 * yv[1] - yv[2]
    yv[-1] = 2 * yv[-2] - yv[-3]
    yc = 0.5 * (yv[:-1] + yv[1:])[:njp1]  # cell centres j = 1..njp1
    shape = (nkp1, njp1, nip1)
    u = 0.5 * np.tanh(2.0 * yc)[None, :, None] + 0.02 * rng.standard_normal(shape)
    v = 0.02 * rng.standard_normal(shape)
    w = 0.02 * rng.standard_normal(shape)
    sc1 = np.broadcast_to(0.5 * (1.0 + np.tanh(2.0 * yc))[None, :, None], shape).copy()
    rholo, rhohi = 1.0, 2.0
    rho = 1.0 / (sc1 / rhohi + (1.0 - sc1) / rholo)
    return {k: np.ascontiguousarray(a.ravel()) for k, a in
            dict(u=u, v=v, w=w, sc1=sc1, rho=rho).items()}


# ------------------------------------------------------------ GPU arm
class GpuStep:
    """Device-resident state and the step sequence (step.F:356-450 order)."""

    def __init__(self, case, dtime):
        import torch
        from fortranutils_gb300 import lester as L
        self.L, self.torch, self.case, self.dt = L, torch, case, dtime
        c = case
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
        z3 = lambda n=c.n3_sg: torch.zeros(n, dtype=torch.float64, device="cuda")  # noqa: E731
        x, y, zc = c.coordinates()
        self.m = {k: z3(c.n2) for k in L.METRIC_NAMES}
        self.dkp, self.dkw = z3(c.n1k), z3(c.n1k)
        L.comp_metric(dev(x), dev(y), dev(zc), self.m, self.dkp, self.dkw)
        self.a = [z3(c.n3_mg) for _ in range(7)]
        m = self.m
        L.coeff_p(m["diu"], m["djv"], m["rdiv"], m["rdju"], m["didjp"], m["rp"], self.dkp,
                  self.dkw, *self.a)
        f = initial_fields(case)
        self.u0 = {k: dev(v) for k, v in f.items()}
        self.u, self.v, self.w = (self.u0[k].clone() for k in "uvw")
        self.sc1, self.rho = self.u0["sc1"].clone(), self.u0["rho"].clone()
        # slip faces first (v = 0 on the walls), so the pressure source is
        # compatible with the all-Neumann/periodic pressure problem
        L.slipbc(None, None, None, None, None, self.m["djp"], None, None, self.u, self.v,
                 z3(), self.w, self.sc1, self.rho, z3())
        for fld in (self.u, self.v, self.w, self.sc1, self.rho):
            L.swap_sc(0, 1, fld, mg_or_sg=2)
        self.ui, self.vi, self.wi = self.u.clone(), self.v.clone(), self.w.clone()
        self.rhonp1 = self.rho.clone()
        self.gam, self.gamsc1, self.sc1var, self.sc1dis = (z3() for _ in range(4))
        self.vdd = torch.ones(c.n3_sg, dtype=torch.float64, device="cuda")
        self.p = z3(c.n3_mg)
        self.s = z3(c.n3_mg)
        self.res = z3(c.n3_mg)
        self.drho, self.srhot, self.srhoux = z3(), z3(), z3()
        L.gpu_sync()

    def step(self):
        L, m, c = self.L, self.m, self.case
        L.subgrid(self.gam, self.gamsc1, self.u, self.v, self.w, self.sc1, self.rho, self.sc1var,
                  self.sc1dis, self.vdd, m["dip"], m["diu"], m["djp"], m["djv"], self.dkp,
                  self.dkw, m["hijp"], m["hjip"], m["hkip"], m["hkjp"], m["rp"])
        sl = self.s[: c.n3_sg]
        L.sour_p(m["diu"], m["djv"], m["rdiv"], m["rdju"], m["didjp"], self.dkp, m["rdidjp"],
                 self.dkw, self.ui, self.vi, self.wi, self.rho, self.rhonp1, self.drho, sl,
                 self.srhot, self.srhoux)
        self.p.zero_()
        L.lmg_solve(*self.a, self.p, self.s, self.res)
        p1 = self.p[: c.n3_sg]
        L.extrap_p(p1)
        L.p_ref_subtract(p1)
        L.uvw_adv(1, m["diu"], m["rp"], self.dkw, self.u, self.ui, self.rhonp1, p1)
        L.uvw_adv(2, m["djv"], m["rp"], self.dkw, self.v, self.vi, self.rhonp1, p1)
        L.uvw_adv(3, m["diu"], m["rp"], self.dkw, self.w, self.wi, self.rhonp1, p1)
        L.slipbc(None, None, None, None, None, m["djp"], None, None, self.u, self.v, self.vi,
                 self.w, self.sc1, self.rho, p1)


def run_gpu(args, rank):
    import torch
    from fortranutils_gb300 import build, lester as L
    build.build()
    torch.cuda.set_device(0)
    case = make_case()
    ncell = case.cells()
    dtime = 0.01
    res = {}
    modes = [("fp64", L.PSOLVE_FP64), ("mixed", L.PSOLVE_MIXED)]
    modes = [m for m in modes if args.mode in ("both", m[0])]
    for mode, ps in modes:
        ctrl = L.default_ctrl(dtime=dtime, model=2, csles=0.5, rholo=1.0, rhohi=2.0, psolve=ps,
                              rtol=1e-8, max_outer=200)
        L.gpu_init(case.geom(), ctrl)
        st = GpuStep(case, dtime)
        stream = torch.cuda.current_stream()
        for _ in range(args.warmup):
            st.step()
        L.gpu_sync()
        cyc = []
        launches0 = L.gpu_launch_count()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        L.gpu_prof(True)
        with ClockSampler(0) as clk:
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(args.steps):
                st.step()
                cyc.append(L.gpu_solve_stats()["cycles"])
            e1.record(stream)
            torch.cuda.synchronize()
        L.gpu_prof(False)
        ms = e0.elapsed_time(e1)
        kms, kl = L.gpu_prof_read()
        stats = L.gpu_solve_stats()
        res[mode] = {"ms_per_step": ms / args.steps, "cycles": float(np.mean(cyc)),
                     "relres": stats["relres"], "launches": L.gpu_launch_count() - launches0,
                     "rb_ms": kms, "rb_launches": kl, "clocks": clk.summary()}
        # e2e: the same step through the C ABI with host (pinned) buffers
        if mode == "mixed" and not args.no_e2e:
            res[mode]["e2e"] = run_e2e(args, st, case)
        del st
        L.gpu_finalize()
        torch.cuda.empty_cache()
    return case, ncell, res


def run_e2e(args, st, case):
    """Projection step with every field on the host: each call copies its
    inputs in and its outputs back (strict drop-in mode)."""
    import torch
    L = st.L
    pin = lambda t: t.detach().cpu().pin_memory().numpy()  # noqa: E731
    h = {k: pin(getattr(st, k)) for k in ("u", "v", "w", "ui", "vi", "wi", "sc1", "rho", "rhonp1",
                                          "gam", "gamsc1", "sc1var", "sc1dis", "vdd", "p", "s",
                                          "res", "drho", "srhot", "srhoux")}
    # device-resident grid data (metrics, coefficients) stay on the device:
    # they are computed once per run, as coeff_p is at istep == 1
    m, dkp, dkw, a = st.m, st.dkp, st.dkw, st.a
    c = case
    bytes_in = bytes_out = 0

    def one():
        nonlocal bytes_in, bytes_out
        L.subgrid(h["gam"], h["gamsc1"], h["u"], h["v"], h["w"], h["sc1"], h["rho"], h["sc1var"],
                  h["sc1dis"], h["vdd"], m["dip"], m["diu"], m["djp"], m["djv"], dkp, dkw,
                  m["hijp"], m["hjip"], m["hkip"], m["hkjp"], m["rp"])
        sl = h["s"][: c.n3_sg]
        L.sour_p(m["diu"], m["djv"], m["rdiv"], m["rdju"], m["didjp"], dkp, m["rdidjp"], dkw,
                 h["ui"], h["vi"], h["wi"], h["rho"], h["rhonp1"], h["drho"], sl, h["srhot"],
                 h["srhoux"])
        h["p"][:] = 0.0
        L.lmg_solve(*a, h["p"], h["s"], h["res"])
        p1 = h["p"][: c.n3_sg]
        L.extrap_p(p1)
        L.p_ref_subtract(p1)
        L.uvw_adv(1, m["diu"], m["rp"], dkw, h["u"], h["ui"], h["rhonp1"], p1)
        L.uvw_adv(2, m["djv"], m["rp"], dkw, h["v"], h["vi"], h["rhonp1"], p1)
        L.uvw_adv(3, m["diu"], m["rp"], dkw, h["w"], h["wi"], h["rhonp1"], p1)
        L.slipbc(None, None, None, None, None, m["djp"], None, None, h["u"], h["v"], h["vi"],
                 h["w"], h["sc1"], h["rho"], p1)

    one()
    L.gpu_sync()
    k = max(1, min(args.steps, 3))
    b0 = L.gpu_xfer_bytes()
    t0 = time.perf_counter()
    for _ in range(k):
        one()
    L.gpu_sync()
    dt = (time.perf_counter() - t0) / k
    b1 = L.gpu_xfer_bytes()
    return {"s_per_step": dt, "h2d_bytes_per_step": (b1[0] - b0[0]) // k,
            "d2h_bytes_per_step": (b1[1] - b0[1]) // k}


# ------------------------------------------------------------- CPU arm
def run_cpu_sample(case, budget_s=25.0):
    """The oracle on the same workload: one projection step with the
    reference algorithm (lexicographic SOR V(1,1) cycles, all levels) to
    ||b - A p|| / ||b|| <= 1e-8.  One thread."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as O
    from fortranutils_gb300 import lester as L
    orc = O.Oracle(case)
    x, y, z = case.coordinates()
    met, dkp, dkw = orc.comp_metric(x, y, z)
    m = {n: np.ascontiguousarray(met[i]) for i, n in enumerate(L.METRIC_NAMES)}
    a = [np.zeros(case.n3_mg) for _ in range(7)]
    orc.coeff_p(m, dkp, dkw, a)
    f = initial_fields(case)
    c = case
    gam, gs1, sv, sd = (np.zeros(c.n3_sg) for _ in range(4))
    vdd = np.ones(c.n3_sg)
    t0 = time.perf_counter()
    orc.subgrid(2, 0.5, 0, gam, gs1, f["u"], f["v"], f["w"], f["sc1"], sv, sd, vdd, m, dkp, dkw)
    s = np.zeros(c.n3_mg)
    outs = [np.zeros(c.n3_sg) for _ in range(4)]
    orc.sour_p(0.01, m, dkp, dkw, f["u"], f["v"], f["w"], f["rho"], f["rho"], outs)
    s[: c.n3_sg] = outs[1]
    p = np.zeros(c.n3_mg)
    r = np.zeros(c.n3_mg)
    cycles, rel = 0, 1.0
    tcyc = []
    while rel > 1e-8 and cycles < 400:
        t1 = time.perf_counter()
        out = orc.lmg_solve(O.mgctrl(nummgits=1, tolf=0.0), a, p, s, r)
        tcyc.append(time.perf_counter() - t1)
        rel = out[0] / out[1] if out[1] > 0 else 0.0
        cycles += 1
        if time.perf_counter() - t0 > budget_s:
            break
    converged = rel <= 1e-8
    p1 = p[: c.n3_sg].copy()
    orc.extrap_p(p1)
    orc.p_ref_subtract(p1)
    for iv, dg in ((1, m["diu"]), (2, m["djv"]), (3, m["diu"])):
        uu = f["uvw"[iv - 1]].copy()
        orc.uvw_adv(iv, 0.01, dg, m["rp"], dkw, uu, f["uvw"[iv - 1]], f["rho"], p1)
    elapsed = time.perf_counter() - t0
    if not converged:
        # extrapolate the remaining cycles at the measured per-cycle cost
        import math
        fac = (rel ** (1.0 / max(cycles, 1)))
        more = math.ceil(math.log(1e-8 / rel) / math.log(fac)) if 0 < fac < 1 else 0
        elapsed += more * float(np.mean(tcyc))
    return {"s_per_step": elapsed, "cycles": cycles, "converged": converged,
            "vcycle_ms": 1e3 * float(np.mean(tcyc)) if tcyc else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer (e2e) leg")
    ap.add_argument("--mode", default="both", choices=["both", "mixed", "fp64"],
                    help="solvers to time (the JSON line needs both)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if world > 1:
        # the path runs on one GPU; extra ranks are independent replicas
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    ncores = 1
    if args.impl == "reference":
        if rank != 0:
            return
        case = make_case()
        cpu = run_cpu_sample(case)
        val = case.cells() / cpu["s_per_step"] / 1e6
        line = {"metric": METRIC, "value": val, "unit": "Mcell-steps/s", "impl": "reference",
                "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": 1e3 * cpu["s_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded numpy default_rng)",
                "config": {"workload": "mixing layer 256x192x128, WALE, projection step "
                                       "(sour_p, lmg_solve to 1e-8, extrap_p, p_ref_subtract, "
                                       "uvw_adv x3)", "cells": case.cells()},
                "cpu_baseline": {"value": val, "unit": "Mcell-steps/s", "cores": ncores,
                                 "kind": "port", "sample": f"one step, {cpu['cycles']} V-cycles"
                                 + ("" if cpu["converged"] else " measured, rest extrapolated")},
                "e2e": {"value": val, "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    case, ncell, res = run_gpu(args, rank)
    if args.mode != "both" or args.no_e2e:
        print(json.dumps({k: {kk: vv for kk, vv in v.items() if kk != "clocks"}
                          for k, v in res.items()}))
        return
    mx, fp = res["mixed"], res["fp64"]
    value = ncell / (mx["ms_per_step"] * 1e-3) / 1e6 * world
    # roofline of the level-1 FP32 red-black half sweep (dominant kernel):
    # algorithmic bytes per launch = 6 B x interior cells (12 B/cell/sweep,
    # read f, b and write f in FP32, matrix-free coefficients, half per colour)
    alg = 6.0 * ncell
    rb_avg_ms = mx["rb_ms"] / max(mx["rb_launches"], 1)
    peaks = {}
    pf = ROOT / "MEASURED_PEAKS.json"
    if pf.exists():
        peaks = json.loads(pf.read_text())
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg / (rb_avg_ms * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu and rank == 0:
        cpu = run_cpu_sample(case)
    e2e = mx["e2e"]
    e2e_val = ncell / e2e["s_per_step"] / 1e6
    line = {
        "metric": METRIC, "value": value, "unit": "Mcell-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mx["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64",
        "data": "synthetic (seeded numpy default_rng, seed 2)",
        "config": {"workload": "mixing layer 256x192x128, WALE, projection step (subgrid, sour_p, "
                               "lmg_solve to 1e-8 from zero, extrap_p, p_ref_subtract, uvw_adv x3, "
                               "slipbc)",
                   "cells": ncell, "l2": "inputs larger than L2, no flush",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "fp64": {"value": ncell / (fp["ms_per_step"] * 1e-3) / 1e6 * world,
                 "ms_per_step": fp["ms_per_step"], "vcycles": fp["cycles"],
                 "vcycle_ms": None},
        "mixed": {"vcycles": mx["cycles"], "relres": mx["relres"]},
        "speedup_mixed_vs_fp64": fp["ms_per_step"] / mx["ms_per_step"],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "k_rb<float> level 1", "avg_launch_ms": rb_avg_ms},
        "e2e": {"value": e2e_val, "unit": "Mcell-steps/s",
                "h2d_bytes_per_step": e2e["h2d_bytes_per_step"],
                "d2h_bytes_per_step": e2e["d2h_bytes_per_step"]},
        "gpu_launches": mx["launches"],
        "clocks": mx["clocks"],
    }
    if cpu is not None:
        cv = ncell / cpu["s_per_step"] / 1e6
        line["cpu_baseline"] = {"value": cv, "unit": "Mcell-steps/s", "cores": ncores,
                                "kind": "port",
                                "sample": f"one projection step, {cpu['cycles']} V-cycles"
                                + ("" if cpu["converged"] else " measured, rest extrapolated")}
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
