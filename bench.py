"""Benchmark: Cahn-Hilliard time steps per second at residual <= tol, on one
GB300 per rank, batched + mixed precision vs the plain FP64 path.

Default workload (ch3d-256): 3D CH on a uniform 256^3 periodic grid,
eps = 0.02, dt = 5e-4, FAS V(2,2), levels 256^3 .. 2^3 (minlevel -7),
residual tolerance 1e-8, spinodal start phi0 = 0.1 + 0.05*U(-1,1) from a
seeded splitmix64 stream, mu0 from phi0.  A step is one CH time step
(CopyQToQold + MultigridIterations to tolerance).  --warmup + --steps time
steps run in each arm (3 + 17 = 20 by default, the configuration's 20 time
steps); the max-norm difference of phi between the mixed arm and the plain
FP64 arm (which is bit-identical to the CPU oracle) after those steps is
reported as error_vs_fp64.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Under torchrun with N > 1 every rank runs an independent replica on its own
GPU (the path does not shard); value is the sum over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "CH steps/s at resid≤1e-8: batched+mixed vs plain FP64, 1 GB300; p50/p99 ms"

WORKLOADS = {
    "ch3d-256": dict(ndims=3, n=256, minlevel=-7, mthbc=[2, 2, 2, 2, 2, 2], eps=0.02, dt=5e-4, tol=1e-8,
                     mean=0.1, amp=0.05, seed=20240503, l2="inputs larger than L2 (q+qold 550 MB FP64)",
                     desc="3D Cahn-Hilliard 256^3 periodic, eps=0.02, dt=5e-4, V(2,2), resid<=1e-8"),
    # a smaller 3D box with the same kernels and a working set still above
    # L2 (relax ~150 MB per sweep): the case the detailed ncu profiles use
    "ch3d-256x256x128": dict(ndims=3, n=256, mx=[256, 256, 128], minlevel=-6, mthbc=[2, 2, 2, 2, 2, 2], eps=0.02,
                             dt=5e-4, tol=1e-8, mean=0.1, amp=0.05, seed=20240503,
                             l2="inputs larger than L2 (q+qold 275 MB FP64)",
                             desc="3D Cahn-Hilliard 256x256x128 periodic, eps=0.02, dt=5e-4, V(2,2), resid<=1e-8"),
    "ch2d-128": dict(ndims=2, n=128, minlevel=-6, mthbc=[2, 2, 2, 2, 10, 10], eps=0.01, dt=1e-3, tol=1e-9,
                     mean=0.0, amp=0.05, seed=20240503,
                     l2="L2-resident (q+qold 0.5 MB FP64), no flush between steps: launch-bound",
                     desc="2D Cahn-Hilliard 128^2 periodic, eps=0.01, dt=1e-3, V(2,2), resid<=1e-9"),
}
# cfg2: adaptive mesh rebuilt before every step by the regrid (TakeTimeSteps'
# AMR pass).  With eps = 0.01 the interface gradient is 1/(sqrt(2) eps) = 71,
# so |grad phi| h exceeds 0.5 on levels 0-1 only; 0.25 lets three levels form.
AMR_WORKLOADS = {
    "ch2d-amr": dict(ndims=2, n=64, minlevel=-5, mthbc=[2, 2, 2, 2, 10, 10], eps=0.01, dt=1e-3, tol=1e-9,
                     maxlevel=3, tagging="gradient", qtol=0.25, ibuffer=1, mgp=4, fill=0.9, maxside=64,
                     radius=0.25, noise=0.01, seed=20240503,
                     desc="2D Cahn-Hilliard AMR: 64^2 periodic root + 3 levels (|grad phi| h > 0.25, "
                          "Berger-Rigoutsos, <= 64 cells per side, regrid every step), circle r=0.25 + 1% "
                          "noise, eps=0.01, dt=1e-3, V(2,2), resid<=1e-9"),
    # cfg4: the three-variable growth plugin (phi, nutrient, pressure) on a
    # 32^3 root with two refinement levels, mixed and FP64 paths
    "growth3d-amr": dict(ndims=3, n=32, minlevel=-4, mthbc=[10] * 6, problem="growth", nrvars=3,
                         params=[0.01, 0.025, 1.5, 2.0, 0.5, 1.0], eps=0.025, dt=0.01, tol=1e-8, maxlevel=2,
                         tagging="gradient", qtol=0.25, ibuffer=1, mgp=4, fill=0.9, maxside=64, radius=0.1,
                         noise=0.02, seed=20240503, init="sphere",
                         desc="3D growth (phi, nutrient, pressure; no reference counterpart): 32^3 root + 2 levels "
                              "(|grad phi| h > 0.25, regrid every step), sphere r = 0.1 + 0.02 U(-1,1), "
                              "eps=0.025, dt=0.01, gamma=1.5, lambda=2, c0=0.5, cpress=1, V(2,2), resid<=1e-8"),
}
NSMOOTH = 2
MAXV = 30


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max-reduce across ranks (gloo on CPU tensors); no-op at N=1."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo")
            self.td = td
            self.pg = True

    def barrier(self):
        if self.pg:
            self.td.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.td.destroy_process_group()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(workload, kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    return d.get(workload, {}).get(kernel)


class Clocks:
    """SM clock and clock-event reasons during the timed region: NVML (the
    driver's libnvidia-ml, through ctypes) read every 2 ms on a thread, or
    nvidia-smi every 25 ms when NVML cannot be loaded.  Read-only queries."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason* bits of nvml.h
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40}
    NVML_CLOCK_SM = 1

    def __init__(self, gpu):
        # the NVML / nvidia-smi name of CUDA device `gpu`: its entry in
        # CUDA_VISIBLE_DEVICES (an index or a UUID) when that is set
        vis = [v.strip() for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
        self.gpu = vis[gpu] if gpu < len(vis) else str(gpu)
        self.proc = None
        self.thread = None

    def _nvml(self):
        import ctypes
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return None
            h = ctypes.c_void_p()
            if self.gpu.isdigit():
                rc = lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(int(self.gpu)), ctypes.byref(h))
            else:
                rc = lib.nvmlDeviceGetHandleByUUID(self.gpu.encode(), ctypes.byref(h))
            if rc != 0:
                return None
            rs = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
            return lib, h, rs or lib.nvmlDeviceGetCurrentClocksThrottleReasons
        except (OSError, AttributeError):
            return None

    def _loop(self, lib, h, rs):
        import ctypes
        clk, mx, r = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        if lib.nvmlDeviceGetMaxClockInfo(h, self.NVML_CLOCK_SM, ctypes.byref(mx)) == 0:
            self.max = float(mx.value)
        while not self.done.is_set():
            if lib.nvmlDeviceGetClockInfo(h, self.NVML_CLOCK_SM, ctypes.byref(clk)) == 0:
                self.sm.append(float(clk.value))
            if rs(h, ctypes.byref(r)) == 0:
                self.reasons.update(nm for nm, bit in self.BITS.items() if r.value & bit)
            time.sleep(0.002)

    def start(self):
        nv = self._nvml()
        if nv:
            import threading
            self.sm, self.max, self.reasons = [], None, set()
            self.done = threading.Event()
            self.thread = threading.Thread(target=self._loop, args=nv, daemon=True)
            self.thread.start()
            return
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.gpu, f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "25"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.thread:
            self.done.set()
            self.thread.join(timeout=5)
            if not self.sm:
                return None
            return {"sm_mhz": statistics.median(self.sm), "sm_max_mhz": self.max, "samples": len(self.sm),
                    "reasons": sorted(self.reasons), "source": "nvml, every 2 ms"}
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        rows = [r.split(",") for r in out.strip().splitlines() if r.strip()]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "samples": len(sm),
                "reasons": sorted(reasons), "source": "nvidia-smi, every 25 ms"}


def root_mx(w):
    """root extents (3 entries) and upper domain corner of a uniform workload"""
    nd, n = w["ndims"], w["n"]
    mx = list(w.get("mx", [n] * nd)) + [1] * (3 - nd)
    return mx, [mx[d] / n if d < nd else 1 for d in range(3)]


def make_hierarchy(pkg, ctx, w):
    mx, up = root_mx(w)
    h = pkg.Hierarchy(ctx, w["ndims"], 2, "ch", [w["dt"], w["eps"]])
    h.build_uniform(mx, w["minlevel"], w["mthbc"], [0, 0, 0], up)
    h.commit()
    return h


def initial_q(pkg, w):
    nd, n = w["ndims"], w["n"]
    mx, _ = root_mx(w)
    q = pkg.initial.ch_spinodal(tuple(mx[:nd]), w["eps"], 1.0 / n, seed=w["seed"], mean=w["mean"], amp=w["amp"])
    return np.asfortranarray(q).ravel(order="F")


def reset(h, q0, w):
    h.put_flat(0, "q", q0)
    h.set_ghost(0, 0)
    h.copy_q_to_qold(w["minlevel"], 0)


def run_arm(h, q0, w, mode, steps, warmup, dist, clocks=None):
    """warmup + timed steps; returns dict of timings and the V-cycle counts."""
    reset(h, q0, w)
    vc = []
    for s in range(warmup):
        n, _ = h.time_step(s == 0, 0, w["minlevel"], NSMOOTH, MAXV, w["tol"], mode=mode, strict=True)
        vc.append(n)
    h.sync()
    dist.barrier()
    if clocks:
        clocks.start()
    l0 = h.launch_count()
    h.mark(0)
    per = []
    for s in range(steps):
        n, res = h.time_step(warmup == 0 and s == 0, 0, w["minlevel"], NSMOOTH, MAXV, w["tol"], mode=mode,
                             strict=True)
        h.mark(1 + (s % 60))
        vc.append(n)
        per.append(h.elapsed_ms(0 if s == 0 else 1 + ((s - 1) % 60), 1 + (s % 60)))
    h.sync()
    ck = clocks.stop() if clocks else None
    total = h.elapsed_ms(0, 1 + ((steps - 1) % 60))
    launches = h.launch_count() - l0
    dist.barrier()
    return dict(total_ms=total, per_ms=per, vcycles=vc, launches=launches, clocks=ck,
                final_resid=res[-1])


def run_e2e(pkg, h, q0, w, mode, steps, warmup, dist, buffers="allocated"):
    """Public-API end to end: per step, H2D of q from pinned host memory,
    the time step, D2H of q into pinned host memory (two pinned buffers
    alternate as input and output, as a host that keeps its state would).
    The buffers come from the CUDA pinned allocator (through torch), or are
    numpy arrays page-locked in place (buffers="registered"); on one GB300 the
    allocator's buffers moved 173-208 GB/s host to device against 184-185 for
    registered ones (two runs each): the link's own variation dominates.
    Returns the total time, the bytes of q and the device time of the
    uploads and of the downloads over the timed steps (events around each
    copy on the hierarchy's stream)."""
    keep = None
    if buffers == "registered":
        bufs = [pkg.pin(np.array(q0, copy=True)), pkg.pin(np.empty_like(q0))]
    else:
        import torch
        keep = [torch.empty(q0.size, dtype=torch.float64, pin_memory=True) for _ in range(2)]
        bufs = [t.numpy() for t in keep]
        bufs[0][:] = q0
    reset(h, q0, w)
    first = True
    cur = 0
    up_ms = down_ms = 0.0
    for s in range(warmup + steps):
        if s == warmup:
            dist.barrier()
            h.mark(10)
        h.mark(12)
        h.put_flat(0, "q", bufs[cur])
        h.mark(13)
        h.time_step(first, 0, w["minlevel"], NSMOOTH, MAXV, w["tol"], mode=mode, strict=True)
        h.mark(14)
        h.get(0, "q", out=bufs[1 - cur])
        h.mark(15)
        if s >= warmup:
            up_ms += h.elapsed_ms(12, 13)
            down_ms += h.elapsed_ms(14, 15)
        cur = 1 - cur
        first = False
    h.mark(11)
    ms = h.elapsed_ms(10, 11)
    dist.barrier()
    nbytes = bufs[0].nbytes
    if keep is None:
        for b in bufs:
            pkg.unpin(b)
    del keep
    return ms, nbytes, up_ms, down_ms


def pct(x, p):
    return float(np.percentile(np.asarray(x), p))


def cpu_baseline(pkg, w, vcycles_per_step, nvc=2):
    """The CPU oracle (C restatement of the reference, 1 thread) on the same
    workload: nvc V-cycles of the first step, scaled to steps/s with the
    V-cycle count per step of the FP64 run."""
    from oracle.bsam_oracle import OracleHierarchy
    nd, n = w["ndims"], w["n"]
    mx, up = root_mx(w)
    o = OracleHierarchy(nd, 2, "ch", [w["dt"], w["eps"]])
    o.build_uniform(mx, w["minlevel"], w["mthbc"], [0, 0, 0], up)
    o.commit()
    o.put(0, "q", initial_q(pkg, w))
    o.set_ghost(0, 0)
    o.fill_down("q", 0, w["minlevel"])
    o.copy_q_to_qold(w["minlevel"], 0)
    t = time.perf_counter()
    o.multigrid_iterations(0, w["minlevel"], NSMOOTH, nvc, 0.0)
    dt = time.perf_counter() - t
    per_v = dt / nvc
    return per_v, dict(value=1.0 / (per_v * vcycles_per_step), unit="steps/s", cores=1, kind="port",
                       sample=f"oracle (C restatement of the reference, 1 thread, -O2 -ffp-contract=off) "
                              f"running {nvc} V-cycles of the first time step of the same "
                              f"workload ({dt:.1f} s); steps/s = 1/(t_vcycle x {vcycles_per_step:.2f} "
                              f"V-cycles per step of the FP64 run)")


def arm_config(args, w, dist):
    """the config block of a uniform workload's JSON line (both arms)"""
    return {"workload": args.workload, "desc": w["desc"], "n": w["n"], "ndims": w["ndims"],
            "minlevel": w["minlevel"], "nsmooth": NSMOOTH, "tol": w["tol"],
            "parallelism": f"replicas x{dist.ws}",
            "l2": w["l2"]}


def reference_arm(args, w, dist):
    """--impl reference: the reference algorithm on the host cores (the CPU
    oracle, one thread like the reference: the reference itself is Fortran
    and no Fortran compiler exists on these machines).  The same time steps
    as the GPU arms: --warmup full steps untimed, then --steps full steps
    timed, each a CopyQToQold + MultigridIterations to the tolerance
    (TakeTimeSteps, bsamroutines.f90:608-816, on a fixed mesh)."""
    if dist.rank != 0:
        return
    import __graft_entry__ as ge
    pkg_initial = ge.load_package().initial  # numpy input generator only; libbsamg is not loaded
    from oracle.bsam_oracle import OracleHierarchy
    nd, n = w["ndims"], w["n"]
    mx, up = root_mx(w)
    o = OracleHierarchy(nd, 2, "ch", [w["dt"], w["eps"]])
    o.build_uniform(mx, w["minlevel"], w["mthbc"], [0, 0, 0], up)
    o.commit()
    q = pkg_initial.ch_spinodal(tuple(mx[:nd]), w["eps"], 1.0 / n, seed=w["seed"], mean=w["mean"], amp=w["amp"])
    o.put(0, "q", q)
    o.set_ghost(0, 0)
    o.copy_q_to_qold(w["minlevel"], 0)
    vc, ts = [], []
    t_warm = time.perf_counter()
    for s in range(args.warmup):
        nv, _ = o.time_step(s == 0, 0, w["minlevel"], NSMOOTH, MAXV, w["tol"])
    t_warm = time.perf_counter() - t_warm
    for s in range(args.steps):
        t = time.perf_counter()
        nv, _ = o.time_step(args.warmup == 0 and s == 0, 0, w["minlevel"], NSMOOTH, MAXV, w["tol"])
        ts.append(time.perf_counter() - t)
        vc.append(nv)
    total = sum(ts)
    value = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded splitmix64 spinodal start, mu0 from phi0)",
        "config": arm_config(args, w, dist),
        "p50_ms": 1e3 * pct(ts, 50), "p99_ms": 1e3 * pct(ts, 99),
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": 1, "kind": "port",
                         "sample": f"oracle (C restatement of the reference, 1 thread, -O2 -ffp-contract=off): "
                                   f"{args.warmup} full time steps untimed ({t_warm:.1f} s), then {args.steps} "
                                   f"full time steps timed ({total:.1f} s), the same steps as the GPU arms"},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "vcycles_per_step": statistics.mean(vc),
    }
    print(json.dumps(line), flush=True)


def amr_params(api, w, step):
    return api.regrid_params(w["maxlevel"], tagging=w["tagging"], initial=step == 0, maxside=w["maxside"],
                             first_id=100000 * (step + 1), ibuffer=w["ibuffer"], minimumgridpoints=w["mgp"],
                             qtolerance=w["qtol"], desiredfillratio=w["fill"])


def amr_run(api, make_root, w, mode, steps, warmup, use_events=True):
    """warmup + timed steps of regrid + time step; returns timings, V-cycle
    counts and the final mesh."""
    qinit = api_qinit(w)
    h = make_root()
    wall, solve, vc, rgt = [], [], [], []
    t_start = None
    for s in range(warmup + steps):
        if s == warmup:
            if use_events:
                h.sync()
            t_start = time.perf_counter()
        t0 = time.perf_counter()
        old = h
        h = h.regrid(amr_params(api, w, s), qinit if s == 0 else None)
        if use_events:
            old.close()
        t1 = time.perf_counter()
        fin = h.level_range()[1]
        kw = dict(mode=mode, strict=True) if use_events else {}
        n, res = h.time_step(s == 0, fin, w["minlevel"], NSMOOTH, MAXV, w["tol"], **kw)
        if use_events:
            h.sync()
        t2 = time.perf_counter()
        if s >= warmup:
            wall.append(t2 - t0)
            solve.append(t2 - t1)
            if hasattr(h, "regrid_timing"):
                rgt.append(h.regrid_timing())
        vc.append(n)
    total = time.perf_counter() - t_start
    return dict(total_s=total, wall=wall, solve=solve, vcycles=vc[warmup:], h=h, regrid_parts=rgt)


def api_qinit(w):
    import __graft_entry__ as ge
    ini = ge.load_package().initial
    if w.get("init") == "sphere":
        return ini.growth_sphere(w["eps"], w["seed"], radius=w["radius"], noise=w["noise"])
    return ini.ch_circle_patch(w["eps"], w["seed"], radius=w["radius"], noise=w["noise"])


def amr_hier_args(w):
    return w["ndims"], w.get("nrvars", 2), w.get("problem", "ch"), w.get("params", [w["dt"], w["eps"]])


def mesh_stats(tab, nd=2):
    levels = {}
    for p in tab:
        if p["level"] < 0:
            continue
        d = levels.setdefault(p["level"], {"patches": 0, "cells": 0})
        d["patches"] += 1
        d["cells"] += int(np.prod(p["mx"][:nd]))
    sides = [max(p["mx"][:nd]) for p in tab if p["level"] > 0]
    hist = {}
    for b in (8, 16, 32, 64, 128):
        hist[f"<={b}"] = sum(1 for x in sides if x <= b) - sum(v for v in hist.values())
    return {"levels": levels, "patch_side_histogram": hist}


def amr_arm(args, w, dist):
    """--workload ch2d-amr: cfg2.  Each step is the reference's TakeTimeSteps
    body with AMR: the regrid (host clustering, new device hierarchy) then
    CopyQToQold + MultigridIterations.  Timed on the host clock with the
    device synchronised after each step, because the regrid is host work."""
    import __graft_entry__ as ge
    ge._load_build_module().build()
    pkg = ge.load_package()
    ctx = pkg.Context(dist.local)
    nd, n = w["ndims"], w["n"]

    def make_root():
        h = pkg.Hierarchy(ctx, *amr_hier_args(w))
        h.build_uniform([n] * nd + [1] * (3 - nd), w["minlevel"], w["mthbc"], [0, 0, 0], [1, 1, 1])
        h.commit()
        h.put(0, "q", api_qinit(w)(0, [n] * nd, [1.0 / n] * nd, [0.0] * nd))
        return h

    out = {}
    modes = w.get("modes", ("mixed", "fp64"))
    for mode in modes:
        dist.barrier()
        r = amr_run(pkg, make_root, w, mode, args.steps, args.warmup)
        r["tab"] = r["h"].patch_table()
        out[mode] = r
    m, f = out[modes[0]], out["fp64"]
    same_mesh = [(p["level"], p["mglobal"]) for p in m["tab"]] == [(p["level"], p["mglobal"]) for p in f["tab"]]
    err = None
    if same_mesh:
        worst = 0.0
        for p in f["tab"]:
            if p["level"] < 0:
                continue
            a, b = m["h"].get(p["id"], "q"), f["h"].get(p["id"], "q")
            k = a.size // w.get("nrvars", 2)
            worst = max(worst, float(np.max(np.abs(a[:k] - b[:k])) / np.max(np.abs(b[:k]))))
        err = worst
    t_m = dist.max(m["total_s"])
    t_f = dist.max(f["total_s"])
    value = dist.ws * args.steps / t_m
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": dist.ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_m / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if modes[0] == "mixed" else "f64",
        "data": "synthetic (seeded splitmix64 noise on a tanh " + ("sphere)" if w.get("init") == "sphere" else "circle)"),
        "config": {"workload": args.workload, "desc": w["desc"], "regrid": "every step (host clustering)",
                   "l2": "L2-resident, launch- and host-bound (working set of a few MB per level)"},
        "p50_ms": 1e3 * pct(m["wall"], 50), "p99_ms": 1e3 * pct(m["wall"], 99),
        "regrid_ms_per_step": 1e3 * (statistics.mean(m["wall"]) - statistics.mean(m["solve"])),
        "solve_ms_per_step": 1e3 * statistics.mean(m["solve"]),
        "vcycles_per_step": statistics.mean(m["vcycles"]),
        "plain_fp64": {"value": dist.ws * args.steps / t_f, "unit": "steps/s", "ms_per_step": 1e3 * t_f / args.steps,
                       "solve_ms_per_step": 1e3 * statistics.mean(f["solve"]),
                       "vcycles_per_step": statistics.mean(f["vcycles"])},
        "speedup_mixed_vs_fp64": t_f / t_m if modes[0] == "mixed" else None,
        "mixed": "run" if modes[0] == "mixed" else "not built for this plugin (the correction smoother is CH's)",
        "error_vs_fp64": {"max_rel_phi": err, "same_mesh": same_mesh, "after_steps": args.warmup + args.steps},
        "mesh": mesh_stats(f["tab"], nd),
        "timing": "host clock around regrid + time step, device synchronised after each step",
    }
    if modes[0] == "mixed":
        hm = m["h"]
        form, ctas, threads, tile, solo = hm.get_solve()
        info = hm.solve_info()
        one_launch = form == 1 and info["phases"] > 0
        line["mixed_solve"] = {
            "form": "one cluster launch per solve" if one_launch else "per-launch graphs (chosen by the autotuner)",
            "ctas": ctas if one_launch else None, "threads": threads if one_launch else None,
            "tile_units": tile if one_launch else None, "one_cta_coarse_cells": solo if one_launch else None,
            "phases_per_program": info["phases"], "levels_in_dsmem": info["dsm_levels"],
            "dsmem_bytes_per_cta": info["data_bytes"], "image_bytes_per_cta": info["image_bytes"],
            "tuned_size_classes": ctx.tune_count()}
    if m["regrid_parts"]:
        keys = m["regrid_parts"][0].keys()
        line["regrid_breakdown_ms"] = {k: statistics.mean(r[k] for r in m["regrid_parts"]) for k in keys}
    if not args.no_cpu_baseline:
        from oracle import bsam_oracle as om

        def oracle_root():
            o = om.OracleHierarchy(*amr_hier_args(w))
            o.build_uniform([n] * nd + [1] * (3 - nd), w["minlevel"], w["mthbc"], [0, 0, 0], [1, 1, 1])
            o.commit()
            o.put(0, "q", api_qinit(w)(0, [n] * nd, [1.0 / n] * nd, [0.0] * nd))
            return o

        class OAPI:  # the oracle behind the same regrid/time-step calls
            regrid_params = staticmethod(om.regrid_params)

        def wrap(o):
            class W:
                def __init__(self, o):
                    self.o = o

                def regrid(self, prm, qinit=None):
                    return W(om.regrid(self.o, prm, qinit))

                def patch_table(self):
                    return self.o.patch_table()

                def level_range(self):
                    return self.o.level_range()

                def time_step(self, *a, **k):
                    return self.o.time_step(*a, **k)
            return W(o)

        ns = 3
        r = amr_run(OAPI, lambda: wrap(oracle_root()), w, "fp64", ns, 1, use_events=False)
        line["cpu_baseline"] = {"value": ns / r["total_s"], "unit": "steps/s", "cores": 1, "kind": "port",
                                "sample": f"oracle (C restatement, 1 thread): regrid + time step, steps 2-{ns + 1} "
                                          f"of the same run ({r['total_s']:.1f} s)"}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    for r in out.values():
        r["h"].close()
    ctx.close()


def amr_reference_arm(args, w, dist):
    """--impl reference for the AMR workload: the oracle (the reference
    algorithm restated in C; the Fortran cannot be built here) runs the
    same steps -- regrid, then the time step -- on one host core."""
    if dist.rank != 0:
        return
    from oracle import bsam_oracle as om
    nd, n = w["ndims"], w["n"]
    qinit = api_qinit(w)
    o = om.OracleHierarchy(*amr_hier_args(w))
    o.build_uniform([n] * nd + [1] * (3 - nd), w["minlevel"], w["mthbc"], [0, 0, 0], [1, 1, 1])
    o.commit()
    o.put(0, "q", qinit(0, [n] * nd, [1.0 / n] * nd, [0.0] * nd))
    ts, vc = [], []
    for s in range(args.warmup + args.steps):
        t = time.perf_counter()
        o = om.regrid(o, amr_params(om, w, s), qinit if s == 0 else None)
        fin = max(p["level"] for p in o.patch_table())
        nv, _ = o.time_step(s == 0, fin, w["minlevel"], NSMOOTH, MAXV, w["tol"])
        if s >= args.warmup:
            ts.append(time.perf_counter() - t)
            vc.append(nv)
    value = len(ts) / sum(ts)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(ts),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded splitmix64 noise on a tanh " + ("sphere)" if w.get("init") == "sphere" else "circle)"),
        "config": {"workload": args.workload, "desc": w["desc"]},
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": 1, "kind": "port",
                         "sample": "every step in full: regrid + CopyQToQold + MultigridIterations"},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "vcycles_per_step": statistics.mean(vc),
    }
    print(json.dumps(line), flush=True)


def serve_arm(args, dist):
    """--workload serve: the serving configuration.  Poisson arrivals (mean
    200/s, seeded) of independent CH requests, replayed in real time against
    the continuous-batching loop, once with the mixed path and once with the
    plain FP64 path; value = completed time steps per second of the mixed run."""
    import __graft_entry__ as ge
    ge._load_build_module().build()
    pkg = ge.load_package()
    duration = max(0.5, args.steps / 10.0)
    out = {}
    for mode in ("mixed", "fp64"):
        ctx = pkg.Context(dist.local, hbm_budget=int(args.serve_budget_gb * 2**30))
        if args.serve_blocking_wait:
            ctx.set_blocking_wait(True)
        warm = pkg.serve.poisson_stream(200.0, 0.05, seed=7, mode=mode)
        pkg.serve.serve(ctx, warm, slots=args.serve_slots, tail_cells=args.serve_tail_cells)
        reqs = pkg.serve.poisson_stream(200.0, duration, seed=2024, mode=mode)
        stats = {}
        done, wall = pkg.serve.serve(ctx, reqs, slots=args.serve_slots, stats=stats,
                                     tail_cells=args.serve_tail_cells)
        ctx.close()
        out[mode] = dict(pkg.serve.summarize(done, wall), **stats)
    m, f = out["mixed"], out["fp64"]
    line = {
        "metric": METRIC, "value": m["steps_per_s"], "unit": "steps/s", "n_gpus": dist.ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 / m["steps_per_s"] if m["steps_per_s"] else None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded Poisson arrivals and spinodal starts)",
        "config": {"workload": "serve", "arrival_rate_per_s": 200.0, "arrival_window_s": duration,
                   "slots": args.serve_slots, "hbm_budget_gb": args.serve_budget_gb,
                   "tail_cells": args.serve_tail_cells, "blocking_wait": bool(args.serve_blocking_wait),
                   "mix": "2D roots {32,64,128,256}^2 or 3D roots {32,64}^3, each with 0-3 nested levels, 1-20 steps"},
        "p50_ms": m["p50_ms"], "p99_ms": m["p99_ms"], "serving_mixed": m, "serving_fp64": f,
        "speedup_mixed_vs_fp64": m["steps_per_s"] / f["steps_per_s"] if f["steps_per_s"] else None,
    }
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=17)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ch3d-256", choices=list(WORKLOADS) + list(AMR_WORKLOADS) + ["serve"])
    ap.add_argument("--serve-slots", type=int, default=64)
    ap.add_argument("--serve-budget-gb", type=float, default=64.0)
    ap.add_argument("--serve-tail-cells", type=int, default=16384)
    ap.add_argument("--serve-blocking-wait", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-buffers", default="allocated", choices=["allocated", "registered"],
                    help="the e2e leg's pinned host buffers: from the CUDA pinned allocator or registered numpy")
    ap.add_argument("--maxv", type=int, default=MAXV,
                    help="V-cycles allowed per step; above 64 the periodic-box solve runs its host loop "
                         "instead of one graph launch (the same cycles, launched one by one)")
    ap.add_argument("--box-sweep", type=int, default=None,
                    help="smoothing form of periodic-box levels (bsamg_set_box_sweep); default: the library's")
    args = ap.parse_args()
    globals()["MAXV"] = args.maxv
    dist = Dist()
    if args.workload == "serve":
        if args.impl == "reference":
            if dist.rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the serving loop has no CPU counterpart in "
                                  "the reference (a single serial solve per run)"}), flush=True)
        else:
            serve_arm(args, dist)
        dist.close()
        return
    if args.workload in AMR_WORKLOADS:
        w = AMR_WORKLOADS[args.workload]
        if args.impl == "reference":
            amr_reference_arm(args, w, dist)
        else:
            amr_arm(args, w, dist)
        dist.close()
        return
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        reference_arm(args, w, dist)
        dist.close()
        return
    import __graft_entry__ as ge
    ge._load_build_module().build()
    pkg = ge.load_package()
    ctx = pkg.Context(dist.local)
    h = make_hierarchy(pkg, ctx, w)
    if args.box_sweep is not None:
        h.set_box_sweep(args.box_sweep)
    q0 = pkg.pin(initial_q(pkg, w))
    N = int(np.prod(root_mx(w)[0]))

    clocks = Clocks(dist.local)
    mixed = run_arm(h, q0, w, "mixed", args.steps, args.warmup, dist, clocks)
    q_mixed = h.get(0, "q")
    ms_mixed = h.time_smoother(0, "mixed", reps=20)
    col_mixed = h.smoother_colours(0, "mixed")
    fp64 = run_arm(h, q0, w, "fp64", args.steps, args.warmup, dist)
    q_fp64 = h.get(0, "q")
    ms_fp64 = h.time_smoother(0, "fp64", reps=10)
    # the same time steps as the resident run (same warm-up), so both legs
    # see the same V-cycle counts
    e2e_ms, qbytes, up_ms, down_ms = (None, 0, 0, 0) if args.no_e2e else run_e2e(
        pkg, h, q0, w, "mixed", args.steps, args.warmup, dist, args.e2e_buffers)

    t_mixed = dist.max(mixed["total_ms"])
    t_fp64 = dist.max(fp64["total_ms"])
    value = dist.ws * args.steps / (t_mixed * 1e-3)
    v_fp64 = dist.ws * args.steps / (t_fp64 * 1e-3)
    nphi = q_fp64.size // 2
    err = float(np.max(np.abs(q_mixed[:nphi] - q_fp64[:nphi])) / np.max(np.abs(q_fp64[:nphi])))
    peak, peak_kind = peaks()
    # uniform periodic workloads with even extents run the periodic-box mixed
    # path (colour-split arrays), the others the general one
    kmix = "k_bx_relax" if all(m == 2 for m in w["mthbc"][:2 * w["ndims"]]) else "k_mx_relax"
    kdesc = "FP32 colour sweep of the correction, finest level"
    if kmix == "k_bx_relax" and col_mixed == 4:
        kmix = "k_bx_smooth"
        kdesc = "one-pass V(2,2) smoothing of the correction (four colour half-sweeps), finest level"
    # per colour half-sweep: e read (N*2*4) + g, phib and e write of that colour (N/2*(2*4+4+2*4)) = 18 N
    # (the per-sweep figure 4*N*V*s + N*s for the two colours); the one-pass smoothing performs four
    # half-sweeps per launch (72 N) while moving 28 N (e, g, phib read once, e written once)
    b_mixed = 18.0 * N * col_mixed
    b_fp64 = 32.0 * N   # q read (N*2*8) + f read and q write of one colour (N/2*(2*8+2*8))
    ach = b_mixed / (ms_mixed * 1e-3) / 1e9
    ach64 = b_fp64 / (ms_fp64 * 1e-3) / 1e9
    vps_m = statistics.mean(mixed["vcycles"][args.warmup:])
    vps_f = statistics.mean(fp64["vcycles"][args.warmup:])
    if dist.rank != 0:
        dist.close()
        return
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": dist.ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_mixed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded splitmix64 spinodal start, mu0 from phi0)",
        "config": arm_config(args, w, dist),
        "p50_ms": pct(mixed["per_ms"], 50), "p99_ms": pct(mixed["per_ms"], 99),
        "vcycles_per_step": vps_m,
        "plain_fp64": {"value": v_fp64, "unit": "steps/s", "ms_per_step": t_fp64 / args.steps,
                       "p50_ms": pct(fp64["per_ms"], 50), "p99_ms": pct(fp64["per_ms"], 99),
                       "vcycles_per_step": vps_f, "gpu_launches": fp64["launches"]},
        "speedup_mixed_vs_fp64": value / v_fp64,
        "error_vs_fp64": {"max_rel_phi": err, "after_steps": args.warmup + args.steps},
        "dof_sweeps_per_s": None,
        "roofline": {"bound": "hbm", "kernel": f"{kmix} ({kdesc})",
                     "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                     "peak_kind": peak_kind, "bytes_per_launch": b_mixed, "ms_per_launch": ms_mixed,
                     "half_sweeps_per_launch": col_mixed,
                     "dram_bytes_needed": (28.0 if col_mixed == 4 else 18.0) * N,
                     "traffic": ncu_traffic(args.workload, kmix)},
        "roofline_fp64": {"bound": "fp64 pipe", "kernel": "k_relax (FP64 colour sweep, finest level)",
                          "achieved_hbm": ach64, "peak_hbm": peak, "frac_hbm": ach64 / peak,
                          "bytes_per_launch": b_fp64, "ms_per_launch": ms_fp64,
                          "traffic": ncu_traffic(args.workload, "k_relax")},
        "gpu_launches": mixed["launches"],
        "clocks": mixed["clocks"],
    }
    # 4 colour sweeps of the finest level per pass pair, 2*NSMOOTH*2 sweeps per V-cycle on the finest level
    line["dof_sweeps_per_s"] = 2 * N * (2 * NSMOOTH) * vps_m * value
    if e2e_ms is not None:
        line["e2e"] = {"value": dist.ws * args.steps / (e2e_ms * 1e-3), "unit": "steps/s",
                       "h2d_bytes_per_step": qbytes, "d2h_bytes_per_step": qbytes,
                       # the host link's share: device time of the copies alone
                       "h2d_ms_per_step": up_ms / args.steps, "d2h_ms_per_step": down_ms / args.steps,
                       "h2d_gbs": qbytes * args.steps / (up_ms * 1e6),
                       "d2h_gbs": qbytes * args.steps / (down_ms * 1e6),
                       "host_buffers": "CUDA pinned allocator" if args.e2e_buffers == "allocated"
                       else "numpy arrays page-locked in place"}
    if not args.no_cpu_baseline:
        per_v, cb = cpu_baseline(pkg, w, vps_f)
        line["cpu_baseline"] = cb
    print(json.dumps(line), flush=True)
    h.close()
    ctx.close()
    dist.close()


if __name__ == "__main__":
    main()
