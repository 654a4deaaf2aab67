"""Continuous-batching request loop over independent CH time-step requests.

A request asks for `steps` CH time steps on its own mesh (2D or 3D root,
optionally with nested refinement levels) from its own seeded start.
Requests are admitted as worker slots and device memory free up: a slot
builds the request's hierarchy, and if the context's HBM budget is exhausted
(`bsamg_commit` returns BSAMG_ERR_BUDGET) it waits until another request
releases its hierarchy, then retries.  Every hierarchy owns a CUDA stream and
the library releases the GIL in every call, so the work of all admitted
requests overlaps on the device; a hierarchy stays resident across all of its
time steps and is freed when the request completes.

Results are deterministic per request (no atomics or order-dependent
reductions anywhere in the library), so a request's result is the same alone
and in a mix.
"""
import math
import queue
import threading
import time

import numpy as np

from .api import BsamgError, Hierarchy

BSAMG_ERR_BUDGET = -3


class Request:
    def __init__(self, rid, ndims, n, levels, steps, eps, dt, seed, arrival=0.0, tol=1e-8, mode="mixed"):
        self.rid, self.ndims, self.n, self.levels, self.steps = rid, ndims, n, levels, steps
        self.eps, self.dt, self.seed, self.arrival, self.tol, self.mode = eps, dt, seed, arrival, tol, mode
        self.start = self.done = None
        self.vcycles = 0
        self.unconverged = 0  # steps that reached maxvcycles above tol
        self.result = None
        self.error = None
        self.phases = {}  # seconds spent in each part of run_request

    @property
    def latency(self):
        return None if self.done is None else self.done - self.arrival


def nested_spec(ndims, n, levels):
    """Patch list of a root n^d grid with its below-root levels and `levels`
    nested refinement levels, each covering the middle half of its parent
    (parent cells n/4+1 .. 3n/4), built with the reference's child rules
    (MakeNewGrid, LIBRARY/bsamroutines.f90:1663-1784)."""
    mthbc = [2] * (2 * ndims) + [10] * (6 - 2 * ndims)
    minlevel = -int(math.log2(n)) + 1
    pats = []
    dx = 1.0 / n
    mb_hi = n // 2 if minlevel < 0 else n
    pats.append(dict(level=0, id=0, parent_id=1 if minlevel < 0 else -1,
                     mx=[n] * ndims + [1] * (3 - ndims), mglobal=[1, n] * ndims + [1, 1] * (3 - ndims),
                     mbounds=[1, mb_hi] * ndims + [1, 1] * (3 - ndims), mthbc=mthbc,
                     dx=[dx] * ndims + [0.0] * (3 - ndims), xlower=[0.0, 0.0, 0.0]))
    cur, d = n, dx
    for l in range(-1, minlevel - 1, -1):
        cur //= 2
        d *= 2
        hi = cur // 2 if l > minlevel else cur
        pats.append(dict(level=l, id=-l, parent_id=-l + 1 if l > minlevel else -1,
                         mx=[cur] * ndims + [1] * (3 - ndims), mglobal=[1, cur] * ndims + [1, 1] * (3 - ndims),
                         mbounds=[1, hi] * ndims + [1, 1] * (3 - ndims), mthbc=mthbc,
                         dx=[d] * ndims + [0.0] * (3 - ndims), xlower=[0.0, 0.0, 0.0]))
    par = pats[0]
    for l in range(1, levels + 1):
        pn = par["mx"][0]
        lo, hi = pn // 4 + 1, 3 * pn // 4
        mx, mg, mb, xl = [1, 1, 1], [1, 1, 1, 1, 1, 1], [1, 1, 1, 1, 1, 1], [0.0] * 3
        for dd in range(ndims):
            mx[dd] = 2 * (hi - lo + 1)
            mb[2 * dd], mb[2 * dd + 1] = lo, hi
            g0 = par["mglobal"][2 * dd] + lo - 1
            g1 = g0 + hi - lo
            mg[2 * dd], mg[2 * dd + 1] = (g0 - 1) * 2 + 1, g1 * 2
            xl[dd] = (lo - 1) * par["dx"][dd] + par["xlower"][dd]
        child = dict(level=l, id=1000 + l, parent_id=par["id"], mx=mx, mglobal=mg, mbounds=mb,
                     mthbc=[999] * (2 * ndims) + [10] * (6 - 2 * ndims),
                     dx=[par["dx"][dd] / 2 for dd in range(ndims)] + [0.0] * (3 - ndims), xlower=xl)
        pats.append(child)
        par = child
    return pats, minlevel


class Server:
    """Worker slots over one Context; submit() requests, then drain().

    A finished request's hierarchy is kept, idle, for the next request of the
    same mesh shape (ndims, root size, levels): that request only sets its
    parameters and zeroes the fields (bsamg_set_params, bsamg_hier_reset),
    and its time steps replay the graphs the first one captured.  Idle
    hierarchies count against the HBM budget; admission frees the oldest
    idle ones before it waits for memory."""

    def __init__(self, ctx, slots=4, retry_wait=0.002, reuse=True, tail_cells=16384):
        self.ctx = ctx
        # many hierarchies share the GPU: the coarse tail of every V-cycle runs
        # in one thread block up to this many cells (bsamg_set_tail_cells)
        self.tail_cells = tail_cells
        self.slots = slots
        self.q = queue.Queue()
        self.mem = threading.Condition()
        self.retry_wait = retry_wait
        self.done = []
        self.waits = 0  # admissions that had to wait for memory
        self.reused = 0  # admissions served by an idle hierarchy
        self.reuse = reuse
        self.idle = []  # (shape key, (Hierarchy, pats, minlevel)), oldest first
        self.idle_lock = threading.Lock()
        self.lock = threading.Lock()
        self.workers = [threading.Thread(target=self._work, daemon=True) for _ in range(slots)]
        for w in self.workers:
            w.start()

    def submit(self, req):
        self.q.put(req)

    def close(self):
        for _ in self.workers:
            self.q.put(None)
        for w in self.workers:
            w.join()
        with self.idle_lock:
            idle, self.idle = self.idle, []
        for _, (h, _, _) in idle:
            h.close()

    @staticmethod
    def _key(req):
        return (req.ndims, req.n, req.levels)

    def _take_idle(self, key):
        with self.idle_lock:
            for x in range(len(self.idle) - 1, -1, -1):  # the most recently used
                if self.idle[x][0] == key:
                    return self.idle.pop(x)[1]
        return None

    def _evict_oldest(self):
        with self.idle_lock:
            if not self.idle:
                return False
            _, (h, _, _) = self.idle.pop(0)
        h.close()
        return True

    def _release(self, req, entry):
        if self.reuse:
            with self.idle_lock:
                self.idle.append((self._key(req), entry))
        else:
            entry[0].close()
        with self.mem:
            self.mem.notify_all()

    def _admit(self, req):
        """An idle hierarchy of the request's shape, or a new one built and
        committed, waiting for memory (after freeing idle ones) if needed."""
        if self.reuse:
            entry = self._take_idle(self._key(req))
            if entry is not None:
                h = entry[0]
                h.set_params([req.dt, req.eps])
                h.reset()
                with self.lock:
                    self.reused += 1
                return entry
        pats, minlevel = nested_spec(req.ndims, req.n, req.levels)
        while True:
            h = Hierarchy(self.ctx, req.ndims, 2, "ch", [req.dt, req.eps])
            for p in pats:
                h.add_patch(p["level"], p["id"], p["parent_id"], p["mx"], p["mglobal"], p["mbounds"], p["mthbc"],
                            p["dx"], p["xlower"])
            used_before = self.ctx.usage()[0]
            try:
                h.commit()
                h.set_tail_cells(self.tail_cells)
                # the per-launch path: many requests share the GPU, and their
                # launches interleave; a one-launch solve would hold its
                # cluster's SMs for a whole step (measured: 129 against 195
                # requests/s at 200 offered)
                h.set_solve(0)
                return h, pats, minlevel
            except BsamgError as e:
                h.close()
                if e.status != BSAMG_ERR_BUDGET:
                    raise
                if self._evict_oldest():
                    continue
                if used_before == 0:  # nothing else held memory: it can never fit
                    raise RuntimeError(f"request {req.rid} needs more than the whole HBM budget") from e
                with self.mem:
                    self.waits += 1
                    self.mem.wait(timeout=self.retry_wait * 10)

    def run_request(self, req):
        """Run one request to completion in the calling thread."""
        t0 = time.perf_counter()
        entry = self._admit(req)
        h, pats, minlevel = entry
        t1 = time.perf_counter()
        ok = False
        try:
            req.start = t1
            for p in pats:  # the seeded start, generated on the device
                if p["level"] >= 0:
                    h.seed_spinodal(p["id"], req.seed + p["id"])
            t2 = time.perf_counter()
            finest = max(p["level"] for p in pats)
            for s in range(req.steps):
                # as the reference, a step that reaches maxvcycles ends there
                # (MultigridIterations exits its loop silently); it is counted
                n, res = h.time_step(s == 0, finest, minlevel, 2, 30, req.tol, mode=req.mode)
                req.vcycles += n
                if res and res[-1] >= req.tol:
                    req.unconverged += 1
            t3 = time.perf_counter()
            req.result = {p["id"]: h.get(p["id"], "q") for p in pats if p["level"] >= 0}
            t4 = time.perf_counter()
            ok = True
        finally:
            if ok:
                self._release(req, entry)
            else:  # a failed run's hierarchy is not reused
                h.close()
                with self.mem:
                    self.mem.notify_all()
        req.done = time.perf_counter()
        req.phases = dict(admit=t1 - t0, init=t2 - t1, steps=t3 - t2, result=t4 - t3, close=req.done - t4)

    def _work(self):
        while True:
            req = self.q.get()
            if req is None:
                return
            try:
                self.run_request(req)
            except Exception as e:  # reported per request, the loop keeps serving
                req.error = repr(e)
                req.done = time.perf_counter()
            with self.lock:
                self.done.append(req)


def poisson_stream(rate, duration, seed, mode="mixed", max_requests=None):
    """Requests of the serving configuration: Poisson arrivals at `rate`/s;
    2D root from {32,64,128,256}^2 or 3D root from {32,64}^3, each with 0-3
    nested levels; 1-20 steps; eps ~ U(0.01, 0.03); own seed."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration or (max_requests and len(out) >= max_requests):
            return out
        if rng.random() < 0.5:
            nd, n = 2, int(rng.choice([32, 64, 128, 256]))
            levels = int(rng.integers(0, 4))
        else:
            nd, n = 3, int(rng.choice([32, 64]))
            levels = int(rng.integers(0, 4))
        steps = int(rng.integers(1, 21))
        eps = float(rng.uniform(0.01, 0.03))
        # the time steps of the 2D and 3D benchmark configurations
        dt = 1e-3 if nd == 2 else 5e-4
        out.append(Request(len(out), nd, n, levels, steps, eps, dt, seed=int(rng.integers(1, 2**31)), arrival=t,
                           mode=mode))


def serve(ctx, requests, slots=4, stats=None, tail_cells=16384):
    """Replay `requests` in real time against a Server; returns the finished
    requests and the wall time from the first arrival to the last completion
    (`stats`, if a dict, receives the number of admissions that waited)."""
    srv = Server(ctx, slots=slots, tail_cells=tail_cells)
    t0 = time.perf_counter()
    for r in requests:
        now = time.perf_counter() - t0
        if r.arrival > now:
            time.sleep(r.arrival - now)
        r.arrival = t0 + r.arrival
        srv.submit(r)
    while True:
        with srv.lock:
            if len(srv.done) == len(requests):
                break
        time.sleep(0.001)
    srv.close()
    if stats is not None:
        stats["admission_waits"] = srv.waits
        stats["reused_hierarchies"] = srv.reused
    wall = max(r.done for r in requests) - t0
    return srv.done, wall


def summarize(done, wall):
    ok = [r for r in done if r.error is None]
    lat = np.array([r.latency for r in ok]) * 1e3 if ok else np.array([0.0])
    steps = sum(r.steps for r in ok)
    errs = {}
    for r in done:
        if r.error is not None:
            errs[r.error] = errs.get(r.error, 0) + 1
    phases = {}
    for r in ok:
        for k, v in r.phases.items():
            phases[k] = phases.get(k, 0.0) + v
    phase_ms = {k: 1e3 * v / len(ok) for k, v in phases.items()} if ok else {}
    queue_ms = float(np.mean([(r.done - r.arrival) * 1e3 - sum(r.phases.values()) * 1e3 for r in ok])) if ok else 0.0
    return dict(requests=len(done), failed=len(done) - len(ok), errors=errs, wall_s=wall,
                mean_phase_ms=phase_ms, mean_queue_ms=queue_ms,
                req_per_s=len(ok) / wall if wall > 0 else 0.0, steps_per_s=steps / wall if wall > 0 else 0.0,
                p50_ms=float(np.percentile(lat, 50)), p99_ms=float(np.percentile(lat, 99)),
                vcycles=sum(r.vcycles for r in ok), unconverged_steps=sum(r.unconverged for r in ok))
