"""Serving loop for transient A-formulation time steps on one GPU.

A request is one backward-Euler step of the A-formulation, or a sequence of
steps that reuses its device state, on a cube hex mesh: each step solves

    (M_sigma + dt C_nu) dA = (J, w) - C_nu A_n,      A_{n+1} = A_n + dt dA

(the CurlCurlEquationSystem residual, src/equation_systems/equation_system.cpp:
133-198, with WeakCurlCurlKernel's -C_nu A_n, src/kernels/weak_curl_curl_kernel.cpp:27-31,
and the coil load of DivFreeSource, src/sources/div_free_source.cpp:72-114).

Continuous batching: requests arrive over time (Poisson), wait in per-size-class
queues, and are admitted as soon as a worker slot and enough device memory
(their estimated HBM footprint) are free; admitted requests run concurrently,
each on its own CUDA stream, so their kernels overlap on the device.  A
request's mesh, factors, preconditioner hierarchy and Krylov state stay
resident until its last step.  The scheduler is plain host logic
(`Scheduler`), the GPU work sits in `GpuExecutor`; the scheduler runs with
any executor, so its behaviour is tested on the CPU with a fake one.
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field

import numpy as np

# size classes by dof count: requests of one class are served in arrival order,
# classes are served round-robin so small requests do not queue behind large ones
CLASS_EDGES = (1e5, 5e5)


def hex_ndof(n, p):
    a = n * p
    return 3 * a * (a + 1) ** 2


def size_class(ndof):
    for k, edge in enumerate(CLASS_EDGES):
        if ndof < edge:
            return k
    return len(CLASS_EDGES)


def footprint_bytes(n, p, precision="mixed"):
    """Conservative device-memory estimate of one resident request (bytes)."""
    N = hex_ndof(n, p)
    ne = n ** 3
    handle = ne * 12 * 12 + N * (1 + 8 * 3 + 4 * 2 + 8 * 2) + 64 * 1024
    work = N * 8 * 6 if precision == "fp64" else N * (8 + 4 * 8)
    aux = (n * p + 1) ** 3 * 4 * 5 + (n + 1) ** 3 * 4 * 11 * 8 // 7
    state = N * 8 * 3  # A, b, dA
    return int(1.15 * (handle + work + aux + state))


@dataclass
class Request:
    rid: int
    arrival: float      # seconds after the stream starts
    n: int              # elements per direction
    p: int              # Nedelec order
    steps: int          # 1, or a resident sequence
    seed: int
    ndof: int = 0
    cls: int = 0
    # filled in by the server
    start: float = -1.0
    finish: float = -1.0
    result: dict = field(default_factory=dict)

    def __post_init__(self):
        self.ndof = hex_ndof(self.n, self.p)
        self.cls = size_class(self.ndof)

    @property
    def latency(self):
        return self.finish - self.arrival


def make_stream(count, rate, seed=0, dof_range=(1e4, 2e6), orders=(1, 2, 3), multi_step_frac=0.3, steps=5):
    """Poisson arrivals (mean `rate` per second) of requests with cube meshes
    whose dof counts are log-uniform in dof_range, orders uniform in `orders`,
    and a fraction of multi-step sequences."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    lo, hi = np.log(dof_range[0]), np.log(dof_range[1])
    for k in range(count):
        t += rng.exponential(1.0 / rate)
        p = int(rng.choice(orders))
        target = np.exp(rng.uniform(lo, hi))
        n = max(2, int(round((target / 3.0) ** (1.0 / 3.0) / p)))
        while hex_ndof(n, p) > dof_range[1] and n > 2:
            n -= 1
        ns = steps if rng.uniform() < multi_step_frac else 1
        out.append(Request(k, t, n, p, ns, int(rng.integers(1 << 31))))
    return out


class Scheduler:
    """Admission and ordering: per-class FIFO queues, round-robin over classes,
    a request is admitted when a slot is free and its footprint fits."""

    def __init__(self, budget_bytes, slots, footprint=footprint_bytes):
        self.budget = budget_bytes
        self.slots = slots
        self.footprint = footprint
        self.queues = [[] for _ in range(len(CLASS_EDGES) + 1)]
        self.in_use = 0
        self.running = 0
        self.rr = 0

    def enqueue(self, req):
        if self.footprint(req.n, req.p) > self.budget:
            raise ValueError("request %d needs more device memory than the whole budget" % req.rid)
        self.queues[req.cls].append(req)

    def pending(self):
        return sum(len(q) for q in self.queues)

    def next_admissible(self):
        """Pop the next request that can start now, or None."""
        if self.running >= self.slots:
            return None
        nq = len(self.queues)
        for k in range(nq):
            c = (self.rr + k) % nq
            q = self.queues[c]
            if q and self.in_use + self.footprint(q[0].n, q[0].p) <= self.budget:
                req = q.pop(0)
                self.in_use += self.footprint(req.n, req.p)
                self.running += 1
                self.rr = (c + 1) % nq
                return req
        return None

    def release(self, req):
        self.in_use -= self.footprint(req.n, req.p)
        self.running -= 1


def run_stream(requests, executor, budget_bytes, slots, time_scale=1.0, clock=time.perf_counter):
    """Serve `requests` (sorted by arrival) with `slots` worker threads.

    executor(req, worker_index) runs the request and returns its result dict.
    Arrival times are real time (scaled by time_scale).  Returns the
    requests with start/finish filled in and the wall time.
    """
    sched = Scheduler(budget_bytes, slots)
    lock = threading.Condition()
    todo = sorted(requests, key=lambda r: r.arrival)
    pos = 0
    done = []
    free_workers = list(range(slots))
    errors = []
    t0 = clock()

    def worker(req, w):
        try:
            req.start = clock() - t0
            req.result = executor(req, w)
        except Exception as e:  # recorded, re-raised after the stream
            errors.append(e)
        finally:
            req.finish = clock() - t0
            with lock:
                sched.release(req)
                free_workers.append(w)
                done.append(req)
                lock.notify_all()

    threads = []
    with lock:
        while len(done) < len(todo):
            now = clock() - t0
            while pos < len(todo) and todo[pos].arrival * time_scale <= now:
                sched.enqueue(todo[pos])
                pos += 1
            while free_workers:
                req = sched.next_admissible()
                if req is None:
                    break
                w = free_workers.pop()
                th = threading.Thread(target=worker, args=(req, w), daemon=True)
                threads.append(th)
                th.start()
            if len(done) >= len(todo):
                break
            wait = None
            if pos < len(todo):
                wait = max(0.0, todo[pos].arrival * time_scale - (clock() - t0))
            lock.wait(timeout=wait if wait is not None else 0.5)
    for th in threads:
        th.join()
    if errors:
        raise errors[0]
    return todo, clock() - t0


def latency_stats(reqs):
    lat = np.array([r.latency for r in reqs])
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "max_s": float(lat.max())}


class GpuExecutor:
    """Runs one request on the GPU: builds the operator for its seeded fields,
    then takes its time steps with device-resident A, b, dA on a dedicated
    stream (one per worker).  keep: False, True, or a predicate on the
    request -- the final A of kept requests is copied to the host (kept).
    The default preconditioner is the additive auxiliary-space form: with the
    multiplicative cycle ("aux_mult") FP32 solves with residual replacement to
    rtol 1e-12 on small requests spend hundreds of iterations between
    replacements near the FP32 floor."""

    def __init__(self, slots, precision="mixed_rr", precond="aux", rtol=1e-12, dt=0.01, keep=False,
                 inner_rtol=None):
        import torch

        self.torch = torch
        self.streams = [torch.cuda.Stream() for _ in range(slots)]
        self.precision = precision
        self.precond = precond
        self.rtol = rtol
        self.dt = dt
        self.keep = keep
        self.kept = {}
        # residual replacement: replace after a 10x drop; refinement: inner solves to 3e-4
        self.inner_rtol = inner_rtol if inner_rtol is not None else (0.1 if precision == "mixed_rr" else 3e-4)

    @staticmethod
    def fields(req):
        """Seeded per-element nu, sigma and the coil current of a request."""
        from . import meshes

        rng = np.random.default_rng(req.seed)
        ne = req.n ** 3
        nu = meshes.loguniform(ne, 1.0, 1e3, rng)
        sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
        I0 = float(rng.uniform(0.5, 2.0))
        return nu, sigma, I0

    def __call__(self, req, w):
        from .operator import GpuHCurlPCGSolver, HCurlOperator

        torch = self.torch
        st = self.streams[w]
        nu, sigma, I0 = self.fields(req)
        with torch.cuda.stream(st):
            op = HCurlOperator(req.n, req.n, req.n, req.p, nu, sigma, dt=self.dt, ess_attr_bits=0x3F, stream=st)
            try:
                N = op.ndof
                # device state: A, the source load f, and the step's work vectors
                A = torch.zeros(N, dtype=torch.float64, device="cuda")
                f = torch.empty_like(A)
                b = torch.empty_like(A)
                dA = torch.empty_like(A)
                op.LoadCoilDevice(f, I0=I0)
                s = GpuHCurlPCGSolver({"Tolerance": self.rtol, "AbsTolerance": 0.0, "MaxIter": 5000,
                                       "Precision": self.precision, "Preconditioner": self.precond,
                                       "InnerTolerance": self.inner_rtol}, op)
                # every step (b = P (f - C A), solve, A += dt dA) runs in the library
                steps = s.StepsDevice(f, A, dA, b, req.steps)
                st.synchronize()
                last = steps[-1] if steps else {"status": "EINVAL", "rel_residual": float("nan")}
                res = {"status": last["status"], "iterations": [r["iterations"] for r in steps],
                       "rel_residual": last["rel_residual"]}
                if self.keep and (not callable(self.keep) or self.keep(req)):
                    self.kept[req.rid] = A.cpu().numpy()
                return res
            finally:
                op.close()
