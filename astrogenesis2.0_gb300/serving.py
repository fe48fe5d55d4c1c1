"""Continuous-batching request loop over the instance API of the force path.

A request is one independent simulation: its particles, its step count and
its massInH.  Requests wait in arrival order.  At every step boundary the loop
admits waiting requests while their particles fit the resident budget (first
come, first served) and advances every resident simulation by one step of the
reference's loop (Simulation.cpp:256-341) with one tree build and one walk
launch over all of them (ag2_step on a context whose instances are the
resident simulations).

Admission does not stall the residents.  A newly admitted request first needs
its initial forces (as Simulation::init computes them before the first step,
Simulation.cpp:120-139); a worker thread computes them in a second context on
its own stream while the residents take their step, and the request joins at
the next boundary (at once when nothing is resident).  A simulation that has
done its steps is read out and leaves at the next boundary, from the same
device copy of the resident state that the new instance layout is built from.

Each simulation's tree, walk and update depend only on its own particles, so
its result is the same as running it alone, bit for bit, whatever else is
resident and whenever it was admitted (tests/test_serving.py).  State stays in
HBM between steps; when the resident set changes, the particle arrays are
repacked on the device (one copy per field) into the new instance layout.
"""
from __future__ import annotations

import collections
import concurrent.futures
import dataclasses
import time

import numpy as np
import torch

import ag2

_CARRY = ("pos", "vel", "acc", "U", "dUdt")  # state that crosses a step boundary
_VEC = {"pos", "vel", "acc"}


@dataclasses.dataclass
class Request:
    rid: int
    pos: np.ndarray
    vel: np.ndarray
    mass: np.ndarray
    type: np.ndarray
    U: np.ndarray
    steps: int
    massInH: float = 0.0
    arrival: float = 0.0

    @property
    def n(self) -> int:
        return int(self.mass.shape[0])


@dataclasses.dataclass
class Result:
    rid: int
    state: dict          # host arrays: pos, vel, acc, U, dUdt
    arrival: float
    admitted: float
    completed: float
    steps: int


class _Resident:
    def __init__(self, req: Request, mass, type_, admitted: float):
        self.req = req
        self.mass = mass      # device tensors of the fields a step does not change
        self.type = type_
        self.left = req.steps
        self.admitted = admitted


class Engine:
    """Resident simulations stepped together; `capacity` particles at most
    (residents and admitted requests whose initial forces are in flight)."""

    def __init__(self, capacity: int, *, e0: float, theta: float, dt: float, G: float = 1.0,
                 stream: torch.cuda.Stream | None = None, clock=time.perf_counter):
        self.capacity = int(capacity)
        self.dt = dt
        self.clock = clock
        self.device = torch.cuda.current_device()
        self.stream = stream or torch.cuda.Stream()
        self.ctx = ag2.Context(self.capacity, G=G, e0=e0, theta=theta)
        self.ctx.set_stream(self.stream.cuda_stream)
        # the initial forces of admitted requests: their own context, stream and host thread
        self.init_stream = torch.cuda.Stream()
        self.init_ctx = ag2.Context(self.capacity, G=G, e0=e0, theta=theta)
        self.init_ctx.set_stream(self.init_stream.cuda_stream)
        self.worker = concurrent.futures.ThreadPoolExecutor(
            max_workers=1, initializer=torch.cuda.set_device, initargs=(self.device,))
        self.pending = None  # (requests, admission time, future of their initial state)
        self.waiting: collections.deque[Request] = collections.deque()
        self.resident: list[_Resident] = []
        self.n = 0
        self.layout_dirty = False
        self.steps_done = 0
        self.particle_steps = 0

    def close(self):
        if self.pending is not None:
            self.pending[2].result()
            self.pending = None
        self.worker.shutdown(wait=True)
        self.ctx.close()
        self.init_ctx.close()

    # -- queue ----------------------------------------------------------------
    def submit(self, req: Request):
        if req.n > self.capacity:
            raise ValueError(f"request {req.rid}: {req.n} particles exceed the capacity {self.capacity}")
        self.waiting.append(req)

    def idle(self) -> bool:
        return not self.resident and not self.waiting and self.pending is None

    def busy(self) -> bool:
        return bool(self.resident)

    # -- device state -----------------------------------------------------------
    def _download(self, ctx, n):
        out = {}
        for f in _CARRY:
            t = torch.empty((n, 3) if f in _VEC else (n,), dtype=torch.float64, device="cuda")
            ctx.download_device(f, t.data_ptr())
            out[f] = t
        return out

    def _initial_forces(self, new: list[Request]):
        """Initial acc and dUdt of newly admitted simulations (their own forest),
        on the worker thread and the initial-force stream; returns once they
        are on the device."""
        c = self.init_ctx
        with torch.cuda.stream(self.init_stream):
            pos = np.concatenate([r.pos for r in new])
            c.upload(pos, np.concatenate([r.mass for r in new]), np.concatenate([r.type for r in new]),
                     vel=np.concatenate([r.vel for r in new]), U=np.concatenate([r.U for r in new]))
            c.set_instances(np.concatenate([[0], np.cumsum([r.n for r in new])]),
                            np.array([r.massInH for r in new]))
            c.build_tree()
            c.sph_density()
            c.forces()
            out = self._download(c, pos.shape[0])
            mass = [torch.from_numpy(np.ascontiguousarray(q.mass, np.float64)).cuda() for q in new]
            type_ = [torch.from_numpy(np.ascontiguousarray(q.type, np.uint8)).cuda() for q in new]
        self.init_stream.synchronize()
        return out, mass, type_

    def _repack(self, joining, now: float) -> list[Result]:
        """New instance layout: the residents that have steps left, then the
        joining requests (their initial state).  Returns the simulations that
        finished, read out of the same device copy of the resident state."""
        done = []
        with torch.cuda.stream(self.stream):
            old = self._download(self.ctx, self.n) if self.resident and self.n else None
            pieces = {f: [] for f in _CARRY}
            keep = []
            off = 0
            for r in self.resident:
                if r.left > 0:
                    for f in _CARRY:
                        pieces[f].append(old[f][off:off + r.req.n])
                    keep.append(r)
                else:
                    host = {f: old[f][off:off + r.req.n].cpu().numpy() for f in _CARRY}
                    done.append(Result(r.req.rid, host, r.req.arrival, r.admitted, self.clock(), r.req.steps))
                off += r.req.n
            if joining is not None:
                new, admitted, (fresh, masses, types) = joining
                for t in list(fresh.values()) + masses + types:
                    t.record_stream(self.stream)  # made on the initial-force stream, used from here on
                off = 0
                for q, m, ty in zip(new, masses, types):
                    for f in _CARRY:
                        pieces[f].append(fresh[f][off:off + q.n])
                    keep.append(_Resident(q, m, ty, admitted))
                    off += q.n
            self.resident = keep
            self.n = sum(r.req.n for r in keep)
            if keep:
                arr = {f: torch.cat(pieces[f]).contiguous() for f in _CARRY}
                mass = torch.cat([r.mass for r in keep]).contiguous()
                type_ = torch.cat([r.type for r in keep]).contiguous()
                c = self.ctx
                c.upload_device(self.n, arr["pos"].data_ptr(), mass.data_ptr(), type_.data_ptr(),
                                arr["vel"].data_ptr(), arr["U"].data_ptr())
                c.set_field_device("acc", arr["acc"].data_ptr())
                c.set_field_device("dUdt", arr["dUdt"].data_ptr())
                c.set_instances(np.concatenate([[0], np.cumsum([r.req.n for r in keep])]),
                                np.array([r.req.massInH for r in keep]))
                self._hold = (arr, mass, type_)  # alive until the next repack
            self.stream.synchronize()
        t = self.clock()
        for d in done:
            d.completed = t
        return done

    # -- one step boundary ---------------------------------------------------------
    def step(self) -> list[Result]:
        """Join the requests whose initial forces are ready and read out the
        finished simulations; admit waiting requests (their initial forces run
        beside this step); advance every resident simulation by one step.
        Returns the simulations that finished."""
        now = self.clock()
        joining = None
        if self.pending is not None:
            new, admitted, fut = self.pending
            joining = (new, admitted, fut.result())
            self.pending = None
        budget = self.capacity - sum(r.req.n for r in self.resident if r.left > 0)
        if joining is not None:
            budget -= sum(q.n for q in joining[0])
        new = []
        while self.waiting and self.waiting[0].n <= budget:
            q = self.waiting.popleft()
            budget -= q.n
            new.append(q)
        stepping = any(r.left > 0 for r in self.resident) or joining is not None
        if new and not stepping:
            # nothing to overlap with: the new requests join now
            joining = (new, now, self._initial_forces(new))
            new = []
        done = []
        if joining is not None or self.layout_dirty:
            done = self._repack(joining, now)
            self.layout_dirty = False
        if new:
            self.pending = (new, now, self.worker.submit(self._initial_forces, new))
        if not self.resident:
            return done
        self.ctx.step(self.dt)  # ends with a check of the walk's status (a synchronisation)
        self.steps_done += 1
        self.particle_steps += self.n
        for r in self.resident:
            r.left -= 1
        if any(r.left == 0 for r in self.resident):
            self.layout_dirty = True
        return done


def run_alone(req: Request, *, e0: float, theta: float, dt: float, G: float = 1.0) -> dict:
    """The same simulation on its own context: initial forces, then its steps."""
    c = ag2.Context(req.n, G=G, e0=e0, theta=theta, massInH=req.massInH)
    c.upload(req.pos, req.mass, req.type, vel=req.vel, U=req.U)
    c.build_tree()
    c.sph_density()
    c.forces()
    for _ in range(req.steps):
        c.step(dt)
    out = {f: c.download(f) for f in _CARRY}
    c.close()
    return out


def serve(engine: Engine, trace: list[Request], *, realtime: bool = True) -> list[Result]:
    """Feed `trace` (sorted by arrival, seconds from the start) to the engine,
    in real time when `realtime`, else all at once; returns every result."""
    t0 = engine.clock()
    pending = collections.deque(sorted(trace, key=lambda r: r.arrival))
    results = []
    while pending or not engine.idle():
        now = engine.clock() - t0
        while pending and (not realtime or pending[0].arrival <= now):
            q = pending.popleft()
            if realtime:
                q.arrival = t0 + q.arrival
            engine.submit(q)
        if engine.idle() and pending:
            time.sleep(max(0.0, pending[0].arrival - (engine.clock() - t0)))
            continue
        results.extend(engine.step())
    return results
