"""Continuous-batching request loop over the instance API of the force path.

A request is one independent simulation: its particles, its step count and
its massInH.  Requests wait in arrival order.  At every step boundary the loop
admits waiting requests while their particles fit the resident budget (first
come, first served), computes their initial forces (as Simulation::init does
before the first step, Simulation.cpp:120-139), and then advances every
resident simulation by one step of the reference's loop (Simulation.cpp:256-341)
with one tree build and one walk launch over all of them (ag2_step on a context
whose instances are the resident simulations).  A simulation that has done its
steps leaves at the next boundary with its final state.

Each simulation's tree, walk and update depend only on its own particles, so
its result is the same as running it alone, bit for bit, whatever else is
resident (tests/test_serving.py).  State stays in HBM between steps; when the
resident set changes, the particle arrays are repacked on the device (one copy
per field) into the new instance layout.
"""
from __future__ import annotations

import collections
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
    """Resident simulations stepped together; `capacity` particles at most."""

    def __init__(self, capacity: int, *, e0: float, theta: float, dt: float, G: float = 1.0,
                 stream: torch.cuda.Stream | None = None, clock=time.perf_counter):
        self.capacity = int(capacity)
        self.dt = dt
        self.clock = clock
        self.stream = stream or torch.cuda.Stream()
        self.ctx = ag2.Context(self.capacity, G=G, e0=e0, theta=theta)
        self.ctx.set_stream(self.stream.cuda_stream)
        self.init_ctx = ag2.Context(self.capacity, G=G, e0=e0, theta=theta)
        self.init_ctx.set_stream(self.stream.cuda_stream)
        self.waiting: collections.deque[Request] = collections.deque()
        self.resident: list[_Resident] = []
        self.n = 0
        self.layout_dirty = False
        self.steps_done = 0
        self.particle_steps = 0

    def close(self):
        self.ctx.close()
        self.init_ctx.close()

    # -- queue ----------------------------------------------------------------
    def submit(self, req: Request):
        if req.n > self.capacity:
            raise ValueError(f"request {req.rid}: {req.n} particles exceed the capacity {self.capacity}")
        self.waiting.append(req)

    def idle(self) -> bool:
        return not self.resident and not self.waiting

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
        """Initial acc and dUdt of newly admitted simulations (their own forest)."""
        c = self.init_ctx
        pos = np.concatenate([r.pos for r in new])
        c.upload(pos, np.concatenate([r.mass for r in new]), np.concatenate([r.type for r in new]),
                 vel=np.concatenate([r.vel for r in new]), U=np.concatenate([r.U for r in new]))
        c.set_instances(np.concatenate([[0], np.cumsum([r.n for r in new])]),
                        np.array([r.massInH for r in new]))
        c.build_tree()
        c.sph_density()
        c.forces()
        return self._download(c, pos.shape[0])

    def _repack(self, new: list[Request], now: float):
        with torch.cuda.stream(self.stream):
            old = self._download(self.ctx, self.n) if self.resident and self.n else None
            fresh = self._initial_forces(new) if new else None
            pieces = {f: [] for f in _CARRY}
            off = 0
            keep = []
            for r in self.resident:
                if r.left > 0:
                    for f in _CARRY:
                        pieces[f].append(old[f][off:off + r.req.n])
                    keep.append(r)
                off += r.req.n
            off = 0
            for q in new:
                for f in _CARRY:
                    pieces[f].append(fresh[f][off:off + q.n])
                res = _Resident(q, torch.from_numpy(np.ascontiguousarray(q.mass, np.float64)).cuda(),
                                torch.from_numpy(np.ascontiguousarray(q.type, np.uint8)).cuda(), now)
                keep.append(res)
                off += q.n
            self.resident = keep
            self.n = sum(r.req.n for r in keep)
            if not keep:
                return
            arr = {f: torch.cat(pieces[f]).contiguous() for f in _CARRY}
            mass = torch.cat([r.mass for r in keep]).contiguous()
            type_ = torch.cat([r.type for r in keep]).contiguous()
            c = self.ctx
            c.upload_device(self.n, arr["pos"].data_ptr(), mass.data_ptr(), type_.data_ptr(), arr["vel"].data_ptr(),
                            arr["U"].data_ptr())
            c.set_field_device("acc", arr["acc"].data_ptr())
            c.set_field_device("dUdt", arr["dUdt"].data_ptr())
            c.set_instances(np.concatenate([[0], np.cumsum([r.req.n for r in keep])]),
                            np.array([r.req.massInH for r in keep]))
            self._hold = (arr, mass, type_)  # alive until the next repack
            self.stream.synchronize()

    # -- one step boundary ---------------------------------------------------------
    def step(self) -> list[Result]:
        """Admit, advance every resident simulation by one step, return finished ones."""
        now = self.clock()
        new = []
        budget = self.capacity - sum(r.req.n for r in self.resident if r.left > 0)
        while self.waiting and self.waiting[0].n <= budget:
            q = self.waiting.popleft()
            budget -= q.n
            new.append(q)
        if new or self.layout_dirty:
            self._repack(new, now)
            self.layout_dirty = False
        if not self.resident:
            return []
        self.ctx.step(self.dt)  # ends with a check of the walk's status (a synchronisation)
        self.steps_done += 1
        self.particle_steps += self.n
        done = []
        fin = [r for r in self.resident if r.left == 1]
        if fin:
            with torch.cuda.stream(self.stream):
                state = self._download(self.ctx, self.n)
                off = 0
                for r in self.resident:
                    if r.left == 1:
                        host = {f: state[f][off:off + r.req.n].cpu().numpy() for f in _CARRY}
                        done.append(Result(r.req.rid, host, r.req.arrival, r.admitted, self.clock(), r.req.steps))
                    off += r.req.n
        t = self.clock()
        for r in self.resident:
            r.left -= 1
        for d in done:
            d.completed = t
        if fin:
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
