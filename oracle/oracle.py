"""ctypes view of the CPU checkers (TEST INFRASTRUCTURE ONLY).

``World(kind="port")`` loads oracle/liboracle.so, the plain-C restatement of
the reference's hot path (ag2_oracle.c); ``World(kind="reference")`` loads
oracle/_ref/libag2ref.so, the reference's own sources behind the same
interface (built only where the reference checkout exists).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU legs use this module, as the checker
and as the timed CPU baseline; the product never does.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libag2ref.so")

FIELDS = {"pos": 0, "vel": 1, "acc": 2, "mass": 3, "h": 4, "rho": 5, "P": 6, "T": 7, "U": 8, "dUdt": 9,
          "vdens": 10}
VECTOR_FIELDS = {"pos", "vel", "acc"}

_libs: dict[str, ctypes.CDLL] = {}
_ref_root: list = []


def reference_checkout():
    """Root of the reference checkout (the directory holding simulation/ and
    input_data/), or None where there is none.  The location is the AG2_REF
    environment variable when set, else the one oracle/Makefile names."""
    if not _ref_root:
        root = os.environ.get("AG2_REF")
        if not root:
            import subprocess

            try:
                r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True, timeout=30)
                root = r.stdout.strip() if r.returncode == 0 else None
            except (OSError, subprocess.SubprocessError):
                root = None
        _ref_root.append(root if root and os.path.isdir(os.path.join(root, "simulation", "src")) else None)
    return _ref_root[0]


def available(kind: str) -> bool:
    return os.path.exists(PORT_LIB if kind == "port" else REF_LIB)


def load(kind: str = "port") -> ctypes.CDLL:
    if kind in _libs:
        return _libs[kind]
    path = PORT_LIB if kind == "port" else REF_LIB
    if not os.path.exists(path):
        raise RuntimeError(f"{path} missing (build it with make -C oracle)")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    D = ctypes.c_double
    I = ctypes.c_int
    L.orc_create.argtypes = [I, P, P, P, P, P]
    L.orc_create.restype = P
    L.orc_destroy.argtypes = [P]
    L.orc_get_G.restype = D
    L.orc_set_G.argtypes = [D]
    L.orc_build.argtypes = [P, I]
    L.orc_visual_density.argtypes = [P, D]
    L.orc_gas_density.argtypes = [P, D]
    L.orc_forces.argtypes = [P, D, D, I]
    L.orc_forces_subset.argtypes = [P, D, D, I, I, P]
    for f in ("orc_kick", "orc_drift", "orc_ueuler", "orc_scale_positions"):
        getattr(L, f).argtypes = [P, D]
        getattr(L, f).restype = None
    L.orc_get.argtypes = [P, I, P]
    L.orc_get.restype = None
    L.orc_set.argtypes = [P, I, P]
    L.orc_set.restype = None
    L.orc_root_radius.argtypes = [P]
    L.orc_root_radius.restype = D
    L.orc_node_count.argtypes = [P]
    L.orc_node_count.restype = ctypes.c_int64
    L.orc_topology.argtypes = [P] * 12
    L.orc_topology.restype = None
    L.orc_leaf_index.argtypes = [P, P]
    L.orc_leaf_index.restype = None
    L.orc_id_hash.argtypes = [ctypes.c_uint64]
    L.orc_id_hash.restype = ctypes.c_uint64
    L.orc_direct_sum.argtypes = [I, P, P, D, D, I, P, P, I]
    L.orc_direct_sum.restype = None
    _libs[kind] = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class World:
    def __init__(self, pos, mass, type_, vel=None, U=None, kind: str = "port", G: float = 1.0):
        self.L = load(kind)
        self.kind = kind
        if kind == "port":
            self.L.orc_set_G(G)
        elif abs(self.L.orc_get_G() - G) > 0:
            raise ValueError("the reference harness is built for G = 1")
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        self.n = pos.shape[0]
        mass = np.ascontiguousarray(mass, np.float64).reshape(self.n)
        type_ = np.ascontiguousarray(type_, np.uint8).reshape(self.n)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float64).reshape(self.n, 3)
        U = None if U is None else np.ascontiguousarray(U, np.float64).reshape(self.n)
        self.h = self.L.orc_create(self.n, _p(pos), _p(vel), _p(mass), _p(U), _p(type_))

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build(self, threads: int = 1):
        self.L.orc_build(self.h, threads)

    def visual_density(self, R: float):
        self.L.orc_visual_density(self.h, R)

    def gas_density(self, massInH: float):
        self.L.orc_gas_density(self.h, massInH)

    def forces(self, e0: float, theta: float, threads: int = 1):
        self.L.orc_forces(self.h, e0, theta, threads)

    def forces_subset(self, e0: float, theta: float, idx, threads: int = 1):
        idx = np.ascontiguousarray(idx, np.int32)
        self.L.orc_forces_subset(self.h, e0, theta, threads, idx.size, _p(idx))

    def kick(self, dt):
        self.L.orc_kick(self.h, dt)

    def drift(self, dt):
        self.L.orc_drift(self.h, dt)

    def ueuler(self, dt):
        self.L.orc_ueuler(self.h, dt)

    def scale_positions(self, f):
        self.L.orc_scale_positions(self.h, f)

    def get(self, field: str) -> np.ndarray:
        shape = (self.n, 3) if field in VECTOR_FIELDS else (self.n,)
        out = np.empty(shape, np.float64)
        self.L.orc_get(self.h, FIELDS[field], _p(out))
        return out

    def set(self, field: str, values):
        a = np.ascontiguousarray(values, np.float64)
        self.L.orc_set(self.h, FIELDS[field], _p(a))

    def root_radius(self) -> float:
        return self.L.orc_root_radius(self.h)

    def node_count(self) -> int:
        return int(self.L.orc_node_count(self.h))

    def topology(self) -> dict:
        nn = self.node_count()
        t = {
            "depth": np.empty(nn, np.int32), "is_leaf": np.empty(nn, np.int32), "particle": np.empty(nn, np.int32),
            "cp_count": np.empty(nn, np.int64), "cp_hash": np.empty(nn, np.uint64), "mass": np.empty(nn),
            "com": np.empty((nn, 3)), "gas_mass": np.empty(nn), "mvel": np.empty((nn, 3)),
            "center": np.empty((nn, 3)), "radius": np.empty(nn),
        }
        order = ["depth", "is_leaf", "particle", "cp_count", "cp_hash", "mass", "com", "gas_mass", "mvel", "center",
                 "radius"]
        self.L.orc_topology(self.h, *[_p(t[k]) for k in order])
        return t

    def leaf_index(self) -> np.ndarray:
        out = np.empty(self.n, np.int64)
        self.L.orc_leaf_index(self.h, _p(out))
        return out


def direct_sum(pos, mass, e0: float, sample, G: float = 1.0, threads: int = 1, kind: str = "port") -> np.ndarray:
    """FP64 direct summation with the reference's softened pair law."""
    L = load(kind)
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
    mass = np.ascontiguousarray(mass, np.float64)
    sample = np.ascontiguousarray(sample, np.int32)
    out = np.empty((sample.size, 3), np.float64)
    L.orc_direct_sum(pos.shape[0], _p(pos), _p(mass), e0, G, sample.size, _p(sample), _p(out), threads)
    return out


def id_hash(ids) -> np.ndarray:
    """orc_id_hash (splitmix64 of id+1) vectorised."""
    z = np.asarray(ids, dtype=np.uint64) + np.uint64(1) + np.uint64(0x9E3779B97F4A7C15)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


# ---- block time steps (Simulation.cpp:188-341), restated over the port -------


def block_dt(acc, eta: float, e0: float, dmin: float, dmax: float) -> np.ndarray:
    """Per-particle step (Simulation.cpp:196-206): eta*sqrt(e0/|a|) clamped to
    [dmin, dmax], floored to a power of two, not below dmin; dmin for a = 0."""
    acc = np.asarray(acc, np.float64)
    a = np.sqrt(acc[:, 0] * acc[:, 0] + acc[:, 1] * acc[:, 1] + acc[:, 2] * acc[:, 2])  # vec3::length
    ts = np.full(a.shape, dmin)
    pos = a > 0
    t = eta * np.sqrt(e0 / a[pos])
    t = np.where(t < dmin, dmin, np.where(dmax < t, dmax, t))  # std::clamp
    t = np.maximum(2.0 ** np.floor(np.log2(t)), dmin)  # std::max(std::pow(2, std::floor(std::log2(t))), min)
    ts[pos] = t
    return ts


def _kick(vel, acc, ts, idx):
    """TimeIntegration::Kick for the particles idx (skipped where acc has a NaN)."""
    ok = idx[~np.isnan(acc[idx]).any(axis=1)]
    vel[ok] = vel[ok] + acc[ok] * ts[ok, None] / 2
    return vel


def block_steps(world: World, type_, eta: float, dmin: float, dmax: float, e0: float, theta: float,
                massInH: float, steps: int, t: float = 0.0, H0: float = 0.0, threads: int = 1,
                end_time: float | None = None):
    """`steps` iterations of the reference's block-time-step loop
    (Simulation.cpp:188-341) on the port, starting from the world's current acc
    (after its initial forces); with `end_time`, iterations while the global
    time is below it, as Simulation::run's `while (globalTime < endTime)`
    (Simulation.cpp:210).  Returns [(global time, particles integrated)] and
    the final (step, next time) arrays."""
    type_ = np.asarray(type_)
    ts = block_dt(world.get("acc"), eta, e0, dmin, dmax)
    tn = t + ts
    log = []
    k = 0
    while (t < end_time) if end_time is not None else (k < steps):
        k += 1
        due = t >= tn
        if due.any():
            ts[due] = block_dt(world.get("acc")[due], eta, e0, dmin, dmax)
            tn[due] = t + ts[due]
        t = float(tn.min())
        act = np.nonzero(tn == t)[0].astype(np.int32)
        acc, vel, pos = world.get("acc"), world.get("vel"), world.get("pos")
        vel = _kick(vel, acc, ts, act)
        pos[act] = pos[act] + vel[act] * ts[act, None]
        world.set("vel", vel)
        world.set("pos", pos)
        world.build(threads)
        if (type_ == 2).any():
            world.gas_density(massInH)
        world.forces_subset(e0, theta, act, threads)
        acc, vel, pos = world.get("acc"), world.get("vel"), world.get("pos")
        U, du = world.get("U"), world.get("dUdt")
        g = act[type_[act] == 2]
        gok = g[~np.isnan(du[g])]
        U[gok] = U[gok] + du[gok] * ts[gok]
        du[g] = 0.0
        pos[act] = pos[act] * np.exp(H0 * ts[act])[:, None]
        vel = _kick(vel, acc, ts, act)
        tn[act] = tn[act] + ts[act]
        world.set("U", U)
        world.set("dUdt", du)
        world.set("pos", pos)
        world.set("vel", vel)
        log.append((t, int(act.size)))
    return log, ts, tn
