"""Python binding of the C-ABI in include/ag2.h (ctypes over lib/libag2.so).

This is the host-side view the tests and bench.py use.  It mirrors the
reference's call sequence: ``Context.build_tree`` is ``Tree::buildTree``
(simulation/src/Physics/Tree/Tree.cpp:24-55), ``sph_density`` is
``Tree::calcGasDensity`` (:119-150), ``forces`` is ``Tree::calculateForces``
(:57-83), ``kick``/``drift``/``ueuler`` are ``TimeIntegration::Kick/Drift/Ueuler``
(simulation/src/Physics/TimeIntegration.cpp:10-40).  There is no CPU fallback:
without the compiled library (or a GPU) every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libag2.so")

OK = 0
E_INVALID, E_CUDA, E_NOMEM, E_COINCIDENT, E_DEPTH, E_STACK, E_NAN, E_CAPACITY = range(-1, -9, -1)
PREC_FP64, PREC_FP32 = 0, 1
FIELDS = {"pos": 0, "vel": 1, "acc": 2, "mass": 3, "h": 4, "rho": 5, "P": 6, "T": 7, "U": 8, "dUdt": 9,
          "vdens": 10, "tstep": 11, "tnext": 12}
VECTOR_FIELDS = {"pos", "vel", "acc"}

# every exported symbol of include/ag2.h
EXPORTS = [
    "ag2_default_params", "ag2_create", "ag2_destroy", "ag2_set_params", "ag2_get_params", "ag2_set_stream",
    "ag2_last_error_string", "ag2_upload", "ag2_upload_device", "ag2_set_field", "ag2_download",
    "ag2_download_fields", "ag2_step_host", "ag2_count",
    "ag2_build_tree", "ag2_visual_density", "ag2_sph_density", "ag2_forces", "ag2_kick", "ag2_drift",
    "ag2_kick_drift", "ag2_ueuler", "ag2_scale_positions", "ag2_step", "ag2_root_radius", "ag2_node_count",
    "ag2_topology", "ag2_walk_records", "ag2_particle_node", "ag2_interactions", "ag2_launch_count", "ag2_direct_sum",
    "ag2_diagnostics", "ag2_fp32_peak_probe", "ag2_autotune", "ag2_root_radius_noalloc", "ag2_phase_timing",
    "ag2_phase_times", "ag2_set_instances", "ag2_instance_radius", "ag2_energy", "ag2_step_graphs",
    "ag2_block_init", "ag2_block_step", "ag2_set_tags", "ag2_get_tags", "ag2_snapshot_size",
    "ag2_snapshot_encode", "ag2_snapshot_write", "ag2_snapshot_wait", "ag2_ic_count", "ag2_load_ics",
    "ag2_inject_fault", "ag2_autotune_walk", "ag2_set_walk_variant",
]

# file formats of ag2_snapshot_* / ag2_load_ics (the reference's format names)
FORMATS = {"ag": 0, "agc": 1, "age": 2, "gadget": 3, "makeGal": 4}


class Params(ctypes.Structure):
    _fields_ = [("G", ctypes.c_double), ("e0", ctypes.c_double), ("theta", ctypes.c_double),
                ("massInH", ctypes.c_double), ("split_threshold", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("group_size", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class WalkConfig(ctypes.Structure):
    """ag2_walk_config (include/ag2.h)."""
    _fields_ = [("variant", ctypes.c_int32), ("regs", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32),
                ("stack", ctypes.c_int32), ("prefetch", ctypes.c_int32), ("group_size", ctypes.c_int32),
                ("ms", ctypes.c_float)]


class AG2Error(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ag2 error {code}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libag2.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run __graft_entry__.build() first")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    D = ctypes.c_double
    I = ctypes.c_int
    dp = ctypes.POINTER(ctypes.c_double)
    L.ag2_default_params.argtypes = [ctypes.POINTER(Params)]
    L.ag2_default_params.restype = None
    L.ag2_create.argtypes = [ctypes.POINTER(P), ctypes.POINTER(Params), ctypes.c_size_t]
    L.ag2_destroy.argtypes = [P]
    L.ag2_set_params.argtypes = [P, ctypes.POINTER(Params)]
    L.ag2_get_params.argtypes = [P, ctypes.POINTER(Params)]
    L.ag2_set_stream.argtypes = [P, P]
    L.ag2_last_error_string.argtypes = [P]
    L.ag2_last_error_string.restype = ctypes.c_char_p
    L.ag2_upload.argtypes = [P, ctypes.c_size_t, P, P, P, P, P]
    L.ag2_upload_device.argtypes = [P, ctypes.c_size_t, P, P, P, P, P]
    L.ag2_set_field.argtypes = [P, I, P, I]
    L.ag2_download.argtypes = [P, I, P, I]
    L.ag2_download_fields.argtypes = [P, I, P, P]
    L.ag2_count.argtypes = [P]
    L.ag2_count.restype = ctypes.c_size_t
    for f in ("ag2_build_tree", "ag2_sph_density", "ag2_forces"):
        getattr(L, f).argtypes = [P]
    for f in ("ag2_visual_density", "ag2_kick", "ag2_drift", "ag2_kick_drift", "ag2_ueuler",
              "ag2_scale_positions"):
        getattr(L, f).argtypes = [P, D]
    L.ag2_step.argtypes = [P, D, D, I, D]
    L.ag2_step_host.argtypes = [P, ctypes.c_size_t, D, D, I, D, P]
    L.ag2_root_radius.argtypes = [P, dp]
    L.ag2_node_count.argtypes = [P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                 ctypes.POINTER(ctypes.c_int32)]
    L.ag2_topology.argtypes = [P] * 12
    L.ag2_particle_node.argtypes = [P, P]
    L.ag2_walk_records.argtypes = [P, P]
    L.ag2_interactions.argtypes = [P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    L.ag2_direct_sum.argtypes = [P, ctypes.c_size_t, P, P]
    L.ag2_diagnostics.argtypes = [P, P]
    L.ag2_energy.argtypes = [P, P]
    L.ag2_step_graphs.argtypes = [P, I]
    L.ag2_block_init.argtypes = [P, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double]
    L.ag2_block_step.argtypes = [P, ctypes.c_double, I, ctypes.c_double, dp, ctypes.POINTER(ctypes.c_int64)]
    L.ag2_fp32_peak_probe.argtypes = [P, dp]
    L.ag2_autotune.argtypes = [P, ctypes.POINTER(ctypes.c_int)]
    L.ag2_root_radius_noalloc.argtypes = [P, ctypes.c_int64, P, P]
    L.ag2_phase_timing.argtypes = [P, I]
    L.ag2_set_instances.argtypes = [P, ctypes.c_int32, P, P]
    L.ag2_instance_radius.argtypes = [P, ctypes.c_int32, dp]
    L.ag2_phase_times.argtypes = [P, I, P, P]
    L.ag2_launch_count.argtypes = [P]
    L.ag2_launch_count.restype = ctypes.c_int64
    L.ag2_set_tags.argtypes = [P, P, P, P, I]
    L.ag2_get_tags.argtypes = [P, P, P, P, I]
    L.ag2_snapshot_size.argtypes = [P, I, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]
    L.ag2_snapshot_encode.argtypes = [P, I, ctypes.c_int64, D, D, D, P, ctypes.c_size_t,
                                      ctypes.POINTER(ctypes.c_size_t)]
    L.ag2_snapshot_write.argtypes = [P, I, ctypes.c_int64, D, D, D, ctypes.c_char_p, I]
    L.ag2_snapshot_wait.argtypes = [P]
    L.ag2_ic_count.argtypes = [ctypes.c_char_p, I, ctypes.POINTER(ctypes.c_int64)]
    L.ag2_load_ics.argtypes = [P, ctypes.c_char_p, I, P]
    L.ag2_inject_fault.argtypes = [P, I, I]
    L.ag2_autotune_walk.argtypes = [P, I, P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.ag2_set_walk_variant.argtypes = [P, I]
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class _HostIO(ctypes.Structure):
    """ag2_host_io (include/ag2.h)."""
    _fields_ = [(k, ctypes.c_void_p) for k in
                ("pos", "vel", "mass", "U", "acc", "type", "pos_out", "vel_out", "acc_out", "U_out")] + \
               [("n_inst", ctypes.c_int32), ("first", ctypes.c_void_p), ("massInH", ctypes.c_void_p)]


class Context:
    """One simulation's device state (particles in HBM, tree, walk arrays)."""

    def __init__(self, capacity: int, *, G: float = 1.0, e0: float = 0.01, theta: float = 0.5,
                 massInH: float = 0.0, split_threshold: int = 100, precision: str = "fp32"):
        self.L = load()
        p = Params()
        self.L.ag2_default_params(ctypes.byref(p))
        p.G, p.e0, p.theta, p.massInH = G, e0, theta, massInH
        p.split_threshold = split_threshold
        p.precision = PREC_FP32 if precision == "fp32" else PREC_FP64
        self.params = p
        h = ctypes.c_void_p()
        rc = self.L.ag2_create(ctypes.byref(h), ctypes.byref(p), int(capacity))
        if rc != OK:
            raise AG2Error(rc, "ag2_create failed")
        self.h = h
        self.n = 0

    # -- helpers ------------------------------------------------------------
    def _check(self, rc: int):
        if rc != OK:
            msg = self.L.ag2_last_error_string(self.h)
            raise AG2Error(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.ag2_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, **kw):
        for k, v in kw.items():
            if k == "precision":
                v = PREC_FP32 if v == "fp32" else PREC_FP64
            setattr(self.params, k, v)
        self._check(self.L.ag2_set_params(self.h, ctypes.byref(self.params)))

    def set_stream(self, stream_handle: int | None):
        self._check(self.L.ag2_set_stream(self.h, ctypes.c_void_p(stream_handle or 0)))

    # -- particles ----------------------------------------------------------
    def upload(self, pos, mass, type_, vel=None, U=None):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        n = pos.shape[0]
        mass = np.ascontiguousarray(mass, dtype=np.float64).reshape(n)
        type_ = np.ascontiguousarray(type_, dtype=np.uint8).reshape(n)
        vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(n, 3)
        U = None if U is None else np.ascontiguousarray(U, dtype=np.float64).reshape(n)
        self._keep = (pos, mass, type_, vel, U)
        self._check(self.L.ag2_upload(self.h, n, _ptr(pos), _ptr(vel), _ptr(mass), _ptr(U), _ptr(type_)))
        self.n = n

    def upload_device(self, n: int, pos_ptr: int, mass_ptr: int, type_ptr: int, vel_ptr: int = 0, U_ptr: int = 0):
        """Upload from device buffers (e.g. torch tensor data_ptr()s)."""
        v = ctypes.c_void_p
        self._check(self.L.ag2_upload_device(self.h, n, v(pos_ptr), v(vel_ptr or None), v(mass_ptr),
                                             v(U_ptr or None), v(type_ptr)))
        self.n = n

    def download(self, field: str, out: np.ndarray | None = None) -> np.ndarray:
        f = FIELDS[field]
        shape = (self.n, 3) if field in VECTOR_FIELDS else (self.n,)
        if out is None:
            out = np.empty(shape, dtype=np.float64)
        elif out.shape != shape or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array of shape %s" % (shape,))
        self._check(self.L.ag2_download(self.h, f, _ptr(out), 0))
        return out

    def download_fields(self, outs: dict) -> dict:
        """Several fields into preallocated host arrays in one call ({field: out})."""
        names = list(outs)
        for f in names:
            shape = (self.n, 3) if f in VECTOR_FIELDS else (self.n,)
            o = outs[f]
            if o.shape != shape or o.dtype != np.float64 or not o.flags.c_contiguous:
                raise ValueError("out must be a C-contiguous float64 array of shape %s" % (shape,))
        codes = (ctypes.c_int * len(names))(*[FIELDS[f] for f in names])
        ptrs = (ctypes.c_void_p * len(names))(*[outs[f].ctypes.data for f in names])
        self._check(self.L.ag2_download_fields(self.h, len(names), codes, ptrs))
        return outs

    def download_device(self, field: str, dst_ptr: int):
        self._check(self.L.ag2_download(self.h, FIELDS[field], ctypes.c_void_p(dst_ptr), 1))

    def set_field(self, field: str, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        self._check(self.L.ag2_set_field(self.h, FIELDS[field], _ptr(a), 0))

    def set_field_device(self, field: str, src_ptr: int):
        """Overwrite one field from a device buffer in the original particle order."""
        self._check(self.L.ag2_set_field(self.h, FIELDS[field], ctypes.c_void_p(src_ptr), 1))

    # -- hot path -----------------------------------------------------------
    def build_tree(self):
        self._check(self.L.ag2_build_tree(self.h))

    def visual_density(self, radius: float):
        self._check(self.L.ag2_visual_density(self.h, radius))

    def sph_density(self):
        self._check(self.L.ag2_sph_density(self.h))

    def forces(self):
        self._check(self.L.ag2_forces(self.h))

    def kick(self, dt):
        self._check(self.L.ag2_kick(self.h, dt))

    def drift(self, dt):
        self._check(self.L.ag2_drift(self.h, dt))

    def kick_drift(self, dt):
        self._check(self.L.ag2_kick_drift(self.h, dt))

    def ueuler(self, dt):
        self._check(self.L.ag2_ueuler(self.h, dt))

    def scale_positions(self, f):
        self._check(self.L.ag2_scale_positions(self.h, f))

    def step(self, dt, hubble_factor=1.0, visual_density=False, visual_radius=0.0):
        self._check(self.L.ag2_step(self.h, dt, hubble_factor, 1 if visual_density else 0, visual_radius))

    def step_host(self, dt, pos, mass, type_, vel=None, U=None, acc=None, out=None, hubble_factor=1.0,
                  visual_density=False, visual_radius=0.0, first=None, massInH=None):
        """One step with host arrays in and out (ag2_step_host): upload, step,
        and pos/vel/acc/U read back into out = {field: array} (arrays may be the
        inputs).  Inputs must be C-contiguous float64 (uint8 type).  `first`
        (and `massInH`) split the particles into simulations, as
        set_instances."""
        n = len(mass)
        arrs = {"pos": pos, "vel": vel, "mass": mass, "U": U, "acc": acc}
        def bad(k, a):
            size = n * (3 if k in VECTOR_FIELDS else 1)
            return a.dtype != np.float64 or not a.flags.c_contiguous or a.size != size

        for k, a in arrs.items():
            if a is not None and bad(k, a):
                raise ValueError(k + " must be a C-contiguous float64 array of n" + (" x 3" if k in VECTOR_FIELDS else ""))
        if type_.dtype != np.uint8 or not type_.flags.c_contiguous or type_.size != n:
            raise ValueError("type must be a C-contiguous uint8 array of n")
        out = out or {}
        for k, a in out.items():
            if k not in ("pos", "vel", "acc", "U") or bad(k, a):
                raise ValueError("bad output array for " + k)
        ptr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
        io = _HostIO(ptr(pos), ptr(vel), ptr(mass), ptr(U), ptr(acc), ptr(type_), ptr(out.get("pos")),
                     ptr(out.get("vel")), ptr(out.get("acc")), ptr(out.get("U")))
        if first is not None:
            first = np.ascontiguousarray(first, np.int64)
            io.n_inst, io.first = len(first) - 1, first.ctypes.data
            if massInH is not None:
                massInH = np.ascontiguousarray(massInH, np.float64)
                io.massInH = massInH.ctypes.data
        self._check(self.L.ag2_step_host(self.h, n, dt, hubble_factor, 1 if visual_density else 0, visual_radius,
                                         ctypes.byref(io)))
        self.n = n
        return out

    def inject_fault(self, site: int, code: int):
        """ag2_inject_fault: site 1 makes the next step_host fail with `code`
        right after the walk (host side only; for tests of the error path)."""
        self._check(self.L.ag2_inject_fault(self.h, site, code))

    # -- introspection --------------------------------------------------------
    def root_radius(self) -> float:
        r = ctypes.c_double()
        self._check(self.L.ag2_root_radius(self.h, ctypes.byref(r)))
        return r.value

    def node_count(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
        self._check(self.L.ag2_node_count(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def particle_node(self) -> np.ndarray:
        out = np.empty(self.n, np.int64)
        self._check(self.L.ag2_particle_node(self.h, _ptr(out)))
        return out

    def interactions(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._check(self.L.ag2_interactions(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def direct_sum(self, ids) -> np.ndarray:
        ids = np.ascontiguousarray(ids, np.int64)
        out = np.empty((ids.size, 3))
        self._check(self.L.ag2_direct_sum(self.h, ids.size, _ptr(ids), _ptr(out)))
        return out

    def diagnostics(self) -> dict:
        out = np.empty(8)
        self._check(self.L.ag2_diagnostics(self.h, _ptr(out)))
        return {"mass": out[0], "ekin": out[1], "momentum": out[2:5], "angmom": out[5:8]}

    def block_init(self, eta: float, min_dt: float, max_dt: float, global_time: float = 0.0):
        """Per-particle power-of-two time steps from the current acc."""
        self._check(self.L.ag2_block_init(self.h, eta, min_dt, max_dt, global_time))

    def block_step(self, H0: float = 0.0, visual_density: bool = False, visual_radius: float = 0.0):
        """One block step; returns (global time, number of particles integrated)."""
        t, k = ctypes.c_double(), ctypes.c_int64()
        self._check(self.L.ag2_block_step(self.h, H0, 1 if visual_density else 0, visual_radius, ctypes.byref(t),
                                          ctypes.byref(k)))
        return t.value, k.value

    def step_graphs(self, enable: bool = True):
        """Run later steps as replays of a captured CUDA graph."""
        self._check(self.L.ag2_step_graphs(self.h, 1 if enable else 0))

    def energy(self) -> dict:
        """Kinetic, potential, thermal and total energy of the current state
        (needs a tree built from the current positions)."""
        out = np.empty(4)
        self._check(self.L.ag2_energy(self.h, _ptr(out)))
        return {"kinetic": out[0], "potential": out[1], "thermal": out[2], "total": out[3]}

    def fp32_peak_gflops(self) -> float:
        g = ctypes.c_double()
        self._check(self.L.ag2_fp32_peak_probe(self.h, ctypes.byref(g)))
        return g.value

    def set_instances(self, first, massInH=None):
        """Split the uploaded particles into independent simulations:
        instance k = upload indices [first[k], first[k+1])."""
        first = np.ascontiguousarray(first, np.int64)
        mih = None if massInH is None else np.ascontiguousarray(massInH, np.float64)
        self._keep_inst = (first, mih)
        self._check(self.L.ag2_set_instances(self.h, first.size - 1, _ptr(first), _ptr(mih)))

    def instance_radius(self, k: int) -> float:
        r = ctypes.c_double()
        self._check(self.L.ag2_instance_radius(self.h, k, ctypes.byref(r)))
        return r.value

    def phase_timing(self, enable: bool = True):
        self._check(self.L.ag2_phase_timing(self.h, 1 if enable else 0))

    def phase_times(self) -> list:
        names = (ctypes.c_char_p * 16)()
        ms = (ctypes.c_float * 16)()
        k = self.L.ag2_phase_times(self.h, 16, names, ms)
        return [(names[i].decode(), ms[i]) for i in range(min(k, 16))]

    def autotune(self) -> int:
        v = ctypes.c_int()
        self._check(self.L.ag2_autotune(self.h, ctypes.byref(v)))
        self.params.group_size = self._get_params().group_size
        return v.value

    def autotune_walk(self) -> dict:
        """ag2_autotune_walk: every candidate (variant, register budget, blocks
        per SM, first-pass stack, group size) with its walk time on the current
        tree, and the one kept."""
        out = (WalkConfig * 16)()
        cnt, chosen = ctypes.c_int(), ctypes.c_int()
        self._check(self.L.ag2_autotune_walk(self.h, 16, out, ctypes.byref(cnt), ctypes.byref(chosen)))
        self.params.group_size = self._get_params().group_size
        cands = [{"variant": c.variant, "regs": c.regs, "blocks_per_sm": c.blocks_per_sm, "stack": c.stack,
                  "prefetch": c.prefetch, "group_size": c.group_size, "ms": c.ms} for c in out[:min(cnt.value, 16)]]
        return {"candidates": cands, "chosen": cands[chosen.value] if 0 <= chosen.value < len(cands) else None}

    def set_walk_variant(self, variant: int):
        self._check(self.L.ag2_set_walk_variant(self.h, variant))

    def _get_params(self) -> "Params":
        p = Params()
        self._check(self.L.ag2_get_params(self.h, ctypes.byref(p)))
        return p

    def launches(self) -> int:
        return int(self.L.ag2_launch_count(self.h))

    # -- snapshot and initial-condition files (DataManager) --------------------
    def set_tags(self, id=None, galaxy_part=None, sfr=None):
        """Particle::id, galaxyPart and sfr in upload order (None: unchanged)."""
        a = None if id is None else np.ascontiguousarray(id, np.uint32)
        b = None if galaxy_part is None else np.ascontiguousarray(galaxy_part, np.uint8)
        c = None if sfr is None else np.ascontiguousarray(sfr, np.float64)
        for x in (a, b, c):
            if x is not None and x.size != self.n:
                raise ValueError("tags need one value per particle")
        self._check(self.L.ag2_set_tags(self.h, _ptr(a), _ptr(b), _ptr(c), 0))

    def tags(self) -> dict:
        out = {"id": np.empty(self.n, np.uint32), "gp": np.empty(self.n, np.uint8), "sfr": np.empty(self.n)}
        self._check(self.L.ag2_get_tags(self.h, _ptr(out["id"]), _ptr(out["gp"]), _ptr(out["sfr"]), 0))
        return out

    def snapshot_size(self, fmt: str, count: int | None = None) -> int:
        """Bytes of the snapshot image (an upper bound for gadget)."""
        cap = ctypes.c_size_t()
        self._check(self.L.ag2_snapshot_size(self.h, FORMATS[fmt], self.n if count is None else count,
                                             ctypes.byref(cap)))
        return cap.value

    def snapshot_bytes(self, fmt: str, count: int | None = None, delta_time: float = 0.0, end_time: float = 0.0,
                       current_time: float = 0.0, out: np.ndarray | None = None):
        """DataManager::saveData's file image of the first `count` particles:
        bytes, or its length when encoded into `out` (a uint8 array, e.g.
        pinned memory)."""
        count = self.n if count is None else count
        buf = np.empty(max(self.snapshot_size(fmt, count), 1), np.uint8) if out is None else out
        ln = ctypes.c_size_t()
        self._check(self.L.ag2_snapshot_encode(self.h, FORMATS[fmt], count, delta_time, end_time, current_time,
                                               _ptr(buf), buf.nbytes, ctypes.byref(ln)))
        return buf[: ln.value].tobytes() if out is None else ln.value

    def snapshot_write(self, path: str, fmt: str, count: int | None = None, delta_time: float = 0.0,
                       end_time: float = 0.0, current_time: float = 0.0, wait: bool = True):
        """Write the snapshot file; with wait=False the file is written in the
        background (snapshot_wait collects the status)."""
        count = self.n if count is None else count
        self._check(self.L.ag2_snapshot_write(self.h, FORMATS[fmt], count, delta_time, end_time, current_time,
                                              str(path).encode(), 0 if wait else 1))

    def snapshot_wait(self):
        self._check(self.L.ag2_snapshot_wait(self.h))

    def load_ics(self, path: str, fmt: str):
        """DataManager::loadICs into the context; returns the header's
        (deltaTime, endTime, currentTime) or (0, 0, time)."""
        t = np.zeros(3)
        self._check(self.L.ag2_load_ics(self.h, str(path).encode(), FORMATS[fmt], _ptr(t)))
        self.n = int(self.L.ag2_count(self.h))
        return tuple(t)


    def topology(self) -> dict:
        nn, _, _ = self.node_count()
        t = {
            "depth": np.empty(nn, np.int32), "is_leaf": np.empty(nn, np.int32), "particle": np.empty(nn, np.int32),
            "cp_count": np.empty(nn, np.int64), "cp_hash": np.empty(nn, np.uint64), "mass": np.empty(nn),
            "com": np.empty((nn, 3)), "gas_mass": np.empty(nn), "mvel": np.empty((nn, 3)),
            "center": np.empty((nn, 3)), "radius": np.empty(nn),
        }
        order = ["depth", "is_leaf", "particle", "cp_count", "cp_hash", "mass", "com", "gas_mass", "mvel", "center",
                 "radius"]
        self._check(self.L.ag2_topology(self.h, *[_ptr(t[k]) for k in order]))
        return t

    def walk_records(self) -> np.ndarray:
        """The FP32 walk's node records, (nodes, 16) float32 in topology() order."""
        nn, _, _ = self.node_count()
        out = np.empty((nn, 16), np.float32)
        self._check(self.L.ag2_walk_records(self.h, _ptr(out)))
        return out


def ic_count(path: str, fmt: str) -> int:
    """Particle count in an initial-condition file's header."""
    L = load()
    n = ctypes.c_int64()
    rc = L.ag2_ic_count(str(path).encode(), FORMATS[fmt], ctypes.byref(n))
    if rc != OK:
        raise AG2Error(rc, "cannot read the header of " + str(path))
    return n.value
