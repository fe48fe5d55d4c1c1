"""TEST INFRASTRUCTURE ONLY: a numpy restatement of the reference's snapshot
writer and initial-condition reader (DataManager::saveData,
File/DataManager.cpp:86-424, and DataManager::loadICs, :434-1332).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it, as
the checker of the library's device encoder and decoder.  Pinned against the
reference itself by tests/test_oracle_snapio.py: the reference's own saveData
and loadICs are compiled into oracle/_ref/libag2ref.so (ref_harness.cpp) and
run on the same particles and files, and tests/golden/ic_examples.json holds
the reference loader's output for the four example initial conditions shipped
with the reference.

Particles are dicts of arrays in the reference's particle-vector order:
pos (n,3), vel (n,3), mass, T, P, vdens (visualDensity), U, sfr (float64),
type, gp (galaxyPart) (uint8), id (uint32).

Departures, all in cases where the reference's result is undefined or
silent: the 4 padding bytes of the ag header are written as zero (the
reference leaves them uninitialised); files whose particle data the
reference would read past the end (it then keeps default values silently)
or whose blocks would overflow its arrays raise FormatError; the makeGal
reader does not shuffle (the reference shuffles with an unseeded
std::random_device); agc files carry no id and get id = file index.
"""
import struct

import numpy as np

FMT_AG, FMT_AGC, FMT_AGE, FMT_GADGET, FMT_MAKEGAL = 0, 1, 2, 3, 4
NAMES = {"ag": FMT_AG, "agc": FMT_AGC, "age": FMT_AGE, "gadget": FMT_GADGET, "makeGal": FMT_MAKEGAL}

# Units.h:6-20
KPC = 3.08567758149137e19
KMS = 1.0e3
MSUN = 1.98847e30

# record layouts of saveData / loadICs (DataManager.cpp:143-155, 183-209, 237-253)
REC = {
    FMT_AG: np.dtype([("pos", "<f8", 3), ("mass", "<f8"), ("T", "<f8"), ("vdens", "<f8"), ("sfr", "<f8"),
                      ("type", "u1"), ("gp", "u1"), ("id", "<u4")]),
    FMT_AGC: np.dtype([("pos", "<f4", 3), ("vdens", "<f4"), ("sfr", "<f4"), ("T", "<f4"), ("type", "u1"),
                       ("gp", "u1")]),
    FMT_AGE: np.dtype([("pos", "<f8", 3), ("vel", "<f8", 3), ("mass", "<f8"), ("T", "<f8"), ("P", "<f8"),
                       ("vdens", "<f8"), ("U", "<f8"), ("type", "u1"), ("gp", "u1"), ("id", "<u4")]),
}
assert [REC[k].itemsize for k in (FMT_AG, FMT_AGC, FMT_AGE)] == [62, 26, 94]


class FormatError(ValueError):
    pass


def _agf_header(types, dt, end, t):
    """AGFHeader (DataManager.h:44-50): counts of types 1, 2, 3, padding, times."""
    c = [int(np.count_nonzero(types == k)) for k in (1, 2, 3)]
    return struct.pack("<3i4x3d", c[0], c[1], c[2], dt, end, t)


def encode(fmt, p, count, dt=0.0, end=0.0, t=0.0):
    """saveData(particles, ..., numberOfParticles=count, deltaTime=dt,
    endTime=end, currentTime=t): the file's bytes."""
    n = len(p["mass"])
    assert 0 <= count <= n
    sl = slice(0, count)
    if fmt in REC:
        rec = np.zeros(count, REC[fmt])
        if fmt == FMT_AGC:
            # static_cast<float> of each double (DataManager.cpp:186-198)
            rec["pos"] = p["pos"][sl].astype(np.float32)
        else:
            rec["pos"] = p["pos"][sl]
        for f in rec.dtype.names:
            if f == "pos":
                continue
            rec[f] = p[f][sl].astype(rec.dtype[f].base)
        return _agf_header(p["type"][sl], dt, end, t) + rec.tobytes()
    if fmt != FMT_GADGET:
        raise FormatError("not a snapshot format")
    ty, gp = p["type"][sl], p["gp"][sl]
    # DataManager.cpp:274-305: the lists and gadget types
    A = (gp == 1) & (ty == 1)  # gadget type 2, pushed to gas_particles
    B = (gp == 3) & (ty == 3)  # gadget type 1, pushed to disk_particles
    C = (gp == 2) & (ty == 1)  # gadget type 3, pushed to halo_particles
    D = ty == 2                # gadget type 0, pushed to gas_particles
    E = ~(A | B | C | D)       # gadget type 0, in no list
    L0 = np.flatnonzero(A | D)
    L1 = np.flatnonzero(C)
    L2 = np.flatnonzero(B)
    order = np.concatenate([L0, L1, L2])
    npart = [int(D.sum() + E.sum()), int(B.sum()), int(A.sum()), int(C.sum()), 0, 0]
    hdr = bytearray(256)  # gadget2Header, memset to zero (DataManager.cpp:266-268)
    struct.pack_into("<6I", hdr, 0, *npart)
    struct.pack_into("<d", hdr, 72, t)           # time
    struct.pack_into("<6I", hdr, 96, *npart)     # npartTotal
    struct.pack_into("<i", hdr, 124, 1)          # num_files
    struct.pack_into("<d", hdr, 152, 1.0)        # HubbleParam
    out = [struct.pack("<I", 256), bytes(hdr), struct.pack("<I", 256)]

    def block(arr):
        b = arr.tobytes()
        out.extend([struct.pack("<I", len(b)), b, struct.pack("<I", len(b))])

    pos = p["pos"][sl][order]
    # prepareData takes the unit as a float (DataManager.cpp:322)
    block((pos / float(np.float32(KPC))).astype(np.float32))
    # the velocity block is prepared from position / Units::KMS
    # (prepareData reads position, DataManager.cpp:322-329, 349-356)
    block((pos / float(np.float32(KMS))).astype(np.float32))
    block(p["id"][sl][order].astype("<u4"))
    block((p["mass"][sl][order] / (MSUN * 1e10)).astype(np.float32))
    if len(L0):
        block((p["U"][sl][L0] / 1e6).astype(np.float32))
    return b"".join(out)


def _empty(n):
    return dict(pos=np.zeros((n, 3)), vel=np.zeros((n, 3)), mass=np.zeros(n), T=np.zeros(n), P=np.zeros(n),
                vdens=np.zeros(n), U=np.zeros(n), sfr=np.zeros(n), type=np.ones(n, np.uint8),
                gp=np.ones(n, np.uint8), id=np.zeros(n, np.uint32))


def _f32(b, off, nbytes, count):
    """`count` floats from the region [off, off+nbytes); bytes past the region
    read as zero (the reference reads a short block into a zeroed array)."""
    raw = np.zeros(4 * count, np.uint8)
    k = min(nbytes, 4 * count)
    raw[:k] = np.frombuffer(b, np.uint8, k, off)
    return raw.view("<f4")


def _u32(b, off, nbytes, count):
    return _f32(b, off, nbytes, count).view("<u4")


def decode(fmt, b):
    """loadICs(particles) on the file bytes b: (particles dict, times3)."""
    size = len(b)
    if fmt in REC:
        # DataManager.cpp:446-573
        if size < 40:
            raise FormatError("short header")
        c1, c2, c3 = struct.unpack_from("<3i", b, 0)
        if min(c1, c2, c3) < 0:
            raise FormatError("negative count")
        n = c1 + c2 + c3
        times = struct.unpack_from("<3d", b, 16)
        R = REC[fmt]
        if 40 + n * R.itemsize > size:
            raise FormatError("records past the end of the file")
        rec = np.frombuffer(b, R, n, 40)
        p = _empty(n)
        p["pos"] = rec["pos"].astype(np.float64)
        for f in R.names:
            if f != "pos":
                p[f] = rec[f].astype(p[f].dtype).reshape(p[f].shape)
        if fmt == FMT_AGC:
            p["id"] = np.arange(n, dtype=np.uint32)
        return p, times
    if fmt == FMT_GADGET:
        return _decode_gadget(b)
    if fmt == FMT_MAKEGAL:
        return _decode_makegal(b)
    raise FormatError("unknown format")


# Gadget type -> (type, galaxyPart) of the gadget reader (DataManager.cpp:1111-1143);
# types 2, 4, 5 keep the default galaxyPart 1
_GAD_TYPE = [(2, 1), (3, 3), (1, 1), (1, 2), (1, 1), (1, 1)]
# and of the makeGal reader (DataManager.cpp:731-760)
_MKG_TYPE = [(2, 1), (3, 3), (1, 1), (1, 2), (1, 1), (1, 2)]


def _decode_gadget(b):
    """DataManager.cpp:811-1322."""
    size = len(b)
    if size < 264:
        raise FormatError("short header")
    if struct.unpack_from("<I", b, 0)[0] != 256:
        raise FormatError("header block size")
    npart = struct.unpack_from("<6I", b, 4)
    massarr = struct.unpack_from("<6d", b, 28)
    time = struct.unpack_from("<d", b, 4 + 72)[0]
    n = sum(npart)
    eps = float(np.float32(1e-10))
    has_ind = any(massarr[k] < eps and npart[k] != 0 for k in range(6))
    pos = [264]

    def block(expected):
        p = pos[0]
        if p + 4 > size:
            raise FormatError("file ends before a block")
        bs = struct.unpack_from("<I", b, p)[0]
        if bs > expected:
            raise FormatError("block larger than its array")
        if p + 8 + bs > size:
            raise FormatError("file ends inside a block")
        if struct.unpack_from("<I", b, p + 4 + bs)[0] != bs:
            raise FormatError("block markers differ")
        pos[0] = p + 8 + bs
        return p + 4, bs

    P = block(12 * n)
    V = block(12 * n)
    I = block(4 * n)
    M = block(4 * n) if has_ind else None
    U = block(4 * npart[0]) if npart[0] > 0 else None
    p = _empty(n)
    p["pos"] = _f32(b, P[0], P[1], 3 * n).astype(np.float64).reshape(n, 3) * KPC
    p["vel"] = _f32(b, V[0], V[1], 3 * n).astype(np.float64).reshape(n, 3) * KMS
    p["id"] = _u32(b, I[0], I[1], n).copy()
    tcode = np.repeat(np.arange(6), npart)
    if has_ind:
        p["mass"] = _f32(b, M[0], M[1], n).astype(np.float64) * MSUN * 1e10
    else:
        p["mass"] = np.array([massarr[t] * MSUN * 1e10 for t in tcode], np.float64).reshape(n)
    if U is not None:
        u = _f32(b, U[0], U[1], npart[0]).astype(np.float64) * 1e6
        p["U"][:npart[0]] = u
    p["type"] = np.array([_GAD_TYPE[t][0] for t in tcode], np.uint8).reshape(n)
    p["gp"] = np.array([_GAD_TYPE[t][1] for t in tcode], np.uint8).reshape(n)
    return p, (0.0, 0.0, time)


def _decode_makegal(b):
    """DataManager.cpp:580-809: the reader's fixed sequence of reads, without
    the final shuffle."""
    size = len(b)
    if size < 280:
        raise FormatError("short header")
    npart = struct.unpack_from("<6i", b, 20)
    mass = struct.unpack_from("<6d", b, 20 + 24)
    time = struct.unpack_from("<d", b, 20 + 72)[0]
    if min(npart) < 0:
        raise FormatError("negative count")
    n = sum(npart)
    typelist = [mass[k] == 0 and npart[k] > 0 for k in range(6)]
    K = sum(npart[k] for k in range(6) if typelist[k])
    off = 280
    regs = []
    for nbytes in (12 * n, 12 * n, 4 * n, 4 * K, 4 * npart[0]):
        off += 16 + 4       # label record, then the block's size
        regs.append((off, nbytes))
        off += nbytes + 4   # the values the reader consumes, then the trailer
    if regs[4][0] + regs[4][1] > size:
        raise FormatError("particle data past the end of the file")
    p = _empty(n)
    tcode = np.repeat(np.arange(6), npart)
    p["pos"] = np.frombuffer(b, "<f4", 3 * n, regs[0][0]).astype(np.float64).reshape(n, 3) * KPC
    p["vel"] = np.frombuffer(b, "<f4", 3 * n, regs[1][0]).astype(np.float64).reshape(n, 3) * KMS
    p["id"] = np.frombuffer(b, "<u4", n, regs[2][0]).copy()
    stream = np.frombuffer(b, "<f4", K, regs[3][0])
    m32 = np.zeros(n, np.float32)
    k = 0
    for t in range(6):
        a, e = sum(npart[:t]), sum(npart[:t + 1])
        if typelist[t]:
            m32[a:e] = stream[k:k + npart[t]]
            k += npart[t]
        else:
            m32[a:e] = np.float32(mass[t])
    p["mass"] = m32.astype(np.float64) * MSUN * 1e10
    p["U"][:npart[0]] = np.frombuffer(b, "<f4", npart[0], regs[4][0]).astype(np.float64) * 1e6
    p["type"] = np.array([_MKG_TYPE[t][0] for t in tcode], np.uint8).reshape(n)
    p["gp"] = np.array([_MKG_TYPE[t][1] for t in tcode], np.uint8).reshape(n)
    return p, (0.0, 0.0, time)


# ---- writers of initial-condition files for tests (not in the reference) ----
def gadget_ic(npart, pos_kpc, vel_kms, ids, massarr, masses=None, u=None, time=0.0):
    """A Gadget-2 format-1 file: header, POS, VEL, ID, [MASS], [U] blocks."""
    hdr = bytearray(256)
    struct.pack_into("<6I", hdr, 0, *npart)
    struct.pack_into("<6d", hdr, 24, *massarr)
    struct.pack_into("<d", hdr, 72, time)
    struct.pack_into("<6I", hdr, 96, *npart)
    out = [struct.pack("<I", 256), bytes(hdr), struct.pack("<I", 256)]
    for arr in (pos_kpc, vel_kms, ids, masses, u):
        if arr is None:
            continue
        bb = np.ascontiguousarray(arr).tobytes()
        out += [struct.pack("<I", len(bb)), bb, struct.pack("<I", len(bb))]
    return b"".join(out)


def makegal_ic(npart, pos_kpc, vel_kms, ids, mass, masses=None, u=None, rho=None, hsml=None, time=0.0):
    """A Gadget-2 format-2 file (labelled blocks) as makeGal writes it."""
    def rec(label, bb):
        return (struct.pack("<i4sii", 8, label, len(bb) + 8, 8) + struct.pack("<I", len(bb)) + bb +
                struct.pack("<I", len(bb)))
    hdr = bytearray(256)
    struct.pack_into("<6i", hdr, 0, *npart)
    struct.pack_into("<6d", hdr, 24, *mass)
    struct.pack_into("<d", hdr, 72, time)
    struct.pack_into("<6i", hdr, 96, *npart)
    out = [rec(b"HEAD", bytes(hdr))]
    for label, arr in ((b"POS ", pos_kpc), (b"VEL ", vel_kms), (b"ID  ", ids), (b"MASS", masses), (b"U   ", u),
                       (b"RHO ", rho), (b"HSML", hsml)):
        if arr is not None:
            out.append(rec(label, np.ascontiguousarray(arr).tobytes()))
    return b"".join(out)


def random_particles(n, seed, all_classes=True):
    """Particles with every (type, galaxyPart) combination the writers sort on."""
    rng = np.random.default_rng(seed)
    p = _empty(n)
    p["pos"] = rng.normal(0, 3 * KPC, (n, 3))
    p["vel"] = rng.normal(0, 200 * KMS, (n, 3))
    p["mass"] = rng.uniform(1e36, 1e38, n)
    p["T"] = rng.uniform(0, 1e6, n)
    p["P"] = rng.uniform(0, 1e-12, n)
    p["vdens"] = rng.uniform(0, 1e-20, n)
    p["U"] = rng.uniform(0, 1e12, n)
    p["sfr"] = rng.uniform(0, 1e-3, n)
    p["type"] = rng.integers(1, 4, n).astype(np.uint8)
    p["gp"] = rng.integers(1, 4 if all_classes else 2, n).astype(np.uint8)
    p["id"] = rng.permutation(n).astype(np.uint32) * 7 + 3
    return p


# ---- the reference itself (oracle/_ref/libag2ref.so, built from its sources) ----
_REF = None


def ref_lib():
    """The reference's DataManager through ref_harness.cpp, or None when
    oracle/_ref was not built (no reference checkout on this machine)."""
    global _REF
    if _REF is None:
        import ctypes
        import os
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "libag2ref.so")
        if not os.path.exists(path):
            return None
        lib = ctypes.CDLL(path)
        P = ctypes.c_void_p
        lib.orc_ref_save.argtypes = ([ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int] + [P] * 11 +
                                     [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double])
        lib.orc_ref_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int] + [P] * 12
        _REF = lib
    return _REF


_FIELDS = ("pos", "vel", "mass", "T", "P", "vdens", "U", "sfr", "type", "gp", "id")


def ref_save(fmt_name, p, count, dt=0.0, end=0.0, t=0.0):
    """The bytes DataManager::saveData writes for these particles."""
    import os
    import tempfile
    lib = ref_lib()
    arrs = [np.ascontiguousarray(p[k]) for k in _FIELDS]
    with tempfile.TemporaryDirectory() as d:
        lib.orc_ref_save((d + "/").encode(), fmt_name.encode(), len(p["mass"]), count,
                         *[a.ctypes.data for a in arrs], 7, dt, end, t)
        with open(os.path.join(d, "7." + fmt_name), "rb") as f:
            return f.read()


def ref_load(path, fmt_name, cap):
    """DataManager::loadICs on a file: (particles, the reader's return value)."""
    import os
    import tempfile
    lib = ref_lib()
    q = _empty(cap)
    arrs = [np.ascontiguousarray(q[k]) for k in _FIELDS]
    ok = np.zeros(1, np.int32)
    with tempfile.TemporaryDirectory() as root:
        os.makedirs(os.path.join(root, "input_data"))
        os.makedirs(os.path.join(root, "a", "b"))
        os.symlink(os.path.abspath(path), os.path.join(root, "input_data", "ic"))
        n = lib.orc_ref_load(os.path.join(root, "a", "b").encode(), b"ic", fmt_name.encode(), cap,
                             *[a.ctypes.data for a in arrs], ok.ctypes.data)
    if n < 0:
        raise OSError("reference loader could not run")
    return {k: a[:n] for k, a in zip(_FIELDS, arrs)}, bool(ok[0])


def canonical_order(p):
    """Indices sorting particles by (id, x, y, z): compares the makeGal reader,
    which shuffles, order-insensitively."""
    return np.lexsort((p["pos"][:, 2], p["pos"][:, 1], p["pos"][:, 0], p["id"]))


def field_digest(p, order=None):
    """sha256 per field of the particle arrays (little-endian bytes)."""
    import hashlib
    out = {}
    for k in _FIELDS:
        a = p[k] if order is None else p[k][order]
        out[k] = hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    return out
