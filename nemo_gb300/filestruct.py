"""NEMO structured binary files (filestruct) and snapshots, in Python.

Format (src/kernel/io/filesecret.c:927-955 puthdr, 1077-1140 gethdr): each
item is a 2-byte magic (0x0992 singular, 0x0b92 plural; byte-swapped magic
means a file of the other endianness), a NUL-terminated type string, for all
but ")" a NUL-terminated tag, for plural items a 0-terminated list of int
dimensions, then the raw data.  Sets are "(" ... ")" with nested items.

Also provides ``bsf`` -- the "mean sigma min max count" fingerprint of all
floating-point values in a file (src/kernel/io/bsf.c:45-160), ignoring the
``cputime`` items as bsf does by default.
"""
from __future__ import annotations

import io
import struct
from dataclasses import dataclass, field

import numpy as np

SING, PLUR = 0x0992, 0x0B92
TYPES = {"a": ("u1", 1), "c": ("S1", 1), "b": ("u1", 1), "s": ("i2", 2), "i": ("i4", 4), "l": ("i8", 8),
         "h": ("i2", 2), "f": ("f4", 4), "d": ("f8", 8)}


@dataclass
class Item:
    type: str
    tag: str | None
    dims: list = field(default_factory=list)
    data: bytes = b""
    items: list = field(default_factory=list)
    endian: str = "<"

    def find(self, tag):
        for it in self.items:
            if it.tag == tag:
                return it
        return None

    def array(self):
        dt, _ = TYPES[self.type]
        a = np.frombuffer(self.data, dtype=np.dtype(self.endian + dt) if dt not in ("S1", "u1") else dt)
        return a.reshape(self.dims) if self.dims else a[0] if len(a) else a

    def text(self):
        s = self.data.decode("latin1")
        return s[:-1] if s.endswith("\0") else s


def _cstr(f):
    out = bytearray()
    while True:
        ch = f.read(1)
        if not ch:
            raise EOFError("EOF inside header string")
        if ch == b"\0":
            return out.decode("latin1")
        out += ch


def read_item(f):
    """Next item of stream f, or None at end of file."""
    raw = f.read(2)
    if len(raw) < 2:
        return None
    (magic,) = struct.unpack("<h", raw)
    end = "<"
    if magic not in (SING, PLUR):
        (magic,) = struct.unpack(">h", raw)
        end = ">"
        if magic not in (SING, PLUR):
            raise ValueError("gethdr: bad magic")
    typ = _cstr(f)
    tag = None if typ == ")" else _cstr(f)
    dims = []
    if magic == PLUR:
        while True:
            (d,) = struct.unpack(end + "i", f.read(4))
            if d == 0:
                break
            dims.append(d)
    it = Item(typ, tag, dims, endian=end)
    if typ == "(":
        while True:
            sub = read_item(f)
            if sub is None:
                raise EOFError(f"EOF inside set {tag}")
            if sub.type == ")":
                break
            it.items.append(sub)
    elif typ != ")":
        n = int(np.prod(dims)) if dims else 1
        it.data = f.read(n * TYPES[typ][1])
    return it


def read_items(path_or_file):
    f = open(path_or_file, "rb") if isinstance(path_or_file, str) else path_or_file
    try:
        out = []
        while True:
            it = read_item(f)
            if it is None:
                return out
            out.append(it)
    finally:
        if isinstance(path_or_file, str):
            f.close()


class Writer:
    def __init__(self, f):
        self.f = f

    def _hdr(self, typ, tag, dims):
        self.f.write(struct.pack("<h", PLUR if dims else SING))
        self.f.write(typ.encode() + b"\0")
        if tag is not None:
            self.f.write(tag.encode() + b"\0")
        if dims:
            self.f.write(struct.pack("<%di" % (len(dims) + 1), *dims, 0))

    def set(self, tag):
        self._hdr("(", tag, None)

    def tes(self):
        self._hdr(")", None, None)

    def data(self, tag, typ, arr, dims=None):
        a = np.ascontiguousarray(arr, dtype=np.dtype("<" + TYPES[typ][0]) if typ not in ("c", "a") else None)
        self._hdr(typ, tag, dims)
        self.f.write(a.tobytes() if hasattr(a, "tobytes") else bytes(a))

    def string(self, tag, s):
        b = s.encode("latin1") + b"\0"
        self._hdr("c", tag, [len(b)])
        self.f.write(b)


@dataclass
class Snapshot:
    nbody: int
    time: float | None
    mass: np.ndarray | None = None
    phase: np.ndarray | None = None
    phi: np.ndarray | None = None
    acc: np.ndarray | None = None
    diagnostics: dict = field(default_factory=dict)


def snapshots(path):
    """All SnapShot sets of a file as Snapshot records (get_snap layout)."""
    out = []
    for it in read_items(path):
        if it.type != "(" or it.tag != "SnapShot":
            continue
        par, pts, dia = it.find("Parameters"), it.find("Particles"), it.find("Diagnostics")
        n = int(par.find("Nobj").array())
        t = par.find("Time")
        s = Snapshot(n, float(t.array()) if t is not None else None)
        if pts is not None:
            for tag, attr in (("Mass", "mass"), ("PhaseSpace", "phase"), ("Potential", "phi"), ("Acceleration", "acc")):
                x = pts.find(tag)
                if x is not None:
                    setattr(s, attr, np.array(x.array(), dtype=np.float64))
        if dia is not None:
            for x in dia.items:
                s.diagnostics[x.tag] = np.array(x.array())
        out.append(s)
    return out


def write_snapshot(w: Writer, mass, phase, time=0.0, phi=None, acc=None):
    n = len(mass)
    w.set("SnapShot")
    w.set("Parameters")
    w.data("Nobj", "i", np.array([n]))
    w.data("Time", "d", np.array([time]))
    w.tes()
    w.set("Particles")
    w.data("CoordSystem", "i", np.array([(1 << 16) | (3 << 8) | 2]))
    w.data("Mass", "d", mass, [n])
    w.data("PhaseSpace", "d", phase, [n, 2, 3])
    if phi is not None:
        w.data("Potential", "d", phi, [n])
    if acc is not None:
        w.data("Acceleration", "d", acc, [n, 3])
    w.tes()
    w.tes()


def bsf(path, ignore="cputime", fmt="%g"):
    """bsf fingerprint: 'mean sigma min max count' of every float/double."""
    vals = []

    def walk(it):
        if it.type == "(":
            for s in it.items:
                walk(s)
        elif it.type in ("f", "d") and it.tag != ignore:
            vals.append(np.asarray(it.array(), dtype=np.float64).ravel())

    for it in read_items(path):
        walk(it)
    v = np.concatenate(vals) if vals else np.zeros(0)
    n = len(v)
    if n == 0:
        return "0 0 0 0 0"
    s1 = s2 = 0.0
    for x in v.tolist():          # sequential FP64 sums, in file order
        s1 += x
        s2 += x * x
    mean = s1 / n
    var = s2 / n - mean * mean
    sig = 0.0 if (v.min() == v.max() or var <= 0) else var ** 0.5
    return " ".join([fmt % mean, fmt % sig, fmt % v.min(), fmt % v.max(), "%d" % n])
