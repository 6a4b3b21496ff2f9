"""CBOR checkpoints in the reference's `App` layout, and products files in its
`Products` layout.

The reference writes `App { state, tasks, config, version }` (src/app.rs:181-186)
with serde and ciborium 0.1 (src/io.rs:24-35), and restarts from it
(src/app.rs:344-350). This module writes and reads the same document shape:

  App        map {"state", "tasks", "config", "version"}
  state      AnyState, externally tagged: {"Relativistic" | "Newtonian": State}
  State      map {"time": f64, "iteration": [num, den] (Rational64),
                  "solution": map {[i, 0]: BlockState}}   (BlockIndex keys)
  BlockState map {"conserved": Array, "scalar_mass": Array}
  Array      ndarray 0.14: map {"v": 1, "dim": [nr, nq], "data": [...]}
             conserved elements are [D, S_r, S_theta, tau]
  tasks      map of RecurringTask {"count", "next_time"}
  config     Configuration {"hydro": {"relativistic" | "newtonian": {...}},
                            "model": {name: {...}}, "mesh": {...}, "control": {...}}

Unpinned detail: the element type of `conserved` (hydro_srhd::srhd_2d::Conserved,
hydro_euler::euler_2d::Conserved) comes from un-vendored crates; it is
written as a four-element array, the serde form of a 4-field tuple struct.
Floats outside the big arrays take the shortest lossless width, as ciborium
does; the array data is written as 8-byte floats (readers accept any width).
"""
from __future__ import annotations

import math
import struct
from dataclasses import asdict
from pathlib import Path

import numpy as np

from . import config as cfg

VERSION = "knc-gb300 0.1"


class CborError(ValueError):
    pass


class F64Array:
    """Marks an array of floats (any shape) to encode as nested CBOR arrays of
    8-byte floats: the last axis becomes the innermost array."""

    def __init__(self, a):
        self.a = np.ascontiguousarray(a, dtype=np.float64)


# ---------------------------------------------------------------- encoding --
def _head(major: int, n: int) -> bytes:
    if n < 24:
        return bytes([(major << 5) | n])
    if n < 1 << 8:
        return bytes([(major << 5) | 24, n])
    if n < 1 << 16:
        return bytes([(major << 5) | 25]) + struct.pack(">H", n)
    if n < 1 << 32:
        return bytes([(major << 5) | 26]) + struct.pack(">I", n)
    return bytes([(major << 5) | 27]) + struct.pack(">Q", n)


def _float(x: float) -> bytes:
    bits = struct.pack(">d", x)
    if not math.isnan(x):
        try:
            h = struct.pack(">e", x)
            if struct.pack(">d", struct.unpack(">e", h)[0]) == bits:
                return b"\xf9" + h
        except OverflowError:
            pass
        try:
            f = struct.pack(">f", x)
            if struct.pack(">d", struct.unpack(">f", f)[0]) == bits:
                return b"\xfa" + f
        except OverflowError:
            pass
    return b"\xfb" + bits


def _f64_array(a: np.ndarray, out: list):
    """Nested arrays of 0xfb floats, vectorised."""
    if a.ndim == 1:
        body = np.empty((a.size, 9), dtype=np.uint8)
        body[:, 0] = 0xFB
        body[:, 1:] = a.astype(">f8").view(np.uint8).reshape(-1, 8)
        out.append(_head(4, a.size))
        out.append(body.tobytes())
        return
    if a.ndim == 2:
        inner = a.shape[1]
        head = _head(4, inner)
        body = np.empty((a.shape[0], len(head) + 9 * inner), dtype=np.uint8)
        body[:, :len(head)] = np.frombuffer(head, dtype=np.uint8)
        vals = body[:, len(head):].reshape(a.shape[0], inner, 9)
        vals[:, :, 0] = 0xFB
        vals[:, :, 1:] = a.astype(">f8").view(np.uint8).reshape(a.shape[0], inner, 8)
        out.append(_head(4, a.shape[0]))
        out.append(body.tobytes())
        return
    out.append(_head(4, a.shape[0]))
    for k in range(a.shape[0]):
        _f64_array(a[k], out)


def _enc(obj, out: list):
    if obj is None:
        out.append(b"\xf6")
    elif obj is True:
        out.append(b"\xf5")
    elif obj is False:
        out.append(b"\xf4")
    elif isinstance(obj, (int, np.integer)):
        n = int(obj)
        out.append(_head(0, n) if n >= 0 else _head(1, -1 - n))
    elif isinstance(obj, (float, np.floating)):
        out.append(_float(float(obj)))
    elif isinstance(obj, str):
        b = obj.encode()
        out.append(_head(3, len(b)))
        out.append(b)
    elif isinstance(obj, (bytes, bytearray)):
        out.append(_head(2, len(obj)))
        out.append(bytes(obj))
    elif isinstance(obj, F64Array):
        _f64_array(obj.a, out)
    elif isinstance(obj, (list, tuple)):
        out.append(_head(4, len(obj)))
        for v in obj:
            _enc(v, out)
    elif isinstance(obj, dict):
        out.append(_head(5, len(obj)))
        for k, v in obj.items():
            _enc(list(k) if isinstance(k, tuple) else k, out)
            _enc(v, out)
    else:
        raise CborError(f"cannot encode {type(obj).__name__}")


def dumps(obj) -> bytes:
    out: list = []
    _enc(obj, out)
    return b"".join(out)


# ---------------------------------------------------------------- decoding --
class _Reader:
    def __init__(self, data: bytes):
        self.b = memoryview(data)
        self.raw = data
        self.p = 0

    def head(self):
        ib = self.b[self.p]
        self.p += 1
        major, info = ib >> 5, ib & 31
        if info < 24:
            return major, info, ib
        if info == 24:
            n = self.b[self.p]
            self.p += 1
        elif info == 25:
            n = struct.unpack_from(">H", self.b, self.p)[0]
            self.p += 2
        elif info == 26:
            n = struct.unpack_from(">I", self.b, self.p)[0]
            self.p += 4
        elif info == 27:
            n = struct.unpack_from(">Q", self.b, self.p)[0]
            self.p += 8
        else:
            raise CborError(f"indefinite or reserved length at byte {self.p - 1}")
        return major, n, ib

    def float_array(self, n: int):
        """n floats of one width, vectorised; None if the run is not uniform."""
        if n == 0:
            return np.empty(0)
        first = self.b[self.p]
        width = {0xFB: 9, 0xFA: 5, 0xF9: 3}.get(first)
        if width is None or self.p + n * width > len(self.b):
            return None
        seg = np.frombuffer(self.raw, dtype=np.uint8, count=n * width, offset=self.p).reshape(n, width)
        if not np.all(seg[:, 0] == first):
            return None
        dt = {9: ">f8", 5: ">f4", 3: ">f2"}[width]
        vals = seg[:, 1:].copy().view(dt).reshape(n).astype(np.float64)
        self.p += n * width
        return vals

    def item(self):
        ib = self.b[self.p]
        if ib >> 5 == 7:   # simple values and floats: the low bits are not a length
            return self.simple()
        major, n, ib = self.head()
        if major == 0:
            return n
        if major == 1:
            return -1 - n
        if major == 2:
            v = bytes(self.b[self.p:self.p + n])
            self.p += n
            return v
        if major == 3:
            v = bytes(self.b[self.p:self.p + n]).decode()
            self.p += n
            return v
        if major == 4:
            start = self.p
            if n and self.b[self.p] in (0xF9, 0xFA, 0xFB):
                arr = self.float_array(n)
                if arr is not None:
                    return arr
                self.p = start
            if n and (self.b[self.p] >> 5) == 4:
                # an array of equal-length float arrays (ndarray data of tuples)
                m = self.b[self.p] & 31
                if m < 24:
                    width = {0xFB: 9, 0xFA: 5, 0xF9: 3}.get(self.b[self.p + 1])
                    if width is not None:
                        stride = 1 + m * width
                        if self.p + n * stride <= len(self.b):
                            seg = np.frombuffer(self.raw, dtype=np.uint8, count=n * stride,
                                                offset=self.p).reshape(n, stride)
                            hdr_ok = np.all(seg[:, 0] == self.b[self.p])
                            cols = seg[:, 1:].reshape(n, m, width)
                            if hdr_ok and np.all(cols[:, :, 0] == self.b[self.p + 1]):
                                dt = {9: ">f8", 5: ">f4", 3: ">f2"}[width]
                                vals = cols[:, :, 1:].copy().view(dt).reshape(n, m).astype(np.float64)
                                self.p += n * stride
                                return vals
            return [self.item() for _ in range(n)]
        if major == 5:
            d = {}
            for _ in range(n):
                k = self.item()
                if isinstance(k, list):
                    k = tuple(k)
                elif isinstance(k, np.ndarray):
                    k = tuple(k.tolist())
                d[k] = self.item()
            return d
        if major == 6:
            return self.item()   # tags carry no meaning in this layout
        raise CborError(f"unsupported item 0x{ib:02x} at byte {self.p - 1}")

    def simple(self):
        ib = self.b[self.p]
        self.p += 1
        if ib == 0xF4:
            return False
        if ib == 0xF5:
            return True
        if ib in (0xF6, 0xF7):
            return None
        for code, fmt, size in ((0xF9, ">e", 2), (0xFA, ">f", 4), (0xFB, ">d", 8)):
            if ib == code:
                v = struct.unpack_from(fmt, self.b, self.p)[0]
                self.p += size
                return float(v)
        raise CborError(f"unsupported simple value 0x{ib:02x} at byte {self.p - 1}")


def loads(data: bytes):
    r = _Reader(bytes(data))
    v = r.item()
    if r.p != len(r.b):
        raise CborError(f"{len(r.b) - r.p} trailing bytes")
    return v


# ---------------------------------------------------------------- the App --
def _ndarray(a: np.ndarray, elem_axis: bool):
    nr, nq = a.shape[:2]
    data = a.reshape(nr * nq, -1) if elem_axis else a.reshape(nr * nq)
    return {"v": 1, "dim": [nr, nq], "data": F64Array(data)}


def _hydro_doc(h):
    d = asdict(h)
    tag = "relativistic" if isinstance(h, cfg.RelativisticHydro) else "newtonian"
    if tag == "newtonian":
        d.pop("riemann_solver", None) if h.riemann_solver == "HLLE" else None
    return {tag: d}


def _mesh_doc(m: cfg.Mesh):
    return {"reference_radius": m.reference_radius, "inner_radius": m.inner_radius,
            "outer_radius": m.outer_radius, "inner_excision_speed": m.inner_excision_speed,
            "outer_excision_speed": m.outer_excision_speed, "num_radial_zones": m.num_radial_zones,
            "num_polar_zones": m.num_polar_zones, "block_size": m.block_size,
            "excision_delay": m.excision_delay}


def _control_doc(c: cfg.Control):
    return {"start_time": c.start_time, "final_time": c.final_time,
            "checkpoint_interval": c.checkpoint_interval, "products_interval": c.products_interval,
            "fold": c.fold, "num_threads": c.num_threads, "snappy_compression": c.snappy_compression,
            "output_directory": c.output_directory}


def default_tasks(start_time: float = 0.0):
    t = {"count": 0, "next_time": start_time}
    return {"write_checkpoint": dict(t), "write_products": dict(t), "iteration_message": dict(t),
            "report_progress": dict(t)}


def app_document(blocks: dict, time: float, iteration, hydro, model_name: str, model_params: dict,
                 mesh: cfg.Mesh, control: cfg.Control, tasks: dict | None = None, version: str = VERSION):
    """blocks: {index: (cons [nr, nq, 4], scalar_mass [nr, nq])}."""
    solution = {(int(i), 0): {"conserved": _ndarray(np.asarray(c), True),
                              "scalar_mass": _ndarray(np.asarray(s), False)}
                for i, (c, s) in sorted(blocks.items())}
    tag = "Relativistic" if isinstance(hydro, cfg.RelativisticHydro) else "Newtonian"
    state = {tag: {"time": float(time), "iteration": [int(iteration[0]), int(iteration[1])],
                   "solution": solution}}
    return {"state": state, "tasks": tasks or default_tasks(control.start_time),
            "config": {"hydro": _hydro_doc(hydro), "model": {model_name: dict(model_params)},
                       "mesh": _mesh_doc(mesh), "control": _control_doc(control)},
            "version": version}


def _array1(a: np.ndarray):
    return {"v": 1, "dim": [int(a.size)], "data": F64Array(np.asarray(a, dtype=np.float64).reshape(-1))}


def products_document(blocks: dict, time: float, hydro, model_name: str, model_params: dict, mesh: cfg.Mesh,
                      control: cfg.Control, version: str = VERSION):
    """Products { time, blocks, config, version } (src/products.rs:30-36).
    blocks: {index: BlockProducts dict as Solver.get_products returns it}:
    radial / polar vertices (Array1), primitive (Array2 of AnyPrimitive, which
    serialises as [velocity_r, velocity_q, mass_density, gas_pressure],
    physics/mod.rs:36-63) and scalar (Array2)."""
    out = {}
    for i, b in sorted(blocks.items()):
        out[(int(i), 0)] = {"radial_vertices": _array1(b["radial_vertices"]),
                            "polar_vertices": _array1(b["polar_vertices"]),
                            "primitive": _ndarray(np.asarray(b["primitive"]), True),
                            "scalar": _ndarray(np.asarray(b["scalar"]), False)}
    return {"time": float(time), "blocks": out,
            "config": {"hydro": _hydro_doc(hydro), "model": {model_name: dict(model_params)},
                       "mesh": _mesh_doc(mesh), "control": _control_doc(control)},
            "version": version}


def write_products(path, solver, hydro, model_name, model_params, mesh, control):
    """Products::try_from_state + io::write_cbor (src/main.rs:51-56, the
    prods.NNNN.cbor files) for a Solver's live state: every block's primitives
    recovered in FP64 on the device."""
    t, _ = solver.time()
    blocks = {i: solver.get_products(i) for i in solver.block_indexes()}
    Path(path).write_bytes(dumps(products_document(blocks, t, hydro, model_name, model_params, mesh, control)))


def read_products(path) -> dict:
    """A prods file back as {"time", "blocks": {index: BlockProducts arrays},
    "config", "version"}."""
    doc = loads(Path(path).read_bytes())
    blocks = {}
    for key, b in doc["blocks"].items():
        index = int(key[0]) if isinstance(key, tuple) else int(key)
        nr, nq = b["primitive"]["dim"]
        blocks[index] = {"radial_vertices": np.asarray(b["radial_vertices"]["data"], dtype=np.float64),
                         "polar_vertices": np.asarray(b["polar_vertices"]["data"], dtype=np.float64),
                         "primitive": np.asarray(b["primitive"]["data"], dtype=np.float64).reshape(nr, nq, 4),
                         "scalar": np.asarray(b["scalar"]["data"], dtype=np.float64).reshape(nr, nq)}
    return {"time": float(doc["time"]), "blocks": blocks, "config": doc["config"], "version": doc["version"]}


def write_checkpoint(path, solver, hydro, model_name, model_params, mesh, control, tasks=None):
    """App::package + io::write_cbor for a Solver's live state."""
    t, it = solver.time()
    doc = app_document(solver.state(), t, it, hydro, model_name, model_params, mesh, control, tasks)
    Path(path).write_bytes(dumps(doc))


class Checkpoint:
    """A decoded App document."""

    def __init__(self, doc: dict):
        self.doc = doc
        (self.kind, st), = doc["state"].items()
        self.time = float(st["time"])
        self.iteration = (int(st["iteration"][0]), int(st["iteration"][1]))
        self.blocks = {}
        for key, bs in st["solution"].items():
            index = int(key[0]) if isinstance(key, tuple) else int(key)
            c = bs["conserved"]
            s = bs["scalar_mass"]
            nr, nq = c["dim"]
            cons = np.asarray(c["data"], dtype=np.float64).reshape(nr, nq, 4)
            scal = np.asarray(s["data"], dtype=np.float64).reshape(nr, nq)
            self.blocks[index] = (cons, scal)
        conf = doc["config"]
        (htag, hp), = conf["hydro"].items()
        self.hydro = (cfg.RelativisticHydro if htag == "relativistic" else cfg.NewtonianHydro).from_dict(hp)
        (self.model_name, self.model_params), = conf["model"].items()
        self.mesh = cfg.Mesh.from_dict(conf["mesh"])
        self.control = cfg.Control.from_dict(conf["control"])
        self.tasks = doc["tasks"]
        self.version = doc["version"]

    def restore(self, solver):
        """Load the blocks, time and iteration into a Solver (App::from_file)."""
        for i in list(solver.block_indexes()):
            if i not in self.blocks:
                solver.remove_block(i)
        for i, (c, s) in sorted(self.blocks.items()):
            solver.add_block(i, c, s)
        solver.set_time(self.time, *self.iteration)


def read_checkpoint(path) -> Checkpoint:
    """io::read_cbor of an App checkpoint."""
    return Checkpoint(loads(Path(path).read_bytes()))
