"""ctypes binding of the CPU oracle (oracle/_build/libknc_oracle.so).

TEST INFRASTRUCTURE ONLY: the checker for the GPU library. Loaded by tests/,
the smoke entry point and the CPU-baseline leg of bench.py; never by the
library. PARITY UNPINNED (see knc_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libknc_oracle.so"


def build(quiet: bool = True) -> Path:
    """Compile the oracle with its Makefile (g++, no external libraries)."""
    r = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    if not quiet:
        print(r.stdout)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        build()
    from knc import abi  # parameter structs shared with the library header
    lib = C.CDLL(str(LIB))
    P = C.c_void_p
    DP = C.POINTER(C.c_double)
    sig = {
        "oracle_create": (C.c_int, [C.POINTER(abi.HydroParams), C.POINTER(abi.MeshParams), C.c_int32, C.POINTER(P)]),
        "oracle_destroy": (None, [P]),
        "oracle_set_model": (C.c_int, [P, C.POINTER(abi.ModelParams)]),
        "oracle_init_from_model": (C.c_int, [P, C.c_double]),
        "oracle_add_block": (C.c_int, [P, C.c_int32, DP, DP]),
        "oracle_remove_block": (C.c_int, [P, C.c_int32]),
        "oracle_set_block_shapes": (C.c_int, [P, C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
        "oracle_block_shape_of": (C.c_int, [P, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
        "oracle_get_block": (C.c_int, [P, C.c_int32, DP, DP]),
        "oracle_get_primitives": (C.c_int, [P, C.c_int32, DP]),
        "oracle_get_products": (C.c_int, [P, C.c_int32, DP, DP, DP, DP]),
        "oracle_num_blocks": (C.c_int, [P, C.POINTER(C.c_int32)]),
        "oracle_block_indexes": (C.c_int, [P, C.POINTER(C.c_int32), C.c_int32]),
        "oracle_set_time": (C.c_int, [P, C.c_double, C.c_int64, C.c_int64]),
        "oracle_get_time": (C.c_int, [P, DP, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
        "oracle_time_step": (C.c_int, [P, DP]),
        "oracle_advance": (C.c_int, [P, C.c_int32]),
        "oracle_advance_dt": (C.c_int, [P, C.c_int32, C.c_double]),
        "oracle_last_error": (C.c_int, [P, C.POINTER(abi.Error)]),
        "oracle_c2p_stats": (C.c_int, [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
        "oracle_prim_to_cons": (None, [C.POINTER(abi.HydroParams), DP, DP]),
        "oracle_cons_to_prim": (C.c_int, [C.POINTER(abi.HydroParams), DP, C.c_double, DP, C.POINTER(C.c_int32)]),
        "oracle_flux": (None, [C.POINTER(abi.HydroParams), DP, C.c_int32, DP, DP, DP]),
        "oracle_riemann": (None, [C.POINTER(abi.HydroParams), DP, DP, C.c_double, C.c_double, C.c_int32, DP]),
        "oracle_plm_gradient": (C.c_double, [C.c_double, C.c_double, C.c_double, C.c_double]),
        "oracle_sources": (None, [C.POINTER(abi.HydroParams), DP, C.c_double, C.c_double, DP]),
        "oracle_max_signal_speed": (C.c_double, [C.POINTER(abi.HydroParams), DP]),
        "oracle_block_geometry": (C.c_int, [C.POINTER(abi.MeshParams), C.c_int32, DP, DP, DP, DP, DP, DP, DP]),
        "oracle_mlp_forward_backward": (None, [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                               C.c_int32, C.c_int32, DP, DP, DP]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """Mirror of knc.Solver over the CPU oracle (same calls, same layouts)."""

    def __init__(self, hydro, mesh, threads: int = 1):
        from knc import abi
        self._abi = abi
        self.lib = load()
        self.hp = hydro.to_c() if hasattr(hydro, "to_c") else hydro
        self.mp = mesh.to_c() if hasattr(mesh, "to_c") else mesh
        h = C.c_void_p()
        st = self.lib.oracle_create(C.byref(self.hp), C.byref(self.mp), threads, C.byref(h))
        if st != 0:
            raise RuntimeError(f"oracle_create failed: {st}")
        self.h = h
        self.nr = int(self.mp.block_size)
        self.nq = int(self.mp.num_polar_zones)

    def close(self):
        if self.h:
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st != 0:
            e = self._abi.Error()
            self.lib.oracle_last_error(self.h, C.byref(e))
            raise RuntimeError(f"{what}: status {st}: {e.message.decode()}")

    def set_model(self, model):
        mp = model.to_c() if hasattr(model, "to_c") else model
        self._check(self.lib.oracle_set_model(self.h, C.byref(mp)), "set_model")

    def init_from_model(self, time: float = 0.0):
        self._check(self.lib.oracle_init_from_model(self.h, time), "init_from_model")

    def add_block(self, index, cons, scalar):
        cons = np.ascontiguousarray(cons, dtype=np.float64)
        scalar = np.ascontiguousarray(scalar, dtype=np.float64)
        self._check(self.lib.oracle_add_block(self.h, index, _d(cons), _d(scalar)), "add_block")

    def remove_block(self, index):
        self._check(self.lib.oracle_remove_block(self.h, index), "remove_block")

    def set_block_shapes(self, first, nr, nq):
        nr = np.ascontiguousarray(nr, dtype=np.int32)
        nq = np.ascontiguousarray(nq, dtype=np.int32)
        i32 = C.POINTER(C.c_int32)
        self._check(self.lib.oracle_set_block_shapes(self.h, first, len(nr), nr.ctypes.data_as(i32),
                                                     nq.ctypes.data_as(i32)), "set_block_shapes")

    def shape_of(self, index):
        a = C.c_int64()
        b = C.c_int64()
        self.lib.oracle_block_shape_of(self.h, index, C.byref(a), C.byref(b))
        return a.value, b.value

    def block_indexes(self):
        n = C.c_int32()
        self.lib.oracle_num_blocks(self.h, C.byref(n))
        out = (C.c_int32 * max(n.value, 1))()
        self.lib.oracle_block_indexes(self.h, out, n.value)
        return [out[k] for k in range(n.value)]

    def get_block(self, index):
        nr, nq = self.shape_of(index)
        cons = np.empty((nr, nq, 4))
        scalar = np.empty((nr, nq))
        self._check(self.lib.oracle_get_block(self.h, index, _d(cons), _d(scalar)), "get_block")
        return cons, scalar

    def state(self):
        return {i: self.get_block(i) for i in self.block_indexes()}

    def get_products(self, index):
        """BlockProducts of a block: radial and polar vertices, primitive
        [nr, nq, 4] in AnyPrimitive order, scalar [nr, nq]."""
        nr, nq = self.shape_of(index)
        rv, qv = np.empty(nr + 1), np.empty(nq + 1)
        prim, scal = np.empty((nr, nq, 4)), np.empty((nr, nq))
        self._check(self.lib.oracle_get_products(self.h, index, _d(rv), _d(qv), _d(prim), _d(scal)), "get_products")
        return {"radial_vertices": rv, "polar_vertices": qv, "primitive": prim, "scalar": scal}

    def get_primitives(self, index):
        """(rho, u_r, u_theta, p, scalar concentration) of a block, [nr, nq, 5]."""
        nr, nq = self.shape_of(index)
        out = np.empty((nr, nq, 5))
        self._check(self.lib.oracle_get_primitives(self.h, index, _d(out)), "get_primitives")
        return out

    def set_time(self, t, num=0, den=1):
        self._check(self.lib.oracle_set_time(self.h, t, num, den), "set_time")

    def time(self):
        t = C.c_double()
        n = C.c_int64()
        d = C.c_int64()
        self.lib.oracle_get_time(self.h, C.byref(t), C.byref(n), C.byref(d))
        return t.value, (n.value, d.value)

    def time_step(self):
        dt = C.c_double()
        self._check(self.lib.oracle_time_step(self.h, C.byref(dt)), "time_step")
        return dt.value

    def advance(self, fold: int = 1, dt=None):
        if dt is None:
            self._check(self.lib.oracle_advance(self.h, fold), "advance")
        else:
            self._check(self.lib.oracle_advance_dt(self.h, fold, float(dt)), "advance_dt")

    def last_error(self):
        e = self._abi.Error()
        self.lib.oracle_last_error(self.h, C.byref(e))
        return e

    def try_advance(self, fold: int = 1):
        return self.lib.oracle_advance(self.h, fold)

    def c2p_stats(self):
        z = C.c_int64()
        it = C.c_int64()
        self.lib.oracle_c2p_stats(self.h, C.byref(z), C.byref(it))
        return z.value, it.value


# ---- point physics -------------------------------------------------------
def prim_to_cons(hp, p):
    lib = load()
    p = np.ascontiguousarray(p, dtype=np.float64)
    u = np.empty(4)
    lib.oracle_prim_to_cons(C.byref(hp), _d(p), _d(u))
    return u


def cons_to_prim(hp, u, guess=-1.0):
    lib = load()
    u = np.ascontiguousarray(u, dtype=np.float64)
    p = np.empty(4)
    it = C.c_int32()
    kind = lib.oracle_cons_to_prim(C.byref(hp), _d(u), guess, _d(p), C.byref(it))
    return kind, p, it.value


def flux(hp, p, axis):
    lib = load()
    p = np.ascontiguousarray(p, dtype=np.float64)
    f = np.empty(4)
    lm = C.c_double()
    lp = C.c_double()
    lib.oracle_flux(C.byref(hp), _d(p), axis, _d(f), C.byref(lm), C.byref(lp))
    return f, lm.value, lp.value


def riemann(hp, pl, pr, sl, sr, axis):
    lib = load()
    pl = np.ascontiguousarray(pl, dtype=np.float64)
    pr = np.ascontiguousarray(pr, dtype=np.float64)
    out = np.empty(5)
    lib.oracle_riemann(C.byref(hp), _d(pl), _d(pr), sl, sr, axis, _d(out))
    return out


def plm_gradient(theta, a, b, c):
    return load().oracle_plm_gradient(theta, a, b, c)


def sources(hp, p, r, theta):
    lib = load()
    p = np.ascontiguousarray(p, dtype=np.float64)
    s = np.empty(4)
    lib.oracle_sources(C.byref(hp), _d(p), r, theta, _d(s))
    return s


def max_signal_speed(hp, p):
    p = np.ascontiguousarray(p, dtype=np.float64)
    return load().oracle_max_signal_speed(C.byref(hp), _d(p))


def block_geometry(mp, index):
    lib = load()
    nr, nq = int(mp.block_size), int(mp.num_polar_zones)
    out = dict(rv=np.empty(nr + 1), qv=np.empty(nq + 1), ar=np.empty((nr + 1, nq)),
               aq=np.empty((nr, nq + 1)), dv=np.empty((nr, nq)), rc=np.empty((nr, nq)),
               qc=np.empty((nr, nq)))
    st = lib.oracle_block_geometry(C.byref(mp), index, *[_d(out[k]) for k in
                                                          ("rv", "qv", "ar", "aq", "dv", "rc", "qc")])
    if st != 0:
        raise RuntimeError("oracle_block_geometry failed")
    return out


def mlp_forward_backward(weights, x, y, round_bf16=True):
    lib = load()
    weights = np.ascontiguousarray(weights, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    n = len(y)
    pred = np.empty(n)
    loss = C.c_double()
    grad = np.empty(len(weights))
    fp = C.POINTER(C.c_float)
    lib.oracle_mlp_forward_backward(weights.ctypes.data_as(fp), x.ctypes.data_as(fp),
                                    y.ctypes.data_as(fp), n, int(bool(round_bf16)), _d(pred), C.byref(loss),
                                    _d(grad))
    return pred, loss.value, grad
