"""Python host over the C ABI of libknc_gpu.so.

`Solver` mirrors the reference's run-loop contract for the hot path:
`advance(fold)` is scheme::advance (src/scheme.rs:212-240), `time_step()` is
State::time_step (src/state.rs:143-162), blocks are BlockState keyed by
BlockIndex (i, 0) (src/state.rs:27-43), and `init_from_model` is
State::from_model over Mesh::grid_blocks (src/state.rs:107-115,
src/mesh.rs:384-397). A failed c2p raises `HydroError` carrying the same
fields as the reference's HydroError (src/physics/mod.rs:109-117).
There is no CPU fallback: every call runs the CUDA library.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


class HydroError(abi.KncError):
    """c2p failure at a zone: kind name, block index, zone, (r, theta), value."""


def _raise(lib, h, status, what):
    if status == abi.KNC_OK:
        return
    e = abi.Error()
    if h:
        lib.knc_last_error(h, C.byref(e))
    info = dict(kind=abi.HYDRO_ERROR_NAMES.get(e.kind, str(e.kind)), block=e.block, i=e.i, j=e.j,
                r=e.r, theta=e.theta, value=e.value)
    msg = f"{what}: {lib.knc_status_string(status).decode()}: {e.message.decode(errors='replace')}"
    if status == abi.KNC_ERR_HYDRO:
        raise HydroError(status, msg, info)
    raise abi.KncError(status, msg, info)


class Solver:
    """One simulation on the current CUDA device (one stream)."""

    def __init__(self, hydro, mesh, precision: int = abi.KNC_PRECISION_FP64):
        self.lib = abi.load()
        self.hydro = hydro
        self.mesh = mesh
        self.hp = hydro.to_c() if hasattr(hydro, "to_c") else hydro
        self.mp = mesh.to_c() if hasattr(mesh, "to_c") else mesh
        h = C.c_void_p()
        st = self.lib.knc_create(C.byref(self.hp), C.byref(self.mp), C.byref(h))
        if st != abi.KNC_OK:
            raise abi.KncError(st, f"knc_create: {self.lib.knc_status_string(st).decode()}")
        self.h = h
        self.nr = int(self.mp.block_size)
        self.nq = int(self.mp.num_polar_zones)
        self._host_cb = None
        if precision != abi.KNC_PRECISION_FP64:
            self.set_precision(precision)

    # ---- lifecycle
    def close(self):
        if getattr(self, "h", None):
            self.lib.knc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, what):
        _raise(self.lib, self.h, st, what)

    # ---- configuration
    def set_model(self, model):
        mp = model.to_c() if hasattr(model, "to_c") else model
        self._check(self.lib.knc_set_model(self.h, C.byref(mp)), "set_model")

    def set_host_model(self, fn):
        """fn(r, theta, t) -> ([u_r, u_theta, rho, p], scalar): the slow path."""
        def cb(r, q, t, out, s, _user):
            any_prim, scalar = fn(r, q, t)
            for k in range(4):
                out[k] = float(any_prim[k])
            s[0] = float(scalar)
        self._host_cb = abi.PRIMITIVE_AT_FN(cb)
        self._check(self.lib.knc_set_host_model(self.h, self._host_cb, None), "set_host_model")

    def set_precision(self, precision: int):
        self._check(self.lib.knc_set_precision(self.h, precision), "set_precision")

    def set_c2p_guess(self, guess: int, weights=None):
        if weights is None:
            self._check(self.lib.knc_set_c2p_guess(self.h, guess, None, 0), "set_c2p_guess")
        else:
            w = np.ascontiguousarray(weights, dtype=np.float32)
            self._check(self.lib.knc_set_c2p_guess(self.h, guess, abi.fptr(w), w.size), "set_c2p_guess")

    def set_batched(self, graph: bool):
        self._check(self.lib.knc_set_batched(self.h, int(bool(graph))), "set_batched")

    def set_tuning(self, tile_rows: int = 8, fused: bool = False, ctas_per_sm: int = 0, tma: bool = False,
                   strip: bool = False, deferred: bool = False):
        """Launch shape: update tiles of tile_rows rows (tma: staged by tensor
        copies), warp strips of tile_rows rows (strip), or the fused stage."""
        form = abi.KNC_UPDATE_STRIP if strip else abi.KNC_UPDATE_TILE_TMA if tma else abi.KNC_UPDATE_TILE
        t = abi.Tuning(tile_rows=int(tile_rows), fused=int(bool(fused)), ctas_per_sm=int(ctas_per_sm),
                       update_form=form, recovery_form=int(bool(deferred)))
        self._check(self.lib.knc_set_tuning(self.h, C.byref(t)), "set_tuning")

    def tuning(self) -> dict:
        t = abi.Tuning()
        self._check(self.lib.knc_get_tuning(self.h, C.byref(t)), "get_tuning")
        return {"tile_rows": t.tile_rows, "fused": bool(t.fused), "ctas_per_sm": t.ctas_per_sm,
                "tma": t.update_form == abi.KNC_UPDATE_TILE_TMA, "strip": t.update_form == abi.KNC_UPDATE_STRIP,
                "deferred": t.recovery_form == abi.KNC_RECOVERY_DEFERRED}

    def autotune(self, reps: int = 5):
        """Time every launch shape on the live state, keep the fastest; returns
        (tuning dict, ms per stage)."""
        t = abi.Tuning()
        ms = C.c_double()
        self._check(self.lib.knc_autotune(self.h, int(reps), C.byref(t), C.byref(ms)), "autotune")
        return {"tile_rows": t.tile_rows, "fused": bool(t.fused), "ctas_per_sm": t.ctas_per_sm,
                "tma": t.update_form == abi.KNC_UPDATE_TILE_TMA, "strip": t.update_form == abi.KNC_UPDATE_STRIP,
                "deferred": t.recovery_form == abi.KNC_RECOVERY_DEFERRED}, ms.value

    def zone_updates(self) -> int:
        n = C.c_int64()
        self._check(self.lib.knc_zone_updates(self.h, C.byref(n)), "zone_updates")
        return n.value

    def set_mixed_w_split(self, w: float):
        self._check(self.lib.knc_set_mixed_w_split(self.h, float(w)), "set_mixed_w_split")

    def set_wait_test(self, polls: int = 0, unreachable: bool = False):
        """Bounded-wait test: the fused stage's grid barriers give up after
        `polls` polls (0: the default); `unreachable` makes the first barrier
        of each fused stage wait for one arrival more than the grid makes."""
        self._check(self.lib.knc_set_wait_test(self.h, int(polls), int(bool(unreachable))), "set_wait_test")

    # ---- state
    def init_from_model(self, time: float = 0.0):
        self._check(self.lib.knc_init_from_model(self.h, float(time)), "init_from_model")

    def set_block_shapes(self, first: int, nr, nq):
        """Uneven blocks: indexes first, first+1, ... get (nr[k], nq[k]) zones."""
        nr = np.ascontiguousarray(nr, dtype=np.int32)
        nq = np.ascontiguousarray(nq, dtype=np.int32)
        if nr.shape != nq.shape or nr.ndim != 1:
            raise ValueError("nr and nq must be 1-d arrays of the same length")
        i32 = C.POINTER(C.c_int32)
        self._check(self.lib.knc_set_block_shapes(self.h, int(first), nr.size, nr.ctypes.data_as(i32),
                                                  nq.ctypes.data_as(i32)), "set_block_shapes")

    def shape_of(self, index: int):
        nr = C.c_int64()
        nq = C.c_int64()
        self._check(self.lib.knc_block_shape_of(self.h, int(index), C.byref(nr), C.byref(nq)), "shape_of")
        return nr.value, nq.value

    def add_block(self, index: int, cons, scalar):
        cons = np.ascontiguousarray(cons, dtype=np.float64)
        scalar = np.ascontiguousarray(scalar, dtype=np.float64)
        nr, nq = self.shape_of(index)
        if cons.shape != (nr, nq, 4) or scalar.shape != (nr, nq):
            raise ValueError(f"block arrays must be ({nr}, {nq}, 4) and ({nr}, {nq})")
        self._check(self.lib.knc_add_block(self.h, int(index), abi.dptr(cons), abi.dptr(scalar)), "add_block")

    def remove_block(self, index: int):
        self._check(self.lib.knc_remove_block(self.h, int(index)), "remove_block")

    def block_indexes(self):
        n = C.c_int32()
        self.lib.knc_num_blocks(self.h, C.byref(n))
        out = (C.c_int32 * max(n.value, 1))()
        self._check(self.lib.knc_block_indexes(self.h, out, n.value), "block_indexes")
        return [out[k] for k in range(n.value)]

    def get_block(self, index: int):
        nr, nq = self.shape_of(index)
        cons = np.empty((nr, nq, 4))
        scalar = np.empty((nr, nq))
        self._check(self.lib.knc_get_block(self.h, int(index), abi.dptr(cons), abi.dptr(scalar)), "get_block")
        return cons, scalar

    def state(self):
        return {i: self.get_block(i) for i in self.block_indexes()}

    def set_state(self, cons, scalar):
        self._check(self.lib.knc_set_state(self.h, abi.dptr(cons), abi.dptr(scalar)), "set_state")

    def get_state(self, cons, scalar):
        self._check(self.lib.knc_get_state(self.h, abi.dptr(cons), abi.dptr(scalar)), "get_state")

    def get_products(self, index: int) -> dict:
        """BlockProducts::try_from_block_state (src/products.rs:43-66): radial
        and polar vertices, primitive [nr, nq, 4] in AnyPrimitive order
        (velocity_r, velocity_q, mass_density, gas_pressure), scalar [nr, nq]."""
        nr, nq = self.shape_of(index)
        rv, qv = np.empty(nr + 1), np.empty(nq + 1)
        prim, scal = np.empty((nr, nq, 4)), np.empty((nr, nq))
        self._check(self.lib.knc_get_products(self.h, int(index), abi.dptr(rv), abi.dptr(qv), abi.dptr(prim),
                                              abi.dptr(scal)), "get_products")
        return {"radial_vertices": rv, "polar_vertices": qv, "primitive": prim, "scalar": scal}

    def get_primitives(self, index: int):
        """(rho, u_r, u_theta, p, scalar concentration) of a block, [nr, nq, 5]."""
        out = np.empty(self.shape_of(index) + (5,))
        self._check(self.lib.knc_get_primitives(self.h, int(index), abi.dptr(out)), "get_primitives")
        return out

    def mark(self, slot: int):
        self._check(self.lib.knc_mark(self.h, slot), "mark")

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_double()
        self._check(self.lib.knc_elapsed_ms(self.h, a, b, C.byref(ms)), "elapsed_ms")
        return ms.value

    def set_profiling(self, on: bool):
        self._check(self.lib.knc_set_profiling(self.h, int(bool(on))), "set_profiling")

    def kernel_times(self):
        """{kind: (total ms, launches)} for ghost / c2p / update since profiling was enabled."""
        ms = (C.c_double * abi.KNC_KERNEL_KINDS)()
        n = (C.c_int64 * abi.KNC_KERNEL_KINDS)()
        self._check(self.lib.knc_kernel_times(self.h, ms, n), "kernel_times")
        names = ["ghost", "c2p", "update", "fused"]
        return {names[k]: (ms[k], n[k]) for k in range(abi.KNC_KERNEL_KINDS)}

    def set_time(self, t: float, num: int = 0, den: int = 1):
        self._check(self.lib.knc_set_time(self.h, float(t), int(num), int(den)), "set_time")

    def time(self):
        t = C.c_double()
        n = C.c_int64()
        d = C.c_int64()
        self.lib.knc_get_time(self.h, C.byref(t), C.byref(n), C.byref(d))
        return t.value, (n.value, d.value)

    # ---- hot path
    def time_step(self) -> float:
        dt = C.c_double()
        self._check(self.lib.knc_time_step(self.h, C.byref(dt)), "time_step")
        return dt.value

    def advance(self, fold: int = 1, dt=None):
        """scheme::advance; with dt given, that time step instead of time_step()."""
        if dt is None:
            self._check(self.lib.knc_advance(self.h, int(fold)), "advance")
        else:
            self._check(self.lib.knc_advance_dt(self.h, int(fold), float(dt)), "advance_dt")

    def advance_host(self, cons, scalar, fold: int = 1, cons_out=None, scalar_out=None):
        """scheme::advance on a host state (the whole-state arrays of
        set_state): uploads it, advances `fold` steps, writes the new state to
        cons_out / scalar_out (default: in place). Page-locked arrays
        (PinnedArray) let the copies run beside the stages."""
        co = cons if cons_out is None else cons_out
        so = scalar if scalar_out is None else scalar_out
        self._check(self.lib.knc_advance_host(self.h, abi.dptr(cons), abi.dptr(scalar), abi.dptr(co), abi.dptr(so),
                                              int(fold)), "advance_host")

    def try_advance(self, fold: int = 1) -> int:
        return self.lib.knc_advance(self.h, int(fold))

    def last_error(self) -> abi.Error:
        e = abi.Error()
        self.lib.knc_last_error(self.h, C.byref(e))
        return e

    def synchronize(self):
        self._check(self.lib.knc_synchronize(self.h), "synchronize")

    # ---- statistics
    def c2p_stats(self):
        z, a, b, f = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.lib.knc_c2p_stats(self.h, C.byref(z), C.byref(a), C.byref(b), C.byref(f)), "c2p_stats")
        return dict(zones=z.value, iters_fp64=a.value, iters_fp32=b.value, fallbacks=f.value)

    def reset_c2p_stats(self):
        self._check(self.lib.knc_reset_c2p_stats(self.h), "reset_c2p_stats")

    def launch_count(self) -> int:
        n = C.c_int64()
        self.lib.knc_launch_count(self.h, C.byref(n))
        return n.value


class PinnedArray:
    """A numpy view of page-locked host memory from knc_host_alloc."""

    def __init__(self, shape, dtype=np.float64):
        self.lib = abi.load()
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        st = self.lib.knc_host_alloc(n, C.byref(p))
        if st != abi.KNC_OK:
            raise abi.KncError(st, "knc_host_alloc failed")
        self.ptr = p
        buf = (C.c_char * n).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            self.lib.knc_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def measure_fp64_peak() -> float:
    lib = abi.load()
    g = C.c_double()
    st = lib.knc_measure_fp64_peak(C.byref(g))
    if st != abi.KNC_OK:
        raise abi.KncError(st, "knc_measure_fp64_peak failed")
    return g.value


def build_solver(workload, precision=abi.KNC_PRECISION_FP64):
    """Solver for a knc.workloads.Workload with its model set and initial data."""
    s = Solver(workload.hydro, workload.mesh, precision=precision)
    workload.apply_shapes(s)
    s.set_model(workload.model)
    s.init_from_model(0.0)
    return s
