"""The oracle against its committed golden vectors (tests/golden/golden.npz,
made by tests/golden/make_golden.py), and the GPU library against the same
small-grid run."""
import numpy as np
import pytest

import knc_oracle as ko
from golden.make_golden import small_grid
from knc import config

G = np.load(__file__.replace("test_golden.py", "golden/golden.npz"))
# bitwise on the machine that made them; libm may differ in the last bit on
# another architecture, so the comparison allows a few ulps
RTOL = 1e-13


def _close(a, b, rtol=RTOL):
    scale = np.maximum(np.abs(b), 1e-300)
    return np.all(np.abs(a - b) <= rtol * scale + 1e-300)


@pytest.mark.parametrize("name,riemann", [("hlle", "HLLE"), ("hllc", "HLLC")])
def test_point_physics_golden(oracle_lib, name, riemann):
    hp = config.RelativisticHydro(4 / 3, 1.5, 0.4, "RK2", riemann).to_c()
    prims = G["prims"]
    n = len(prims)
    cons = np.array([ko.prim_to_cons(hp, p) for p in prims])
    assert _close(cons, G[f"{name}_cons"])
    rec = np.array([ko.cons_to_prim(hp, u)[1] for u in cons])
    assert _close(rec, G[f"{name}_rec"], 1e-10)
    its = np.array([ko.cons_to_prim(hp, u)[2] for u in cons])
    assert np.array_equal(its, G[f"{name}_iters"])
    fl = np.array([[ko.riemann(hp, prims[k], prims[(k + 1) % n], 0.2, 0.7, ax) for ax in (0, 1)]
                   for k in range(n)])
    ref = G[f"{name}_flux"]
    assert np.all(np.abs(fl - ref) <= 1e-12 * np.abs(ref).max(axis=-1, keepdims=True))


def test_grid_golden(oracle_lib):
    hydro, mesh, model = small_grid()
    o = ko.Oracle(hydro, mesh, threads=2)
    o.set_model(model)
    o.init_from_model(0.0)
    idx = o.block_indexes()
    assert idx == list(G["grid_blocks"])
    assert _close(np.stack([o.get_block(i)[0] for i in idx]), G["grid_init"])
    o.advance(5)
    assert _close(np.stack([o.get_block(i)[0] for i in idx]), G["grid_cons"], 1e-12)
    t, (num, den) = o.time()
    assert t == G["grid_time"][0] and (num, den) == (G["grid_time"][1], G["grid_time"][2])


@pytest.mark.gpu
def test_gpu_grid_golden():
    import knc
    hydro, mesh, model = small_grid()
    s = knc.Solver(hydro, mesh)
    s.set_model(model)
    s.init_from_model(0.0)
    idx = s.block_indexes()
    init = np.stack([s.get_block(i)[0] for i in idx])
    assert _close(init, G["grid_init"])
    s.advance(5)
    cons = np.stack([s.get_block(i)[0] for i in idx])
    scale = np.abs(G["grid_cons"]).max(axis=(0, 1, 2))
    assert np.all(np.abs(cons - G["grid_cons"]).max(axis=(0, 1, 2)) <= 1e-12 * scale)
