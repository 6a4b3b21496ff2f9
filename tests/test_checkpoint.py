"""CBOR checkpoints in the reference's App layout (src/app.rs:181-186,
src/state.rs:27-43, src/io.rs:24-35): codec round trips, the document shape,
and a restart that continues exactly like an uninterrupted run."""
import struct

import numpy as np
import pytest

from knc import checkpoint as ck
from knc import config, workloads


def test_cbor_scalars_shortest_float_width():
    assert ck.dumps(0.0) == b"\xf9\x00\x00"
    assert ck.dumps(1.5) == b"\xf9\x3e\x00"
    assert ck.dumps(1e-13)[0] == 0xFB
    assert ck.dumps(0.1)[0] == 0xFB
    assert ck.dumps(100000.5)[0] == 0xFA         # exact in f32, beyond f16
    for v in [0, 1, 23, 24, 255, 256, 65535, 65536, 2 ** 40, -1, -25, "RK2", None, True, False]:
        assert ck.loads(ck.dumps(v)) == v


def test_cbor_structures():
    doc = {"a": [1, 2.5, "x"], (3, 0): {"v": 1}, "b": None, "arr": ck.F64Array(np.arange(6.0).reshape(3, 2))}
    back = ck.loads(ck.dumps(doc))
    assert back["a"] == [1, 2.5, "x"] and back[(3, 0)] == {"v": 1} and back["b"] is None
    assert np.array_equal(back["arr"], np.arange(6.0).reshape(3, 2))


def test_app_document_shape():
    w = workloads.wind_small()
    blocks = {0: (np.ones((2, 3, 4)), np.zeros((2, 3)))}
    ctl = config.Control(start_time=0.0, final_time=1.0, checkpoint_interval=0.1, fold=10)
    doc = ck.loads(ck.dumps(ck.app_document(blocks, 0.5, (7, 2), w.hydro, "wind", {"rho0": 1.0}, w.mesh, ctl)))
    assert list(doc) == ["state", "tasks", "config", "version"]
    st = doc["state"]["Relativistic"]
    assert list(st) == ["time", "iteration", "solution"]
    assert st["iteration"] == [7, 2]
    bs = st["solution"][(0, 0)]
    assert bs["conserved"]["v"] == 1 and bs["conserved"]["dim"] == [2, 3]
    assert bs["conserved"]["data"].shape == (6, 4)
    assert doc["config"]["hydro"]["relativistic"]["runge_kutta_order"] == "RK2"
    assert list(doc["tasks"]) == ["write_checkpoint", "write_products", "iteration_message", "report_progress"]
    assert list(doc["config"]["mesh"])[:3] == ["reference_radius", "inner_radius", "outer_radius"]


def test_checkpoint_file_round_trip(tmp_path, oracle_lib):
    import knc_oracle
    w = workloads.wind_small()
    o = knc_oracle.Oracle(w.hydro, w.mesh, threads=4)
    o.set_model(w.model)
    o.init_from_model(0.0)
    o.advance(3)
    ctl = config.Control(start_time=0.0, final_time=1e-9, checkpoint_interval=1e-10, fold=3)
    t, it = o.time()
    path = tmp_path / "chkpt.0000.cbor"
    path.write_bytes(ck.dumps(ck.app_document(o.state(), t, it, w.hydro, "wind", {"rho0": 1.0, "ur": 1.0},
                                              w.mesh, ctl)))
    c = ck.read_checkpoint(path)
    assert c.time == t and c.iteration == it and c.kind == "Relativistic"
    for i, (cons, scal) in o.state().items():
        assert np.array_equal(c.blocks[i][0], cons) and np.array_equal(c.blocks[i][1], scal)
    assert c.mesh == w.mesh and c.hydro == w.hydro and c.control == ctl
    assert c.model_name == "wind" and c.model_params["ur"] == 1.0


@pytest.mark.gpu
def test_restart_continues_exactly(tmp_path):
    import knc
    w = workloads.wind_small()
    ctl = config.Control(start_time=0.0, final_time=1e-9, checkpoint_interval=1e-10, fold=3)
    a = knc.build_solver(w)
    a.advance(4)
    path = tmp_path / "chkpt.cbor"
    ck.write_checkpoint(path, a, w.hydro, "wind", {}, w.mesh, ctl)
    a.advance(4)
    b = knc.Solver(w.hydro, w.mesh)
    b.set_model(w.model)
    ck.read_checkpoint(path).restore(b)
    b.advance(4)
    assert a.time() == b.time()
    sa, sb = a.state(), b.state()
    for i in sa:
        assert np.array_equal(sa[i][0], sb[i][0]) and np.array_equal(sa[i][1], sb[i][1])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["wind_small", "uneven_small"])
def test_restart_across_implementations(tmp_path, oracle_lib, name):
    """A checkpoint the GPU solver writes restarts the oracle, and one the
    oracle writes restarts the GPU solver; every continuation equals the
    uninterrupted oracle run bit for bit. uneven_small: RK3 on blocks of
    uneven shape with both excision surfaces moving, so the restart also
    carries the block set and the time the excision radii follow."""
    import knc
    import knc_oracle
    from helpers import make_pair
    w = workloads.WORKLOADS[name]()
    ctl = config.Control(start_time=0.0, final_time=1e-9, checkpoint_interval=1e-10, fold=3)
    g, o = make_pair(w)
    g.advance(4)
    o.advance(4)
    from_gpu = tmp_path / "from_gpu.cbor"
    ck.write_checkpoint(from_gpu, g, w.hydro, "wind", {}, w.mesh, ctl)
    o2 = knc_oracle.Oracle(w.hydro, w.mesh, threads=8)
    w.apply_shapes(o2)
    o2.set_model(w.model)
    ck.read_checkpoint(from_gpu).restore(o2)
    from_oracle = tmp_path / "from_oracle.cbor"
    t, it = o.time()
    from_oracle.write_bytes(ck.dumps(ck.app_document(o.state(), t, it, w.hydro, "wind", {}, w.mesh, ctl)))
    g2 = knc.Solver(w.hydro, w.mesh)
    w.apply_shapes(g2)
    g2.set_model(w.model)
    ck.read_checkpoint(from_oracle).restore(g2)
    for s in (g, o, o2, g2):
        s.advance(4)
    ref = o.state()
    for s in (g, o2, g2):
        assert s.time() == o.time()
        st = s.state()
        assert sorted(st) == sorted(ref)
        for i in ref:
            assert np.array_equal(st[i][0], ref[i][0]) and np.array_equal(st[i][1], ref[i][1]), i


def test_products_file_round_trip(tmp_path, oracle_lib):
    """Products { time, blocks, config, version } with BlockProducts arrays
    (src/products.rs:17-36) written from the oracle's export and read back."""
    import knc_oracle
    w = workloads.wind_small()
    o = knc_oracle.Oracle(w.hydro, w.mesh, threads=4)
    o.set_model(w.model)
    o.init_from_model(0.0)
    o.advance(2)
    ctl = config.Control(start_time=0.0, final_time=1e-9, checkpoint_interval=1e-10, fold=2)
    blocks = {i: o.get_products(i) for i in o.block_indexes()}
    t, _ = o.time()
    doc = ck.products_document(blocks, t, w.hydro, "wind", {}, w.mesh, ctl)
    assert list(doc) == ["time", "blocks", "config", "version"]
    b0 = doc["blocks"][(0, 0)]
    assert list(b0) == ["radial_vertices", "polar_vertices", "primitive", "scalar"]
    assert b0["primitive"]["dim"] == [64, 128] and b0["radial_vertices"]["dim"] == [65]
    path = tmp_path / "prods.0000.cbor"
    path.write_bytes(ck.dumps(doc))
    back = ck.read_products(path)
    assert back["time"] == t
    for i, b in blocks.items():
        for k in ("radial_vertices", "polar_vertices", "primitive", "scalar"):
            assert np.array_equal(back["blocks"][i][k], b[k])
    # AnyPrimitive order: the wind's radial four-velocity is ~1, its density ~r^-2
    p = back["blocks"][0]["primitive"]
    assert abs(p[10, 10, 0] - 1.0) < 1e-3 and p[10, 10, 2] > p[10, 10, 3]
