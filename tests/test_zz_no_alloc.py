"""knc_recover_primitives_noalloc: the primitive recovery for callers that
cannot let the library allocate device memory (their own allocator owns the
GPU, or their loop cannot take cudaMalloc's implicit synchronisation).

The caller owns the device buffers (here torch allocates them, standing in
for such a caller's pool). The output must equal knc_get_primitives', the
regular entry point, on two calls in a row (the fixed scratch keeps the
previous call's contents, so the second call checks that nothing leaks from
the first). This file sorts last so that a run stopping at its first failure
has already run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _call(lib, abi, hp, mp, index, d_cons, d_scal, d_prim):
    err = abi.Error()
    st = lib.knc_recover_primitives_noalloc(C.byref(hp), C.byref(mp), index, _ptr(d_cons), _ptr(d_scal),
                                            _ptr(d_prim), None, C.byref(err))
    return st, err


def test_noalloc_matches_get_primitives_twice():
    torch = pytest.importorskip("torch")
    import knc
    from knc import abi, workloads
    w = workloads.wind_small()
    s = knc.build_solver(w)
    s.advance(3)
    lib = abi.load()
    for index in (2, 0):   # two calls in a row, different blocks
        cons, scal = s.get_block(index)
        d_cons = torch.from_numpy(cons).cuda()
        d_scal = torch.from_numpy(scal).cuda()
        d_prim = torch.full((s.nr, s.nq, 5), float("nan"), dtype=torch.float64, device="cuda")
        st, err = _call(lib, abi, s.hp, s.mp, index, d_cons, d_scal, d_prim)
        assert st == abi.KNC_OK, err.message.decode()
        torch.cuda.synchronize()
        got = d_prim.cpu().numpy()
        ref = s.get_primitives(index)
        # the same arithmetic as knc_get_primitives: equal bit for bit (the
        # NaN fill of d_prim catches zones the call did not write)
        assert np.array_equal(got, ref), np.abs(got - ref).max(axis=(0, 1))


def test_noalloc_rejects_blocks_beyond_the_scratch():
    torch = pytest.importorskip("torch")
    from knc import abi, config
    lib = abi.load()
    hp = config.RelativisticHydro(4 / 3, 1.5, 0.4, "RK2", "HLLE").to_c()
    mesh = config.Mesh(reference_radius=1.0, inner_radius=1.0, outer_radius=10.0, inner_excision_speed=0.0,
                       outer_excision_speed=0.0, num_polar_zones=4096, block_size=64, num_radial_zones=100)
    assert 64 * 4096 > abi.KNC_NOALLOC_MAX_ZONES
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    st, err = _call(lib, abi, hp, mesh.to_c(), 0, d, d, d)
    assert st == abi.KNC_ERR_INVALID_ARGUMENT
    assert b"KNC_NOALLOC_MAX_ZONES" in err.message


def test_noalloc_reports_the_failing_zone():
    torch = pytest.importorskip("torch")
    import knc
    from knc import abi, workloads
    w = workloads.wind_small()
    s = knc.build_solver(w)
    cons, scal = s.get_block(1)
    cons = cons.copy()
    cons[5, 7, 0] = -1.0
    lib = abi.load()
    d_prim = torch.empty((s.nr, s.nq, 5), dtype=torch.float64, device="cuda")
    st, err = _call(lib, abi, s.hp, s.mp, 1, torch.from_numpy(cons).cuda(), torch.from_numpy(scal).cuda(), d_prim)
    assert st == abi.KNC_ERR_HYDRO
    assert (err.kind, err.block, err.i, err.j) == (abi.KNC_HYDRO_NEGATIVE_DENSITY, 1, 5, 7)
