"""Parity at the benchmarked size: the 4096 x 1024 wind (64 blocks of
64 x 1024) and the Newtonian sphere on the same grid, GPU against the CPU
oracle.

The other parity tests run grids of at most 64 x 128 blocks; these run the
bench's own workload for a few steps (the oracle takes about a second per
RK2 step on it with all host threads):
  - FP64 wind, 2 RK2 steps: bitwise equal (the FP64 stage computes every
    expression in the oracle's order without FMA contraction);
  - FP64 Newtonian sphere, HLLC, one adaptive-dt step: bitwise equal, time
    step included;
  - mixed wind, 2 RK2 steps: density L1 against the oracle below 1e-6.
"""
import os

import numpy as np
import pytest

from helpers import make_pair, zone_relative_errors

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 8


def _l1_comoving_density(g, o):
    num = den = 0.0
    for i in o.block_indexes():
        a = g.get_primitives(i)[..., 0]
        b = o.get_primitives(i)[..., 0]
        num += float(np.abs(a - b).sum())
        den += float(np.abs(b).sum())
    return num / den


def test_wind_large_two_steps_bitwise():
    from knc import workloads
    w = workloads.wind_large()
    assert w.zones == 4096 * 1024
    g, o = make_pair(w, threads=THREADS)
    g.advance(2)
    o.advance(2)
    assert max(zone_relative_errors(g.state(), o.state())) == 0.0
    assert g.time() == o.time()


def test_sphere_large_hllc_adaptive_step_bitwise():
    from knc import workloads
    w = workloads.sphere_large(riemann="HLLC")
    w.hydro.adaptive_time_step = True
    g, o = make_pair(w, threads=THREADS)
    assert g.time_step() == o.time_step()
    g.advance(1)
    o.advance(1)
    assert max(zone_relative_errors(g.state(), o.state())) == 0.0
    assert g.time() == o.time()


def test_wind_large_mixed_density_l1():
    from knc import abi, workloads
    w = workloads.wind_large()
    g, o = make_pair(w, threads=THREADS)
    g.set_precision(abi.KNC_PRECISION_MIXED)
    g.set_batched(True)
    g.advance(2)
    o.advance(2)
    l1 = _l1_comoving_density(g, o)
    print("wind 4096x1024 mixed vs oracle, 2 RK2 steps: density L1", l1)
    assert l1 <= 1e-6
