"""Shared helpers of the test suite (pairing the GPU library with the oracle)."""
from __future__ import annotations

import numpy as np


def make_pair(workload, threads=8, gpu=True):
    import knc_oracle
    ora = knc_oracle.Oracle(workload.hydro, workload.mesh, threads=threads)
    workload.apply_shapes(ora)
    ora.set_model(workload.model)
    ora.init_from_model(0.0)
    g = None
    if gpu:
        import knc
        g = knc.Solver(workload.hydro, workload.mesh)
        workload.apply_shapes(g)
        g.set_model(workload.model)
        g.init_from_model(0.0)
    return g, ora


def field_errors(state_a, state_b, momentum_scale=False):
    """Max relative difference per conserved field over all blocks.

    Relative to the field's largest magnitude over the grid (so a field that
    is zero everywhere compares absolutely). With `momentum_scale` the polar
    momentum S_theta is measured against the largest momentum component
    (|S_r| or |S_theta|): in a radial flow S_theta is rounding noise around
    zero, and its own maximum is no scale for it."""
    keys = sorted(state_b)
    assert sorted(state_a) == keys, (sorted(state_a), keys)
    out = []
    for q in range(5):
        num = 0.0
        den = 0.0
        for k in keys:
            a = state_a[k][0][..., q] if q < 4 else state_a[k][1]
            b = state_b[k][0][..., q] if q < 4 else state_b[k][1]
            num = max(num, float(np.abs(a - b).max()))
            den = max(den, float(np.abs(b).max()))
            if momentum_scale and q == 2:
                den = max(den, float(np.abs(state_b[k][0][..., 1]).max()))
        out.append(num / den if den > 0 else num)
    return out


def zone_relative_errors(state_a, state_b):
    """Max over zones of |a - b| / |b| per conserved field (zones with b == 0
    compare absolutely)."""
    keys = sorted(state_b)
    out = []
    for q in range(5):
        worst = 0.0
        for k in keys:
            a = state_a[k][0][..., q] if q < 4 else state_a[k][1]
            b = state_b[k][0][..., q] if q < 4 else state_b[k][1]
            d = np.abs(a - b)
            scale = np.where(b != 0, np.abs(b), 1.0)
            worst = max(worst, float((d / scale).max()))
        out.append(worst)
    return out
