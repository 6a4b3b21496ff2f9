"""Learned initial pressure guess for the cons -> prim Newton recovery.

The network (3 -> 64 -> 64 -> 1, SiLU, BF16 weights, FP32 accumulation) is
trained on the GPU by the library's own forward / backward / Adam kernels, on
(conserved, primitive) pairs the solver itself produces: sampled from a live
state (`sample_pairs`) and generated with the solver's prim -> cons over a
range of Lorentz factors and temperatures (`generate_pairs`). The packed
weight layout is documented in include/knc.h.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


def init_weights(seed: int = 0) -> np.ndarray:
    """Xavier-uniform weights, zero biases, input normalisation unset (the
    trainer fills it from the data)."""
    rng = np.random.default_rng(seed)
    w = np.zeros(abi.KNC_MLP_NUM_PARAMS, dtype=np.float32)
    H = abi.KNC_MLP_HIDDEN

    def xavier(fan_in, fan_out, n):
        a = np.sqrt(6.0 / (fan_in + fan_out))
        return rng.uniform(-a, a, n).astype(np.float32)

    w[abi.KNC_MLP_OFF_W1:abi.KNC_MLP_OFF_W1 + 3 * H] = xavier(3, H, 3 * H)
    w[abi.KNC_MLP_OFF_W2:abi.KNC_MLP_OFF_W2 + H * H] = xavier(H, H, H * H)
    w[abi.KNC_MLP_OFF_W3:abi.KNC_MLP_OFF_W3 + H] = xavier(H, 1, H)
    return w


def generate_pairs(gamma: float, n: int, w_range=(1.0, 1000.0), t_range=(1e-6, 1e2), seed: int = 1) -> np.ndarray:
    """[n, 8] rows (D, S_r, S_q, tau, rho, u_r, u_q, p): Lorentz factor and
    p / rho log-uniform over the ranges, rho log-uniform over [1e-3, 1e3]."""
    lib = abi.load()
    out = np.empty((n, 8))
    st = lib.knc_generate_pairs(gamma, w_range[0], w_range[1], t_range[0], t_range[1], seed, n, abi.dptr(out))
    if st != abi.KNC_OK:
        raise abi.KncError(st, "knc_generate_pairs failed")
    return out


def sample_pairs(solver, stride: int = 1, capacity: int | None = None) -> np.ndarray:
    """Pairs from the live state of a Solver (every `stride`-th zone)."""
    if capacity is None:
        capacity = sum(solver.nr * solver.nq for _ in solver.block_indexes()) // stride + 1
    out = np.empty((capacity, 8))
    n = C.c_int64()
    st = solver.lib.knc_sample_pairs(solver.h, stride, abi.dptr(out), capacity, C.byref(n))
    if st != abi.KNC_OK:
        raise abi.KncError(st, "knc_sample_pairs failed")
    return out[:n.value]


def features(pairs: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Network inputs and target log(p / D) of pairs, as the device forms them:
    (log(tau / D), -log(1 - |S| / (D + tau)), log((tau (tau + 2D) - S^2) / D^2))."""
    p = np.asarray(pairs, dtype=np.float64)
    d, ss, tau = p[:, 0], p[:, 1] ** 2 + p[:, 2] ** 2, p[:, 3]
    e = tau + d
    a = tau * (tau + 2.0 * d) - ss
    df, ef = d.astype(np.float32), e.astype(np.float32)
    xs = np.sqrt(ss.astype(np.float32)) / ef
    x = np.stack([np.log(tau.astype(np.float32) / df),
                  np.log1p(xs) - np.log((a + d * d).astype(np.float32) / (ef * ef)),
                  np.log(a.astype(np.float32) / (df * df))], axis=1).astype(np.float32)
    y = np.log(p[:, 7] / p[:, 0]).astype(np.float32)
    return x, y


def set_normalisation(weights: np.ndarray, x: np.ndarray) -> np.ndarray:
    w = weights.copy()
    mean = x.mean(axis=0)
    std = np.maximum(x.std(axis=0), 1e-6)
    w[abi.KNC_MLP_OFF_XMEAN:abi.KNC_MLP_OFF_XMEAN + 3] = mean
    w[abi.KNC_MLP_OFF_XSCALE:abi.KNC_MLP_OFF_XSCALE + 3] = 1.0 / std
    return w


def train(pairs: np.ndarray, weights: np.ndarray | None = None, steps: int = 4000, batch: int = 8192,
          lr: float = 3e-3, seed: int = 1) -> tuple[np.ndarray, float]:
    """Train on the device; returns (weights, mean squared error of log p)."""
    lib = abi.load()
    pairs = np.ascontiguousarray(pairs, dtype=np.float64)
    w = np.ascontiguousarray(init_weights(seed) if weights is None else weights, dtype=np.float32).copy()
    tp = abi.MlpTrainParams(steps=steps, batch=batch, lr=lr, beta1=0.9, beta2=0.999, eps=1e-8, seed=seed)
    loss = C.c_float()
    st = lib.knc_mlp_train(abi.dptr(pairs), len(pairs), abi.fptr(w), C.byref(tp), C.byref(loss))
    if st != abi.KNC_OK:
        raise abi.KncError(st, "knc_mlp_train failed")
    return w, float(loss.value)


def forward_backward(weights: np.ndarray, x: np.ndarray, y: np.ndarray):
    """Device forward + backward on given rows: (pred, mean loss, grad)."""
    lib = abi.load()
    w = np.ascontiguousarray(weights, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    pred = np.empty(len(y), dtype=np.float32)
    grad = np.empty(abi.KNC_MLP_NUM_PARAMS, dtype=np.float32)
    loss = C.c_float()
    st = lib.knc_mlp_forward_backward(abi.fptr(w), abi.fptr(x), abi.fptr(y), len(y), abi.fptr(pred),
                                      C.byref(loss), abi.fptr(grad))
    if st != abi.KNC_OK:
        raise abi.KncError(st, "knc_mlp_forward_backward failed")
    return pred, float(loss.value), grad


def train_default(gamma: float = 4.0 / 3.0, n_pairs: int = 10_000_000, steps: int = 6000, seed: int = 1,
                  extra_pairs: np.ndarray | None = None):
    """The configuration used by the benchmark: 10M generated pairs over
    W in [1, 1000], p / rho in [1e-6, 1e2], plus any pairs sampled from runs."""
    pairs = generate_pairs(gamma, n_pairs, seed=seed)
    if extra_pairs is not None and len(extra_pairs):
        pairs = np.concatenate([pairs, extra_pairs])
    return train(pairs, steps=steps, seed=seed)
