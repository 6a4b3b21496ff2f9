"""The learned c2p guess: device forward/backward against the CPU reference,
training on the device, and what the trained network gains over the plain
guess (Newton iterations to the same 1e-12 residual)."""
import numpy as np
import pytest

import knc_oracle

pytestmark = pytest.mark.gpu


def test_device_gradients_match_cpu_reference():
    from knc import abi, learned
    rng = np.random.default_rng(3)
    w = learned.init_weights(3)
    w[abi.KNC_MLP_OFF_XMEAN:abi.KNC_MLP_OFF_XMEAN + 3] = 0.1
    w[abi.KNC_MLP_OFF_XSCALE:abi.KNC_MLP_OFF_XSCALE + 3] = 0.9
    x = rng.normal(size=(1000, 3)).astype(np.float32)
    y = rng.normal(size=1000).astype(np.float32)
    pd, ld, gd = learned.forward_backward(w, x, y)
    po, lo, go = knc_oracle.mlp_forward_backward(w, x, y, round_bf16=True)
    assert np.abs(pd - po).max() <= 1e-4 * max(1.0, np.abs(po).max())
    assert ld == pytest.approx(lo, rel=1e-4)
    for name, off, n in [("W1", 0, 192), ("b1", 192, 64), ("W2", 256, 4096), ("b2", 4352, 64),
                         ("W3", 4416, 64), ("b3", 4480, 1)]:
        scale = np.abs(go[off:off + n]).max()
        assert np.abs(gd[off:off + n] - go[off:off + n]).max() <= 1e-4 * scale, name


def test_training_reduces_loss(trained_mlp):
    w, loss = trained_mlp
    assert loss < 0.02, loss


def test_learned_guess_needs_fewer_iterations(trained_mlp):
    """Held-out pairs: Newton iterations to |f| < 1e-12 (D + tau) from the
    learned guess versus the plain guess, on the CPU reference Newton."""
    import knc
    from knc import learned
    w, _ = trained_mlp
    pairs = learned.generate_pairs(4.0 / 3.0, 3000, seed=99)
    x, y = learned.features(pairs)
    pred, _, _ = learned.forward_backward(w, x, y)
    hp = knc.RelativisticHydro(4.0 / 3.0, 1.5, 0.4, "RK2", "HLLE").to_c()
    it_plain, it_learn = [], []
    for k in range(len(pairs)):
        u = pairs[k, :4]
        guess = min(u[0] * np.exp(pred[k]), (4.0 / 3.0 - 1.0) * u[3])
        kind_p, prim_p, a = knc_oracle.cons_to_prim(hp, u, -1.0)
        kind_l, prim_l, b = knc_oracle.cons_to_prim(hp, u, guess)
        assert kind_p == kind_l
        # both stop at |f| < 1e-12 (D + tau); at Lorentz factor W that residual
        # fixes the velocity only to about W^2 1e-12 and p to 1e-12 (D + tau)
        w2 = 1.0 + prim_p[1] ** 2 + prim_p[2] ** 2
        assert np.allclose(prim_p[:3], prim_l[:3], rtol=1e-11 * w2 + 1e-12, atol=0.0)
        assert abs(prim_p[3] - prim_l[3]) <= 1e-11 * (u[0] + u[3])
        it_plain.append(a)
        it_learn.append(b)
    gain = np.mean(it_plain) - np.mean(it_learn)
    print(f"Newton iterations per zone: plain {np.mean(it_plain):.3f}  learned {np.mean(it_learn):.3f}")
    assert gain > 0.5, (np.mean(it_plain), np.mean(it_learn))


def test_fp64_path_with_learned_guess(trained_mlp):
    """The FP64 stage from the learned guess converges to the same residual:
    the state agrees with the plain-guess run to the recovery tolerance."""
    import knc
    from helpers import field_errors, make_pair
    from knc import abi, workloads
    w, _ = trained_mlp
    wl = workloads.jet_small()
    a, _ = make_pair(wl, gpu=True)
    b, _ = make_pair(wl, gpu=True)
    b.set_c2p_guess(abi.KNC_GUESS_MLP, w)
    a.reset_c2p_stats()
    b.reset_c2p_stats()
    a.advance(20)
    b.advance(20)
    # W = 100 in the nozzle: the 1e-12 residual fixes primitives to ~W^2 1e-12
    assert max(field_errors(a.state(), b.state())) <= 1e-7
    sa, sb = a.c2p_stats(), b.c2p_stats()
    ia, ib = sa["iters_fp64"] / sa["zones"], sb["iters_fp64"] / sb["zones"]
    print(f"FP64 path iterations per zone: plain {ia:.3f} learned {ib:.3f} fallbacks {sb['fallbacks']}")
    # the jet's gas is cold (p / rho = 1e-3), where the plain guess already
    # converges in about two iterations; the learned start must not cost more
    assert ib <= ia * 1.05
