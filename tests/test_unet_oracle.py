"""The U-Net oracle (oracle/unet.py) checked on the CPU: its analytic
gradients against central finite differences of its own loss, with the bf16
rounding points switched off so that the loss is smooth in the parameters."""
import numpy as np
import pytest

from oracle import unet


@pytest.fixture
def smooth(monkeypatch):
    monkeypatch.setattr(unet, "bf16", lambda x: np.asarray(x, np.float32))


def _case(seed=3, n=32):
    rng = np.random.default_rng(seed)
    P = unet.init_params(seed)
    for k in P:
        if k.endswith(".b"):
            P[k] = rng.normal(0, 0.05, P[k].shape).astype(np.float32)
    P["out.w"] = (P["out.w"] * 10).astype(np.float32)
    r = rng.normal(0, 1, (n, n)).astype(np.float32)
    e = rng.normal(0, 1, (n, n)).astype(np.float32)
    return P, r, e


def test_gradients_match_finite_differences(smooth):
    P, r, e = _case()
    L0, G, _ = unet.loss_and_grads(P, r, e)
    assert np.isfinite(L0)
    rng = np.random.default_rng(11)
    checked = 0
    for name in ["enc0.w", "enc1.w", "enc3.w", "dec2.w", "dec0.w", "out.w", "enc2.b", "dec1.b", "out.b"]:
        flat = P[name].reshape(-1)
        g = G[name].reshape(-1)
        # the entries with the largest gradients: finite differences resolve them
        for idx in np.argsort(-np.abs(g))[:3]:
            h = 1e-3 * max(1.0, abs(float(flat[idx])))
            old = flat[idx]
            flat[idx] = old + h
            Lp = unet.loss_and_grads(P, r, e)[0]
            flat[idx] = old - h
            Lm = unet.loss_and_grads(P, r, e)[0]
            flat[idx] = old
            fd = (Lp - Lm) / (2 * h)
            assert abs(fd - g[idx]) <= 0.05 * abs(g[idx]) + 1e-6, (name, idx, fd, g[idx])
            checked += 1
    assert checked == 25  # out.b has a single entry


def test_forward_is_positively_homogeneous():
    # y(c r) = c y(r) up to the rounding of rms: the network's output scales
    # with its input, so a preconditioner built on it scales with the residual.
    P, r, _ = _case()
    y1, _ = unet.forward(P, r)
    y2, _ = unet.forward(P, 4.0 * r)
    np.testing.assert_allclose(y2, 4.0 * y1, rtol=1e-5, atol=1e-6 * float(np.abs(y1).max()))
