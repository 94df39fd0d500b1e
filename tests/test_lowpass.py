"""The rate filter of the autograd loss (flybrain.autograd.lowpass_rates) against the recursion it
states, r_t = a r_{t-1} + (1 - a) s_t / dt, run step by step in float64 -- across several of its
internal blocks -- and its gradient against the recursion's transpose."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("dt,tau,T", [(0.1, 20.0, 5000), (0.5, 5.0, 700), (1.0, 20.0, 3)])
def test_lowpass_matches_recursion(dt, tau, T):
    from flybrain.autograd import lowpass_rates
    rng = np.random.default_rng(T)
    s = (rng.random((T, 9)) < 0.05).astype(np.float64) * rng.uniform(0.2, 1.0, (T, 9))
    a = np.exp(-dt / tau)
    c = (1 - a) / (dt / 1000)
    r, ref = np.zeros(9), np.zeros((T, 9))
    for t in range(T):
        r = a * r + c * s[t]
        ref[t] = r
    got = lowpass_rates(torch.tensor(s), dt, tau).numpy()
    np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-9 * max(1.0, ref.max()))
    # dL/ds_k for L = sum_t w_t r_t is c * sum_{t>=k} a^(t-k) w_t
    w = rng.normal(0, 1, (T, 9))
    x = torch.tensor(s, requires_grad=True)
    (lowpass_rates(x, dt, tau) * torch.tensor(w)).sum().backward()
    g, acc = np.zeros((T, 9)), np.zeros(9)
    for t in range(T - 1, -1, -1):
        acc = a * acc + w[t]
        g[t] = c * acc
    np.testing.assert_allclose(x.grad.numpy(), g, rtol=1e-9, atol=1e-9 * np.abs(g).max())
