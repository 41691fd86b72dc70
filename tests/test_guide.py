"""The path-guiding network: the FP64 oracle's analytic gradient (CPU), and
the device's FP16 tensor-core forward, gradient and Adam training against it
(GPU, through the C ABI)."""
import numpy as np
import pytest

from common import are


def random_params(n, seed, scale=1.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.zeros(n, np.float32)
    # He-like scales per layer (offsets as oracle/orc_guide.c)
    sizes = [(64, 256), (64,), (64, 64), (64,), (64, 64), (64,), (64, 64), (64,), (48, 64), (48,)]
    off = 0
    for sh in sizes:
        k = int(np.prod(sh))
        fan = sh[1] if len(sh) == 2 else 64
        p[off:off + k] = rng.uniform(-1, 1, k) * np.sqrt(6.0 / fan) * scale * (0.3 if len(sh) == 1 else 1.0)
        off += k
    assert off == n
    return p


def random_samples(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    s = np.zeros((n, 13), np.float32)
    s[:, 0:3] = rng.uniform(-1, 1, (n, 3))
    nrm = rng.normal(size=(n, 3))
    s[:, 3:6] = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3))
    s[:, 6:9] = wo / np.linalg.norm(wo, axis=1, keepdims=True)
    w = rng.normal(size=(n, 3))
    s[:, 9:12] = w / np.linalg.norm(w, axis=1, keepdims=True)
    s[:, 12] = rng.exponential(1.0, n)
    return s


def test_oracle_gradient_matches_finite_differences(oracle):
    n_p = oracle.lib.orc_guide_num_params()
    p = random_params(n_p, 1, scale=0.5)
    s = random_samples(8, 2)
    loss, g = oracle.guide_loss_grad(p, s)
    rng = np.random.Generator(np.random.PCG64(3))
    # a few hundred coordinates across all layers, central differences in FP64 via float32 params
    idx = np.concatenate([rng.choice(16384, 60, replace=False), 16384 + rng.choice(64, 10, replace=False),
                          16448 + rng.choice(4096, 40, replace=False), 28928 + rng.choice(40 * 64, 60, replace=False),
                          32000 + rng.choice(40, 20, replace=False)])
    for i in idx:
        h = max(1e-3 * abs(float(p[i])), 1e-3)
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        hh = (float(pp[i]) - float(pm[i])) / 2
        fd = (oracle.guide_loss_grad(pp, s)[0] - oracle.guide_loss_grad(pm, s)[0]) / (2 * hh)
        assert abs(fd - g[i]) <= 2e-3 * max(1.0, abs(g[i])) + 1e-6, (i, fd, g[i])
    assert np.all(g[28928 + 40 * 64:32000] == 0) and np.all(g[32040:] == 0)  # unused outputs


def test_oracle_mixture_is_normalised(oracle):
    rng = np.random.Generator(np.random.PCG64(5))
    o = rng.normal(size=48) * 2
    # integrate the mixture pdf over the sphere by a fine quadrature
    th = (np.arange(400) + 0.5) / 400 * np.pi
    ph = (np.arange(800) + 0.5) / 800 * 2 * np.pi
    tot = 0.0
    for t in th:
        for p in ph[::8]:
            w = np.array([np.sin(t) * np.cos(p), np.sin(t) * np.sin(p), np.cos(t)])
            tot += oracle.guide_pdf(o, w) * np.sin(t)
    tot *= (np.pi / 400) * (2 * np.pi / 100)
    assert abs(tot - 1.0) < 0.02, tot


@pytest.mark.gpu
def test_device_forward_matches_oracle(gpu_lib, oracle):
    g = are.Guide(seed=7)
    p = random_params(g.n_params, 11)
    g.params = p
    s = random_samples(4099, 12)  # not a multiple of 16
    out = g.forward(s[:, :9])
    ref = oracle.guide_forward(p, s[:, :9])
    err = np.abs(out[:, :40] - ref[:, :40])
    assert np.all(np.isfinite(out))
    print(f"\n[guide forward] max abs error {np.max(err):.3g}, mean {np.mean(err):.3g}, "
          f"output scale {np.max(np.abs(ref)):.3g}")
    # FP16 inputs and weights, FP32 accumulation.  Measured on GB300: max 0.0035 on outputs of scale 5.3
    # (6.6e-4 relative), mean 4.4e-4; the bounds are about ten times those
    assert np.max(err) < 0.007 * max(1.0, np.max(np.abs(ref))), np.max(err)
    assert np.mean(err) < 0.0045, np.mean(err)


@pytest.mark.gpu
def test_device_gradient_matches_oracle(gpu_lib, oracle):
    g = are.Guide(seed=7)
    p = random_params(g.n_params, 21, scale=0.7)
    g.params = p
    s = random_samples(1000, 22)
    loss, grad = g.gradient(s)
    rloss, rgrad = oracle.guide_loss_grad(p, s)
    assert abs(loss - rloss) < 0.02 * abs(rloss) + 1e-3, (loss, rloss)
    cos = np.dot(grad, rgrad) / (np.linalg.norm(grad) * np.linalg.norm(rgrad))
    rel = np.linalg.norm(grad - rgrad) / np.linalg.norm(rgrad)
    assert cos > 0.995 and rel < 0.08, (cos, rel)
    # every layer separately (offsets as oracle/orc_guide.c)
    for a, b in [(0, 16384), (16384, 16448), (16448, 20544), (28864, 28928), (28928, 32000), (32000, 32048)]:
        ga, ra = grad[a:b], rgrad[a:b]
        if np.linalg.norm(ra) > 0:
            assert np.linalg.norm(ga - ra) / np.linalg.norm(ra) < 0.15, (a, b)


@pytest.mark.gpu
def test_device_training_learns_a_direction_field(gpu_lib, oracle):
    """Incident radiance that comes from one direction per region of space:
    Adam steps on the device raise the mixture's density at the true
    directions by a large factor (what the trained network gains over the
    untrained one: a uniform-ish density of 1/(4 pi))."""
    rng = np.random.Generator(np.random.PCG64(31))
    g = are.Guide(seed=3)

    def batch(n):
        s = random_samples(n, int(rng.integers(1 << 30)))
        # target direction depends on the position's octant
        octant = (s[:, 0] > 0) * 1 + (s[:, 1] > 0) * 2 + (s[:, 2] > 0) * 4
        dirs = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [0.6, 0.8, 0],
                         [0, 0.6, -0.8]], np.float32)
        d = dirs[octant] + rng.normal(scale=0.15, size=(n, 3)).astype(np.float32)
        s[:, 9:12] = d / np.linalg.norm(d, axis=1, keepdims=True)
        s[:, 12] = 1.0
        return s, dirs[octant]

    test, truth = batch(2048)
    p0 = g.params
    before = np.mean([np.log(oracle.guide_pdf(o, w)) for o, w in zip(oracle.guide_forward(p0, test[:, :9]), truth)])
    losses = [g.train(batch(1 << 14)[0], lr=1e-2) for _ in range(150)]
    p1 = g.params
    after = np.mean([np.log(oracle.guide_pdf(o, w)) for o, w in zip(oracle.guide_forward(p1, test[:, :9]), truth)])
    assert losses[-1] < losses[0] - 1.0, (losses[0], losses[-1])
    assert after > before + 2.0, (before, after)  # density at the true direction up by > e^2


@pytest.mark.gpu
def test_device_mixture_density_matches_oracle(gpu_lib, oracle):
    """The packed mixture the renderer samples gives the oracle's density."""
    rng = np.random.Generator(np.random.PCG64(17))
    g = are.Guide(seed=9)
    p = g.params
    feat = rng.uniform(-1, 1, (300, 9)).astype(np.float32)
    mix = g.mixture(feat)
    raw = oracle.guide_forward(p, feat)
    w = rng.normal(size=(300, 3))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    for m, o, d in zip(mix, raw, w):
        mu, kappa = m[:32].reshape(8, 4)[:, :3], m[:32].reshape(8, 4)[:, 3]
        pi, nrm = m[32:].reshape(8, 2)[:, 0], m[32:].reshape(8, 2)[:, 1]
        assert abs(pi.sum() - 1) < 1e-5 and np.allclose(np.linalg.norm(mu, axis=1), 1, atol=1e-6)
        q = float(np.sum(pi * nrm * np.exp(kappa * (mu @ d - 1))))
        r = oracle.guide_pdf(o, d)
        assert abs(q - r) <= 0.03 * r + 1e-4, (q, r)


@pytest.mark.gpu
def test_bounded_wait_gives_up_and_the_next_call_succeeds(gpu_lib, oracle):
    """The tensor-core inference's waits are bounded: with the first MMA
    wait of each warpgroup allowed no polls, every block takes the give-up
    path (error bit 16, work in flight drained, tensor memory freed) and the
    call reports ARE_ERR_KERNEL_TIMEOUT; the context stays usable, so the next
    call with the default bound returns the right answer."""
    g = are.Guide(seed=11)
    rng = np.random.Generator(np.random.PCG64(5))
    feat = rng.uniform(-1, 1, (5000, 9)).astype(np.float32)
    g.set_wait_limit(0)
    with pytest.raises(are.AreError) as e:
        g.forward(feat)
    assert e.value.status == 5 and "16" in str(e.value)
    with pytest.raises(are.AreError) as e:  # the mixture path too
        g.mixture(feat)
    assert e.value.status == 5
    g.set_wait_limit(-1)
    out = g.forward(feat)
    ref = oracle.guide_forward(g.params, feat)
    assert np.abs(out[:, :40] - ref[:, :40]).max() < 0.05 * max(1.0, np.abs(ref).max())


@pytest.mark.gpu
def test_training_wait_gives_up_and_the_step_is_skipped(gpu_lib, oracle):
    """The training kernel's tensor-core waits are bounded the same way: with
    no polls allowed for the first MMA wait, are_guide_train reports
    ARE_ERR_KERNEL_TIMEOUT and the weights are unchanged (the step's gradients
    are flagged and Adam skips it); with the default bound the next step
    trains."""
    g = are.Guide(seed=13)
    s = random_samples(3000, 41)
    p0 = g.params
    g.set_wait_limit(0)
    with pytest.raises(are.AreError) as e:
        g.train(s, lr=1e-2)
    assert e.value.status == 5 and "16" in str(e.value)
    with pytest.raises(are.AreError) as e:  # the gradient alone as well
        g.gradient(s)
    assert e.value.status == 5
    assert np.array_equal(g.params, p0)
    g.set_wait_limit(-1)
    loss = g.train(s, lr=1e-2)
    assert np.isfinite(loss)
    assert not np.array_equal(g.params, p0)
    _, grad = g.gradient(s)
    _, rgrad = oracle.guide_loss_grad(g.params, s)
    assert np.dot(grad, rgrad) / (np.linalg.norm(grad) * np.linalg.norm(rgrad)) > 0.995
