"""are_tonemap on the GPU: bytes identical to the reference's quantisation
(experiments/rt.cpp:384-386 gamma, src/texture.cpp:378-383 linear) as
restated by the oracle, for random values, values next to every byte step,
special values, unaligned and ragged buffers, host and device pointers."""
import numpy as np
import pytest
import torch

from common import are

pytestmark = pytest.mark.gpu


def step_neighbourhood(mode, gamma, oracle):
    """Floats within 8 ulps of every byte step of the oracle's map."""
    xs = np.linspace(0, 1, 1 << 16, dtype=np.float32)
    q = oracle.quantize(xs, mode, gamma).astype(np.int32)
    edges = np.nonzero(np.diff(q))[0]
    out = []
    for e in edges:
        lo, hi = xs[e], xs[e + 1]
        # bisect to the exact step in float bits
        a, b = lo.view(np.uint32).item(), hi.view(np.uint32).item()
        qa = oracle.quantize(np.array([lo]), mode, gamma)[0]
        while b - a > 1:
            m = (a + b) // 2
            if oracle.quantize(np.array([m], np.uint32).view(np.float32), mode, gamma)[0] > qa:
                b = m
            else:
                a = m
        out.append(np.arange(b - 8, b + 9, dtype=np.uint32).view(np.float32))
    return np.concatenate(out)


SPECIAL = np.array([0.0, -0.0, 1.0, -1e-30, 1e-45, 1 - 2 ** -24, 1 + 2 ** -23, 3e38, np.inf, -np.inf, np.nan,
                    -np.nan], np.float32)


@pytest.mark.parametrize("mode,gamma", [(are.TONEMAP_GAMMA, 2.2), (are.TONEMAP_GAMMA, 2.0), (are.TONEMAP_LINEAR, 1.0)])
def test_tonemap_bit_exact(gpu_lib, oracle, mode, gamma):
    rng = np.random.default_rng(11)
    v = np.concatenate([rng.uniform(-0.25, 1.25, 1_000_003).astype(np.float32), step_neighbourhood(mode, gamma, oracle),
                        SPECIAL])
    got = are.tonemap(v, mode, gamma)
    ref = oracle.quantize(v, mode, gamma)
    bad = np.nonzero(got != ref)[0]
    assert bad.size == 0, (bad[:5], v[bad[:5]], got[bad[:5]], ref[bad[:5]])


def test_tonemap_device_pointers_unaligned_and_ragged(gpu_lib, oracle):
    rng = np.random.default_rng(12)
    for n in (1, 3, 4, 5, 1023, 600 * 600 * 3):
        for off in (0, 1, 3):
            src = torch.from_numpy(rng.uniform(-0.1, 1.1, n + off).astype(np.float32)).cuda()
            dst = torch.zeros(n + 5, dtype=torch.uint8, device="cuda")
            are.tonemap_device(src.data_ptr() + 4 * off, n, dst.data_ptr() + off)
            torch.cuda.synchronize()
            got = dst.cpu().numpy()[off:off + n]
            ref = oracle.quantize(src.cpu().numpy()[off:], 0, 2.2)
            assert np.array_equal(got, ref), (n, off)
            assert not dst.cpu().numpy()[off + n:].any()  # nothing written past the end


def test_tonemap_empty_and_bad_arguments(gpu_lib):
    assert are.tonemap(np.zeros(0, np.float32)).size == 0
    with pytest.raises(are.AreError):
        are.tonemap(np.zeros(3, np.float32), mode=7)
    with pytest.raises(are.AreError):
        are.tonemap(np.zeros(3, np.float32), gamma=0.0)


def test_render_tonemap_write(gpu_lib, oracle, tmp_path):
    s, cam, par = are.build_config(are.CONFIG_CORNELL)
    par = dict(par, width=64, height=48, spp=8)
    sc = are.Scene(s)
    img, _, _ = sc.render(cam, par)
    rgb8 = are.tonemap(img)
    assert np.array_equal(rgb8, oracle.quantize(img, 0, 2.2))
    p = tmp_path / "cornell.ppm"
    are.write_ppm(p, rgb8)
    assert p.read_bytes()[:13] == b"P6\n64 48\n255\n"
    sc.close()


def test_cli_renders_the_same_image(gpu_lib, oracle, tmp_path):
    import subprocess

    cli = are.LIB_PATH.parent / "are_render"
    ppm, pfm = tmp_path / "c.ppm", tmp_path / "c.pfm"
    r = subprocess.run([str(cli), "--config", "cornell", "--width", "64", "--height", "48", "--spp", "8", "--seed", "5",
                        "--out", str(ppm), "--pfm", str(pfm)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    s, cam, par = are.build_config(are.CONFIG_CORNELL)
    sc = are.Scene(s)
    img, _, _ = sc.render(cam, dict(par, width=64, height=48, spp=8, seed=5))
    sc.close()
    data = pfm.read_bytes()
    header = b"PF\n64 48\n-1.0\n"
    body = np.frombuffer(data[len(header):], "<f4").reshape(48, 64, 3)[::-1]
    assert np.array_equal(body, img)  # same core, same seed: the same image
    assert ppm.read_bytes()[13:] == oracle.quantize(img, 0, 2.2).tobytes()
