"""CPU checks of the oracle parts that have no counterpart in the reference
(its FFT is an unused FFTW wrapper and it has no learned multiplier), pinned
instead against independent computations: the oracle's direct DFT against
numpy.fft, and its MLP forward pass and hand-written backward pass against a
numpy FP64 restatement and central finite differences. Plus the host-side
arithmetic the measurements rest on: algorithmic bytes of the headline
workload, and the multiplier family of the learned-multiplier training."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("dims", [[4, 6, 8], [8, 8, 8, 8], [2, 12, 6, 4], [32]])
@pytest.mark.parametrize("sign", [-1, 1])
def test_oracle_dft_matches_numpy(oracle, dims, sign):
    """sites in lexicographic order with the last extent fastest; sign -1 is
    the forward transform exp(-2 pi i k.x/L), both unnormalised"""
    rng = np.random.default_rng(3)
    V = int(np.prod(dims))
    data = rng.normal(size=(V, 3)) + 1j * rng.normal(size=(V, 3))
    got = oracle.fft(dims, data, sign)
    a = data.reshape(*dims, 3)
    axes = tuple(range(len(dims)))
    ref = np.fft.fftn(a, axes=axes) if sign < 0 else np.fft.ifftn(a, axes=axes) * V
    np.testing.assert_allclose(got, ref.reshape(V, 3), rtol=0, atol=1e-10 * V)


def np_mlp(x, p, w):
    """numpy FP64 restatement: params W1[w][3] b1[w] W2[w][w] b2[w] W3[w] b3"""
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + 3 * w].reshape(w, 3); o += 3 * w
    b1 = p[o:o + w]; o += w
    W2 = p[o:o + w * w].reshape(w, w); o += w * w
    b2 = p[o:o + w]; o += w
    W3 = p[o:o + w]; o += w
    b3 = p[o]
    h1 = np.tanh(np.asarray(x, dtype=np.float64) @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ W3 + b3


@pytest.mark.parametrize("width", [32, 64])
def test_oracle_mlp_forward_and_backward(oracle, width):
    rng = np.random.default_rng(width)
    n = 50
    npar = oracle.mlp_nparams(width)
    assert npar == width * width + 6 * width + 1
    params = (rng.normal(size=npar) * 0.3).astype(np.float32)
    x = rng.normal(size=(n, 3)).astype(np.float32)
    t = rng.normal(size=n).astype(np.float32)
    y = oracle.mlp_forward(x, params, width)
    np.testing.assert_allclose(y, np_mlp(x, params, width), rtol=1e-6, atol=1e-6)
    loss, grad = oracle.mlp_grad(x, t, params, width)

    def np_loss(p):
        return float(np.mean((np_mlp(x, p, width) - t.astype(np.float64)) ** 2))

    p64 = params.astype(np.float64)
    assert loss == pytest.approx(np_loss(p64), rel=1e-12)
    # central differences on a sample of parameters from every layer
    idx = np.unique(np.concatenate([rng.choice(npar, 60, replace=False), [0, 3 * width, npar - 1]]))
    h = 1e-5
    for i in idx:
        e = np.zeros(npar)
        e[i] = h
        fd = (np_loss(p64 + e) - np_loss(p64 - e)) / (2 * h)
        assert grad[i] == pytest.approx(fd, rel=1e-5, abs=1e-8), i


def test_headline_algorithmic_bytes():
    """SU(3) FP32 32^4: links 72 B, momenta 32 B (8 algebra reals) per link;
    the fused MD launch reads U and P and writes P (momentum step), then reads
    U and P and writes U_new (link update): 312 B per link"""
    sys.path.insert(0, ROOT)
    import bench

    _, Ub, Pb = bench.sizes([32] * 4, 4)
    links = 4 * 32 ** 4
    assert Ub == 72 * links and Pb == 32 * links
    assert (Ub + 2 * Pb) + (2 * Ub + Pb) == 312 * links == 1308622848


def test_multiplier_family():
    from mesh_gb300 import landau_learn as ll

    p2min, p2max = 0.0381, 16.0
    p2 = np.exp(np.linspace(np.log(p2min), np.log(p2max), 200))
    plain = ll.family_mult(0.08, 1.0, p2, p2min, p2max)
    np.testing.assert_allclose(plain, 0.08 * p2max / p2)
    damped = ll.family_mult(0.08, 0.35, p2, p2min, p2max)
    # the factor on the shortest wavelengths fades in from p2max/4 to p2max
    below = p2 <= p2max / 4
    np.testing.assert_allclose(damped[below], plain[below])
    assert damped[-1] == pytest.approx(0.35 * plain[-1])
    r = damped / plain
    assert np.all(np.diff(r) <= 1e-12)
    tab, lo, hi = ll.family_table(0.08, 0.35, p2min, p2max)
    assert tab.dtype == np.float32 and len(tab) == ll.TABLE_N
    assert lo < np.log(p2min) and hi > np.log(p2max)
    f = ll.features(np.array([-1.0, 0.0]), 6.2, 1e-7)
    np.testing.assert_allclose(f, [[-1.0, 1.0, 0.0], [0.0, 1.0, 0.0]], atol=1e-12)
