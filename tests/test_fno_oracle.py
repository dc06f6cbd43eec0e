"""CPU checks of the surrogate's FP64 reference: the DFT-matrix form equals
the FFT definition, and its hand-written backward equals finite
differences of the loss."""
import numpy as np

from geoflac_gb300.fno import FnoConfig, init_params
from oracle import fno_ref

TINY = FnoConfig(H=16, W=32, C=8, m1=4, m2=4, layers=2, cin=16, P=16, cout=16)


def _data(cfg, B=2, seed=3):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((B, cfg.H, cfg.W, cfg.cin))
    t = rng.standard_normal((B, cfg.H, cfg.W, cfg.cout))
    return x, t


def test_dft_form_equals_fft_definition():
    p = init_params(TINY, seed=1)
    p = {k: v * (30.0 if k.startswith("R") else 1.0) for k, v in p.items()}  # make the spectral path matter
    x, _ = _data(TINY)
    a = fno_ref.forward_fft(TINY, p, x)
    b, _ = fno_ref.forward_dft(TINY, p, x)
    assert np.abs(a - b).max() <= 1e-10 * np.abs(a).max()


def test_backward_matches_finite_differences():
    p = {k: v.astype(np.float64) for k, v in init_params(TINY, seed=2).items()}
    p = {k: v * (30.0 if k.startswith("R") else 1.0) for k, v in p.items()}
    x, t = _data(TINY)
    out, rec = fno_ref.forward_dft(TINY, p, x)
    _, dout = fno_ref.mse_grad(out, t)
    g = fno_ref.backward_dft(TINY, p, rec, dout)
    rng = np.random.default_rng(7)
    eps = 1e-5
    for k in p:
        d = rng.standard_normal(p[k].shape)
        pp = dict(p)
        pm = dict(p)
        pp[k] = p[k] + eps * d
        pm[k] = p[k] - eps * d
        lp = fno_ref.mse_grad(fno_ref.forward_dft(TINY, pp, x)[0], t)[0]
        lm = fno_ref.mse_grad(fno_ref.forward_dft(TINY, pm, x)[0], t)[0]
        fd = (lp - lm) / (2 * eps)
        an = float((g[k] * d).sum())
        assert abs(fd - an) <= 1e-6 * max(abs(fd), 1e-12) + 1e-12, (k, fd, an)
