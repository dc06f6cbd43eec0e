"""The surrogate's tensor-core forward and backward against the FP64
reference (oracle/fno_ref.py), through the library's kernels.

Tolerances (BF16 operands, FP32 accumulation): forward output within 3e-2
and every parameter gradient within 5e-2 relative L2 of the reference; a
few Adam steps on one batch must lower the loss."""
import numpy as np
import pytest

from geoflac_gb300.fno import Fno, FnoConfig, init_params
from oracle import fno_ref

pytestmark = pytest.mark.gpu

TINY = FnoConfig(H=16, W=32, C=16, m1=4, m2=4, layers=2, cin=16, P=32, cout=16)


def _bf16_round(a):
    torch = pytest.importorskip("torch")
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(torch.bfloat16).float().numpy()


def _setup(seed=5, B=8, rscale=30.0):
    torch = pytest.importorskip("torch")
    p = init_params(TINY, seed=seed)
    p = {k: (v * (rscale if k.startswith("R") else 1.0)).astype(np.float32) for k, v in p.items()}
    rng = np.random.default_rng(seed)
    x = _bf16_round(rng.standard_normal((B, TINY.H, TINY.W, TINY.cin)))
    t = rng.standard_normal((B, TINY.H, TINY.W, TINY.cout)).astype(np.float32)
    net = Fno(TINY, params=p)
    xd = torch.from_numpy(x).cuda().to(torch.bfloat16)
    return net, p, x, t, xd


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


def test_forward_matches_fft_definition():
    torch = pytest.importorskip("torch")
    net, p, x, _, xd = _setup()
    out = net.forward(xd).cpu().numpy()
    ref = fno_ref.forward_fft(TINY, {k: _bf16_round(v) if not k.endswith("_b") and not k[1:].isdigit()
                                     else v for k, v in p.items()}, x)
    assert _rel(out, ref) <= 3e-2, _rel(out, ref)


def test_gradients_match_fp64_reference():
    torch = pytest.importorskip("torch")
    net, p, x, t, xd = _setup()
    out = net.forward(xd, train=True)
    td = torch.from_numpy(t).cuda()
    loss, dout = net.loss_grad(out, td)
    g = net.backward(dout)
    torch.cuda.synchronize()
    out_ref, rec = fno_ref.forward_dft(TINY, p, x)
    dout_ref = dout.float().cpu().numpy().astype(np.float64)
    gref = fno_ref.backward_dft(TINY, p, rec, dout_ref)
    errs = {k: _rel(g[k].cpu().numpy().reshape(gref[k].shape), gref[k]) for k in gref}
    assert max(errs.values()) <= 5e-2, errs
    assert abs(loss.item() - fno_ref.mse_grad(out_ref, t)[0]) <= 5e-2 * fno_ref.mse_grad(out_ref, t)[0]


def test_adam_steps_lower_the_loss():
    """40 Adam steps fitting the output of another (teacher) network."""
    torch = pytest.importorskip("torch")
    net, p, x, _, xd = _setup(rscale=1.0)
    teacher = {k: v.astype(np.float64) * (30.0 if k.startswith("R") else 1.0)
               for k, v in init_params(TINY, seed=11).items()}
    t = fno_ref.forward_fft(TINY, teacher, x).astype(np.float32)
    td = torch.from_numpy(t).cuda()
    losses = []
    for _ in range(40):
        out = net.forward(xd, train=True)
        loss, dout = net.loss_grad(out, td)
        net.backward(dout)
        net.adam(lr=5e-3)
        losses.append(loss.item())
    assert losses[-1] < 0.1 * losses[0], losses
