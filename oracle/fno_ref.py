"""FP64 reference of the surrogate network (test infrastructure: it checks
the tensor-core kernels, it is never the thing run or shipped).

Two forwards:
  forward_fft  the Fourier neural operator by its definition (numpy rfft2,
               keep k1 < m1 and k1 >= H - m1, k2 < m2, complex mixing, irfft2);
  forward_dft  the same network written with the truncated DFT matrices the
               GPU kernels use, recording what the backward needs;
and backward_dft, the gradient of the mean-squared error with respect to
every parameter, written out by hand for the DFT form.  tests/ check
forward_dft against forward_fft and backward_dft against finite
differences, then the GPU forward and gradients against these.
"""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np
from scipy.special import erf


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_d(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def _complex_R(cfg, R):
    """R[(k2, q)][i][o][re|im] -> Rc[k2, q, i, o] complex"""
    Rc = R[..., 0].astype(np.float64) + 1j * R[..., 1].astype(np.float64)
    return Rc.reshape(cfg.m2, cfg.Q, cfg.C, cfg.C)


def forward_fft(cfg, p: Dict[str, np.ndarray], x: np.ndarray) -> np.ndarray:
    x = x.astype(np.float64)
    v = x @ p["lift_w"].astype(np.float64).T + p["lift_b"]
    B, H, W, _ = v.shape
    for l in range(cfg.layers):
        xh = np.fft.rfft2(v, axes=(1, 2))
        oh = np.zeros_like(xh)
        Rc = _complex_R(cfg, p[f"R{l}"])
        for q in range(cfg.Q):
            k1 = cfg.k1(q)
            # out[b, k2, o] = sum_i xh[b, k1, k2, i] R[k2, q, i, o]
            oh[:, k1, :cfg.m2, :] = np.einsum("bki,kio->bko", xh[:, k1, :cfg.m2, :], Rc[:, q])
        s = np.fft.irfft2(oh, s=(H, W), axes=(1, 2))
        z = v @ p[f"w{l}"].astype(np.float64).T + p[f"b{l}"] + s
        v = gelu(z) if l < cfg.layers - 1 else z
    h = gelu(v @ p["p1_w"].astype(np.float64).T + p["p1_b"])
    return h @ p["p2_w"].astype(np.float64).T + p["p2_b"]


def _mats(cfg):
    from geoflac_gb300.fno import dft_matrices
    return dft_matrices(cfg)


def spectral_dft(cfg, mats, v, R):
    """S(v) with the kernels' matrices; returns s and the mode coefficients U"""
    B, H, W, C = v.shape
    m2, Q = cfg.m2, cfg.Q
    vt = v.transpose(0, 1, 3, 2)                        # [B, H, C, W]
    Xw = vt @ mats["FW"].T                              # [B, H, C, 2m2]
    Xt = Xw.transpose(0, 2, 3, 1)                       # [B, C, 2m2, H]
    Y = Xt @ mats["FH"].T                               # [B, C, 2m2, 2Q]
    Yc, Ys = Y[..., :Q], Y[..., Q:]
    Ure = Yc[:, :, :m2, :] + Ys[:, :, m2:, :]           # [B, C, m2, Q]
    Uim = Yc[:, :, m2:, :] - Ys[:, :, :m2, :]
    Uc = Ure + 1j * Uim
    Rc = _complex_R(cfg, R)                             # [m2, Q, C, C]
    Vc = np.einsum("bikq,kqio->bokq", Uc, Rc)           # [B, C(o), m2, Q]
    Vt = np.stack([Vc.real, Vc.imag], axis=-1).reshape(B, C, m2, 2 * Q)
    Z = Vt @ mats["IH"].T                               # [B, C, m2, 2H]
    Zt = Z.reshape(B, C, m2, H, 2).transpose(0, 3, 1, 2, 4).reshape(B, H, C, 2 * m2)
    s = Zt @ mats["IW"].T                               # [B, H, C, W]
    return s.transpose(0, 1, 3, 2), Uc


def forward_dft(cfg, p, x) -> Tuple[np.ndarray, dict]:
    mats = _mats(cfg)
    P = {k: v.astype(np.float64) for k, v in p.items()}
    x = x.astype(np.float64)
    v = x @ P["lift_w"].T + P["lift_b"]
    rec = {"x": x, "v": [], "z": [], "U": []}
    for l in range(cfg.layers):
        s, U = spectral_dft(cfg, mats, v, P[f"R{l}"])
        z = v @ P[f"w{l}"].T + P[f"b{l}"] + s
        rec["v"].append(v)
        rec["z"].append(z)
        rec["U"].append(U)
        v = gelu(z) if l < cfg.layers - 1 else z
    zp = v @ P["p1_w"].T + P["p1_b"]
    h = gelu(zp)
    out = h @ P["p2_w"].T + P["p2_b"]
    rec.update(vL=v, zp=zp, h=h)
    return out, rec


def spectral_dft_bwd(cfg, mats, ds, U, R):
    """gradient of <ds, S(v)> w.r.t. v and R"""
    B, H, W, C = ds.shape
    m2, Q = cfg.m2, cfg.Q
    dZt = ds.transpose(0, 1, 3, 2) @ mats["IW"]         # [B, H, C, 2m2]
    dZ = dZt.reshape(B, H, C, m2, 2).transpose(0, 2, 3, 1, 4).reshape(B, C, m2, 2 * H)
    dVt = dZ @ mats["IH"]                               # [B, C, m2, 2Q]
    dVr = dVt.reshape(B, C, m2, Q, 2)
    dVc = dVr[..., 0] + 1j * dVr[..., 1]                # d/dRe + i d/dIm
    Rc = _complex_R(cfg, R)
    # V = sum_i U R  (complex); real gradients: dU = dV conj(R), dR = conj(U) dV
    dUc = np.einsum("bokq,kqio->bikq", dVc, np.conj(Rc))
    dRc = np.einsum("bikq,bokq->kqio", np.conj(U), dVc)
    dR = np.stack([dRc.real, dRc.imag], axis=-1).reshape(cfg.modes, C, C, 2)
    dUre, dUim = dUc.real, dUc.imag                     # [B, C, m2, Q]
    dY = np.zeros((B, C, 2 * m2, 2 * Q))
    dY[:, :, :m2, :Q] += dUre
    dY[:, :, m2:, Q:] += dUre
    dY[:, :, m2:, :Q] += dUim
    dY[:, :, :m2, Q:] -= dUim
    dXt = dY @ mats["FH"]                               # [B, C, 2m2, H]
    dXw = dXt.transpose(0, 3, 1, 2)                     # [B, H, C, 2m2]
    dvt = dXw @ mats["FW"]                              # [B, H, C, W]
    return dvt.transpose(0, 1, 3, 2), dR


def backward_dft(cfg, p, rec, dout) -> Dict[str, np.ndarray]:
    """parameter gradients for the output gradient dout"""
    mats = _mats(cfg)
    P = {k: v.astype(np.float64) for k, v in p.items()}
    g = {}
    B, H, W, _ = dout.shape
    M = B * H * W
    d2 = dout.reshape(M, -1)
    g["p2_w"] = d2.T @ rec["h"].reshape(M, -1)
    g["p2_b"] = d2.sum(0)
    dh = d2 @ P["p2_w"]
    dzp = dh * gelu_d(rec["zp"].reshape(M, -1))
    g["p1_w"] = dzp.T @ rec["vL"].reshape(M, -1)
    g["p1_b"] = dzp.sum(0)
    dv = (dzp @ P["p1_w"]).reshape(B, H, W, -1)
    for l in reversed(range(cfg.layers)):
        z = rec["z"][l]
        dz = dv * gelu_d(z) if l < cfg.layers - 1 else dv
        v = rec["v"][l]
        g[f"w{l}"] = dz.reshape(M, -1).T @ v.reshape(M, -1)
        g[f"b{l}"] = dz.reshape(M, -1).sum(0)
        dvs, g[f"R{l}"] = spectral_dft_bwd(cfg, mats, dz, rec["U"][l], P[f"R{l}"])
        dv = dvs + dz @ P[f"w{l}"]
    g["lift_w"] = dv.reshape(M, -1).T @ rec["x"].reshape(M, -1)
    g["lift_b"] = dv.reshape(M, -1).sum(0)
    return g


def mse_grad(out, target):
    n = out.size
    return float(((out - target) ** 2).mean()), 2.0 * (out - target) / n
