"""Fourier neural operator that predicts an ensemble member's state several
hundred steps ahead, trained and run by the library's own kernels
(include/geoflac_fno.h): every matrix product is the tcgen05 BF16 GEMM with
FP32 accumulation, every other operation one of the FNO kernels.  PyTorch
only allocates the device buffers and provides the stream.

Architecture (per pixel of an H x W grid, channels last):
  lift      z0 = x Wl^T + bl                       (cin -> C)
  layer l   z  = v Wl^T + bl + S_l(v),  v' = GELU(z) (no GELU after the last)
            S_l = truncated 2-D DFT (Q = 2*m1 H-modes: k1 < m1 and k1 >= H - m1;
                  m2 W-modes k2 < m2), per-mode complex C x C mixing, inverse DFT
  project   out = GELU(v P1^T + p1) P2^T + p2       (C -> P -> cout)
The truncated DFTs are products with DFT matrices (FW, FH forward, IH, IW
inverse, normalised like numpy's rfft2 / irfft2).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Dict, Optional

import numpy as np

from . import capi

_F = None


def _lib():
    global _F
    if _F is not None:
        return _F
    lib = capi.load_library()
    vp, i, ll, f = C.c_void_p, C.c_int, C.c_longlong, C.c_float
    sig = {
        "gf_gemm_bf16": [vp, vp, vp, i, i, i, i, ll, ll, ll, ll, ll, ll, i, f, f, vp, vp],
        "gf_gemm_error": [],
        "gf_fno_transpose": [vp, vp, i, ll, i, i, i, vp],
        "gf_fno_cast": [vp, vp, ll, i, i, vp],
        "gf_fno_gelu": [vp, vp, ll, i, vp],
        "gf_fno_gelu_bwd": [vp, vp, i, vp, vp, ll, vp],
        "gf_gemm_bf16_ex": [vp, vp, vp, i, i, i, i, ll, ll, ll, ll, ll, ll, i, f, f, vp, vp, i, vp],
        "gf_fno_spec_combine": [vp, vp, i, i, i, i, vp],
        "gf_fno_spec_combine_bwd": [vp, vp, i, i, i, i, vp],
        "gf_fno_expand_modes": [vp, vp, vp, i, i, vp],
        "gf_fno_modes_grad": [vp, vp, i, i, vp],
        "gf_fno_colsum": [vp, vp, ll, i, i, vp],
        "gf_fno_sum_batches": [vp, vp, i, ll, i, vp],
        "gf_fno_adam": [vp, vp, vp, vp, ll, f, f, f, f, i, f, vp],
        "gf_fno_mse": [vp, vp, vp, i, vp, ll, f, vp],
        "gf_fno_mse_weighted": [vp, vp, vp, i, vp, ll, f, vp, ll, i, vp],
        "gf_fno_add": [vp, vp, vp, vp, ll, vp],
        "gf_fno_pack_input": [vp, vp, vp, vp, i, i, i, vp],
        "gf_fno_pack_target": [vp, vp, vp, vp, ll, vp],
        "gf_fno_unpack": [vp, vp, vp, vp, ll, vp],
        "gf_fno_gather_rows": [vp, vp, vp, i, ll, vp],
    }
    for n, a in sig.items():
        fn = getattr(lib, n)
        fn.restype = C.c_int
        fn.argtypes = a
    _F = lib
    return lib


class FnoError(RuntimeError):
    pass


def _ck(rc, what):
    if rc != 0:
        raise FnoError(f"{what}: status {rc}")


def _p(t):
    return None if t is None else t.data_ptr()


@dataclass
class FnoConfig:
    H: int = 128
    W: int = 384
    C: int = 64
    m1: int = 24
    m2: int = 24
    layers: int = 4
    cin: int = 16
    P: int = 128
    cout: int = 16

    @property
    def Q(self) -> int:
        return 2 * self.m1

    @property
    def modes(self) -> int:
        return self.Q * self.m2

    def k1(self, q: int) -> int:
        return q if q < self.m1 else self.H - 2 * self.m1 + q


def dft_matrices(cfg: FnoConfig) -> Dict[str, np.ndarray]:
    """FP64 DFT matrices of the truncated transforms (row layouts as the
    kernels use them)."""
    H, W, m2, Q = cfg.H, cfg.W, cfg.m2, cfg.Q
    w = np.arange(W)
    h = np.arange(H)
    k2 = np.arange(m2)
    thw = 2 * np.pi * np.outer(k2, w) / W            # [m2, W]
    FW = np.concatenate([np.cos(thw), -np.sin(thw)])  # [2 m2, W]: Re, Im of sum x e^{-i th}
    k1 = np.array([cfg.k1(q) for q in range(Q)])
    thh = 2 * np.pi * np.outer(k1, h) / H            # [Q, H]
    FH = np.concatenate([np.cos(thh), np.sin(thh)])  # [2Q, H]
    # inverse along H (complex -> complex), columns (q, re|im), rows (h, re|im), 1/H
    IH = np.zeros((2 * H, 2 * Q))
    ch, sh = np.cos(thh).T / H, np.sin(thh).T / H    # [H, Q]
    IH[0::2, 0::2] = ch
    IH[0::2, 1::2] = -sh
    IH[1::2, 0::2] = sh
    IH[1::2, 1::2] = ch
    # inverse along W (Hermitian half spectrum -> real), columns (k2, re|im), 1/W
    ck = np.where(k2 == 0, 1.0, 2.0)
    IW = np.zeros((W, 2 * m2))
    IW[:, 0::2] = (ck[None, :] * np.cos(thw.T)) / W
    IW[:, 1::2] = (-ck[None, :] * np.sin(thw.T)) / W
    return {"FW": FW, "FH": FH, "IH": IH, "IW": IW}


def init_params(cfg: FnoConfig, seed: int = 0) -> Dict[str, np.ndarray]:
    """FP32 parameters: uniform fan-in scaled dense weights, complex mode
    weights R[l][(k2, q)][i][o][re|im] scaled by 1/(C*C)."""
    rng = np.random.default_rng(seed)

    def dense(o, i):
        b = 1.0 / math.sqrt(i)
        return rng.uniform(-b, b, size=(o, i)).astype(np.float32), rng.uniform(-b, b, size=o).astype(np.float32)

    p = {}
    p["lift_w"], p["lift_b"] = dense(cfg.C, cfg.cin)
    for l in range(cfg.layers):
        p[f"R{l}"] = (rng.uniform(0, 1, size=(cfg.modes, cfg.C, cfg.C, 2)) / (cfg.C * cfg.C)).astype(np.float32)
        p[f"w{l}"], p[f"b{l}"] = dense(cfg.C, cfg.C)
    p["p1_w"], p["p1_b"] = dense(cfg.P, cfg.C)
    p["p2_w"], p["p2_b"] = dense(cfg.cout, cfg.P)
    return p


class Fno:
    """Device-resident FNO: parameters (FP32 master copies), Adam moments,
    forward with saved activations, backward, optimizer step."""

    def __init__(self, cfg: FnoConfig, params: Optional[Dict[str, np.ndarray]] = None, seed: int = 0):
        import torch

        self.torch = torch
        self.cfg = cfg
        self.lib = _lib()
        dev = "cuda"
        params = params if params is not None else init_params(cfg, seed)
        self.p = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in params.items()}
        self.g = {k: torch.zeros_like(v) for k, v in self.p.items()}
        self.m = {k: torch.zeros_like(v) for k, v in self.p.items()}
        self.v = {k: torch.zeros_like(v) for k, v in self.p.items()}
        self.t = 0
        mats = dft_matrices(cfg)
        bf = torch.bfloat16
        self.mat = {}
        for k, a in mats.items():
            self.mat[k] = torch.from_numpy(np.ascontiguousarray(a)).to(dev).to(bf)
            self.mat[k + "T"] = torch.from_numpy(np.ascontiguousarray(a.T)).to(dev).to(bf)
        self.saved = None

    # ---------------------------------------------------------------- kernels
    @property
    def s(self):
        return self.torch.cuda.current_stream().cuda_stream

    def gemm(self, A, B, Cout, batch, M, N, K, lda, sA, ldb, sB, ldc, sC, alpha=1.0, beta=0.0, bias=None,
             aux=None, act=0, keep_c=True):
        """keep_c=False (with aux): the FP32 C is only read (beta) or absent
        (Cout None), and only the BF16 activation is written."""
        if not keep_c:
            c_bf16 = 2
        else:
            c_bf16 = 1 if Cout.dtype == self.torch.bfloat16 else 0
        _ck(self.lib.gf_gemm_bf16_ex(_p(A), _p(B), _p(Cout), batch, M, N, K, lda, sA, ldb, sB, ldc, sC, c_bf16,
                                     alpha, beta, _p(bias), _p(aux), act, self.s), "gemm")

    def mm(self, A, Bw, out, M, N, K, beta=0.0, bias=None, aux=None, act=0, keep_c=True):
        """out[M, N] (+)= A[M, K] Bw[N, K]^T (+ bias); aux = BF16 out or GELU(out)."""
        self.gemm(A, Bw, out, 1, M, N, K, K, 0, K, 0, N, 0, 1.0, beta, bias, aux, act, keep_c)

    def tr(self, src, dst, batch, rows, cols):
        _ck(self.lib.gf_fno_transpose(_p(src), _p(dst), batch, rows, cols,
                                      int(src.dtype == self.torch.bfloat16), int(dst.dtype == self.torch.bfloat16),
                                      self.s), "transpose")

    def tr_pairs(self, src, dst, batch, rows, cols):
        """transpose of a matrix of BF16 (re, im) pairs, moved as 32-bit words"""
        f32 = self.torch.float32
        _ck(self.lib.gf_fno_transpose(_p(src.view(f32)), _p(dst.view(f32)), batch, rows, cols, 0, 0, self.s),
            "transpose")

    def bf16(self, t):
        out = self.torch.empty(t.shape, dtype=self.torch.bfloat16, device=t.device)
        _ck(self.lib.gf_fno_cast(_p(t), _p(out), t.numel(), int(t.dtype == self.torch.bfloat16), 1, self.s), "cast")
        return out

    def gelu(self, z, out):
        _ck(self.lib.gf_fno_gelu(_p(z), _p(out), z.numel(), int(out.dtype == self.torch.bfloat16), self.s), "gelu")

    def gelu_bwd(self, z, da, dz, dz_b=None):
        _ck(self.lib.gf_fno_gelu_bwd(_p(z), _p(da), int(da.dtype == self.torch.bfloat16), _p(dz), _p(dz_b),
                                     z.numel(), self.s), "gelu_bwd")

    def colsum(self, X, out, rows, cols):
        _ck(self.lib.gf_fno_colsum(_p(X), _p(out), rows, cols, 0, self.s), "colsum")

    def wgrad(self, dz_rows, x_rows, M, n_out, n_in, out):
        """out[n_out, n_in] = dz^T x over M rows, split over K chunks"""
        torch = self.torch
        S = 1
        for cand in (512, 384, 256, 128, 64, 32, 16, 8, 4, 2, 1):
            if (M % cand == 0 and (M // cand) % 8 == 0 and M // cand >= 1024) or cand == 1:
                S = cand
                break
        Kc = M // S
        # each chunk of Kc rows transposed on its own: dzT[s] = dz[s*Kc:(s+1)*Kc]^T
        dzT = torch.empty((S, n_out, Kc), dtype=torch.bfloat16, device="cuda")
        xT = torch.empty((S, n_in, Kc), dtype=torch.bfloat16, device="cuda")
        self.tr(dz_rows, dzT, S, Kc, n_out)
        self.tr(x_rows, xT, S, Kc, n_in)
        part = torch.empty((S, n_out, n_in), dtype=torch.float32, device="cuda")
        self.gemm(dzT, xT, part, S, n_out, n_in, Kc, Kc, n_out * Kc, Kc, n_in * Kc, n_in, n_out * n_in)
        _ck(self.lib.gf_fno_sum_batches(_p(part), _p(out), S, n_out * n_in, 0, self.s), "sum_batches")

    # ---------------------------------------------------------------- forward
    def spectral(self, v, l, B, save):
        """S_l(v) for v BF16 [B, H, W, C] -> FP32 [B, H, W, C]"""
        torch, cfg = self.torch, self.cfg
        H, W, Cc, m2, Q = cfg.H, cfg.W, cfg.C, cfg.m2, cfg.Q
        bf = torch.bfloat16
        vt = torch.empty((B, H, Cc, W), dtype=bf, device="cuda")
        self.tr(v, vt, B * H, W, Cc)
        Xw = torch.empty((B, H, Cc, 2 * m2), dtype=bf, device="cuda")
        self.mm(vt, self.mat["FW"], Xw, B * H * Cc, 2 * m2, W)
        Xt = torch.empty((B, Cc, 2 * m2, H), dtype=bf, device="cuda")
        self.tr(Xw, Xt, B, H, Cc * 2 * m2)
        Y = torch.empty((B, Cc, 2 * m2, 2 * Q), dtype=torch.float32, device="cuda")
        self.mm(Xt, self.mat["FH"], Y, B * Cc * 2 * m2, 2 * Q, H)
        U = torch.empty((cfg.modes, B, 2 * Cc), dtype=bf, device="cuda")
        _ck(self.lib.gf_fno_spec_combine(_p(Y), _p(U), B, Cc, m2, Q, self.s), "spec_combine")
        Rm = torch.empty((cfg.modes, 2 * Cc, 2 * Cc), dtype=bf, device="cuda")
        RmT = torch.empty_like(Rm)
        _ck(self.lib.gf_fno_expand_modes(_p(self.p[f"R{l}"]), _p(Rm), _p(RmT), cfg.modes, Cc, self.s), "expand")
        V = torch.empty((cfg.modes, B, 2 * Cc), dtype=bf, device="cuda")
        n2 = 2 * Cc
        self.gemm(U, Rm, V, cfg.modes, B, n2, n2, n2, B * n2, n2, n2 * n2, n2, B * n2)
        Vt = torch.empty((B, Cc, m2, 2 * Q), dtype=bf, device="cuda")
        self.tr_pairs(V, Vt, 1, cfg.modes, B * Cc)
        Z = torch.empty((B, Cc, m2, 2 * H), dtype=bf, device="cuda")
        self.mm(Vt, self.mat["IH"], Z, B * Cc * m2, 2 * H, 2 * Q)
        Zt = torch.empty((B, H, Cc, 2 * m2), dtype=bf, device="cuda")
        self.tr_pairs(Z, Zt, B, Cc * m2, H)
        # s[b, h] = IW Zt[b, h]^T, channels last: one IW for all (b, h)
        s_cl = torch.empty((B, H, W, Cc), dtype=torch.float32, device="cuda")
        self.gemm(self.mat["IW"], Zt, s_cl, B * H, W, Cc, 2 * m2, 2 * m2, -1, 2 * m2, Cc * 2 * m2, Cc, W * Cc)
        if save:
            return s_cl, (U, RmT)
        return s_cl, None

    def forward(self, x, train: bool = False):
        """x: BF16 [B, H, W, cin] -> FP32 [B, H, W, cout]"""
        torch, cfg = self.torch, self.cfg
        B = x.shape[0]
        M = B * cfg.H * cfg.W
        bf = torch.bfloat16
        wb = {k: self.bf16(self.p[k]) for k in self.p if not k.startswith("R") and not k.endswith("_b")
              and not (k.startswith("b") and k[1:].isdigit())}
        # inference keeps only the BF16 activations (no FP32 copies of the
        # pre-activations, which only the backward pass reads)
        z = torch.empty((M, cfg.C), dtype=torch.float32, device="cuda") if train else None
        v = torch.empty((M, cfg.C), dtype=bf, device="cuda")
        self.mm(x.view(M, cfg.cin), wb["lift_w"], z, M, cfg.C, cfg.cin, bias=self.p["lift_b"], aux=v, keep_c=train)
        saved = {"x": x, "v": [], "z": [], "spec": [], "wb": wb}
        for l in range(cfg.layers):
            s_cl, sp = self.spectral(v.view(B, cfg.H, cfg.W, cfg.C), l, B, train)
            zl = s_cl.view(M, cfg.C)
            vn = torch.empty((M, cfg.C), dtype=bf, device="cuda")
            # z = v W^T + b + S(v); next input GELU(z) (z itself after the last layer)
            self.mm(v, wb[f"w{l}"], zl, M, cfg.C, cfg.C, beta=1.0, bias=self.p[f"b{l}"], aux=vn,
                    act=1 if l < cfg.layers - 1 else 0, keep_c=train)
            if train:
                saved["v"].append(v)
                saved["z"].append(zl)
                saved["spec"].append(sp)
            v = vn
        zp = torch.empty((M, cfg.P), dtype=torch.float32, device="cuda") if train else None
        hh = torch.empty((M, cfg.P), dtype=bf, device="cuda")
        self.mm(v, wb["p1_w"], zp, M, cfg.P, cfg.C, bias=self.p["p1_b"], aux=hh, act=1, keep_c=train)
        out = torch.empty((M, cfg.cout), dtype=torch.float32, device="cuda")
        self.mm(hh, wb["p2_w"], out, M, cfg.cout, cfg.P, bias=self.p["p2_b"])
        if train:
            saved.update(vL=v, zp=zp, h=hh)
            self.saved = saved
        return out.view(B, cfg.H, cfg.W, cfg.cout)

    # ---------------------------------------------------------------- backward
    def spectral_bwd(self, ds_cl, l, B, sp):
        """ds_cl FP32 [B, H, W, C] -> dv FP32 [B, H, W, C]; fills g[R_l]"""
        torch, cfg = self.torch, self.cfg
        H, W, Cc, m2, Q = cfg.H, cfg.W, cfg.C, cfg.m2, cfg.Q
        bf = torch.bfloat16
        U, RmT = sp
        ds = torch.empty((B, H, Cc, W), dtype=bf, device="cuda")
        self.tr(ds_cl, ds, B * H, W, Cc)
        dZt = torch.empty((B, H, Cc, 2 * m2), dtype=bf, device="cuda")
        self.mm(ds, self.mat["IWT"], dZt, B * H * Cc, 2 * m2, W)
        dZ = torch.empty((B, Cc, m2, 2 * H), dtype=bf, device="cuda")
        self.tr_pairs(dZt, dZ, B, H, Cc * m2)
        dVt = torch.empty((B, Cc, m2, 2 * Q), dtype=bf, device="cuda")
        self.mm(dZ, self.mat["IHT"], dVt, B * Cc * m2, 2 * Q, 2 * H)
        dV = torch.empty((cfg.modes, B, 2 * Cc), dtype=bf, device="cuda")
        self.tr_pairs(dVt, dV, 1, B * Cc, cfg.modes)
        n2 = 2 * Cc
        dU = torch.empty((cfg.modes, B, n2), dtype=torch.float32, device="cuda")
        self.gemm(dV, RmT, dU, cfg.modes, B, n2, n2, n2, B * n2, n2, n2 * n2, n2, B * n2)
        # dRm[mode] = dV[mode]^T U[mode]
        dVT = torch.empty((cfg.modes, n2, B), dtype=bf, device="cuda")
        UT = torch.empty((cfg.modes, n2, B), dtype=bf, device="cuda")
        self.tr(dV, dVT, cfg.modes, B, n2)
        self.tr(U, UT, cfg.modes, B, n2)
        dRm = torch.empty((cfg.modes, n2, n2), dtype=torch.float32, device="cuda")
        self.gemm(dVT, UT, dRm, cfg.modes, n2, n2, B, B, n2 * B, B, n2 * B, n2, n2 * n2)
        _ck(self.lib.gf_fno_modes_grad(_p(dRm), _p(self.g[f"R{l}"]), cfg.modes, Cc, self.s), "modes_grad")
        dY = torch.empty((B, Cc, 2 * m2, 2 * Q), dtype=bf, device="cuda")
        _ck(self.lib.gf_fno_spec_combine_bwd(_p(dU), _p(dY), B, Cc, m2, Q, self.s), "combine_bwd")
        dXt = torch.empty((B, Cc, 2 * m2, H), dtype=bf, device="cuda")
        self.mm(dY, self.mat["FHT"], dXt, B * Cc * 2 * m2, H, 2 * Q)
        dXw = torch.empty((B, H, Cc, 2 * m2), dtype=bf, device="cuda")
        self.tr(dXt, dXw, B, Cc * 2 * m2, H)
        dvt = torch.empty((B, H, Cc, W), dtype=torch.float32, device="cuda")
        self.mm(dXw, self.mat["FWT"], dvt, B * H * Cc, W, 2 * m2)
        dv = torch.empty((B, H, W, Cc), dtype=torch.float32, device="cuda")
        self.tr(dvt, dv, B * H, Cc, W)
        return dv

    def backward(self, dout):
        """dout: gradient of the loss w.r.t. the output, BF16 [B, H, W, cout]"""
        torch, cfg = self.torch, self.cfg
        sv = self.saved
        B = dout.shape[0]
        M = B * cfg.H * cfg.W
        bf = torch.bfloat16
        wb = sv["wb"]
        d2 = dout.reshape(M, cfg.cout)
        self.wgrad(d2, sv["h"], M, cfg.cout, cfg.P, self.g["p2_w"])
        d2f = torch.empty((M, cfg.cout), dtype=torch.float32, device="cuda")
        _ck(self.lib.gf_fno_cast(_p(d2), _p(d2f), d2.numel(), 1, 0, self.s), "cast")
        self.colsum(d2f, self.g["p2_b"], M, cfg.cout)
        p2T = torch.empty((cfg.P, cfg.cout), dtype=bf, device="cuda")
        self.tr(wb["p2_w"], p2T, 1, cfg.cout, cfg.P)
        dh = torch.empty((M, cfg.P), dtype=torch.float32, device="cuda")
        self.mm(d2, p2T, dh, M, cfg.P, cfg.cout)
        dzp = torch.empty_like(dh)
        dzp_b = torch.empty(dh.shape, dtype=bf, device="cuda")
        self.gelu_bwd(sv["zp"], dh, dzp, dzp_b)
        self.wgrad(dzp_b, sv["vL"], M, cfg.P, cfg.C, self.g["p1_w"])
        self.colsum(dzp, self.g["p1_b"], M, cfg.P)
        p1T = torch.empty((cfg.C, cfg.P), dtype=bf, device="cuda")
        self.tr(wb["p1_w"], p1T, 1, cfg.P, cfg.C)
        dv = torch.empty((M, cfg.C), dtype=torch.float32, device="cuda")
        self.mm(dzp_b, p1T, dv, M, cfg.C, cfg.P)
        for l in reversed(range(cfg.layers)):
            zl = sv["z"][l]
            if l < cfg.layers - 1:
                dz = torch.empty_like(dv)
                dz_b = torch.empty(dv.shape, dtype=bf, device="cuda")
                self.gelu_bwd(zl, dv, dz, dz_b)
            else:
                dz = dv
                dz_b = self.bf16(dz)
            self.wgrad(dz_b, sv["v"][l], M, cfg.C, cfg.C, self.g[f"w{l}"])
            self.colsum(dz, self.g[f"b{l}"], M, cfg.C)
            dv_spec = self.spectral_bwd(dz.view(B, cfg.H, cfg.W, cfg.C), l, B, sv["spec"][l])
            wT = torch.empty((cfg.C, cfg.C), dtype=bf, device="cuda")
            self.tr(wb[f"w{l}"], wT, 1, cfg.C, cfg.C)
            self.mm(dz_b, wT, dv_spec.view(M, cfg.C), M, cfg.C, cfg.C, beta=1.0)
            dv = dv_spec.view(M, cfg.C)
        dz0_b = self.bf16(dv)
        self.wgrad(dz0_b, sv["x"].reshape(M, cfg.cin), M, cfg.C, cfg.cin, self.g["lift_w"])
        self.colsum(dv, self.g["lift_b"], M, cfg.C)
        self.saved = None
        return self.g

    def loss_grad(self, out, target, weight=None):
        """mean-squared error, optionally weighted per pixel and channel (weight
        [H, W, cout], the same for every sample, or [batch, H, W, cout]), and
        its BF16 gradient w.r.t. the output"""
        torch = self.torch
        loss = torch.zeros(1, dtype=torch.float64, device="cuda")
        dout = torch.empty(out.shape, dtype=torch.bfloat16, device="cuda")
        if weight is None:
            _ck(self.lib.gf_fno_mse(_p(out), _p(target), _p(dout), 1, _p(loss), out.numel(), 1.0, self.s), "mse")
        else:
            _ck(self.lib.gf_fno_mse_weighted(_p(out), _p(target), _p(dout), 1, _p(loss), out.numel(), 1.0,
                                             _p(weight), 1, weight.numel(), self.s), "mse")
        return loss, dout

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, wd=0.0):
        self.t += 1
        for k, p in self.p.items():
            _ck(self.lib.gf_fno_adam(_p(p), _p(self.g[k]), _p(self.m[k]), _p(self.v[k]), p.numel(), lr, b1, b2, eps,
                                     self.t, wd, self.s), "adam")

    def params_numpy(self) -> Dict[str, np.ndarray]:
        return {k: v.detach().cpu().numpy() for k, v in self.p.items()}
