"""Learned fast-forward of ensemble members.

1. Snapshots: the ensemble driver advances a sweep and samples every
   member onto the FNO grid every `interval` steps (gf_batch_sample):
   consecutive samples form (t, t + interval) training pairs.
2. Training: the FNO (geoflac_gb300.fno) learns the normalised increment
   of the 9 fields from the fields at t plus the member's 4 sweep
   parameters, with the library's own forward/backward kernels and Adam.
3. Screening: for a fresh sweep at time t, predict t + interval for every
   member, write the prediction into the member's mesh (gf_batch_inject)
   and gate it with the force-imbalance residual of the injected state
   (gf_batch_force_residual).  Members above the tolerance are restored and
   advanced by the plain FLAC step; the plain step stays the arbiter of the error.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import capi
from .batch import Batch
from .fno import Fno, FnoConfig, _ck, _p

NCH = 9
FIELD_NAMES = ("vx", "vz", "sxx", "szz", "sxz", "aps", "temp", "crust_fraction", "uz")
PARAM_NAMES = ("friction", "crust_km", "moho_t", "v_cm_yr")
CRUST_PHASE = 2


def params_array(prms: List[dict]) -> np.ndarray:
    return np.array([[p[k] for k in PARAM_NAMES] for p in prms], dtype=np.float32)


@dataclass
class Snapshots:
    grids: "object"            # device FP32 [n_members, n_snap, H, W, 9]
    params: np.ndarray         # [n_members, 4]
    interval: int
    residual_true: np.ndarray  # force residual of the plain states (per snapshot, member)
    seconds: float = 0.0


def generate(batch: Batch, prms: List[dict], n_snap: int, interval: int, H: int, W: int) -> Snapshots:
    """n_snap samples of every member, `interval` plain steps apart."""
    import torch

    n = len(batch.members)
    grids = torch.empty((n, n_snap, H, W, NCH), dtype=torch.float32, device="cuda")
    tmp = torch.empty((n, H, W, NCH), dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(batch.stream)
    res = []
    t0 = time.time()
    for k in range(n_snap):
        if k:
            batch.step(interval)
        batch.sample(tmp, H, W, CRUST_PHASE)
        with torch.cuda.stream(stream):
            grids[:, k].copy_(tmp)
        res.append(batch.force_residual())
    torch.cuda.synchronize()
    return Snapshots(grids, params_array(prms), interval, np.array(res), time.time() - t0)


@dataclass
class Normaliser:
    stats: "object"    # device FP32 [26]: mean[9], std[9], pmean[4], pstd[4]
    stats_d: "object"  # device FP32 [18]: mean and std of the increments

    @staticmethod
    def fit(snaps: Snapshots) -> "Normaliser":
        import torch

        g = snaps.grids
        x = g[:, :-1].reshape(-1, NCH)
        d = (g[:, 1:] - g[:, :-1]).reshape(-1, NCH)
        mean, std = x.mean(0), x.std(0).clamp_min(1e-30)
        dmean, dstd = d.mean(0), d.std(0).clamp_min(1e-30)
        pm = torch.from_numpy(snaps.params.mean(0)).cuda()
        ps = torch.from_numpy(snaps.params.std(0) + 1e-6).cuda()
        return Normaliser(torch.cat([mean, std, pm, ps]).float().contiguous(),
                          torch.cat([dmean, dstd]).float().contiguous())


class Surrogate:
    def __init__(self, cfg: FnoConfig, norm: Normaliser, seed: int = 0):
        self.cfg = cfg
        self.net = Fno(cfg, seed=seed)
        self.norm = norm
        self.lib = self.net.lib
        self.history: List[float] = []

    @property
    def s(self):
        return self.net.s

    def pack(self, raw_x, prm_dev, out):
        n = raw_x.shape[0]
        _ck(self.lib.gf_fno_pack_input(_p(raw_x), _p(prm_dev), _p(self.norm.stats), _p(out), n, self.cfg.H,
                                       self.cfg.W, self.s), "pack_input")

    def train(self, snaps: Snapshots, epochs: int, batch: int = 64, lr: float = 1e-3, seed: int = 0,
              max_pairs: Optional[int] = None, surface_weight: float = 64.0) -> Dict[str, float]:
        """Adam over all (t, t + interval) pairs, cosine learning rate; the
        displacement channel of the top grid rows (the topography) is
        weighted by `surface_weight` in the loss."""
        import torch

        cfg = self.cfg
        wgt = torch.ones((cfg.H, cfg.W, cfg.cout), dtype=torch.float32, device="cuda")
        wgt[:2, :, 8] = surface_weight
        n, ns = snaps.grids.shape[0], snaps.grids.shape[1]
        pairs = [(m, k) for m in range(n) for k in range(ns - 1)]
        if max_pairs:
            pairs = pairs[:max_pairs]
        rng = np.random.default_rng(seed)
        row_bytes = cfg.H * cfg.W * NCH * 4
        flat = snaps.grids.view(n * ns, cfg.H, cfg.W, NCH)
        prm_all = torch.from_numpy(snaps.params).cuda()
        xb = torch.empty((batch, cfg.H, cfg.W, NCH), dtype=torch.float32, device="cuda")
        yb = torch.empty_like(xb)
        inp = torch.empty((batch, cfg.H, cfg.W, cfg.cin), dtype=torch.bfloat16, device="cuda")
        tgt = torch.empty((batch, cfg.H, cfg.W, cfg.cout), dtype=torch.float32, device="cuda")
        prm_b = torch.empty((batch, 4), dtype=torch.float32, device="cuda")
        steps = epochs * (len(pairs) // batch)
        t0 = time.time()
        it = 0
        for ep in range(epochs):
            order = rng.permutation(len(pairs))
            for b0 in range(0, len(order) - batch + 1, batch):
                sel = [pairs[i] for i in order[b0:b0 + batch]]
                ix = torch.tensor([m * ns + k for m, k in sel], dtype=torch.int64).cuda()
                iy = torch.tensor([m * ns + k + 1 for m, k in sel], dtype=torch.int64).cuda()
                ip = torch.tensor([m for m, _ in sel], dtype=torch.int64).cuda()
                _ck(self.lib.gf_fno_gather_rows(_p(flat), _p(xb), _p(ix), batch, row_bytes, self.s), "gather")
                _ck(self.lib.gf_fno_gather_rows(_p(flat), _p(yb), _p(iy), batch, row_bytes, self.s), "gather")
                _ck(self.lib.gf_fno_gather_rows(_p(prm_all), _p(prm_b), _p(ip), batch, 16, self.s), "gather")
                self.pack(xb, prm_b, inp)
                _ck(self.lib.gf_fno_pack_target(_p(yb), _p(xb), _p(self.norm.stats_d), _p(tgt),
                                                batch * cfg.H * cfg.W, self.s), "pack_target")
                out = self.net.forward(inp, train=True)
                loss, dout = self.net.loss_grad(out, tgt, wgt)
                self.net.backward(dout)
                lr_t = 0.5 * lr * (1.0 + math.cos(math.pi * it / max(steps, 1)))
                self.net.adam(lr=lr_t)
                it += 1
                if it % 16 == 0 or it == steps:
                    self.history.append(loss.item())
        torch.cuda.synchronize()
        return {"steps": it, "seconds": time.time() - t0, "final_loss": self.history[-1] if self.history else None,
                "first_loss": self.history[0] if self.history else None}

    def predict(self, raw_x, params: np.ndarray, batch: int = 64):
        """raw fields at t (device [n, H, W, 9]) -> predicted fields at t + interval"""
        import torch

        cfg = self.cfg
        n = raw_x.shape[0]
        out = torch.empty_like(raw_x)
        prm = torch.from_numpy(params.astype(np.float32)).cuda()
        inp = torch.empty((batch, cfg.H, cfg.W, cfg.cin), dtype=torch.bfloat16, device="cuda")
        for b0 in range(0, n, batch):
            nb = min(batch, n - b0)
            self.pack(raw_x[b0:b0 + nb], prm[b0:b0 + nb], inp[:nb])
            pred = self.net.forward(inp[:nb])
            _ck(self.lib.gf_fno_unpack(_p(pred), _p(raw_x[b0:b0 + nb]), _p(self.norm.stats_d), _p(out[b0:b0 + nb]),
                                       nb * cfg.H * cfg.W, self.s), "unpack")
        return out


def rel_errors(pred, true, base):
    """relative L2 errors per member: topography (displacement on the top grid
    row) and plastic strain; and the same for the persistence forecast
    `base` (the fields at t)."""
    def rel(a, b):
        num = (a - b).reshape(a.shape[0], -1).norm(dim=1)
        den = b.reshape(b.shape[0], -1).norm(dim=1).clamp_min(1e-30)
        return (num / den).cpu().numpy()

    topo = lambda g: g[:, 0, :, 8]
    aps = lambda g: g[..., 5]
    return {"topography": rel(topo(pred), topo(true)), "plastic_strain": rel(aps(pred), aps(true)),
            "topography_persistence": rel(topo(base), topo(true)),
            "plastic_strain_persistence": rel(aps(base), aps(true))}


def calibrate_tolerance(batch: Batch, H: int, W: int, factor: float = 2.0) -> Dict[str, float]:
    """Gate tolerance from plain states written through the grid: the force
    residual of inject(sample(state)) for every member (a perfect forecast
    seen through the same representation); tol = factor x its 95th
    percentile.  Leaves the members holding the re-injected fields."""
    import torch

    n = len(batch.members)
    g = torch.empty((n, H, W, NCH), dtype=torch.float32, device="cuda")
    batch.sample(g, H, W, CRUST_PHASE)
    plain = batch.force_residual()
    batch.inject(g, H, W)
    rt = batch.force_residual()
    return {"tol": float(factor * np.quantile(rt, 0.95)), "plain_max": float(plain.max()),
            "roundtrip_p95": float(np.quantile(rt, 0.95)), "roundtrip_max": float(rt.max())}


def screen(batch: Batch, sur: Surrogate, prms: List[dict], interval: int, tol: float) -> Dict[str, object]:
    """Fast-forward every member by `interval` steps with the surrogate; the
    members whose injected state fails the force-imbalance gate are restored
    and advanced by the plain step.  Returns the predicted / recomputed
    fields at t + interval (device [n, H, W, 9]) and the timings."""
    import torch

    cfg = sur.cfg
    n = len(batch.members)
    H, W = cfg.H, cfg.W
    torch.cuda.synchronize()
    t0 = time.time()
    batch.backup()  # restore point for the members the gate rejects
    t_save = time.time() - t0
    raw = torch.empty((n, H, W, NCH), dtype=torch.float32, device="cuda")
    ts = time.time()
    batch.sample(raw, H, W, CRUST_PHASE)
    torch.cuda.synchronize()
    t1 = time.time()
    t_sample = t1 - ts
    pred = sur.predict(raw, params_array(prms))
    torch.cuda.synchronize()
    t_pred = time.time() - t1
    ti = time.time()
    batch.inject(pred, H, W)
    t_inject = time.time() - ti
    ti = time.time()
    resid = batch.force_residual()
    t_resid = time.time() - ti
    fail = np.nonzero(resid > tol)[0]
    t2 = time.time()
    out = pred
    rr = {}
    if len(fail):
        sub = [batch.members[k] for k in fail]
        batch.restore(fail)
        sb = Batch(sub)
        # the parent's CTA build with one item per thread: a few members
        # then still spread over every SM
        cfg_sub = dict(batch.config())
        cfg_sub["items_per_thread"] = 1
        sb.set_config(**cfg_sub)
        rr["prepare"] = time.time() - t2
        stream = torch.cuda.ExternalStream(sb.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sb.step(interval)
        e1.record(stream)
        torch.cuda.synchronize()
        rr["step_host"] = time.time() - t2 - rr["prepare"]
        rr["step_gpu"] = e0.elapsed_time(e1) / 1e3
        g = torch.empty((len(sub), H, W, NCH), dtype=torch.float32, device="cuda")
        sb.sample(g, H, W, CRUST_PHASE)
        torch.cuda.synchronize()
        for r, k in enumerate(fail):  # plain results replace the rejected forecasts (device copies)
            out[int(k)].copy_(g[r])
        sb.close()
    torch.cuda.synchronize()
    t_rerun = time.time() - t2
    return {"fields": out, "raw_t": raw, "residual": resid, "rerun": fail.tolist(), "rerun_detail": rr,
            "seconds": time.time() - t0, "seconds_save": t_save, "seconds_sample": t_sample,
            "seconds_predict": t_pred, "seconds_inject": t_inject, "seconds_residual": t_resid,
            "seconds_rerun": t_rerun}
