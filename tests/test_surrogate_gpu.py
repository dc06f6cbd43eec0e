"""Surrogate pipeline end to end on a small sweep: snapshots from the
ensemble driver, training with the library's FNO kernels, screening of a
fresh sweep through the force-imbalance gate.

What the network gains over the method without it: its topography and
plastic-strain forecast of the fresh sweep is compared with the
persistence forecast (fields unchanged over the interval), the forecast a
screening without the network would make; the network must have the lower
topography error.  The gate must pass states written through the grid and
reject a deliberately corrupted forecast."""
import numpy as np
import pytest

from geoflac_gb300 import inpgen
from geoflac_gb300.batch import Batch
from geoflac_gb300.flac import Flac, new_state
from geoflac_gb300.fno import FnoConfig
from geoflac_gb300 import surrogate as S

pytestmark = pytest.mark.gpu

SCALE = (24, 8, 48, 16)
CFG = FnoConfig(H=32, W=96, C=32, m1=8, m2=8, layers=3, cin=16, P=64, cout=16)
INTERVAL = 100


def _sweep(workdir, n, seed, tag):
    ms, prms = [], []
    for k in range(n):
        m, prm = inpgen.ensemble_member(k, seed=seed, scale=SCALE)
        p, c, s = new_state(m.write(str(workdir / f"sg_{tag}_{k}.inp")))
        ms.append(Flac(p, c, s, "mixed"))
        prms.append(prm)
    return ms, prms


def test_surrogate_trains_screens_and_beats_persistence(workdir):
    torch = pytest.importorskip("torch")
    ms, prms = _sweep(workdir, 32, 101, "train")
    b = Batch(ms)
    snaps = S.generate(b, prms, n_snap=9, interval=INTERVAL, H=CFG.H, W=CFG.W)
    assert torch.isfinite(snaps.grids).all()
    cal = S.calibrate_tolerance(b, CFG.H, CFG.W)
    sur = S.Surrogate(CFG, S.Normaliser.fit(snaps), seed=1)
    info = sur.train(snaps, epochs=40, batch=32, lr=2e-3)
    assert info["final_loss"] < 0.5 * info["first_loss"], info
    # fresh sweep: a plain copy for the truth, a screened copy
    fa, prm_f = _sweep(workdir, 16, 202, "truth")
    fb, _ = _sweep(workdir, 16, 202, "screen")
    ba, bb = Batch(fa), Batch(fb)
    ba.step(INTERVAL)
    bb.step(INTERVAL)
    res = S.screen(bb, sur, prm_f, INTERVAL, cal["tol"])
    ba.step(INTERVAL)
    truth = torch.empty_like(res["fields"])
    ba.sample(truth, CFG.H, CFG.W, S.CRUST_PHASE)
    torch.cuda.synchronize()
    err = S.rel_errors(res["fields"], truth, res["raw_t"])
    assert np.isfinite(err["topography"]).all()
    assert np.median(err["topography"]) < np.median(err["topography_persistence"]), err
    # a forecast with the stresses scaled by 3 does not balance gravity
    bad = res["raw_t"].clone()
    bad[..., 2:5] *= 3.0
    bb.inject(bad, CFG.H, CFG.W)
    r_bad = bb.force_residual()
    assert (r_bad > cal["tol"]).all(), (r_bad, cal)
