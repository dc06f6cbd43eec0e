"""The FP32 pre-check of the FP64 plastic return map (plastic_keeps_trial in
geoflac_gb300/csrc/gf_kernels.cuh), restated with numpy float32 (IEEE single,
one rounding per operation, correctly rounded square root, as the device
code is built) and checked against the FP64 evaluation of rh_plastic.f90's
decisions (s1 >= ten_max at line 111, fs < 0 at lines 134-135) on stress
states placed at and around the tension cut-off and the Mohr-Coulomb yield
surface, down to one ulp of FP64 margin: whenever the pre-check says the
trial stress is kept, the FP64 evaluation keeps it too (the same FP32
evaluation without the error margins is wrong on about 900 of these 200,000
states).  It also says so for most states with a margin of 1e-3."""
import numpy as np

F = np.float32


def fp64_keeps(s11i, s22i, s12i, anphi, amc, ten):
    """rh_plastic.f90:60-135 in FP64, the operations of the device code"""
    with np.errstate(all="ignore"):
        return _fp64_keeps(s11i, s22i, s12i, anphi, amc, ten)


def _fp64_keeps(s11i, s22i, s12i, anphi, amc, ten):
    sdif = s11i - s22i
    s0 = 0.5 * (s11i + s22i)
    rad = 0.5 * np.sqrt(sdif * sdif + (4.0 * s12i) * s12i)
    s1, s3 = s0 - rad, s0 + rad
    tension = s1 >= ten
    s3 = np.where(s3 >= ten, ten, s3)
    fs = (s1 - s3 * anphi) + amc
    return ~tension & ~(fs < 0.0), s1, fs


def fp32_keeps(s11i, s22i, s12i, anphi, amc, ten):
    """plastic_keeps_trial"""
    with np.errstate(all="ignore"):
        a, b, q = F(s11i), F(s22i), F(s12i)
        A = np.maximum(np.maximum(np.abs(a), np.abs(b)), np.abs(q))
        d = a - b
        s0 = F(0.5) * (a + b)
        r = F(0.5) * np.sqrt(d * d + (F(4.0) * q) * q)
        s1, sii = s0 - r, s0 + r
        tn, ap, am = F(ten), F(anphi), F(amc)
        at = np.abs(tn)
        s3 = np.fmin(sii, tn)
        fs = (s1 - s3 * ap) + am
        e_s1 = F(3.4e-6) * A + F(2.4e-7) * at + F(1e-30)
        e_fs = F(1.2e-7) * (F(40.0) * A + ap * (F(52.0) * A + F(10.0) * at) + F(4.0) * am) + F(1e-30)
        return (s1 + e_s1 < tn) & (fs > e_fs)


def _states(rng, n):
    """Stresses of crustal magnitude, friction 5-45 deg, cohesion 0-1e8."""
    s0 = -10.0 ** rng.uniform(5, 9.5, n) * rng.choice([1, -0.01], n)
    rad = 10.0 ** rng.uniform(3, 9, n)
    th = rng.uniform(0, np.pi, n)
    s11i = s0 + rad * np.cos(th)
    s22i = s0 - rad * np.cos(th)
    s12i = rad * np.sin(th)
    phi = np.radians(rng.uniform(5, 45, n))
    anphi = (1 + np.sin(phi)) / (1 - np.sin(phi))
    amc = 2.0 * rng.uniform(0, 1e8, n) * np.sqrt(anphi)
    ten = np.minimum(rng.uniform(0, 1e7, n) + 1e6, amc / np.sqrt(anphi) / np.tan(phi) + 1.0)
    return s11i, s22i, s12i, anphi, amc, ten


def test_pre_check_never_keeps_a_trial_stress_that_fp64_rejects():
    rng = np.random.default_rng(11)
    n = 200000
    s11i, s22i, s12i, anphi, amc, ten = _states(rng, n)
    _, s1, fs = fp64_keeps(s11i, s22i, s12i, anphi, amc, ten)
    # move each state onto the yield surface (fs = 0) or the cut-off
    # (s1 = ten) by shifting the mean stress, then off it by a relative
    # margin from one ulp to 1e-3, both ways
    shift_fs = fs / (anphi - 1.0)  # fs changes by -(anphi - 1) per unit of mean-stress increase
    shift_t = ten - s1
    margin = rng.choice([0.0, 1e-16, 1e-12, 1e-9, 1e-7, 1e-6, 1e-5, 1e-3], n) * rng.choice([1, -1], n)
    scale = np.abs(s11i) + np.abs(s22i) + np.abs(s12i)
    for shift in (shift_fs, shift_t):
        a = s11i + shift + margin * scale
        b = s22i + shift + margin * scale
        keeps, _, _ = fp64_keeps(a, b, s12i, anphi, amc, ten)
        pre = fp32_keeps(a, b, s12i, anphi, amc, ten)
        bad = np.nonzero(pre & ~keeps)[0]
        assert bad.size == 0, (a[bad[:3]], b[bad[:3]], s12i[bad[:3]])
        # every state at a wide margin on the elastic side passes the pre-check
        wide = keeps & (np.abs(margin) >= 1e-3)
        assert pre[wide].mean() > 0.95, pre[wide].mean()


def test_pre_check_on_random_states_and_edge_values():
    rng = np.random.default_rng(12)
    s11i, s22i, s12i, anphi, amc, ten = _states(rng, 200000)
    keeps, _, _ = fp64_keeps(s11i, s22i, s12i, anphi, amc, ten)
    pre = fp32_keeps(s11i, s22i, s12i, anphi, amc, ten)
    assert not np.any(pre & ~keeps)
    assert pre[keeps].mean() > 0.99
    # zeros, tiny magnitudes, NaN and overflow never pass unless FP64 agrees
    for v in (0.0, 1e-45, 1e-300, 1e39, np.inf, np.nan):
        x = np.full(4, v)
        keeps, _, _ = fp64_keeps(x, x * 0.5, x * 0.25, np.full(4, 3.0), np.full(4, 1e7), np.full(4, 1e6))
        with np.errstate(all="ignore"):
            pre = fp32_keeps(x, x * 0.5, x * 0.25, np.full(4, 3.0), np.full(4, 1e7), np.full(4, 1e6))
        assert not np.any(pre & ~keeps), v
