"""The seeded synthetic workloads have the shapes, sizes and distributions of
the benchmark configurations (no dataset is involved anywhere)."""
import numpy as np

import gala_gb300 as g
from gala_gb300 import workloads as W


def test_config1_hernquist_ics():
    w = W.hernquist_ics()
    assert w.shape == (6, 1024)
    r = np.linalg.norm(w[:3], axis=0)
    assert r.min() >= 5.0 and r.max() <= 20.0
    vc = np.sqrt(g.units.G * 1e11 * r / (r + 1.0) ** 2)
    ratio = np.linalg.norm(w[3:], axis=0) / vc
    assert abs(np.median(ratio) - 1.0) < 0.05
    # tangential before the per-component scatter: small radial component on average
    cosang = np.sum(w[:3] * w[3:], axis=0) / (r * np.linalg.norm(w[3:], axis=0))
    assert abs(np.mean(cosang)) < 0.02 and np.std(cosang) < 0.15


def test_config2_mw_composite_and_ics(oracle):
    pot = W.mw_composite()
    kinds = [type(c).__name__ for c in pot.values()]
    assert kinds == ["HernquistPotential", "HernquistPotential", "MiyamotoNagaiPotential", "NFWPotential"]
    w = W.mw_ics(20000)
    assert w.shape == (6, 20000)
    R = np.hypot(w[0], w[1])
    assert R.min() >= 2.0 and R.max() <= 30.0 and np.abs(w[2]).max() <= 2.0
    # the closed-form circular speed used for the ICs is the composite's own
    Rs = np.linspace(2.0, 30.0, 15)
    grad = oracle.gradient(pot, np.stack([Rs, np.zeros(15), np.zeros(15)]))
    np.testing.assert_allclose(W._mw_vcirc_numpy(Rs), np.sqrt(Rs * grad[0]), rtol=1e-12)
    # v = v_c phi_hat + isotropic N(0, 30 km/s)
    phi = np.arctan2(w[1], w[0])
    vt = -w[3] * np.sin(phi) + w[4] * np.cos(phi)
    sig = 30.0 * g.units.KMS_TO_KPC_MYR
    np.testing.assert_allclose(np.mean(vt - W._mw_vcirc_numpy(R)), 0.0, atol=3 * sig / np.sqrt(20000))
    np.testing.assert_allclose(np.std(w[5]), sig, rtol=0.03)


def test_config3_uneven_steps():
    nsteps, dt, method = W.uneven_steps()
    assert nsteps.shape == dt.shape == method.shape == (262144,)
    assert nsteps.min() >= 100 and nsteps.max() <= 20000
    assert abs(np.median(np.log(nsteps)) - 0.5 * np.log(100 * 20000)) < 0.02
    assert abs(nsteps.sum() / 9.85e8 - 1.0) < 0.01
    assert set(np.unique(dt)) == {0.1, 0.5, 1.0}
    assert int(method.sum()) == 131072


def test_config4_scf_coefficients():
    S, T = W.scf_coefficients()
    assert S.shape == T.shape == (13, 9, 9)
    assert S[0, 0, 0] == 1.0
    n = np.arange(13)[:, None, None]
    l = np.arange(9)[None, :, None]
    m = np.arange(9)[None, None, :]
    zero = np.broadcast_to(m > l, S.shape)
    assert np.all(S[zero] == 0) and np.all(T[zero] == 0) and np.all(T[:, :, 0] == 0)
    # the free coefficients are N(0, 1) draws scaled by exp(-n/2) (l + 1)^-2
    amp = np.broadcast_to(np.exp(-0.5 * n) * (l + 1.0) ** -2, S.shape)
    free_s = ~zero.copy()
    free_s[0, 0, 0] = False
    free_t = ~zero & np.broadcast_to(m > 0, S.shape)
    z = np.concatenate([(S / amp)[free_s], (T / amp)[free_t]])
    assert z.size > 700
    assert abs(np.mean(z)) < 0.15 and abs(np.std(z) - 1.0) < 0.1


def test_config5_stream_progenitors():
    w0, m, b = W.stream_progenitors()
    assert w0.shape == (6, 512) and m.shape == b.shape == (512,)
    assert m.min() >= 1e4 and m.max() <= 1e6
    assert b.min() >= 5e-3 and b.max() <= 20e-3
    R = np.hypot(w0[0], w0[1])
    assert R.min() >= 2.0 and R.max() <= 30.0
