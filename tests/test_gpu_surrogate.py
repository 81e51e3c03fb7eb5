"""The learned potential surrogate on the GPU.

* training kernels: forward, input gradient and the parameter gradient of the
  value + input-gradient loss against the numpy FP64 oracle (oracle/mlp_oracle.py);
* Adam update against numpy;
* BF16 tensor-core inference against the FP64 oracle of the same network;
* a trained surrogate of an SCF halo: force accuracy, the analytic fallback,
  integrated orbits, and what it gains over the analytic SCF force.
"""
import time

import numpy as np
import pytest

import gala_gb300 as g
from gala_gb300 import surrogate as S
from gala_gb300 import workloads as W
from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scf():
    return W.scf_potential(nmax=6, lmax=4)


def _random_batch(B, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1, 1, (B, 3)).astype(np.float32)
    ys = rng.normal(0, 0.3, B).astype(np.float32)
    Gs = rng.normal(0, 0.3, (B, 3)).astype(np.float32)
    return X, ys, Gs


def test_forward_and_train_step_match_oracle(scf):
    import torch

    from gala_gb300 import _abi

    sp = S.SurrogatePotential(scf, seed=3)
    p = sp.params.cpu().numpy().astype(np.float64)
    X, ys, Gs = _random_batch(96, 4)
    y, G = sp.forward_fp32(torch.from_numpy(X))
    y_ref, G_ref, _ = M.forward(p, X.astype(np.float64))
    np.testing.assert_allclose(y.cpu().numpy(), y_ref, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(G.cpu().numpy(), G_ref, rtol=1e-4, atol=1e-5)

    dev = sp.dev
    grads = torch.zeros_like(sp.params)
    ws = torch.empty(int(_abi.load().gx_mlp_train_workspace_floats(96)), dtype=torch.float32, device=dev)
    loss = torch.zeros(2, dtype=torch.float32, device=dev)
    Xd, yd, Gd = (torch.from_numpy(a).to(dev) for a in (X, ys, Gs))
    import ctypes as C

    _abi.call("gx_mlp_train_step", sp.params.data_ptr(), grads.data_ptr(), Xd.data_ptr(), yd.data_ptr(),
              Gd.data_ptr(), None, 96, C.c_float(0.8), C.c_float(1.2), ws.data_ptr(), loss.data_ptr(), None)
    L, gref = M.loss_and_grad(p, X.astype(np.float64), ys.astype(np.float64), Gs.astype(np.float64), 0.8, 1.2)
    gk = grads.cpu().numpy()
    scale = np.abs(gref).max()
    assert np.max(np.abs(gk - gref)) <= 2e-4 * scale, np.max(np.abs(gk - gref)) / scale
    Lk = 0.8 * loss[0].item() + 1.2 * loss[1].item()
    assert abs(Lk - L) <= 1e-4 * abs(L)


def test_adam_matches_numpy():
    import ctypes as C

    import torch

    from gala_gb300 import _abi

    rng = np.random.default_rng(5)
    n = 1000
    p, gr = rng.normal(size=n).astype(np.float32), rng.normal(size=n).astype(np.float32)
    m, v = rng.normal(size=n).astype(np.float32) * 0.1, rng.uniform(0, 1, n).astype(np.float32)
    tp, tg, tm, tv = (torch.from_numpy(a.copy()).cuda() for a in (p, gr, m, v))
    _abi.call("gx_mlp_adam", tp.data_ptr(), tg.data_ptr(), tm.data_ptr(), tv.data_ptr(), n, C.c_float(1e-3),
              C.c_float(0.9), C.c_float(0.999), C.c_float(1e-8), 7, None)
    m2 = 0.9 * m + 0.1 * gr
    v2 = 0.999 * v + 0.001 * gr * gr
    p2 = p - 1e-3 * (m2 / (1 - 0.9 ** 7)) / (np.sqrt(v2 / (1 - 0.999 ** 7)) + 1e-8)
    np.testing.assert_allclose(tp.cpu().numpy(), p2, rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("engine,split", [("tcgen05", 3), ("tcgen05", 2), ("mma", 2)])
def test_tensor_core_inference_matches_fp64_network(scf, engine, split):
    """The tensor-core kernels (tcgen05 with TMEM accumulators, and warp-level
    mma.sync) evaluate the same function as the FP64 oracle of the network (to
    the precision of their operands: FP16, or BF16 weights with BF16 hi + lo
    activations).  FP16 operands carry 11-bit weights against BF16's 8, so the
    FP16 mode is held to a 2x tighter bound."""
    sp = S.SurrogatePotential(scf, seed=6, split=split)
    sp.export()
    x = sp.sample_positions(3000, seed=7)
    grad, phi = sp.gradient_and_energy(x, engine=engine)
    xd = x.cpu().numpy()
    xh, r, n, rho, drho = S.input_map(xd, sp.r_min, sp.r_max)
    p = sp.params.cpu().numpy().astype(np.float64)
    y, Gx, _ = M.forward(p, xh.T)
    phiH = -sp.GM / (r + sp.r_s)
    dphiH = sp.GM / (r + sp.r_s) ** 2
    phi0, dphi0 = S.scf_l0(scf, r)
    ng = np.sum(n * Gx.T, axis=0)
    J = (rho / r) * (Gx.T - n * ng) + drho * n * ng
    grad_ref = (dphi0 + dphiH * y) * n + phiH * J
    phi_ref = phi0 + phiH * y
    err = np.linalg.norm(grad.cpu().numpy() - grad_ref, axis=0) / np.linalg.norm(grad_ref, axis=0)
    # weights are FP16 / BF16 in the kernel, FP64 in the oracle
    bound = 5e-3 if split == 3 else 1e-2
    assert np.median(err) < bound, np.median(err)
    # (an untrained network can make Phi cross zero, so compare on the global scale)
    np.testing.assert_allclose(phi.cpu().numpy(), phi_ref, rtol=0, atol=1e-3 * np.abs(phi_ref).max())


def test_spherical_base_matches_scf_monopole(scf, oracle):
    """Phi_0 of the surrogate equals the l = 0 terms of the analytic SCF."""
    S0 = np.zeros_like(scf.parameters["Snlm"])
    S0[:, 0, 0] = scf.parameters["Snlm"][:, 0, 0]
    mono = g.SCFPotential(m=scf.parameters["m"], r_s=scf.parameters["r_s"], Snlm=S0, Tnlm=np.zeros_like(S0))
    r = np.geomspace(0.5, 200, 50)
    q = np.vstack([r * 0.6, r * 0.0 + 1e-3, r * 0.8])
    rr = np.linalg.norm(q, axis=0)
    phi0, dphi0 = S.scf_l0(scf, rr)
    np.testing.assert_allclose(phi0, oracle.energy(mono, q), rtol=1e-10)
    gr = oracle.gradient(mono, q)
    np.testing.assert_allclose(dphi0, np.sum(gr * q, axis=0) / rr, rtol=1e-8)


def test_fallback_outside_trained_radii(scf, oracle):
    sp = S.SurrogatePotential(scf, r_min=0.5, r_max=200.0, seed=8)
    q = np.array([[0.2, 0.0, 0.1], [300.0, 10.0, -5.0], [0.0, 250.0, 1.0]]).T
    grad, _ = sp.gradient_and_energy(q)
    ref = oracle.gradient(scf, q)
    np.testing.assert_allclose(grad.cpu().numpy(), ref, rtol=1e-4)


def test_trained_surrogate_accuracy(scf, oracle):
    """A short training run on the small SCF halo: the loss falls, and force and
    potential reach the accuracy this network class reaches at that length
    (median force error < 2e-2, potential < 2e-3; the config-4 network trained
    30,000 steps reaches ~3e-3 and ~2e-4, see the bench)."""
    sp = S.SurrogatePotential(scf, seed=9)
    sp.make_dataset(n_samples=1 << 20)
    hist = sp.train(steps=1500, batch=8192, log_every=500)
    assert hist[-1][1] < hist[0][1]
    x = sp.sample_positions(20000, seed=10)
    grad, phi = sp.gradient_and_energy(x)
    xh = x.cpu().numpy()
    ref = scf.gradient(xh)
    err = np.linalg.norm(grad.cpu().numpy() - ref, axis=0) / np.linalg.norm(ref, axis=0)
    assert np.median(err) < 2e-2, np.median(err)
    perr = np.abs(phi.cpu().numpy() - scf.energy(xh)) / np.abs(scf.energy(xh))
    assert np.median(perr) < 2e-3, np.median(perr)


def test_surrogate_gain_at_equal_accuracy():
    """What the trained network gains over the method without it, at equal
    accuracy, both timed on the GPU: the config-4 SCF host (nmax 12, lmax 8)
    and its surrogate after a short training; the analytic SCF cut at the
    lowest degree L whose force error is no larger than the surrogate's is the
    method without the network at the same accuracy.  The surrogate's FP32
    leapfrog must outrun that analytic leapfrog."""
    import torch

    full = W.scf_potential()
    sp = S.SurrogatePotential(full, seed=21)
    sp.make_dataset(n_samples=1 << 21)
    sp.train(steps=3000, batch=8192, log_every=1000)
    x = sp.sample_positions(20000, seed=22)
    xh = x.cpu().numpy()
    ref = full.gradient(xh)

    def ferr(gr):
        return np.median(np.linalg.norm(gr - ref, axis=0) / np.linalg.norm(ref, axis=0))

    e_sur = ferr(sp.gradient_and_energy(x)[0].cpu().numpy())
    cut = None
    for L in range(full.lmax + 1):
        if ferr(S.truncated_scf(full, L).gradient(xh)) <= e_sur:
            cut = S.SurrogatePotential(S.truncated_scf(full, L), seed=0)
            break
    assert cut is not None and cut.scf.lmax < full.lmax, "the surrogate should be worth a truncation"
    w0 = W.scf_ics(1 << 16, seed=23)

    def rate(fn):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return (1 << 16) * 50 / (time.perf_counter() - t0)

    v_sur = rate(lambda: sp.integrate_leapfrog(w0, 1.0, 50))
    v_cut = rate(lambda: cut.integrate_leapfrog(w0, 1.0, 50, analytic=True))
    assert v_sur > v_cut, (v_sur, v_cut, cut.scf.lmax, e_sur)


def test_surrogate_leapfrog_runs_and_matches_fp32_forces(scf):
    sp = S.SurrogatePotential(scf, seed=12)
    sp.export()
    w0 = W.scf_ics(200, seed=13)
    out, fb = sp.integrate_leapfrog(w0, dt=1.0, n_steps=50)
    o = out.cpu().numpy()
    assert np.isfinite(o).all()
    assert not np.array_equal(o, w0)
    assert int(fb.item()) == 0


def test_tcgen05_matches_mma_engine(scf):
    """Both tensor-core engines run BF16 weights with BF16 hi + lo activations
    and FP32 accumulation; they differ in accumulation order and in the SiLU
    (the tcgen05 kernel uses tanh.approx, relative error ~2^-11), both below
    the BF16 weight rounding.  Sizes that are not a multiple of the 128-row
    tile exercise the partial last tile."""
    sp = S.SurrogatePotential(scf, seed=8, split=2)
    sp.export()
    for n in (1, 127, 129, 5000):
        x = sp.sample_positions(n, seed=9)
        g_tc, p_tc = sp.gradient_and_energy(x, engine="tcgen05")
        g_mm, p_mm = sp.gradient_and_energy(x, engine="mma")
        d = np.linalg.norm((g_tc - g_mm).cpu().numpy(), axis=0) / np.linalg.norm(g_mm.cpu().numpy(), axis=0)
        assert np.median(d) < 1e-3 and np.max(d) < 2e-2, (n, np.median(d), np.max(d))
        np.testing.assert_allclose(p_tc.cpu().numpy(), p_mm.cpu().numpy(), rtol=0,
                                   atol=1e-3 * np.abs(p_mm.cpu().numpy()).max())


def test_tcgen05_leapfrog_matches_mma_leapfrog(scf):
    sp = S.SurrogatePotential(scf, seed=10, split=2)
    sp.export()
    w0 = W.scf_ics(700, seed=11)
    o_tc, fb_tc = sp.integrate_leapfrog(w0, 1.0, 50, engine="tcgen05")
    o_mm, fb_mm = sp.integrate_leapfrog(w0, 1.0, 50, engine="mma")
    err = np.linalg.norm((o_tc - o_mm)[:3].cpu().numpy(), axis=0) / np.linalg.norm(o_mm[:3].cpu().numpy(), axis=0)
    assert np.median(err) < 1e-4, np.median(err)
    assert int(fb_tc.item()) == int(fb_mm.item())



def test_integrate_orbit_with_surrogate_and_file_round_trip(scf, tmp_path):
    """The surrogate through the drop-in call: integrate_orbit with
    Integrator_kwargs surrogate= (an object or a saved file), snapshots every
    out_stride steps, equal to the same chunked run through the surrogate's own
    call; refused for other integrators."""
    import torch

    sp = S.SurrogatePotential(scf, seed=14)
    sp.export()
    w0 = W.scf_ics(300, seed=15)
    o = scf.integrate_orbit(w0, dt=1.0, n_steps=40, Integrator="leapfrog",
                            Integrator_kwargs=dict(surrogate=sp, out_stride=10))
    w = o.w()
    assert w.shape == (6, 5, 300)
    np.testing.assert_array_equal(o.t, np.arange(0.0, 41.0, 10.0))
    np.testing.assert_array_equal(w[:, 0], w0)
    wd = torch.from_numpy(w0).cuda()
    for _ in range(4):
        wd, _ = sp.integrate_leapfrog(wd, 1.0, 10)
    np.testing.assert_array_equal(w[:, -1], wd.cpu().numpy())
    path = tmp_path / "surrogate.npz"
    sp.save(path)
    o2 = scf.integrate_orbit(w0, dt=1.0, n_steps=40, Integrator="leapfrog",
                             Integrator_kwargs=dict(surrogate=str(path), out_stride=10))
    np.testing.assert_array_equal(o2.w(), w)
    last = scf.integrate_orbit(w0, dt=1.0, n_steps=40, Integrator="leapfrog",
                               Integrator_kwargs=dict(surrogate=sp), save_all=False)
    assert last.w().shape == (6, 1, 300)
    with pytest.raises(ValueError, match="LeapfrogIntegrator"):
        scf.integrate_orbit(w0, dt=1.0, n_steps=4, Integrator="dop853", Integrator_kwargs=dict(surrogate=sp))
