"""GPU parity of the direct n-body and mock-stream kernels against the oracle
(itself pinned bit for bit to gala's own dop853 / Fwrapper_direct_nbody /
mockstream loop, tests/test_mockstream_oracle.py).

Tolerances
  * external potential and bodies made of sqrt / division only (Hernquist,
    Plummer): every right-hand side and every error / stiffness norm is
    computed in the oracle's order (sequential norms in gala's component order,
    no contraction); the one difference is the step-size factor pow(err, 1/8),
    where CUDA's pow and glibc's may differ by an ulp, so states agree to 1e-13
    of their scale;
  * the Milky-Way composite (pow in Miyamoto-Nagai, log in NFW): CUDA's and
    glibc's pow/log may differ by an ulp; states agree to 1e-11 of their scale;
  * the Fardal sampler takes d2Phi/dr2 as a second difference of Phi with the
    fixed step h = 0.01 kpc (c_d2_dr2): an ulp of Phi (~1e-17 kpc^2/Myr^2)
    over h^2 = 1e-4 against d2Phi/dr2 ~ 1e-4 Myr^-2 is ~1e-9 relative, so
    release offsets from the progenitor agree to 2e-9 of their scale;
  * stiffness exits (hlamb > 6.1 after an accepted step) are decided on
    quantities whose last bits differ between any two builds: gala's own -Ofast
    and strict builds disagree on one of the eight systems of the stiffness
    case, so that test bounds the number of differing decisions.
"""
import numpy as np
import pytest

import gala_gb300 as g
from gala_gb300 import _abi
from gala_gb300 import workloads as W
from gala_gb300.mockstream import FardalStreamDF, MockStreamGenerator
from gala_gb300.nbody import DirectNBody, bodies_to_device, integrate_systems, pack_bodies

from ._cases import stream_case

pytestmark = pytest.mark.gpu

MW_TOL = 1e-11
EXACT_OPS_TOL = 1e-13


def _scale_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _release_systems_gpu(c, pot=None, stats=False):
    """gx_mockstream_dop853 on a stream_case's release stage."""
    import torch

    from gala_gb300._device import ptr, stream_handle

    pot = c["pot"] if pot is None else pot
    dev = torch.device("cuda")
    rel = c["rel"]
    t = c["t"]
    S = c["stream_w0"].shape[0]
    nbody_w = torch.from_numpy(np.ascontiguousarray(c["orbits"][:, rel])).to(dev)
    sw0 = torch.from_numpy(np.ascontiguousarray(c["stream_w0"])).to(dev)
    rt = torch.from_numpy(np.ascontiguousarray(t[rel])).to(dev)
    off = torch.from_numpy(np.concatenate([[0], np.cumsum(c["nstream"])]).astype(np.int64)).to(dev)
    out = torch.empty_like(sw0)
    nb_out = torch.empty((S, 1, 6), dtype=torch.float64, device=dev)
    status = torch.zeros((S, len(rel)), dtype=torch.int32, device=dev)
    st = torch.zeros((S, len(rel), 4), dtype=torch.int64, device=dev)
    counter = torch.zeros(1, dtype=torch.int64, device=dev)
    bd = bodies_to_device(c["bodies"], dev)
    H = g.Hamiltonian(pot)
    _abi.call("gx_mockstream_dop853", pot.packed().for_device(), H._frame_ref(), S, 1, ptr(bd), ptr(nbody_w),
              len(rel), ptr(rt), ptr(off), int(c["nstream"].max()), ptr(sw0), int(sw0.shape[1]), float(t[-1]),
              float(t[rel][1] - t[rel][0]), 1e-10, 1e-10, 0, ptr(out), ptr(nb_out), ptr(status), ptr(st),
              ptr(counter), stream_handle())
    torch.cuda.synchronize()
    res = (out.cpu().numpy(), nb_out.cpu().numpy(), status.cpu().numpy())
    return res + (st.cpu().numpy(),) if stats else res


def _oracle_release(oracle, c, pot=None):
    pot = c["pot"] if pot is None else pot
    rel, t = c["rel"], c["t"]
    return oracle.mockstream_systems(pot, c["bodies"], c["orbits"][:, rel], t[rel], c["nstream"], c["stream_w0"],
                                     t[-1], t[rel][1] - t[rel][0], nthreads=8)


# ----------------------------------------------------------- direct n-body
def _nbody_batch(n_sys=5):
    pots = [g.PlummerPotential(m=2e9, b=0.4), g.HernquistPotential(m=5e9, c=1.0), None, None]
    bodies = pack_bodies([pots[:2]] * n_sys)
    w0 = np.stack([np.ascontiguousarray(W.mw_ics(4, seed=40 + s).T) for s in range(n_sys)])
    w0[:, 1, :3] = w0[:, 0, :3] + np.array([1.0, 0.5, -0.2])
    t = g.parse_time_specification(dt=1.0, n_steps=200)
    return bodies, w0, t


@pytest.mark.parametrize("ext", ["hernquist", "mw"])
def test_nbody_systems_match_oracle(oracle, ext):
    pot = g.HernquistPotential(m=1e11, c=1.0) if ext == "hernquist" else W.mw_composite()
    bodies, w0, t = _nbody_batch()
    out, status = integrate_systems(pot, bodies, w0, t, nstiff=-1)
    out = out.cpu().numpy()
    assert np.all(status.cpu().numpy() == 1)
    for s in range(w0.shape[0]):
        ref, res = oracle.nbody_dop853(pot, np.concatenate([bodies[s], pack_bodies([None, None])]), 2, w0[s], t)
        assert res == 1
        assert _scale_err(out[s], ref) < (EXACT_OPS_TOL if ext == "hernquist" else MW_TOL)


def test_nbody_final_state_and_stride(oracle):
    pot = W.mw_composite()
    bodies, w0, t = _nbody_batch(3)
    full, _ = integrate_systems(pot, bodies, w0, t)
    strided, _ = integrate_systems(pot, bodies, w0, t, out_stride=7)
    final, _ = integrate_systems(pot, bodies, w0, t, save_all=False)
    full = full.cpu().numpy()
    np.testing.assert_array_equal(strided.cpu().numpy(), full[:, ::7])
    # the last stored row is the dense-output polynomial at s = 1, y_old + (y_new - y_old),
    # which can differ from y_new by an ulp (in gala as well)
    np.testing.assert_allclose(final.cpu().numpy(), full[:, -1], rtol=1e-15, atol=1e-300)


def test_directnbody_api_reorders_like_gala(oracle):
    """Null-potential bodies listed first are moved behind the massive ones for
    the integration and put back afterwards (core.py:211-280)."""
    pot = W.mw_composite()
    pps = [None, g.PlummerPotential(m=2e9, b=0.4), None, g.HernquistPotential(m=5e9, c=1.0)]
    w0 = W.mw_ics(4, seed=50)
    w0[:3, 3] = w0[:3, 1] + np.array([0.8, -0.4, 0.1])
    nb = DirectNBody(g.PhaseSpacePosition.from_w(w0), pps, external_potential=pot)
    orbit = nb.integrate_orbit(dt=1.0, n_steps=150)
    t = g.parse_time_specification(dt=1.0, n_steps=150)
    idx = np.array([1, 3, 0, 2])
    ref, res = oracle.nbody_dop853(pot, pack_bodies([pps[i] for i in idx]), 2, w0[:, idx].T, t)
    ref = ref[:, np.argsort(idx)]  # (ntimes, nbodies, 6)
    got = orbit.w()  # (6, ntimes, nbodies)
    assert got.shape == (6, len(t), 4)
    assert _scale_err(np.moveaxis(got, 0, -1), ref) < MW_TOL


# ------------------------------------------------------------ release systems
def test_release_systems_hernquist(oracle):
    pot = g.HernquistPotential(m=1e11, c=1.0)
    c = stream_case(n_streams=3, n_steps=120)
    # progenitor orbits and release states in this potential (oracle)
    c = _restage(oracle, c, pot)
    out, nb_out, status = _release_systems_gpu(c, pot)
    ref_out, ref_nb, ref_status, _ = _oracle_release(oracle, c, pot)
    np.testing.assert_array_equal(status, ref_status)
    assert _scale_err(out, ref_out) < EXACT_OPS_TOL
    assert _scale_err(nb_out, ref_nb) < EXACT_OPS_TOL


def test_release_systems_match_oracle_mw(oracle):
    c = stream_case(n_streams=4, n_steps=200)
    out, nb_out, status, stats = _release_systems_gpu(c, stats=True)
    ref_out, ref_nb, ref_status, ref_stats = _oracle_release(oracle, c)
    np.testing.assert_array_equal(status, ref_status)
    assert np.all(status[:, c["nstream"] > 0] == 1)
    assert _scale_err(out, ref_out) < MW_TOL
    assert _scale_err(nb_out, ref_nb) < MW_TOL
    # the step sequences agree (accepted steps per system)
    np.testing.assert_array_equal(stats[..., 2], ref_stats[..., 2])


def test_release_systems_several_per_release(oracle):
    """Two particles per tail (5-lane systems) released every 3rd step."""
    c = stream_case(n_streams=2, n_steps=90, n_per_tail=2, release_every=3)
    # the bodies on the release grid, as mockstream_dop853 re-integrates them
    rel, t = c["rel"], c["t"]
    for s in range(2):
        ob, _ = oracle.nbody_dop853(c["pot"], c["bodies"][s], 1, c["w0"][:, s].reshape(1, 6), t[rel])
        c["orbits"][s, rel] = ob
    out, nb_out, status = _release_systems_gpu(c)
    ref_out, ref_nb, ref_status, _ = _oracle_release(oracle, c)
    np.testing.assert_array_equal(status, ref_status)
    assert _scale_err(out, ref_out) < MW_TOL


def _restage(oracle, c, pot):
    """Recompute a stream_case's progenitor orbits and release states in `pot`."""
    t = c["t"]
    df = FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(c["seed"]))
    orbits, sw0 = [], []
    for s in range(c["bodies"].shape[0]):
        orb, res = oracle.nbody_dop853(pot, c["bodies"][s], 1, c["w0"][:, s].reshape(1, 6), t)
        assert res == 1
        orbits.append(orb)
        draws = df._draws(int(c["offset"][-1]))
        sw0.append(oracle.fardal_sample(pot, orb.reshape(len(t), 6), np.full(len(t), c["m"][s]), t, c["offset"],
                                        draws, g.units.G))
    c = dict(c)
    c["orbits"] = np.stack(orbits)
    c["stream_w0"] = np.stack(sw0)
    return c


# ------------------------------------------------------------------ sampler
def test_fardal_sampler_matches_oracle(oracle):
    import torch

    c = stream_case(n_streams=3, n_steps=100)
    t = c["t"]
    S = c["orbits"].shape[0]
    df = FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(c["seed"]))
    prog_w = torch.from_numpy(np.ascontiguousarray(c["orbits"].reshape(S, len(t), 6))).cuda()
    m = np.repeat(c["m"][:, None], len(t), axis=1)
    w, rt, lt, off = df.sample_device(c["pot"], prog_w, t, m, c["counts"])
    w = w.cpu().numpy()
    np.testing.assert_array_equal(off, c["offset"])
    for s in range(S):
        rel = w[s] - np.repeat(c["orbits"][s, :, 0], 2 * c["counts"], axis=0)
        ref = c["stream_w0"][s] - np.repeat(c["orbits"][s, :, 0], 2 * c["counts"], axis=0)
        assert _scale_err(rel, ref) < 2e-9
    assert lt[0] == "t" and lt[1] == "l" and len(lt) == w.shape[1]
    np.testing.assert_array_equal(rt, np.repeat(t, 2 * c["counts"]))


def test_streakline_sampler_matches_oracle(oracle):
    """The streakline DF runs the same GPU sampler with constant placement."""
    import torch

    from gala_gb300.mockstream import StreaklineStreamDF

    c = stream_case(n_streams=2, n_steps=60)
    t = c["t"]
    S = c["orbits"].shape[0]
    df = StreaklineStreamDF()
    prog_w = torch.from_numpy(np.ascontiguousarray(c["orbits"].reshape(S, len(t), 6))).cuda()
    m = np.repeat(c["m"][:, None], len(t), axis=1)
    w, rt, lt, off = df.sample_device(c["pot"], prog_w, t, m, c["counts"])
    w = w.cpu().numpy()
    for s in range(S):
        ref = oracle.fardal_sample(c["pot"], c["orbits"][s].reshape(len(t), 6), m[s], t, off,
                                   df._draws(int(off[-1])), g.units.G)
        base = np.repeat(c["orbits"][s, :, 0], 2 * c["counts"], axis=0)
        assert _scale_err(w[s] - base, ref - base) < 2e-9


@pytest.mark.parametrize("kind", [1, 2])
def test_lagrange_cloud_and_chen_samplers_match_oracle(oracle, kind):
    """The Lagrange-cloud (kind 1) and Chen (kind 2) DFs on the GPU sampler."""
    import torch

    from gala_gb300.mockstream import ChenStreamDF, LagrangeCloudStreamDF

    c = stream_case(n_streams=2, n_steps=60)
    t = c["t"]
    S = c["orbits"].shape[0]
    df = (LagrangeCloudStreamDF(v_disp=1.5, random_state=np.random.RandomState(7)) if kind == 1
          else ChenStreamDF(random_state=np.random.RandomState(7)))
    prog_w = torch.from_numpy(np.ascontiguousarray(c["orbits"].reshape(S, len(t), 6))).cuda()
    m = np.repeat(c["m"][:, None], len(t), axis=1)
    w, rt, lt, off = df.sample_device(c["pot"], prog_w, t, m, c["counts"])
    w = w.cpu().numpy()
    rs = np.random.RandomState(7)  # the draws of stream s follow those of streams 0..s-1
    df_ref = (LagrangeCloudStreamDF(v_disp=1.5, random_state=rs) if kind == 1 else ChenStreamDF(random_state=rs))
    for s in range(S):
        draws = df_ref._draws(int(off[-1]))
        ref = oracle.stream_sample(c["pot"], c["orbits"][s].reshape(len(t), 6), m[s], t, off, kind, draws, g.units.G)
        base = np.repeat(c["orbits"][s, :, 0], 2 * c["counts"], axis=0)
        assert _scale_err(w[s] - base, ref - base) < 2e-9


# ---------------------------------------------------------------- generator
def _oracle_run(oracle, pot, prog_pot, w0, m, t, seed, release_every=1, n_per_tail=1, df=None, kind=0):
    """gala's MockStreamGenerator.run with the oracle for every numerical step
    (FardalStreamDF unless another DF and its sampler kind are given)."""
    bodies = pack_bodies([prog_pot])
    orb, res = oracle.nbody_dop853(pot, bodies, 1, w0.reshape(1, 6), t)
    assert res == 1
    orbit_t = t
    if t[1] < t[0]:
        orb = orb[::-1].copy()
        orbit_t = t[::-1].copy()
    if df is None:
        df = FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(seed))
    counts = df.release_counts(len(t), release_every, n_per_tail)
    offset = np.concatenate([[0], np.cumsum(2 * counts)]).astype(np.int64)
    sw0 = oracle.stream_sample(pot, orb.reshape(len(t), 6), np.full(len(t), m), orbit_t, offset, kind,
                               df._draws(int(offset[-1])), g.units.G)
    rel = np.nonzero(counts > 0)[0]
    if 0 not in rel:
        rel = np.insert(rel, 0, 0)
    nb, st, status = oracle.mockstream_dop853(pot, bodies, orb[0].reshape(1, 6), orbit_t[rel], sw0, orbit_t[rel],
                                              orbit_t[-1], 2 * counts[rel])
    return st, nb


@pytest.mark.parametrize("case", ["forward", "backward", "release_every"])
def test_generator_run_matches_oracle(oracle, case):
    pot = W.mw_composite()
    w0 = W.mw_ics(1, seed=60)[:, 0]
    prog_pot = g.PlummerPotential(m=2e5, b=0.01)
    kw = dict(dt=1.0, n_steps=150)
    extra = {}
    if case == "backward":
        kw = dict(dt=-1.0, n_steps=150)
    if case == "release_every":
        extra = dict(release_every=4, n_particles=3)
    gen = MockStreamGenerator(FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(7)),
                              g.Hamiltonian(pot), progenitor_potential=prog_pot)
    stream, nbody = gen.run(g.PhaseSpacePosition.from_w(w0), 2e5, **extra, **kw)
    t = g.parse_time_specification(**kw)
    ref_st, ref_nb = _oracle_run(oracle, pot, prog_pot, w0, 2e5, t, 7, extra.get("release_every", 1),
                                 extra.get("n_particles", 1))
    got = np.vstack([stream.xyz, stream.v_xyz]).T
    assert got.shape == ref_st.shape
    assert _scale_err(got, ref_st) < 1e-10
    assert _scale_err(np.vstack([nbody.xyz, nbody.v_xyz]).T, ref_nb) < 1e-10
    assert set(np.unique(stream.lead_trail)) == {"t", "l"}


@pytest.mark.parametrize("which", ["streakline", "lagrange", "chen"])
def test_generator_with_other_dfs_matches_oracle(oracle, which):
    """Whole runs with the streakline, Lagrange-cloud and Chen DFs against the
    oracle.  These release particles at the Jacobi radius itself (Fardal's sit
    near 2 r_J), where the progenitor's pull amplifies the ulp-level
    differences of the force forms more: 1e-9 of the stream's extent
    (measured 1.2e-10 and 1.6e-10 for the first two)."""
    from gala_gb300.mockstream import ChenStreamDF, LagrangeCloudStreamDF, StreaklineStreamDF

    def make(seed):
        rs = np.random.RandomState(seed)
        return {"streakline": lambda: StreaklineStreamDF(random_state=rs),
                "lagrange": lambda: LagrangeCloudStreamDF(v_disp=1.0, random_state=rs),
                "chen": lambda: ChenStreamDF(random_state=rs)}[which]()

    kind = {"streakline": 0, "lagrange": 1, "chen": 2}[which]
    pot = W.mw_composite()
    w0 = W.mw_ics(1, seed=61)[:, 0]
    prog_pot = g.PlummerPotential(m=2e5, b=0.01)
    kw = dict(dt=1.0, n_steps=120)
    gen = MockStreamGenerator(make(9), g.Hamiltonian(pot), progenitor_potential=prog_pot)
    stream, nbody = gen.run(g.PhaseSpacePosition.from_w(w0), 2e5, **kw)
    t = g.parse_time_specification(**kw)
    ref_st, ref_nb = _oracle_run(oracle, pot, prog_pot, w0, 2e5, t, 9, df=make(9), kind=kind)
    got = np.vstack([stream.xyz, stream.v_xyz]).T
    assert got.shape == ref_st.shape
    assert _scale_err(got, ref_st) < 1e-9
    assert _scale_err(np.vstack([nbody.xyz, nbody.v_xyz]).T, ref_nb) < 1e-10


def test_run_batch_equals_sequential_runs():
    pot = W.mw_composite()
    w0, m, b = W.stream_progenitors(3, seed=70)
    pots = W.stream_progenitor_potentials(m, b)
    gen = MockStreamGenerator(FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(3)),
                              g.Hamiltonian(pot))
    res = gen.run_batch(w0, m, progenitor_potentials=pots, dt=1.0, n_steps=80)
    df = FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(3))
    for s in range(3):
        gen1 = MockStreamGenerator(df, g.Hamiltonian(pot), progenitor_potential=pots[s])
        st, nb = gen1.run(g.PhaseSpacePosition.from_w(w0[:, s]), m[s], dt=1.0, n_steps=80)
        one = res.stream(s)
        np.testing.assert_array_equal(one.xyz, st.xyz)
        np.testing.assert_array_equal(one.v_xyz, st.v_xyz)
        np.testing.assert_array_equal(res.nbody(s).xyz, nb.xyz)


def test_stream_edge_cases():
    pot = W.mw_composite()
    w0 = W.mw_ics(1, seed=61)[:, 0]
    gen = MockStreamGenerator(FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(1)),
                              g.Hamiltonian(pot), progenitor_potential=g.PlummerPotential(m=1e5, b=0.01))
    # no release at t0 (a zero-count first entry is inserted, as gala does) and a
    # release at the very last time (integrated over zero time: stays put)
    n = np.zeros(21, dtype=int)
    n[5] = 1
    n[-1] = 1
    stream, _ = gen.run(g.PhaseSpacePosition.from_w(w0), 1e5, n_particles=n, dt=1.0, n_steps=20)
    assert stream.xyz.shape == (3, 4)
    np.testing.assert_array_equal(stream.release_time, [5.0, 5.0, 20.0, 20.0])
    # leading tail only
    gen_l = MockStreamGenerator(FardalStreamDF(gala_modified=False, trail=False,
                                               random_state=np.random.RandomState(1)), g.Hamiltonian(pot))
    stream_l, _ = gen_l.run(g.PhaseSpacePosition.from_w(w0), 1e5, dt=1.0, n_steps=10)
    assert stream_l.xyz.shape == (3, 11) and set(stream_l.lead_trail) == {"l"}


def test_releases_wider_than_a_warp_match_oracle(oracle):
    """20 particles per tail at every time: 41-member DOP853 systems, one CTA
    each (gx_mockstream_dop853_wide), against the oracle's run."""
    pot = W.mw_composite()
    w0 = W.mw_ics(1, seed=62)[:, 0]
    prog_pot = g.PlummerPotential(m=2e5, b=0.01)
    gen = MockStreamGenerator(FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(7)),
                              g.Hamiltonian(pot), progenitor_potential=prog_pot)
    stream, nbody = gen.run(g.PhaseSpacePosition.from_w(w0), 2e5, dt=1.0, n_steps=40, n_particles=20)
    t = g.parse_time_specification(dt=1.0, n_steps=40)
    ref_st, ref_nb = _oracle_run(oracle, pot, prog_pot, w0, 2e5, t, 7, 1, 20)
    got = np.vstack([stream.xyz, stream.v_xyz]).T
    assert got.shape == ref_st.shape == (41 * 40, 6)
    assert _scale_err(got, ref_st) < 1e-9
    assert _scale_err(np.vstack([nbody.xyz, nbody.v_xyz]).T, ref_nb) < 1e-10


def test_stiffness_exit_matches_oracle(oracle):
    """dop853_step tests stiffness after every accepted step (nstiff = 1) and
    gala returns -4 at the first detection.  For this progenitor (m = 6.0e5,
    b = 16 pc on a disk orbit) three of the first eight release systems are
    stiff in the oracle's arithmetic over 2 Gyr (two or three in gala's own
    builds): with err_if_fail=1 the run raises gala's RuntimeError; with
    err_if_fail=0 the stiff systems keep their state at detection."""
    pot = W.mw_composite()
    w0, m, b = W.stream_progenitors(64, seed=1006)
    prog_pot = g.PlummerPotential(m=m[1], b=b[1])
    counts = np.zeros(2001, dtype=int)
    counts[:8] = 1

    def gen():
        return MockStreamGenerator(FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(1)),
                                   g.Hamiltonian(pot), progenitor_potential=prog_pot)

    psp = g.PhaseSpacePosition.from_w(w0[:, 1])
    with pytest.raises(RuntimeError, match="-4"):
        gen().run(psp, m[1], n_particles=counts, dt=1.0, n_steps=2000)
    res = gen().run_batch(w0[:, 1:2], m[1:2], progenitor_potentials=[prog_pot], n_particles=counts, dt=1.0,
                          n_steps=2000, Integrator_kwargs=dict(err_if_fail=0))
    status = res.status.cpu().numpy()[0]
    got = res.stream_w[0].cpu().numpy()
    t = g.parse_time_specification(dt=1.0, n_steps=2000)
    ref_st, ref_nb = _oracle_run(oracle, pot, prog_pot, w0[:, 1], m[1], t, 1, n_per_tail=counts)
    ref_status = _oracle_run_status(oracle, pot, prog_pot, w0[:, 1], m[1], t, 1, counts)
    assert np.sum(status == -4) >= 2
    assert np.sum(status != ref_status) <= 1, (status, ref_status)
    both_ok = np.repeat((status == 1) & (ref_status == 1), 2)
    assert _scale_err(got[both_ok], ref_st[both_ok]) < 1e-8


def _oracle_run_status(oracle, pot, prog_pot, w0, m, t, seed, counts):
    bodies = pack_bodies([prog_pot])
    orb, _ = oracle.nbody_dop853(pot, bodies, 1, w0.reshape(1, 6), t)
    df = FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(seed))
    offset = np.concatenate([[0], np.cumsum(2 * counts)]).astype(np.int64)
    sw0 = oracle.fardal_sample(pot, orb.reshape(len(t), 6), np.full(len(t), m), t, offset,
                               df._draws(int(offset[-1])), g.units.G)
    rel = np.nonzero(counts > 0)[0]
    _, _, status = oracle.mockstream_dop853(pot, bodies, orb[0].reshape(1, 6), t[rel], sw0, t[rel], t[-1],
                                            2 * counts[rel])
    return status


# ------------------------------------------------------------------ Leapfrog
def _release_leapfrog_gpu(c, pot=None, precision="fp64"):
    import torch

    from gala_gb300._device import ptr, stream_handle

    pot = c["pot"] if pot is None else pot
    dev = torch.device("cuda")
    rel, t = c["rel"], c["t"]
    S = c["stream_w0"].shape[0]
    nbody_w = torch.from_numpy(np.ascontiguousarray(c["orbits"][:, rel])).to(dev)
    sw0 = torch.from_numpy(np.ascontiguousarray(c["stream_w0"])).to(dev)
    rt = torch.from_numpy(np.ascontiguousarray(t[rel])).to(dev)
    off = torch.from_numpy(np.concatenate([[0], np.cumsum(c["nstream"])]).astype(np.int64)).to(dev)
    out = torch.empty_like(sw0)
    nb_out = torch.empty((S, 1, 6), dtype=torch.float64, device=dev)
    status = torch.zeros((S, len(rel)), dtype=torch.int32, device=dev)
    bd = bodies_to_device(c["bodies"], dev)
    name = "gx_mockstream_leapfrog" if precision == "fp64" else "gx_mockstream_leapfrog_fp32"
    _abi.call(name, pot.packed().for_device(), S, 1, ptr(bd), ptr(nbody_w), len(rel), ptr(rt), ptr(off),
              int(c["nstream"].max()), ptr(sw0), int(sw0.shape[1]), float(t[-1]), float(t[1] - t[0]), ptr(out),
              ptr(nb_out), ptr(status), stream_handle())
    torch.cuda.synchronize()
    return out.cpu().numpy(), nb_out.cpu().numpy(), status.cpu().numpy()


def _restage_leapfrog(oracle, c, pot):
    t = c["t"]
    df = FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(c["seed"]))
    orbits, sw0 = [], []
    for s in range(c["bodies"].shape[0]):
        orb = oracle.leapfrog_nbody(pot, c["bodies"][s], 1, c["w0"][:, s].reshape(1, 6), t)
        orbits.append(orb)
        sw0.append(oracle.fardal_sample(pot, orb.reshape(len(t), 6), np.full(len(t), c["m"][s]), t, c["offset"],
                                        df._draws(int(c["offset"][-1])), g.units.G))
    c = dict(c)
    c["orbits"] = np.stack(orbits)
    c["stream_w0"] = np.stack(sw0)
    return c


@pytest.mark.parametrize("ext", ["hernquist", "mw"])
def test_nbody_leapfrog_matches_oracle(oracle, ext):
    from gala_gb300.nbody import integrate_systems_leapfrog

    pot = g.HernquistPotential(m=1e11, c=1.0) if ext == "hernquist" else W.mw_composite()
    bodies, w0, t = _nbody_batch()
    out = integrate_systems_leapfrog(pot, bodies, w0, t).cpu().numpy()
    final = integrate_systems_leapfrog(pot, bodies, w0, t, save_all=False).cpu().numpy()
    np.testing.assert_array_equal(final, out[:, -1])
    for s in range(w0.shape[0]):
        ref = oracle.leapfrog_nbody(pot, np.concatenate([bodies[s], pack_bodies([None, None])]), 2, w0[s], t)
        if ext == "hernquist":
            np.testing.assert_array_equal(out[s], ref)
        else:
            assert _scale_err(out[s], ref) < 1e-11


def test_release_leapfrog_bit_exact_hernquist(oracle):
    pot = g.HernquistPotential(m=1e11, c=1.0)
    c = _restage_leapfrog(oracle, stream_case(n_streams=3, n_steps=120, leapfrog=True), pot)
    out, nb_out, status = _release_leapfrog_gpu(c, pot)
    rel, t = c["rel"], c["t"]
    ref_out, ref_nb = oracle.mockstream_leapfrog_systems(pot, c["bodies"], c["orbits"][:, rel], t[rel], c["nstream"],
                                                         c["stream_w0"], t[-1], t[1] - t[0], nthreads=8)
    assert np.all(status == 1)
    np.testing.assert_array_equal(out, ref_out)
    np.testing.assert_array_equal(nb_out, ref_nb)


def test_release_leapfrog_fp32c_accuracy(oracle):
    """The FP32-compensated form against the FP64 one on the same release
    systems (MW composite, 2 x 300 Myr): positions agree to ~1e-6 of the orbit."""
    c = stream_case(n_streams=4, n_steps=300, leapfrog=True)
    o64, nb64, _ = _release_leapfrog_gpu(c)
    o32, nb32, st = _release_leapfrog_gpu(c, precision="fp32c")
    assert np.all(st == 1)
    err = np.linalg.norm(o32[..., :3] - o64[..., :3], axis=-1) / np.linalg.norm(o64[..., :3], axis=-1)
    q = np.percentile(err, [50, 90, 99])
    # the few particles that cross the progenitor's core are chaotic: any
    # rounding difference grows there (gala's own -Ofast and strict builds differ
    # most on those), so the bound is on the distribution, not the maximum
    assert q[0] < 1e-6 and q[1] < 1e-5 and np.mean(err > 1e-3) < 0.02, (q, np.max(err), np.mean(err > 1e-3))
    assert _scale_err(nb32, nb64) < 1e-5


@pytest.mark.parametrize("case", ["forward", "backward", "release_every"])
def test_generator_leapfrog_matches_oracle(oracle, case):
    pot = W.mw_composite()
    w0 = W.mw_ics(1, seed=62)[:, 0]
    prog_pot = g.PlummerPotential(m=2e5, b=0.01)
    kw = dict(dt=1.0, n_steps=150) if case != "backward" else dict(dt=-1.0, n_steps=150)
    extra = dict(release_every=4, n_particles=2) if case == "release_every" else {}
    gen = MockStreamGenerator(FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(9)),
                              g.Hamiltonian(pot), progenitor_potential=prog_pot)
    stream, nbody = gen.run(g.PhaseSpacePosition.from_w(w0), 2e5, Integrator="leapfrog", **extra, **kw)
    t = g.parse_time_specification(**kw)
    bodies = pack_bodies([prog_pot])
    orb = oracle.leapfrog_nbody(pot, bodies, 1, w0.reshape(1, 6), t)
    orbit_t = t
    if t[1] < t[0]:
        orb, orbit_t = orb[::-1].copy(), t[::-1].copy()
    df = FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(9))
    counts = df.release_counts(len(t), extra.get("release_every", 1), extra.get("n_particles", 1))
    offset = np.concatenate([[0], np.cumsum(2 * counts)]).astype(np.int64)
    sw0 = oracle.fardal_sample(pot, orb.reshape(len(t), 6), np.full(len(t), 2e5), orbit_t, offset,
                               df._draws(int(offset[-1])), g.units.G)
    rel = np.nonzero(counts > 0)[0]
    if 0 not in rel:
        rel = np.insert(rel, 0, 0)
    ref_nb, ref_st = oracle.mockstream_leapfrog(pot, bodies, orb[0].reshape(1, 6), orbit_t, sw0, orbit_t[rel],
                                                orbit_t[-1], 2 * counts[rel])
    got = np.vstack([stream.xyz, stream.v_xyz]).T
    assert _scale_err(got, ref_st) < 1e-10
    assert _scale_err(np.vstack([nbody.xyz, nbody.v_xyz]).T, ref_nb) < 1e-10


def test_directnbody_leapfrog(oracle):
    pot = W.mw_composite()
    pps = [None, g.PlummerPotential(m=2e9, b=0.4), g.HernquistPotential(m=5e9, c=1.0)]
    w0 = W.mw_ics(3, seed=51)
    w0[:3, 2] = w0[:3, 1] + np.array([0.8, -0.4, 0.1])
    nb = DirectNBody(g.PhaseSpacePosition.from_w(w0), pps, external_potential=pot)
    orbit = nb.integrate_orbit(dt=0.5, n_steps=200, Integrator="leapfrog")
    t = g.parse_time_specification(dt=0.5, n_steps=200)
    idx = np.array([1, 2, 0])
    ref = oracle.leapfrog_nbody(pot, pack_bodies([pps[i] for i in idx]), 2, w0[:, idx].T, t)[:, np.argsort(idx)]
    assert _scale_err(np.moveaxis(orbit.w(), 0, -1), ref) < 1e-11


@pytest.mark.parametrize("sparse", [False, True])
def test_leapfrog_progenitor_reaches_the_final_time(sparse):
    """gala's regression tests (tests/dynamics/mockstream/test_mockstream.py:663-753): with
    the Leapfrog integrator the progenitor (a test particle here) ends where a direct
    Leapfrog orbit ends, whether particles are released every step or every fifth step
    with none at the last one.  gala uses MilkyWayPotential(version="latest"); v1 here.
    On the oracle the two agree bit for bit."""
    from gala_gb300.mockstream import ChenStreamDF

    mw = g.MilkyWayPotential()
    K = g.units.KMS_TO_KPC_MYR
    w0 = np.array([13.0, 0.0, 20.0, 0.0, 130.0 * K, 50.0 * K])
    t = np.arange(0.0, 200.0 if sparse else 100.0, 1.0)
    n = np.zeros(len(t), dtype=int)
    n[:: 5 if sparse else 1] = 1
    gen = MockStreamGenerator(ChenStreamDF(random_state=np.random.RandomState(1)), g.Hamiltonian(mw))
    _, prog = gen.run(g.PhaseSpacePosition.from_w(w0), 2.5e4, n_particles=n, t=t, Integrator="leapfrog")
    expected = mw.integrate_orbit(w0, t=t, Integrator="leapfrog").w()[:3, -1]
    np.testing.assert_allclose(prog.xyz.squeeze(), expected, rtol=1e-10, atol=1e-10)


def test_large_leapfrog_release_and_dop853_burst(oracle):
    """gala's one-burst setting (test_mockstream_class.py:41-97) through the generator:
    with Leapfrog the 2000 particles released at once run as groups of 7 with copies
    of the progenitor (split_releases, bit-identical to one system on the oracle) and
    match the oracle's single system; with DOP853 the release is one system wider
    than a warp, integrated by one CTA, and matches the oracle's system.  The
    particles are released at the pericentre of a near-radial orbit, next to a
    4 pc progenitor: a few of them amplify any rounding difference
    (the sampler's d2Phi/dr2, CUDA's log) up to 1e-4 of the scale, while the bulk is
    unaffected.  So the stream is held to its distribution -- median below 1e-8 and
    90th percentile below 1e-7 of the scale (1e-10 and 2e-10 when the oracle's own
    release states are perturbed by 2e-9) -- and the progenitor to 1e-10."""
    from .test_mockstream_oracle import _one_burst

    pot, bodies, orb, t, sw0, rel, counts = _one_burst(oracle, leapfrog=True)
    ref_nb, ref_st = oracle.mockstream_leapfrog(pot, bodies, orb[0].reshape(1, 6), t, sw0, t[rel], t[-1],
                                                2 * counts[rel])
    K = g.units.KMS_TO_KPC_MYR
    w0 = np.array([10.0, 0, 0, 0, 10 * K, 0])

    def gen():
        return MockStreamGenerator(FardalStreamDF(gala_modified=True, random_state=np.random.default_rng(seed=42)),
                                   g.Hamiltonian(pot), progenitor_potential=g.PlummerPotential(m=2.5e4, b=0.004))

    stream, nbody = gen().run(g.PhaseSpacePosition.from_w(w0), 2.5e4, n_particles=counts, dt=1.0, n_steps=100,
                              Integrator="leapfrog")
    got = np.vstack([stream.xyz, stream.v_xyz]).T
    assert got.shape == ref_st.shape
    err = np.linalg.norm(got - ref_st, axis=1) / np.abs(ref_st).max()
    assert np.median(err) < 1e-8 and np.quantile(err, 0.9) < 1e-7, np.quantile(err, [0.5, 0.9, 1.0])
    assert _scale_err(np.vstack([nbody.xyz, nbody.v_xyz]).T, ref_nb) < 1e-10
    # the batch result keeps one status per release time, however the releases were split
    res = gen().run_batch(w0.reshape(6, 1), np.array([2.5e4]), progenitor_potentials=[g.PlummerPotential(m=2.5e4,
                          b=0.004)], n_particles=counts, dt=1.0, n_steps=100, Integrator="leapfrog")
    rel_t = np.nonzero(np.asarray(counts) > 0)[0]
    assert tuple(res.status.shape) == (1, len(rel_t) + (0 not in rel_t))
    st = res.status.cpu().numpy()[0]
    assert np.all(st[-len(rel_t):] == 1) and np.all(st[:len(st) - len(rel_t)] == 0)  # 0: nothing released
    # DOP853: the 2001-member release is one system (the CTA-per-system kernel);
    # gala's own asserted values (test_mockstream_class.py:84-97) and the oracle's
    # system, held to the same distribution bounds
    pot, bodies, orb, t, sw0, rel, counts = _one_burst(oracle)
    ref_nb, ref_st, ref_status = oracle.mockstream_dop853(pot, bodies, orb[0].reshape(1, 6), t[rel], sw0, t[rel],
                                                          t[-1], 2 * counts[rel])
    stream, nbody = gen().run(g.PhaseSpacePosition.from_w(w0), 2.5e4, n_particles=counts, dt=1.0, n_steps=100)
    got = np.vstack([stream.xyz, stream.v_xyz]).T
    assert got.shape == ref_st.shape
    err = np.linalg.norm(got - ref_st, axis=1) / np.abs(ref_st).max()
    assert np.median(err) < 1e-8 and np.quantile(err, 0.9) < 1e-7, np.quantile(err, [0.5, 0.9, 1.0])
    nbw = np.vstack([nbody.xyz, nbody.v_xyz]).T
    assert _scale_err(nbw, ref_nb) < 1e-10
    np.testing.assert_allclose(nbw.reshape(-1)[:6], [-9.72388107, -1.28632464, 0.0, -0.04714419, -0.016754, 0.0],
                               rtol=0, atol=1e-8)


_DF_CASES = [("streakline", {}), ("fardal", {"gala_modified": True}), ("lagrange", {"v_disp": 1.0})]


@pytest.mark.parametrize("which,kw", _DF_CASES)
@pytest.mark.parametrize("pot", ["hernquist", "milkyway"])
def test_df_sample_like_gala(which, kw, pot):
    """gala's test_init_sample (tests/dynamics/mockstream/test_df.py:24-52): two particles
    per time with both tails, one with either tail off, identical output for identical
    random states (gala zips its kwargs list, so ChenStreamDF is not sampled there)."""
    from gala_gb300.mockstream import LagrangeCloudStreamDF, StreaklineStreamDF

    DF = {"streakline": StreaklineStreamDF, "fardal": FardalStreamDF, "lagrange": LagrangeCloudStreamDF}[which]
    p = g.HernquistPotential(m=1e12, c=5.0) if pot == "hernquist" else g.MilkyWayPotential()
    orbit = g.Hamiltonian(p).integrate_orbit(np.array([10.0, 0, 0, 0, 0.2, 0]), dt=1.0, n_steps=100)
    n = len(orbit.t)
    assert len(DF(**kw).sample(orbit, 1e4).x) == 2 * n
    assert len(DF(lead=False, **kw).sample(orbit, 1e4).x) == n
    assert len(DF(trail=False, **kw).sample(orbit, 1e4).x) == n
    o1 = DF(random_state=np.random.RandomState(42), **kw).sample(orbit, 1e4)
    o2 = DF(random_state=np.random.RandomState(42), **kw).sample(orbit, 1e4)
    assert np.array_equal(o1.xyz, o2.xyz) and np.array_equal(o1.v_xyz, o2.v_xyz) and len(o1.x) == 2 * n


def test_fp32_dop853_release_systems_match_fp64():
    """Mock streams with precision="fp32c" and DOP853: the release systems run
    with FP32 stages and forces and FP64 step control (atol 1e-10, rtol 1e-8)
    and land on the FP64 form's particles (rtol 1e-10): median final-position
    difference within 1e-5 of the position, 99 % within 1e-3."""
    pot = W.mw_composite()
    S = 16
    w0, m, b = W.stream_progenitors(S)
    pots = W.stream_progenitor_potentials(m, b)

    def run(precision, rtol):
        gen = MockStreamGenerator(FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(3)), pot)
        return gen.run_batch(w0, m, progenitor_potentials=pots, dt=1.0, n_steps=300,
                             Integrator_kwargs=dict(precision=precision, atol=1e-10, rtol=rtol, err_if_fail=0))

    r64 = run("fp64", 1e-10)
    r32 = run("fp32c", 1e-8)
    s64, s32 = r64.stream_w.cpu().numpy(), r32.stream_w.cpu().numpy()
    st64, st32 = r64.status.cpu().numpy(), r32.status.cpu().numpy()
    ok = np.repeat((st64 == 1) & (st32 == 1), 2, axis=1)[:, :s64.shape[1]]
    err = (np.linalg.norm(s32[..., :3] - s64[..., :3], axis=-1) / np.linalg.norm(s64[..., :3], axis=-1))[ok]
    assert np.mean(st32[st64 == 1] == 1) > 0.98
    assert np.median(err) < 1e-5 and np.quantile(err, 0.99) < 1e-3, np.quantile(err, [0.5, 0.99, 1.0])
    # the returned bodies are those of the last release system (mockstream.pyx:291-293),
    # which the FP32 form integrates with FP32 stages too
    np.testing.assert_allclose(r32.nbody_w.cpu().numpy(), r64.nbody_w.cpu().numpy(), rtol=1e-5)


# ------------------------------------------------------------ animate mode
def _animate_gpu(c, output_every, pot=None):
    """gx_mockstream_dop853_animate on a stream_case: every stream's bodies at
    t[0], the whole grid, particles released at every grid time."""
    import torch

    from gala_gb300._device import ptr, stream_handle

    pot = c["pot"] if pot is None else pot
    dev = torch.device("cuda")
    t = c["t"]
    S, n_rows = c["stream_w0"].shape[:2]
    M = 1 + n_rows
    lib = _abi.load()
    n_out = int(lib.gx_mockstream_animate_snapshots(len(t), output_every))
    nbytes = int(lib.gx_mockstream_wide_scratch_bytes(S, M))
    scratch = torch.empty(nbytes // 8, dtype=torch.float64, device=dev)
    snap = torch.empty((S, 6, n_out, M), dtype=torch.float64, device=dev)
    w_out = torch.empty((S, M, 6), dtype=torch.float64, device=dev)
    status = torch.zeros((S, len(t)), dtype=torch.int32, device=dev)
    stats = torch.zeros((S, 4), dtype=torch.int64, device=dev)
    nb0 = torch.from_numpy(np.ascontiguousarray(c["w0"].T.reshape(S, 1, 6))).to(dev)
    sw0 = torch.from_numpy(np.ascontiguousarray(c["stream_w0"])).to(dev)
    td = torch.from_numpy(np.ascontiguousarray(t)).to(dev)
    nd = torch.from_numpy((2 * c["counts"]).astype(np.int32)).to(dev)
    bd = bodies_to_device(c["bodies"], dev)
    _abi.call("gx_mockstream_dop853_animate", pot.packed().for_device(), g.Hamiltonian(pot)._frame_ref(), S, 1,
              ptr(bd), ptr(nb0), len(t), ptr(td), float(t[1] - t[0]), ptr(nd), ptr(sw0), n_rows, output_every,
              1e-10, 1e-10, 0, ptr(scratch), nbytes, ptr(snap), ptr(w_out), ptr(status), ptr(stats), stream_handle())
    torch.cuda.synchronize()
    # (S, 6, n_out, M) -> (S, n_out, M, 6), the oracle's layout
    return (snap.permute(0, 2, 3, 1).cpu().numpy(), w_out.cpu().numpy(), status.cpu().numpy(),
            stats.cpu().numpy())


@pytest.mark.parametrize("n_steps,output_every,release_every", [(61, 3, 2), (40, 1, 1), (17, 2, 4)])
def test_animate_matches_oracle(oracle, n_steps, output_every, release_every):
    """One growing system per stream, stepped interval by interval: the
    snapshots, final states, per-interval status and summed counters match
    the oracle (itself bit-identical to gala's dop853 on the same system).
    The error and stiffness norms are CTA sums in another order than gala's
    sequential ones, and the MW composite's pow / log differ by an ulp, so the
    states agree to 1e-10 of their scale, not bit for bit."""
    c = stream_case(n_streams=3, n_steps=n_steps, release_every=release_every)
    snap, w, status, stats = _animate_gpu(c, output_every)
    from tests.test_mockstream_oracle import _animate_args

    for s in range(3):
        r_snap, _, r_w, r_status, r_stats = oracle.mockstream_animate(c["pot"], **_animate_args(c, s, output_every))
        assert snap[s].shape == r_snap.shape
        np.testing.assert_array_equal(np.isnan(snap[s]), np.isnan(r_snap))
        np.testing.assert_array_equal(status[s], r_status)
        live = ~np.isnan(r_snap)
        assert np.abs(snap[s][live] - r_snap[live]).max() < 1e-10 * np.abs(r_snap[live]).max()
        assert _scale_err(w[s], r_w) < 1e-10
        # steps, accepted and rejected steps: an accept / reject decision taken on
        # a rounding-level difference may differ, nothing more
        assert np.abs(stats[s][1:] - r_stats[1:]).max() <= 2


def test_animate_one_burst_system_matches_oracle(oracle):
    """gala's one-burst setting in the animate mode: 1,000 particles per tail
    released at t[0] join a 2,001-member system for all of its 40 intervals."""
    c = stream_case(n_streams=1, n_steps=40)
    counts = np.zeros(41, dtype=int)
    counts[0] = 1000
    from gala_gb300.mockstream import FardalStreamDF as DF

    df = DF(gala_modified=True, random_state=np.random.RandomState(5))
    offset = np.concatenate([[0], np.cumsum(2 * counts)]).astype(np.int64)
    orb = c["orbits"][0]
    c["stream_w0"] = oracle.fardal_sample(c["pot"], orb.reshape(41, 6), np.full(41, c["m"][0]), c["t"], offset,
                                          df._draws(int(offset[-1])), g.units.G)[None]
    c["counts"] = counts
    snap, w, status, _ = _animate_gpu(c, 10)
    from tests.test_mockstream_oracle import _animate_args

    r_snap, _, r_w, r_status, _ = oracle.mockstream_animate(c["pot"], **_animate_args(c, 0, 10))
    assert w.shape == (1, 2001, 6)
    np.testing.assert_array_equal(status[0], r_status)
    assert _scale_err(w[0], r_w) < 1e-10
    assert _scale_err(snap[0], r_snap) < 1e-10


@pytest.mark.parametrize("dt,nsteps,output_every,release_every,n_particles,trail",
                         [(1, 16, 1, 1, 1, True), (-1, 17, 2, 4, 4, False), (1, 17, 2, 1, 4, True),
                          (-1, 16, 1, 4, 1, True)])
def test_run_with_output_every_writes_galas_file(tmp_path, dt, nsteps, output_every, release_every, n_particles,
                                                 trail):
    """gala's test_animate (tests/dynamics/mockstream/test_mockstream.py:259-319):
    the file's shapes, finite first snapshot, equal times in both groups; and the
    returned stream equals the file's last snapshot."""
    pot = W.mw_composite()
    prog_pot = g.PlummerPotential(m=2e5, b=0.01)
    gen = MockStreamGenerator(FardalStreamDF(gala_modified=True, trail=trail, random_state=np.random.RandomState(2)),
                              g.Hamiltonian(pot), progenitor_potential=prog_pot)
    fn = tmp_path / "animate.hdf5"
    w0 = g.PhaseSpacePosition.from_w(W.mw_ics(1, seed=64)[:, 0])
    stream, nbody = gen.run(w0, 2e5, dt=dt, n_steps=nsteps, release_every=release_every, n_particles=n_particles,
                            output_every=output_every, output_filename=str(fn), overwrite=True)
    from gala_gb300.hdf5 import File

    with File(str(fn), "r") as f:
        st = g.Orbit.from_hdf5(f["stream"])
        nb = g.Orbit.from_hdf5(f["nbody"])
    n_out = 1 + nsteps // output_every + int(nsteps % output_every != 0)
    tail_n = (1 + int(trail)) * n_particles
    assert st.xyz.shape[1:] == (n_out, tail_n * (nsteps // release_every + 1))
    assert nb.xyz.shape[1:] == (n_out, 1)
    # gala's stream_orbits[:, 0]: particle 0 (released at the first time) at every snapshot
    assert np.isfinite(st.xyz[:, :, 0]).all() and np.isfinite(st.v_xyz[:, :, 0]).all()
    np.testing.assert_array_equal(nb.t, st.t)
    assert np.isfinite(nb.xyz).all() and np.isfinite(nb.t).all()
    np.testing.assert_array_equal(st.xyz[:, -1], stream.xyz)
    np.testing.assert_array_equal(nb.v_xyz[:, -1], nbody.v_xyz)


def test_fp32_animate_matches_fp64_animate():
    """The animate mode with FP32 stages and forces and FP64 step control
    (precision="fp32c", atol 1e-10, rtol 1e-8) lands on the FP64 animate
    run's particles (rtol 1e-10): median snapshot-position difference within
    1e-5 of the position, 99 % within 1e-3; the same NaN pattern; every
    interval succeeds."""
    pot = W.mw_composite()
    S = 8
    w0, m, b = W.stream_progenitors(S)
    pots = W.stream_progenitor_potentials(m, b)

    def run(precision, rtol):
        gen = MockStreamGenerator(FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(4)), pot)
        return gen.run_batch(w0, m, progenitor_potentials=pots, dt=1.0, n_steps=300, output_every=20,
                             Integrator_kwargs=dict(precision=precision, atol=1e-10, rtol=rtol))

    r64, r32 = run("fp64", 1e-10), run("fp32c", 1e-8)
    s64, s32 = r64.snapshots.cpu().numpy(), r32.snapshots.cpu().numpy()
    np.testing.assert_array_equal(np.isnan(s64), np.isnan(s32))
    assert np.all(r32.status.cpu().numpy()[:, 1:] == 1)
    live = ~np.isnan(s64[:, 0])  # (S, n_out, M)
    d = np.linalg.norm(s32[:, :3] - s64[:, :3], axis=1)[live] / np.linalg.norm(s64[:, :3], axis=1)[live]
    assert np.median(d) < 1e-5 and np.quantile(d, 0.99) < 1e-3, np.quantile(d, [0.5, 0.99, 1.0])
    np.testing.assert_array_equal(r32.stream_w.cpu().numpy(), np.transpose(s32[:, :, -1, 1:], (0, 2, 1)))


@pytest.mark.parametrize("mode", ["releases", "animate"])
def test_rotating_frame_stream_matches_oracle(oracle, mode):
    """A mock stream in a ConstantRotatingFrame: the progenitor integrated in the
    rotating frame, the DF sampled in the static frame (the orbit turned there at
    its times, each particle back at its release time, df.pyx:172-233), the
    release systems -- or the animate mode's growing system -- integrated in the
    rotating frame; against the oracle's pipeline (gala's rotation restated,
    oracle/orbit_oracle.py)."""
    from oracle import orbit_oracle as OO

    pot = W.mw_composite()
    Omega = np.array([0.0, 0.0, 0.025])
    frame = g.ConstantRotatingFrame(Omega=Omega)
    w0 = W.mw_ics(1, seed=66)[:, 0]
    prog_pot = g.PlummerPotential(m=2e5, b=0.01)
    seed, n_steps = 9, 80
    gen = MockStreamGenerator(FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(seed)),
                              g.Hamiltonian(pot, frame=frame), progenitor_potential=prog_pot)
    kw = dict(dt=1.0, n_steps=n_steps)
    if mode == "animate":
        res = gen.run_batch(w0[:, None], 2e5, progenitor_potentials=[prog_pot], output_every=8, **kw)
        got = res.stream_w[0].cpu().numpy()
        got_nb = res.nbody_w[0].cpu().numpy()
    else:
        stream, nbody = gen.run(g.PhaseSpacePosition.from_w(w0), 2e5, **kw)
        got = np.vstack([stream.xyz, stream.v_xyz]).T
        got_nb = np.vstack([nbody.xyz, nbody.v_xyz]).T

    # the oracle's pipeline
    t = g.parse_time_specification(**kw)
    bodies = pack_bodies([prog_pot])
    orb, res_o = oracle.nbody_dop853(pot, bodies, 1, w0.reshape(1, 6), t, frame=frame)
    assert res_o == 1
    prog = orb.reshape(len(t), 6)
    px, pv = OO.constantrotating_static(Omega, prog[:, :3].T, prog[:, 3:].T, t, -1.0)
    df = FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(seed))
    counts = df.release_counts(len(t))
    offset = np.concatenate([[0], np.cumsum(2 * counts)]).astype(np.int64)
    sw_static = oracle.fardal_sample(pot, np.vstack([px, pv]).T, np.full(len(t), 2e5), t, offset,
                                     df._draws(int(offset[-1])), g.units.G)
    rt = np.repeat(t, 2 * counts)
    sx, sv = OO.constantrotating_static(Omega, sw_static[:, :3].T, sw_static[:, 3:].T, rt, 1.0)
    sw0 = np.vstack([sx, sv]).T
    if mode == "animate":
        _, _, w_fin, status, _ = oracle.mockstream_animate(pot, bodies, orb[0].reshape(1, 6), t, sw0, 2 * counts,
                                                           output_every=8, frame=frame)
        assert np.all(status == 1)
        ref, ref_nb = w_fin[1:], w_fin[:1]
    else:
        rel = np.nonzero(counts > 0)[0]
        ref_nb, ref, status = oracle.mockstream_dop853(pot, bodies, orb[0].reshape(1, 6), t[rel], sw0, t[rel], t[-1],
                                                       2 * counts[rel], frame=frame)
        assert np.all(status[counts[rel] > 0] == 1)
    assert got.shape == ref.shape
    assert _scale_err(got, ref) < 1e-9
    assert _scale_err(got_nb, ref_nb) < 1e-10


def _wide_system(n_massive, n_test, seed):
    """A cluster of Plummer bodies plus test particles in the MW composite, far
    enough apart that the orbits are regular over the test's span."""
    rng = np.random.default_rng(seed)
    pots = [g.PlummerPotential(m=float(m), b=0.05) for m in rng.uniform(1e5, 1e6, n_massive)] + [None] * n_test
    w0 = np.ascontiguousarray(W.mw_ics(1, seed=seed).T).repeat(n_massive + n_test, axis=0)
    w0[:, :3] += rng.normal(0, 0.5, size=(n_massive + n_test, 3))
    w0[:, 3:] += rng.normal(0, 0.005, size=(n_massive + n_test, 3))
    return pots, w0


@pytest.mark.parametrize("save_all", [True, False])
def test_nbody_systems_wider_than_a_warp_match_oracle(oracle, save_all):
    """Systems of 48 particles (24 massive): one CTA per system
    (gx_nbody_dop853_wide, dop853_helper's arguments, dense output onto the
    grid), against the oracle's direct_nbody_dop853 on each system."""
    pot = W.mw_composite()
    t = g.parse_time_specification(dt=1.0, n_steps=80)
    systems = [_wide_system(24, 24, 80 + s) for s in range(3)]
    bodies = pack_bodies([p[:24] for p, _ in systems])
    w0 = np.stack([w for _, w in systems])
    out, status = integrate_systems(pot, bodies, w0, t, save_all=save_all, nstiff=-1)
    out = out.cpu().numpy()
    assert np.all(status.cpu().numpy() == 1)
    for s, (pots, w) in enumerate(systems):
        ref, res = oracle.nbody_dop853(pot, pack_bodies(pots), 24, w, t, save_all=save_all)
        assert res == 1
        assert _scale_err(out[s], ref) < 1e-10


def test_directnbody_of_forty_bodies_and_a_stream_with_many_perturbers(oracle):
    """DirectNBody.integrate_orbit with 40 bodies (beyond one warp), and a mock
    stream whose progenitor has 32 perturbers (every release system wider than a
    warp), against the oracle."""
    from gala_gb300.nbody import DirectNBody

    pot = W.mw_composite()
    pots, w = _wide_system(20, 20, 90)
    psp = g.PhaseSpacePosition(pos=w[:, :3].T, vel=w[:, 3:].T)
    orb = DirectNBody(psp, pots, external_potential=pot).integrate_orbit(dt=1.0, n_steps=100)
    t = g.parse_time_specification(dt=1.0, n_steps=100)
    ref, res = oracle.nbody_dop853(pot, pack_bodies(pots), 20, w, t)
    assert res == 1
    got = np.concatenate([orb.xyz, orb.v_xyz]).transpose(1, 2, 0)
    assert _scale_err(got, ref) < 1e-10

    prog_pot = g.PlummerPotential(m=2e5, b=0.01)
    ppots, pw = _wide_system(32, 0, 91)
    nb = DirectNBody(g.PhaseSpacePosition(pos=pw[1:, :3].T, vel=pw[1:, 3:].T), ppots[1:], external_potential=pot)
    gen = MockStreamGenerator(FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(4)),
                              g.Hamiltonian(pot), progenitor_potential=prog_pot)
    stream, nbody_w = gen.run(g.PhaseSpacePosition.from_w(pw[0]), 2e5, nbody=nb, dt=1.0, n_steps=20)
    # the oracle's pipeline: the bodies, Fardal releases around body 0, the release systems
    bodies = pack_bodies([prog_pot] + ppots[1:])
    t = g.parse_time_specification(dt=1.0, n_steps=20)
    orbw, res = oracle.nbody_dop853(pot, bodies, 32, pw, t)
    assert res == 1
    df = FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(4))
    counts = df.release_counts(len(t))
    offset = np.concatenate([[0], np.cumsum(2 * counts)]).astype(np.int64)
    sw0 = oracle.fardal_sample(pot, orbw[:, 0], np.full(len(t), 2e5), t, offset, df._draws(int(offset[-1])),
                               g.units.G)
    rel = np.nonzero(counts > 0)[0]
    ref_nb, ref_st, st = oracle.mockstream_dop853(pot, bodies, pw, t[rel], sw0, t[rel], t[-1], 2 * counts[rel])
    assert np.all(st == 1)
    got = np.vstack([stream.xyz, stream.v_xyz]).T
    assert _scale_err(got, ref_st) < 1e-9
