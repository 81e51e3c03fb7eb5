"""The direct n-body and mock-stream oracle pinned against gala's own compiled code.

gala's dop853(), Fwrapper_direct_nbody, c_nbody_acceleration and c_d2_dr2 are
built from the gala sources (oracle/_ref) with the argument lists of
direct_nbody_dop853 / dop853_helper and of mockstream_dop853 / dop853_step; the
restatement must reproduce them bit for bit when both are built without
fast-math.  The golden fixture holds gala's release-build (-Ofast) outputs for
machines without the gala sources.
"""
import numpy as np
import pytest

import gala_gb300 as g
from gala_gb300 import workloads as W
from gala_gb300.nbody import pack_bodies

from ._cases import stream_case

OFAST_RTOL = 1e-11


def _nbody_system():
    mw = W.mw_composite()
    pots = [g.PlummerPotential(m=2e9, b=0.4), g.HernquistPotential(m=5e9, c=1.0), None, None]
    bodies = pack_bodies(pots)
    w0 = np.ascontiguousarray(W.mw_ics(4, seed=31).T)
    w0[1, :3] = w0[0, :3] + np.array([1.0, 0.5, -0.2])
    t = g.parse_time_specification(dt=1.0, n_steps=300)
    return mw, bodies, w0, t


def _stream_args(c, s):
    rel = c["rel"]
    return dict(bodies=c["bodies"][s], nbody_w0=c["w0"][:, s].reshape(1, 6), time=c["t"][rel],
                stream_w0=c["stream_w0"][s], stream_t1=c["t"][rel], tfinal=c["t"][-1], nstream=c["nstream"])


def test_nbody_oracle_matches_gala(oracle, gala_ref_strict):
    mw, bodies, w0, t = _nbody_system()
    w_o, res_o = oracle.nbody_dop853(mw, bodies, 2, w0, t)
    w_r, res_r = gala_ref_strict.nbody_dop853(mw, bodies, 2, w0, t)
    assert res_o == res_r == 1
    np.testing.assert_array_equal(w_o, w_r)
    # the massive pair really interacts: the test particles' orbits differ from the pair's
    assert np.ptp(w_o[:, 1, :3] - w_o[:, 0, :3]) > 0.1


def test_nbody_oracle_final_state_matches_gala(oracle, gala_ref_strict):
    mw, bodies, w0, t = _nbody_system()
    w_o, _ = oracle.nbody_dop853(mw, bodies, 2, w0, t, save_all=False)
    w_r, _ = gala_ref_strict.nbody_dop853(mw, bodies, 2, w0, t, save_all=False)
    np.testing.assert_array_equal(w_o, w_r)


def test_mockstream_oracle_matches_gala(oracle, gala_ref_strict):
    c = stream_case(n_streams=2, n_steps=120)
    for s in range(2):
        a = _stream_args(c, s)
        nb_o, st_o, stat_o = oracle.mockstream_dop853(c["pot"], **a)
        nb_r, st_r, stat_r = gala_ref_strict.mockstream_dop853(c["pot"], **a)
        np.testing.assert_array_equal(stat_o, stat_r)
        assert np.all(stat_o[c["nstream"] > 0] == 1)
        np.testing.assert_array_equal(st_o, st_r)
        np.testing.assert_array_equal(nb_o, nb_r)


def test_mockstream_release_every_matches_gala(oracle, gala_ref_strict):
    """Releases every 3rd step, 2 particles per tail: the bodies are
    re-integrated on the coarser release grid (h0 = 3 dt)."""
    c = stream_case(n_streams=1, n_steps=90, n_per_tail=2, release_every=3)
    a = _stream_args(c, 0)
    nb_o, st_o, stat_o = oracle.mockstream_dop853(c["pot"], **a)
    nb_r, st_r, stat_r = gala_ref_strict.mockstream_dop853(c["pot"], **a)
    np.testing.assert_array_equal(st_o, st_r)
    np.testing.assert_array_equal(nb_o, nb_r)
    np.testing.assert_array_equal(stat_o, stat_r)


def test_mockstream_systems_match_per_stream(oracle):
    """The batched release-system layout equals gala's per-stream loop."""
    c = stream_case(n_streams=3, n_steps=80)
    rel = c["rel"]
    nbody_w = c["orbits"][:, rel]  # (S, n_release, 1, 6)
    t = c["t"]
    out, nb_out, status, stats = oracle.mockstream_systems(
        c["pot"], c["bodies"], nbody_w, t[rel], c["nstream"], c["stream_w0"], t[-1], t[rel][1] - t[rel][0],
        nthreads=4)
    for s in range(3):
        nb_o, st_o, stat_o = oracle.mockstream_dop853(c["pot"], **_stream_args(c, s))
        np.testing.assert_array_equal(out[s], st_o)
        np.testing.assert_array_equal(nb_out[s], nb_o)
        np.testing.assert_array_equal(status[s], stat_o)
    assert np.all(stats[status == 1][:, 2] > 0)


def test_d2_dr2_matches_gala(oracle, gala_ref_strict):
    q = W.mw_ics(32, seed=5)[:3].T.copy()
    mw = W.mw_composite()
    np.testing.assert_array_equal(oracle.d2_dr2(mw, q), gala_ref_strict.d2_dr2(mw, q))


def test_fardal_sample_geometry(oracle):
    """Each released particle sits at (kx rj, 0, kz rj) in the progenitor's
    rotating frame (x along r, z along L), trailing at +rj and leading at -rj,
    with r_J = (G m / (Omega^2 - d2Phi/dr2))^(1/3) (df.pyx:61-92, 410-450)."""
    mw = W.mw_composite()
    w = W.mw_ics(5, seed=8).T.copy()
    t = np.arange(5.0)
    m = np.full(5, 3e5)
    counts = np.full(5, 2)
    offset = np.concatenate([[0], np.cumsum(2 * counts)])
    draws = np.random.default_rng(1).normal([2, 0, 0.3, 0], 0.5, size=(int(offset[-1]), 4))
    out = oracle.fardal_sample(mw, w, m, t, offset, draws, g.units.G)
    d2 = oracle.d2_dr2(mw, w[:, :3])
    for i in range(5):
        x, v = w[i, :3], w[i, 3:]
        L = np.cross(x, v)
        Om = np.linalg.norm(L) / np.dot(x, x)
        rj = (g.units.G * m[i] / (Om * Om - d2[i])) ** (1 / 3)
        vj = Om * rj
        e0, e2 = x / np.linalg.norm(x), L / np.linalg.norm(L)
        e1 = -np.cross(e0, e2)
        for k, row in enumerate(range(offset[i], offset[i + 1])):
            sgn = 1.0 if k < 2 else -1.0
            dx, dv = out[row, :3] - x, out[row, 3:] - v
            kx, kz, kvt, kvz = draws[row]
            np.testing.assert_allclose([dx @ e0, dx @ e1, dx @ e2], sgn * rj * np.array([kx, 0, kz]),
                                       rtol=0, atol=1e-12 * rj)
            np.testing.assert_allclose([dv @ e0, dv @ e1, dv @ e2], sgn * vj * np.array([0, kvt * kx, kvz]),
                                       rtol=0, atol=1e-12 * vj)


def test_mockstream_golden(oracle, golden):
    d = golden("mockstream_dop853.npz")
    c = stream_case(n_streams=int(d["n_streams"]), n_steps=int(d["n_steps"]))
    np.testing.assert_array_equal(c["stream_w0"], d["stream_w0"])
    for s in range(c["stream_w0"].shape[0]):
        nb_o, st_o, stat_o = oracle.mockstream_dop853(c["pot"], **_stream_args(c, s))
        np.testing.assert_array_equal(stat_o, d["status"][s])
        scale = np.abs(d["stream"][s]).max(axis=0)
        np.testing.assert_allclose(st_o, d["stream"][s], rtol=0, atol=OFAST_RTOL * scale.max())
        np.testing.assert_allclose(nb_o, d["nbody"][s], rtol=OFAST_RTOL, atol=0)


def test_nbody_golden(oracle, golden):
    d = golden("nbody_dop853.npz")
    mw, bodies, w0, t = _nbody_system()
    np.testing.assert_array_equal(w0, d["w0"])
    w_o, res = oracle.nbody_dop853(mw, bodies, 2, w0, t)
    assert res == 1
    np.testing.assert_allclose(w_o[::50], d["w"], rtol=OFAST_RTOL, atol=OFAST_RTOL * np.abs(d["w"]).max())


@pytest.mark.parametrize("bad", ["scf_body"])
def test_unsupported_body_types_raise(bad):
    with pytest.raises(NotImplementedError):
        pack_bodies([W.scf_potential(nmax=2, lmax=1)])


# ----------------------------------------------------------------- Leapfrog
def test_leapfrog_nbody_oracle_matches_gala(oracle, gala_ref_strict):
    mw, bodies, w0, t = _nbody_system()
    a = oracle.leapfrog_nbody(mw, bodies, 2, w0, t)
    b = gala_ref_strict.leapfrog_nbody(mw, bodies, 2, w0, t)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(oracle.leapfrog_nbody(mw, bodies, 2, w0, t, save_all=False), a[-1])


def _lf_stream_args(c, s):
    rel = c["rel"]
    return dict(bodies=c["bodies"][s], nbody_w0=c["w0"][:, s].reshape(1, 6), full_time=c["t"],
                stream_w0=c["stream_w0"][s], stream_t1=c["t"][rel], tfinal=c["t"][-1], nstream=c["nstream"])


def test_mockstream_leapfrog_oracle_matches_gala(oracle, gala_ref_strict):
    c = stream_case(n_streams=2, n_steps=150, leapfrog=True)
    for s in range(2):
        nb_o, st_o = oracle.mockstream_leapfrog(c["pot"], **_lf_stream_args(c, s))
        nb_r, st_r = gala_ref_strict.mockstream_leapfrog(c["pot"], **_lf_stream_args(c, s))
        np.testing.assert_array_equal(st_o, st_r)
        np.testing.assert_array_equal(nb_o, nb_r)


def test_mockstream_leapfrog_release_every_matches_gala(oracle, gala_ref_strict):
    c = stream_case(n_streams=1, n_steps=90, n_per_tail=2, release_every=4, leapfrog=True)
    nb_o, st_o = oracle.mockstream_leapfrog(c["pot"], **_lf_stream_args(c, 0))
    nb_r, st_r = gala_ref_strict.mockstream_leapfrog(c["pot"], **_lf_stream_args(c, 0))
    np.testing.assert_array_equal(st_o, st_r)
    np.testing.assert_array_equal(nb_o, nb_r)


def test_mockstream_leapfrog_systems_match_per_stream(oracle):
    c = stream_case(n_streams=3, n_steps=80, leapfrog=True)
    rel, t = c["rel"], c["t"]
    out, nb_out = oracle.mockstream_leapfrog_systems(c["pot"], c["bodies"], c["orbits"][:, rel], t[rel],
                                                     c["nstream"], c["stream_w0"], t[-1], t[1] - t[0], nthreads=4)
    for s in range(3):
        nb_o, st_o = oracle.mockstream_leapfrog(c["pot"], **_lf_stream_args(c, s))
        np.testing.assert_array_equal(out[s], st_o)
        np.testing.assert_array_equal(nb_out[s], nb_o)


def test_mockstream_leapfrog_golden(oracle, golden):
    d = golden("mockstream_leapfrog.npz")
    c = stream_case(n_streams=int(d["n_streams"]), n_steps=int(d["n_steps"]), leapfrog=True)
    np.testing.assert_array_equal(c["stream_w0"], d["stream_w0"])
    for s in range(c["stream_w0"].shape[0]):
        nb_o, st_o = oracle.mockstream_leapfrog(c["pot"], **_lf_stream_args(c, s))
        scale = np.abs(d["stream"][s]).max()
        # gala's -Ofast build contracts and reorders; particles passing the
        # progenitor's core amplify that to ~1e-11 of the stream's extent
        np.testing.assert_allclose(st_o, d["stream"][s], rtol=0, atol=1e-9 * scale)
        np.testing.assert_allclose(nb_o, d["nbody"][s], rtol=1e-11, atol=0)
    np.testing.assert_allclose(oracle.leapfrog_nbody(c["pot"], *_lf_nbody_args()), d["nbody_leapfrog"],
                               rtol=0, atol=1e-11 * np.abs(d["nbody_leapfrog"]).max())


def _lf_nbody_args():
    mw, bodies, w0, t = _nbody_system()
    return bodies, 2, w0, t


def test_streakline_release_geometry(oracle):
    """StreaklineStreamDF (df.pyx:242-319): particles at -/+ r_J along the
    progenitor's radius vector, -/+ v_J along e_y = -(x_hat x L_hat), nothing
    drawn -- the Fardal placement with constants (1, 0, 1, 0); the random state
    is not consumed."""
    from gala_gb300.mockstream import StreaklineStreamDF

    rs = np.random.RandomState(3)
    state = rs.get_state()[1].copy()
    df = StreaklineStreamDF(random_state=rs)
    draws = df._draws(8)
    assert np.array_equal(rs.get_state()[1], state)
    np.testing.assert_array_equal(draws, np.tile([1.0, 0.0, 1.0, 0.0], (8, 1)))
    mw = W.mw_composite()
    w = W.mw_ics(4, seed=9).T.copy()
    t = np.arange(4.0)
    m = np.full(4, 2e5)
    offset = np.array([0, 2, 4, 6, 8])
    out = oracle.fardal_sample(mw, w, m, t, offset, draws, g.units.G)
    d2 = oracle.d2_dr2(mw, w[:, :3])
    for i in range(4):
        x, v = w[i, :3], w[i, 3:]
        L = np.cross(x, v)
        Om = np.linalg.norm(L) / np.dot(x, x)
        rj = (g.units.G * m[i] / (Om * Om - d2[i])) ** (1 / 3)
        e0, e2 = x / np.linalg.norm(x), L / np.linalg.norm(L)
        e1 = -np.cross(e0, e2)
        for k, sgn in enumerate((1.0, -1.0)):
            row = offset[i] + k
            np.testing.assert_allclose(out[row, :3] - x, sgn * rj * e0, rtol=0, atol=1e-12 * rj)
            np.testing.assert_allclose(out[row, 3:] - v, sgn * Om * rj * e1, rtol=0, atol=1e-12 * Om * rj)


def _sat_frame(oracle, mw, w, m):
    d2 = oracle.d2_dr2(mw, w[:, :3])
    frames = []
    for i in range(len(w)):
        x, v = w[i, :3], w[i, 3:]
        L = np.cross(x, v)
        Om = np.linalg.norm(L) / np.dot(x, x)
        rj = (g.units.G * m[i] / (Om * Om - d2[i])) ** (1 / 3)
        e0, e2 = x / np.linalg.norm(x), L / np.linalg.norm(L)
        frames.append((rj, Om * rj, e0, -np.cross(e0, e2), e2))
    return frames


def test_lagrange_cloud_release_geometry(oracle):
    """LagrangeCloudStreamDF (df.pyx:460-555): -/+ r_J along x, the satellite-frame
    velocity three normal(0, v_disp) draws per particle, drawn in gala's order."""
    from gala_gb300.mockstream import LagrangeCloudStreamDF

    df = LagrangeCloudStreamDF(v_disp=2.0, random_state=np.random.RandomState(5))
    draws = df._draws(8)
    rs = np.random.RandomState(5)
    seq = np.array([[rs.normal(0, 2.0 * g.units.KMS_TO_KPC_MYR) for _ in range(3)] for _ in range(8)])
    np.testing.assert_array_equal(draws, seq)
    mw = W.mw_composite()
    w = W.mw_ics(4, seed=10).T.copy()
    m = np.full(4, 2e5)
    offset = np.array([0, 2, 4, 6, 8])
    out = oracle.stream_sample(mw, w, m, np.arange(4.0), offset, 1, draws, g.units.G)
    for i, (rj, vj, e0, e1, e2) in enumerate(_sat_frame(oracle, mw, w, m)):
        for k, sgn in enumerate((1.0, -1.0)):
            row = offset[i] + k
            d = draws[row]
            np.testing.assert_allclose(out[row, :3] - w[i, :3], sgn * rj * e0, rtol=0, atol=1e-12 * rj)
            np.testing.assert_allclose(out[row, 3:] - w[i, 3:], d[0] * e0 + d[1] * e1 + d[2] * e2, rtol=0,
                                       atol=1e-15)


def test_chen_release_geometry(oracle):
    """ChenStreamDF (df.pyx:557-703): offset Dr = r r_J in the direction (theta,
    phi) of the satellite frame, velocity Dv = v sqrt(2 G m / Dr) in the direction
    (beta, alpha); the leading tail turns phi and alpha by pi; one
    multivariate-normal sample per particle in gala's order."""
    from gala_gb300.mockstream import ChenStreamDF

    df = ChenStreamDF(random_state=np.random.RandomState(6))
    draws = df._draws(8)
    rs = np.random.RandomState(6)
    seq = np.array([rs.multivariate_normal(ChenStreamDF._MEAN, ChenStreamDF._cov()) for _ in range(8)])
    np.testing.assert_array_equal(draws, seq)
    mw = W.mw_composite()
    w = W.mw_ics(4, seed=11).T.copy()
    m = np.full(4, 2e5)
    offset = np.array([0, 2, 4, 6, 8])
    out = oracle.stream_sample(mw, w, m, np.arange(4.0), offset, 2, draws, g.units.G)
    for i, (rj, vj, e0, e1, e2) in enumerate(_sat_frame(oracle, mw, w, m)):
        for k in range(2):
            row = offset[i] + k
            r, ph, th, vv, al, be = draws[row]
            ph, th, al, be = np.radians([ph, th, al, be])
            if k == 1:
                ph, al = ph + np.pi, al + np.pi
            Dr = r * rj
            Dv = vv * np.sqrt(2 * g.units.G * m[i] / Dr)
            dx = Dr * np.array([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), np.sin(th)])
            dv = Dv * np.array([np.cos(be) * np.cos(al), np.cos(be) * np.sin(al), np.sin(be)])
            np.testing.assert_allclose(out[row, :3] - w[i, :3], dx @ np.stack([e0, e1, e2]), rtol=0,
                                       atol=1e-12 * rj)
            np.testing.assert_allclose(out[row, 3:] - w[i, 3:], dv @ np.stack([e0, e1, e2]), rtol=0,
                                       atol=1e-12 * abs(Dv) + 1e-15)


def test_leapfrog_progenitor_reaches_the_final_time_oracle(oracle):
    """gala's Leapfrog regression tests (test_mockstream.py:663-753) on the oracle's
    mockstream_leapfrog: with releases every step, or every fifth step and none at
    the last, the progenitor's final position is the direct Leapfrog orbit's, bit for
    bit (gala compares positions); its velocity is within an ulp, since the release
    stage restarts Leapfrog from (x, v) at the last release and re-forms the
    half-step velocity there."""
    from gala_gb300.mockstream import ChenStreamDF
    from gala_gb300.nbody import pack_bodies

    mw = g.MilkyWayPotential()
    K = g.units.KMS_TO_KPC_MYR
    w0 = np.array([13.0, 0, 20.0, 0, 130 * K, 50 * K])
    bodies = pack_bodies([None])
    for sparse in (False, True):
        t = np.arange(0, 200.0 if sparse else 100.0, 1.0)
        counts = np.zeros(len(t), dtype=np.int64)
        counts[:: 5 if sparse else 1] = 1
        orb = oracle.leapfrog_nbody(mw, bodies, 1, w0.reshape(1, 6), t)
        offset = np.concatenate([[0], np.cumsum(2 * counts)]).astype(np.int64)
        draws = ChenStreamDF(random_state=np.random.RandomState(1))._draws(int(offset[-1]))
        sw0 = oracle.stream_sample(mw, orb.reshape(len(t), 6), np.full(len(t), 2.5e4), t, offset, 2, draws, g.units.G)
        rel = np.nonzero(counts > 0)[0]
        ref_nb, _ = oracle.mockstream_leapfrog(mw, bodies, orb[0].reshape(1, 6), t, sw0, t[rel], t[-1],
                                               2 * counts[rel])
        direct = oracle.fixed(mw, w0[:, None], t, "leapfrog")[:, -1, 0]
        assert np.array_equal(ref_nb.reshape(-1)[:3], direct[:3])
        np.testing.assert_allclose(ref_nb.reshape(-1)[3:6], direct[3:], rtol=1e-15, atol=0)


def _one_burst(oracle, leapfrog=False):
    """gala's test_one_burst setting (tests/dynamics/mockstream/test_mockstream_class.py:41-97):
    NFW from v_c = 232.8 km/s at 8.2 kpc (r_s = 15), progenitor from (10, 0, 0) kpc at
    10 km/s with a Plummer potential (2.5e4 Msun, b = 4 pc), 1000 particles per tail
    released at the minimum radius of the 100-step Leapfrog orbit, Fardal draws from
    numpy.random.default_rng(42)."""
    from gala_gb300.mockstream import FardalStreamDF

    K = g.units.KMS_TO_KPC_MYR
    pot = g.NFWPotential.from_circular_velocity(v_c=232.8 * K, r_s=15.0, r_ref=8.2)
    w0 = np.array([10.0, 0, 0, 0, 10 * K, 0])
    t = g.parse_time_specification(dt=1.0, n_steps=100)
    r = np.linalg.norm(oracle.fixed(pot, w0[:, None], t, "leapfrog")[:3, :, 0], axis=0)
    counts = np.zeros(len(t), dtype=np.int64)
    counts[r[0:150].argmin()] = 1000
    bodies = pack_bodies([g.PlummerPotential(m=2.5e4, b=0.004)])
    if leapfrog:
        orb = oracle.leapfrog_nbody(pot, bodies, 1, w0.reshape(1, 6), t)
    else:
        orb, res = oracle.nbody_dop853(pot, bodies, 1, w0.reshape(1, 6), t)
        assert res == 1
    df = FardalStreamDF(gala_modified=True, random_state=np.random.default_rng(seed=42))
    offset = np.concatenate([[0], np.cumsum(2 * counts)]).astype(np.int64)
    sw0 = oracle.stream_sample(pot, orb.reshape(len(t), 6), np.full(len(t), 2.5e4), t, offset, 0,
                               df._draws(int(offset[-1])), g.units.G)
    rel = np.insert(np.nonzero(counts > 0)[0], 0, 0)
    return pot, bodies, orb, t, sw0, rel, counts


def test_one_burst_reproduces_galas_values(oracle):
    """The whole stream pipeline on the oracle -- sampling, the progenitor's n-body
    DOP853 and one 2001-particle release system -- reproduces the values gala's test
    asserts (test_mockstream_class.py:84-97, given to 8-9 digits)."""
    pot, bodies, orb, t, sw0, rel, counts = _one_burst(oracle)
    nb, st, status = oracle.mockstream_dop853(pot, bodies, orb[0].reshape(1, 6), t[rel], sw0, t[rel], t[-1],
                                              2 * counts[rel])
    stream0 = [-10.07444187, -1.37424641, 0.06310397, -0.05672946, -0.01837671, 0.00038504]
    prog = [-9.72388107, -1.28632464, 0.0, -0.04714419, -0.016754, 0.0]
    np.testing.assert_allclose(st[0], stream0, rtol=0, atol=1e-8)
    np.testing.assert_allclose(nb.reshape(-1)[:6], prog, rtol=0, atol=1e-8)


def test_leapfrog_release_split_is_exact(oracle):
    """Releases larger than a Leapfrog system are integrated in groups at the same
    time (split_releases); the result is bit-identical to one system per release."""
    from gala_gb300.mockstream import split_releases

    src, sizes = split_releases([0, 20, 3, 7], 7)
    assert src.tolist() == [0, 1, 1, 1, 2, 3] and sizes.tolist() == [0, 7, 7, 6, 3, 7]
    pot, bodies, orb, t, sw0, rel, counts = _one_burst(oracle, leapfrog=True)
    nb1, st1 = oracle.mockstream_leapfrog(pot, bodies, orb[0].reshape(1, 6), t, sw0, t[rel], t[-1], 2 * counts[rel])
    src, sizes = split_releases(2 * counts[rel], 7)
    nb2, st2 = oracle.mockstream_leapfrog(pot, bodies, orb[0].reshape(1, 6), t, sw0, t[rel][src], t[-1], sizes)
    assert len(src) > 200 and np.array_equal(st1, st2) and np.array_equal(nb1, nb2)


def test_dfs_refuse_no_tails():
    """gala's test_expected_failure (test_df.py:55-58) for every DF."""
    from gala_gb300.mockstream import ChenStreamDF, FardalStreamDF, LagrangeCloudStreamDF, StreaklineStreamDF

    for DF, kw in ((StreaklineStreamDF, {}), (FardalStreamDF, {"gala_modified": True}),
                   (LagrangeCloudStreamDF, {"v_disp": 1.0}), (ChenStreamDF, {})):
        with pytest.raises(ValueError):
            DF(lead=False, trail=False, **kw)


# ------------------------------------------------------------ animate mode
def _animate_args(c, s, output_every):
    """mockstream_dop853_animate's inputs: the whole orbit grid, the bodies at
    t[0] and the particles released at every grid time (zeros included)."""
    return dict(bodies=c["bodies"][s], nbody_w0=c["w0"][:, s].reshape(1, 6), t=c["t"], stream_w0=c["stream_w0"][s],
                nstream=2 * c["counts"], output_every=output_every)


def _n_output(nsteps, output_every):
    """gala's snapshot count (test_mockstream.py:304-306)."""
    return 1 + nsteps // output_every + int(nsteps % output_every != 0)


@pytest.mark.parametrize("n_steps,output_every,release_every", [(61, 3, 2), (40, 1, 1), (17, 2, 4)])
def test_mockstream_animate_oracle_matches_gala(oracle, gala_ref_strict, n_steps, output_every, release_every):
    c = stream_case(n_streams=1, n_steps=n_steps, release_every=release_every)
    a = _animate_args(c, 0, output_every)
    snap_o, t_o, w_o, st_o, stats = oracle.mockstream_animate(c["pot"], **a)
    snap_r, t_r, w_r, st_r, _ = gala_ref_strict.mockstream_animate(c["pot"], **a)
    assert snap_o.shape[0] == _n_output(n_steps, output_every)
    np.testing.assert_array_equal(st_o, st_r)
    assert np.all(st_o == 1) and stats[1] >= n_steps
    np.testing.assert_array_equal(t_o, t_r)
    np.testing.assert_array_equal(snap_o, snap_r)  # NaNs in the same places
    np.testing.assert_array_equal(w_o, w_r)


def test_mockstream_animate_snapshots(oracle):
    """Snapshot j holds the bodies and exactly the particles released at or
    before its time; the first is the initial state, the last the final one."""
    c = stream_case(n_streams=1, n_steps=30, release_every=4, n_per_tail=2)
    a = _animate_args(c, 0, 4)
    snap, snap_t, w_final, status, _ = oracle.mockstream_animate(c["pot"], **a)
    t, ns = c["t"], a["nstream"]
    assert snap_t.tolist() == [t[i] for i in (0, 4, 8, 12, 16, 20, 24, 28, 30)]
    released = np.cumsum(ns)
    for j, tj in enumerate(snap_t):
        i = int(np.nonzero(t == tj)[0][0])
        live = 1 + released[i]
        assert np.all(np.isfinite(snap[j, :live])) and np.all(np.isnan(snap[j, live:]))
    np.testing.assert_array_equal(snap[0, 1:1 + ns[0]], c["stream_w0"][0][:ns[0]])
    np.testing.assert_array_equal(snap[-1], w_final)


def test_mockstream_animate_agrees_with_release_systems(oracle):
    """One growing system and one system per release integrate the same
    test-particle orbits in the same progenitor field; at rtol 1e-10 the final
    streams agree to the integration tolerance, not bit for bit."""
    c = stream_case(n_streams=1, n_steps=60)
    _, _, w_a, _, _ = oracle.mockstream_animate(c["pot"], **_animate_args(c, 0, 10))
    nb, st, _ = oracle.mockstream_dop853(c["pot"], **_stream_args(c, 0))
    scale = np.abs(st).max(axis=0)
    np.testing.assert_allclose(w_a[1:], st, rtol=0, atol=1e-7 * scale.max())
    np.testing.assert_allclose(w_a[0], nb[0], rtol=1e-7)


def test_mockstream_animate_golden(oracle, golden):
    d = golden("mockstream_animate.npz")
    c = stream_case(n_streams=1, n_steps=int(d["n_steps"]), release_every=int(d["release_every"]))
    np.testing.assert_array_equal(c["stream_w0"][0], d["stream_w0"])
    snap, snap_t, w, status, _ = oracle.mockstream_animate(c["pot"], **_animate_args(c, 0, int(d["output_every"])))
    np.testing.assert_array_equal(status, d["status"])
    np.testing.assert_array_equal(snap_t, d["snap_t"])
    np.testing.assert_array_equal(np.isnan(snap), np.isnan(d["snap"]))
    scale = np.nanmax(np.abs(d["snap"]))
    np.testing.assert_allclose(snap, d["snap"], rtol=0, atol=OFAST_RTOL * scale)
