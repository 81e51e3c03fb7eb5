"""Shared test cases: named potentials covering every component type and the
shift/rotate path (used by the tests and by tests/golden/make_golden.py)."""
import gala_gb300 as g
from gala_gb300 import workloads as W


def potentials():
    """Named potentials covering every component type and the shift/rotate path."""
    from scipy.spatial.transform import Rotation

    rot = Rotation.from_euler("zyx", [30.0, 20.0, -45.0], degrees=True).as_matrix()
    shifted = g.CCompositePotential()
    shifted["a"] = g.HernquistPotential(m=2e10, c=0.8, origin=[0.5, -0.3, 0.2])
    shifted["b"] = g.MiyamotoNagaiPotential(m=5e10, a=2.5, b=0.3, R=rot)
    shifted["c"] = g.NFWPotential(m=3e11, r_s=12.0, c=0.8, origin=[0.1, 0.0, -0.2], R=rot)
    return {
        "kepler": g.KeplerPotential(m=1e11),
        "hernquist": g.HernquistPotential(m=1e11, c=0.5),
        "plummer": g.PlummerPotential(m=1e10, b=0.6),
        "miyamotonagai": g.MiyamotoNagaiPotential(m=6.8e10, a=3.0, b=0.28),
        "sphericalnfw": g.NFWPotential(m=5.4e11, r_s=15.6),
        "flattenednfw": g.NFWPotential(m=5.4e11, r_s=15.6, c=0.8),
        "triaxialnfw": g.NFWPotential(m=5.4e11, r_s=15.6, a=1.2, b=1.0, c=0.8),
        "mw": W.mw_composite(),
        "shifted_rotated": shifted,
    }


def stream_case(n_streams=2, n_steps=150, dt=1.0, seed=21, n_per_tail=1, release_every=1, leapfrog=False):
    """A small batch of mock streams in the MW composite, built with the oracle:
    Plummer progenitors, progenitor orbits from gala's own n-body DOP853
    semantics, Fardal release states from seeded draws.  Returns a dict of the
    inputs of the release stage (layout of the GPU entry points).  With
    leapfrog=True the progenitor orbits come from gala's Leapfrog n-body loop."""
    import numpy as np

    from gala_gb300.mockstream import FardalStreamDF
    from gala_gb300.nbody import pack_bodies
    from oracle import Oracle

    orc = Oracle("strict")
    mw = W.mw_composite()
    w0, m, b = W.stream_progenitors(n_streams, seed=seed)
    pots = W.stream_progenitor_potentials(m, b)
    bodies = pack_bodies([[p] for p in pots])
    t = g.parse_time_specification(dt=dt, n_steps=n_steps)
    df = FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(seed))
    counts = df.release_counts(len(t), release_every, n_per_tail)
    offset = np.concatenate([[0], np.cumsum(2 * counts)]).astype(np.int64)
    orbits, stream_w0 = [], []
    for s in range(n_streams):
        if leapfrog:
            orb = orc.leapfrog_nbody(mw, bodies[s], 1, w0[:, s].reshape(1, 6), t)
        else:
            orb, res = orc.nbody_dop853(mw, bodies[s], 1, w0[:, s].reshape(1, 6), t, nstiff=-1)
            assert res == 1
        orbits.append(orb)
        draws = df._draws(int(offset[-1]))
        stream_w0.append(orc.fardal_sample(mw, orb.reshape(len(t), 6), np.full(len(t), m[s]), t, offset, draws,
                                           g.units.G))
    rel = np.nonzero(counts > 0)[0]
    if 0 not in rel:
        rel = np.insert(rel, 0, 0)
    return dict(pot=mw, bodies=bodies, w0=w0, m=m, b=b, t=t, counts=counts, offset=offset,
                orbits=np.stack(orbits), stream_w0=np.stack(stream_w0), rel=rel, nstream=2 * counts[rel],
                seed=seed)
