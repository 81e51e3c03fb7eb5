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
