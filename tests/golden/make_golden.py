"""Generate the golden fixtures in tests/golden/ from gala's OWN compiled code.

Run in a container that has the gala sources (oracle/Makefile compiles them into
oracle/_ref/libgalaref.so with gala's release flags, -Ofast):

    python tests/golden/make_golden.py

Every fixture holds seeded inputs and the outputs gala's C/C++ produced for
them (Leapfrog / Ruth4 loops of leapfrog.pyx / ruth4.pyx around gala's
c_gradient, and gala's dop853() called as dop853_helper calls it).  SCF
fixtures are a fixed subset of the Fortran SCF known-answer data that gala's
own tests use (tests/potential/scf/data/*-accp.dat.gz, positions.dat.gz,
*.coeff), converted to Lowing-2011 coefficients as test_accp_fortran.py does.
"""
from __future__ import annotations

import sys
from math import factorial
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import gala_gb300 as g  # noqa: E402
from gala_gb300 import workloads as W  # noqa: E402
from oracle import Oracle, build  # noqa: E402
from tests._cases import potentials  # noqa: E402

OUT = Path(__file__).resolve().parent
GALA_TESTS = Path("/root/reference/tests")
SNAP_EVERY = 50


def make_potential_fixture(ref: Oracle):
    rng = np.random.default_rng(7)
    q = rng.normal(0.0, 8.0, size=(3, 64))
    data = {"q": q}
    for name, pot in potentials().items():
        data[f"{name}/gradient"] = ref.gradient(pot, q)
        data[f"{name}/value"] = ref.energy(pot, q)
        if name not in ("flattenednfw", "triaxialnfw"):
            data[f"{name}/density"] = ref.density(pot, q)
        w = np.vstack([q, rng.normal(0, 0.2, size=(3, 64))])
        data[f"{name}/w"] = w
        data[f"{name}/hamiltonian_gradient"] = ref.hamiltonian_gradient(pot, w)
    np.savez_compressed(OUT / "potentials.npz", **data)


def make_integrator_fixtures(ref: Oracle):
    # Hernquist m=1e11, c=0.5 with dt = +2 and -2 over 1024 steps (the setting of
    # gala's tests/integrate/test_cyintegrators.py), seeded ICs.
    pot = g.HernquistPotential(m=1e11, c=0.5)
    w0 = W.hernquist_ics(24, seed=11, m=1e11, c=0.5)
    data = {"w0": w0}
    for sign, tag in [(1.0, "fwd"), (-1.0, "bwd")]:
        t = g.parse_time_specification(dt=2.0 * sign, n_steps=1024)
        data[f"t_{tag}"] = t
        for method in ("leapfrog", "ruth4"):
            w = ref.fixed(pot, w0, t, method, save_all=True)
            data[f"{method}_{tag}"] = w[:, ::SNAP_EVERY, :]
            data[f"{method}_{tag}_final"] = w[:, -1, :]
    np.savez_compressed(OUT / "hernquist_fixed.npz", **data)

    # MW composite DOP853, two batches of 10 plus a ragged batch of 3
    mw = W.mw_composite()
    w0 = W.mw_ics(23, seed=12)
    t = g.parse_time_specification(dt=0.5, n_steps=2000)
    w, st, _ = ref.dop853(mw, w0, t, atol=1e-12, rtol=1e-10, nbatch=10)
    assert np.all(st == 1), st
    np.savez_compressed(OUT / "mw_dop853.npz", w0=w0, t=t, w=w[:, ::SNAP_EVERY, :], final=w[:, -1, :],
                        status=st, nbatch=10, atol=1e-12, rtol=1e-10)

    # MW composite, Leapfrog and Ruth4 (composite with MN pow and NFW log)
    w0 = W.mw_ics(16, seed=13)
    t = g.parse_time_specification(dt=1.0, n_steps=1000)
    data = {"w0": w0, "t": t}
    for method in ("leapfrog", "ruth4"):
        w = ref.fixed(mw, w0, t, method, save_all=True)
        data[method] = w[:, ::SNAP_EVERY, :]
    np.savez_compressed(OUT / "mw_fixed.npz", **data)

    # rotating frame, DOP853 (Hamiltonian with ConstantRotatingFrame)
    frame = g.ConstantRotatingFrame(Omega=[0.0, 0.0, 0.04])
    w0 = W.mw_ics(8, seed=14)
    t = g.parse_time_specification(dt=0.5, n_steps=800)
    w, st, _ = ref.dop853(mw, w0, t, atol=1e-12, rtol=1e-10, nbatch=8, frame=frame)
    np.savez_compressed(OUT / "mw_rotating_dop853.npz", w0=w0, t=t, w=w[:, ::SNAP_EVERY, :], final=w[:, -1, :],
                        status=st, omega=np.array([0.0, 0.0, 0.04]))


def lowing_coefficients(coeff_path):
    coeff = np.atleast_2d(np.loadtxt(coeff_path, skiprows=1))
    nmax = coeff[:, 0].astype(int).max()
    lmax = coeff[:, 1].astype(int).max()
    S = np.zeros((nmax + 1, lmax + 1, lmax + 1))
    T = np.zeros((nmax + 1, lmax + 1, lmax + 1))
    for n, l, m, cc, sc in coeff:
        if l != 0:  # H&O 1992 -> Lowing 2011 normalisation (test_accp_fortran.py)
            fac = np.sqrt(4 * np.pi) * np.sqrt((2 * l + 1) / (4 * np.pi) * factorial(int(l - m)) /
                                               factorial(int(l + m)))
            cc /= fac
            sc /= fac
        S[int(n), int(l), int(m)] = cc
        T[int(n), int(l), int(m)] = sc
    return S, T


def make_scf_fixture():
    data_dir = GALA_TESTS / "potential" / "scf" / "data"
    xyz = np.loadtxt(data_dir / "positions.dat.gz", skiprows=1)
    idx = np.random.default_rng(3).choice(len(xyz), 400, replace=False)
    idx.sort()
    data = {"xyz": xyz[idx].T.copy()}
    for name in ["simple-hernquist", "multi-hernquist", "simple-nonsph", "random", "wang-zhao"]:
        S, T = lowing_coefficients(data_dir / f"{name}.coeff")
        accp = np.loadtxt(data_dir / f"{name}-accp.dat.gz")[idx]
        data[f"{name}/S"] = S
        data[f"{name}/T"] = T
        data[f"{name}/grad"] = accp[:, :3].T.copy()   # gala compares gradient to these directly
        data[f"{name}/pot"] = -accp[:, -1]            # and the potential to minus the last column
    np.savez_compressed(OUT / "scf_fortran.npz", **data)


def make_stream_fixtures(ref: Oracle):
    """gala's direct_nbody_dop853 and mockstream_dop853 (gala's own dop853(),
    Fwrapper_direct_nbody, c_nbody_acceleration) on the shared test cases."""
    from tests._cases import stream_case
    from tests.test_mockstream_oracle import _nbody_system, _stream_args

    mw, bodies, w0, t = _nbody_system()
    w, res = ref.nbody_dop853(mw, bodies, 2, w0, t)
    assert res == 1
    np.savez_compressed(OUT / "nbody_dop853.npz", w0=w0, t=t, w=w[::50])

    n_streams, n_steps = 2, 120
    c = stream_case(n_streams=n_streams, n_steps=n_steps)
    out = {"n_streams": n_streams, "n_steps": n_steps, "stream_w0": c["stream_w0"]}
    streams, nbodies, status = [], [], []
    for s in range(n_streams):
        nb, st, stat = ref.mockstream_dop853(c["pot"], **_stream_args(c, s))
        streams.append(st)
        nbodies.append(nb)
        status.append(stat)
    np.savez_compressed(OUT / "mockstream_dop853.npz", stream=np.stack(streams), nbody=np.stack(nbodies),
                        status=np.stack(status), **out)

    # Leapfrog: leapfrog_integrate_nbody and mockstream_leapfrog
    from tests.test_mockstream_oracle import _lf_nbody_args, _lf_stream_args

    c = stream_case(n_streams=n_streams, n_steps=n_steps, leapfrog=True)
    streams, nbodies = [], []
    for s in range(n_streams):
        nb, st = ref.mockstream_leapfrog(c["pot"], **_lf_stream_args(c, s))
        streams.append(st)
        nbodies.append(nb)
    np.savez_compressed(OUT / "mockstream_leapfrog.npz", stream=np.stack(streams), nbody=np.stack(nbodies),
                        n_streams=n_streams, n_steps=n_steps, stream_w0=c["stream_w0"],
                        nbody_leapfrog=ref.leapfrog_nbody(c["pot"], *_lf_nbody_args()))


def make_animate_fixture(ref: Oracle):
    """gala's mockstream_dop853_animate (gala's dop853() on the growing system,
    interval by interval) on a shared test case: 41 steps, a release every 2nd
    step, a snapshot every 3rd."""
    from tests._cases import stream_case
    from tests.test_mockstream_oracle import _animate_args

    n_steps, release_every, output_every = 41, 2, 3
    c = stream_case(n_streams=1, n_steps=n_steps, release_every=release_every)
    snap, snap_t, w, status, _ = ref.mockstream_animate(c["pot"], **_animate_args(c, 0, output_every))
    np.savez_compressed(OUT / "mockstream_animate.npz", snap=snap, snap_t=snap_t, w=w, status=status,
                        stream_w0=c["stream_w0"][0], n_steps=n_steps, release_every=release_every,
                        output_every=output_every)


def make_io_fixture():
    """gala's own serialisation test inputs, kept as text: the potential YAML
    files of tests/potential/potential/ (read by test_io.py) and one HDF5 file
    written by libhdf5 (an EXP coefficient file read by test_exp.py), base64."""
    import base64
    import json

    pdir = GALA_TESTS / "potential" / "potential"
    data = {
        "yaml": {n: (pdir / n).read_text() for n in ("Plummer.yml", "Composite.yml", "ccomposite.yml", "lm10.yml",
                                                      "HarmonicOscillator1D.yml")},
        "hdf5_base64": {n: base64.b64encode((pdir / n).read_bytes()).decode()
                        for n in ("EXP-Hernquist-single-coefs.hdf5",)},
    }
    (OUT / "io_reference_files.json").write_text(json.dumps(data, indent=1) + "\n")


if __name__ == "__main__":
    # python tests/golden/make_golden.py [potentials integrators scf streams animate io]
    which = set(sys.argv[1:]) or {"potentials", "integrators", "scf", "streams", "animate", "io"}
    if "io" in which and GALA_TESTS.exists():
        make_io_fixture()
    which.discard("io")
    if not which:
        sys.exit(0)
    build(ref=True)
    ref = Oracle("ref")
    if "potentials" in which:
        make_potential_fixture(ref)
    if "integrators" in which:
        make_integrator_fixtures(ref)
    if "scf" in which and GALA_TESTS.exists():
        make_scf_fixture()
    if "streams" in which:
        make_stream_fixtures(ref)
    if "animate" in which:
        make_animate_fixture(ref)
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, p.stat().st_size)
