"""CPU tests: the C-ABI library exports what include/gala_gb300.h declares, the
ctypes mirror matches the header, and the host-side API behaves like gala's."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import gala_gb300 as g
from gala_gb300 import _abi, workloads
from gala_gb300.integrate import parse_time_specification

ROOT = Path(__file__).resolve().parents[1]


def _declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(gx_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_loads_and_exports_every_declared_symbol():
    lib = _abi.load()  # builds with nvcc if needed; loads without touching a GPU
    declared = _declared_functions()
    assert declared, "no declarations found"
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_abi.SIGNATURES) >= declared, declared - set(_abi.SIGNATURES)
    assert lib.gx_abi_version() == 3


def test_struct_layout_matches_header():
    # gx_component: 4+4+8+4+4 + 3*8 + 9*8 = 120 bytes, 8-byte aligned
    assert C.sizeof(_abi.gx_component) == 120
    assert _abi.gx_component.q0.offset == 24
    assert C.sizeof(_abi.gx_potential) == 48
    assert C.sizeof(_abi.gx_frame) == 32


def test_invalid_descriptor_is_rejected_without_gpu():
    """Argument validation happens on the host before any CUDA call."""
    lib = _abi.load()
    pot = g.HernquistPotential(m=1e11, c=1.0)
    desc = pot.packed().desc
    desc.n_dim = 2
    rc = lib.gx_potential_value(C.byref(desc), 0.0, None, 10, None, None)
    assert rc == _abi.GX_ERR_INVALID_ARGUMENT
    assert b"n_dim" in lib.gx_last_error_message()
    desc.n_dim = 3
    rc = lib.gx_dop853_integrate_hamiltonian(C.byref(desc), None, None, 10, None, 100, 1e-10, 1e-10, 0, 0.0, 0, 1,
                                             0, 1, None, None, None, None)
    assert rc == _abi.GX_ERR_INVALID_ARGUMENT
    assert b"nbatch" in lib.gx_last_error_message()


def test_parameter_packing_is_gala_layout():
    G = g.units.G
    assert np.array_equal(g.HernquistPotential(m=2.0, c=3.0).packed().params, [G, 2.0, 3.0])
    assert np.array_equal(g.MiyamotoNagaiPotential(1.0, 2.0, 3.0).packed().params, [G, 1.0, 2.0, 3.0])
    nfw = g.NFWPotential(m=5.0, r_s=2.0)
    assert np.array_equal(nfw.packed().params, [G, 5.0, 2.0, 1.0, 1.0, 1.0])
    assert nfw.packed().components[0].type == _abi.GX_POT_SPHERICALNFW
    assert g.NFWPotential(m=5.0, r_s=2.0, c=0.9).packed().components[0].type == _abi.GX_POT_FLATTENEDNFW
    assert g.NFWPotential(m=5.0, r_s=2.0, a=1.1, c=0.9).packed().components[0].type == _abi.GX_POT_TRIAXIALNFW
    S = np.arange(8.0).reshape(2, 2, 2)
    scf = g.SCFPotential(m=1.0, r_s=2.0, Snlm=S, Tnlm=-S)
    p = scf.packed().params
    assert np.array_equal(p[:5], [G, 1.0, 1.0, 1.0, 2.0])
    assert np.array_equal(p[5:13], S.ravel()) and np.array_equal(p[13:], -S.ravel())


def test_composite_order_and_shift_flag():
    mw = g.MilkyWayPotential()
    pk = mw.packed()
    assert [pk.components[i].type for i in range(4)] == [_abi.GX_POT_MIYAMOTONAGAI, _abi.GX_POT_HERNQUIST,
                                                         _abi.GX_POT_HERNQUIST, _abi.GX_POT_SPHERICALNFW]
    assert all(pk.components[i].do_shift_rotate == 0 for i in range(4))
    sh = g.HernquistPotential(m=1.0, c=1.0, origin=[1.0, 0, 0])
    assert sh.packed().components[0].do_shift_rotate == 1
    with pytest.raises(ValueError):
        mw["extra"] = g.NullPotential()
    comp = g.HernquistPotential(m=1.0, c=1.0) + g.PlummerPotential(m=1.0, b=1.0)
    assert len(comp) == 2


@pytest.mark.parametrize("kw,expected", [
    (dict(dt=0.5, n_steps=4), np.cumsum(np.append([0.0], np.ones(5) * 0.5))[:-1]),
    (dict(dt=0.5, n_steps=4, t1=10.0), np.cumsum(np.append([0.0], np.ones(5) * 0.5))[:-1] + 10.0),
    (dict(dt=1.0, t1=0.0, t2=3.5), np.array([0.0, 1.0, 2.0, 3.0])),
    (dict(dt=-1.0, t1=3.0, t2=0.5), np.array([3.0, 2.0, 1.0, 0.5])),
    (dict(n_steps=5, t1=0.0, t2=1.0), np.linspace(0, 1, 5)),
    (dict(t=np.array([0.0, 2.0, 5.0])), np.array([0.0, 2.0, 5.0])),
])
def test_time_specification_like_gala(kw, expected):
    assert np.array_equal(parse_time_specification(None, **kw), expected)


def test_time_specification_errors():
    with pytest.raises(ValueError):
        parse_time_specification(None, dt=0.0, t1=0.0, t2=1.0)
    with pytest.raises(ValueError):
        parse_time_specification(None, dt=1.0, t1=1.0, t2=0.0)
    with pytest.raises(ValueError):
        parse_time_specification(None, n_steps=10)


def test_integrator_lookup():
    assert g.get_integrator("LeapFrog") is g.LeapfrogIntegrator
    assert g.get_integrator("dop853") is g.DOPRI853Integrator
    assert g.get_integrator("dopri853") is g.DOPRI853Integrator
    assert g.get_integrator(g.Ruth4Integrator) is g.Ruth4Integrator
    with pytest.raises(ValueError):
        g.get_integrator("euler")


def test_product_path_fails_loudly_without_gpu():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    pot = g.HernquistPotential(m=1e11, c=1.0)
    with pytest.raises(RuntimeError, match="CUDA"):
        pot.integrate_orbit(np.ones((6, 2)), dt=1.0, n_steps=10)
    with pytest.raises(RuntimeError, match="CUDA"):
        pot.gradient(np.ones((3, 2)))


def test_integrate_orbit_argument_errors_come_before_the_device():
    """gala's argument errors (chamiltonian.pyx:282-310, leapfrog.pyx:61-68,
    timespec.py:91-145) are raised whether or not a GPU is present."""
    pot = g.HernquistPotential(m=1e11, c=1.0)
    w0 = np.ones((6, 2))
    with pytest.raises(ValueError, match="shape"):
        pot.integrate_orbit(np.ones((5, 2)), dt=1.0, n_steps=10)
    with pytest.raises(ValueError):
        pot.integrate_orbit(w0, dt=0.0, t1=0.0, t2=1.0)
    with pytest.raises(ValueError, match="ntimes"):
        pot.integrate_orbit(w0, t=np.array([0.0]))
    H = g.Hamiltonian(pot, frame=g.ConstantRotatingFrame(Omega=[0.0, 0.0, 1e-2]))
    for integ, name in ((g.LeapfrogIntegrator, "Leapfrog"), (g.Ruth4Integrator, "Ruth4")):
        with pytest.warns(RuntimeWarning, match="non-static frame"):
            with pytest.raises(TypeError, match=f"{name} integration is currently only supported for StaticFrame"):
                H.integrate_orbit(w0, Integrator=integ, dt=1.0, n_steps=10)
    for kw, msg in ((dict(nbatch=0), "nbatch"), (dict(nbatch=2000), "nbatch"), (dict(out_stride=0), "out_stride")):
        with pytest.raises(ValueError, match=msg):
            pot.integrate_orbit(w0, Integrator=g.DOPRI853Integrator, Integrator_kwargs=kw, dt=1.0, n_steps=10)
    with pytest.raises(ValueError):
        pot.integrate_orbit(w0, Integrator="euler", dt=1.0, n_steps=10)


def test_nbody_and_mockstream_argument_errors(tmp_path):
    """Constructor and argument checks of DirectNBody (nbody/core.py:25-95) and
    MockStreamGenerator / stream DFs (mockstream_generator.py:20-100, df.pyx:48-60)."""
    from gala_gb300.mockstream import FardalStreamDF, MockStreamGenerator
    from gala_gb300.nbody import DirectNBody

    pot = workloads.mw_composite()
    psp = g.PhaseSpacePosition(pos=np.ones((3, 2)), vel=np.zeros((3, 2)))
    with pytest.raises(TypeError, match="PhaseSpacePosition"):
        DirectNBody(np.ones((6, 2)), [None, None], external_potential=pot)
    with pytest.raises(ValueError, match="must match the number of particle"):
        DirectNBody(psp, [None], external_potential=pot)
    nb = DirectNBody(psp, [g.PlummerPotential(m=1e6, b=0.01), None], external_potential=pot)
    with pytest.raises(NotImplementedError):
        nb.integrate_orbit(Integrator=g.Ruth4Integrator, dt=1.0, n_steps=4)
    with pytest.raises(ValueError, match="leading or trailing"):
        FardalStreamDF(gala_modified=True, lead=False, trail=False)
    df = FardalStreamDF(gala_modified=True)
    with pytest.warns(FutureWarning):
        FardalStreamDF()
    with pytest.raises(ValueError, match="n_particles"):
        df.release_counts(10, n_particles=np.ones(9))
    with pytest.raises(TypeError, match="BaseStreamDF"):
        MockStreamGenerator(object(), pot)
    with pytest.raises(TypeError, match="progenitor_potential"):
        MockStreamGenerator(df, pot, progenitor_potential=1.0)
    gen = MockStreamGenerator(df, pot, progenitor_potential=g.PlummerPotential(m=1e5, b=0.01))
    prog = g.PhaseSpacePosition(pos=[10.0, 0, 0], vel=[0, 0.2, 0])
    with pytest.raises(ValueError, match="DOPRI853Integrator and LeapfrogIntegrator"):
        gen.run(prog, 1e5, Integrator=g.Ruth4Integrator, dt=1.0, n_steps=4)
    # the animate mode's checks, all before any integration (mockstream_generator.py:296-336,
    # mockstream.pyx:116-134)
    with pytest.raises(ValueError, match="filename"):
        gen.run(prog, 1e5, output_every=2, dt=1.0, n_steps=4)
    with pytest.raises(ValueError, match="filename"):
        gen.run(prog, 1e5, output_every=2, Integrator="leapfrog", dt=1.0, n_steps=4)
    with pytest.raises(NotImplementedError, match="LeapfrogIntegrator"):
        gen.run(prog, 1e5, output_every=2, output_filename="x.h5", Integrator="leapfrog", dt=1.0, n_steps=4)
    with pytest.raises(ValueError, match="precision"):
        gen.run(prog, 1e5, output_every=2, output_filename="x.h5", Integrator_kwargs=dict(precision="fp16"),
                dt=1.0, n_steps=4)
    with pytest.raises(ValueError, match="positive"):
        gen.run(prog, 1e5, output_every=0, output_filename="x.h5", dt=1.0, n_steps=4)
    existing = tmp_path / "exists.hdf5"
    existing.write_bytes(b"")
    with pytest.raises(OSError, match="already exists"):
        gen.run(prog, 1e5, output_every=2, output_filename=str(existing), dt=1.0, n_steps=4)
    with pytest.raises(OSError, match="already exists"), pytest.warns(UserWarning, match="8 GB"):
        gen.run(prog, 1e5, output_every=1, output_filename=str(existing), n_particles=200_000, dt=1.0,
                n_steps=4000)
    other = DirectNBody(psp, [None, None], external_potential=g.HernquistPotential(m=1e11, c=1.0))
    with pytest.raises(ValueError, match="external potential"):
        gen.run(prog, 1e5, nbody=other, dt=1.0, n_steps=4)
    with pytest.raises(ValueError, match="prog_w0"):
        gen.run_batch(np.ones((5, 3)), 1e5, dt=1.0, n_steps=4)
    with pytest.raises(ValueError, match="one progenitor potential"):
        gen.run_batch(np.ones((6, 3)), 1e5, progenitor_potentials=[None], dt=1.0, n_steps=4)


def _int_entry_points():
    return [n for n, (res, args) in _abi.SIGNATURES.items() if res is C.c_int and args]


@pytest.mark.parametrize("variant", ["null_descriptor_negative_sizes", "null_buffers"])
@pytest.mark.parametrize("name", _int_entry_points())
def test_every_entry_point_rejects_bad_arguments_on_the_host(name, variant):
    """Each C entry point validates its descriptor, sizes and pointers before
    any CUDA call: NULL descriptors with negative sizes, or a valid descriptor
    with positive sizes and NULL buffers, return GX_ERR_INVALID_ARGUMENT with
    a message (no GPU is needed to see it)."""
    lib = _abi.load()
    _, args = _abi.SIGNATURES[name]
    pk = g.HernquistPotential(m=1e11, c=1.0).packed()
    frame = g.StaticFrame().c_frame()
    vals = []
    for a in args:
        if a in (_abi._I64, _abi._I32):
            vals.append(-1 if variant == "null_descriptor_negative_sizes" else 4)
        elif a in (C.c_double, C.c_float):
            vals.append(1e-3)
        elif a is _abi._PP:
            vals.append(None if variant == "null_descriptor_negative_sizes" else pk.for_host())
        elif a is _abi._P:
            vals.append(None)
        else:  # the frame descriptor
            vals.append(None if variant == "null_descriptor_negative_sizes" else C.byref(frame))
    rc = getattr(lib, name)(*vals)
    assert rc == _abi.GX_ERR_INVALID_ARGUMENT
    assert lib.gx_last_error_message()


def test_public_calls_open_nvtx_ranges(monkeypatch):
    """Each public GPU call runs inside an NVTX range named gala_gb300.<call>
    (the range opens before any argument check, so a failing call shows too)."""
    import contextlib

    import torch

    seen = []

    @contextlib.contextmanager
    def fake_range(name):
        seen.append(name)
        yield

    monkeypatch.setattr(torch.cuda.nvtx, "range", fake_range)
    pot = g.HernquistPotential(m=1e11, c=1.0)
    with pytest.raises(ValueError):
        pot.integrate_orbit(np.ones((5, 2)), dt=1.0, n_steps=4)
    with pytest.raises(ValueError):
        pot.energy(np.ones((2, 2)))
    assert seen == ["gala_gb300.integrate_orbit", "gala_gb300.potential_eval"]


def test_symplectic_entry_points_refuse_rotating_frames_on_the_host():
    """leapfrog.pyx:61-68 / ruth4.pyx: a non-static frame is refused with gala's
    message; the C entry points return GX_ERR_UNSUPPORTED before any CUDA call."""
    lib = _abi.load()
    pk = g.HernquistPotential(m=1e11, c=1.0).packed()
    fr = g.ConstantRotatingFrame(Omega=[0.0, 0.0, 0.1]).c_frame()
    for name, label in (("gx_leapfrog_integrate_hamiltonian", b"Leapfrog"), ("gx_ruth4_integrate_hamiltonian", b"Ruth4")):
        rc = getattr(lib, name)(pk.for_host(), C.byref(fr), None, 0, None, 3, 1, None, None)
        assert rc == _abi.GX_ERR_UNSUPPORTED
        assert lib.gx_last_error_message() == label + b" integration is currently only supported for StaticFrame"


class _Quantity:
    """A stand-in for an astropy Quantity: value, unit and to_value(unit)."""

    SCALE = {"Msun": 1.0, "kpc": 1.0, "pc": 1e-3, "": 1.0, "Gyr": 1e3}

    def __init__(self, value, unit):
        self.value, self.unit = value, unit

    def to_value(self, unit):
        if (self.unit in ("kpc", "pc")) != (unit == "kpc") and unit != "":
            raise ValueError(f"cannot convert {self.unit} to {unit}")
        return np.asarray(self.value) * self.SCALE[self.unit] / self.SCALE[unit]


def test_quantity_parameters_are_converted_not_stripped():
    pot = g.HernquistPotential(m=_Quantity(1e11, "Msun"), c=_Quantity(260.0, "pc"))
    assert pot.parameters["c"] == pytest.approx(0.26) and pot.parameters["m"] == 1e11
    with pytest.raises(ValueError):
        g.HernquistPotential(m=1e11, c=_Quantity(1.0, "Gyr"))
    nfw = g.NFWPotential(m=1e11, r_s=_Quantity(12000.0, "pc"), c=_Quantity(0.9, ""))
    assert nfw.parameters["r_s"] == pytest.approx(12.0) and nfw.parameters["c"] == 0.9


def test_phase_space_objects_with_units_are_converted():
    """Any object with xyz / v_xyz (gala's PhaseSpacePosition) gives kpc and kpc/Myr."""
    from gala_gb300.dynamics import phase_space_array

    class _PSP:
        def __init__(self, xyz, v_xyz):
            self.xyz, self.v_xyz = xyz, v_xyz

    class _Q(_Quantity):
        SCALE = {"pc": 1e-3, "kpc": 1.0, "kpc / Myr": 1.0, "km / s": g.units.KMS_TO_KPC_MYR}

        def to_value(self, unit):
            return np.asarray(self.value) * self.SCALE[self.unit] / self.SCALE[unit]

    w = phase_space_array(_PSP(_Q([[8000.0], [0.0], [0.0]], "pc"), _Q([[0.0], [220.0], [0.0]], "km / s")))
    np.testing.assert_allclose(w[:, 0], [8.0, 0, 0, 0, 220 * g.units.KMS_TO_KPC_MYR, 0])
    own = g.PhaseSpacePosition(pos=[1.0, 2, 3], vel=[4.0, 5, 6])
    assert np.array_equal(phase_space_array(own), [1.0, 2, 3, 4, 5, 6])
    with pytest.raises(ValueError, match="shape"):   # still validated before the device
        g.HernquistPotential(m=1e11, c=1.0).integrate_orbit(_PSP(np.ones((2, 1)), np.ones((2, 1))), dt=1.0,
                                                            n_steps=3)


def test_time_specification_with_quantities():
    class _T(_Quantity):
        SCALE = {"Myr": 1.0, "Gyr": 1e3}

        def to_value(self, unit):
            return np.asarray(self.value) * self.SCALE[self.unit] / self.SCALE[unit]

    t = parse_time_specification(None, dt=_T(0.001, "Gyr"), n_steps=3)
    np.testing.assert_allclose(t, [0.0, 1.0, 2.0, 3.0])
    t = parse_time_specification(None, t=_T([0.0, 0.5], "Gyr"))
    np.testing.assert_allclose(t, [0.0, 500.0])


def test_nfw_from_circular_velocity_with_quantities():
    """gala's TestSphericalNFWFromCircVel setting (test_all_builtin.py:286-300):
    v_c = 220 km/s at r_ref = 8 kpc with r_s = 20 kpc; the circular speed at
    r_ref is v_c (checked with the closed-form NFW enclosed mass)."""
    class _V(_Quantity):
        SCALE = {"km / s": g.units.KMS_TO_KPC_MYR, "kpc / Myr": 1.0, "kpc": 1.0}

        def to_value(self, unit):
            return np.asarray(self.value) * self.SCALE[self.unit] / self.SCALE[unit]

    pot = g.NFWPotential.from_circular_velocity(v_c=_V(220.0, "km / s"), r_s=_V(20.0, "kpc"), r_ref=_V(8.0, "kpc"))
    m, r_s, r = pot.parameters["m"], pot.parameters["r_s"], 8.0
    menc = m * (np.log(1 + r / r_s) - (r / r_s) / (1 + r / r_s))
    np.testing.assert_allclose(np.sqrt(g.units.G * menc / r), 220.0 * g.units.KMS_TO_KPC_MYR, rtol=1e-12)
    for r_ref in (3.0, 8.0, 21.7234):                # gala's test_circ_vel radii, plain floats
        p = g.NFWPotential.from_circular_velocity(v_c=0.22, r_s=20.0, r_ref=r_ref)
        m, u = p.parameters["m"], r_ref / 20.0
        v = np.sqrt(g.units.G * m * (np.log(1 + u) - u / (1 + u)) / r_ref)
        np.testing.assert_allclose(v, 0.22, rtol=1e-12)


def test_large_composite_packs_a_component_table():
    """More than GX_MAX_COMPONENTS components (gala has no limit): the packed
    descriptor keeps every component, the library writes a component table of
    the stated size, and a bad component is refused before anything is written."""
    n = _abi.GX_MAX_COMPONENTS + 1
    comp = g.CompositePotential(**{f"h{i}": g.HernquistPotential(m=1e9, c=0.1, origin=[0.01 * i, 0, 0])
                                   for i in range(n)})
    pk = comp.packed()
    assert pk.desc.n_components == n and pk.large
    lib = _abi.load()
    nbytes = lib.gx_component_table_bytes(n)
    assert nbytes > 0 and nbytes % n == 0
    buf = np.zeros(nbytes, dtype=np.uint8)
    assert lib.gx_pack_component_table(pk.for_host(), buf.ctypes.data, nbytes) == _abi.GX_OK
    assert buf.any()
    assert lib.gx_pack_component_table(pk.for_host(), buf.ctypes.data, nbytes - 1) == _abi.GX_ERR_INVALID_ARGUMENT
    pk.components[3].type = 99
    assert lib.gx_pack_component_table(pk.for_host(), buf.ctypes.data, nbytes) == _abi.GX_ERR_INVALID_ARGUMENT
    ok = g.CompositePotential(**{f"h{i}": g.HernquistPotential(m=1e9, c=0.1) for i in range(_abi.GX_MAX_COMPONENTS)})
    assert not ok.packed().large


def test_stepped_time_grids_are_running_sums():
    """dt, t1, t2 grids: each time is the previous one plus dt (gala's running
    sum, timespec.py:100-121); a forward grid stops short of t2, a backward one
    ends on t2 exactly."""
    rng = np.random.default_rng(0)

    def running(t1, t2, dt):
        out, x = [], t1
        while (x < t2) if dt > 0 else (x > t2):
            out.append(x)
            x += dt
        if dt < 0 and out[-1] != t2:
            out.append(t2)
        return np.array(out)

    for _ in range(500):
        t1 = rng.uniform(-100, 100)
        span = rng.uniform(0.1, 500)
        dt = rng.choice([0.1, 1 / 3, 0.7, 1.0, rng.uniform(0.01, 5)])
        for sgn in (1, -1):
            got = g.parse_time_specification(dt=sgn * dt, t1=t1, t2=t1 + sgn * span)
            assert np.array_equal(got, running(t1, t1 + sgn * span, sgn * dt))


def test_debug_library_reports_its_build():
    """libgala_gb300_debug.so is the same ABI with the device-side check records
    (GX_DEBUG_CHECKS); the release library keeps none and says so."""
    import ctypes as C

    rel, dbg = _abi.load(), _abi.load_debug()
    assert rel.gx_debug_enabled() == 0 and dbg.gx_debug_enabled() == 1
    assert dbg.gx_abi_version() == rel.gx_abi_version()
    out = (C.c_int64 * 9)()
    assert rel.gx_debug_read(C.cast(out, C.c_void_p), 0) == _abi.GX_ERR_UNSUPPORTED
    assert b"release library" in rel.gx_last_error_message()


def test_rotating_frame_transform_matches_galas_rotation():
    """rotate_frame / PhaseSpacePosition.to_frame against the oracle's restatement
    of gala's static <-> constant-rotating transformations
    (transformations.py:96-191), and the round trip."""
    from gala_gb300.hamiltonian import rotate_frame
    from oracle import orbit_oracle as OO

    rng = np.random.default_rng(3)
    Omega = np.array([0.01, -0.02, 0.03])
    w = rng.normal(size=(40, 6))
    t = rng.uniform(-500, 500, 40)
    for to_rot, sign in ((True, 1.0), (False, -1.0)):
        got = rotate_frame(w, t, Omega, to_rotating=to_rot)
        px, pv = OO.constantrotating_static(Omega, w[:, :3].T, w[:, 3:].T, t, sign)
        np.testing.assert_allclose(got, np.vstack([px, pv]).T, rtol=0, atol=1e-14)
    fr = g.ConstantRotatingFrame(Omega=Omega)
    o = g.Orbit(pos=w[:, :3].T.reshape(3, 8, 5), vel=w[:, 3:].T.reshape(3, 8, 5), t=np.linspace(0, 70, 8),
                frame=g.StaticFrame())
    back = o.to_frame(fr).to_frame(g.StaticFrame())
    np.testing.assert_allclose(back.pos, o.pos, atol=1e-13)
    np.testing.assert_allclose(back.vel, o.vel, atol=1e-13)
    psp = g.PhaseSpacePosition(pos=[1.0, 2.0, 3.0], vel=[0.1, 0.2, 0.3], frame=g.StaticFrame())
    with pytest.raises(ValueError, match="Time"):
        psp.to_frame(fr)
    with pytest.raises(ValueError, match="current_frame"):
        g.PhaseSpacePosition(pos=[1.0, 2.0, 3.0], vel=[0.1, 0.2, 0.3]).to_frame(fr)


def test_batch_queue_regions_taken():
    """BatchIntegrator._taken_slots: the orbits a (possibly cancelled) run took
    are the first q[1] 32-orbit blocks of the lead region (at most one block per
    SM sub-partition, whole chunks) and the first q[0] chunks after it."""
    import torch

    from gala_gb300.batch import BatchIntegrator

    b = object.__new__(BatchIntegrator)
    b.sms = 152
    b.config = {"chunk": 64}
    b.order = torch.arange(64 * 1000, dtype=torch.int32)
    b.counter = torch.zeros(1026, dtype=torch.int32)
    n_lead = 4 * 152 // 2                      # 304 chunks = 608 blocks
    b.counter[1] = 5                           # five lead blocks
    b.counter[0] = 3                           # three main chunks
    assert b._taken_slots() == [(0, 160), (n_lead * 64, (n_lead + 3) * 64)]
    b.counter[1] = 10_000                      # every lead block (and the probes beyond)
    b.counter[0] = 10_000
    assert b._taken_slots() == [(0, n_lead * 64), (n_lead * 64, 1000 * 64)]
    assert b.chunks_taken() == 1000
    b.config = {"chunk": 32}
    b.order = torch.arange(32 * 100, dtype=torch.int32)   # fewer chunks than the lead region
    b.counter[1], b.counter[0] = 100, 1
    assert b._taken_slots() == [(0, 3200), (3200, 3200)]
