"""Orbit / stream IO without h5py or PyYAML: the HDF5 subset (gala_gb300.hdf5)
and the potential YAML form (gala_gb300.potential_io), checked against files
that gala's own tests read (tests/golden/io_reference_files.json, made by
make_golden.py from tests/potential/potential/ of the reference)."""
import base64
import json
import struct
from pathlib import Path

import numpy as np
import pytest

import gala_gb300 as g
from gala_gb300 import hdf5
from gala_gb300 import potential_io as pio
from gala_gb300.mockstream import MockStream

GOLDEN = json.loads((Path(__file__).parent / "golden" / "io_reference_files.json").read_text())


@pytest.fixture
def exp_file(tmp_path):
    p = tmp_path / "exp.hdf5"
    p.write_bytes(base64.b64decode(GOLDEN["hdf5_base64"]["EXP-Hernquist-single-coefs.hdf5"]))
    return p


# ------------------------------------------------------------------ HDF5 reading
def test_reads_a_libhdf5_file(exp_file):
    """An EXP coefficient file: attributes of four types (vlen UTF-8 strings in
    a global heap, int32, float64 scalar and vector), nested groups, a compound
    dataset and a root header continued in a second block."""
    f = hdf5.File(exp_file, "r")
    assert list(f.keys()) == ["count", "snapshots"]
    a = f.attrs
    assert a["geometry"] == "sphere" and a["name"] == "EXP-Hernquist" and a["CoefficientOutputVersion"] == "1.0"
    assert a["config"] == "" and a["forceID"] == ""
    assert int(a["lmax"]) == 4 and int(a["nmax"]) == 10 and float(a["scale"]) == 1.0
    assert a["lmax"].dtype == np.int32
    assert f["count"][()] == 1 and f["count"].dtype == np.uint32
    snap = f["snapshots/00000000"]
    assert float(snap.attrs["Time"]) == 0.0 and np.array_equal(snap.attrs["Center"], np.zeros(3))
    c = snap["coefficients"][()]
    assert c.shape == (15, 10) and c.dtype.names == ("r", "i")   # (lmax+1)(lmax+2)/2 x nmax
    # a Hernquist sphere in its own basis: only the lowest radial l = m = 0 term
    assert c["r"][0, 0] == pytest.approx(2.05) and np.count_nonzero(c["r"]) == 1 and not np.any(c["i"])


def _messages(path):
    """{(object kind, message type): [message bodies]} of every object in a file."""
    rd = hdf5._Reader(Path(path).read_bytes())
    out = {}

    def walk(addr):
        msgs = rd.messages(addr)
        kinds = {t for t, _, _ in msgs}
        kind = "group" if 0x11 in kinds else "dataset"
        for t, flags, body in msgs:
            out.setdefault((kind, t), []).append((flags, body))
        for child in rd.group_links(msgs).values():
            walk(child)

    walk(rd.root_header)
    return out


def test_writer_encodings_are_libhdf5s(exp_file, tmp_path):
    """Write the same kinds of objects the EXP file holds and compare the
    message encodings byte for byte (addresses aside)."""
    fn = tmp_path / "mine.h5"
    with hdf5.File(fn, "w") as f:
        f["count"] = np.uint32(1)
        f.attrs["geometry"] = "sphere"
        f.attrs["lmax"] = np.int32(4)
        f.attrs["scale"] = 1.0
        s = f.create_group("snapshots/00000000")
        s.attrs["Time"] = 0.0
        s.attrs["Center"] = np.zeros(3)
    ref, mine = _messages(exp_file), _messages(fn)
    # datatype, dataspace and fill-value messages of the scalar uint32 dataset
    for t in (0x01, 0x03, 0x05):
        assert mine[("dataset", t)][0] == ref[("dataset", t)][0], hex(t)
    # attribute messages: everything except the 16-byte global-heap IDs
    ref_attrs = {b[8:8 + b[2]].rstrip(b"\0"): b for _, b in ref[("group", 0x0C)]}
    for _, body in mine[("group", 0x0C)]:
        name = body[8:8 + body[2]].rstrip(b"\0")
        r = ref_attrs[name]
        if name == b"geometry":
            assert body[:-16] == r[:-16] and len(body) == len(r)
            assert struct.unpack_from("<I", body, len(body) - 16) == struct.unpack_from("<I", r, len(r) - 16)
        else:
            assert body == r, name
    # symbol-table messages point at a B-tree and a local heap in both
    assert len(mine[("group", 0x11)][0][1]) == len(ref[("group", 0x11)][0][1]) == 16


# ------------------------------------------------------------------ HDF5 writing
def test_hdf5_round_trip_of_every_supported_kind(tmp_path):
    fn = tmp_path / "kinds.h5"
    rng = np.random.default_rng(5)
    data = {"f64": rng.normal(size=(3, 4, 5)), "f32": rng.normal(size=7).astype(np.float32),
            "i64": np.arange(-3, 3, dtype=np.int64), "u8": np.arange(9, dtype=np.uint8).reshape(3, 3),
            "S1": np.array([b"t", b"l", b"t"], dtype="S1"), "scalar": np.float64(2.5), "empty": np.zeros((0, 3))}
    with hdf5.File(fn, "w") as f:
        for k, v in data.items():
            f[k] = v
        f["vstr"] = "utf-8 text é"
        f["vbytes"] = b"ascii bytes"
        f["vlist"] = [b"kpc", b"Myr", b""]
        f["vstr"].attrs["unit"] = ""
        for k in range(40):   # 40 links: five symbol-table nodes under one B-tree node
            f[f"many/k{k:03d}"] = np.int32(k)
        f.create_group("a/b/c").attrs["deep"] = np.arange(3.0)
    r = hdf5.File(fn, "r")
    for k, v in data.items():
        got = r[k][()]
        assert np.array_equal(got, v) and np.asarray(got).dtype == np.asarray(v).dtype, k
    assert r["vstr"][()] == "utf-8 text é" and r["vbytes"][()] == b"ascii bytes"
    assert list(r["vlist"][()]) == [b"kpc", b"Myr", b""] and r["vstr"].attrs["unit"] == ""
    assert list(r["many"].keys()) == [f"k{k:03d}" for k in range(40)]
    assert all(int(r[f"many/k{k:03d}"][()]) == k for k in range(40))
    assert np.array_equal(r["a/b/c"].attrs["deep"], np.arange(3.0)) and "a/b" in r and "a/x" not in r


def test_hdf5_limits_and_errors(tmp_path):
    f = hdf5.File(tmp_path / "big.h5", "w")
    for k in range(257):
        f[f"g/k{k}"] = np.int32(k)
    with pytest.raises(ValueError):
        f.create_group("g")
    with pytest.raises(TypeError):
        f["b"] = np.array([True])
    with pytest.raises(ValueError, match="at most 256"):
        f.close()
    assert not (tmp_path / "big.h5").exists()
    ok = tmp_path / "ok.h5"
    with hdf5.File(ok, "w") as f:
        f["x"] = 1.0
    r = hdf5.File(ok, "r")
    with pytest.raises(ValueError, match="read-only"):
        r["y"] = 2.0
    with pytest.raises(KeyError):
        r["nope"]
    with pytest.raises(FileExistsError):
        hdf5.File(ok, "x")
    (tmp_path / "text.h5").write_bytes(b"not hdf5 at all")
    with pytest.raises(OSError, match="signature"):
        hdf5.File(tmp_path / "text.h5", "r")


# ------------------------------------------------------------------ potential YAML
def test_reads_gala_potential_yaml_files():
    """The assertions of gala's test_io.py (test_read_plummer, test_read_composite,
    test_read_lm10's component values) on the same files."""
    y = GOLDEN["yaml"]
    p = pio.load(y["Plummer.yml"])
    assert isinstance(p, g.PlummerPotential)
    assert np.allclose(p.parameters["m"], 1e11) and np.allclose(p.parameters["b"], 0.26)
    c = pio.load(y["Composite.yml"])
    assert type(c).__name__ == "CompositePotential" and list(c) == ["halo", "disk"]
    assert np.allclose([c["disk"].parameters[k] for k in "mab"], [1e11, 6.5, 0.26])
    lm10 = pio.yaml_load(y["lm10.yml"])          # LM10's logarithmic halo is not implemented here
    disk = lm10["components"][0]
    assert lm10["type"] == "custom" and disk["name"] == "disk"
    assert pio.from_dict(disk).parameters == {"m": 150000.0, "a": 10.0, "b": 0.26}
    cc = pio.yaml_load(y["ccomposite.yml"])      # the OrderedDict-tagged parameter form
    kep = pio.from_dict(cc["components"][0])
    assert isinstance(kep, g.KeplerPotential) and kep.parameters["m"] == 1e11
    for name in ("ccomposite.yml", "lm10.yml", "HarmonicOscillator1D.yml"):
        with pytest.raises(ValueError, match="not available"):
            pio.load(y[name])
    for name, text in y.items():                 # the YAML subset round-trips every file
        assert pio.yaml_load(pio.yaml_dump(pio.yaml_load(text))) == pio.yaml_load(text), name


def test_potential_dict_round_trip_and_units(tmp_path):
    rng = np.random.default_rng(2)
    S = rng.normal(size=(4, 3, 3))
    pots = [g.MilkyWayPotential(), g.NFWPotential(m=5e11, r_s=12.0, c=0.9),
            g.SCFPotential(m=1e12, r_s=20.0, Snlm=S, Tnlm=-S),
            g.CCompositePotential(a=g.KeplerPotential(m=1e10), b=g.PlummerPotential(m=1e9, b=0.3))]
    for pot in pots:
        fn = tmp_path / "p.yml"
        pio.save(pot, fn)
        back = pio.load(fn)
        assert type(back) is type(pot)
        assert pio.to_dict(back) == pio.to_dict(pot)
        assert np.array_equal(back.packed().params, pot.packed().params)
    d = pio.to_dict(pots[0])
    assert d["type"] == "custom" and d["extra_args"] == {"version": "v1"}
    assert d["components"][0]["parameters"]["m_unit"] == "solMass"
    # parameters given in other units, or in a file's unit system, come back in kpc / Msun
    txt = "class: HernquistPotential\nparameters:\n  c: 700.0\n  c_unit: pc\n  m: 1.0e11\nunits:\n  length: kpc\n" \
          "  mass: solMass\n  time: Myr\n"
    assert pio.load(txt).parameters == {"m": 1e11, "c": pytest.approx(0.7)}
    txt = "class: PlummerPotential\nparameters:\n  b: 300.0\n  m: 1.0e9\nunits:\n  length: pc\n  mass: solMass\n" \
          "  time: Myr\n"
    assert pio.load(txt).parameters["b"] == pytest.approx(0.3)
    with pytest.raises(ValueError, match="not supported"):
        pio.load("class: PlummerPotential\nparameters:\n  b: 1.0\n  b_unit: furlong\n  m: 1.0\n")
    with pytest.raises(NotImplementedError):
        pio.from_dict({"class": "MilkyWayPotential", "type": "custom", "components": [],
                       "extra_args": {"version": "v2"}})


# ------------------------------------------------------------------ Orbit / stream files
def test_orbit_and_stream_files_in_galas_layout(tmp_path):
    rng = np.random.default_rng(3)
    w = rng.normal(size=(6, 11, 4))
    H = g.Hamiltonian(g.MilkyWayPotential(), frame=g.ConstantRotatingFrame(Omega=[0.0, 0.0, 0.03]))
    orbit = g.Orbit.from_w(w, t=np.linspace(0.0, 10.0, 11), hamiltonian=H)
    fn = tmp_path / "orbit.h5"
    orbit.to_hdf5(fn)
    f = hdf5.File(fn, "r")                       # orbit.py:236-260 / core.py:572-601 / io.py:28-47
    assert set(f) == {"pos", "vel", "time", "frame", "potential"}
    assert f["pos"].attrs["unit"] == "kpc" and f["vel"].attrs["unit"] == "kpc / Myr"
    assert f["time"].attrs["unit"] == "Myr" and f["pos"].shape == (3, 11, 4)
    assert f["frame"].attrs["module"] == "gala.potential.frame.builtin.frames"
    assert f["frame"].attrs["class"] == "ConstantRotatingFrame"
    assert list(f["frame/units"][()]) == [b"kpc", b"Myr", b"solMass", b"rad", b"km / s"]
    assert f["frame/parameters/Omega"].attrs["unit"] == "1 / Myr"
    assert isinstance(f["potential"][()], bytes)  # gala stores yaml.dump(...).encode()
    back = g.Orbit.from_hdf5(fn)
    assert np.array_equal(back.pos, orbit.pos) and np.array_equal(back.vel, orbit.vel)
    assert np.array_equal(back.t, orbit.t) and np.array_equal(back.frame.Omega, [0.0, 0.0, 0.03])
    assert pio.to_dict(back.potential) == pio.to_dict(H.potential)
    # an orbit file whose potential this library lacks still loads, with a warning
    fn2 = tmp_path / "lm10.h5"
    with hdf5.File(fn2, "w") as f2:
        quantity_pos = np.ones((3, 2))
        f2["pos"] = quantity_pos
        f2["pos"].attrs["unit"] = "pc"
        f2["vel"] = quantity_pos
        f2["vel"].attrs["unit"] = "km / s"
        f2["potential"] = GOLDEN["yaml"]["lm10.yml"].encode()
    with pytest.warns(RuntimeWarning, match="could not be rebuilt"):
        o2 = g.Orbit.from_hdf5(fn2)
    assert o2.potential is None and np.allclose(o2.pos, 1e-3)
    assert np.allclose(o2.vel, g.units.KMS_TO_KPC_MYR)
    # mock stream: release times and tails (mockstream/core.py:106-150)
    ms = MockStream(pos=w[:3, 0], vel=w[3:, 0], frame=g.StaticFrame(), release_time=np.arange(4.0),
                    lead_trail=np.array(list("tltl")))
    ms.to_hdf5(tmp_path / "ms.h5")
    f3 = hdf5.File(tmp_path / "ms.h5", "r")
    assert f3["lead_trail"].dtype == np.dtype("S1") and f3["release_time"].attrs["unit"] == "Myr"
    m2 = MockStream.from_hdf5(tmp_path / "ms.h5")
    assert np.array_equal(m2.pos, ms.pos) and np.array_equal(m2.release_time, ms.release_time)
    assert list(m2.lead_trail) == list("tltl") and isinstance(m2.frame, g.StaticFrame)
    p = g.PhaseSpacePosition(pos=w[:3, 0], vel=w[3:, 0])
    p.to_hdf5(tmp_path / "p.h5")
    assert g.PhaseSpacePosition.from_hdf5(tmp_path / "p.h5").frame is None


def test_yaml_subset_edge_cases():
    text = """# hand-written file
class: HernquistPotential   # trailing comment
parameters:
  m: 5.0e9
  c: 1.
  note: "a # inside \\"quotes\\""
  other: 'it''s'
  tag: x#y
  arr: [[1.0, 2.0],   # rows may wrap
        [3.0, -4.5e-3]]
  empty: {}
  none: []
  flag: true
  nothing: null
list:
- 1
- two
- key: v
  deeper:
    - 3
"""
    d = pio.yaml_load(text)
    assert d["class"] == "HernquistPotential"
    p = d["parameters"]
    assert p["m"] == 5e9 and p["c"] == 1.0 and p["note"] == 'a # inside "quotes"' and p["other"] == "it's"
    assert p["tag"] == "x#y" and p["arr"] == [[1.0, 2.0], [3.0, -4.5e-3]]
    assert p["empty"] == {} and p["none"] == [] and p["flag"] is True and p["nothing"] is None
    assert d["list"] == [1, "two", {"key": "v", "deeper": [3]}]
    assert pio.yaml_load(pio.yaml_dump(d)) == d
    # numbers that must stay numbers, strings that must stay strings
    vals = {"a": 1e-5, "b": 1e20, "c": -0.0, "d": "1.5", "e": "true", "f": "", "g": "km / s", "h": 7}
    back = pio.yaml_load(pio.yaml_dump(vals))
    assert back == vals and isinstance(back["d"], str) and isinstance(back["h"], int)
    assert "1.0e-05" in pio.yaml_dump({"a": 1e-5})   # YAML 1.1 needs the dot before the exponent
    with pytest.raises(ValueError, match="tag"):
        pio.yaml_load("a: !!python/object:foo.Bar {}\n")


def test_hdf5_random_trees_round_trip(tmp_path):
    """Seeded random trees: nested groups, unicode names, every supported type,
    attributes everywhere, strings longer than a 4 KB heap collection, more
    strings than one collection holds, and groups near the 256-link limit."""
    rng = np.random.default_rng(11)
    alphabet = list("abcdefghijklmnopqrstuvwxyz_0123456789") + ["é", "ß", "λ"]

    def name():
        return "".join(rng.choice(alphabet, size=int(rng.integers(1, 24))))

    def value():
        kind = int(rng.integers(0, 7))
        shape = tuple(int(s) for s in rng.integers(0, 5, size=int(rng.integers(0, 4))))
        if kind == 0:
            return rng.normal(size=shape)
        if kind == 1:
            return rng.integers(-2**40, 2**40, size=shape)
        if kind == 2:
            return rng.normal(size=shape).astype(np.float32)
        if kind == 3:
            return "".join(rng.choice(alphabet, size=int(rng.integers(0, 6000))))
        if kind == 4:
            return ("".join(rng.choice(alphabet[:37], size=int(rng.integers(0, 50))))).encode()
        if kind == 5:
            return [name() for _ in range(int(rng.integers(1, 400)))]
        return np.array([name().encode()[:3] for _ in range(int(rng.integers(1, 9)))], dtype="S3")

    expect = {}

    def fill(group, path, depth):
        for _ in range(int(rng.integers(1, 12 if depth else 250))):
            nm = name()
            if nm in group:
                continue
            if depth < 3 and rng.random() < 0.25:
                sub = group.create_group(nm)
                sub.attrs[name()] = rng.normal()
                fill(sub, f"{path}/{nm}", depth + 1)
            else:
                v = value()
                group[nm] = v
                an = name()
                group[nm].attrs[an] = name()
                expect[f"{path}/{nm}"] = (v, an, group[nm].attrs[an])

    fn = tmp_path / "random.h5"
    with hdf5.File(fn, "w") as f:
        fill(f, "", 0)
    r = hdf5.File(fn, "r")
    assert len(expect) > 150
    for path, (v, an, av) in expect.items():
        got = r[path][()]
        if isinstance(v, list):
            assert list(got) == v, path
        elif isinstance(v, (str, bytes)):
            assert got == v, path
        else:
            assert np.array_equal(got, v) and np.asarray(got).dtype == np.asarray(v).dtype, path
        assert r[path].attrs[an] == av


@pytest.mark.parametrize("config", ["plain", "time", "frame", "frame+potential"])
def test_gala_orbit_io_cases(tmpdir, config):
    """gala's test_io (tests/dynamics/test_orbit.py:610-641): the four orbits written
    into an open file and read back by name, with frame and potential equal."""
    x = np.array([[1, 2, 3.0], [1, 2, 3.0]]).T
    v = np.array([[1, 2, 3.0], [1, 2, 3.0]]).T * g.units.KMS_TO_KPC_MYR
    kw = {}
    if config != "plain":
        kw["t"] = [5.0, 99.0]
    if "frame" in config:
        kw["frame"] = g.StaticFrame()
    if "potential" in config:
        kw["potential"] = g.HernquistPotential(m=1e10, c=0.5)
    obj = g.Orbit(pos=x, vel=v, **kw)
    fn = str(tmpdir.join("thing.hdf5"))
    with hdf5.File(fn, "w") as f:
        obj.to_hdf5(f)
    obj2 = g.Orbit.from_hdf5(fn)
    assert np.allclose(obj.xyz, obj2.xyz) and np.allclose(obj.v_xyz, obj2.v_xyz)
    if obj.t is not None:
        assert np.allclose(obj.t, obj2.t)
    else:
        assert obj2.t is None
    assert type(obj.frame) is type(obj2.frame)
    if obj.potential is None:
        assert obj2.potential is None
    else:
        assert pio.to_dict(obj.potential) == pio.to_dict(obj2.potential)
