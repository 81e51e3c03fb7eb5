"""Potentials to and from gala's YAML form (src/gala/potential/potential/io.py).

``to_dict`` / ``from_dict`` follow gala's dictionary layout (io.py:160-262 and
:76-157): ``class``, ``units`` (physical type -> unit name), ``parameters``
(values, with ``<name>_unit`` entries), and for composites ``type``
(``composite`` or ``custom``) with a ``components`` list whose items carry a
``name``.  ``save`` / ``load`` write and read that dictionary as YAML.

PyYAML is not a dependency of this library, so the YAML here is the subset
these files use: block mappings and sequences, plain and quoted scalars, flow
sequences of numbers (nested, as coefficient arrays are written), and the
``!!python/object/apply:collections.OrderedDict`` form (a ``dictitems``
mapping) that older gala versions wrote for parameter dictionaries.  Values
are converted to this library's fixed galactic units (kpc, Myr, Msun, rad) when
a ``<name>_unit`` entry names another unit of length, mass, time, speed or
angle.
"""
from __future__ import annotations

import math
import os
import re

import numpy as np

__all__ = ["to_dict", "from_dict", "save", "load"]


# ============================================================================
# YAML subset: parsing
# ============================================================================
_INT = re.compile(r"^[-+]?(0|[1-9][0-9_]*)$")
_FLOAT = re.compile(r"^[-+]?(\.[0-9]+|[0-9][0-9_]*(\.[0-9_]*)?)([eE][-+]?[0-9]+)?$")
_ODICT_TAG = "!!python/object/apply:collections.OrderedDict"


def _scalar(text: str):
    """A plain or quoted scalar (YAML 1.1 core types, as PyYAML resolves them)."""
    s = text.strip()
    if s.startswith('"') and s.endswith('"') and len(s) >= 2:
        body = s[1:-1]
        out, i = [], 0
        esc = {"n": "\n", "t": "\t", '"': '"', "\\": "\\", "/": "/", "0": "\0", "r": "\r"}
        while i < len(body):
            ch = body[i]
            if ch == "\\" and i + 1 < len(body):
                nxt = body[i + 1]
                if nxt == "x":
                    out.append(chr(int(body[i + 2:i + 4], 16)))
                    i += 4
                    continue
                if nxt == "u":
                    out.append(chr(int(body[i + 2:i + 6], 16)))
                    i += 6
                    continue
                out.append(esc.get(nxt, nxt))
                i += 2
                continue
            out.append(ch)
            i += 1
        return "".join(out)
    if s.startswith("'") and s.endswith("'") and len(s) >= 2:
        return s[1:-1].replace("''", "'")
    if s in ("", "~", "null", "Null", "NULL"):
        return None
    if s in ("true", "True", "TRUE", "yes", "Yes", "on", "On"):
        return True
    if s in ("false", "False", "FALSE", "no", "No", "off", "Off"):
        return False
    if s in (".inf", ".Inf", ".INF", "+.inf"):
        return math.inf
    if s in ("-.inf", "-.Inf", "-.INF"):
        return -math.inf
    if s in (".nan", ".NaN", ".NAN"):
        return math.nan
    if _INT.match(s):
        return int(s.replace("_", ""))
    if _FLOAT.match(s) and any(c.isdigit() for c in s):
        return float(s.replace("_", ""))
    return s


def _split_flow(body: str):
    """Top-level comma-separated items of a flow sequence's inside."""
    items, depth, cur, quote = [], 0, [], None
    for ch in body:
        if quote:
            cur.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in "\"'":
            quote = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
        elif ch == "," and depth == 0:
            items.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    if "".join(cur).strip():
        items.append("".join(cur))
    return items


def _flow(text: str):
    """A flow sequence or mapping ([...] / {...}), possibly nested."""
    s = text.strip()
    if s.startswith("["):
        return [_flow(item) for item in _split_flow(s[1:-1])]
    if s.startswith("{"):
        out = {}
        for item in _split_flow(s[1:-1]):
            k, _, v = item.partition(":")
            out[_scalar(k)] = _flow(v)
        return out
    return _scalar(s)


def _strip_comment(line: str) -> str:
    """The line without a trailing comment (a '#' at the start or after a space,
    outside quotes)."""
    quote = None
    for i, ch in enumerate(line):
        if quote:
            if ch == quote:
                quote = None
        elif ch in "\"'":
            quote = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            return line[:i].rstrip()
    return line


def _lines(text: str):
    """(indent, content) of each meaningful line; flow collections that span
    lines are joined onto their first line."""
    out = []
    pending = None
    for raw in text.splitlines():
        raw = _strip_comment(raw)
        stripped = raw.strip()
        if pending is not None:
            pending[1] += " " + stripped
            if _balanced(pending[1]):
                out.append(tuple(pending))
                pending = None
            continue
        if not stripped or stripped.startswith("#") or stripped in ("---", "..."):
            continue
        indent = len(raw) - len(raw.lstrip(" "))
        if not _balanced(stripped):
            pending = [indent, stripped]
            continue
        out.append((indent, stripped))
    if pending is not None:
        raise ValueError("unterminated flow collection in YAML text")
    return out


def _balanced(s: str) -> bool:
    depth, quote = 0, None
    for ch in s:
        if quote:
            if ch == quote:
                quote = None
        elif ch in "\"'":
            quote = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
    return depth <= 0


def _split_key(content: str):
    """(key, rest) of a mapping entry, or None when content is not one."""
    depth, quote = 0, None
    for i, ch in enumerate(content):
        if quote:
            if ch == quote:
                quote = None
            continue
        if ch in "\"'":
            quote = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
        elif ch == ":" and depth == 0 and (i + 1 == len(content) or content[i + 1] == " "):
            return _scalar(content[:i]), content[i + 1:].strip()
    return None


class _BlockParser:
    def __init__(self, text):
        self.t = _lines(text)

    def parse(self):
        if not self.t:
            return None
        value, i = self.block(0, self.t[0][0])
        if i != len(self.t):
            raise ValueError(f"unexpected YAML content: {self.t[i][1]!r}")
        return value

    def block(self, i, indent):
        content = self.t[i][1]
        if content == "-" or content.startswith("- "):
            return self.sequence(i, indent)
        if _split_key(content) is None:
            return _flow(content), i + 1
        return self.mapping(i, indent)

    def value(self, rest, i, indent):
        """The value after 'key:' or '- ' whose text is rest; i is the next line."""
        tag = None
        if rest.startswith("!!"):
            tag, _, rest = rest.partition(" ")
            rest = rest.strip()
        if rest:
            v = _flow(rest)
        elif i < len(self.t) and (self.t[i][0] > indent or (
                self.t[i][0] == indent and (self.t[i][1] == "-" or self.t[i][1].startswith("- ")))):
            v, i = self.block(i, self.t[i][0])
        else:
            v = None
        if tag == _ODICT_TAG:
            if not isinstance(v, dict) or "dictitems" not in v:
                raise ValueError("an OrderedDict tag needs a 'dictitems' mapping")
            v = v["dictitems"]
        elif tag == "!!python/tuple":
            v = list(v)
        elif tag is not None:
            raise ValueError(f"unsupported YAML tag {tag}")
        return v, i

    def mapping(self, i, indent):
        out = {}
        while i < len(self.t) and self.t[i][0] == indent:
            content = self.t[i][1]
            if content == "-" or content.startswith("- "):
                break
            kv = _split_key(content)
            if kv is None:
                raise ValueError(f"expected 'key: value' in YAML, got {content!r}")
            key, rest = kv
            out[key], i = self.value(rest, i + 1, indent)
        return out, i

    def sequence(self, i, indent):
        out = []
        while i < len(self.t) and self.t[i][0] == indent:
            content = self.t[i][1]
            if not (content == "-" or content.startswith("- ")):
                break
            rest = content[1:].lstrip()
            if rest and _split_key(rest) is not None and not rest.startswith(("[", "{", "!!")):
                # "- key: value" opens a mapping indented to where 'key' starts
                sub = indent + (len(content) - len(rest))
                self.t[i] = (sub, rest)
                v, i = self.mapping(i, sub)
            else:
                v, i = self.value(rest, i + 1, indent)
            out.append(v)
        return out, i


def yaml_load(text: str):
    """Parse the YAML subset described in the module docstring."""
    return _BlockParser(text).parse()


# ============================================================================
# YAML subset: writing (block style, sorted keys, numbers and lists of numbers
# in flow style, as PyYAML's dump with default_flow_style=None writes them)
# ============================================================================
_PLAIN_OK = re.compile(r"^[A-Za-z_/][A-Za-z0-9_ ./()*+-]*$")


def _float_text(x: float) -> str:
    if math.isnan(x):
        return ".nan"
    if math.isinf(x):
        return ".inf" if x > 0 else "-.inf"
    r = repr(float(x))
    if "e" in r and "." not in r.split("e")[0]:
        mant, ex = r.split("e")
        r = f"{mant}.0e{ex}"  # YAML 1.1 floats need a dot before the exponent
    return r


def _scalar_text(v) -> str:
    if v is None:
        return "null"
    if isinstance(v, (bool, np.bool_)):
        return "true" if v else "false"
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    if isinstance(v, (float, np.floating)):
        return _float_text(float(v))
    s = str(v)
    if s and _PLAIN_OK.match(s) and not s.endswith(" ") and not isinstance(_scalar(s), (bool, type(None))) \
            and isinstance(_scalar(s), str):
        return s
    return '"' + s.replace("\\", "\\\\").replace('"', '\\"').replace("\n", "\\n") + '"'


def _flow_text(v) -> str:
    if isinstance(v, (list, tuple, np.ndarray)):
        return "[" + ", ".join(_flow_text(x) for x in v) + "]"
    return _scalar_text(v)


def _is_flow(v) -> bool:
    if isinstance(v, np.ndarray):
        return True
    return isinstance(v, (list, tuple)) and all(not isinstance(x, dict) for x in v)


def _emit(v, indent: int, out: list):
    pad = " " * indent
    if isinstance(v, dict):
        if not v:
            out[-1] += " {}"
            return
        for k in sorted(v, key=str):
            x = v[k]
            key = _scalar_text(k)
            if isinstance(x, dict) and x:
                out.append(f"{pad}{key}:")
                _emit(x, indent + 2, out)
            elif isinstance(x, (list, tuple)) and not _is_flow(x):
                out.append(f"{pad}{key}:")
                _emit(x, indent, out)
            elif isinstance(x, dict):
                out.append(f"{pad}{key}: {{}}")
            else:
                out.append(f"{pad}{key}: {_flow_text(x)}")
        return
    if isinstance(v, (list, tuple)) and not _is_flow(v):
        for x in v:
            if isinstance(x, dict) and x:
                sub = []
                _emit(x, indent + 2, sub)
                out.append(f"{pad}- " + sub[0].lstrip())
                out.extend(sub[1:])
            else:
                out.append(f"{pad}- {_flow_text(x)}")
        return
    out.append(pad + _flow_text(v))


def yaml_dump(d) -> str:
    """The YAML text of a dictionary of the kinds ``to_dict`` returns."""
    out = []
    _emit(d, 0, out)
    return "\n".join(out) + "\n"


# ============================================================================
# units: the names gala writes (astropy's unit strings) and their value in
# this library's galactic units
# ============================================================================
def _unit_table():
    from .units import KMS_TO_KPC_MYR

    kpc_per_km = 1.0 / 3.0856775814913673e16
    myr_s = 3.15576e13  # Julian-year Myr in seconds
    t = {
        "length": {"kpc": 1.0, "pc": 1e-3, "Mpc": 1e3, "km": kpc_per_km, "m": kpc_per_km * 1e-3,
                   "AU": 4.84813681109536e-9, "au": 4.84813681109536e-9},
        "mass": {"solMass": 1.0, "Msun": 1.0, "M_sun": 1.0, "kg": 1.0 / 1.988409870698051e30},
        "time": {"Myr": 1.0, "Gyr": 1e3, "yr": 1e-6, "kyr": 1e-3, "s": 1.0 / myr_s},
        "speed": {"kpc / Myr": 1.0, "km / s": KMS_TO_KPC_MYR, "pc / Myr": 1e-3, "m / s": KMS_TO_KPC_MYR * 1e-3},
        "angle": {"rad": 1.0, "deg": math.pi / 180.0, "arcsec": math.pi / 648000.0,
                  "mas": math.pi / 648000000.0},
        "angular speed": {"rad / Myr": 1.0, "mas / yr": math.pi / 648000000.0 * 1e6},
        "frequency": {"1 / Myr": 1.0, "1 / Gyr": 1e-3, "1 / yr": 1e6, "rad / Myr": 1.0,
                      "km / (kpc s)": KMS_TO_KPC_MYR},
        "dimensionless": {"": 1.0},
    }
    return t


def _unit_factor(unit: str, physical_type: str | None = None) -> float:
    """Value of one `unit` in galactic units; physical_type, when given, must match."""
    unit = " ".join(str(unit).split())
    for typ, units in _unit_table().items():
        if unit in units and (physical_type is None or typ == physical_type or
                              (physical_type == "frequency" and typ == "angular speed")):
            return units[unit]
    raise ValueError(f"unit {unit!r} is not supported" + (f" for a {physical_type}" if physical_type else ""))


# physical type of each parameter of the potentials this library implements
# (PotentialParameter declarations, src/gala/potential/potential/builtin/core.py)
_PARAM_TYPES = {
    "KeplerPotential": {"m": "mass"},
    "HernquistPotential": {"m": "mass", "c": "length"},
    "PlummerPotential": {"m": "mass", "b": "length"},
    "MiyamotoNagaiPotential": {"m": "mass", "a": "length", "b": "length"},
    "NFWPotential": {"m": "mass", "r_s": "length", "a": "dimensionless", "b": "dimensionless",
                     "c": "dimensionless"},
    "SCFPotential": {"m": "mass", "r_s": "length", "Snlm": "dimensionless", "Tnlm": "dimensionless"},
    "NullPotential": {},
}
_UNIT_NAME = {"mass": "solMass", "length": "kpc", "dimensionless": ""}
_GALACTIC_UNITS = {"length": "kpc", "time": "Myr", "mass": "solMass", "angle": "rad", "speed": "km / s"}


# ============================================================================
# dictionaries (io.py:76-262)
# ============================================================================
def _system_factors(units_block) -> dict:
    """Factor to galactic units for each physical type of a file's unit system."""
    factors = {}
    if not units_block:
        return factors
    table = _unit_table()
    for unit in units_block.values():
        unit = " ".join(str(unit).split())
        for typ, units in table.items():
            if unit in units:
                factors.setdefault(typ, units[unit])
                break
        else:
            raise ValueError(f"unit {unit!r} of the potential's unit system is not supported")
    return factors


def _unpack_params(cls_name, params, factors) -> dict:
    """Parameter values in galactic units (io.py:14-34, with the unit applied)."""
    types = _PARAM_TYPES.get(cls_name, {})
    out = {}
    for key, item in params.items():
        if key.endswith("_unit") and key[:-5] in params:
            continue
        if isinstance(item, str):
            out[key] = item
            continue
        val = np.array(item, dtype=np.float64) if isinstance(item, (list, tuple)) else float(item)
        ptype = types.get(key)
        unit = params.get(key + "_unit")
        if unit not in (None, ""):
            val = val * _unit_factor(unit, None if ptype in (None, "dimensionless") else ptype)
        elif ptype is not None:
            val = val * factors.get(ptype, 1.0)
        out[key] = val
    return out


def _potential_class(name):
    from . import potential as gp

    cls = getattr(gp, name, None)
    if not (isinstance(cls, type) and issubclass(cls, gp.PotentialBase)):
        raise ValueError(f"potential class {name!r} is not available in gala_gb300")
    return cls


def _parse_component(component):
    try:
        class_name = component["class"]
    except KeyError as e:
        raise KeyError("Potential dictionary must contain a key 'class' for specifying the name of the "
                       "Potential class.") from e
    cls = _potential_class(class_name)
    factors = _system_factors(component.get("units"))
    params = _unpack_params(class_name, component.get("parameters") or {}, factors)
    params = {**params, **(component.get("extra_args") or {})}
    return cls(**params)


def from_dict(d, module=None):
    """The potential described by a dictionary (io.py:76-157): a single
    component, a ``composite`` (components added under their names, in order)
    or a ``custom`` composite class built from per-component parameter groups."""
    if d.get("type") == "composite":
        p = _potential_class(d["class"])()
        for i, component in enumerate(d["components"]):
            p[component.get("name", str(i))] = _parse_component(component)
        return p
    if d.get("type") == "custom":
        groups = {}
        for component in d["components"]:
            _parse_component(component)  # validates the component
            try:
                name = component["name"]
            except KeyError as e:
                raise KeyError("For custom potentials, component specification must include the component name "
                               "(e.g., name: 'blah')") from e
            groups[name] = _unpack_params(component["class"], component.get("parameters") or {},
                                          _system_factors(component.get("units")))
        groups = {**groups, **(d.get("extra_args") or {})}
        return _potential_class(d["class"])(**groups)
    return _parse_component(d)


def _to_dict_help(potential) -> dict:
    """One component (io.py:184-198): class, units, parameters with units."""
    name = type(potential).__name__
    d = {"class": name, "units": dict(_GALACTIC_UNITS)}
    types = _PARAM_TYPES.get(name, {})
    if potential.parameters:
        params = {}
        for key, val in potential.parameters.items():
            params[key] = val.tolist() if hasattr(val, "tolist") else float(val)
            params[key + "_unit"] = _UNIT_NAME.get(types.get(key, "dimensionless"), "")
        d["parameters"] = params
    return d


def to_dict(potential) -> dict:
    """Dictionary form of a potential (io.py:201-262).  As in gala, a
    component's origin and rotation are not part of it."""
    from . import potential as gp

    if isinstance(potential, gp.CompositePotential):
        name = type(potential).__name__
        d = {"class": name}
        if isinstance(potential, gp.MilkyWayPotential):
            d["extra_args"] = {"version": potential.version}
        d["components"] = []
        for k, p in potential.items():
            c = _to_dict_help(p)
            c["name"] = k
            d["components"].append(c)
        d["type"] = "composite" if name in ("CompositePotential", "CCompositePotential") else "custom"
        return d
    return _to_dict_help(potential)


def save(potential, f):
    """Write the potential's YAML to a filename or a writable file object (io.py:320-366)."""
    text = yaml_dump(to_dict(potential))
    if hasattr(f, "write"):
        f.write(text)
    else:
        with open(f, "w", encoding="utf-8") as fh:
            fh.write(text)


def load(f, module=None):
    """A potential from a YAML file name, a file object or YAML text (io.py:265-317)."""
    if hasattr(f, "read"):
        text = f.read()
    elif isinstance(f, (str, os.PathLike)) and os.path.exists(os.fspath(f)):
        with open(os.path.abspath(f), encoding="utf-8") as fh:
            text = fh.read()
    elif isinstance(f, str) and ":" in f:
        text = f
    else:
        raise FileNotFoundError(f)
    if isinstance(text, bytes):
        text = text.decode("utf-8")
    return from_dict(yaml_load(text), module=module)
