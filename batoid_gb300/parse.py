"""Optic descriptions: a YAML-subset reader and the optic builder.

The reference loads telescopes from YAML with PyYAML (batoid/optic.py:60-95)
and builds them in batoid/parse.py:6-236.  PyYAML is not available here, so
``yaml_load`` reads the subset these files use: block mappings and block
sequences by indentation, ``- key: value`` sequence items, flow sequences
``[a, b, ...]`` (possibly spanning lines), scalars (numbers, booleans, null,
plain or quoted strings), comments, anchors ``&name`` and aliases ``*name``.
``parse_optic`` follows the reference's construction rules: coordinate
systems accumulate down the tree (shifts then rotations, in key order), media
default from the parent, ``Clear*`` obscurations are negated ``Obsc*``, and
a Lens's two faces get the lens medium inside.
"""
import glob
import os
import re

import numpy as np

# ---------------------------------------------------------------------------
# YAML subset
# ---------------------------------------------------------------------------


def _strip_comment(line):
    out = []
    quote = None
    for ch in line:
        if quote:
            out.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in "'\"":
            quote = ch
        elif ch == "#":
            break
        out.append(ch)
    return "".join(out).rstrip()


def _logical_lines(text):
    """(indent, content) pairs with comments removed and multi-line flow
    sequences joined."""
    lines = []
    pending = None
    for raw in text.splitlines():
        line = _strip_comment(raw)
        if pending is not None:
            pending[1] += " " + line.strip()
            if pending[1].count("[") <= pending[1].count("]"):
                lines.append(tuple(pending))
                pending = None
            continue
        if not line.strip():
            continue
        indent = len(line) - len(line.lstrip(" "))
        content = line.strip()
        if content.count("[") > content.count("]"):
            pending = [indent, content]
            continue
        lines.append((indent, content))
    if pending is not None:
        raise ValueError("unterminated flow sequence")
    return lines


_NUM = re.compile(r"^[-+]?(\d+\.?\d*([eE][-+]?\d+)?|\.\d+([eE][-+]?\d+)?|\d+[eE][-+]?\d+)$")


class _Loader:
    def __init__(self, text):
        self.lines = _logical_lines(text)
        self.anchors = {}

    def scalar(self, s):
        s = s.strip()
        if s.startswith("*"):
            return self.anchors[s[1:].strip()]
        if s.startswith("&"):
            name, _, rest = s[1:].partition(" ")
            val = self.scalar(rest)
            self.anchors[name] = val
            return val
        if s.startswith("["):
            return self.flow(s)
        if len(s) >= 2 and s[0] == s[-1] and s[0] in "'\"":
            return s[1:-1]
        if s in ("true", "True", "TRUE"):
            return True
        if s in ("false", "False", "FALSE"):
            return False
        if s in ("null", "Null", "~", ""):
            return None
        if _NUM.match(s):
            if re.match(r"^[-+]?\d+$", s):
                return int(s)
            return float(s)
        if s.lower() in (".inf", "+.inf"):
            return float("inf")
        if s.lower() == "-.inf":
            return float("-inf")
        return s

    def flow(self, s):
        s = s.strip()
        assert s[0] == "[" and s[-1] == "]", s
        inner = s[1:-1].strip()
        if not inner:
            return []
        items, depth, cur = [], 0, []
        for ch in inner:
            if ch == "[":
                depth += 1
            elif ch == "]":
                depth -= 1
            if ch == "," and depth == 0:
                items.append("".join(cur))
                cur = []
            else:
                cur.append(ch)
        items.append("".join(cur))
        return [self.scalar(it) for it in items if it.strip() != ""]

    def block(self, i, indent):
        """Parse the block starting at line i (whose indent is `indent`)."""
        if self.lines[i][1].startswith("- ") or self.lines[i][1] == "-":
            return self.sequence(i, indent)
        return self.mapping(i, indent)

    def _value_after_key(self, rest, i, indent):
        """Value of `key: rest` at line i; nested blocks are deeper-indented
        (or a sequence at the same indent)."""
        anchor = None
        if rest.startswith("&") and " " not in rest.strip():
            anchor = rest.strip()[1:]
            rest = ""
        if rest:
            return self.scalar(rest), i + 1
        j = i + 1
        if j < len(self.lines) and (self.lines[j][0] > indent or
                                    (self.lines[j][0] == indent and self.lines[j][1].startswith("-"))):
            val, j = self.block(j, self.lines[j][0])
        else:
            val = None
        if anchor:
            self.anchors[anchor] = val
        return val, j

    def mapping(self, i, indent):
        out = {}
        while i < len(self.lines) and self.lines[i][0] == indent and not self.lines[i][1].startswith("-"):
            content = self.lines[i][1]
            key, sep, rest = content.partition(":")
            if not sep:
                raise ValueError(f"expected 'key: value' at {content!r}")
            out[key.strip()] = None
            val, i = self._value_after_key(rest.strip(), i, indent)
            out[key.strip()] = val
        return out, i

    def sequence(self, i, indent):
        out = []
        while i < len(self.lines) and self.lines[i][0] == indent and (
                self.lines[i][1].startswith("- ") or self.lines[i][1] == "-"):
            rest = self.lines[i][1][1:].strip()
            if not rest:
                j = i + 1
                if j < len(self.lines) and self.lines[j][0] > indent:
                    val, i = self.block(j, self.lines[j][0])
                else:
                    val, i = None, i + 1
                out.append(val)
            elif re.match(r"^[^\[\]'\"]+:(\s|$)", rest):
                # "- key: value" starts a mapping whose keys sit at the column of `key`
                col = indent + (len(self.lines[i][1]) - len(rest))
                self.lines[i] = (col, rest)
                val, i = self.mapping(i, col)
                out.append(val)
            else:
                out.append(self.scalar(rest))
                i += 1
        return out, i


def yaml_load(text):
    ld = _Loader(text)
    if not ld.lines:
        return None
    val, i = ld.block(0, ld.lines[0][0])
    if i != len(ld.lines):
        raise ValueError(f"unparsed content at line {i}: {ld.lines[i]!r}")
    return val


def data_dirs():
    dirs = [os.path.join(os.path.dirname(__file__), "data")]
    extra = os.environ.get("BATOID_DATADIR")
    if extra:
        dirs.extend(extra.split(os.pathsep))
    return dirs


def load_yaml_file(filename):
    """Read a YAML optic file; bare names are searched under the data dirs."""
    if not os.path.exists(filename):
        for d in data_dirs():
            hits = [p for p in glob.glob(os.path.join(d, "**", "*.yaml"), recursive=True)
                    if os.path.basename(p) == filename]
            if hits:
                filename = hits[0]
                break
        else:
            raise FileNotFoundError(filename)
    with open(filename) as f:
        return yaml_load(f.read())


# ---------------------------------------------------------------------------
# optic construction (reference rules: batoid/parse.py)
# ---------------------------------------------------------------------------


def _bt():
    import batoid_gb300
    return batoid_gb300


def parse_obscuration(config):
    bt = _bt()
    config = dict(config)
    typ = config.pop("type")
    simple = {"ObscCircle": bt.ObscCircle, "ObscAnnulus": bt.ObscAnnulus, "ObscRay": bt.ObscRay,
              "ObscRectangle": bt.ObscRectangle, "ObscPolygon": bt.ObscPolygon}
    if typ in simple:
        return simple[typ](**config)
    if typ == "ObscNegation":
        return bt.ObscNegation(parse_obscuration(config["original"]))
    if typ in ("ObscUnion", "ObscIntersection"):
        items = [parse_obscuration(c) for c in config["items"]]
        return getattr(bt, typ)(items)
    if typ.startswith("Clear"):
        config["type"] = typ.replace("Clear", "Obsc")
        return bt.ObscNegation(parse_obscuration(config))
    raise ValueError(f"Unknown obscuration type {typ}")


def parse_surface(config):
    bt = _bt()
    config = dict(config)
    typ = config.pop("type")
    if typ == "Sum":
        return bt.Sum([parse_surface(c) for c in config["items"]])
    cls = {"Plane": bt.Plane, "Tilted": bt.Tilted, "Sphere": bt.Sphere, "Paraboloid": bt.Paraboloid,
           "Quadric": bt.Quadric, "Asphere": bt.Asphere, "Zernike": bt.Zernike, "Bicubic": bt.Bicubic}
    if typ not in cls:
        raise ValueError(f"Unknown surface type {typ}")
    return cls[typ](**config)


def parse_coordSys(config, coordSys=None):
    """Apply x/y/z/shift and rotX/rotY/rotZ in key order, in the local frame."""
    bt = _bt()
    if coordSys is None:
        coordSys = bt.CoordSys()
    for k, v in config.items():
        if k == "x":
            coordSys = coordSys.shiftLocal([v, 0.0, 0.0])
        elif k == "y":
            coordSys = coordSys.shiftLocal([0.0, v, 0.0])
        elif k == "z":
            coordSys = coordSys.shiftLocal([0.0, 0.0, v])
        elif k == "shift":
            coordSys = coordSys.shiftLocal(v)
        elif k == "rotX":
            coordSys = coordSys.rotateLocal(bt.RotX(v))
        elif k == "rotY":
            coordSys = coordSys.rotateLocal(bt.RotY(v))
        elif k == "rotZ":
            coordSys = coordSys.rotateLocal(bt.RotZ(v))
    return coordSys


def parse_medium(config):
    bt = _bt()
    from numbers import Real
    if config is None:
        return None
    if isinstance(config, bt.Medium):
        return config
    if isinstance(config, Real):
        return bt.ConstMedium(config)
    config = dict(config)
    typ = config.pop("type")
    cls = {"ConstMedium": bt.ConstMedium, "TableMedium": bt.TableMedium, "SellmeierMedium": bt.SellmeierMedium,
           "SumitaMedium": bt.SumitaMedium, "Air": bt.Air}
    return cls[typ](**config)


_EXTRA = ("backDist", "sphereRadius", "pupilSize", "pupilObscuration", "R_outer", "R_inner")


def parse_optic(config, coordSys=None, inMedium=None, outMedium=None):
    bt = _bt()
    config = dict(config)
    if coordSys is None:
        coordSys = bt.CoordSys()
    if inMedium is None:
        inMedium = bt.ConstMedium(1.0)
    obscuration = parse_obscuration(config.pop("obscuration")) if "obscuration" in config else None
    name = config.pop("name", "")
    if "coordSys" in config:
        coordSys = parse_coordSys(config.pop("coordSys"), coordSys)
    inMedium = parse_medium(config.pop("inMedium", inMedium))
    outMedium = parse_medium(config.pop("outMedium", outMedium))
    if outMedium is None:
        outMedium = inMedium
    kwargs = {k: config[k] for k in _EXTRA if k in config}
    if "stopSurface" in config:
        kwargs["stopSurface"] = parse_optic(config["stopSurface"])
    typ = config.pop("type")
    leaf = {"Mirror": bt.Mirror, "RefractiveInterface": bt.RefractiveInterface, "Baffle": bt.Baffle,
            "Detector": bt.Detector}
    if typ in leaf:
        return leaf[typ](parse_surface(config.pop("surface")), name=name, coordSys=coordSys,
                         obscuration=obscuration, inMedium=inMedium, outMedium=outMedium, **kwargs)
    if typ == "OPDScreen":
        return bt.OPDScreen(parse_surface(config.pop("surface")), parse_surface(config.pop("screen")), name=name,
                            coordSys=coordSys, obscuration=obscuration, inMedium=inMedium,
                            outMedium=outMedium, **kwargs)
    if typ == "Lens":
        medium = parse_medium(config.pop("medium"))
        ic = config.pop("items")
        items = [parse_optic(ic[0], coordSys=coordSys, inMedium=inMedium, outMedium=medium),
                 parse_optic(ic[1], coordSys=coordSys, inMedium=medium, outMedium=outMedium)]
        return bt.Lens(items, name=name, coordSys=coordSys, inMedium=inMedium, outMedium=outMedium,
                       medium=medium, **kwargs)
    if typ == "CompoundOptic":
        items = [parse_optic(c, coordSys=coordSys, inMedium=inMedium, outMedium=outMedium)
                 for c in config.pop("items")]
        return bt.CompoundOptic(items, inMedium=inMedium, outMedium=outMedium, name=name, coordSys=coordSys,
                                **kwargs)
    if typ == "Interface":
        return bt.Interface(parse_surface(config.pop("surface")), name=name, coordSys=coordSys, **kwargs)
    raise ValueError(f"Unknown optic type: {typ}")
