"""Reader for ``gimic.inp`` files.

Accepts the reference's keyword language (doc/input.rst:1-20; grammar of
src/fgimic/getkw.py:687-729): ``name = value``, ``name = [a, b, ...]``,
sections ``Name { ... }`` and ``Name(arg) { ... }``, ``#`` comments, double
quoted strings and ``|`` line continuation.  Keywords are typed and defaulted
by the schema of src/gimic.in:59-147 and checked as in ``check_grid`` /
``check_top`` (src/gimic.in:161-283).  Errors raise ``InputError`` with the
reference's messages.
"""
import re

_IVAL = re.compile(r"[-]?\d+$")
_DVAL = re.compile(r"-?\d+\.?\d*([dDeE][+-]?\d+)?", re.I)
_LVAL = re.compile(r"(0|1|yes|no|true|false|on|off)$", re.I)
_YES = re.compile(r"(1|yes|true|on)$", re.I)


class InputError(ValueError):
    pass


# (type, default); default None means "no default, must be set to be used"
_TOP = {
    "title": ("STR", ("",)), "debug": ("INT", (0,)), "calc": ("STR", None), "backend": ("STR", ("gimic",)),
    "basis": ("STR", ("mol",)), "density": ("STR", ("",)), "mofile": ("STR", ("",)), "mos": ("INT_ARRAY", (0, 0)),
    "xdens": ("STR", ("XDENS",)), "magnet_axis": ("STR", ("",)), "magnet": ("DBL_ARRAY", (0.0, 0.0, 0.0)),
    "openshell": ("BOOL", (False,)), "dryrun": ("BOOL", (False,)),
}
_SECTIONS = {
    "Advanced": {"screening": ("BOOL", (False,)), "screening_thrs": ("DBL", (1.0e-8,)),
                 "spherical": ("BOOL", (True,)), "GIAO": ("BOOL", (True,)), "diamag": ("BOOL", (True,)),
                 "paramag": ("BOOL", (True,)), "lip_order": ("INT", (3,))},
    "Essential": {"acid": ("BOOL", (False,)), "jmod": ("BOOL", (False,)), "prop": ("BOOL", (False,))},
    "Grid": {"type": ("STR", ("even",)), "file": ("STR", None), "origin": ("DBL_ARRAY", None),
             "ivec": ("DBL_ARRAY", None), "jvec": ("DBL_ARRAY", None), "lengths": ("DBL_ARRAY", None),
             "bond": ("INT_ARRAY", None), "fixpoint": ("INT", None), "coord1": ("DBL_ARRAY", None),
             "coord2": ("DBL_ARRAY", None), "fixcoord": ("DBL_ARRAY", None), "distance": ("DBL", None),
             "rotation": ("DBL_ARRAY", (0.0, 0.0, 0.0)), "rotation_origin": ("DBL_ARRAY", (0.0, 0.0, 0.0)),
             "spacing": ("DBL_ARRAY", None), "height": ("DBL_ARRAY", None), "width": ("DBL_ARRAY", None),
             "radius": ("DBL", (-1.0,)), "gridplot": ("INT", None), "grid_points": ("INT_ARRAY", None),
             "gauss_order": ("INT", (7,))},
    "Gimlet": {"teletype": ("BOOL", (True,)), "printlevel": ("INT", (3,)), "rel_prec": ("DBL", (1.0e-4,)),
               "order": ("INT", (7,)), "max_depth": ("INT", (10,)), "initial_scale": ("INT", (0,)),
               "wavelet": ("STR", ("I",)), "boxes": ("INT_ARRAY", (1, 1, 1)),
               "translation": ("INT_ARRAY", (0, 0, 0)), "origin": ("DBL_ARRAY", (0.0, 0.0, 0.0))},
}
_LENGTHS = {("Grid", k): n for k, n in [("origin", 3), ("ivec", 3), ("jvec", 3), ("lengths", 3), ("bond", 2),
                                        ("coord1", 3), ("coord2", 3), ("fixcoord", 3), ("spacing", 3),
                                        ("height", 2), ("width", 2), ("grid_points", 3)]}


def _convert(name, typ, vals):
    out = []
    for v in vals:
        if typ in ("INT", "INT_ARRAY"):
            if not _IVAL.match(v):
                raise InputError("getkw: Not an integer: %s = %s" % (name, v))
            out.append(int(v))
        elif typ in ("DBL", "DBL_ARRAY"):
            if not _DVAL.match(v):
                raise InputError("getkw: Not a real: %s = %s" % (name, v))
            out.append(float(re.sub("[dD]", "e", v)))
        elif typ in ("BOOL", "BOOL_ARRAY"):
            if not _LVAL.match(v):
                raise InputError("getkw: Not a bool: %s = %s" % (name, v))
            out.append(bool(_YES.match(v)))
        else:
            out.append(v)
    return out


def _tokens(text):
    text = re.sub(r"\|[ \t]*\n", " ", text)  # line continuation
    toks = []
    i, n, line = 0, len(text), 1
    while i < n:
        c = text[i]
        if c == "\n":
            line += 1
            i += 1
        elif c in " \t\r":
            i += 1
        elif c == "#":
            while i < n and text[i] != "\n":
                i += 1
        elif c == '"':
            j = text.find('"', i + 1)
            if j < 0:
                raise InputError("unterminated string on line %d" % line)
            toks.append(("str", text[i + 1:j], line))
            i = j + 1
        elif c in "{}[]()=,":
            toks.append((c, c, line))
            i += 1
        else:
            j = i
            while j < n and text[j] not in " \t\r\n#{}[]()=,\"":
                j += 1
            toks.append(("word", text[i:j], line))
            i = j
    return toks


class Section:
    def __init__(self, name, arg=None):
        self.name = name
        self.arg = arg
        self.keys = {}
        self.sects = {}

    def __repr__(self):
        return "Section(%s(%s), %s, %s)" % (self.name, self.arg, self.keys, list(self.sects))


def parse_text(text):
    toks = _tokens(text)
    pos = 0
    top = Section("top")
    stack = [top]

    def expect(kind):
        nonlocal pos
        if pos >= len(toks) or toks[pos][0] != kind:
            where = toks[pos][2] if pos < len(toks) else "EOF"
            raise InputError("input error near line %s: expected '%s'" % (where, kind))
        pos += 1
        return toks[pos - 1]

    while pos < len(toks):
        kind, val, line = toks[pos]
        if kind == "}":
            if len(stack) == 1:
                raise InputError("unbalanced '}' on line %d" % line)
            stack.pop()
            pos += 1
            continue
        if kind != "word":
            raise InputError("input error on line %d near '%s'" % (line, val))
        name = val
        pos += 1
        nxt = toks[pos][0] if pos < len(toks) else None
        if nxt == "=":
            pos += 1
            if pos < len(toks) and toks[pos][0] == "[":
                pos += 1
                vals = []
                while True:
                    k, v, _ = toks[pos]
                    if k in ("word", "str"):
                        vals.append(v)
                        pos += 1
                    if toks[pos][0] == ",":
                        pos += 1
                        continue
                    expect("]")
                    break
                stack[-1].keys[name] = vals
            else:
                k, v, _ = toks[pos]
                if k not in ("word", "str"):
                    raise InputError("input error on line %d: missing value for %s" % (line, name))
                stack[-1].keys[name] = [v]
                pos += 1
        elif nxt in ("{", "("):
            arg = None
            if nxt == "(":
                pos += 1
                k, v, _ = toks[pos]
                arg = v
                pos += 1
                expect(")")
            expect("{")
            s = Section(name, arg)
            stack[-1].sects[name] = s
            stack.append(s)
        else:
            raise InputError("input error on line %d near '%s'" % (line, name))
    if len(stack) != 1:
        raise InputError("unterminated section '%s'" % stack[-1].name)
    return top


class Input:
    """Typed view of a parsed gimic.inp: ``inp.get('Grid.type')`` returns the
    value (scalar for 1-element keywords, list otherwise), ``inp.is_set(path)``
    tells whether the user gave the keyword (``keyword_is_set`` in the
    Fortran driver)."""

    def __init__(self, raw):
        self._val = {}
        self._set = set()
        self.grid_arg = None
        self.sections_set = set()
        for name, vals in raw.keys.items():
            if name not in _TOP:
                raise InputError("Unknown keyword: %s" % name)
            self._store(name, _TOP[name][0], vals)
        for sname, sect in raw.sects.items():
            if sname not in _SECTIONS:
                raise InputError("Unknown section: %s" % sname)
            self.sections_set.add(sname)
            if sname == "Grid":
                self.grid_arg = sect.arg if sect.arg is not None else "std"
            for name, vals in sect.keys.items():
                schema = _SECTIONS[sname]
                if name not in schema:
                    raise InputError("Unknown keyword: %s.%s" % (sname, name))
                n = _LENGTHS.get((sname, name))
                if n is not None and len(vals) != n:
                    raise InputError("keyword length mismatch %s(%i): %i" % (name, n, len(vals)))
                self._store(sname + "." + name, schema[name][0], vals)
        if self.grid_arg is None:
            self.grid_arg = "std"

    def _store(self, path, typ, vals):
        self._val[path] = _convert(path, typ, vals)
        self._set.add(path)

    def is_set(self, path):
        return path in self._set

    def get(self, path, default=None):
        if path in self._val:
            v = self._val[path]
        else:
            if "." in path:
                sname, name = path.split(".", 1)
                spec = _SECTIONS[sname][name]
            else:
                spec = _TOP[path]
            if spec[1] is None:
                return default
            v = list(spec[1])
        return v[0] if len(v) == 1 else v


def check(inp):
    """check_top and check_grid of src/gimic.in:161-283."""
    calc = inp.get("calc")
    if calc not in ("cdens", "integral", "divj", "edens", "gimlet"):
        raise InputError("Error: unknown option calc = %s" % calc)
    omagn, pmagn = inp.is_set("magnet"), inp.is_set("magnet_axis")
    if omagn and pmagn:
        raise InputError("Error: Both magnet vector and axis set simultaneously!")
    if not omagn and not pmagn:
        raise InputError("Error: Direction of magnetic field must be set!")
    if pmagn and inp.get("magnet_axis") in ("T", "X"):
        inp._val["magnet_axis"] = ["X"]
    arg = inp.grid_arg
    g = lambda k: inp.is_set("Grid." + k)
    err = "Error: Required option '%s' not set for grid(%s)!"
    if "Grid" not in inp.sections_set:
        return inp
    if arg in ("std", "base"):
        for k in ("origin", "ivec", "jvec", "lengths"):
            if not g(k):
                raise InputError(err % (k, arg))
        flag = (1 if g("spacing") else 0) + (2 if g("grid_points") else 0)
        if flag == 0:
            raise InputError("Error: Either spacing or grid_points must be set")
        if flag == 3:
            raise InputError("Error: Both spacing and grid_points set!")
    elif arg == "file":
        if not g("file"):
            raise InputError(err % ("file", arg))
        return inp
    elif arg == "bond":
        if not g("distance"):
            raise InputError(err % ("distance", arg))
        if g("origin"):
            raise InputError("Error: Keyword 'origin' incompatible with 'bond' grids")
        if not (g("fixpoint") or g("fixcoord")):
            raise InputError("Error: Either fixpoint or fixcoord must be specified")
        if not (g("width") and g("height")):
            raise InputError("Error: missing or incomplete specification for width and height")
        if g("bond"):
            if g("coord1") or g("coord2"):
                raise InputError("Error: Both bond and coord(s) have been specified")
        elif g("coord1"):
            if not g("coord2"):
                raise InputError("Error: coord2 not specified")
        elif g("coord2"):
            raise InputError("Error: coord1 not specified")
        else:
            raise InputError("Error: Invalid bond specification")
    else:
        raise InputError("Error: unknown grid type '%s'" % arg)
    if inp.get("Grid.type") == "even":
        if g("gauss_order"):
            raise InputError("Error: 'gauss_order' incompatible with type=even grids")
        if g("spacing") and g("grid_points"):
            raise InputError("Error: both spacing and grid_points cannot be specified")
        if not g("spacing") and not g("grid_points"):
            raise InputError("Error: either spacing or grid_points must be specified")
    return inp


def read(path_or_text, is_text=False):
    text = path_or_text if is_text else open(path_or_text).read()
    return check(Input(parse_text(text)))
