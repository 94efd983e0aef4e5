"""Generate tests/golden/plugin_params.json from the reference's plugins.

Reads the ``type = ...;`` line and the ``params { ... };`` block of every
objects/<name>.cl of the Lensed source tree (the plugin surface of
kernel/object.cl:1-33) and stores, per plugin, its kind and its parameters
in declaration order as [name, type, lower, upper, default]:

* type: the index in kernel/object.cl's enum (PARAMETER = 0, POSITION_X,
  POSITION_Y, RADIUS, MAGNITUDE, AXIS_RATIO, POS_ANGLE);
* bounds: UNBOUNDED = {0, 0}, POS_BOUND = {0, +FLT_MAX},
  NEG_BOUND = {-FLT_MAX, 0}, or a literal {lo, hi}; omitted = {0, 0};
* default: the literal when given (a negative zero is kept), else 0.

File names with '-' map to plugin names with '_' (sersic-old -> sersic_old).

Usage: python tests/golden/make_plugin_params.py [path-to-lensed-source-tree]
"""
import glob
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FLT_MAX = 3.4028234663852886e38
TYPES = ["PARAMETER", "POSITION_X", "POSITION_Y", "RADIUS", "MAGNITUDE", "AXIS_RATIO", "POS_ANGLE"]
BOUNDS = {"UNBOUNDED": [0.0, 0.0], "POS_BOUND": [0.0, FLT_MAX], "NEG_BOUND": [-FLT_MAX, 0.0]}


def _real(tok: str) -> float:
    tok = tok.strip().rstrip("fF")
    if tok in ("+FLT_MAX", "FLT_MAX"):
        return FLT_MAX
    if tok == "-FLT_MAX":
        return -FLT_MAX
    return float(tok)


def parse_plugin(text: str):
    text = re.sub(r"//[^\n]*", "", text)
    kind = re.search(r"\btype\s*=\s*(LENS|SOURCE|FOREGROUND)\s*;", text).group(1)
    body = re.search(r"\bparams\s*\{(.*?)\}\s*;", text, re.S).group(1)
    pars = []
    # entries: { "name" [, TYPE [, BOUNDS [, default]]] } with BOUNDS a macro or {lo, hi}
    for m in re.finditer(r"\{\s*\"(\w+)\"\s*((?:,\s*(?:\{[^}]*\}|[^,{}]+))*)\s*\}", body):
        name, rest = m.group(1), m.group(2)
        fields = re.findall(r",\s*(\{[^}]*\}|[^,{}]+)", rest)
        fields = [f.strip() for f in fields]
        ptype = TYPES.index(fields[0]) if len(fields) > 0 else 0
        if len(fields) > 1:
            b = fields[1]
            if b.startswith("{"):
                lo, hi = [x for x in b.strip("{}").split(",")]
                bounds = [_real(lo), _real(hi)]
            else:
                bounds = list(BOUNDS[b])
        else:
            bounds = [0.0, 0.0]
        default = _real(fields[2]) if len(fields) > 2 else 0.0
        pars.append([name, ptype, bounds[0], bounds[1], default])
    return kind, pars


def main(root):
    out = {}
    for path in sorted(glob.glob(os.path.join(root, "objects", "*.cl"))):
        name = os.path.splitext(os.path.basename(path))[0].replace("-", "_")
        kind, pars = parse_plugin(open(path).read())
        out[name] = {"kind": kind, "params": pars}
    dest = os.path.join(HERE, "plugin_params.json")
    with open(dest, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    print(f"wrote {len(out)} plugins to {dest}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LENSED_SOURCE", "/root/reference"))
