"""The Python mirrors of the C ABI's structs (lensed_gb300/__init__.py) against
include/lensed_gb300.h: a C unit compiled against the header prints the size
of each struct and the offset of each field, which must equal ctypes' (a
field added to the header and not to the mirror, or in another order, shifts
everything after it)."""
import os
import subprocess

import pytest

import lensed_gb300 as lg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "lg_image_desc": lg._ImageDesc,
    "lg_object_desc": lg._ObjectDesc,
    "lg_options": lg._Options,
    "lg_nested_options": lg.NestedOptions,
    "lg_nested_result": lg.NestedResult,
    "lg_flow_options": lg.FlowOptions,
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    d = tmp_path_factory.mktemp("abi")
    src = ['#include <stddef.h>', '#include <stdio.h>', '#include "lensed_gb300.h"', "int main(void)", "{"]
    for cname, py in STRUCTS.items():
        src.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            src.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    src += ["    return 0;", "}"]
    c = d / "layout.c"
    c.write_text("\n".join(src) + "\n")
    exe = str(d / "layout")
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(c), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    layout = {}
    for line in out.splitlines():
        name, field, value = line.split()
        layout[(name, field)] = int(value)
    return layout


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_python_mirror_matches_the_header(c_layout, cname):
    py = STRUCTS[cname]
    assert c_layout[(cname, "size")] == lg.C.sizeof(py), cname
    for fname, _ in py._fields_:
        assert c_layout[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_flow_defaults():
    """lg_flow_defaults: the documented defaults of the learned proposal
    (FP32-weight training steps, the default wait budget)."""
    o = lg.lib().lg_flow_defaults()
    assert (o.layers, o.width, o.hidden, o.epochs, o.batch) == (8, 128, 2, 200, 256)
    assert o.wait_tries == 0 and o.train_tc == 0
    assert o.lr == 1e-3 and o.patience == 4 and o.lag == 800
