"""Generate tests/golden/fixtures.npz from the reference's own test data.

Reads the 16 batch-mode configurations tests/{lens,source,foreground}/*.ini
of the Lensed source tree and the model images they point at (each is a
noiseless render at the listed delta priors, 100x100 pixels, origin (1, 1),
scale 1).  Stores, per case: the object plugins in list order, the parameter
values in object order and the model image (float32).  The rule used to make
the images is not recorded in the reference; the tests use the default g3k7.

The Sersic sources of these images were rendered with the older linear
b(n) of objects/sersic-old.cl, so the cases map "sersic" to the sersic_old
plugin.

Usage: python tests/golden/make_golden.py [path-to-lensed-source-tree]
"""
import glob
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from lensed_gb300 import fits  # noqa: E402

# parameter names per plugin, in the order of the reference's params blocks
NAMES = {
    "sis": ["x", "y", "r"], "sis_plus_shear": ["x", "y", "r", "g1", "g2"], "nsis": ["x", "y", "r", "rc"],
    "sie": ["x", "y", "r", "q", "pa"], "sie_plus_shear": ["x", "y", "r", "q", "pa", "g1", "g2"],
    "nsie": ["x", "y", "r", "rc", "q", "pa"], "point_mass": ["x", "y", "r"],
    "epl": ["x", "y", "r", "t", "q", "pa"], "epl_plus_shear": ["x", "y", "r", "t", "q", "pa", "g1", "g2"],
    "sersic": ["x", "y", "r", "mag", "n", "q", "pa"], "exponential": ["x", "y", "rs", "mag", "q", "pa"],
    "devauc": ["x", "y", "r", "mag", "q", "pa"], "gauss": ["x", "y", "sigma", "mag", "q", "pa"],
    "sky": ["bg", "dx", "dy"],
}


def main(root):
    out = {}
    cases = []
    for ini in sorted(glob.glob(os.path.join(root, "tests", "*", "*.ini"))):
        text = open(ini).read()
        objs = re.findall(r"^(\w+)\s*=\s*(\w+)\s*$", text.split("[objects]")[1].split("[priors]")[0], re.M)
        pri = dict(re.findall(r"^(\w+\.\w+)\s*=\s*(\S+)\s*$", text.split("[priors]")[1], re.M))
        params = [float(pri[f"{oid}.{pn}"]) for oid, pl in objs for pn in NAMES[pl]]
        image = re.search(r"^image\s*=\s*(\S+)", text, re.M).group(1)
        arr, pcs = fits.read_image(os.path.join(os.path.dirname(ini), image), dtype=np.float64)
        name = os.path.relpath(ini, os.path.join(root, "tests"))[:-4].replace("/", "__")
        plugins = ["sersic_old" if pl == "sersic" else pl for _, pl in objs]
        out[f"{name}__image"] = arr.astype(np.float32)
        out[f"{name}__params"] = np.array(params, np.float64)
        out[f"{name}__plugins"] = np.array(plugins)
        cases.append(name)
    out["cases"] = np.array(cases)
    np.savez_compressed(os.path.join(HERE, "fixtures.npz"), **out)
    print(f"wrote {len(cases)} cases")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LENSED_SOURCE", "/root/reference"))
