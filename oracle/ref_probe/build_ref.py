"""Build recipe for oracle/_ref/ (test infrastructure only): compiles, from the reference's
source tree in place, a probe of its k-d tree against its vendored nanoflann, its scalar
MurmurHash3 function (util.cpp:643-688, extracted into a temporary file) and its vendored
rply PLY reader with a probe. Outputs only into oracle/_ref/."""
from __future__ import annotations

import os
import re
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "..", "_ref")
# The reference's source tree: SM_REFERENCE_DIR, else the build container's copy (this
# recipe is the one place that names it; nothing on the GPU machine reads it).
REF = os.environ.get("SM_REFERENCE_DIR") or "/root/reference"


def available() -> bool:
    return os.path.exists(os.path.join(REF, "kdtree", "nanoflann.hpp"))


def build_kd() -> str:
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libkd_ref_probe.so")
    src = os.path.join(HERE, "kd_ref_probe.cpp")
    if os.path.exists(so) and os.path.getmtime(so) >= os.path.getmtime(src):
        return so
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                    "-I", os.path.join(REF, "kdtree"), "-o", so, src], check=True)
    return so


def build_ply() -> str:
    """Compile the reference's vendored rply (third_party/rply/rply/rply.c) with a probe that
    reads PLY files through it the way the reference's readPLY does."""
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libply_ref_probe.so")
    src = os.path.join(HERE, "ply_ref_probe.c")
    rply = os.path.join(REF, "third_party", "rply", "rply")
    if os.path.exists(so) and os.path.getmtime(so) >= os.path.getmtime(src):
        return so
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-I", rply, "-o", so, src,
                    os.path.join(rply, "rply.c")], check=True)
    return so


def build_murmur() -> str:
    """Compile the reference's own scalar murmurhash3 (util.cpp) into a probe library."""
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libmurmur_ref_probe.so")
    text = open(os.path.join(REF, "util.cpp")).read()
    m = re.search(r"uint32_t murmurhash3\(const int \*key, uint32_t len, uint32_t seed\) \{",
                  text)
    if not m:
        raise RuntimeError("reference murmurhash3 not found in util.cpp")
    i, depth = m.end(), 1
    while depth:
        depth += {"{": 1, "}": -1}.get(text[i], 0)
        i += 1
    body = text[m.start():i]
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "murmur_probe.cpp")
        with open(src, "w") as f:
            f.write("#include <cstdint>\n" + body +
                    "\nextern \"C\" uint32_t ref_murmur(const int *k, uint32_t len, "
                    "uint32_t seed) { return murmurhash3(k, len, seed); }\n")
        subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-o", so, src],
                       check=True)
    return so
