"""CPU: ReconParams and ImageParams of include/cudasirecon.h have the
reference's exact layout (src/cudaSirecon/cudaSireconImpl.h:104-195).

SR_getReconParams / SR_getImageParams hand out references into the object, so
a caller compiled against the reference's header reads and writes these
structs in place.  The test cuts both struct definitions out of the
reference's header, compiles them in a namespace next to this library's
header, and static_asserts, for every member, the same offset and the same
type, and the same size of both structs (g++, the host compiler of both).
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_HDR = "/root/reference/src/cudaSirecon/cudaSireconImpl.h"


def ref_structs():
    text = open(REF_HDR).read()
    a = text.index("struct ReconParams {")
    b = text.index("struct ImageParams {")
    c = text.index("};", b) + 2
    return text[a:c]


def members(struct_body: str):
    body = re.sub(r"/\*.*?\*/", "", struct_body, flags=re.S)
    body = re.sub(r"//[^\n]*", "", body)
    names = []
    for decl in body.split(";"):
        decl = decl.split("{")[-1].strip()
        if not decl or decl == "}":
            continue
        # type then comma-separated declarators
        m = re.match(r"^((?:unsigned\s+|const\s+)*[\w:<>]+(?:<[^>]*>)?)\s+(.*)$", decl, flags=re.S)
        if not m:
            continue
        for d in m.group(2).split(","):
            n = re.sub(r"[\*\s]|\[.*?\]", "", d)
            if n:
                names.append(n)
    return names


@pytest.mark.skipif(not os.path.exists(REF_HDR), reason="reference sources not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_reconparams_imageparams_layout_matches_reference(tmp_path):
    src = ref_structs()
    i = src.index("struct ImageParams {")
    rp, ipm = members(src[:i]), members(src[i:])
    assert len(rp) == 70 and len(ipm) == 13, (len(rp), len(ipm))
    checks = []
    for s_name, names in (("ReconParams", rp), ("ImageParams", ipm)):
        checks.append(f"static_assert(sizeof(ref::{s_name}) == sizeof(::{s_name}), \"sizeof {s_name}\");")
        for n in names:
            checks.append(f"static_assert(offsetof(ref::{s_name}, {n}) == offsetof(::{s_name}, {n}), "
                          f"\"offset of {s_name}::{n}\");")
            checks.append(f"static_assert(std::is_same_v<decltype(ref::{s_name}::{n}), decltype(::{s_name}::{n})>, "
                          f"\"type of {s_name}::{n}\");")
    tu = tmp_path / "layout.cpp"
    tu.write_text("#include <cstddef>\n#include <string>\n#include <type_traits>\n#include <vector>\n"
                  "namespace ref {\n" + src + "\n}\n#include \"cudasirecon.h\"\n" + "\n".join(checks) + "\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wno-invalid-offsetof", "-I",
                        os.path.join(ROOT, "include"), str(tu)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
