"""The ctypes mirrors of the C ABI's structs (tiny-path-tracer_gb300/tpt)
have the C layout: for every struct of include/tpt.h, a C program compiled
here reports sizeof and offsetof of each field, and the Python class must
have the same fields at the same offsets and the same size.  A field added
on one side only would shift every later field and corrupt calls silently."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tpt.h")

PAIRS = {
    "tpt_scene_info": "SceneInfo",
    "tpt_render_params": "RenderParams",
    "tpt_render_stats": "RenderStats",
    "tpt_batch_item": "BatchItem",
    "tpt_guide_params": "GuideParams",
    "tpt_guide_stats": "GuideStats",
    "tpt_nrc_params": "NrcParams",
    "tpt_nrc_stats": "NrcStats",
    "tpt_config": "Config",
}


def c_fields(text, struct):
    end = text.index("} %s;" % struct)
    body = text[text.rindex("typedef struct {", 0, end) + len("typedef struct {"):end]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        rest = re.match(r"^(?:const\s+)?[A-Za-z_0-9]+\s*\**\s*(.*)$", decl).group(1)
        for nm in rest.split(","):
            nm = re.sub(r"\[.*\]", "", nm.strip().lstrip("*")).strip()
            if nm:
                names.append(nm)
    return names


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    text = open(HEADER).read()
    fields = {s: c_fields(text, s) for s in PAIRS}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "tpt.h"', "int main(void) {"]
    for s, names in fields.items():
        offs = " ".join("%zu" for _ in names)
        args = ", ".join("offsetof(%s, %s)" % (s, n) for n in names)
        lines.append('  printf("%s %%zu %s\\n", sizeof(%s), %s);' % (s, offs, s, args))
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        w = line.split()
        layout[w[0]] = (int(w[1]), [int(x) for x in w[2:]], fields[w[0]])
    return layout


@pytest.mark.parametrize("struct", list(PAIRS))
def test_ctypes_mirror_matches_c(built, c_layout, struct):
    import tpt

    size, offsets, names = c_layout[struct]
    py = getattr(tpt, PAIRS[struct])
    py_names = [f[0] for f in py._fields_]
    assert py_names == names, (py_names, names)
    assert [getattr(py, n).offset for n in names] == offsets
    assert C.sizeof(py) == size



def test_learned_parameter_names_are_checked():
    """The learned renderers' keyword parameters go into the C structs by
    name: a known name sets the field, an unknown one (a typo) raises rather
    than being dropped silently."""
    import tpt

    n = tpt.NrcParams()
    tpt._set_fields(n, {"train_steps": 7, "spread_c": 0.5}, "tpt_nrc_params")
    assert n.train_steps == 7 and abs(n.spread_c - 0.5) < 1e-7
    with pytest.raises(TypeError, match="train_step"):
        tpt._set_fields(n, {"train_step": 7}, "tpt_nrc_params")
    g = tpt.GuideParams()
    with pytest.raises(TypeError, match="alpah"):
        tpt._set_fields(g, {"alpah": 0.25}, "tpt_guide_params")
