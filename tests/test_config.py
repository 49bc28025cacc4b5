"""The formats either side of the render loop of main.cpp: config.ini
(main.cpp:29-56 through the vendored inipp), the scene camera it rebuilds
(main.cpp:86-90) and the side-by-side PPM strip (main.cpp:222-243).  Host
code only: no GPU."""
import numpy as np
import pytest

import tpt
from tpt import scenes

DEFAULTS = dict(width=400, height=200, sample=10, recur_depth=50, fov=90.0, allow_bonus_pic=0, bonus_pic=10,
                aperture=pytest.approx(0.2), start_time=0.0, end_time=1.0)

SHIPPED = """[DEFAULT]
width = 400
height = 400
sample = 50
recur_depth = 15
fov = 90.0
allow_bonus_pic = 0
bonus_pic = 10
[BLUR]
aperture = 0.1
[CAM_MOTION]
start_time = 0.0
end_time = 0.0
"""


def test_defaults_are_main_cpp(built):
    assert tpt.config() == DEFAULTS


def test_shipped_config_ini(built):
    c = tpt.config(SHIPPED)
    assert (c["width"], c["height"], c["sample"], c["recur_depth"]) == (400, 400, 50, 15)
    assert c["aperture"] == pytest.approx(0.1) and c["end_time"] == 0.0 and c["fov"] == 90.0


def test_inipp_grammar(built):
    text = """
width = 7
; a comment
[DEFAULT]
  width   =   640
width = 10
height = 12.5
sample = 33 junk
recur_depth = 0x10
fov=45
[BLUR
aperture = 0.5
[BLUR]
   aperture=0.25
[CAM_MOTION]
start_time = -1e-1
end_time
= 3
"""
    c = tpt.config(text)
    assert c["width"] == 640          # keys before a section belong to section ""; first definition wins
    assert c["height"] == 200         # "12.5" does not convert to int: the default stands
    assert c["sample"] == 10          # trailing junk: unchanged
    assert c["recur_depth"] == 50     # "0x10": '0' then junk
    assert c["fov"] == 45.0
    assert c["aperture"] == pytest.approx(0.25)   # "[BLUR" is not a section header
    assert c["start_time"] == pytest.approx(-0.1)
    assert c["end_time"] == 1.0


def test_missing_file_keeps_defaults(built, tmp_path):
    assert tpt.config(path=str(tmp_path / "absent.ini")) == DEFAULTS
    f = tmp_path / "config.ini"
    f.write_text(SHIPPED)
    assert tpt.config(path=str(f))["recur_depth"] == 15


def test_scene_camera_follows_config(built):
    sc = tpt.Scene(scenes.cornell().text())
    cam = sc.camera()
    assert cam["lookfrom"] == [278, 278, -800] and cam["vfov"] == 40
    cfg = tpt.config(SHIPPED)
    sc.apply_config(cfg)
    c2 = sc.camera()
    assert c2["lookfrom"] == cam["lookfrom"] and c2["focus"] == cam["focus"]
    assert c2["vfov"] == 90.0 and c2["aspect"] == 1.0 and c2["aperture"] == pytest.approx(0.1)
    assert (c2["time0"], c2["time1"]) == (0.0, 0.0)


def test_ppm_strip(built, tmp_path):
    rng = np.random.default_rng(1)
    a = rng.integers(0, 256, (3, 4, 3), dtype=np.uint8)
    b = rng.integers(0, 256, (3, 4, 3), dtype=np.uint8)
    p = tmp_path / "strip.ppm"
    tpt.write_ppm_strip(str(p), [a, b])
    tok = p.read_text().split()
    assert tok[:4] == ["P3", "8", "3", "255"]
    vals = np.array(tok[4:], dtype=np.int64).reshape(3, 8, 3)
    np.testing.assert_array_equal(vals, np.concatenate([a, b], axis=1))


KEYS = ["width", "height", "sample", "recur_depth", "fov", "allow_bonus_pic", "bonus_pic", "aperture",
        "start_time", "end_time"]


def _fuzz_ini(rng) -> str:
    """Random config.ini-like text: the real keys, sections (good and
    broken), comments, blanks, duplicates, values that do and do not convert."""
    secs = ["[DEFAULT]", "[BLUR]", "[CAM_MOTION]", "[BLUR", "[]", "[ DEFAULT ]"]
    vals = ["640", " 7 ", "-3", "12.5", "1e2", "0x10", "33 junk", "", "true", "+5", "0.125", "-1e-1", "nan", "4  "]
    lines = []
    for _ in range(rng.integers(3, 25)):
        r = rng.random()
        if r < 0.2:
            lines.append(secs[rng.integers(len(secs))])
        elif r < 0.3:
            lines.append("; " + KEYS[rng.integers(len(KEYS))] + " = 1")
        elif r < 0.35:
            lines.append("= 5")
        else:
            k = KEYS[rng.integers(len(KEYS))]
            pad = " " * int(rng.integers(0, 3))
            lines.append(f"{pad}{k}{pad}={pad}{vals[rng.integers(len(vals))]}")
    return "\n".join(lines) + "\n"


def test_config_matches_reference_parser(built):
    """Against the reference's own inipp and main.cpp extraction (compiled
    from the reference checkout into oracle/_ref when it is present)."""
    import pyoracle

    if not pyoracle.ref_available():
        pytest.skip("reference harness not built (no reference checkout)")
    rng = np.random.default_rng(7)
    for case in [SHIPPED, ""] + [_fuzz_ini(rng) for _ in range(300)]:
        ours = tpt.config(case)
        ref = pyoracle.ref_config_parse(case)
        for k, r in zip(KEYS, ref):
            assert ours[k] == pytest.approx(r, nan_ok=True), (k, case)


def test_read_ppm_p3_p6_and_errors(built, tmp_path):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, (5, 7, 3), dtype=np.uint8)
    p3 = tmp_path / "a.ppm"
    tpt.write_ppm(str(p3), img)
    np.testing.assert_array_equal(tpt.read_ppm(str(p3)), img)
    p6 = tmp_path / "b.ppm"
    p6.write_bytes(b"P6\n# a comment\n7 5\n255\n" + img.tobytes())
    np.testing.assert_array_equal(tpt.read_ppm(str(p6)), img)
    p15 = tmp_path / "c.ppm"  # maxval 15: rescaled to 0..255
    p15.write_text("P3 2 1 15\n0 7 15 15 0 1\n")
    np.testing.assert_array_equal(tpt.read_ppm(str(p15)), [[[0, 119, 255], [255, 0, 17]]])
    bad = tmp_path / "bad.ppm"
    bad.write_text("P3 2 2 255\n1 2 3\n")   # truncated
    with pytest.raises(tpt.TptError):
        tpt.read_ppm(str(bad))
    bad.write_text("P5 2 2 255\n")           # greyscale: not an RGB image
    with pytest.raises(tpt.TptError):
        tpt.read_ppm(str(bad))
