"""The command line (python -m clovers_gb300) against clovers-cli's
(main.rs, render.rs:16-49, lib.rs:17-25, validate.rs:14-31): the same
subcommands, options, short forms and defaults; `validate` loads a scene
without a GPU."""

import json
import os
import subprocess
import sys

import pytest

from clovers_gb300 import __main__ as cli
from clovers_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_render_defaults():
    g, o = cli.options(cli.parser().parse_args(["render", "-i", "scene.json"]))
    assert (g.debug, g.quiet) == (False, False)
    assert (o.input, o.output, o.width, o.height, o.samples, o.max_depth) == ("scene.json", None, 1024, 1024, 64, 64)
    assert (o.mode, o.sampler, o.bvh, o.formats) == ("path-tracing", "random", "sah", ["png"])


def test_render_short_options():
    args = ["--debug", "-q", "render", "-i", "a.json", "-o", "out/x", "-w", "32", "-h", "16", "-s", "4", "-d", "8",
            "-m", "normal-map", "--sampler", "random", "--bvh", "lam", "-f", "png", "exr"]
    g, o = cli.options(cli.parser().parse_args(args))
    assert (g.debug, g.quiet) == (True, True)
    assert (o.output, o.width, o.height, o.samples, o.max_depth) == ("out/x", 32, 16, 4, 8)
    assert (o.mode, o.bvh, o.formats) == ("normal-map", "lam", ["png", "exr"])


def test_render_rejects_unknown_values():
    for bad in (["render", "-i", "a.json", "-m", "ambient-occlusion"], ["render", "-i", "a.json", "-f", "jpg"],
                ["render"]):
        with pytest.raises(SystemExit):
            cli.parser().parse_args(bad)


def test_validate(tmp_path, capsys):
    good = scenes.write_scene(scenes.enclosed_box(), str(tmp_path / "box.json"))
    assert cli.main(["validate", good]) == 0
    assert "successfully validated" in capsys.readouterr().out
    sc = scenes.enclosed_box()
    for o in sc["objects"]:
        o.pop("priority", None)
    bad = str(tmp_path / "noprio.json")
    with open(bad, "w") as f:
        json.dump(sc, f)
    assert cli.main(["validate", bad]) == 1
    assert cli.main(["validate", str(tmp_path / "scene.txt")]) == 1


def test_module_entry_point(tmp_path):
    good = scenes.write_scene(scenes.enclosed_box(), str(tmp_path / "box.json"))
    p = subprocess.run([sys.executable, "-m", "clovers_gb300", "validate", good], cwd=ROOT,
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0 and "successfully validated" in p.stdout


def test_render_banner_and_quiet(capsys):
    """render.rs:112-125: the banner unless quiet (checked before any GPU work: the
    scene file type is refused right after it)."""
    assert cli.main(["render", "-i", "scene.txt", "-w", "32", "-h", "16", "-s", "4", "-d", "8"]) == 1
    out = capsys.readouterr().out
    assert out.splitlines()[:6] == ["clovers \U0001F340 path tracing renderer", "", "32x16 resolution",
                                    "4 samples per pixel", "using the random sampler", "8 max bounce depth"]
    assert cli.main(["render", "-i", "scene.txt", "-m", "normal-map"]) == 1
    assert "rendering a normalmap" in capsys.readouterr().out
    assert cli.main(["-q", "render", "-i", "scene.txt"]) == 1
    assert capsys.readouterr().out == ""


def test_blue_sampler_is_refused_clearly(capsys):
    """--sampler blue: the reference's spp check (render.rs:127-129), then a clear
    refusal (the blue-noise tables are not part of this build)."""
    assert cli.main(["-q", "render", "-i", "a.json", "--sampler", "blue", "-s", "3"]) == 1
    assert "only supports the following sample-per-pixel counts" in capsys.readouterr().err
    assert cli.main(["-q", "render", "-i", "a.json", "--sampler", "blue", "-s", "4"]) == 1
    assert "blue-noise sampler is not available" in capsys.readouterr().err
