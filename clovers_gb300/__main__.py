"""Command line of the render path, as clovers-cli has it (clovers-cli/src/main.rs).

    python -m clovers_gb300 [--debug] [-q] render -i scene.json [-o out] [-w 1024] [-h 1024] [-s 64]
                            [-d 64] [-m path-tracing] [--sampler random] [--bvh sah] [-f png exr]
    python -m clovers_gb300 validate scene.json

The options, their short forms and defaults are those of render.rs:16-49 and
lib.rs:17-25 (`-h` is the height, as in the reference; help is `--help`).
`validate` loads a scene file as validate.rs:14-31 does (SAH, 1x1) and reports
success; it needs no GPU.
"""

import argparse
import sys

from . import ClvError, GlobalOptions, RenderOptions, Scene, render


def parser():
    p = argparse.ArgumentParser(prog="clovers", description="clovers path tracing renderer (GB300)")
    p.add_argument("--debug", action="store_true", help="enable some debug logging")
    p.add_argument("-q", "--quiet", action="store_true", help="suppress most of the text output")
    sub = p.add_subparsers(dest="command", required=True)
    r = sub.add_parser("render", add_help=False, help="render a given scene file")
    r.add_argument("--help", action="help", help="show this help message and exit")
    r.add_argument("-i", "--input", required=True, help="input filename / location")
    r.add_argument("-o", "--output", default=None,
                   help="output file path, without extension (default: ./renders/unix_timestamp)")
    r.add_argument("-w", "--width", type=int, default=1024, help="width of the image in pixels")
    r.add_argument("-h", "--height", type=int, default=1024, help="height of the image in pixels")
    r.add_argument("-s", "--samples", type=int, default=64, help="number of samples per pixel")
    r.add_argument("-d", "--max-depth", type=int, default=64, help="maximum evaluated bounce depth for each ray")
    r.add_argument("-m", "--mode", default="path-tracing",
                   choices=["path-tracing", "normal-map", "bvh-test-count", "primitive-test-count"])
    r.add_argument("--sampler", default="random", choices=["random", "blue"])
    r.add_argument("--bvh", default="sah", choices=["sah", "lam"])
    r.add_argument("-f", "--formats", nargs="+", default=["png"], choices=["png", "exr"])
    v = sub.add_parser("validate", help="validate a given scene file")
    v.add_argument("input", help="input filename / location")
    return p


def options(args):
    """The parsed command line as (GlobalOptions, RenderOptions)."""
    g = GlobalOptions(debug=args.debug, quiet=args.quiet)
    if args.command != "render":
        return g, None
    return g, RenderOptions(input=args.input, output=args.output, width=args.width, height=args.height,
                            samples=args.samples, max_depth=args.max_depth, mode=args.mode, sampler=args.sampler,
                            bvh=args.bvh, formats=list(args.formats))


def main(argv=None):
    args = parser().parse_args(argv)
    g, o = options(args)
    try:
        if args.command == "validate":
            if not args.input.endswith(".json"):
                raise ClvError(-1, "Unknown file type")
            Scene.from_json(args.input, 1, 1).close()
            print("✅ Scene file successfully validated!")
        else:
            render(g, o)
    except ClvError as e:
        print("Error: %s" % e, file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
