"""Output encoders for the film (clovers-cli/src/write.rs).

* PNG: 8-bit sRGB with the reference's two tEXt chunks (write.rs:54-74).
* EXR: the raw XYZ(E) film as three float channels named R, G, B with the
  XYZ chromaticities red (1,0), green (0,1), blue (0,0), white (1/3,1/3)
  (write.rs:97-125).  Written uncompressed, one scanline per block.
"""

import os
import struct
import zlib

import numpy as np

MODE_NAMES = {"path-tracing": "PathTracing", "normal-map": "NormalMap", "bvh-test-count": "BvhTestCount",
              "primitive-test-count": "PrimitiveTestCount"}


def _chunk(tag, data):
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def png_bytes(rgb, width, height, texts=()):
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8).reshape(height, width, 3)
    raw = np.zeros((height, 1 + 3 * width), np.uint8)
    raw[:, 1:] = rgb.reshape(height, 3 * width)
    out = [b"\x89PNG\r\n\x1a\n", _chunk(b"IHDR", struct.pack(">IIBBBBB", width, height, 8, 2, 0, 0, 0))]
    for key, value in texts:
        out.append(_chunk(b"tEXt", key.encode("latin-1") + b"\0" + value.encode("latin-1", "replace")))
    out.append(_chunk(b"IDAT", zlib.compress(raw.tobytes(), 6)))
    out.append(_chunk(b"IEND", b""))
    return b"".join(out)


def format_duration(seconds):
    """The render duration as the reference prints it (render.rs:150-151 formats
    it with the humantime crate, 2.x, which is not vendored): the non-zero
    components among days, hours, minutes, seconds, milliseconds, microseconds
    and nanoseconds, largest first, separated by spaces, with the suffixes
    "day"/"days", "h", "m", "s", "ms", "us", "ns"; "0s" for no time at all.
    Longer units (months, years) do not occur for a render."""
    ns = max(0, int(round(float(seconds) * 1e9)))
    if ns == 0:
        return "0s"
    secs, frac = divmod(ns, 1_000_000_000)
    days, rem = divmod(secs, 86400)
    parts = []
    if days:
        parts.append("%d%s" % (days, "day" if days == 1 else "days"))
    h, rem = divmod(rem, 3600)
    m, s = divmod(rem, 60)
    ms, rest = divmod(frac, 1_000_000)
    us, n = divmod(rest, 1000)
    for value, unit in ((h, "h"), (m, "m"), (s, "s"), (ms, "ms"), (us, "us"), (n, "ns")):
        if value:
            parts.append("%d%s" % (value, unit))
    return " ".join(parts)


def write_png(path, rgb, width, height, render_options=None, duration_s=None):
    texts = []
    if render_options is not None:
        mode = MODE_NAMES.get(render_options.mode, render_options.mode)
        common = ("Rendered with the clovers path tracing engine. Scene file %s rendered using the %s rendering "
                  "mode at %dx%d resolution" % (render_options.input, mode, width, height))
        details = (", %d samples per pixel, %d max ray bounce depth." % (render_options.samples,
                                                                         render_options.max_depth)
                   if render_options.mode == "path-tracing" else ".")
        stats = "Rendering finished in %s, using %d threads." % (format_duration(duration_s or 0.0),
                                                                  os.cpu_count() or 1)
        texts = [("Comment", common + details + " " + stats), ("Software", "clovers")]
    with open(path, "wb") as f:
        f.write(png_bytes(rgb, width, height, texts))


def _attr(name, typ, payload):
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(payload)) + payload


def exr_bytes(xyz, width, height):
    px = np.ascontiguousarray(xyz, dtype=np.float32).reshape(height, width, 3)
    chl = b""
    for ch in ("B", "G", "R"):  # channels are stored in alphabetical order
        chl += ch.encode() + b"\0" + struct.pack("<iB3xii", 2, 0, 1, 1)
    chl += b"\0"
    header = b"".join([
        _attr("channels", "chlist", chl),
        _attr("compression", "compression", b"\0"),
        _attr("dataWindow", "box2i", struct.pack("<iiii", 0, 0, width - 1, height - 1)),
        _attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, width - 1, height - 1)),
        _attr("lineOrder", "lineOrder", b"\0"),
        _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)),
        _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0)),
        _attr("screenWindowWidth", "float", struct.pack("<f", 1.0)),
        _attr("chromaticities", "chromaticities", struct.pack("<8f", 1.0, 0.0, 0.0, 1.0, 0.0, 0.0,
                                                              1.0 / 3.0, 1.0 / 3.0)),
        _attr("software", "string", b"clovers"),
    ]) + b"\0"
    start = 8 + len(header) + 8 * height
    line_bytes = 3 * 4 * width
    offsets = struct.pack("<%dQ" % height, *[start + y * (8 + line_bytes) for y in range(height)])
    lines = []
    for y in range(height):
        row = px[y]
        data = np.concatenate([row[:, 2], row[:, 1], row[:, 0]]).astype("<f4").tobytes()
        lines.append(struct.pack("<ii", y, len(data)) + data)
    return b"\x76\x2f\x31\x01" + struct.pack("<I", 2) + header + offsets + b"".join(lines)


def write_exr(path, xyz, width, height):
    with open(path, "wb") as f:
        f.write(exr_bytes(xyz, width, height))
