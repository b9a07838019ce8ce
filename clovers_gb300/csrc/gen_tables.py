"""Regenerate ``spectral_tables.h`` from the reference's published data tables.

The renderer needs two data sets that must be identical to the reference's,
value for value, so they are extracted rather than re-typed:

* the xy-chromaticity grid of Meng et al. 2015, "Physically Meaningful
  Rendering using Tristimulus Colours" (168 cells, 186 spectra of 81 samples,
  the four 3x2 colour-space matrices and ``equal_energy_reflectance``), as
  carried by ``clovers/src/spectrum/spectra_xyz_5nm_380_780_097.rs``;
* the CIE illuminant SPDs (D50, D65, LED B1..V2, FL1..FL3.15), as carried by
  ``clovers/src/illuminants/*.csv`` and turned into per-nanometre maps by
  ``clovers/build.rs:12-111``.

Doubles are written with ``repr`` (round-trip exact).  Illuminant values are
written as their decimal text with an ``f`` suffix so that the C compiler does
the single decimal->binary32 rounding, exactly like Rust's f32 literal parse in
the reference's generated ``phf`` maps.

Usage: ``python gen_tables.py <clovers reference root>``; the output is
committed, so this only runs when the data changes.
"""

import os
import re
import sys

LAMBDA_MIN, LAMBDA_MAX = 380, 780  # clovers/src/wavelength.rs:14-16


def _nums(text):
    return [t.strip() for t in text.split(",") if t.strip()]


def grid_tables(src):
    s = open(src).read()

    def scalar(name):
        m = re.search(r"const\s+%s\s*:\s*\w+\s*=\s*([-0-9.eE+]+)\s*;" % name, s)
        return float(m.group(1))

    def mat(name):
        m = re.search(r"const\s+%s\s*:\s*\[f64;\s*6\]\s*=\s*\[([^\]]*)\]" % name, s)
        return [float(x) for x in _nums(m.group(1))]

    cells = re.findall(
        r"spectrum_grid_cell_t\s*\{\s*inside:\s*(\d+),\s*num_points:\s*(\d+),\s*idx:\s*\[([^\]]*)\]", s)
    pts = re.findall(
        r"spectrum_data_point_t\s*\{\s*xystar:\s*\[([^\]]*)\],\s*uv:\s*\[([^\]]*)\],\s*spectrum:\s*\[([^\]]*)\]", s)
    assert len(cells) == 168 and len(pts) == 186
    return {
        "eer": scalar("equal_energy_reflectance"),
        "xy_to_uv": mat("spectrum_mat_xy_to_uv"),
        "cells": [(int(a), int(b), [int(x) for x in _nums(c)]) for a, b, c in cells],
        "points": [([float(x) for x in _nums(u)], [float(x) for x in _nums(sp)]) for _, u, sp in pts],
    }


def csv_columns(path, ncols):
    cols = [dict() for _ in range(ncols)]
    for line in open(path):
        line = line.strip()
        if not line:
            continue
        parts = line.split(",")
        lam = int(parts[0])
        for i in range(ncols):
            cols[i][lam] = parts[1 + i]
    return cols


ILLUMINANTS = (
    [("D50", "CIE_std_illum_D50.csv", 0), ("D65", "CIE_std_illum_D65.csv", 0)]
    + [(n, "CIE_illum_LEDs_1nm.csv", i) for i, n in enumerate(
        ["LED_B1", "LED_B2", "LED_B3", "LED_B4", "LED_B5", "LED_BH1", "LED_RGB1", "LED_V1", "LED_V2"])]
    + [(n, "CIE_illum_FLs_1nm.csv", i) for i, n in enumerate(
        ["FL%d" % k for k in range(1, 13)] + ["FL3_%d" % k for k in range(1, 16)])]
)


def main(ref_root, out_path):
    g = grid_tables(os.path.join(ref_root, "clovers/src/spectrum/spectra_xyz_5nm_380_780_097.rs"))
    ill_dir = os.path.join(ref_root, "clovers/src/illuminants")
    csv_cache = {}
    out = []
    w = out.append
    w("// Generated by gen_tables.py from the reference's spectral data; do not edit.")
    w("// Meng et al. 2015 xy grid (clovers/src/spectrum/spectra_xyz_5nm_380_780_097.rs)")
    w("// and CIE illuminant SPDs (clovers/src/illuminants/*.csv via clovers/build.rs).")
    w("#pragma once")
    w("namespace clv_tables {")
    w("static const double kEqualEnergyReflectance = %r;" % g["eer"])
    w("static const double kXyToUv[6] = {%s};" % ", ".join(repr(x) for x in g["xy_to_uv"]))
    w("struct GridCell { int inside; int num_points; int idx[6]; };")
    w("static const GridCell kGrid[168] = {")
    for inside, num, idx in g["cells"]:
        w("  {%d, %d, {%s}}," % (inside, num, ", ".join(str(i) for i in idx)))
    w("};")
    w("struct GridPoint { double uv[2]; double spectrum[81]; };")
    w("static const GridPoint kPoints[186] = {")
    for uv, sp in g["points"]:
        w("  {{%s}, {%s}}," % (", ".join(repr(x) for x in uv), ", ".join(repr(x) for x in sp)))
    w("};")
    w("static const int kNumIlluminants = %d;" % len(ILLUMINANTS))
    w("static const char* const kIlluminantNames[%d] = {%s};" % (
        len(ILLUMINANTS), ", ".join('"%s"' % n for n, _, _ in ILLUMINANTS)))
    w("// Power at each integer wavelength 380..779 nm; 0 where the CSV has no entry.")
    w("static const float kIlluminants[%d][%d] = {" % (len(ILLUMINANTS), LAMBDA_MAX - LAMBDA_MIN))
    for name, fname, col in ILLUMINANTS:
        if fname not in csv_cache:
            ncols = len(open(os.path.join(ill_dir, fname)).readline().strip().split(",")) - 1
            csv_cache[fname] = csv_columns(os.path.join(ill_dir, fname), ncols)
        colmap = csv_cache[fname][col]
        vals = []
        for lam in range(LAMBDA_MIN, LAMBDA_MAX):
            v = colmap.get(lam)
            vals.append("0.0f" if v is None else (v if ("." in v or "e" in v or "E" in v) else v + ".0") + "f")
        w("  /* %s */ {%s}," % (name, ", ".join(vals)))
    w("};")
    w("}  // namespace clv_tables")
    with open(out_path, "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else "../reference"
    main(ref, os.path.join(os.path.dirname(os.path.abspath(__file__)), "spectral_tables.h"))
