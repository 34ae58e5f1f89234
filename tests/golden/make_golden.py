"""Extracts golden vectors from the reference crate's own source into JSON fixtures.

Run with the root of a reference checkout as the argument, or in the
SHOCOVOX_REFERENCE environment variable (it is not needed at test time; the
fixtures are committed):

    python tests/golden/make_golden.py <reference checkout>

Outputs
  tests/golden/luts.json      the constant look-up tables of src/spatial/lut.rs
                              (OCTANT_OFFSET_REGION_LUT, BITMAP_MASK_FOR_OCTANT_LUT,
                              BITMAP_INDEX_LUT, OCTANT_STEP_RESULT_LUT,
                              RAY_TO_NODE_OCCUPANCY_BITMASK_LUT), parsed from the
                              Rust literals.
  tests/golden/known_rays.json  the fixed rays of the known-answer tests in
                              src/raytracing/tests.rs, src/spatial/raytracing/tests.rs
                              and src/spatial/math/tests.rs, keyed by test name, with
                              the float literals kept as written (parsed as f32 by
                              the tests).
"""
import json
import os
import re
import sys


def _strip_comments(src):
    return re.sub(r"//[^\n]*", "", src)


def _const_body(src, name):
    m = re.search(r"pub\(crate\) const " + name + r"\s*:[^=]*=\s*", src)
    if not m:
        raise SystemExit("constant %s not found" % name)
    i = m.end()
    depth = 0
    for j in range(i, len(src)):
        c = src[j]
        if c == "[":
            depth += 1
        elif c == "]":
            depth -= 1
            if depth == 0:
                return src[i:j + 1]
    raise SystemExit("unterminated constant %s" % name)


def _ints(body):
    return [int(t, 0) for t in re.findall(r"0x[0-9A-Fa-f]+|\d+", body)]


def extract_luts(ref):
    src = _strip_comments(open(os.path.join(ref, "src/spatial/lut.rs")).read())
    offs = _const_body(src, "OCTANT_OFFSET_REGION_LUT")
    offsets = [[float(v) for v in re.findall(r"[xyz]:\s*([0-9.]+)", blk)]
               for blk in re.findall(r"V3c\s*\{([^}]*)\}", offs)]
    out = {
        "OCTANT_OFFSET_REGION_LUT": offsets,
        "BITMAP_MASK_FOR_OCTANT_LUT": _ints(_const_body(src, "BITMAP_MASK_FOR_OCTANT_LUT")),
        "BITMAP_INDEX_LUT": _ints(_const_body(src, "BITMAP_INDEX_LUT")),
        "OCTANT_STEP_RESULT_LUT": _ints(_const_body(src, "OCTANT_STEP_RESULT_LUT")),
        "RAY_TO_NODE_OCCUPANCY_BITMASK_LUT": _ints(_const_body(src, "RAY_TO_NODE_OCCUPANCY_BITMASK_LUT")),
    }
    assert len(out["OCTANT_OFFSET_REGION_LUT"]) == 8
    assert len(out["BITMAP_MASK_FOR_OCTANT_LUT"]) == 8
    assert len(out["BITMAP_INDEX_LUT"]) == 64
    assert len(out["OCTANT_STEP_RESULT_LUT"]) == 27
    assert len(out["RAY_TO_NODE_OCCUPANCY_BITMASK_LUT"]) == 512
    # keep u64 values exact in JSON: store them as hex strings
    for k in ("BITMAP_MASK_FOR_OCTANT_LUT", "RAY_TO_NODE_OCCUPANCY_BITMASK_LUT"):
        out[k] = ["0x%016x" % v for v in out[k]]
    return out


_RAY_RE = re.compile(
    r"Ray\s*\{\s*origin:\s*V3c\s*\{\s*x:\s*([-0-9.e]+),\s*y:\s*([-0-9.e]+),\s*z:\s*([-0-9.e]+),?\s*\},\s*"
    r"direction:\s*V3c\s*\{\s*x:\s*([-0-9.e]+),\s*y:\s*([-0-9.e]+),\s*z:\s*([-0-9.e]+),?\s*\}",
    re.S)


def extract_rays(ref, relpath):
    src = _strip_comments(open(os.path.join(ref, relpath)).read())
    rays = {}
    parts = re.split(r"\bfn\s+(test_\w+)\s*\(", src)
    for k in range(1, len(parts), 2):
        name, body = parts[k], parts[k + 1]
        found = [list(m) for m in _RAY_RE.findall(body)]
        if found:
            rays[name] = [{"origin": r[:3], "direction": r[3:]} for r in found]
    return rays


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SHOCOVOX_REFERENCE", "")
    if not ref or not os.path.isdir(os.path.join(ref, "src")):
        sys.exit("usage: make_golden.py <reference checkout> (or set SHOCOVOX_REFERENCE)")
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "luts.json"), "w") as f:
        json.dump(extract_luts(ref), f, indent=1)
    rays = {}
    for rel in ("src/raytracing/tests.rs", "src/spatial/raytracing/tests.rs", "src/spatial/math/tests.rs"):
        for name, v in extract_rays(ref, rel).items():
            rays[rel + "::" + name] = v
    with open(os.path.join(here, "known_rays.json"), "w") as f:
        json.dump(rays, f, indent=1, sort_keys=True)
    print("wrote luts.json and known_rays.json (%d tests with literal rays)" % len(rays))


if __name__ == "__main__":
    main()
