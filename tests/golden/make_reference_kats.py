"""Extract the known-answer values of the reference's unit tests into
tests/golden/reference_kats.json.

Reads the reference's Rust test modules as text (the reference cannot be
built here: no Rust toolchain), finds each assert by pattern and records the
literal values with their file:line.  Run from the repository root with the
path of a reference checkout, as an argument or in PPM_REFERENCE:

    python tests/golden/make_reference_kats.py REF
"""
import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PPM_REFERENCE", "")
if __name__ == "__main__" and not os.path.isdir(os.path.join(REF, "src")):
    sys.exit("usage: make_reference_kats.py REF (a checkout of the reference; or set PPM_REFERENCE)")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")
NUM = r"(-?[0-9]+(?:\.[0-9]+)?(?:e-?[0-9]+)?)"


def grep(rel, pattern, n_groups):
    path = os.path.join(REF, rel)
    with open(path) as f:
        lines = f.read().split("\n")
    out = []
    for i, line in enumerate(lines, 1):
        m = re.search(pattern, line)
        if m:
            vals = [m.group(k + 1) for k in range(n_groups)]
            out.append({"where": f"{rel}:{i}", "values": vals, "text": line.strip()})
    if not out:
        raise SystemExit(f"pattern not found in {rel}: {pattern}")
    return out


def main():
    kats = {}
    # tracer.rs test_filter
    f = grep("src/tracer.rs", r"assert_eq!\((wt[1-4]), " + NUM + r"\);", 2)
    kats["filters"] = [{"where": e["where"], "name": e["values"][0], "value": float(e["values"][1])} for e in f]
    r = grep("src/tracer.rs", r"let r = " + NUM + r" \* " + NUM + ";", 2)
    kats["filters_r"] = {"where": r[0]["where"], "value": float(r[0]["values"][0]) * float(r[0]["values"][1])}
    corr = grep("src/tracer.rs", r"const CORR: Flt\s+= " + NUM + r"; //" + NUM + ";", 2)
    kats["gauss_corr"] = {"where": corr[0]["where"], "code": float(corr[0]["values"][0]),
                          "comment": float(corr[0]["values"][1])}
    # algebra.rs normalize
    n = grep("src/ray/algebra.rs",
             r"assert_eq!\(v3\.normalize\(\), Some\(Vector3::new\(" + NUM + ", " + NUM + ", " + NUM + r"\)\)\);", 3)
    kats["normalize"] = {"where": n[0]["where"], "input": [1.0, -2.0, 3.0], "value": [float(v) for v in n[0]["values"]]}
    # geometry.rs
    rd = grep("src/ray/geometry.rs", r"Vector3::new\(" + NUM + ", " + NUM + ", " + NUM + r"\)\)\);", 3)
    kats["ray_dir"] = {"where": rd[0]["where"], "input": [1.0, 1.0, 1.0], "value": [float(v) for v in rd[0]["values"]]}
    tg = grep("src/ray/geometry.rs", r"r\.target\(" + NUM + r"\), Vector3::new\(" + NUM + ", " + NUM + ", " + NUM, 4)
    kats["target"] = {"where": tg[0]["where"], "ray": [1.0, 1.0, 1.0, -1.0, -1.0, -1.0],
                      "t": float(tg[0]["values"][0]), "value": [float(v) for v in tg[0]["values"][1:]]}
    gn = grep("src/ray/geometry.rs", r"(po|pa)\.get_normal.*Vector3::new\(" + NUM + ", " + NUM + ", " + NUM, 4)
    kats["polygon_normal"] = [{"where": e["where"], "shape": e["values"][0],
                               "p0": [0.0, 0.0, 0.0], "p1": [2.0, 1.0, 0.0], "p2": [0.0, 1.0, 2.0],
                               "value": [float(v) for v in e["values"][1:]]} for e in gn]
    # physics.rs
    cn = grep("src/ray/physics.rs", r"assert_eq!\(c3, Color::new\(" + NUM + ", " + NUM + ", " + NUM + r"\)\);", 3)
    kats["color_normalize"] = {"where": cn[0]["where"], "input": [0.4, 0.78, 1.0],
                               "value": [float(v) for v in cn[0]["values"]]}
    dw = grep("src/ray/physics.rs", r"decide_wavelength\(" + NUM + r"\), Wavelength::(Red|Green|Blue)\);", 2)
    kats["decide_wavelength"] = [{"where": e["where"], "p": float(e["values"][0]),
                                  "wl": {"Red": 0, "Green": 1, "Blue": 2}[e["values"][1]]} for e in dw]
    ps = grep("src/ray/physics.rs", r"let ps = \[" + NUM + ", " + NUM + ", " + NUM + ", " + NUM + ", " + NUM + r"\];", 5)
    cu = grep("src/ray/physics.rs", r"check_under\(&ps, " + NUM + r" ?\), ([0-9]+)\);", 2)
    kats["check_under"] = {"where": ps[0]["where"], "ps": [float(v) for v in ps[0]["values"]],
                           "cases": [{"where": e["where"], "p": float(e["values"][0]), "index": int(e["values"][1])}
                                     for e in cu]}
    ior = grep("src/ray/physics.rs", r"assert_eq!\(relative_ior\(" + NUM + ", " + NUM + r"\), " + NUM + r"\);", 3)
    kats["relative_ior_test"] = {"where": ior[0]["where"], "a": float(ior[0]["values"][0]),
                                 "b": float(ior[0]["values"][1]), "asserted": float(ior[0]["values"][2])}
    # kdtreetest.rs demo points and within radii
    pts = grep("src/bin/kdtreetest.rs", r"let (p[1-6]) = Photon::new\(&Wavelength::\w+, &Ray::new\(&Vector3::new\("
               + NUM + ", " + NUM + ", " + NUM, 4)
    win = grep("src/bin/kdtreetest.rs", r"kdtree\.within\(&Vector3::new\(0\.0, 0\.0, 0\.0\)\.v, ([0-9.*]+),", 1)
    radii = []
    for e in win:
        expr = e["values"][0]
        a = [float(x) for x in expr.split("*")]
        radii.append({"where": e["where"], "r2": a[0] * a[1] if len(a) == 2 else a[0]})
    kats["kdtree_demo"] = {"points": [{"where": e["where"], "name": e["values"][0],
                                       "pos": [float(v) for v in e["values"][1:]]} for e in pts],
                           "within": radii}
    with open(OUT, "w") as f:
        json.dump(kats, f, indent=1)
    print(OUT)


if __name__ == "__main__":
    main()
