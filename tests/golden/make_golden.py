"""Generate golden vectors from the reference's own arithmetic.

Builds oracle/_ref/ref_probe (oracle/ref_build.sh compiles the reference's
header-only Binner::Key and Waveform_Sine against host stand-ins for the
non-vendored rtac_base headers) and records its answers for a fixed, seeded
set of inputs into tests/golden/ref_keys.json, ref_waveforms.json and
ref_directivity.json (the receiver directivity builders of src/Directivity.cpp).
Needs the reference tree (the argument, else where oracle/ref_build.sh looks
for it); the tests only read the committed JSON files.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
PROBE = ROOT / "oracle" / "_ref" / "ref_probe"

F32 = np.float32

# (bins, min, max, margin): benchmark sensors, the reference's example YAMLs
# (Oculus M1200d: Linspace(0.1, 6.5, 500); EA400: Linspace(0.1, 49.999, 1049)),
# and degenerate shapes.
KEY_CONFIGS = [
    (4096, 0.5, 100.0, 1.5799),
    (1024, 0.3, 40.0, 1.2806),
    (4096, 0.3, 120.0, 0.9647),
    (8192, 0.3, 120.0, 0.4824),
    (2048, 1.0, 60.0, 2.0),
    (500, 0.1, 6.5, 0.012826),
    (1049, 0.1, 49.999, 0.192),
    (256, 0.1, 6.5, 0.0),
    (2, 0.0, 1.0, 0.25),
    (1, 0.3, 40.0, 0.5),
    (3, 10.0, 10.5, 100.0),
    (100, -5.0, 5.0, 1.0),
]


def f32hex(x) -> str:
    return float(F32(x)).hex()


def edge_travels(nbins, lo, hi, margin, rng) -> np.ndarray:
    res = (hi - lo) / nbins
    m, M = lo - 0.5 * res, hi + 0.5 * res
    a = (nbins - 1) / (M - m) if M > m else 0.0
    vals = [-1.0, 0.0, -0.0, lo, hi, lo - margin, hi + margin, m, M, m - margin, M + margin,
            0.5 * (lo + hi), 1e-30, 1e30, -1e30, 3.0e9]
    if a > 0:
        for k in list(range(0, min(nbins, 6))) + list(range(max(0, nbins - 6), nbins + 3)):
            edge = m + (k - 0.5 + 0.5) / a   # where fmaf(a, t, b) crosses k
            for d in (-1e-6, 0.0, 1e-6):
                vals.append(edge * (1 + d) if edge != 0 else d)
        # (-1, 0) truncation band below bin 0 and the unit-mixing bound tests
        for q in (-1.5, -1.0, -0.999, -0.5, -0.001, -2.0, -3.0):
            vals.append(m + (q + 0.0) / a)
    span = (hi - lo) + 4 * margin + 4 * res
    vals += list(rng.uniform(lo - margin - 2 * res - 0.1 * span, hi + margin + 2 * res + 0.1 * span, 400))
    return np.array(vals, dtype=F32)


def run_probe(lines):
    res = subprocess.run([str(PROBE)], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    return res.stdout.strip().split("\n")


def main():
    subprocess.run([str(ROOT / "oracle" / "ref_build.sh"), *sys.argv[1:2]], check=True)
    if not PROBE.exists():
        raise SystemExit("no reference tree: pass its path, or set RTAC_SIMULATION_REFERENCE")
    rng = np.random.Generator(np.random.PCG64(2024))

    key_cases = []
    lines = []
    for (nb, lo, hi, mg) in KEY_CONFIGS:
        t = edge_travels(nb, lo, hi, mg, rng)
        key_cases.append(dict(bins=nb, min=f32hex(lo), max=f32hex(hi), margin=f32hex(mg),
                              travel=[f32hex(x) for x in t]))
        lines.append(" ".join(["KEY", str(nb), f32hex(lo), f32hex(hi), f32hex(mg), str(len(t))] +
                              [f32hex(x) for x in t]))
    out = run_probe(lines)
    for case, line in zip(key_cases, out):
        tok = line.split()
        assert tok[0] == "KEY"
        case["a"], case["b"], case["lower"], case["upper"] = tok[1:5]
        case["keys"] = [None if k == "x" else int(k) for k in tok[5:]]
    (HERE / "ref_keys.json").write_text(json.dumps(dict(
        source="rtac_simulation include/rtac_simulation/Binner.h:25-54 compiled by oracle/ref_build.sh",
        cases=key_cases), indent=0))

    wave_cases = [(1.2e6, 2.5651e-5, 8), (38.0e3, 128.0e-6, 8), (200.0e3, 5.0e-5, 8), (1.2e6, 1.0e-5, 4),
                  (38.0e3, 1.0e-3, 2), (1.2e6, 0.0, 8)]
    lines = [f"WAVE {f32hex(f)} {f32hex(d)} {os_}" for f, d, os_ in wave_cases]
    out = run_probe(lines)
    waves = []
    for (f, d, os_), line in zip(wave_cases, out):
        tok = line.split()
        size = int(tok[1])
        vals = [float.fromhex(x) for x in tok[2:]]
        waves.append(dict(frequency=f32hex(f), duration=f32hex(d), oversampling=os_, size=size,
                          re=[float(v).hex() for v in vals[0::2]], im=[float(v).hex() for v in vals[1::2]]))
    (HERE / "ref_waveforms.json").write_text(json.dumps(dict(
        source="rtac_simulation include/rtac_simulation/Waveform.h:96-138 compiled by oracle/ref_build.sh",
        cases=waves), indent=0))
    # Directivity tables (src/Directivity.cpp): small parameter sets so that
    # the fixtures stay small; lengths in metres.
    dir_cases = [("RECT", (1.56e-3, 8.0e-3, 1.25e-3), "single-sided", 2),
                 ("RECT", (1.56e-3, 4.0e-3, 1.25e-3), "none", 4),
                 ("DISK", (0.15, 0.0395), "single-sided", 1),
                 ("DISK", (0.05, 0.0395), "none", 2)]
    lines = [" ".join([kind] + [f32hex(x) for x in par] + [baffle, str(os_)]) for kind, par, baffle, os_ in dir_cases]
    out = run_probe(lines)
    dirs = []
    for (kind, par, baffle, os_), line in zip(dir_cases, out):
        tok = line.split()
        w, h = int(tok[1]), int(tok[2])
        dirs.append(dict(kind=kind, params=[f32hex(x) for x in par], baffle=baffle, oversampling=os_,
                         width=w, height=h, values=tok[3:]))
    (HERE / "ref_directivity.json").write_text(json.dumps(dict(
        source="rtac_simulation src/Directivity.cpp:59-166 compiled by oracle/ref_build.sh", cases=dirs)))
    print(f"wrote {len(key_cases)} key cases, {len(waves)} waveform cases, {len(dirs)} directivity tables")


if __name__ == "__main__":
    main()
