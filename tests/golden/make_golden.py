"""Extract the reference's regression golds for the MPFA-O Richards path.

Reads the ``*.regression.gold`` files (max/min/mean and sampled-cell liquid
pressures after the full Newton + LU runs) and the PETSc-binary initial
condition of the richards driver problem from a TDycore checkout, and writes
``golden.json`` next to this script.  Run from the repository root:

    python tests/golden/make_golden.py /path/to/TDycore
"""
import base64
import json
import struct
import sys
from pathlib import Path

CASES = {
    # name: (gold file, description of the run that produced it)
    "transient-snes-mpfaof90": "demo/transient/transient-snes-mpfaof90.regression.gold",
    "transient-snes-mpfaof90-dirichlet": "demo/transient/transient-snes-mpfaof90-dirichlet.regression.gold",
    "transient-snes-mpfaof90-seepage": "demo/transient/transient-snes-mpfaof90-seepage.regression.gold",
    "transient-snes-mpfaof90-tdydriver": "demo/transient/transient-snes-mpfaof90-tdydriver.regression.gold",
    "transient-mpfaof90": "demo/transient/transient-mpfaof90.regression.gold",
    "transient-mpfaof90-tpf": "demo/transient/transient-mpfaof90-tpf.regression.gold",
    "transient-mpfaof90-neumann": "demo/transient/transient-mpfaof90-neumann.regression.gold",
    "transient-mpfaof90-tpf-neumann": "demo/transient/transient-mpfaof90-tpf-neumann.regression.gold",
    "richards-driver-snes-prob1": "demo/richards/richards-driver-snes-prob1.regression.gold",
}


def parse_gold(text):
    out = {"sampled": {}}
    for line in text.splitlines():
        line = line.strip()
        if ":" not in line or line.startswith("--"):
            continue
        key, val = [s.strip() for s in line.split(":", 1)]
        if key in ("Max", "Min", "Mean"):
            out[key.lower()] = float(val)
        else:
            out["sampled"][key] = float(val)
    return out


def read_petsc_vec(path):
    raw = Path(path).read_bytes()
    classid, n = struct.unpack(">ii", raw[:8])
    assert classid == 1211214, "not a PETSc Vec binary"
    return list(struct.unpack(">%dd" % n, raw[8:8 + 8 * n]))


def main(ref):
    ref = Path(ref)
    data = {"source": "TDycore regression gold files", "cases": {}}
    for name, rel in CASES.items():
        data["cases"][name] = {"file": rel, **parse_gold((ref / rel).read_text())}
    vec = ref / "demo/richards/richards_driver_snes_prob1_3x3x3_random.vec"
    data["richards_prob1_ic"] = read_petsc_vec(vec)
    # the file itself (80 bytes), for the PETSc-binary reader test
    data["richards_prob1_ic_petsc_binary_b64"] = base64.b64encode(vec.read_bytes()).decode()
    # the gold files' text, for the regression-output format test
    data["gold_text"] = {name: (ref / rel).read_text() for name, rel in CASES.items()}
    out = Path(__file__).resolve().parent / "golden.json"
    out.write_text(json.dumps(data, indent=1, sort_keys=True))
    print("wrote", out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/TDycore")
    main(sys.argv[1])
