"""Regenerate tests/golden/d8_identity_pins.json from the reference test file.

The reference pins a 64-bit FNV-1a hash of every component of the D8 flow
object for 17 hermetic fixtures x 4 option configurations
(tests/cpp/test_flow_d8_identity.cpp, table `k_pins`). This script reads that
table as text and writes it out as JSON so that the tests need no reference
checkout at run time.

    python tests/golden/extract_d8_pins.py /path/to/lsdtt3    (or set LSDTT3_SRC)
"""
import json
import os
import re
import sys

COMPONENTS = ["receiver", "direction", "donors", "outlets", "topo", "svector", "area", "weighted"]


def main(ref_root: str) -> None:
    src = os.path.join(ref_root, "tests", "cpp", "test_flow_d8_identity.cpp")
    text = open(src).read()
    pins = {}
    for m in re.finditer(r'\{"([a-z0-9_]+/[a-z_]+)", \{([^}]*)\}\}', text):
        key = m.group(1)
        vals = [v.strip() for v in m.group(2).split(",")]
        vals = [int(v.replace("ULL", ""), 16) for v in vals]
        assert len(vals) == len(COMPONENTS), key
        pins[key] = {c: f"0x{v:016x}" for c, v in zip(COMPONENTS, vals)}
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "d8_identity_pins.json")
    with open(out, "w") as f:
        json.dump({"source": "tests/cpp/test_flow_d8_identity.cpp (k_pins)", "absent": "0xabad1deaabad1dea",
                   "pins": pins}, f, indent=1, sort_keys=True)
    print(f"{len(pins)} pins -> {out}")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LSDTT3_SRC", "")
    if not root:
        sys.exit("usage: extract_d8_pins.py /path/to/lsdtt3 (or set LSDTT3_SRC)")
    main(root)
