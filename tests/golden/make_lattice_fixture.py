"""Extracts the reference's velocity sets from src/lbm/lattice.mojo (get_D2Q9, get_D3Q19, get_D3Q27):
the directions in the reference's order (rest first, each direction followed by its opposite) and
the weights as the numerator / denominator pairs the reference writes, and the order of the
symmetric stress components (get_stress_indices) for D = 2 and 3, into lattices.json.  Run in a
checkout that has the reference at REF (an environment variable; the script stops when it is unset)."""
import json
import os
import sys
import re
from pathlib import Path

REF = Path(os.environ["REF"]) if os.environ.get("REF") else None  # the reference checkout
SRC = "src/lbm/lattice.mojo"
OUT = Path(__file__).with_name("lattices.json")
NAMES = ("D2Q9", "D3Q19", "D3Q27")


def _block(body: str, start: str, close: str) -> str:
    """The text from the line holding `start` to the first later line that is `close` alone."""
    i = body.index(start)
    j = body.index("\n", i)
    k = re.compile(r"^\s*" + re.escape(close) + r"\s*$", re.M).search(body, j).start()
    return body[j:k]


def extract(text: str) -> dict:
    """The fixture's content from the text of the reference's lattice file."""
    out = {"source": SRC}
    for name in NAMES:
        i = text.index(f"def get_{name}[")
        nxt = text.find("\ndef ", i + 1)
        body = text[i: nxt if nxt >= 0 else len(text)]
        dirs = []
        for line in _block(body, "directions_list", "]").splitlines():
            m = re.match(r"\s*\[\s*(-?\d+)\s*,\s*(-?\d+)\s*(?:,\s*(-?\d+)\s*)?\]", line)
            if m:
                dirs.append([int(v) for v in m.groups() if v is not None])
        weights = []
        for line in _block(body, "weights = Vector", ")").splitlines():
            m = re.match(r"\s*(\d+(?:\.\d*)?)\s*/\s*(\d+(?:\.\d*)?)\s*(?:,|#|$)", line)
            if m:
                weights.append([float(m.group(1)), float(m.group(2))])
        out[name] = {"directions": dirs, "weights": weights}
    i = text.index("def get_stress_indices[")
    nxt = text.find("\ndef ", i + 1)
    body = text[i: nxt if nxt >= 0 else len(text)]
    out["stress_pairs"] = {}
    for d in (2, 3):
        j = body.index(f"elif D == {d}:")
        k = body.index("return", j)
        out["stress_pairs"][str(d)] = [[int(a), int(b)] for a, b in re.findall(r"\[\s*(\d)\s*,\s*(\d)\s*\]", body[j:k])]
    return out


def main():
    if REF is None:
        sys.exit("set REF to the root of a reference checkout")
    fix = extract((REF / SRC).read_text())
    OUT.write_text(json.dumps(fix, indent=1) + "\n")
    print(f"wrote {OUT}: " + ", ".join(f"{n} {len(fix[n]['directions'])}" for n in NAMES))


if __name__ == "__main__":
    main()
