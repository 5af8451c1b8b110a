"""Extracts the Re = 100 column of the Ghia, Ghia & Shin (1982) cavity centre-line tables that the
reference ships (benchmarks/LDC/u_velocity_results.txt, benchmarks/LDC/v_velocity_results.csv)
into ghia_re100.json.  Run in a checkout that has the reference at REF (an environment variable; the script stops when it is unset)."""
import json
import os
import sys
from pathlib import Path

REF = Path(os.environ["REF"]) if os.environ.get("REF") else None  # the reference checkout
OUT = Path(__file__).with_name("ghia_re100.json")


def column(path: Path, sep: str | None):
    rows = [ln.split(sep) for ln in path.read_text().splitlines() if ln.strip()]
    head = [h.strip() for h in rows[0]]
    j = head.index("100")
    return [[float(r[0]), float(r[j])] for r in rows[1:]]


def main() -> int:
    if REF is None:
        sys.exit("set REF to the root of a reference checkout")
    u = column(REF / "benchmarks/LDC/u_velocity_results.txt", None)
    v = column(REF / "benchmarks/LDC/v_velocity_results.csv", ",")
    OUT.write_text(json.dumps({"source": "benchmarks/LDC/u_velocity_results.txt, v_velocity_results.csv (Re=100)",
                               "u_vs_y": u, "v_vs_x": v}, indent=1))
    print(f"wrote {OUT} ({len(u)} u points, {len(v)} v points)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
