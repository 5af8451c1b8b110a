"""Extracts the DFG (Schäfer-Turek) 2D cylinder benchmark at Re = 20 as the reference records it in
benchmarks/Cylinder2D/CylinderFlow_Re20.mojo: the target drag and lift coefficients and the drag
and lift the reference itself reached at each resolution, into dfg_re20.json.  Run in a checkout
that has the reference at REF (an environment variable; the script stops when it is unset)."""
import json
import os
import re
import sys
from pathlib import Path

REF = Path(os.environ["REF"]) if os.environ.get("REF") else None  # the reference checkout
SRC = "benchmarks/Cylinder2D/CylinderFlow_Re20.mojo"
OUT = Path(__file__).with_name("dfg_re20.json")


def extract(text: str) -> dict:
    """The fixture's content from the text of the reference's benchmark file."""
    cd = float(re.search(r"Drag coefficient:\s*Cd\s*=\s*([0-9.eE+-]+)", text).group(1))
    cl = float(re.search(r"Lift coefficient:\s*Cl\s*=\s*([0-9.eE+-]+)", text).group(1))
    # the recorded runs: a resolution header ("1024 x 256:"), optionally a collision name, then
    # "Drag Force: value" / "Lift Force: value" lines
    runs, res, coll = [], None, "not stated"
    for line in text.splitlines():
        m = re.match(r"\s*(\d+)\s*x\s*(\d+)\s*:", line)
        if m:
            res, coll = [int(m.group(1)), int(m.group(2))], "not stated"
            continue
        m = re.match(r"\s*(SRT|TRT|KBC)\s*:", line)
        if m:
            coll = m.group(1)
            continue
        m = re.search(r"(Drag|Lift) Force:\s*([0-9.eE+-]+),", line)
        if m and res:
            key = "drag" if m.group(1) == "Drag" else "lift"
            if not runs or runs[-1]["grid"] != res or runs[-1]["collision"] != coll or key in runs[-1]:
                runs.append({"grid": res, "collision": coll})
            runs[-1][key] = float(m.group(2))
    return {"source": SRC, "Cd": cd, "Cl": cl, "reference_runs": runs}


def main() -> int:
    if REF is None:
        sys.exit("set REF to the root of a reference checkout")
    fix = extract((REF / SRC).read_text())
    OUT.write_text(json.dumps(fix, indent=1))
    print(f"wrote {OUT}: Cd {fix['Cd']}, Cl {fix['Cl']}, {len(fix['reference_runs'])} recorded runs")
    return 0


if __name__ == "__main__":
    sys.exit(main())
