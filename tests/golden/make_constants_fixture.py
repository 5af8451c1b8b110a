"""Extracts two tables of the reference into constants.json: the node flags of struct Flags
(src/lbm/constants.mojo: the low-nibble enum and the high-bit masks) and the keyword defaults of
LBM_Config.__init__ (src/lbm/config.mojo).  Run in a checkout that has the reference at REF (an
environment variable; the script stops when it is unset)."""
import json
import os
import sys
import re
from pathlib import Path

REF = Path(os.environ["REF"]) if os.environ.get("REF") else None  # the reference checkout
FLAGS_SRC = "src/lbm/constants.mojo"
CONFIG_SRC = "src/lbm/config.mojo"
OUT = Path(__file__).with_name("constants.json")


def extract_flags(text: str) -> dict:
    """name -> value of the `comptime NAME: UInt8 = value` members of struct Flags."""
    i = text.index("struct Flags")
    j = text.find("\nstruct ", i + 1)
    body = text[i: j if j >= 0 else len(text)]
    out = {}
    for m in re.finditer(r"comptime\s+(\w+)\s*:\s*UInt8\s*=\s*(0b[01]+|0x[0-9a-fA-F]+|\d+)", body):
        out[m.group(1)] = int(m.group(2), 0)
    return out


def _value(v: str):
    v = v.strip()
    if v in ("True", "False"):
        return v == "True"
    if v == "None":
        return None
    if v == "{}":
        return []
    if v[:1] in "'\"":
        return v[1:-1]
    return float(v)


def extract_config_defaults(text: str) -> dict:
    """name -> default of the keyword parameters of LBM_Config.__init__."""
    i = text.index("struct LBM_Config")
    i = text.index("def __init__(", i)
    j = text.index("):", i)
    out = {}
    for line in text[i:j].splitlines():
        m = re.match(r"\s*(\w+)\s*:\s*[^=]+?=\s*(.+?),?\s*$", line)
        if m:
            out[m.group(1)] = _value(m.group(2))
    return out


def extract(flags_text: str, config_text: str) -> dict:
    return {"flags_source": FLAGS_SRC, "config_source": CONFIG_SRC, "flags": extract_flags(flags_text),
            "config_defaults": extract_config_defaults(config_text)}


def main():
    if REF is None:
        sys.exit("set REF to the root of a reference checkout")
    fix = extract((REF / FLAGS_SRC).read_text(), (REF / CONFIG_SRC).read_text())
    OUT.write_text(json.dumps(fix, indent=1) + "\n")
    print(f"wrote {OUT}: {fix['flags']} {fix['config_defaults']}")


if __name__ == "__main__":
    main()
