"""Extracts the l2 / linf golden vectors of the reference's test suite into
reference_goldens.json (run once where the reference sources are available;
the tests read only the JSON).

    python tests/golden/extract_goldens.py <reference>/test

Each `@trixi_testset "name"` block of test/*.jl contributes an entry keyed
"<file>:<line> <name>" with its `l2=[...]` and `linf=[...]` arrays (numbers as
written in the file) and the keyword overrides that follow them (tspan,
polydeg, cells, ...), kept verbatim as text."""
import json
import os
import re
import sys

NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"


def parse_array(text, key):
    m = re.search(r"\b" + key + r"\s*=\s*\[(.*?)\]", text, re.S)
    if not m:
        return None
    return [float(x) for x in re.findall(NUM, m.group(1))]


def extract(test_dir):
    out = {}
    for fn in sorted(os.listdir(test_dir)):
        if not fn.endswith(".jl"):
            continue
        lines = open(os.path.join(test_dir, fn)).read().split("\n")
        starts = [(i, re.match(r'\s*@trixi_testset\s+"([^"]+)"', l).group(1))
                  for i, l in enumerate(lines) if re.match(r'\s*@trixi_testset\s+"', l)]
        for k, (i, name) in enumerate(starts):
            end = starts[k + 1][0] if k + 1 < len(starts) else len(lines)
            block = "\n".join(lines[i:end])
            l2, linf = parse_array(block, "l2"), parse_array(block, "linf")
            if l2 is None or linf is None:
                continue
            tail = block[block.find("linf"):]
            tail = tail[tail.find("]") + 1:]
            overrides = tail[:tail.find(")\n")].strip().strip(",").strip()
            out[f"test/{fn}:{i + 1} {name}"] = {"l2": l2, "linf": linf,
                                                "overrides": " ".join(overrides.split())}
    return out


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    data = extract(sys.argv[1])
    with open(os.path.join(here, "reference_goldens.json"), "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    print(len(data), "testsets")
