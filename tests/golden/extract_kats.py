"""Extract the reference's golden test values into ``reference_kats.json``.

Run with the path of a checkout of the reference source tree (read only):

    python tests/golden/extract_kats.py <path-to-moldyn-checkout>

The reference is Rust and cannot be built or run in this environment, so its
known-answer tests are read as text: every
``assert_eq!(format!("{:.8}", <expr>), "<value>")`` in the listed test
functions is recorded with the number of integrator steps that precede it in
the function body (``verlet.calculate(...)`` calls, with ``for _ in 0..N``
loops multiplied out).  The resulting JSON is committed; tests read only the
JSON, never the reference tree.
"""
from __future__ import annotations

import json
import os
import re
import sys

FILES = {
    "solver/src/lib.rs": ["lennard_jones", "update_force_lennard_jones", "verlet_with_lennard_jones",
                          "verlet_lj_1000_iterations", "energies", "temperature", "pressure"],
    "cli/src/tests.rs": ["initialization", "solvation"],
}

ASSERT_FMT = re.compile(r'assert_eq!\(\s*format!\("\{:\.8\}",\s*(.+?)\),\s*"([^"]+)"\s*\)', re.S)
ASSERT_EQ = re.compile(r'assert_eq!\(\s*([^,]+?),\s*([^;]+?)\);')
FOR_LOOP = re.compile(r'for\s+_\s+in\s+0\.\.(\d+)')


def function_body(src: str, name: str) -> tuple[str, int]:
    m = re.search(r"fn\s+%s\s*\(\s*\)\s*\{" % re.escape(name), src)
    if not m:
        raise KeyError(name)
    i = m.end()
    depth = 1
    while depth:
        c = src[i]
        depth += (c == "{") - (c == "}")
        i += 1
    line = src.count("\n", 0, m.start()) + 1
    return src[m.end():i - 1], line


def scan(body: str, first_line: int, relpath: str):
    """Walk statements in order, tracking integrator steps taken so far."""
    records = []
    steps = 0
    loop_mult = []  # stack of (depth, multiplier)
    depth = 0
    pos = 0
    tokens = re.finditer(r'for\s+_\s+in\s+0\.\.\d+\s*\{|\{|\}|\.calculate\(|solve\(&path|'
                         r'assert_eq!\(\s*format!\("\{:\.8\}".+?\);|assert_eq!\(.+?\);', body, re.S)
    for tok in tokens:
        t = tok.group(0)
        line = first_line + body.count("\n", 0, tok.start())
        if t.startswith("for"):
            depth += 1
            loop_mult.append((depth, int(FOR_LOOP.search(t).group(1))))
        elif t == "{":
            depth += 1
        elif t == "}":
            if loop_mult and loop_mult[-1][0] == depth:
                loop_mult.pop()
            depth -= 1
        elif t == ".calculate(":
            mult = 1
            for _, m in loop_mult:
                mult *= m
            steps += mult
        elif t.startswith("solve(&path"):
            # cli/src/tests.rs:59-62: solve(path, state, method, custom, use_potentials, iteration_count, ...)
            args = body[tok.start() + len("solve("):body.index(");", tok.end())]
            parts = [p.strip() for p in args.replace("\n", " ").split(",")]
            steps += int(parts[5].lstrip("&"))
        elif t.startswith("assert_eq!(") and "format!" in t:
            m = ASSERT_FMT.search(t)
            records.append({"expr": " ".join(m.group(1).split()), "value": m.group(2),
                            "after_steps": steps, "source": f"{relpath}:{line}"})
        else:
            m = ASSERT_EQ.search(t)
            if m:
                records.append({"expr": " ".join(m.group(1).split()),
                                "equals": " ".join(m.group(2).split()),
                                "after_steps": steps, "source": f"{relpath}:{line}"})
    return records


def main(root: str) -> None:
    out = {"generator": "tests/golden/extract_kats.py", "tests": {}}
    for rel, names in FILES.items():
        with open(os.path.join(root, rel)) as f:
            src = f.read()
        for name in names:
            body, line = function_body(src, name)
            out["tests"][name] = {"source": f"{rel}:{line}", "asserts": scan(body, line, rel)}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    n = sum(len(t["asserts"]) for t in out["tests"].values())
    print(f"wrote {dst}: {len(out['tests'])} tests, {n} asserts")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/extract_kats.py <path-to-moldyn-checkout>")
    main(sys.argv[1])
