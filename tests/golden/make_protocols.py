"""Golden vectors for emt6ro.protocols: the reference's protocol tool
(tools/convert_protocols.py of the reference checkout, imported from there)
run on a seeded protocol file.

Writes into tests/golden/:
  protocols_in.txt    12 protocols in the two-line format: 1-indexed (tumor-ca)
                      and 0-indexed ones, one with an off-grid step, one with a
                      repeated step, one out of range, an empty pair of lines
  protocols_ref.json  what the tool made of it: parse_two_line, validate (the
                      returned dict and the printed lines), to_emt6_python_form,
                      the two-line text of that form, diff against it (count
                      and printed lines)

Run from the repository root: python tests/golden/make_protocols.py
"""
import contextlib
import importlib.util
import io
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
from oracle.build import REFERENCE_ROOT  # noqa: E402


def reference_tool():
    path = REFERENCE_ROOT / "tools" / "convert_protocols.py"
    spec = importlib.util.spec_from_file_location("ref_convert_protocols", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def protocol_text(seed=77):
    rng = np.random.default_rng(seed)
    lines = []
    for k in range(12):
        n = int(rng.integers(1, 6))
        steps = np.sort(rng.choice(np.arange(0, 160), n, replace=False)) * 300
        if k % 3 == 0:
            steps = steps + 1  # tumor-ca's 1-indexed steps
        steps = [int(s) for s in steps]
        doses = [float(d) for d in np.round(rng.integers(1, 20, n) * 0.25, 2)]
        if k == 4:
            steps[0] += 7  # off the grid
        if k == 7 and n > 1:
            steps[1] = steps[0]  # a repeated step
        if k == 9:
            steps[-1] = 200_100  # out of range
        lines.append(" ".join(repr(d) for d in doses))
        lines.append(" ".join(str(s) for s in steps))
        if k == 5:
            lines += ["", ""]
    return "\n".join(lines) + "\n"


def main():
    ref = reference_tool()
    src = HERE / "protocols_in.txt"
    src.write_text(protocol_text())
    prots = ref.parse_two_line(src)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        stats = ref.validate(prots, label=str(src.name))
    canon = ref.to_emt6_python_form(prots)
    out = HERE / "_canon.txt"
    ref.write_two_line(canon, out)
    canon_text = out.read_text()
    out.unlink()
    dbuf = io.StringIO()
    with contextlib.redirect_stdout(dbuf):
        ndiff = ref.diff(prots, canon)
    doc = {"parsed": prots, "validate": stats, "validate_stdout": buf.getvalue(),
           "emt6": canon, "emt6_two_line": canon_text, "diff": ndiff,
           "diff_stdout": dbuf.getvalue()}
    (HERE / "protocols_ref.json").write_text(json.dumps(doc, indent=1))
    print(json.dumps(stats))


if __name__ == "__main__":
    main()
