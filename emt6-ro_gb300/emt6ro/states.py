"""Tumour states between tumor-ca's JSON and the .txt state format.

tumor-ca, the cellular automaton EMT6-Ro was ported from, keeps a state as
JSON.  PARAMS.L is the side of its square grid; STATE holds L x L grids W
(1 where a cell is), CHO, OX and GI (substrates), RepT (time in repair), R
(accumulated dose), HRS (hours into the cycle) and gMET (cycle phase), and
lMET, the sites of each metabolic mode ('prolif', 'prolif_an', 'quiesc',
'quiesc_an', and 'dead') as 1-based column-major indices c * L + r + 1;
CYCLES holds per-site cycle boundaries t_G1, t_S, t_G2, t_M, t_D.

The .txt format is a state's interior (src/emt6ro/state/state.cc:9-82): its
height and width, then per site in row-major order the state (1: a cell),
cho, ox and gi, and for a cell its time in repair, irradiation,
proliferation time, five cycle times, mode and phase.

The mapping is the one of the reference's tools/convert_state.py: a site
holds a cell when W is 1 and an lMET mode list names it (a later list wins
over an earlier one); sites on the 'dead' list become vacant; RepT, R and HRS
are time in repair, irradiation and proliferation time; t_G1 .. t_D the
cycle times (zeros when the JSON has no CYCLES); gMET the phase.  Substrates
can be scaled on the way (1e15 takes tumor-ca's mol to EMT6-Ro's units,
1e-15 back).  Numbers are written with nine significant digits, so a state
goes JSON -> .txt -> JSON unchanged to float32 precision.

    info = tumorca_to_txt("state.json", "tumor.txt", scale=1e15)
    tumor = load_tumorca("state.json", params, scale=1e15)      # a TumorState
    txt_to_tumorca("tumor.txt", "out.json", template="state.json")

Command line (the reference tool's subcommands):

    python -m emt6ro.states json-to-txt state.json tumor.txt [--scale S]
    python -m emt6ro.states txt-to-json tumor.txt out.json --template state.json [--scale S]
    python -m emt6ro.states roundtrip-test state.json [--tmpdir DIR]
"""
from __future__ import annotations

import argparse
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

MODE_LISTS = ("prolif", "prolif_an", "quiesc", "quiesc_an")  # lMET name of mode 0..3
CYCLE_KEYS = ("t_G1", "t_S", "t_G2", "t_M", "t_D")
STATE_GRIDS = ("W", "CHO", "OX", "GI", "RepT", "R", "HRS", "gMET")


def _site_of(index: int, side: int):
    """(row, column) of a 1-based column-major grid index."""
    return (index - 1) % side, (index - 1) // side


def _index_of(r: int, c: int, side: int) -> int:
    return c * side + r + 1


def _g(x) -> str:
    return f"{float(x):.9g}"


def _grids(doc: dict):
    side = int(doc["PARAMS"]["L"])
    st = doc["STATE"]
    grids = {k: st[k] for k in STATE_GRIDS}
    cyc = doc.get("CYCLES", {})
    cycles = [cyc.get(k) for k in CYCLE_KEYS]
    return side, grids, (cycles if all(v is not None for v in cycles) else None), st["lMET"]


def tumorca_to_text(doc: dict, scale: float = 1.0):
    """The .txt text of a tumor-ca state document and a summary of the
    conversion (sites with a cell, vacant sites, dead-listed sites, sites
    listed with a mode but W = 0, whether per-site cycle times were present)."""
    side, g, cycles, lmet = _grids(doc)
    mode = np.full((side, side), -1, np.int64)
    for m, name in enumerate(MODE_LISTS):
        for idx in lmet.get(name, []):
            r, c = _site_of(int(idx), side)
            if not (0 <= r < side and 0 <= c < side):
                raise ValueError(f"lMET index {idx} outside a grid of side {side}")
            mode[r, c] = m
    dead = np.zeros((side, side), bool)
    for idx in lmet.get("dead", []):
        r, c = _site_of(int(idx), side)
        if 0 <= c < side:  # an index past the grid names no site
            dead[r, c] = True

    info = {"L": side, "n_occupied": 0, "n_vacant": 0, "n_dead_skipped": int(dead.sum()),
            "n_w0_with_mode": 0, "scale": scale, "have_cycles": cycles is not None}
    out = [f"{side}\n{side}\n"]
    for r in range(side):
        for c in range(side):
            w = int(g["W"][r][c])
            has_mode = mode[r, c] >= 0
            if w == 1 and not has_mode and not dead[r, c]:
                raise ValueError(f"Site ({r},{c}) has W=1 but no lMET entry: "
                                 "the JSON is inconsistent.")
            if w == 0 and has_mode and not dead[r, c]:
                info["n_w0_with_mode"] += 1
            cell = w == 1 and has_mode and not dead[r, c]
            subs = (_g(float(g[k][r][c]) * scale) for k in ("CHO", "OX", "GI"))
            out.append("1\n" if cell else "0\n")
            out.append("\n".join(subs) + "\n")
            if cell:
                info["n_occupied"] += 1
                out.append("".join(_g(g[k][r][c]) + "\n" for k in ("RepT", "R", "HRS")))
                if cycles is not None:
                    out.append("".join(_g(t[r][c]) + "\n" for t in cycles))
                else:
                    out.append("0\n" * 5)
                out.append(f"{int(mode[r, c])}\n{int(g['gMET'][r][c])}\n")
            else:
                info["n_vacant"] += 1
    return "".join(out), info


def tumorca_to_txt(json_path, txt_path, scale: float = 1.0) -> dict:
    """Write the .txt state of a tumor-ca JSON file; returns the summary."""
    doc = json.loads(Path(json_path).read_text())
    text, info = tumorca_to_text(doc, scale)
    Path(txt_path).write_text(text)
    return info


def text_to_tumorca(text: str, template: dict, scale: float = 1.0):
    """A tumor-ca document from .txt text: the template's top-level fields
    (its PARAMS.L set to the state's side) with STATE and CYCLES replaced.
    Returns (document, summary)."""
    if "PARAMS" not in template:
        raise ValueError("the template has no PARAMS block")
    tok = iter(text.split())
    height, width = int(next(tok)), int(next(tok))
    if height != width:
        raise ValueError(f"Non-square grid {height}x{width} not supported.")
    side = height
    doc = json.loads(json.dumps(template))
    if int(doc["PARAMS"]["L"]) != side:
        doc["PARAMS"]["L"] = side

    def zeros(kind):
        return [[kind(0)] * side for _ in range(side)]

    st = {"W": zeros(int), "CHO": zeros(float), "OX": zeros(float), "GI": zeros(float),
          "RepT": zeros(float), "R": zeros(float), "HRS": zeros(float), "gMET": zeros(int),
          "lMET": {name: [] for name in MODE_LISTS + ("dead",)}, "ch": zeros(int)}
    cyc = {k: zeros(float) for k in CYCLE_KEYS}
    for r in range(side):
        for c in range(side):
            s = int(next(tok))
            for k in ("CHO", "OX", "GI"):
                st[k][r][c] = float(next(tok)) * scale
            if s != 1:
                continue
            st["W"][r][c] = 1
            for k in ("RepT", "R", "HRS"):
                st[k][r][c] = float(next(tok))
            for k in CYCLE_KEYS:
                cyc[k][r][c] = float(next(tok))
            m, phase = int(next(tok)), int(next(tok))
            if not 0 <= m < len(MODE_LISTS):
                raise ValueError(f"Unknown mode {m} at ({r},{c}).")
            st["lMET"][MODE_LISTS[m]].append(_index_of(r, c, side))
            st["gMET"][r][c] = phase
    doc["STATE"] = st
    doc["CYCLES"] = cyc
    return doc, {"L": side, "n_occupied": sum(map(sum, st["W"])), "scale": scale}


def txt_to_tumorca(txt_path, json_path, template, scale: float = 1.0) -> dict:
    """Write a tumor-ca JSON file for a .txt state; template is a tumor-ca
    JSON file (or document) whose PARAMS and other top-level fields are kept."""
    tdoc = template if isinstance(template, dict) else json.loads(Path(template).read_text())
    doc, info = text_to_tumorca(Path(txt_path).read_text(), tdoc, scale)
    with Path(json_path).open("w") as f:
        json.dump(doc, f, separators=(",", ":"))
    return info


def load_tumorca(json_path, params, scale: float = 1.0):
    """A tumor-ca JSON state as a TumorState (border ring added by the loader)."""
    from .simulation import load_state
    doc = json.loads(Path(json_path).read_text())
    text, _ = tumorca_to_text(doc, scale)
    with tempfile.TemporaryDirectory() as d:
        p = Path(d) / "state.txt"
        p.write_text(text)
        return load_state(p, params)


def roundtrip_check(json_path, tmpdir=None, eps: float = 1e-6) -> list:
    """JSON -> .txt -> JSON; the differences found (empty when none): whole
    grids W, CHO, OX, GI everywhere, per-cell fields (RepT, R, HRS, gMET,
    CYCLES) where both sides hold a cell, lMET mode lists as sets."""
    a = json.loads(Path(json_path).read_text())
    text, _ = tumorca_to_text(a, 1.0)
    b, _ = text_to_tumorca(text, a, 1.0)
    if tmpdir is not None:
        Path(tmpdir).mkdir(parents=True, exist_ok=True)
        (Path(tmpdir) / "roundtrip.txt").write_text(text)
        (Path(tmpdir) / "roundtrip.json").write_text(json.dumps(b, separators=(",", ":")))
    both = (np.asarray(a["STATE"]["W"]) == 1) & (np.asarray(b["STATE"]["W"]) == 1)
    fails = []

    def cmp(name, x, y, mask=None):
        x, y = np.asarray(x, float), np.asarray(y, float)
        if x.shape != y.shape:
            fails.append(f"{name}: shape {x.shape} vs {y.shape}")
            return
        d = np.abs(x - y) if mask is None else np.abs(x - y)[mask]
        if d.size and d.max() > eps:
            fails.append(f"{name}: max |diff| {d.max():.3g} > {eps:.3g}")

    for k in ("W", "CHO", "OX", "GI"):
        cmp(k, a["STATE"][k], b["STATE"][k])
    for k in ("RepT", "R", "HRS", "gMET"):
        cmp(k, a["STATE"][k], b["STATE"][k], both)
    for k in MODE_LISTS:
        sa = set(map(int, a["STATE"]["lMET"].get(k, [])))
        sb = set(map(int, b["STATE"]["lMET"].get(k, [])))
        if sa != sb:
            fails.append(f"lMET[{k}]: {len(sa - sb)} only before, {len(sb - sa)} only after")
    if "CYCLES" in a:
        for k in CYCLE_KEYS:
            if k in a["CYCLES"]:
                cmp(f"CYCLES.{k}", a["CYCLES"][k], b["CYCLES"][k], both)
    return fails


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="tumor-ca JSON <-> .txt tumour states")
    sub = ap.add_subparsers(dest="cmd", required=True)
    p = sub.add_parser("json-to-txt")
    p.add_argument("input_json", type=Path)
    p.add_argument("output_txt", type=Path)
    p.add_argument("--scale", type=float, default=1.0)
    p = sub.add_parser("txt-to-json")
    p.add_argument("input_txt", type=Path)
    p.add_argument("output_json", type=Path)
    p.add_argument("--template", type=Path, required=True)
    p.add_argument("--scale", type=float, default=1.0)
    p = sub.add_parser("roundtrip-test")
    p.add_argument("input_json", type=Path)
    p.add_argument("--tmpdir", type=Path, default=None)
    args = ap.parse_args(argv)
    if args.cmd == "json-to-txt":
        info = tumorca_to_txt(args.input_json, args.output_txt, args.scale)
        print(f"Wrote {args.output_txt}: L={info['L']} occupied={info['n_occupied']} "
              f"vacant={info['n_vacant']} scale={info['scale']}")
        return 0
    if args.cmd == "txt-to-json":
        info = txt_to_tumorca(args.input_txt, args.output_json, args.template, args.scale)
        print(f"Wrote {args.output_json}: L={info['L']} occupied={info['n_occupied']} "
              f"scale={info['scale']}")
        return 0
    fails = roundtrip_check(args.input_json, args.tmpdir)
    for f in fails:
        print("FAIL:", f)
    print("PASS" if not fails else f"{len(fails)} fields differ")
    return 1 if fails else 0


if __name__ == "__main__":
    sys.exit(main())
