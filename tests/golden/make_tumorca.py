"""Golden vectors for emt6ro.states: the reference's own state converter
(tools/convert_state.py of the reference checkout, imported from there) run
on seeded synthetic tumor-ca states.

Writes into tests/golden/:
  tumorca_small.json          a 16 x 16 tumor-ca state with CYCLES: cells of all
                              four modes, cells on the 'dead' list, a site listed
                              with a mode but W = 0
  tumorca_small_nocyc.json    the same without CYCLES
  tumorca_small.ref.txt       json_to_txt(tumorca_small.json, scale=1)
  tumorca_small.ref_e15.txt   json_to_txt(tumorca_small.json, scale=1e15)
  tumorca_small_nocyc.ref.txt json_to_txt(tumorca_small_nocyc.json)
  tumorca_small.ref_rt.json   txt_to_json(tumorca_small.ref.txt, template=tumorca_small.json)
  tumorca_small.ref_rt_e15.json
                              txt_to_json(tumorca_small.ref_e15.txt, template=..., scale=1e-15)
  tumorca_small.ref_info.json the summaries the reference returned

Run from the repository root: python tests/golden/make_tumorca.py
"""
import importlib.util
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
from oracle.build import REFERENCE_ROOT  # noqa: E402

MODES = ("prolif", "prolif_an", "quiesc", "quiesc_an")
CYCLES = ("t_G1", "t_S", "t_G2", "t_M", "t_D")


def reference_converter():
    path = REFERENCE_ROOT / "tools" / "convert_state.py"
    spec = importlib.util.spec_from_file_location("ref_convert_state", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def synthetic_state(side=16, seed=2024):
    rng = np.random.default_rng(seed)
    rr, cc = np.mgrid[0:side, 0:side]
    disc = (rr - side / 2 + 0.5) ** 2 + (cc - side / 2 + 0.5) ** 2 <= (side / 2 - 2) ** 2
    w = (disc & (rng.random((side, side)) < 0.85)).astype(int)
    mode = rng.integers(0, 4, (side, side))
    dead = (w == 1) & (rng.random((side, side)) < 0.08)
    lmet = {k: [] for k in MODES + ("dead",)}
    for r in range(side):
        for c in range(side):
            idx = c * side + r + 1
            if dead[r, c]:
                lmet["dead"].append(idx)
            elif w[r, c]:
                lmet[MODES[mode[r, c]]].append(idx)
    # a site listed with a mode but without a cell (counted, written vacant)
    lmet["quiesc"].append(1)
    w[0, 0] = 0

    def grid(scale, digits=6):
        return np.round(rng.random((side, side)) * scale, digits).tolist()

    state = {"W": w.tolist(), "CHO": grid(3e-13, 18), "OX": grid(1e-13, 18),
             "GI": grid(2e-18, 24), "RepT": grid(4.0), "R": grid(2.5), "HRS": grid(20.0),
             "gMET": rng.integers(0, 5, (side, side)).tolist(), "lMET": lmet,
             "ch": np.zeros((side, side), int).tolist()}
    base = np.cumsum(rng.random((5, side, side)) * 8 + 1, axis=0)
    cycles = {k: np.round(base[i], 5).tolist() for i, k in enumerate(CYCLES)}
    return {"PARAMS": {"L": side, "dt": 6.0, "note": "synthetic"}, "STATE": state,
            "CYCLES": cycles}


def main():
    ref = reference_converter()
    doc = synthetic_state()
    small = HERE / "tumorca_small.json"
    small.write_text(json.dumps(doc, separators=(",", ":")))
    nocyc = dict(doc)
    del nocyc["CYCLES"]
    small_nc = HERE / "tumorca_small_nocyc.json"
    small_nc.write_text(json.dumps(nocyc, separators=(",", ":")))
    info = {
        "txt": ref.json_to_txt(small, HERE / "tumorca_small.ref.txt", scale=1.0),
        "txt_e15": ref.json_to_txt(small, HERE / "tumorca_small.ref_e15.txt", scale=1e15),
        "txt_nocyc": ref.json_to_txt(small_nc, HERE / "tumorca_small_nocyc.ref.txt"),
        "rt": ref.txt_to_json(HERE / "tumorca_small.ref.txt", HERE / "tumorca_small.ref_rt.json",
                              small, scale=1.0),
        "rt_e15": ref.txt_to_json(HERE / "tumorca_small.ref_e15.txt",
                                  HERE / "tumorca_small.ref_rt_e15.json", small, scale=1e-15),
    }
    (HERE / "tumorca_small.ref_info.json").write_text(json.dumps(info, indent=1))
    print(json.dumps(info))


if __name__ == "__main__":
    main()
