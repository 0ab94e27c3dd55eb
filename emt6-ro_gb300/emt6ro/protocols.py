"""Irradiation protocol files: the two-line text format shared with tumor-ca.

A file holds one protocol per pair of lines: the doses (Gy), then the steps at
which they are given, both space-separated (the format read and written by
the reference's tools/convert_protocols.py).  tumor-ca matches a dose to a
step by equality and its files use 1-indexed steps on the 300-step grid
(k*300 + 1); this simulator fires a dose at step (s // resolution) *
resolution, so 1-indexed protocols are shifted down by one step before use.

    protocols = read_protocols("protocols.txt")
    report = validate(protocols)                # indexing, range, duplicates
    exp.add_irradiations(to_experiment(protocols))

The reference tool's subcommands run as

    python -m emt6ro.protocols validate FILE [--steps N] [--resolution R]
    python -m emt6ro.protocols to-emt6 FILE --out OUT.json [--canonicalize]
    python -m emt6ro.protocols to-tumor-ca IN.json OUT.txt
    python -m emt6ro.protocols diff A B        (two-line files or JSON)

with the tool's JSON form (a list of protocols, each a list of [step, dose])
and exit codes (validate: 1 when an event is off the grid or out of range;
diff: 1 when anything differs).
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path
from typing import List, Tuple

Protocol = List[Tuple[int, float]]


def read_protocols(path) -> List[Protocol]:
    """Protocols of a two-line file as lists of (step, dose); blank pairs skipped."""
    lines = Path(path).read_text().splitlines()
    out: List[Protocol] = []
    for k in range(0, len(lines) - 1, 2):
        doses_line, steps_line = lines[k].split(), lines[k + 1].split()
        if not doses_line and not steps_line:
            continue
        if len(doses_line) != len(steps_line):
            raise ValueError(f"{path}: protocol starting at line {k + 1} has "
                             f"{len(doses_line)} doses but {len(steps_line)} steps")
        out.append([(int(s), float(d)) for d, s in zip(doses_line, steps_line)])
    return out


def write_protocols(protocols, path) -> None:
    """Write protocols (lists of (step, dose)) in the two-line format."""
    text = []
    for prot in protocols:
        text.append(" ".join(repr(float(d)) for _, d in prot))
        text.append(" ".join(str(int(s)) for s, _ in prot))
    Path(path).write_text("\n".join(text) + ("\n" if text else ""))


def validate(protocols, n_steps: int = 144_000, resolution: int = 300) -> dict:
    """Counts of events in range, on the grid (0-indexed, s % resolution == 0)
    or one past it (1-indexed), off the grid (the first five in
    `examples_unaligned`), and repeated steps within a protocol
    (`duplicates_per_protocol`); `indexing` names the convention the file
    follows: "0-indexed", "1-indexed", "mixed-0-and-1", "unaligned" or
    "empty" (the reference tool's report)."""
    stats = {"n_protocols": len(protocols), "n_events": 0, "n_in_range": 0,
             "n_out_of_range": 0, "n_aligned_0": 0, "n_aligned_1": 0, "n_unaligned": 0,
             "duplicates_per_protocol": 0, "examples_unaligned": []}
    for prot in protocols:
        seen = set()
        for step, _ in prot:
            stats["n_events"] += 1
            stats["n_in_range" if 0 <= step < n_steps else "n_out_of_range"] += 1
            r = step % resolution
            key = "n_aligned_0" if r == 0 else ("n_aligned_1" if r == 1 else "n_unaligned")
            stats[key] += 1
            if key == "n_unaligned" and len(stats["examples_unaligned"]) < 5:
                stats["examples_unaligned"].append(step)
            stats["duplicates_per_protocol"] += step in seen
            seen.add(step)
    a0, a1, off = stats["n_aligned_0"], stats["n_aligned_1"], stats["n_unaligned"]
    if stats["n_events"] == 0:
        stats["indexing"] = "empty"
    elif off:
        stats["indexing"] = "unaligned"
    elif a0 and a1:
        stats["indexing"] = "mixed-0-and-1"
    else:
        stats["indexing"] = "0-indexed" if a0 else "1-indexed"
    return stats


def report_line(stats: dict, resolution: int = 300, label: str = "") -> str:
    """The tool's one-line summary of a validate() report."""
    prefix = f"[{label}] " if label else ""
    return (f"{prefix}protocols={stats['n_protocols']} events={stats['n_events']} "
            f"in_range={stats['n_in_range']} out_of_range={stats['n_out_of_range']} "
            f"resolution={resolution} aligned_0={stats['n_aligned_0']} "
            f"aligned_1={stats['n_aligned_1']} unaligned={stats['n_unaligned']} "
            f"duplicates={stats['duplicates_per_protocol']} indexing={stats['indexing']}")


def to_zero_indexed(protocols, resolution: int = 300) -> List[Protocol]:
    """Shift every protocol whose steps are all one past the grid down by one."""
    out = []
    for prot in protocols:
        if prot and all(s % resolution == 1 for s, _ in prot):
            out.append([(int(s) - 1, float(d)) for s, d in prot])
        else:
            out.append([(int(s), float(d)) for s, d in prot])
    return out


def to_experiment(protocols, resolution: int = 300) -> List[Protocol]:
    """Protocols ready for Experiment.add_irradiations: 0-indexed, sorted by step."""
    return [sorted(p, key=lambda e: e[0]) for p in to_zero_indexed(protocols, resolution)]


def write_json(protocols, path) -> None:
    """The tool's JSON form: a list of protocols, each a list of [step, dose]."""
    with Path(path).open("w") as f:
        json.dump([[[int(t), float(d)] for t, d in p] for p in protocols], f)


def read_json(path) -> List[Protocol]:
    return [[(int(t), float(d)) for t, d in p] for p in json.loads(Path(path).read_text())]


def _read_any(path) -> List[Protocol]:
    return read_json(path) if Path(path).suffix == ".json" else read_protocols(path)


def diff(a, b, out=print) -> int:
    """Differences between two protocol lists: a count mismatch, protocols
    of different lengths, and differing (step, dose) events, each reported
    through `out`; returns their number."""
    n = 0
    if len(a) != len(b):
        out(f"WARNING: protocol counts differ: {len(a)} vs {len(b)}")
        n += 1
    for i, (pa, pb) in enumerate(zip(a, b)):
        if len(pa) != len(pb):
            out(f"protocol {i}: |a|={len(pa)} |b|={len(pb)}")
            n += 1
            continue
        for j, (ea, eb) in enumerate(zip(pa, pb)):
            if tuple(ea) != tuple(eb):
                out(f"protocol {i} event {j}: {tuple(ea)} vs {tuple(eb)}")
                n += 1
    out(f"total diffs: {n} out of {max(len(a), len(b))} protocols compared")
    return n


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="irradiation protocol files (two-line format)")
    sub = ap.add_subparsers(dest="cmd", required=True)
    p = sub.add_parser("validate")
    p.add_argument("path", type=Path)
    p.add_argument("--steps", type=int, default=144_000)
    p.add_argument("--resolution", type=int, default=300)
    p = sub.add_parser("to-emt6")
    p.add_argument("path", type=Path)
    p.add_argument("--out", type=Path, required=True)
    p.add_argument("--canonicalize", action="store_true")
    p = sub.add_parser("to-tumor-ca")
    p.add_argument("path_json", type=Path)
    p.add_argument("out_text", type=Path)
    p = sub.add_parser("diff")
    p.add_argument("a", type=Path)
    p.add_argument("b", type=Path)
    args = ap.parse_args(argv)
    if args.cmd == "validate":
        stats = validate(read_protocols(args.path), args.steps, args.resolution)
        print(report_line(stats, args.resolution, str(args.path)))
        if stats["examples_unaligned"]:
            print(f"[{args.path}]   unaligned step examples: {stats['examples_unaligned']}")
        return 0 if stats["n_unaligned"] == 0 and stats["n_out_of_range"] == 0 else 1
    if args.cmd == "to-emt6":
        prots = read_protocols(args.path)
        if args.canonicalize:
            prots = to_experiment(prots)
        write_json(prots, args.out)
        print(f"Wrote {args.out}: {len(prots)} protocols, {sum(map(len, prots))} events")
        return 0
    if args.cmd == "to-tumor-ca":
        prots = read_json(args.path_json)
        write_protocols(prots, args.out_text)
        print(f"Wrote {args.out_text}: {len(prots)} protocols")
        return 0
    return 1 if diff(_read_any(args.a), _read_any(args.b)) else 0


if __name__ == "__main__":
    sys.exit(main())
