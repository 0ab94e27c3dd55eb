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
"""
from __future__ import annotations

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
    or one past it (1-indexed), off the grid, and repeated steps within a
    protocol; `indexing` names the convention the file follows."""
    stats = {"n_protocols": len(protocols), "n_events": 0, "n_in_range": 0,
             "n_out_of_range": 0, "n_aligned_0": 0, "n_aligned_1": 0, "n_unaligned": 0,
             "n_repeated_steps": 0}
    for prot in protocols:
        seen = set()
        for step, _ in prot:
            stats["n_events"] += 1
            stats["n_in_range" if 0 <= step < n_steps else "n_out_of_range"] += 1
            r = step % resolution
            key = "n_aligned_0" if r == 0 else ("n_aligned_1" if r == 1 else "n_unaligned")
            stats[key] += 1
            stats["n_repeated_steps"] += step in seen
            seen.add(step)
    a0, a1, off = stats["n_aligned_0"], stats["n_aligned_1"], stats["n_unaligned"]
    if stats["n_events"] == 0:
        stats["indexing"] = "empty"
    elif off:
        stats["indexing"] = "unaligned"
    elif a0 and a1:
        stats["indexing"] = "mixed"
    else:
        stats["indexing"] = "0-indexed" if a0 else "1-indexed"
    return stats


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
