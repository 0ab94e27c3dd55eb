"""Protocol files (the two-line dose/step text format of the reference's
tools/convert_protocols.py): round trips, indexing detection, the shift of
tumor-ca's 1-indexed steps onto the 300-step grid, and that a converted file
gives the same dose table as the protocol written directly."""
import numpy as np
import pytest


def test_round_trip(tmp_path):
    from emt6ro import protocols as P
    prots = [[(7200, 1.25), (21600, 1.25)], [(0, 10.0)], [(300, 0.25), (600, 9.75)]]
    P.write_protocols(prots, tmp_path / "p.txt")
    text = (tmp_path / "p.txt").read_text().splitlines()
    assert text[0] == "1.25 1.25" and text[1] == "7200 21600" and len(text) == 6
    assert P.read_protocols(tmp_path / "p.txt") == prots


def test_read_rejects_ragged_pairs(tmp_path):
    from emt6ro import protocols as P
    (tmp_path / "bad.txt").write_text("1.0 2.0\n300\n")
    with pytest.raises(ValueError, match="2 doses but 1 steps"):
        P.read_protocols(tmp_path / "bad.txt")


def test_validate_and_indexing():
    from emt6ro import protocols as P
    one = [[(1, 2.0), (8701, 3.0)], [(12601, 5.0)]]
    v = P.validate(one)
    assert v["indexing"] == "1-indexed" and v["n_aligned_1"] == 3 and v["n_events"] == 3
    zero = P.to_zero_indexed(one)
    assert zero == [[(0, 2.0), (8700, 3.0)], [(12600, 5.0)]]
    assert P.validate(zero)["indexing"] == "0-indexed"
    odd = [[(5, 1.0), (5, 1.0), (200_000, 1.0)]]
    v = P.validate(odd)
    assert v["indexing"] == "unaligned" and v["duplicates_per_protocol"] == 1
    assert v["n_out_of_range"] == 1 and v["examples_unaligned"] == [5, 5, 200_000]
    assert P.validate([[(0, 1.0)], [(1, 1.0)]])["indexing"] == "mixed-0-and-1"
    assert P.validate([])["indexing"] == "empty"


def test_converted_file_gives_the_same_dose_table(tmp_path):
    from emt6ro import protocols as P, workloads as wl
    direct = [[(21600, 1.25), (7200, 1.25)], [(600, 4.0)]]
    # the same protocols as a tumor-ca file would carry them: 1-indexed steps
    P.write_protocols([[(s + 1, d) for s, d in p] for p in direct], tmp_path / "tc.txt")
    loaded = P.to_experiment(P.read_protocols(tmp_path / "tc.txt"))
    assert loaded[0] == sorted(direct[0])
    assert np.array_equal(wl.protocol_doses(loaded, 480), wl.protocol_doses(direct, 480))


def _golden():
    import json
    from conftest import GOLDEN
    return GOLDEN, json.loads((GOLDEN / "protocols_ref.json").read_text())


def test_tool_outputs_match_the_reference_tool(capsys):
    """tests/golden/make_protocols.py ran the reference's
    tools/convert_protocols.py on protocols_in.txt: parsing, the validate
    report (dict and printed lines), the EMT6-Ro form, its two-line text and
    the diff against it must be the same here."""
    from emt6ro import protocols as P
    G, ref = _golden()
    parsed = P.read_protocols(G / "protocols_in.txt")
    assert parsed == [[tuple(e) for e in p] for p in ref["parsed"]]
    stats = P.validate(parsed)
    assert stats == ref["validate"]
    lines = [P.report_line(stats, 300, "protocols_in.txt")]
    lines.append(f"[protocols_in.txt]   unaligned step examples: {stats['examples_unaligned']}")
    assert "\n".join(lines) + "\n" == ref["validate_stdout"]
    emt6 = P.to_experiment(parsed)
    assert emt6 == [[tuple(e) for e in p] for p in ref["emt6"]]
    out = []
    assert P.diff(parsed, emt6, out.append) == ref["diff"]
    assert "\n".join(out) + "\n" == ref["diff_stdout"]


def test_tool_command_line(tmp_path, capsys):
    import json
    from emt6ro import protocols as P
    G, ref = _golden()
    assert P.main(["validate", str(G / "protocols_in.txt")]) == 1  # off-grid and out of range
    assert P.main(["to-emt6", str(G / "protocols_in.txt"), "--out", str(tmp_path / "e.json"),
                   "--canonicalize"]) == 0
    assert (tmp_path / "e.json").read_text() == json.dumps(ref["emt6"])
    assert P.main(["to-tumor-ca", str(tmp_path / "e.json"), str(tmp_path / "t.txt")]) == 0
    assert (tmp_path / "t.txt").read_text() == ref["emt6_two_line"]
    assert P.main(["diff", str(tmp_path / "t.txt"), str(tmp_path / "e.json")]) == 0
    assert P.main(["diff", str(G / "protocols_in.txt"), str(tmp_path / "e.json")]) == 1
    P.write_protocols([[(0, 1.0)]], tmp_path / "ok.txt")
    assert P.main(["validate", str(tmp_path / "ok.txt")]) == 0
