"""tumor-ca JSON <-> .txt state conversion (emt6ro.states) against the
reference's own converter (tools/convert_state.py) on the golden vectors of
tests/golden/make_tumorca.py, plus the round trips the reference's
tools/test_convert_state_txt.py and its roundtrip-test check, and loading
a converted state into the simulator's format."""
import json

import numpy as np
import pytest

from conftest import GOLDEN


def _states():
    from emt6ro import states
    return states


@pytest.mark.parametrize("src,ref,scale", [
    ("tumorca_small.json", "tumorca_small.ref.txt", 1.0),
    ("tumorca_small.json", "tumorca_small.ref_e15.txt", 1e15),
    ("tumorca_small_nocyc.json", "tumorca_small_nocyc.ref.txt", 1.0),
])
def test_json_to_txt_is_the_reference_text(src, ref, scale, tmp_path):
    S = _states()
    info = S.tumorca_to_txt(GOLDEN / src, tmp_path / "out.txt", scale=scale)
    assert (tmp_path / "out.txt").read_text() == (GOLDEN / ref).read_text()
    key = {"tumorca_small.ref.txt": "txt", "tumorca_small.ref_e15.txt": "txt_e15",
           "tumorca_small_nocyc.ref.txt": "txt_nocyc"}[ref]
    assert info == json.loads((GOLDEN / "tumorca_small.ref_info.json").read_text())[key]


@pytest.mark.parametrize("txt,ref,scale,key", [
    ("tumorca_small.ref.txt", "tumorca_small.ref_rt.json", 1.0, "rt"),
    ("tumorca_small.ref_e15.txt", "tumorca_small.ref_rt_e15.json", 1e-15, "rt_e15"),
])
def test_txt_to_json_is_the_reference_document(txt, ref, scale, key, tmp_path):
    S = _states()
    info = S.txt_to_tumorca(GOLDEN / txt, tmp_path / "out.json", GOLDEN / "tumorca_small.json",
                            scale=scale)
    assert (tmp_path / "out.json").read_text() == (GOLDEN / ref).read_text()
    assert info == json.loads((GOLDEN / "tumorca_small.ref_info.json").read_text())[key]


def test_roundtrip_json_txt_json():
    """A document without dead-listed cells or mode entries on empty sites
    (the reference's own txt_to_json output) survives JSON -> .txt -> JSON;
    the synthetic one loses exactly those, as in the reference."""
    S = _states()
    assert S.roundtrip_check(GOLDEN / "tumorca_small.ref_rt.json") == []
    assert S.main(["roundtrip-test", str(GOLDEN / "tumorca_small.ref_rt.json")]) == 0
    fails = S.roundtrip_check(GOLDEN / "tumorca_small.json")
    assert [f.split(":")[0] for f in fails] == ["W", "lMET[quiesc]"]


def test_roundtrip_txt_json_txt_on_tumour_states(params, tmp_path):
    """.txt -> JSON -> .txt on states written by save_state (the tumour-lib
    states as the reference loads them, a seeded disc): every field equal."""
    import emt6ro.simulation as sim
    from emt6ro import workloads as wl
    S = _states()
    g = np.load(GOLDEN / "ref_states.npz")["states"]
    template = json.loads((GOLDEN / "tumorca_small.json").read_text())
    for sites in (g[0], g[6], wl.disc_tumor(params, 9, seed=3).sites):
        sim.save_state(sim.TumorState(sites), tmp_path / "a.txt")
        S.txt_to_tumorca(tmp_path / "a.txt", tmp_path / "a.json", template)
        S.tumorca_to_txt(tmp_path / "a.json", tmp_path / "b.txt")
        a = (tmp_path / "a.txt").read_text().split()
        b = (tmp_path / "b.txt").read_text().split()
        assert len(a) == len(b)
        assert np.allclose(np.array(a, float), np.array(b, float), rtol=1e-7, atol=0)


def test_load_tumorca_matches_the_txt_loader(params, tmp_path):
    import emt6ro.simulation as sim
    S = _states()
    S.tumorca_to_txt(GOLDEN / "tumorca_small.json", tmp_path / "s.txt", scale=1e15)
    a = sim.load_state(tmp_path / "s.txt", params).sites
    b = S.load_tumorca(GOLDEN / "tumorca_small.json", params, scale=1e15).sites
    assert a.shape == (18, 18) and a.tobytes() == b.tobytes()
    assert int((a["state"] == 1).sum()) == 93


def test_inconsistent_documents_are_refused(tmp_path):
    S = _states()
    doc = json.loads((GOLDEN / "tumorca_small.json").read_text())
    for name in ("prolif", "prolif_an", "quiesc", "quiesc_an"):  # drop one cell's entry
        if doc["STATE"]["lMET"][name]:
            idx = doc["STATE"]["lMET"][name].pop()
            break
    r, c = (idx - 1) % 16, (idx - 1) // 16
    assert doc["STATE"]["W"][r][c] == 1
    with pytest.raises(ValueError, match="W=1 but no lMET entry"):
        S.tumorca_to_text(doc)
    doc = json.loads((GOLDEN / "tumorca_small.json").read_text())
    doc["STATE"]["lMET"]["prolif"].append(16 * 16 + 1)
    with pytest.raises(ValueError, match="outside a grid"):
        S.tumorca_to_text(doc)
    (tmp_path / "r.txt").write_text("2\n3\n")
    with pytest.raises(ValueError, match="Non-square"):
        S.txt_to_tumorca(tmp_path / "r.txt", tmp_path / "r.json", doc)
    (tmp_path / "m.txt").write_text("1\n1\n1\n1\n1\n1\n0\n0\n0\n1\n2\n3\n4\n5\n7\n0\n")
    with pytest.raises(ValueError, match="Unknown mode 7"):
        S.txt_to_tumorca(tmp_path / "m.txt", tmp_path / "m.json", doc)
    with pytest.raises(ValueError, match="PARAMS"):
        S.txt_to_tumorca(tmp_path / "m.txt", tmp_path / "m.json", {"STATE": {}})
