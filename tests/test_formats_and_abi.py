"""File formats (parameters JSON, tumour text) and the C ABI surface, on the
CPU: the library's host-side loaders are compared with the reference's own
loaders (golden fixtures from tests/golden/make_golden.py), every symbol
declared in include/*.h is exported and bound, and errors come
back as exceptions with the reference's messages."""
import json
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

from oracle.build import REFERENCE_ROOT as REF  # noqa: E402  (the reference checkout, if present)


def _N():
    from emt6ro import _native as N
    return N


def test_library_exports_every_declared_symbol():
    N = _N()
    declared = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        declared |= set(re.findall(
            r"^\s*(?:const char \*|void \*|int |void |emt6_batch \*)(emt6_\w+)\(",
            h.read_text(), re.M))
    assert len(declared) >= 45
    L = N.lib()
    for name in declared:
        assert hasattr(L, name), name
    assert declared == set(N.declared_symbols())
    assert L.emt6_version() == 1


def test_defaults_equal_reference_json(params):
    g = np.load(GOLDEN / "ref_params.npz")
    assert bytes(params.native) == g["default"].tobytes()


def test_parameter_loader_vs_reference(tmp_path):
    import emt6ro.simulation as sim
    g = np.load(GOLDEN / "ref_params.npz")
    if (REF / "data").exists():
        p = sim.load_parameters(REF / "data" / "default-parameters.json")
        assert bytes(p.native) == g["default"].tobytes()
        d = sim.load_parameters(REF / "data" / "test" / "dummy-parameters.json")
        assert bytes(d.native) == g["dummy"].tobytes()
    # the same schema written here: every value 1 (parameters-test.cc:16-40)
    subs = {"cho": 1, "ox": 1, "gi": 1}
    doc = {"lattice_dims": {"height": 1, "width": 1}, "time_step": 1,
           "diffusion_params": {"coeffs": subs, "time_step": 1},
           "metabolism": {k: subs for k in ("aerobic_proliferation", "anaerobic_proliferation",
                                            "aerobic_quiescence", "anaerobic_quiescence")},
           "external_levels": subs, "death_gi": 1, "quiescence_gi": 1, "death_gi_production": 1,
           "cycle_times": {k: {"mean": 1, "stddev": 1} for k in ("g1", "s", "g2", "m", "d")},
           "cell_repair": {"delay_time": {"coeff": 1, "exp_coeff": 1},
                           "survival_prob": {"coeff": 1, "exp_coeff": 1},
                           "repair_half_time": 1}}
    f = tmp_path / "dummy.json"
    f.write_text(json.dumps(doc))
    p = sim.load_parameters(f)
    assert bytes(p.native) == g["dummy"].tobytes()
    del doc["cell_repair"]["repair_half_time"]
    f.write_text(json.dumps(doc))
    with pytest.raises(RuntimeError, match="repair_half_time"):
        sim.load_parameters(f)
    with pytest.raises(RuntimeError, match="Could not open the file"):
        sim.load_parameters(tmp_path / "missing.json")


def test_state_loader_vs_reference(params):
    import emt6ro.simulation as sim
    g = np.load(GOLDEN / "ref_states.npz")["states"]
    assert g.shape == (10, 53, 53)
    if not (REF / "data").exists():
        pytest.skip("reference data files not present")
    for k in range(1, 11):
        s = sim.load_state(REF / "data" / "tumor-lib" / f"tumor-{k}.txt", params)
        assert s.sites.tobytes() == g[k - 1].tobytes(), k


def test_state_roundtrip_and_views(params, tmp_path):
    import emt6ro.simulation as sim
    from emt6ro import workloads as wl
    g = np.load(GOLDEN / "ref_states.npz")["states"]
    for sites in (wl.disc_tumor(params, 12, seed=1).sites, g[3]):
        st = sim.TumorState(sites)
        sim.save_state(st, tmp_path / "s.txt")
        back = sim.load_state(tmp_path / "s.txt", params)
        for f in ("state", "mode", "phase"):
            assert (back.sites[f] == sites[f]).all()
        for f in ("cho", "ox", "gi", "proliferation_time", "cycle_times"):
            np.testing.assert_allclose(back.sites[f], sites[f], rtol=1e-5)  # 6-digit text
    s = sim.TumorState(g[0])
    assert s.occupancy().shape == (53, 53) and s.cho().shape == (53, 53)
    assert (s.occupancy()[0] == sim.SiteState.Mocked).all()
    assert int((s.occupancy() == 1).sum()) == 321
    with pytest.raises(RuntimeError, match="Could not open the file"):
        sim.load_state(tmp_path / "nope.txt", params)


def test_truncated_state_is_rejected(params, tmp_path):
    import emt6ro.simulation as sim
    f = tmp_path / "t.txt"
    f.write_text("3\n3\n0\n275\n14\n0.00199\n1\n100\n")
    with pytest.raises(RuntimeError, match="truncated"):
        sim.load_state(f, params)


def test_oversize_lattice_is_rejected(tmp_path):
    """The on-chip kernels hold interiors up to 54 x 60; larger lattices are
    refused with a clear error (the reference's tile stops at 55,
    diffusion.cu:13)."""
    import emt6ro.simulation as sim
    from emt6ro import workloads as wl
    p = wl.default_parameters()
    p.native.lattice_height = 80
    st = np.zeros((82, 82), dtype=_N().SITE_DTYPE)
    with pytest.raises(RuntimeError, match="exceed the supported"):
        sim.Experiment(p, [sim.TumorState(st)], 1, 1)


def test_occupied_border_is_rejected(params):
    import emt6ro.simulation as sim
    from emt6ro import workloads as wl
    s = wl.disc_tumor(params, 5, seed=0).sites.copy()
    s["state"][0, 10] = 1
    with pytest.raises(RuntimeError, match="border"):
        sim.Experiment(params, [sim.TumorState(s)], 1, 1)


def test_add_irradiations_checks_protocol_count():
    from emt6ro.simulation.backend import _Experiment
    e = object.__new__(_Experiment)
    e.protocols_num = 2
    with pytest.raises(RuntimeError, match="Wrong number of protocols. Expected: 2"):
        e.add_irradiations([[(0, 1.0)]])


def test_experiment_result_shape_api():
    import emt6ro.simulation as sim
    assert sim.INSTR_HIST_N == 300 and sim.INSTR_HIST_DX == 0.1
    import inspect
    sig = inspect.signature(sim.Experiment.__init__)
    assert list(sig.parameters)[:8] == ["self", "params", "tumors", "runs", "protocols_num",
                                        "gpu_id", "simulation_steps", "protocol_resolution"]
    assert sig.parameters["simulation_steps"].default == 144000
    assert sig.parameters["protocol_resolution"].default == 300


def test_integration_c_example_compiles(tmp_path):
    """The C example in INTEGRATION.md compiles against include/ without warnings."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    doc = (ROOT / "INTEGRATION.md").read_text()
    a = doc.index("```c\n") + 5
    code = doc[a:doc.index("```", a)]
    code = code.replace('#include "emt6ro_gb300.h"', '#include "emt6ro_gb300.h"\nint main(void) {')
    src = tmp_path / "example.c"
    src.write_text("#include <stdio.h>\n#include <stdlib.h>\n" + code + "return 0; }\n")
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
                        "-c", str(src), "-o", str(tmp_path / "example.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
