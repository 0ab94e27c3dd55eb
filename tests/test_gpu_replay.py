"""Protocol-file replay (emt6ro.replay, the reference's
tools/run_protocols_gpu.py): one index space over the whole file, so the
counts for a seed are the same whatever the chunking and equal one
Experiment over all protocols; the results file has one row per protocol,
tumour-major then run-major, and a metadata file."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

def _default_parameters_json():
    """The default parameter block in the reference's JSON schema
    (data/default-parameters.json)."""
    def subs(a, b, c):
        return {"cho": a, "ox": b, "gi": c}
    return {"lattice_dims": {"height": 51, "width": 51}, "time_step": 6,
            "diffusion_params": {"coeffs": subs(0.7, 1.3409874655051011, 0.81048692970088532),
                                 "time_step": 0.25},
            "metabolism": {"aerobic_proliferation": subs(21.6, 9.96, 0.0),
                           "anaerobic_proliferation": subs(54.0, 0.0, -3.0e-3),
                           "aerobic_quiescence": subs(18.0, 8.28, 0.0),
                           "anaerobic_quiescence": subs(45.0, 0.0, -3.0e-5)},
            "external_levels": subs(275.0, 14.0, 1.99e-3), "death_gi": 5.0e-2,
            "quiescence_gi": 1.99e-2, "death_gi_production": 0.0,
            "cycle_times": {k: {"mean": m, "stddev": sd} for k, (m, sd) in
                            zip(("g1", "s", "g2", "m", "d"),
                                ((6, 1), (10, 2), (2, 0), (2, 0), (0.1, 0)))},
            "cell_repair": {"delay_time": {"coeff": 3.3414, "exp_coeff": 0.1492},
                            "survival_prob": {"coeff": 1.0, "exp_coeff": -0.4993},
                            "repair_half_time": 0.8}}


PROTOCOLS = [[(0, 2.0), (1200, 1.25)], [(300, 4.0)], [], [(600, 1.0), (900, 1.5)],
             [(600, 0.5)]]  # within the 1,500 steps replayed


def test_replay_is_one_experiment_whatever_the_chunking(params):
    import emt6ro.simulation as sim
    from emt6ro import workloads as wl
    from emt6ro.replay import replay
    tumors = [wl.disc_tumor(params, 6, seed=1), wl.disc_tumor(params, 9, seed=2)]
    reps, steps = 3, 1500
    a = replay(params, tumors, PROTOCOLS, reps, steps, seed=99, protocol_chunk=2)
    b = replay(params, tumors, PROTOCOLS, reps, steps, seed=99)
    exp = sim.Experiment(params, tumors, runs=reps, protocols_num=len(PROTOCOLS),
                         simulation_steps=steps, seed=99)
    exp.add_irradiations(PROTOCOLS)
    exp.run(steps)
    c = exp.get_results()
    assert a.shape == (5, 2, 3)
    assert np.array_equal(a, b) and np.array_equal(a, c)
    assert a.min() > 0


def test_replay_command_line(params, tmp_path):
    import emt6ro.simulation as sim
    from emt6ro import protocols as P, workloads as wl
    from emt6ro.replay import main, replay
    tumors = [wl.disc_tumor(params, 7, seed=3), wl.disc_tumor(params, 5, seed=4)]
    paths = []
    for k, t in enumerate(tumors):
        paths.append(tmp_path / f"tumor-{k}.txt")
        sim.save_state(t, paths[-1])
    # tumor-ca's 1-indexed steps, as protocol files carry them (the two-line
    # format has no empty protocol: a blank pair of lines is skipped)
    prots = [p for p in PROTOCOLS if p]
    P.write_protocols([[(s + 1, d) for s, d in p] for p in prots], tmp_path / "p.txt")
    pfile = tmp_path / "params.json"
    pfile.write_text(json.dumps(_default_parameters_json()))
    assert bytes(sim.load_parameters(pfile).native) == bytes(params.native)
    assert main(["--protocols", str(tmp_path / "p.txt"), "--tumors", *map(str, paths),
                 "--params", str(pfile), "--reps", "2", "--steps", "1500", "--seed", "7",
                 "--protocol-chunk", "3", "--out", str(tmp_path / "r.txt")]) == 0
    rows = [list(map(int, line.split())) for line in (tmp_path / "r.txt").read_text().splitlines()]
    loaded = [sim.load_state(p, params) for p in paths]
    want = replay(params, loaded, prots, 2, 1500, seed=7)
    assert rows == want.reshape(len(prots), -1).tolist()
    meta = json.loads((tmp_path / "r.txt.meta.json").read_text())
    assert meta["n_protocols"] == 4 and meta["reps_per_tumor"] == 2 and meta["seed"] == 7
