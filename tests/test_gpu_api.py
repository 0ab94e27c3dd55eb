"""The drop-in Python API on the GPU: emt6ro.simulation.Experiment behaves as
the reference's (python/emt6ro/simulation/__init__.py, backend.cc:16-136):
result shape (protocol, tumour, run), run/get_results state errors, doses
accumulating into protocol bins, reset, state() views, the GA fitness model."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    from emt6ro import workloads as wl
    params = wl.default_parameters()
    tumors = [wl.disc_tumor(params, 7, seed=1), wl.disc_tumor(params, 10, seed=2)]
    return params, tumors


def test_experiment_shape_and_state_errors(setup):
    import emt6ro.simulation as sim
    params, tumors = setup
    e = sim.Experiment(params, tumors, 3, 2, seed=5)
    with pytest.raises(RuntimeError, match="First you have to run the experiment"):
        e.get_results()
    e.add_irradiations([[(300, 2.0)], []])
    e.run(400)
    with pytest.raises(RuntimeError, match="Experiment already running"):
        e.run(10)
    r = e.get_results()
    assert r.shape == (2, 2, 3) and r.dtype == np.uint32
    with pytest.raises(RuntimeError, match="Wrong number of protocols"):
        e.add_irradiations([[(0, 1.0)]])
    # a dose past the protocol length is refused (the reference writes it into
    # the next protocol's bins, backend.cc:97-99 + protocol.h:16-18)
    with pytest.raises(RuntimeError, match="beyond the protocol length"):
        e.add_irradiations([[(144_000, 1.0)], []])
    states = e.state()
    assert len(states) == 12
    counts = np.array([(s.occupancy() == 1).sum() for s in states]).reshape(2, 2, 3)
    assert (counts == r).all()
    assert states[0].cho().shape == (53, 53)


def test_experiment_matches_batch_and_oracle(setup, oracle):
    """(protocol, tumour, run) order; doses accumulate in bin step // 300."""
    import emt6ro.simulation as sim
    from emt6ro import workloads as wl
    params, tumors = setup
    prots = [[(0, 1.0), (100, 1.0), (620, 0.5)], [(1200, 3.0)]]
    e = sim.Experiment(params, tumors, 2, 2, seed=17)
    e.add_irradiations(prots)
    e.run(1300)
    r = e.get_results()
    dose = wl.protocol_doses(prots, 480)
    assert dose[0][0] == 2.0 and dose[0][2] == 0.5 and dose[1][4] == 3.0
    ob = oracle.Batch(oracle.params_copy(params), 8, 17)
    i = 0
    for p in range(2):
        for t in range(2):
            for _ in range(2):
                ob.set(i, tumors[t].sites, dose[p])
                i += 1
    ob.run(1300, nthreads=8)
    assert (r.reshape(-1) == ob.counts()).all()


def test_experiment_other_resolution_and_length(setup, oracle):
    """simulation_steps = 6,000 and protocol_resolution = 60: doses accumulate
    in bin step // 60 and fire at its first step; a run past the protocol
    length gives no further doses (protocol.h:9-18)."""
    import emt6ro.simulation as sim
    from emt6ro import workloads as wl
    params, tumors = setup
    prots = [[(0, 1.0), (90, 1.0), (130, 0.5), (5999, 2.0)], [(59, 3.0), (4200, 1.0)]]
    e = sim.Experiment(params, tumors, 2, 2, 0, 6000, 60, seed=29)
    e.add_irradiations(prots)
    with pytest.raises(RuntimeError, match="beyond the protocol length"):
        e.add_irradiations([[(6000, 1.0)], []])
    e.run(6600)
    r = e.get_results()
    dose = wl.protocol_doses(prots, 100, 60)
    assert dose[0][1] == 1.0 and dose[0][2] == 0.5 and dose[0][99] == 2.0
    assert dose[1][0] == 3.0 and dose[1][70] == 1.0
    ob = oracle.Batch(oracle.params_copy(params), 8, 29)
    i = 0
    for p in range(2):
        for t in range(2):
            for _ in range(2):
                ob.set(i, tumors[t].sites, dose[p], resolution=60, length=6000)
                i += 1
    ob.run(6600, nthreads=8)
    assert (r.reshape(-1) == ob.counts()).all()


def test_reset_restores_initial_states(setup):
    import emt6ro.simulation as sim
    params, tumors = setup
    e = sim.Experiment(params, tumors, 1, 1, seed=3)
    e.add_irradiations([[(0, 5.0)]])
    e.run(2000)
    e.get_results()
    e.reset()
    s = e.state()
    assert s[0].sites.tobytes() == tumors[0].sites.tobytes()
    assert s[1].sites.tobytes() == tumors[1].sites.tobytes()
    e.run(1)  # doses were zeroed: no irradiation at step 0
    e.get_results()
    assert all((x.irradiation() == 0).all() for x in e.state())


def test_ga_model_predict(setup):
    from emt6ro.ga_model import EMT6RoModel
    params, tumors = setup
    m = EMT6RoModel(params, tumors, num_protocols=3, num_tests=2, num_gpus=1, num_steps=600,
                    seed=1)
    prots = [[(0, 2.5)], [(300, 1.25), (599, 1.25)], []]
    f = m.predict(prots)
    assert f.shape == (3,)
    assert (f > 1000).all() and (f < 1500).all()
    f2 = m.predict(prots)  # reset between generations: fresh epoch, same distribution
    assert f2.shape == (3,)


def test_ga_model_fitness_equals_reference_flow_and_ignores_sharding(setup):
    """EMT6RoModel's persistent sharded batches give, for a fixed seed, exactly
    the fitness of the reference's flow on one GPU (one Experiment per GPU:
    add_irradiations, run, get_results, 1500 - mean, reset;
    python/emt6ro/ga_model/model.py:36-54) over two generations, and the same
    fitness whether the population is one shard or split into two or three
    (random streams keyed by the global simulation index)."""
    import emt6ro.simulation as sim
    from emt6ro.ga_model import EMT6RoModel
    params, tumors = setup
    gens = [[[(0, 2.5)], [(300, 1.25), (599, 1.25)], []],
            [[(600, 4.0)], [], [(0, 1.0), (900, 3.0)]]]
    steps, R = 6000, 6
    e = sim.Experiment(params, tumors, R, 3, 0, steps, 300, seed=77)
    expected = []
    for prots in gens:
        e.add_irradiations(prots)
        e.run(steps)
        res = e.get_results().reshape((1, 3, -1))
        expected.append(1500 - res.mean(0).mean(1))
        e.reset()
    assert not np.array_equal(expected[0], expected[1])
    models = [EMT6RoModel(params, tumors, 3, R, num_gpus=1, num_steps=steps, seed=77),
              EMT6RoModel(params, tumors, 3, R // 2, num_steps=steps, seed=77, devices=[0, 0]),
              EMT6RoModel(params, tumors, 3, R // 3, num_steps=steps, seed=77,
                          devices=[0, 0, 0])]
    assert [len(m.shards) for m in models] == [1, 2, 3]
    for prots, exp in zip(gens, expected):
        for m in models:
            assert np.array_equal(m.predict(prots), exp)


def test_instrumentation_counters(setup):
    import emt6ro.simulation as sim
    params, tumors = setup
    sim.reset_instr_counters()
    e = sim.Experiment(params, tumors, 2, 1, seed=9)
    e.add_irradiations([[(0, 4.0)]])
    e.run(12000)  # the repair delay after 4 Gy is about 6 h = 3640 steps
    e.get_results()
    c = sim.read_instr_counters()
    n0 = 2 * sum(int((t.occupancy() == 1).sum()) for t in tumors)
    # every cell alive after step 0's state update is irradiated once
    assert 0.8 * n0 <= c.irradiation_events <= n0
    assert 0 < c.repair_kills <= c.repair_decisions
    h = sim.read_instr_histograms()
    assert len(h) == 600 and sum(h[:300]) == c.repair_decisions == sum(h[300:])
    sim.reset_instr_counters()
    assert sim.read_instr_counters().repair_decisions == 0
