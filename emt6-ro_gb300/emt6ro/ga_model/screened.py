"""Protocol fitness with surrogate pre-screening.

Same contract as EMT6RoModel.predict (fitness = 1500 - mean final living-cell
count over the tumours and runs, python/emt6ro/ga_model/model.py:33-54), but
the whole population is first scored by the learned surrogate and only the
best `keep_frac` is simulated in full; the simulated protocols get their
simulated fitness, the rest their predicted fitness.  `last` records what the
call did (counts, timings, the surrogate's predictions for the simulated
protocols) so callers can check the surrogate against simulation.
"""
from __future__ import annotations

import time

from .. import simulation as sim
from ..surrogate import prescreen


class ScreenedModel:
    def __init__(self, params, tumors, surrogate, num_tests, keep_frac=0.05, num_steps=144000,
                 protocol_resolution=300, gpu_id=0, seed=None):
        self.params = params
        self.tumors = tumors
        self.surrogate = surrogate
        self.num_tests = num_tests
        self.keep_frac = keep_frac
        self.num_steps = num_steps
        self.protocol_resolution = protocol_resolution
        self.gpu_id = gpu_id
        self.seed = seed
        self.last = {}

    def predict(self, protocols):
        P = len(protocols)
        keep = max(1, int(round(self.keep_frac * P)))
        t0 = time.perf_counter()
        elite, pred = prescreen(self.surrogate, protocols, self.tumors, keep)
        t1 = time.perf_counter()
        exp = sim.Experiment(self.params, self.tumors, self.num_tests, keep, self.gpu_id,
                             self.num_steps, self.protocol_resolution,
                             seed=self.seed)
        exp.add_irradiations([protocols[i] for i in elite])
        exp.run(self.num_steps)
        simulated = exp.get_results().reshape(keep, -1).mean(1)
        t2 = time.perf_counter()
        counts = pred.copy()
        counts[elite] = simulated
        self.last = {"elite": elite, "predicted": pred[elite], "simulated": simulated,
                     "surrogate_s": t1 - t0, "simulation_s": t2 - t1}
        return 1500 - counts
