"""Protocol fitness with surrogate pre-screening.

Same contract as EMT6RoModel.predict (fitness = 1500 - mean final living-cell
count over the tumours and runs, python/emt6ro/ga_model/model.py:33-54), but
the whole population is first scored by the learned surrogate and only the
best `keep_frac` is simulated in full; the simulated protocols get their
simulated fitness, the rest their predicted fitness.  `last` records what the
call did (counts, timings, the surrogate's predictions for the simulated
protocols) so callers can check the surrogate against simulation.

The elites are simulated on one Batch handle that every generation reuses
(created on the first call, rebuilt only when the number of elites changes):
predict uploads the elites' doses, runs the horizon as persistent CTAs over
the device work queue, reads the counts and resets the states.
"""
from __future__ import annotations

import os
import time

import numpy as np

from ..batch import Batch
from ..surrogate import prescreen
from .model import DEFAULT_SCHEDULE


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
        self.seed = int.from_bytes(os.urandom(8), "little") if seed is None else int(seed)
        self.last = {}
        self._batch = None
        self._keep = 0

    def _elite_batch(self, keep):
        if self._batch is None or self._keep != keep:
            T, R = len(self.tumors), self.num_tests
            idx = np.arange(keep * T * R)
            self._batch = Batch(self.params, self.tumors, [[] for _ in range(keep)],
                                ((idx // R) % T).astype(np.int32),
                                (idx // (T * R)).astype(np.int32),
                                protocol_resolution=self.protocol_resolution,
                                protocol_length=self.num_steps, device=self.gpu_id,
                                seed=self.seed)
            self._batch.set_schedule(*DEFAULT_SCHEDULE)
            self._keep = keep
        return self._batch

    def predict(self, protocols):
        P = len(protocols)
        keep = max(1, int(round(self.keep_frac * P)))
        t0 = time.perf_counter()
        elite, pred = prescreen(self.surrogate, protocols, self.tumors, keep)
        t1 = time.perf_counter()
        b = self._elite_batch(keep)
        b.add_irradiations([protocols[i] for i in elite])
        b.run(self.num_steps)
        simulated = b.counts().reshape(keep, -1).mean(1)
        b.reset()
        t2 = time.perf_counter()
        counts = pred.copy()
        counts[elite] = simulated
        self.last = {"elite": elite, "predicted": pred[elite], "simulated": simulated,
                     "surrogate_s": t1 - t0, "simulation_s": t2 - t1}
        return 1500 - counts
