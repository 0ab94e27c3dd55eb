"""Fitness model of irradiation protocols (python/emt6ro/ga_model/model.py:5-54)."""
from .. import simulation as sim
import numpy as np


class EMT6RoModel:
    """
    Model calculating fitness of irradiation protocols: fitness = 1500 - mean
    final living-cell count over tumours, runs and GPUs.

    One Experiment per GPU (num_gpus); each holds num_protocols x tumours x
    num_tests simulations.  The GPUs run concurrently: every Experiment is
    started before any result is read.
    """

    def __init__(self, params, tumors, num_protocols, num_tests, num_gpus=1, num_steps=144000,
                 protocol_resolution=300, seed=None):
        self.num_steps = num_steps
        self.protocol_resolution = protocol_resolution
        self.params = params
        self.tumors = tumors
        self.num_protocols = num_protocols
        self.num_tests = num_tests
        self.num_gpus = num_gpus
        self.experiments = [
            sim.Experiment(params, tumors, self.num_tests, self.num_protocols, g, self.num_steps,
                           self.protocol_resolution,
                           seed=None if seed is None else seed + 7919 * g)
            for g in range(self.num_gpus)]

    def predict(self, protocols):
        """
        Returns fitness of each protocol.

        protocols: list of lists of pairs (simulation step, irradiation dose)
        """
        assert len(protocols) == self.num_protocols
        for experiment in self.experiments:
            experiment.add_irradiations(protocols)
            experiment.run(self.num_steps)
        results = [experiment.get_results().reshape((1, self.num_protocols, -1))
                   for experiment in self.experiments]
        results = np.concatenate(results)
        results = results.mean(0).mean(1)
        fitness = 1500 - results
        for experiment in self.experiments:
            experiment.reset()
        return fitness
