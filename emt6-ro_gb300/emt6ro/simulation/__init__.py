"""Drop-in replacement of the reference's ``emt6ro.simulation`` package
(python/emt6ro/simulation/__init__.py), backed by the GB300 CUDA library."""
from .backend import _Experiment, load_parameters, load_state, save_state
from .backend import read_instr_counters, reset_instr_counters, InstrCounters
from .backend import read_instr_histograms, INSTR_HIST_N, INSTR_HIST_DX
from .backend import Parameters, TumorState, SiteState, Coords
import numpy as np


class Experiment:
    """
    Reusable simulation object with fixed initial tumour states
    (python/emt6ro/simulation/__init__.py:6-73).

    Simulations are laid out (protocol, tumour, run).  ``seed`` (an addition
    to the reference signature) fixes the counter-based random stream; the
    default draws one from the OS like the reference's std::random_device.
    """

    def __init__(self, params, tumors, runs, protocols_num, gpu_id=0, simulation_steps=144000,
                 protocol_resolution=300, seed=None):
        self.result_shape = (protocols_num, len(tumors), runs)
        self._experiment = _Experiment(params, tumors, runs, protocols_num, simulation_steps,
                                       protocol_resolution, gpu_id, seed=seed)

    def run(self, nsteps):
        """Start nsteps simulation steps; returns immediately."""
        self._experiment.run(nsteps)

    def get_results(self):
        """Wait for the started run and return the living-cell counts as a
        (protocol, tumour, run) array."""
        res = np.array(self._experiment.results())
        return res.reshape(self.result_shape)

    def add_irradiations(self, protocols):
        """protocols: one list of (step, dose) pairs per protocol; doses
        accumulate into the bin step // protocol_resolution."""
        self._experiment.add_irradiations(protocols)

    def reset(self):
        """Restore the initial states, the step counter and empty protocols."""
        self._experiment.reset()

    def state(self):
        """All simulation lattices, in (protocol, tumour, run) order."""
        return self._experiment.state()
