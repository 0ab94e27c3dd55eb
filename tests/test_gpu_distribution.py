"""Distribution parity with the reference's own CPU path.

tests/golden/dist_refcpu.npz holds 1000 replicate final living-cell counts per
case from the reference's host-compiled cell model and std::mt19937 engine
driving the restated kernels (tests/golden/make_distribution.py).  The GPU
simulator, with its own Philox stream, must match in mean, 10/50/90%
quantiles and a two-sample Kolmogorov-Smirnov test (p > 0.01)."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = {
    "r10_2x1.25Gy_36h": (10, 0, [(6 * 600, 1.25), (18 * 600, 1.25)], 36 * 600),
    "r8_1x4Gy_24h": (8, 5, [(2 * 600, 4.0)], 24 * 600),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_final_count_distribution_matches_reference_cpu_path(name, params):
    from scipy import stats
    import emt6ro.simulation as sim
    from emt6ro import workloads as wl
    path = GOLDEN / "dist_refcpu.npz"
    if not path.exists():
        pytest.skip("distribution fixture not generated")
    ref = np.load(path)[name].astype(np.float64)
    radius, tseed, prot, steps = CASES[name]
    tumor = wl.disc_tumor(params, radius, seed=tseed)
    e = sim.Experiment(params, [tumor], len(ref), 1, seed=2024)
    e.add_irradiations([prot])
    e.run(steps)
    ours = e.get_results().reshape(-1).astype(np.float64)
    assert ours.size == ref.size >= 1000
    p = stats.ks_2samp(ours, ref).pvalue
    assert p > 0.01, (p, ours.mean(), ref.mean())
    assert abs(ours.mean() - ref.mean()) <= 0.02 * ref.mean()
    for q in (0.1, 0.5, 0.9):
        assert abs(np.quantile(ours, q) - np.quantile(ref, q)) <= 0.03 * np.quantile(ref, q) + 2
