"""Seeded synthetic workloads: disc tumours, irradiation protocols, default
parameters.

Tumours follow the benchmark description: cells fill a centred disc of radius
r on the 51 x 51 interior (53 x 53 with the border ring); each cell's phase is
drawn G1/S/G2/M with probabilities 0.45/0.30/0.15/0.10, its cycle-phase end
times are cumulative normal draws as in createCell
(src/emt6ro/simulation/cell-division.h:10-19), and its proliferation clock is
uniform within the drawn phase.  Substrates start at the external levels,
mode is aerobic proliferation, no irradiation.
"""
from __future__ import annotations

import numpy as np

from . import _native as N
from .simulation.backend import Parameters, TumorState

HOUR_STEPS = 600         # 6-s steps (data/default-parameters.json "time_step": 6)
PROTOCOL_RESOLUTION = 300  # 30 min


def default_parameters() -> Parameters:
    """The reference's data/default-parameters.json as a parameter block."""
    p = N.Params()
    p.lattice_height, p.lattice_width = 51, 51
    p.time_step = 6.0
    p.diffusion_coeffs[:] = [0.7, 1.3409874655051011, 0.81048692970088532]
    p.diffusion_time_step = 0.25
    p.metabolism[0][:] = [21.6, 9.96, 0.0]
    p.metabolism[1][:] = [54.0, 0.0, -3.0e-3]
    p.metabolism[2][:] = [18.0, 8.28, 0.0]
    p.metabolism[3][:] = [45.0, 0.0, -3.0e-5]
    p.external_levels[:] = [275.0, 14.0, 1.99e-3]
    p.death_gi = 5.0e-2
    p.quiescence_gi = 1.99e-2
    p.death_gi_production = 0.0
    for i, (m, s) in enumerate([(6, 1), (10, 2), (2, 0), (2, 0), (0.1, 0)]):
        p.cycle_times[i][0] = m
        p.cycle_times[i][1] = s
    p.delay_time_coeff, p.delay_time_exp_coeff = 3.3414, 0.1492
    p.survival_prob_coeff, p.survival_prob_exp_coeff = 1.0, -0.4993
    p.repair_half_time = 0.8
    return Parameters(p)


PHASE_PROBS = (0.45, 0.30, 0.15, 0.10)


def disc_tumor(params: Parameters, radius: float, seed: int,
               center: tuple[int, int] | None = None) -> TumorState:
    """Seeded disc tumour on the parameters' lattice (border ring MOCKED)."""
    p = params.native if isinstance(params, Parameters) else params
    H, W = p.lattice_height + 2, p.lattice_width + 2
    rng = np.random.default_rng(seed)
    g = np.zeros((H, W), dtype=N.SITE_DTYPE)
    ext = np.array(p.external_levels[:], np.float32)
    g["cho"], g["ox"], g["gi"] = ext
    g["state"] = 0
    g["state"][0, :] = 2
    g["state"][-1, :] = 2
    g["state"][:, 0] = 2
    g["state"][:, -1] = 2
    cr, cc = center if center is not None else (H // 2, W // 2)
    rr, cols = np.mgrid[0:H, 0:W]
    inside = ((rr - cr) ** 2 + (cols - cc) ** 2 <= radius * radius)
    inside[0, :] = inside[-1, :] = False
    inside[:, 0] = inside[:, -1] = False
    n = int(inside.sum())
    mean = np.array([p.cycle_times[i][0] for i in range(5)], np.float32)
    sd = np.array([p.cycle_times[i][1] for i in range(5)], np.float32)
    z = rng.standard_normal((n, 5)).astype(np.float32)
    inc = (sd * z + mean).astype(np.float32)
    times = np.cumsum(inc, axis=1, dtype=np.float32)
    phase = rng.choice(4, size=n, p=PHASE_PROBS)
    lo = np.where(phase == 0, np.float32(0), times[np.arange(n), np.maximum(phase - 1, 0)])
    hi = times[np.arange(n), phase]
    u = rng.random(n).astype(np.float32)
    prolif = (lo + (hi - lo) * u).astype(np.float32)
    cells = g[inside]
    cells["state"] = 1
    cells["cycle_times"] = times
    cells["phase"] = phase.astype(np.uint8)
    cells["proliferation_time"] = prolif
    cells["mode"] = 0
    g[inside] = cells
    return TumorState(g)


def protocol_2x125gy():
    """2 x 1.25 Gy at hours 12 and 36."""
    return [(12 * HOUR_STEPS, 1.25), (36 * HOUR_STEPS, 1.25)]


def random_protocol(rng, k: int, total_gy: float = 10.0, quantum: float = 0.25,
                    window_steps: int = 48 * HOUR_STEPS, grid: int = PROTOCOL_RESOLUTION):
    """k doses of whole quanta summing to total_gy at distinct grid times in the window."""
    if k <= 0:
        return []
    q = int(round(total_gy / quantum))
    cuts = np.sort(rng.choice(np.arange(1, q), size=k - 1, replace=False)) if k > 1 else []
    parts = np.diff(np.concatenate([[0], cuts, [q]])).astype(int)
    slots = np.sort(rng.choice(window_steps // grid, size=k, replace=False))
    return [(int(s) * grid, float(n) * quantum) for s, n in zip(slots, parts)]


def ga_protocols(n: int = 100, seed: int = 1000):
    """1-8 doses, 0.25-Gy quanta, 10 Gy total, on the 30-min grid in the first 48 h."""
    rng = np.random.default_rng(seed)
    return [random_protocol(rng, int(rng.integers(1, 9))) for _ in range(n)]


def ga_tumors(params: Parameters, n: int = 20, seed0: int = 1):
    """n tumours, disc radius uniform in 6..14, seeds seed0.."""
    out = []
    for i in range(n):
        rng = np.random.default_rng(seed0 + i)
        r = int(rng.integers(6, 15))
        out.append(disc_tumor(params, r, seed=10_000 + seed0 + i))
    return out


def ragged_batch(params: Parameters, n_sims: int = 30000, seed: int = 2024,
                   horizons=(72_000, 144_000, 288_000), n_tumors: int = 64):
    """Ragged batch: disc radius 2..20, 0-12 doses, horizons mixed uniformly.
    Returns (tumours, protocols, sim_tumor, sim_protocol, sim_horizon)."""
    rng = np.random.default_rng(seed)
    radii = rng.integers(2, 21, n_tumors)
    tumors = [disc_tumor(params, int(r), seed=seed * 7 + i) for i, r in enumerate(radii)]
    n_prot = 256
    prots = [random_protocol(rng, int(rng.integers(0, 13))) for _ in range(n_prot)]
    sim_tumor = rng.integers(0, n_tumors, n_sims).astype(np.int32)
    sim_protocol = rng.integers(0, n_prot, n_sims).astype(np.int32)
    sim_horizon = rng.choice(np.asarray(horizons, np.uint32), n_sims).astype(np.uint32)
    return tumors, prots, sim_tumor, sim_protocol, sim_horizon


def protocol_doses(protocols, bins: int, resolution: int = PROTOCOL_RESOLUTION) -> np.ndarray:
    """Dose table (n_protocols x bins): doses accumulate into bin step // resolution."""
    d = np.zeros((len(protocols), bins), np.float32)
    for i, prot in enumerate(protocols):
        for t, dose in prot:
            if not 0 <= int(t) // resolution < bins:
                raise ValueError(f"irradiation step {int(t)} is beyond the protocol length")
            d[i, int(t) // resolution] += np.float32(dose)
    return d
