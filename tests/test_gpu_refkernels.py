"""The oracle's restatement of each reference kernel, held to that kernel's
own output on the GPU, one kernel at a time.

oracle/_ref/emt6ro_ref_sm103a.cubin is the reference's device code compiled
from its sources (oracle/build.py); oracle/ref_gpu_driver.cu launches one of
its kernels alone on lattices the test builds:

  findOccupied    (src/emt6ro/simulation/simulation.cu:41-64): list order
                  and size bit-exact against orc_rebuild_list;
  findROIsKernel  (src/emt6ro/diffusion/diffusion.cu:16-108): ROI and border
                  mask bit-exact against orc_find_roi;
  diffusionKernel (diffusion.cu:122-191): one step of 23 + 1 substeps within
                  1e-5 relative (denominator max(|x|, 1e-3 x external
                  level)) of the oracle's FP64 evaluation, and of this
                  project's kernel.

oracle/_ref/emt6ro_ref_cell_sm103a.cubin is the reference's cell model
(cell/cell.cu with the templated Site::step, divideCell, chooseNeighbour)
built for the GPU with nvcc's defaults; it is driven with the golden
vectors' injected draws and compared with the host-compiled reference
(tests/golden/*.npz, which this project's kernels match bit for bit).

Every lattice stays inside the reference's fixed buffers: at most 29
occupied sites per findOccupied thread (checked by occupancy_bound)."""
import ctypes

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

H = W = 53
# (radius, centre, density); radius 0 with density 1 is a single cell, None
# an empty lattice, a pair of discs is given as a list
CASES = [None, (0, (26, 26), 1.0), (3, (26, 26), 0.9), (8, (20, 30), 0.9), (10, (26, 26), 0.9),
         (13, (26, 26), 0.95), (12, (14, 3), 0.9), (9, (49, 47), 0.9),
         [(5, (10, 10), 0.9), (5, (40, 44), 0.9)], (13, (3, 26), 0.9), (13, (26, 26), 0.3),
         (6, (26, 49), 0.9)]


def _lattice(case, rng, params):
    from oracle import pyoracle as po
    g = np.zeros((H, W), dtype=po.SITE_DTYPE)
    g["state"][0, :] = g["state"][-1, :] = 2
    g["state"][:, 0] = g["state"][:, -1] = 2
    rr, cc = np.mgrid[0:H, 0:W]
    inner = (rr > 0) & (rr < H - 1) & (cc > 0) & (cc < W - 1)
    discs = [] if case is None else (case if isinstance(case, list) else [case])
    for radius, (r0, c0), density in discs:
        disc = ((rr - r0) ** 2 + (cc - c0) ** 2 <= radius ** 2) & inner
        g["state"][disc & (rng.random((H, W)) < density)] = 1
    ext = np.array(params.native.external_levels[:], np.float32)
    for f, name in enumerate(("cho", "ox", "gi")):
        g[name] = (ext[f] * (0.2 + 0.8 * rng.random((H, W)))).astype(np.float32)
    g["ox"][g["state"] == 1] *= np.float32(0.02)  # hypoxic core, ox near zero
    g["cycle_times"] = np.float32([6, 16, 18, 20, 20.1])
    return g


@pytest.fixture(scope="module")
def ref_kernels(params):
    from oracle import pyrefgpu
    if not pyrefgpu.available():
        pytest.skip("reference cubin not built (needs the reference checkout)")
    rng = np.random.default_rng(8080)
    lattices = [_lattice(c, rng, params) for c in CASES]
    for g in lattices:
        per, _ = pyrefgpu.occupancy_bound(g)
        assert per <= 29
    n = len(lattices)
    sim = pyrefgpu.RefGpuSimulation(params, lattices, np.zeros((1, 480), np.float32),
                                    np.arange(n, dtype=np.int32), np.zeros(n, np.int32), seed=5)
    fields0 = sim.fields()
    occupied = sim.find_occupied()
    rois, masks = sim.find_rois()
    sim.diffuse()
    fields1 = sim.fields()
    sim.close()
    return lattices, fields0, occupied, rois, masks, fields1


@pytest.mark.parametrize("case", range(len(CASES)))
def test_find_occupied_matches_oracle(case, ref_kernels, oracle):
    lattices, _, occupied, _, _, _ = ref_kernels
    st = np.ascontiguousarray(lattices[case]["state"].reshape(-1))
    lo = np.zeros(H * W + 256, np.uint16)
    no = oracle.oracle().L.orc_rebuild_list(st, H, W, lo)
    theirs = occupied[case]
    assert len(theirs) == no
    assert (theirs[:, 0].astype(np.int64) * W + theirs[:, 1] == lo[:no]).all()


@pytest.mark.parametrize("case", range(len(CASES)))
def test_find_roi_matches_oracle(case, ref_kernels, oracle):
    lattices, _, _, rois, masks, _ = ref_kernels
    st = np.ascontiguousarray(lattices[case]["state"].reshape(-1))
    ro = np.zeros(5, np.int32)
    mo = np.zeros(H * W + 512, np.uint8)
    oracle.oracle().L.orc_find_roi(st, H, W, ro, mo)
    assert rois[case].tolist() == ro[:4].tolist()
    if ro[2] > 0:
        m = (ro[2] + 2) * (ro[3] + 2)
        assert (masks[case][:m] == mo[:m]).all()


@pytest.mark.parametrize("case", range(len(CASES)))
def test_diffusion_matches_fp64_oracle_and_this_kernel(case, ref_kernels, params, oracle):
    from emt6ro import _native as N
    lattices, fields0, _, _, _, fields1 = ref_kernels
    st = np.ascontiguousarray(lattices[case]["state"].reshape(-1))
    ro = np.zeros(5, np.int32)
    mo = np.zeros(H * W + 512, np.uint8)
    L = oracle.oracle().L
    L.orc_find_roi(st, H, W, ro, mo)
    f0 = fields0[case]
    f64 = np.ascontiguousarray(f0.reshape(-1).astype(np.float64))
    L.orc_diffuse_f64(f64, H, W, ro, mo, ctypes.byref(oracle.params_copy(params)))
    ours = np.ascontiguousarray(f0.reshape(-1).copy())
    N.check(N.lib().emt6_test_diffuse(ctypes.byref(params.native), N.ptr(ours), H, W, N.ptr(ro),
                                      1, 0))
    theirs = fields1[case].astype(np.float64)
    ref64 = f64.reshape(3, H, W)
    mine = ours.reshape(3, H, W).astype(np.float64)
    ext = np.array(params.native.external_levels[:], np.float64)
    if ro[2] == 0:
        assert (fields1[case] == f0).all()  # no ROI: the kernel returns at once
    for f in range(3):
        eps = 1e-3 * ext[f]
        rel = np.abs(theirs[f] - ref64[f]) / np.maximum(np.abs(ref64[f]), eps)
        assert rel.max() <= 1e-5, (f, rel.max())
        rel = np.abs(theirs[f] - mine[f]) / np.maximum(np.abs(ref64[f]), eps)
        assert rel.max() <= 2e-5, (f, rel.max())


def _ulps(a, b):
    """Distance in units in the last place between float32 arrays."""
    ia = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    ib = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return np.abs(ia - ib)


def test_device_built_reference_site_step(params):
    """Site::step of the reference's own device build against its host build
    (the golden vectors, which this project's kernel reproduces bit for bit),
    on the same 6,000 sites and injected draws.  The device build evaluates
    expf with CUDA's routine and contracts a*b+c into FMAs, so the repair
    delay and survival probability may differ in the last bits; every
    decision (alive, ready, draws used, phase, mode, state) must agree except
    where a float lies within a few ulps of its threshold, and every float
    within 4 ulps."""
    from oracle import pyrefgpu
    if not pyrefgpu.cell_available():
        pytest.skip("reference cell cubin not built (needs the reference checkout)")
    g = np.load(GOLDEN / "site_step.npz")
    sites = np.ascontiguousarray(g["sites"].copy())
    ready, used = pyrefgpu.site_step(params, sites, g["vac"], g["dose"], g["draws"])
    out = g["out"]
    decisions = ((ready != g["ready"]) | (used != g["used"]) | (sites["state"] != out["state"]) |
                 (sites["phase"] != out["phase"]) | (sites["mode"] != out["mode"]))
    assert decisions.sum() <= 3, np.nonzero(decisions)[0][:20]
    same = ~decisions
    worst = {}
    for f in ("cho", "ox", "gi", "time_in_repair", "irradiation", "repair_delay_time",
              "proliferation_time", "cycle_times"):
        u = _ulps(sites[f][same], out[f][same])
        worst[f] = int(u.max()) if u.size else 0
    assert max(worst.values()) <= 4, worst
    exact = sum(sites[k].tobytes() == out[k].tobytes() for k in range(len(sites)))
    print(f"device-built reference Site::step: {exact} of {len(sites)} sites bit-identical to "
          f"the host build; decisions differ on {int(decisions.sum())}; worst ulps {worst}")


def test_device_built_reference_choose_and_divide(params):
    """chooseNeighbour and divideCell of the reference's device build against
    the host-build golden vectors: neighbour choice identical on every
    uniform (including u = 1); parents and children within 4 ulps (a child
    of an irradiated parent gets its repair delay from CUDA's expf, whose
    error bound is 2 ulps, times the delay coefficient)."""
    from oracle import pyrefgpu
    if not pyrefgpu.cell_available():
        pytest.skip("reference cell cubin not built (needs the reference checkout)")
    g = np.load(GOLDEN / "choose.npz")
    rc = pyrefgpu.choose(g["u"], 26, 26)
    assert (rc == g["rc"]).all()
    g = np.load(GOLDEN / "divide.npz")
    parents = np.ascontiguousarray(g["parents"].copy())
    children = pyrefgpu.divide(params, parents, g["z"])
    for f in ("time_in_repair", "irradiation", "repair_delay_time", "proliferation_time",
              "cycle_times"):
        assert _ulps(parents[f], g["parents_out"][f]).max() <= 4, f
        assert _ulps(children[f], g["children"][f]).max() <= 4, f
    exact = sum(children[k].tobytes() == g["children"][k].tobytes() for k in range(len(children)))
    print(f"device-built reference divideCell: {exact} of {len(children)} children "
          "bit-identical to the host build")
    assert (parents["phase"] == g["parents_out"]["phase"]).all()
    assert (children["phase"] == g["children"]["phase"]).all()
