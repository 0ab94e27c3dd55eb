"""Device functions of the CUDA library vs the oracle and the reference's golden
vectors, through the C ABI.  Bit-exact: Philox, the double-precision
exp/log/sincos kernels, Box-Muller normals, Site::step with injected draws,
chooseNeighbour, divideCell, the occupied list and the ROI/mask.  Diffusion:
bit-exact vs the oracle's FP32 formula and within 1e-5 relative of the FP64
evaluation of the reference's formula (per step)."""
import ctypes

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _N():
    from emt6ro import _native as N
    return N


def _bytes_equal(a, b):
    return np.ascontiguousarray(a).tobytes() == np.ascontiguousarray(b).tobytes()


def _site_mismatch(a, b):
    bad = {}
    for f in a.dtype.names:
        x = np.ascontiguousarray(a[f]).reshape(len(a), -1).view(np.uint8)
        y = np.ascontiguousarray(b[f]).reshape(len(b), -1).view(np.uint8)
        ne = (x != y).any(1)
        if ne.any():
            bad[f] = int(ne.sum())
    return bad


def test_philox_matches_oracle_and_kat(oracle):
    N = _N()
    rng = np.random.default_rng(0)
    n = 4096
    ctr = rng.integers(0, 2**32, (n, 4), dtype=np.uint64).astype(np.uint32)
    key = rng.integers(0, 2**32, (n, 2), dtype=np.uint64).astype(np.uint32)
    # Random123 known-answer vectors for philox4x32-10
    ctr[0], key[0] = [0, 0, 0, 0], [0, 0]
    ctr[1], key[1] = [0xffffffff] * 4, [0xffffffff] * 2
    ctr[2], key[2] = [0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]
    out = np.zeros((n, 4), np.uint32)
    N.check(N.lib().emt6_test_philox(N.ptr(ctr), N.ptr(key), N.ptr(out), n, 0))
    assert out[0].tolist() == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert out[1].tolist() == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert out[2].tolist() == [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]
    L = oracle.oracle().L
    for i in range(0, n, 97):
        o = np.zeros(4, np.uint32)
        L.orc_philox4x32_10(np.ascontiguousarray(ctr[i]), np.ascontiguousarray(key[i]), o)
        assert o.tolist() == out[i].tolist()


def test_double_math_bit_exact(oracle):
    N = _N()
    rng = np.random.default_rng(1)
    n = 20000
    x = np.concatenate([rng.uniform(-25, 8, n - 4), [0.0, -0.0, 1e-30, -20.0]]).astype(np.float32)
    u = np.concatenate([rng.random(n - 3), [2.0**-24, 1.0, 0.5]]).astype(np.float64)
    e = np.zeros(n, np.float32)
    lg = np.zeros(n, np.float64)
    sn = np.zeros(n, np.float64)
    cs = np.zeros(n, np.float64)
    N.check(N.lib().emt6_test_math(N.ptr(x), N.ptr(e), N.ptr(u), N.ptr(lg), N.ptr(sn), N.ptr(cs),
                                   n, 0))
    L = oracle.oracle().L
    s = ctypes.c_double()
    c = ctypes.c_double()
    for i in range(0, n, 7):
        assert np.float32(L.orc_expf(float(x[i]))).tobytes() == e[i].tobytes()
        assert L.orc_log_core(float(u[i])) == lg[i]
        v = u[i] - np.floor(u[i])
        L.orc_sincos2pi(float(v), ctypes.byref(s), ctypes.byref(c))
        assert (s.value, c.value) == (sn[i], cs[i])


def test_division_normals_bit_exact(oracle):
    N = _N()
    n = 3000
    rng = np.random.default_rng(2)
    step = rng.integers(0, 300000, n).astype(np.uint32)
    sim = rng.integers(0, 40000, n).astype(np.uint32)
    seed = 0x1234567890ABCDEF
    z = np.zeros((n, 5), np.float32)
    N.check(N.lib().emt6_test_normals(seed, N.ptr(step), N.ptr(sim), 3, N.ptr(z), n, 0))
    L = oracle.oracle().L
    for i in range(0, n, 5):
        zo = np.zeros(5, np.float32)
        L.orc_division_normals(seed, int(step[i]), int(sim[i]), 3, zo)
        assert zo.tobytes() == z[i].tobytes()
    assert abs(z.mean()) < 0.05 and abs(z.std() - 1) < 0.05


def test_site_step_matches_reference_golden(params):
    """Site::step (site/site.h:62-82) driven by injected draws: the device model
    reproduces the reference's own host-compiled function bit for bit."""
    N = _N()
    g = np.load(GOLDEN / "site_step.npz")
    sites = g["sites"].copy()
    n = len(sites)
    ready = np.zeros(n, np.int32)
    used = np.zeros(n, np.int32)
    N.check(N.lib().emt6_test_site_step(ctypes.byref(params.native), N.ptr(sites),
                                        N.ptr(np.ascontiguousarray(g["vac"])),
                                        N.ptr(np.ascontiguousarray(g["dose"])),
                                        N.ptr(np.ascontiguousarray(g["draws"])), N.ptr(ready),
                                        N.ptr(used), n, 0))
    assert (ready == g["ready"]).all()
    assert (used == g["used"]).all()
    assert _site_mismatch(sites, g["out"]) == {}


def test_choose_neighbour_matches_golden():
    N = _N()
    g = np.load(GOLDEN / "choose.npz")
    u = np.ascontiguousarray(g["u"])
    rc = np.zeros((len(u), 2), np.int32)
    N.check(N.lib().emt6_test_choose(N.ptr(u), 26, 26, N.ptr(rc), len(u), 0))
    assert (rc == g["rc"]).all()


def test_divide_matches_golden(params):
    N = _N()
    g = np.load(GOLDEN / "divide.npz")
    parents = g["parents"].copy()
    z = np.ascontiguousarray(g["z"])
    children = np.zeros(len(parents), dtype=N.SITE_DTYPE)
    N.check(N.lib().emt6_test_divide(ctypes.byref(params.native), N.ptr(parents), N.ptr(z),
                                     N.ptr(children), len(parents), 0))
    exp_p = g["parents_out"]
    exp_c = g["children"]
    cell_fields = ["time_in_repair", "irradiation", "repair_delay_time", "proliferation_time",
                   "cycle_times", "mode", "phase"]
    for f in cell_fields:
        assert _bytes_equal(parents[f], exp_p[f]), f
        assert _bytes_equal(children[f], exp_c[f]), f


def _random_lattice(rng, H, W, radius, center, density=0.9):
    st = np.zeros((H, W), np.uint8)
    st[0, :] = st[-1, :] = 2
    st[:, 0] = st[:, -1] = 2
    rr, cc = np.mgrid[0:H, 0:W]
    disc = (rr - center[0]) ** 2 + (cc - center[1]) ** 2 <= radius ** 2
    disc &= (rr > 0) & (rr < H - 1) & (cc > 0) & (cc < W - 1)
    st[disc & (rng.random((H, W)) < density)] = 1
    return st


@pytest.mark.parametrize("case", range(12))
def test_list_and_roi_match_oracle(case, oracle):
    N = _N()
    rng = np.random.default_rng(100 + case)
    H = W = 53
    radius = [0, 1, 3, 8, 12, 15, 19, 24, 30, 5, 10, 40][case]
    center = (int(rng.integers(2, 51)), int(rng.integers(2, 51)))
    st = np.ascontiguousarray(_random_lattice(rng, H, W, radius, center))
    L = oracle.oracle().L
    lst = np.zeros(H * W + 256, np.uint16)
    n = ctypes.c_uint32()
    N.check(N.lib().emt6_test_list(N.ptr(st), H, W, N.ptr(lst), ctypes.byref(n), 0))
    lo = np.zeros(H * W + 256, np.uint16)
    no = L.orc_rebuild_list(st.reshape(-1), H, W, lo)
    assert n.value == no
    assert (lst[:no] == lo[:no]).all()
    roi = np.zeros(8, np.int32)
    mask = np.zeros(H * W + 512, np.uint8)
    N.check(N.lib().emt6_test_roi(N.ptr(st), H, W, N.ptr(roi), N.ptr(mask), 0))
    ro = np.zeros(5, np.int32)
    mo = np.zeros(H * W + 512, np.uint8)
    L.orc_find_roi(st.reshape(-1), H, W, ro, mo)
    assert roi[:5].tolist() == ro.tolist()
    m = (ro[2] + 2) * (ro[3] + 2) if ro[2] > 0 else 0
    assert (mask[:m] == mo[:m]).all()


def _diffusion_parity(st, rng, params, oracle):
    """One diffusion step of lattice st's ROI on both kernel paths: bit-exact
    against the oracle's FP32 formula and within 1e-5 relative of the FP64
    evaluation of the reference formula.  Returns (rows, columns, paths run)."""
    N = _N()
    H, W = st.shape
    L = oracle.oracle().L
    roi = np.zeros(5, np.int32)
    mask = np.zeros(H * W + 512, np.uint8)
    L.orc_find_roi(np.ascontiguousarray(st.reshape(-1)), H, W, roi, mask)
    assert roi[2] > 0
    ext = np.array(params.native.external_levels[:], np.float32)
    fld = np.empty((3, H, W), np.float32)
    for f in range(3):
        fld[f] = ext[f] * (0.2 + 0.8 * rng.random((H, W)))
    fld[1][st == 1] *= 0.02  # hypoxic core, ox near zero
    f32 = fld.reshape(-1).copy()
    p = params.native
    po_p = oracle.params_copy(params)
    L.orc_diffuse_f32(f32, H, W, roi, mask, ctypes.byref(po_p))
    f64 = np.ascontiguousarray(fld.reshape(-1).astype(np.float64))
    L.orc_diffuse_f64(f64, H, W, roi, mask, ctypes.byref(po_p))
    nrow, ncol = roi[2] + 2, roi[3] + 2
    ran = []
    for v in (0, 1):
        g = np.ascontiguousarray(fld.reshape(-1).copy())
        rc = N.lib().emt6_test_diffuse(ctypes.byref(p), N.ptr(g), H, W, N.ptr(roi), v, 0)
        if v == 0 and rc == N.EMT6_ERR_LIMIT:
            # the narrow path holds regions up to 32 x 31, and 33 x 33 ones
            # whose first and last ring are fixed
            assert nrow > 32 or ncol > 31
            continue
        N.check(rc)
        ran.append(v)
        assert g.tobytes() == f32.tobytes(), f"variant {v} differs from the FP32 oracle"
        gf = g.reshape(3, H, W).astype(np.float64)
        rf = f64.reshape(3, H, W)
        for f in range(3):
            eps = 1e-3 * float(ext[f])
            rel = np.abs(gf[f] - rf[f]) / np.maximum(np.abs(rf[f]), eps)
            assert rel.max() <= 1e-5, (v, f, rel.max())
    if nrow <= 32 and ncol <= 31:
        assert ran == [0, 1]
    return nrow, ncol, ran


@pytest.mark.parametrize("case", range(10))
def test_diffusion_step_parity(case, params, oracle):
    """One diffusion step (23 free substeps + final ROI pass) of near-centred
    discs from 9 x 9 to 55 x 55 regions."""
    rng = np.random.default_rng(200 + case)
    H = W = 53
    radius = [3, 6, 9, 11, 13, 14, 16, 19, 22, 26][case]
    center = (26 + int(rng.integers(-4, 5)), 26 + int(rng.integers(-4, 5)))
    st = _random_lattice(rng, H, W, radius, center, density=0.95)
    nrow, ncol, ran = _diffusion_parity(st, rng, params, oracle)
    if radius in (13, 14):
        assert 0 in ran  # 31-wide unclipped ROI: the shifted narrow mapping
    if (nrow, ncol) == (35, 35):
        assert 0 in ran  # distance-16 unclipped ROI: the ring mapping


@pytest.mark.parametrize("radius", range(0, 17))
def test_diffusion_unclipped_discs_of_every_distance(radius, params, oracle):
    """Full unclipped discs of every distance up to 16 (regions of 3 x 3 to
    35 x 35 sites): bit-exact against the FP32 oracle and within 1e-5 of the
    FP64 formula, on both kernel paths; every one of them runs on the narrow
    kernel (the largest with the ring mapping)."""
    rng = np.random.default_rng(300 + radius)
    H = W = 53
    center = (26 + int(rng.integers(-3, 4)), 26 + int(rng.integers(-3, 4)))
    st = _random_lattice(rng, H, W, radius, center, density=1.0)
    nrow, ncol, ran = _diffusion_parity(st, rng, params, oracle)
    assert nrow == ncol and nrow <= 35
    assert 0 in ran  # every unclipped disc up to distance 16 runs on the narrow kernel


@pytest.mark.parametrize("radius", [22, 23, 24])
def test_diffusion_large_unclipped_discs(radius, params, oracle):
    """Unclipped discs of distance 22-24 on the wide kernel (47 x 47 regions
    on three-column bands, 49 x 49 on the same bands shifted to rows and
    columns 1..48, 51 x 51 on two-column tiles): bit-exact against the FP32
    oracle and within 1e-5 of the FP64 formula."""
    rng = np.random.default_rng(500 + radius)
    st = _random_lattice(rng, 53, 53, radius, (26, 26), density=1.0)
    nrow, ncol, ran = _diffusion_parity(st, rng, params, oracle)
    assert (nrow, ncol) == (2 * radius + 3,) * 2 and ran == [1]


# Tumours against the lattice edge: ROIs clipped to fewer columns than rows,
# which reach the register layouts a centred disc does not (eight-lane bands
# of 2 columns with 3-4 rows and of 3 columns with 4 rows, the wide kernel's
# three-column bands on a 41 x 32 region, two-column wide tiles of 14 rows),
# and clipped regions exactly as wide as a layout's lanes hold columns
# (16, 24, 32, 48) with free sites in a ring column: the shuffle that fetches
# column 0's left neighbour must not wrap to the opposite ring column there.
# (radius, centre, seed, expected rows x columns)
_CLIPPED = [(4, (26, 2), 1402, (13, 11)), (6, (26, 2), 1602, (17, 14)),
            (6, (26, 20), 1620, (17, 17)), (9, (26, 5), 1905, (25, 21)),
            (11, (26, 7), 2107, (29, 25)), (13, (26, 2), 2302, (33, 25)),
            (16, (26, 4), 2604, (41, 32)), (17, (26, 2), 2702, (41, 31)),
            (19, (26, 9), 2909, (49, 40)), (6, (26, 4), 1604, (19, 16)),
            (10, (26, 8), 2008, (27, 24)), (13, (3, 13), 135313, (27, 32)),
            (20, (8, 22), 205822, (41, 48))]
# strips of occupied sites along the left edge: (columns, expected shape)
_STRIPS = [(1, (25, 14)), (2, (27, 16))]


@pytest.mark.parametrize("case", range(len(_CLIPPED) + len(_STRIPS)))
def test_diffusion_clipped_regions(case, params, oracle):
    H = W = 53
    if case < len(_CLIPPED):
        radius, center, seed, shape = _CLIPPED[case]
        rng = np.random.default_rng(seed)
        st = _random_lattice(rng, H, W, radius, center, density=0.95)
    else:
        # 23 rows of one or two columns: a 25 x 14 or 27 x 16 region
        cols, shape = _STRIPS[case - len(_CLIPPED)]
        rng = np.random.default_rng(77 + cols)
        st = np.zeros((H, W), np.uint8)
        st[0, :] = st[-1, :] = st[:, 0] = st[:, -1] = 2
        st[14:37, 1:1 + cols] = 1
    nrow, ncol, _ = _diffusion_parity(st, rng, params, oracle)
    assert (nrow, ncol) == shape
