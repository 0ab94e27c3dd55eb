"""ctypes wrapper of oracle/ref_gpu_driver.cu: the reference's own CUDA kernels
(built from its sources into oracle/_ref/emt6ro_ref_sm103a.cubin) driven by a
restatement of its Simulation host loop (src/emt6ro/simulation/simulation.cu).

Test and benchmark infrastructure only: it is the reference's GPU simulator,
timed beside the product and used as a distribution check on it, never part
of the product path.

Only workloads checked to stay inside the reference's fixed buffers may run
here: at most 32 occupied sites per findOccupied thread (the columns c and
c + 32 of the bordered lattice, simulation.cu:44-50) and at most 1023 entries
in a simulation's occupied list between two rebuilds (simulation.cu:58,
cell pushes one child per step for 128 steps).  `occupancy_bound` computes
the first figure for an initial state; callers keep a margin for growth.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "emt6ro_ref_sm103a.cubin"
CELL_CUBIN = HERE / "_ref" / "emt6ro_ref_cell_sm103a.cubin"
LIB = HERE / "_build" / "libref_gpu.so"

_lib = None


def available() -> bool:
    return CUBIN.exists()


def cell_available() -> bool:
    return CELL_CUBIN.exists()


def _load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            from oracle import build
            build.build_ref_gpu_driver()
        L = ctypes.CDLL(str(LIB))
        vp, u32, i64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int64
        L.refgpu_create.restype = vp
        L.refgpu_create.argtypes = [ctypes.c_char_p, vp, vp, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, vp, vp, vp, ctypes.c_int, u32, u32, u32, i64,
                                    u32]
        L.refgpu_error.restype = ctypes.c_char_p
        L.refgpu_error.argtypes = [vp]
        L.refgpu_run.restype = ctypes.c_int
        L.refgpu_run.argtypes = [vp, u32]
        L.refgpu_counts.restype = ctypes.c_int
        L.refgpu_counts.argtypes = [vp, vp]
        L.refgpu_stream.restype = vp
        L.refgpu_stream.argtypes = [vp]
        L.refgpu_destroy.restype = None
        L.refgpu_destroy.argtypes = [vp]
        for name in ("refgpu_find_occupied", "refgpu_get_fields"):
            getattr(L, name).restype = ctypes.c_int
            getattr(L, name).argtypes = [vp, vp]
        L.refgpu_find_rois.restype = ctypes.c_int
        L.refgpu_find_rois.argtypes = [vp, vp, vp]
        L.refgpu_diffuse.restype = ctypes.c_int
        L.refgpu_diffuse.argtypes = [vp]
        L.refgpu_cell_error.restype = ctypes.c_char_p
        L.refgpu_cell_error.argtypes = []
        L.refgpu_site_step.restype = ctypes.c_int
        L.refgpu_site_step.argtypes = [ctypes.c_char_p, vp, vp, vp, vp, vp, ctypes.c_int, vp, vp,
                                       i64]
        L.refgpu_divide.restype = ctypes.c_int
        L.refgpu_divide.argtypes = [ctypes.c_char_p, vp, vp, vp, vp, i64]
        L.refgpu_choose.restype = ctypes.c_int
        L.refgpu_choose.argtypes = [ctypes.c_char_p, vp, ctypes.c_int, ctypes.c_int, vp, i64]
        _lib = L
    return _lib


def _cell_check(rc: int) -> None:
    if rc != 0:
        raise RuntimeError(_lib.refgpu_cell_error().decode())


def site_step(params, sites: np.ndarray, vac: np.ndarray, dose: np.ndarray,
              draws: np.ndarray):
    """The reference's device-compiled Site::step<R> (site/site.h:62-82) on
    each site with injected draws (n x k floats).  Updates sites (oracle
    SITE_DTYPE) in place; returns (ready, draws used)."""
    L = _load()
    n = len(sites)
    vac = np.ascontiguousarray(vac, np.uint32)
    dose = np.ascontiguousarray(dose, np.float32)
    draws = np.ascontiguousarray(draws, np.float32).reshape(n, -1)
    ready = np.zeros(n, np.int32)
    used = np.zeros(n, np.int32)
    p = params.native if hasattr(params, "native") else params
    _cell_check(L.refgpu_site_step(str(CELL_CUBIN).encode(), ctypes.addressof(p),
                                   sites.ctypes.data, vac.ctypes.data, dose.ctypes.data,
                                   draws.ctypes.data, draws.shape[1], ready.ctypes.data,
                                   used.ctypes.data, n))
    return ready, used


def divide(params, parents: np.ndarray, z: np.ndarray) -> np.ndarray:
    """The reference's device-compiled divideCell<R> (cell-division.h:21-30)
    with five injected standard normals per parent; parents updated in place,
    returns the children."""
    L = _load()
    n = len(parents)
    z = np.ascontiguousarray(z, np.float32).reshape(n, 5)
    children = np.zeros(n, dtype=parents.dtype)
    p = params.native if hasattr(params, "native") else params
    _cell_check(L.refgpu_divide(str(CELL_CUBIN).encode(), ctypes.addressof(p),
                                parents.ctypes.data, z.ctypes.data, children.ctypes.data, n))
    return children


def choose(u: np.ndarray, r: int, c: int) -> np.ndarray:
    """The reference's device-compiled chooseNeighbour<R> (cell-division.h:44-54)
    of site (r, c) for each uniform: (n, 2) int32 (row, column)."""
    L = _load()
    u = np.ascontiguousarray(u, np.float32)
    rc = np.zeros((len(u), 2), np.int32)
    _cell_check(L.refgpu_choose(str(CELL_CUBIN).encode(), u.ctypes.data, r, c, rc.ctypes.data,
                                len(u)))
    return rc


def occupancy_bound(sites: np.ndarray) -> tuple[int, int]:
    """(largest occupied count of one findOccupied thread, occupied sites)."""
    st = np.asarray(sites)["state"]
    h, w = st.shape
    occ = st[: h - 1, : w - 1] == 1
    cols = occ.sum(axis=0)
    per = np.zeros(32, np.int64)
    for c, n in enumerate(cols):
        per[c % 32] += n
    return int(per.max()), int(occ.sum())


class RefGpuSimulation:
    """One reference Simulation over n simulations (tumour x protocol map)."""

    def __init__(self, params, tumors, doses, sim_tumor, sim_protocol, seed, resolution=300,
                 length=144_000):
        self._h = None
        stack = np.ascontiguousarray(np.stack([np.asarray(getattr(t, "sites", t))
                                               for t in tumors]))
        n_t, H, W = stack.shape
        for t in stack:
            per, total = occupancy_bound(t)
            if per > 29 or total > 1023 - 256:
                raise ValueError(f"initial state too large for the reference's buffers "
                                 f"({per} per thread, {total} sites)")
        L = _load()
        doses = np.ascontiguousarray(doses, np.float32)
        st = np.ascontiguousarray(sim_tumor, np.int32)
        sp = np.ascontiguousarray(sim_protocol, np.int32)
        self.n = len(st)
        self._shape = (H, W)
        self._hw = H * W
        self._keep = (stack, doses, st, sp)
        p = params.native if hasattr(params, "native") else params
        self._h = L.refgpu_create(str(CUBIN).encode(), ctypes.addressof(p),
                                  stack.ctypes.data, n_t, H, W, st.ctypes.data, sp.ctypes.data,
                                  doses.ctypes.data, doses.shape[0], doses.shape[1], resolution,
                                  length, self.n, seed)
        err = L.refgpu_error(self._h).decode()
        if err:
            L.refgpu_destroy(self._h)
            self._h = None
            raise RuntimeError(err)

    @property
    def stream(self) -> int:
        return _lib.refgpu_stream(self._h)

    def run(self, nsteps: int) -> None:
        if _lib.refgpu_run(self._h, nsteps) != 0:
            raise RuntimeError(_lib.refgpu_error(self._h).decode())

    def counts(self) -> np.ndarray:
        out = np.zeros(self.n, np.uint32)
        if _lib.refgpu_counts(self._h, out.ctypes.data) != 0:
            raise RuntimeError(_lib.refgpu_error(self._h).decode())
        return out

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise RuntimeError(_lib.refgpu_error(self._h).decode())

    def find_occupied(self) -> list[np.ndarray]:
        """One findOccupied launch: per simulation the occupied (row, column)
        pairs in the kernel's order."""
        buf = np.zeros((self.n, 1024), np.uint32)
        self._check(_lib.refgpu_find_occupied(self._h, buf.ctypes.data))
        out = []
        for row in buf:
            k = int(row[0])
            out.append(row[1:1 + k].view(np.int16).reshape(k, 2).copy())
        return out

    def find_rois(self) -> tuple[np.ndarray, np.ndarray]:
        """One findROIsKernel launch: (n x 4 int16 ROIs (origin row, column,
        height, width), n x H*W mask bytes)."""
        rois = np.zeros((self.n, 4), np.int16)
        masks = np.zeros((self.n, self._hw), np.uint8)
        self._check(_lib.refgpu_find_rois(self._h, rois.ctypes.data, masks.ctypes.data))
        return rois, masks

    def diffuse(self) -> None:
        """One diffusionKernel launch with the last ROIs and masks."""
        self._check(_lib.refgpu_diffuse(self._h))

    def fields(self) -> np.ndarray:
        """(n, 3, H, W) float32 substrate fields."""
        out = np.zeros((self.n, 3, self._shape[0], self._shape[1]), np.float32)
        self._check(_lib.refgpu_get_fields(self._h, out.ctypes.data))
        return out

    def close(self) -> None:
        if self._h:
            _lib.refgpu_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
